"""The fused contraction's oracle on the CPU: loop_dgemm.c (the skeleton's
reference DGEMM, branches/old/python/macaroni/ccsd_t2_8_skeleton.F:214-292)
and the sort -> DGEMM -> sort chain (:174-184), pinned against numpy and,
as the skeleton itself checks its dgemm, exactly on the number_array fill
(:439-447) whose sums are all exact."""
import numpy as np
import pytest

from oracle import oracle as O


def colmajor(flat, rows, cols):
    return flat.reshape(cols, rows).T


@pytest.mark.parametrize("case", [1, 2, 3, 4])
def test_loop_dgemm_every_case_matches_numpy(case):
    rng = np.random.default_rng(case)
    m, n, k = 7, 5, 9
    if case == 1:
        ra, ca, rb, cb = m, k, k, n
    elif case == 2:
        ra, ca, rb, cb = m, k, n, k
    elif case == 3:
        ra, ca, rb, cb = k, m, k, n
    else:
        ra, ca, rb, cb = k, m, n, k
    a = rng.uniform(-1, 1, ra * ca)
    b = rng.uniform(-1, 1, rb * cb)
    c0 = rng.uniform(-1, 1, m * n)
    A, B = colmajor(a, ra, ca), colmajor(b, rb, cb)
    opa = A if case in (1, 2) else A.T
    opb = B if case in (1, 3) else B.T
    want = 0.5 * colmajor(c0, m, n) - 1.5 * (opa @ opb)
    c = c0.copy()
    O.loop_dgemm(-1.5, 0.5, a, b, c, ra, ca, rb, cb, m, n, case)
    np.testing.assert_allclose(colmajor(c, m, n), want, rtol=1e-13, atol=1e-13)


def test_loop_dgemm_refuses_mismatched_shapes():
    a = np.zeros(6)
    with pytest.raises(ValueError):
        O.loop_dgemm(1.0, 0.0, a, a, a.copy(), 2, 3, 2, 3, 2, 3, 3)


def test_skeleton_number_array_fill_is_exact():
    """ccsd_t2_8_skeleton.F:60-158: number_array operands, tce_sort_4 4321
    and 2143, dgemm('T','N') checked against loop_dgemm case 3 with
    compare_arrays (exact); the sums are integers below 2^53, so any
    summation order gives these bits."""
    d1, d2, d3, d4, d5, d6 = 8, 9, 4, 5, 6, 7
    t = np.arange(1, d5 * d6 * d1 * d2 + 1, dtype=np.float64)
    v = np.arange(1, d3 * d4 * d5 * d6 + 1, dtype=np.float64)
    got = O.contract_4x4(t, (d5, d6, d1, d2), (4, 3, 2, 1), v, (d3, d4, d5, d6), (2, 1, 4, 3),
                         (2, 1, 4, 3))
    want = np.einsum("cdab,efcd->efab", t.reshape(d5, d6, d1, d2).astype(np.int64),
                     v.reshape(d3, d4, d5, d6).astype(np.int64)).reshape(-1)
    assert np.array_equal(got, want.astype(np.float64))


@pytest.mark.parametrize("seed", range(4))
def test_contract_chain_matches_einsum(seed):
    """Random perms of both operands and of the result, every factor case."""
    rng = np.random.default_rng(seed)
    pa = tuple(int(x) + 1 for x in rng.permutation(4))
    pb = tuple(int(x) + 1 for x in rng.permutation(4))
    pc = tuple(int(x) + 1 for x in rng.permutation(4))
    sa = list(rng.integers(2, 6, 4))
    sb = list(rng.integers(2, 6, 2)) + sa[2:]
    # raw dims whose permutation gives the sorted dims
    da = [0] * 4
    db = [0] * 4
    for q in range(4):
        da[pa[q] - 1] = int(sa[q])
        db[pb[q] - 1] = int(sb[q])
    a = rng.uniform(-1, 1, int(np.prod(da)))
    b = rng.uniform(-1, 1, int(np.prod(db)))
    a_s = a.reshape(da).transpose([p - 1 for p in pa]).reshape(sa[0] * sa[1], -1)
    b_s = b.reshape(db).transpose([p - 1 for p in pb]).reshape(sb[0] * sb[1], -1)
    c_sort = (b_s @ a_s.T).reshape(sb[0], sb[1], sa[0], sa[1])
    c_ref = c_sort.transpose([p - 1 for p in pc]).reshape(-1)
    for f, g in ((1.0, 0.0), (-0.5, 1.0), (0.3, 2.0)):
        y = rng.uniform(-1, 1, c_ref.size)
        got = O.contract_4x4(a, da, pa, b, db, pb, pc, alpha=0.75, factor=f, acc_factor=g,
                             out=y.copy())
        want = g * y + f * 0.75 * c_ref
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12)


def test_contract_entry_validates_arguments_on_host():
    """The C ABI checks shapes, permutations and the mode before touching
    any memory or the GPU (no CUDA device needed)."""
    import ctypes

    from spaghetty_gb300._lib import int_array, lib
    L = lib()
    d4 = int_array((4, 4, 4, 4))
    ok = int_array((1, 2, 3, 4))
    buf = np.zeros(256)
    p = ctypes.c_void_p(buf.ctypes.data)

    def call(dims_b=d4, perm_a=ok, mode=0, a=p):
        return L.spaghetty_contract_4x4(a, d4, perm_a, p, dims_b, ok, p, ok, 1.0, 1.0, 0.0, mode,
                                        None)
    assert call(mode=5) == 9                                   # SPAGHETTY_ERR_CONFIG
    assert call(perm_a=int_array((1, 2, 2, 4))) == 2           # SPAGHETTY_ERR_PERM
    assert call(dims_b=int_array((4, 4, 3, 4))) == 3           # contracted dims differ
    assert call(dims_b=int_array((4, 0, 4, 4))) == 3           # a zero extent
    assert call(a=None) == 5                                   # SPAGHETTY_ERR_NULL
    assert L.spaghetty_contract_last_error() == 5
    big = int_array((1 << 16, 1 << 16, 1, 1))
    assert L.spaghetty_contract_4x4(p, big, ok, p, big, ok, p, ok, 1.0, 1.0, 0.0, 0, None) == 4


def test_ccsd_t2_8_checks_sizes_on_host():
    import ctypes

    from spaghetty_gb300._lib import lib
    ir = lambda v: ctypes.byref(ctypes.c_int(v))   # noqa: E731
    buf = np.zeros(16)
    p = ctypes.c_void_p(buf.ctypes.data)
    # dims 2 each: every tensor holds 16 elements; size_c one short
    rc = lib().ccsd_t2_8_status(p, ir(16), p, ir(16), p, ir(15), *[ir(2)] * 6)
    assert rc == 3
    rc = lib().ccsd_t2_8_status(p, ir(16), p, ir(16), p, ir(16), *[ir(2)] * 5, ir(0))
    assert rc == 3


def _verify(da, pa, db, pb, pc):
    import ctypes

    from spaghetty_gb300._lib import int_array, lib
    st = (ctypes.c_int64 * 4)()
    rc = lib().spaghetty_contract_verify(int_array(da), int_array(pa), int_array(db),
                                         int_array(pb), int_array(pc), st)
    return rc, list(st)


def test_contract_verify_replays_kernel_addresses():
    """spaghetty_contract_verify replays the kernel's own index arithmetic on
    the CPU (operand reads, tile walk, result writes under every thread
    shape) for the skeleton's shapes and 300 random problems."""
    for d in [(16,) * 6, (3, 5, 7, 2, 6, 5), (17, 2, 9, 4, 1, 33), (18, 18, 17, 18, 3, 5),
              (1, 1, 1, 1, 1, 1)]:
        d1, d2, d3, d4, d5, d6 = d
        rc, st = _verify((d5, d6, d1, d2), (4, 3, 2, 1), (d3, d4, d5, d6), (2, 1, 4, 3), (2, 1, 4, 3))
        assert rc == 0 and st[:3] == [d1 * d2, d3 * d4, d5 * d6], (d, rc, st)
    rng = np.random.default_rng(77)
    for _ in range(300):
        pa = tuple(int(x) + 1 for x in rng.permutation(4))
        pb = tuple(int(x) + 1 for x in rng.permutation(4))
        pc = tuple(int(x) + 1 for x in rng.permutation(4))
        sa = [int(x) for x in rng.integers(1, 40, 4)]
        sb = [int(x) for x in rng.integers(1, 40, 2)] + sa[2:]
        da, db = [0] * 4, [0] * 4
        for q in range(4):
            da[pa[q] - 1] = sa[q]
            db[pb[q] - 1] = sb[q]
        rc, st = _verify(da, pa, db, pb, pc)
        assert rc == 0, (da, pa, db, pb, pc, rc)
        assert st[3] == -(-st[0] // 16) * -(-st[1] // 16)


def test_contract_verify_refuses_bad_shapes():
    assert _verify((4, 4, 4, 4), (1, 2, 3, 4), (4, 4, 5, 4), (1, 2, 3, 4), (1, 2, 3, 4))[0] == 3
    assert _verify((4, 4, 4, 4), (1, 2, 3, 3), (4, 4, 4, 4), (1, 2, 3, 4), (1, 2, 3, 4))[0] == 2
    # 2^29 elements in a: beyond the replay's limit (13); 2^60 result tiles: overflow (4)
    assert _verify((1 << 15, 1 << 14, 1, 1), (1, 2, 3, 4), (4, 4, 1, 1), (1, 2, 3, 4),
                   (1, 2, 3, 4))[0] == 13
    assert _verify((1 << 15,) * 2 + (1, 1), (1, 2, 3, 4), (1 << 15,) * 2 + (1, 1), (1, 2, 3, 4),
                   (1, 2, 3, 4))[0] == 4


def test_python_wrappers_check_buffer_sizes():
    """The C ABI cannot see buffer sizes; the Python wrappers check them
    against the dims before any call (no GPU needed: they raise first)."""
    import torch

    from spaghetty_gb300.contract import ccsd_t2_8, contract_4x4
    with pytest.raises(ValueError):
        ccsd_t2_8(np.zeros(15), np.zeros(16), np.zeros(16), (2,) * 6)
    with pytest.raises(ValueError):
        ccsd_t2_8(np.zeros(16), np.zeros(16), np.zeros(8), (2,) * 6)
    with pytest.raises(ValueError):   # contracted dims differ
        contract_4x4(torch.zeros(16, dtype=torch.float64), (2, 2, 2, 2), (1, 2, 3, 4),
                     torch.zeros(24, dtype=torch.float64), (2, 2, 3, 2), (1, 2, 3, 4),
                     torch.zeros(16, dtype=torch.float64), (1, 2, 3, 4))


def test_ccsd_t2_8_wrapper_checks_dtype_and_layout():
    """The drop-in reads 8 bytes per element from each buffer's start: the
    wrapper refuses other dtypes and strided arrays before any call."""
    import torch

    from spaghetty_gb300.contract import ccsd_t2_8
    with pytest.raises(TypeError):
        ccsd_t2_8(np.zeros(16, dtype=np.float32), np.zeros(16), np.zeros(16), (2,) * 6)
    with pytest.raises(TypeError):
        ccsd_t2_8(np.zeros(16), np.zeros(32)[::2], np.zeros(16), (2,) * 6)
    with pytest.raises(TypeError):
        ccsd_t2_8(np.zeros(16), np.zeros(16), torch.zeros(16, dtype=torch.float32), (2,) * 6)
    with pytest.raises(TypeError):
        ccsd_t2_8(np.zeros(16), np.zeros(16), torch.zeros(32, dtype=torch.float64)[::2], (2,) * 6)
