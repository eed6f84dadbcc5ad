"""The fused contraction (sort -> DGEMM('T','N') -> sort in one kernel) on the
GPU: bit-identical to the oracle's chain of tce_sort_4 calls around the
skeleton's loop_dgemm case 3 (branches/old/python/macaroni/
ccsd_t2_8_skeleton.F:174-184, :214-292) in exact mode, within rounding of
it in fma mode, through the C ABI."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from spaghetty_gb300._lib import int_array, lib
from tests._util import first_mismatch

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).reshape(-1).view(np.uint64)


def t2_8_oracle(t, v, d):
    d1, d2, d3, d4, d5, d6 = d
    return O.contract_4x4(t, (d5, d6, d1, d2), (4, 3, 2, 1), v, (d3, d4, d5, d6), (2, 1, 4, 3),
                          (2, 1, 4, 3))


@pytest.mark.parametrize("d", [(16, 16, 16, 16, 16, 16), (3, 5, 7, 2, 6, 5), (5, 7, 3, 9, 11, 3),
                               (17, 2, 9, 4, 1, 33), (1, 1, 1, 1, 1, 1), (18, 18, 17, 18, 3, 5),
                               (24, 24, 24, 24, 8, 9)])
def test_ccsd_t2_8_host_buffers_bits(cuda, d):
    """The Fortran drop-in on host arrays (staged through the device), the
    skeleton's shapes with tiles that are not multiples of the kernel's
    16 x 16 x 32 blocking; on 152 SMs the tile counts (up to 256, 420 and
    1296) select each of the three thread shapes (256, 128 and 64 threads
    per tile)."""
    from spaghetty_gb300.contract import ccsd_t2_8
    d1, d2, d3, d4, d5, d6 = d
    rng = np.random.default_rng(sum(d))
    t = rng.uniform(-1, 1, d5 * d6 * d1 * d2)
    v = rng.uniform(-1, 1, d3 * d4 * d5 * d6)
    c = np.full(d1 * d2 * d3 * d4, np.nan)
    ccsd_t2_8(t, v, c, d)
    want = t2_8_oracle(t, v, d)
    assert np.array_equal(bits(c), bits(want)), first_mismatch(c, want)


def test_ccsd_t2_8_device_buffers_and_fortran_alias(cuda):
    d = (6, 7, 8, 5, 9, 4)
    d1, d2, d3, d4, d5, d6 = d
    rng = np.random.default_rng(5)
    t = rng.uniform(-1, 1, d5 * d6 * d1 * d2)
    v = rng.uniform(-1, 1, d3 * d4 * d5 * d6)
    want = t2_8_oracle(t, v, d)
    dt, dv = torch.from_numpy(t).to(cuda), torch.from_numpy(v).to(cuda)
    dc = torch.zeros(d1 * d2 * d3 * d4, dtype=torch.float64, device=cuda)
    ir = lambda x: ctypes.byref(ctypes.c_int(int(x)))   # noqa: E731
    lib().ccsd_t2_8_(ctypes.c_void_p(dt.data_ptr()), ir(t.size), ctypes.c_void_p(dv.data_ptr()),
                     ir(v.size), ctypes.c_void_p(dc.data_ptr()), ir(dc.numel()), *map(ir, d))
    torch.cuda.synchronize()
    assert np.array_equal(bits(dc.cpu().numpy()), bits(want))


def random_case(rng):
    pa = tuple(int(x) + 1 for x in rng.permutation(4))
    pb = tuple(int(x) + 1 for x in rng.permutation(4))
    pc = tuple(int(x) + 1 for x in rng.permutation(4))
    sa = [int(x) for x in rng.integers(1, 12, 4)]
    sb = [int(x) for x in rng.integers(1, 12, 2)] + sa[2:]
    da, db = [0] * 4, [0] * 4
    for q in range(4):
        da[pa[q] - 1] = sa[q]
        db[pb[q] - 1] = sb[q]
    return da, pa, db, pb, pc


@pytest.mark.parametrize("seed", range(6))
def test_contract_4x4_random_perms_every_factor_bits(cuda, seed):
    """Random operand and result permutations, alpha != 1, and every factor
    class of the result sort (sort and sortacc, 1 / -1 / 2^k / any, and the
    general g): the oracle's bits."""
    from spaghetty_gb300.contract import contract_4x4, contract_shapes
    rng = np.random.default_rng(100 + seed)
    da, pa, db, pb, pc = random_case(rng)
    a = rng.uniform(-1, 1, int(np.prod(da)))
    b = rng.uniform(-1, 1, int(np.prod(db)))
    _, _, _, dc = contract_shapes(da, pa, db, pb, pc)
    nc = int(np.prod(dc))
    ga, gb = torch.from_numpy(a).to(cuda), torch.from_numpy(b).to(cuda)
    for alpha in (1.0, -0.75):
        for f, g in ((1.0, 0.0), (-1.0, 0.0), (0.5, 0.0), (0.3, 0.0), (1.0, 1.0), (-1.0, 1.0),
                     (0.25, 1.0), (-0.7, 1.0), (0.6, 2.5)):
            y = rng.uniform(-1, 1, nc)
            want = O.contract_4x4(a, da, pa, b, db, pb, pc, alpha, f, g, out=y.copy())
            gc = torch.from_numpy(y).to(cuda)
            contract_4x4(ga, da, pa, gb, db, pb, gc, pc, alpha, f, g)
            got = gc.cpu().numpy()
            assert np.array_equal(bits(got), bits(want)), (da, pa, db, pb, pc, alpha, f, g,
                                                           first_mismatch(got, want))


@pytest.mark.parametrize("mode", ["fma", "mma"])
def test_contract_fma_mode_within_rounding(cuda, mode):
    """fma mode (fused multiply-adds) and mma mode (FP64 matrix
    instructions): the same sums within K roundings of the exact mode's
    result (relative to the sum of |products|)."""
    from spaghetty_gb300.contract import contract_4x4, contract_shapes
    rng = np.random.default_rng(7)
    # sorted operands (20, 24 | 16, 18) and (20, 22 | 16, 18): M 480, N 440, K 288
    da, pa = (24, 16, 20, 18), (3, 1, 2, 4)
    db, pb = (18, 16, 22, 20), (4, 3, 2, 1)
    pc = (2, 4, 1, 3)
    M, N, K, dc = contract_shapes(da, pa, db, pb, pc)
    a = rng.uniform(-1, 1, int(np.prod(da)))
    b = rng.uniform(-1, 1, int(np.prod(db)))
    want = O.contract_4x4(a, da, pa, b, db, pb, pc)
    bound = O.contract_4x4(np.abs(a), da, pa, np.abs(b), db, pb, pc)
    ga, gb = torch.from_numpy(a).to(cuda), torch.from_numpy(b).to(cuda)
    gc = torch.empty(int(np.prod(dc)), dtype=torch.float64, device=cuda)
    contract_4x4(ga, da, pa, gb, db, pb, gc, pc, mode=mode)
    got = gc.cpu().numpy()
    tol = 2 * K * np.finfo(np.float64).eps * bound
    assert np.all(np.abs(got - want) <= tol)
    assert not np.array_equal(got, want)   # the fused roundings do differ somewhere


def test_contract_integer_fill_both_modes_exact(cuda):
    """The skeleton's number_array fill (integer values, exact sums): every
    mode gives exactly the integer result."""
    from spaghetty_gb300.contract import contract_4x4
    d1, d2, d3, d4, d5, d6 = 8, 9, 4, 5, 6, 7
    t = np.arange(1, d5 * d6 * d1 * d2 + 1, dtype=np.float64)
    v = np.arange(1, d3 * d4 * d5 * d6 + 1, dtype=np.float64)
    want = t2_8_oracle(t, v, (d1, d2, d3, d4, d5, d6))
    gt, gv = torch.from_numpy(t).to(cuda), torch.from_numpy(v).to(cuda)
    for mode in ("exact", "fma", "mma"):
        gc = torch.empty(want.size, dtype=torch.float64, device=cuda)
        contract_4x4(gt, (d5, d6, d1, d2), (4, 3, 2, 1), gv, (d3, d4, d5, d6), (2, 1, 4, 3), gc,
                     (2, 1, 4, 3), mode=mode)
        assert np.array_equal(gc.cpu().numpy(), want), mode


def test_contract_argument_errors(cuda):
    L = lib()
    a = torch.zeros(4 * 4 * 4 * 4, dtype=torch.float64, device=cuda)
    b = torch.zeros(4 * 4 * 4 * 4, dtype=torch.float64, device=cuda)
    c = torch.zeros(4 * 4 * 4 * 4, dtype=torch.float64, device=cuda)
    p = lambda t: ctypes.c_void_p(t.data_ptr())   # noqa: E731
    d4 = int_array((4, 4, 4, 4))
    ok = int_array((1, 2, 3, 4))

    def call(a_, b_, c_, dims_b=d4, perm_a=ok, mode=0):
        return L.spaghetty_contract_4x4(a_, d4, perm_a, b_, dims_b, ok, c_, ok, 1.0, 1.0, 0.0,
                                        mode, None)
    assert call(p(a), p(b), p(c)) == 0
    assert call(p(a), p(b), p(c), dims_b=int_array((4, 4, 4, 5))) == 3    # contracted dims differ
    assert call(p(a), p(b), p(c), perm_a=int_array((1, 1, 3, 4))) == 2   # not a permutation
    assert call(p(a), p(b), p(a)) == 6                                    # result overlaps a
    assert call(p(a), p(b), p(c), mode=3) == 9                            # unknown mode
    host = np.zeros(256)
    assert call(p(a), p(b), ctypes.c_void_p(host.ctypes.data)) == 8       # host memory, async form
    assert L.spaghetty_contract_last_error() == 8
    torch.cuda.synchronize()


def test_unfused_chain_with_cublas_agrees(cuda):
    """The benchmark's unfused comparison (three sorts around torch.matmul,
    i.e. cuBLAS DGEMM) computes the same contraction, within rounding."""
    import spaghetty_gb300 as S
    from spaghetty_gb300.contract import contract_4x4
    d1, d2, d3, d4, d5, d6 = 5, 6, 7, 4, 9, 3
    M, N, K = d1 * d2, d3 * d4, d5 * d6
    rng = np.random.default_rng(31)
    t = torch.from_numpy(rng.uniform(-1, 1, d5 * d6 * d1 * d2)).to(cuda)
    v = torch.from_numpy(rng.uniform(-1, 1, d3 * d4 * d5 * d6)).to(cuda)
    a_s, b_s = torch.empty_like(t), torch.empty_like(v)
    c_s = torch.empty(M * N, dtype=torch.float64, device=cuda)
    c1, c2 = torch.empty_like(c_s), torch.empty_like(c_s)
    S.sort_generic(t, a_s, (d5, d6, d1, d2), (4, 3, 2, 1), 1.0, 0.0)
    S.sort_generic(v, b_s, (d3, d4, d5, d6), (2, 1, 4, 3), 1.0, 0.0)
    torch.matmul(b_s.view(N, K), a_s.view(M, K).t(), out=c_s.view(N, M))
    S.sort_generic(c_s, c1, (d4, d3, d2, d1), (2, 1, 4, 3), 1.0, 0.0)
    contract_4x4(t, (d5, d6, d1, d2), (4, 3, 2, 1), v, (d3, d4, d5, d6), (2, 1, 4, 3), c2,
                 (2, 1, 4, 3))
    torch.testing.assert_close(c1, c2, rtol=1e-12, atol=1e-12)
