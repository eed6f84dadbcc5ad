"""GPU parity: the CUDA kernels, called through the C ABI, against the
reference (golden digests made by the reference's own nests) and the oracle,
bit for bit.  Shapes are the sort4/sort6 configurations and the edge cases
the reference's tester covers (trunk/generator2.py:446-629: every
permutation, factors 1 and 37, the init_4d_array fixture), plus odd
extents, unit dims, misaligned buffers and guard bands.  The full-size
configurations (100^4, 16^6, 20^6, the non-cubic rank-6 shape, the batched
mix) are checked in test_fullsize_gpu.py."""
import ctypes
import itertools
import random

import numpy as np
import pytest

from oracle import oracle as O
from spaghetty_gb300 import sort_generic
from spaghetty_gb300._lib import int_array, lib
from spaghetty_gb300.workloads import TRIPLES_SORT6
from tests._util import (bits_equal, call_dropin, first_mismatch, golden, golden_inputs,
                         parse_key)

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def dev(a, cuda):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(cuda)


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def gpu_sort(u, dims, perm, f, g, y0, cuda, via="dropin"):
    """Run one sort on the GPU through the C ABI; returns the output (numpy)."""
    du = dev(u, cuda)
    ds = dev(y0, cuda) if g else torch.zeros(du.numel(), dtype=torch.float64, device=cuda)
    torch.cuda.synchronize()
    if via == "dropin" and g in (0.0, 1.0) and len(dims) in (2, 4, 6, 8):
        name = "tce_sort%s_%d" % ("acc" if g else "", len(dims))
        call_dropin(name, du.data_ptr(), ds.data_ptr(), dims, perm, f)
        assert lib().spaghetty_last_error() == 0
    else:
        sort_generic(du, ds, dims, perm, f, g)
    return host(ds)


def check(got, want, what):
    if not bits_equal(got, want):
        pytest.fail("%s: mismatch %s" % (what, first_mismatch(got, want)))


# ---------------------------------------------------------------------------
def test_golden_digests_all_perms(cuda):
    """All 4032 golden cases (24 rank-4 and 720 rank-6 permutations, sort and
    sortacc, factors 1, -1, 37, +-0.5, integer fixture) reproduce the
    reference nests' output digests."""
    bad = []
    for key, digest in golden().items():
        dims, inp, perm, f, g = parse_key(key)
        u, s0 = golden_inputs(dims, inp)
        out = gpu_sort(u, dims, perm, f, g, s0, cuda)
        if O.digest(out)[:16] != digest:
            bad.append(key)
    assert not bad, bad[:10]


@pytest.mark.parametrize("acc", [False, True])
def test_sort4_plain_30(cuda, acc):
    """The plain 30^4 workload, b(i,j,k,l) = f*a(l,k,j,i) with f = -0.5, for every perm."""
    dims = (30, 30, 30, 30)
    n = 30 ** 4
    u = O.seeded_uniform(n, 1)
    y = O.seeded_uniform(n, 2)
    for perm in itertools.permutations((1, 2, 3, 4)):
        want = O.np_sort(u, dims, perm, -0.5, 1.0 if acc else 0.0, out=y)
        got = gpu_sort(u, dims, perm, -0.5, 1.0 if acc else 0.0, y, cuda)
        check(got, want, ("sort4", perm, acc))
    # and against the scalar C restatement of old_sort_4 for the headline perm
    want = O.old_sort(u, dims, (4, 3, 2, 1), -0.5, out=(y.copy() if acc else None), acc=acc)
    got = gpu_sort(u, dims, (4, 3, 2, 1), -0.5, 1.0 if acc else 0.0, y, cuda)
    check(got, want, "old_sort_4 4321")


@pytest.mark.parametrize("dims", [(20, 20, 20, 20), (50, 50, 50, 50), (17, 29, 64, 100)])
def test_sort4_sweep_sizes(cuda, dims):
    n = int(np.prod(dims))
    u = O.seeded_uniform(n, 3)
    y = O.seeded_uniform(n, 4)
    for perm in itertools.permutations((1, 2, 3, 4)):
        for f in (1.0, -1.0, 0.5):
            for g in (0.0, 1.0):
                want = O.np_sort(u, dims, perm, f, g, out=y)
                got = gpu_sort(u, dims, perm, f, g, y, cuda)
                check(got, want, (dims, perm, f, g))


def test_sort6_all_perms_10(cuda):
    dims = (10,) * 6
    n = 10 ** 6
    u = O.seeded_uniform(n, 5)
    y = O.seeded_uniform(n, 6)
    for i, perm in enumerate(itertools.permutations(range(1, 7))):
        g = float(i % 2)
        want = O.np_sort(u, dims, perm, -0.5, g, out=y)
        got = gpu_sort(u, dims, perm, -0.5, g, y, cuda)
        check(got, want, ("sort6 10^6", perm, g))


def test_odd_extents_and_unit_dims(cuda):
    rnd = random.Random(5)
    ext = [1, 2, 3, 5, 7, 31, 33]
    for it in range(120):
        r = rnd.choice([2, 3, 4, 5, 6, 7, 8])
        dims = tuple(rnd.choice(ext) for _ in range(r))
        if np.prod(dims) > 2_000_000:
            continue
        perm = list(range(1, r + 1))
        rnd.shuffle(perm)
        n = int(np.prod(dims))
        u = O.fixture_values(n, it)
        y = O.fixture_values(n, 500 + it)
        f = rnd.choice([1.0, -1.0, 0.3, 37.0])
        g = rnd.choice([0.0, 1.0, -2.5])
        want = O.np_sort(u, dims, perm, f, g, out=y)
        got = gpu_sort(u, dims, perm, f, g, y, cuda, via="generic")
        check(got, want, (dims, perm, f, g))


def test_rank2_rank8_dropins(cuda):
    for dims, perm in [((33, 65), (2, 1)), ((3, 2, 4, 3, 2, 5, 2, 3), (8, 1, 7, 2, 6, 3, 5, 4))]:
        n = int(np.prod(dims))
        u = O.fixture_values(n, 40)
        y = O.fixture_values(n, 41)
        for g in (0.0, 1.0):
            want = O.old_sort(u, dims, perm, 0.25, out=(y.copy() if g else None), acc=bool(g))
            got = gpu_sort(u, dims, perm, 0.25, g, y, cuda)
            check(got, want, (dims, perm, g))


def test_guard_bands_and_misaligned_buffers(cuda):
    """Outputs written exactly in place: canaries around the output stay
    untouched, including buffers offset by one double (no 16-byte alignment)."""
    G = 37
    canary = -12345.678
    for dims, perm in [((30, 30, 30, 30), (1, 2, 3, 4)), ((30, 30, 30, 30), (4, 3, 2, 1)),
                       ((17, 29, 64, 10), (2, 1, 3, 4)), ((7, 3, 5), (3, 1, 2))]:
        n = int(np.prod(dims))
        for off in (0, 1):
            u = O.fixture_values(n, 60)
            y = O.fixture_values(n, 61)
            bu = torch.full((n + 2 * G,), canary, dtype=torch.float64, device=cuda)
            bs = torch.full((n + 2 * G,), canary, dtype=torch.float64, device=cuda)
            vu = bu[G + off:G + off + n]
            vs = bs[G + off:G + off + n]
            vu.copy_(torch.from_numpy(u))
            vs.copy_(torch.from_numpy(y))
            for g in (0.0, 1.0):
                vs.copy_(torch.from_numpy(y))
                sort_generic(vu, vs, dims, perm, -0.5, g)
                got = host(vs)
                check(got, O.np_sort(u, dims, perm, -0.5, g, out=y), (dims, perm, off, g))
                b = host(bs)
                assert np.all(b[:G + off] == canary) and np.all(b[G + off + n:] == canary)


def test_host_buffers_are_staged(cuda):
    """The drop-ins accept host pointers (pageable numpy and pinned torch)."""
    dims = (17, 29, 64, 10)
    n = int(np.prod(dims))
    u = O.fixture_values(n, 70)
    y = O.fixture_values(n, 71)
    for perm in [(4, 3, 2, 1), (1, 2, 3, 4), (2, 1, 3, 4)]:
        s = np.zeros(n)
        call_dropin("tce_sort_4", u.ctypes.data, s.ctypes.data, dims, perm, -0.5)
        assert lib().spaghetty_last_error() == 0
        check(s, O.np_sort(u, dims, perm, -0.5), ("host sort", perm))
        s = y.copy()
        call_dropin("tce_sortacc_4", u.ctypes.data, s.ctypes.data, dims, perm, 37.0)
        check(s, O.np_sort(u, dims, perm, 37.0, 1.0, out=y), ("host sortacc", perm))
        pu = torch.from_numpy(u).pin_memory()
        ps = torch.from_numpy(y).pin_memory()
        call_dropin("tce_sortacc_4", pu.data_ptr(), ps.data_ptr(), dims, perm, 0.5)
        check(ps.numpy(), O.np_sort(u, dims, perm, 0.5, 1.0, out=y), ("pinned", perm))
        # pinned buffers moved in slabs through the copy/sort/copy pipeline
        assert lib().spaghetty_set_option(2, 1) == 0
        try:
            for f, g in ((-0.5, 0.0), (37.0, 1.0)):
                ps = torch.from_numpy(y).pin_memory()
                call_dropin("tce_sortacc_4" if g else "tce_sort_4", pu.data_ptr(), ps.data_ptr(),
                            dims, perm, f)
                assert lib().spaghetty_last_error() == 0
                check(ps.numpy(), O.np_sort(u, dims, perm, f, g, out=y), ("pipelined", perm, g))
        finally:
            lib().spaghetty_set_option(2, 0)
        # pinned buffers staged through device copies instead of used in place
        assert lib().spaghetty_set_option(1, 0) == 0
        try:
            ps = torch.from_numpy(y).pin_memory()
            call_dropin("tce_sortacc_4", pu.data_ptr(), ps.data_ptr(), dims, perm, -1.0)
            check(ps.numpy(), O.np_sort(u, dims, perm, -1.0, 1.0, out=y), ("pinned staged", perm))
        finally:
            lib().spaghetty_set_option(1, 1)
        # mixed: device input, host output (pageable and pinned)
        du = dev(u, cuda)
        s = np.zeros(n)
        call_dropin("tce_sort_4", du.data_ptr(), s.ctypes.data, dims, perm, 1.0)
        check(s, O.np_sort(u, dims, perm, 1.0), ("mixed", perm))
        ps = torch.zeros(n, dtype=torch.float64).pin_memory()
        call_dropin("tce_sort_4", du.data_ptr(), ps.data_ptr(), dims, perm, 0.5)
        check(ps.numpy(), O.np_sort(u, dims, perm, 0.5), ("mixed pinned", perm))


def test_async_on_side_stream(cuda):
    dims = (30, 30, 30, 30)
    n = 30 ** 4
    u = O.seeded_uniform(n, 80)
    du = dev(u, cuda)
    ds = torch.empty_like(du)
    st = torch.cuda.Stream()
    torch.cuda.synchronize()
    with torch.cuda.stream(st):
        rc = lib().spaghetty_sort_async(4, ctypes.c_void_p(du.data_ptr()),
                                        ctypes.c_void_p(ds.data_ptr()), int_array(dims),
                                        int_array((3, 1, 4, 2)), -0.5, 0.0,
                                        ctypes.c_void_p(st.cuda_stream))
        assert rc == 0
    st.synchronize()
    check(ds.cpu().numpy(), O.np_sort(u, dims, (3, 1, 4, 2), -0.5), "side stream")


def test_status_form_bad_perm_leaves_output(cuda):
    from tests._util import call_status
    du = torch.zeros(16, dtype=torch.float64, device=cuda)
    ds = torch.full((16,), 3.0, dtype=torch.float64, device=cuda)
    rc = call_status("tce_sort_4_status", du.data_ptr(), ds.data_ptr(), (2, 2, 2, 2),
                     (2, 2, 3, 4), 1.0)
    assert rc == 2
    assert torch.all(ds == 3.0)


def test_i8_shims(cuda):
    """-i8 NWChem builds pass 8-byte integers; the _i8 drop-ins narrow them."""
    import ctypes
    dims = (7, 30, 9, 16)
    n = int(np.prod(dims))
    u = O.fixture_values(n, 90)
    y = O.fixture_values(n, 91)
    du = dev(u, cuda)
    L = lib()
    r8 = lambda v: ctypes.byref(ctypes.c_int64(v))  # noqa: E731
    for name, g in (("tce_sort_4_i8", 0.0), ("tce_sortacc_4_i8_", 1.0)):
        ds = dev(y, cuda)
        torch.cuda.synchronize()
        getattr(L, name)(ctypes.c_void_p(du.data_ptr()), ctypes.c_void_p(ds.data_ptr()),
                         *[r8(d) for d in dims], *[r8(p) for p in (3, 1, 4, 2)],
                         ctypes.byref(ctypes.c_double(-0.5)))
        assert L.spaghetty_last_error() == 0
        check(host(ds), O.np_sort(u, dims, (3, 1, 4, 2), -0.5, g, out=y), name)
    # out-of-range 8-byte value: rejected, output untouched
    ds = dev(y, cuda)
    L.tce_sort_4_i8(ctypes.c_void_p(du.data_ptr()), ctypes.c_void_p(ds.data_ptr()),
                    r8(1 << 40), r8(30), r8(9), r8(16), r8(3), r8(1), r8(4), r8(2),
                    ctypes.byref(ctypes.c_double(1.0)))
    assert L.spaghetty_last_error() == 3
    check(host(ds), y, "untouched")


@pytest.mark.parametrize("dims", [(6, 20, 9, 34), (10, 12, 14, 16)])
def test_every_forced_variant_rank4(cuda, dims):
    """Every (box, block shape, pipeline) the tuner can force, TMA-staged
    kernels with 2/3/4/6 load stages and the same-order layout included,
    gives the oracle's bits for every perm, sort and sortacc."""
    from spaghetty_gb300.autotune import candidates, clear
    L = lib()
    n = int(np.prod(dims))
    u = O.seeded_uniform(n, 21)
    y = O.seeded_uniform(n, 22)
    du, dy = dev(u, cuda), dev(y, cuda)
    ran = {"tma": 0, "other": 0}
    try:
        for perm in itertools.permutations((1, 2, 3, 4)):
            for op, f in ((0, -0.5), (1, 0.75)):
                g = float(op)
                want = dev(O.np_sort(u, dims, perm, f, g, out=y), cuda)
                _, cands = candidates(dims, perm, op)
                for box, nt, ept, st in cands:
                    if L.spaghetty_tune_set(4, int_array(dims), int_array(perm), op,
                                            int_array(box), nt, ept, st) != 0:
                        continue
                    s = dy.clone()
                    sort_generic(du, s, dims, perm, f, g)
                    torch.cuda.synchronize()
                    if not torch.equal(s, want):
                        pytest.fail("variant %s: mismatch %s" % (
                            (dims, perm, op, box, nt, ept, st),
                            first_mismatch(s.cpu().numpy(), want.cpu().numpy())))
                    ran["tma" if st >= 12 else "other"] += 1
                clear()
    finally:
        clear()
    assert ran["tma"] > 0 and ran["other"] > 0
    assert lib().spaghetty_device_status() == 0


def test_async_form_checks_memory_and_binds_device(cuda):
    """The asynchronous entry refuses host memory (no launch on a pointer
    the GPU cannot read) and works from a fresh host thread that has no
    CUDA context yet (the tensor-map encoding needs one)."""
    import threading
    L = lib()
    dims = (24, 24, 24, 24)
    n = int(np.prod(dims))
    uh = O.seeded_uniform(n, 41)
    sh = np.zeros(n)
    rc = L.spaghetty_sort_async(4, uh.ctypes.data_as(ctypes.c_void_p), sh.ctypes.data_as(ctypes.c_void_p),
                                int_array(dims), int_array((4, 3, 2, 1)), 0.5, 0.0, None)
    assert rc == 8 and not sh.any()      # SPAGHETTY_ERR_MEMSPACE
    du = dev(uh, cuda)
    want = O.np_sort(uh, dims, (4, 3, 2, 1), 0.75, 0.0)
    out = {}

    s = torch.empty(n, dtype=torch.float64, device=cuda)
    torch.cuda.synchronize()

    def worker():   # only the library touches CUDA on this thread
        out["rc"] = L.spaghetty_sort_async(4, ctypes.c_void_p(du.data_ptr()), ctypes.c_void_p(s.data_ptr()),
                                           int_array(dims), int_array((4, 3, 2, 1)), 0.75, 0.0, None)

    t = threading.Thread(target=worker)
    t.start()
    t.join()
    assert out["rc"] == 0, L.spaghetty_last_cuda_error()
    check(host(s), want, "async sort from a fresh thread")


def test_forced_tma_variants_rank6(cuda):
    """Forced TMA-staged variants of rank-6 sorts (six folded dims merged
    into five map dims) give the oracle's bits."""
    from spaghetty_gb300.autotune import candidates, clear
    L = lib()
    dims = (4, 6, 4, 6, 4, 6)
    n = int(np.prod(dims))
    u = O.seeded_uniform(n, 51)
    y = O.seeded_uniform(n, 52)
    du, dy = dev(u, cuda), dev(y, cuda)
    rnd = random.Random(13)
    perms = list(TRIPLES_SORT6[:6]) + [tuple(rnd.sample(range(1, 7), 6)) for _ in range(6)]
    ran = 0
    try:
        for perm in perms:
            for op, f in ((0, 0.5), (1, -1.0)):
                want = dev(O.np_sort(u, dims, perm, f, float(op), out=y), cuda)
                _, cands = candidates(dims, perm, op)
                for box, nt, ept, st in cands:
                    if st < 12 or L.spaghetty_tune_set(6, int_array(dims), int_array(perm), op,
                                                       int_array(box), nt, ept, st) != 0:
                        continue
                    s = dy.clone()
                    sort_generic(du, s, dims, perm, f, float(op))
                    torch.cuda.synchronize()
                    assert torch.equal(s, want), (perm, op, box, nt, ept, st)
                    ran += 1
                clear()
    finally:
        clear()
    assert ran > 0


def test_pipelined_host_slabs(cuda):
    """Pinned host buffers moved in slabs through the copy/sort/copy
    pipeline (three streams), against the oracle, sort and sortacc: slabs of
    the output's slowest index with pitched uploads (2413), of the input's
    slowest index with pitched downloads (3142), and a permutation that no
    slab index serves, which falls back to the kernels working on the pinned
    buffers in place (4321)."""
    dims = (64, 96, 80, 48)
    n = int(np.prod(dims))
    u = O.fixture_values(n, 72)
    y = O.fixture_values(n, 73)
    pu = torch.from_numpy(u).pin_memory()
    assert lib().spaghetty_set_option(2, 1) == 0
    try:
        for perm in [(4, 3, 2, 1), (2, 4, 1, 3), (3, 1, 4, 2)]:
            for f, g in ((-0.5, 0.0), (0.75, 1.0)):
                ps = torch.from_numpy(y).pin_memory()
                call_dropin("tce_sortacc_4" if g else "tce_sort_4", pu.data_ptr(), ps.data_ptr(),
                            dims, perm, f)
                assert lib().spaghetty_last_error() == 0
                check(ps.numpy(), O.np_sort(u, dims, perm, f, g, out=y), ("pipelined slabs", perm, g))
    finally:
        lib().spaghetty_set_option(2, 0)
