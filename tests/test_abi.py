"""The C-ABI library on the CPU: it loads, exports every symbol the header
declares, and its host-side logic (validation, folding, planning, index
safety of every launch) is right.  No kernel is launched here."""
import ctypes
import itertools
import os
import random
import re

import numpy as np
import pytest

from spaghetty_gb300._lib import LIB_PATH, PROTOTYPES, int_array, lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                      "include", "spaghetty_gb300.h")


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*([a-z_][a-z0-9_]*)\s*\(",
                       text, flags=re.M)
    return sorted(set(names))


def test_library_is_in_tree_and_loads():
    assert os.path.exists(LIB_PATH)
    assert os.path.dirname(LIB_PATH).endswith("spaghetty_gb300")
    assert lib().spaghetty_version().startswith(b"spaghetty_gb300")


def test_exports_every_header_symbol():
    names = header_functions()
    assert "tce_sort_4" in names and "tce_sortacc_6_" in names and len(names) >= 29
    L = ctypes.CDLL(LIB_PATH)
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # and the Python binding declares a prototype for each of them
    assert set(names) <= set(PROTOTYPES), sorted(set(names) - set(PROTOTYPES))


def test_host_selftest():
    assert lib().spaghetty_selftest() == 0


def plan(dims, perm, op=0):
    from spaghetty_gb300 import plan as P
    return P(dims, perm, op)


def verify(dims, perm, op=0, sms=152):
    st = (ctypes.c_int64 * 4)()
    rc = lib().spaghetty_plan_verify(len(dims), int_array(dims), int_array(perm), op, sms, st)
    return rc, list(st)


@pytest.mark.parametrize("dims,perm,rank,kind", [
    ((30, 30, 30, 30), (1, 2, 3, 4), 1, "flat"),
    ((30, 30, 30, 30), (2, 1, 3, 4), 3, "direct"),
    ((30, 30, 30, 30), (3, 4, 1, 2), 2, "tiled"),
    ((30, 30, 30, 30), (4, 3, 2, 1), 4, "tiled"),
    ((16,) * 6, (1, 2, 3, 4, 5, 6), 1, "flat"),
    ((16,) * 6, (4, 5, 6, 1, 2, 3), 2, "tiled"),
    ((1, 7, 1, 9), (3, 1, 4, 2), 2, "tiled"),
    ((5, 1, 1, 1), (2, 3, 4, 1), 1, "flat"),
])
def test_folding(dims, perm, rank, kind):
    p = plan(dims, perm)
    # tiled and direct plans run on the TMA-staged kernel when its boxes
    # allow it (direct ones with the same-order layout); small transposes
    # (both stride-1 extents <= 32, product <= 128) on the warp-shuffle kernel
    assert p["rank"] == rank and (p["kind"] == kind or (kind in ("tiled", "direct") and p["kind"] == "tma")
                                  or (kind == "tiled" and p["kind"] == "warp"))
    assert int(np.prod(p["dims"])) == int(np.prod(dims))


def test_plan_invariants_all_rank4_rank6():
    cases = [((30,) * 4, p) for p in itertools.permutations((1, 2, 3, 4))]
    cases += [((100,) * 4, p) for p in itertools.permutations((1, 2, 3, 4))]
    cases += [((17, 29, 64, 100), p) for p in itertools.permutations((1, 2, 3, 4))]
    cases += [((16,) * 6, p) for p in itertools.permutations(range(1, 7))]
    cases += [((12, 20, 16, 20, 12, 16), p) for p in itertools.permutations(range(1, 7))]
    for (dims, perm), op in itertools.product(cases, (0, 1)):
        p = plan(dims, perm, op)
        if p["kind"] == "flat":
            continue
        vol = int(np.prod(p["box"]))
        assert vol <= p["threads"] * p["ept"] <= 4096, (dims, perm, p)
        assert all(1 <= b <= d for b, d in zip(p["box"], p["dims"]))
        # both sides get coalesced rows (at least 16 doubles, 128 bytes)
        # unless that side is shorter overall
        total = int(np.prod(p["dims"]))
        assert p["run_in"] >= min(16, total) and p["run_out"] >= min(16, total), (dims, perm, p)
        npartial = sum(1 for b, d in zip(p["box"], p["dims"]) if d % b)
        assert npartial <= 2
        # every plan's shared memory fits one CTA (227 KB opt-in)
        assert p["smem_bytes"] <= 232448, (dims, perm, p)


def test_launch_index_safety_rank4_all_perms():
    """Every launch the sort4 configs make is replayed on the host: reads and
    writes in bounds, each output written once from the right input."""
    for dims in [(3, 5, 7, 2), (1, 31, 33, 5), (30, 30, 30, 30), (17, 29, 64, 10),
                 (8, 8, 8, 8), (40, 8, 13, 37), (2, 1, 9, 4)]:
        for perm in itertools.permutations((1, 2, 3, 4)):
            for op in (0, 1):
                rc, st = verify(dims, perm, op)
                assert rc == 0, (dims, perm, op, rc)


def test_launch_index_safety_rank6_triples_and_random():
    from spaghetty_gb300.workloads import TRIPLES_SORT6
    for perm in TRIPLES_SORT6:
        for dims in [(6, 7, 5, 6, 8, 9), (10,) * 6]:
            rc, _ = verify(dims, perm, 1)
            assert rc == 0, (dims, perm)
    rnd = random.Random(3)
    for _ in range(200):
        r = rnd.choice([2, 3, 5, 6, 7, 8])
        dims = [rnd.randint(1, 40 if r <= 3 else 9) for _ in range(r)]
        if np.prod(dims) > 3e6:
            continue
        perm = list(range(1, r + 1))
        rnd.shuffle(perm)
        rc, _ = verify(dims, perm, rnd.randint(0, 2), rnd.choice([1, 8, 152]))
        assert rc == 0, (dims, perm)


@pytest.mark.parametrize("perm,code", [((1, 1, 2, 3), 2), ((0, 1, 2, 3), 2), ((1, 2, 3, 5), 2)])
def test_bad_permutation_status(perm, code):
    from tests._util import call_status
    u = np.zeros(16)
    s = np.zeros(16)
    rc = call_status("tce_sort_4_status", u.ctypes.data, s.ctypes.data, (2, 2, 2, 2), perm, 1.0)
    assert rc == code
    assert lib().spaghetty_last_error() == code


def test_negative_dim_and_empty():
    from tests._util import call_status
    u = np.zeros(4)
    s = np.zeros(4)
    assert call_status("tce_sort_4_status", u.ctypes.data, s.ctypes.data,
                       (2, -1, 2, 1), (1, 2, 3, 4), 1.0) == 3
    # a zero extent is an empty tensor: nothing to do, like the reference's
    # zero-trip loops
    assert call_status("tce_sort_4_status", u.ctypes.data, s.ctypes.data,
                       (2, 0, 2, 1), (4, 3, 2, 1), 1.0) == 0


def test_void_dropin_prints_reference_diagnostic(capfd):
    from tests._util import call_dropin
    u = np.zeros(16)
    s = np.full(16, 7.0)
    call_dropin("tce_sort_4", u.ctypes.data, s.ctypes.data, (2, 2, 2, 2), (1, 2, 2, 4), 1.0)
    err = capfd.readouterr().err
    assert "something is wrong" in err
    assert np.all(s == 7.0)  # output untouched
    assert lib().spaghetty_last_error() == 2


def test_alias_rejected():
    from tests._util import call_status
    buf = np.zeros(32)
    rc = call_status("tce_sort_4_status", buf.ctypes.data, buf.ctypes.data + 8 * 4,
                     (2, 2, 2, 2), (4, 3, 2, 1), 1.0)
    assert rc == 6


def test_tune_set_validation():
    L = lib()
    d = int_array((30, 30, 30, 30))
    p = int_array((4, 3, 2, 1))
    assert L.spaghetty_tune_set(4, d, p, 0, int_array((30, 2, 2, 30)), 128, 8, 3) == 9  # too small
    assert L.spaghetty_tune_set(4, d, p, 0, int_array((30, 2, 2, 31)), 512, 8, 3) == 9  # > extent
    assert L.spaghetty_tune_set(4, d, p, 0, int_array((30, 2, 2, 30)), 512, 8, 0) == 0
    assert plan((30, 30, 30, 30), (4, 3, 2, 1))["box"] == [30, 2, 2, 30]
    assert L.spaghetty_tune_set(4, d, p, 0, int_array((15, 1, 1, 15)), 256, 1, 0) == 0
    assert plan((30, 30, 30, 30), (4, 3, 2, 1))["box"] == [15, 1, 1, 15]
    assert verify((30, 30, 30, 30), (4, 3, 2, 1))[0] == 0
    assert L.spaghetty_tune_set(0, None, None, 0, None, 0, 0, 0) == 0   # clear
    assert plan((30, 30, 30, 30), (4, 3, 2, 1))["box"] != [15, 1, 1, 15]


def test_tma_candidates_replay_rank4():
    """Every TMA-staged candidate the tuner can force is replayed on the host.
    Perms that keep the stride-1 index get the same-order layout (identity
    permute step, output map listed in input order)."""
    from spaghetty_gb300.autotune import candidates, clear
    L = lib()
    same_order_seen = 0
    try:
        for dims in [(10, 12, 14, 16), (6, 20, 9, 34), (4, 6, 50, 40)]:
            for perm in itertools.permutations((1, 2, 3, 4)):
                for op in (0, 1):
                    _, cands = candidates(dims, perm, op)
                    for box, nt, ept, st in cands:
                        if st < 12:
                            continue
                        rc = L.spaghetty_tune_set(4, int_array(dims), int_array(perm), op,
                                                  int_array(box), nt, ept, st)
                        assert rc in (0, 9, 12), (dims, perm, box, rc)
                        if rc:
                            continue
                        p = plan(dims, perm, op)
                        assert p["kind"] == "tma" and p["stages"] == st - 10
                        assert p["smem_bytes"] <= 232448
                        vrc, _ = verify(dims, perm, op)
                        assert vrc == 0, (dims, perm, op, box, nt, ept, st)
                        if perm[-1] == 4:
                            same_order_seen += 1
                    clear()
    finally:
        clear()
    assert same_order_seen > 0


def test_batch_tune_set_validation():
    L = lib()
    assert L.spaghetty_batch_tune_set(4, 8, 16, 16, 32, 512) == 0
    assert L.spaghetty_batch_tune_set(4, 12, 20, 8, 8, 256) == 0      # overlapping bucket replaces
    assert L.spaghetty_batch_tune_set(4, 8, 16, 16, 32, 2048) == 9    # volume above 1024
    assert L.spaghetty_batch_tune_set(9, 8, 16, 16, 32, 512) == 9     # rank
    assert L.spaghetty_batch_tune_set(4, 16, 8, 16, 32, 512) == 9     # empty range
    assert L.spaghetty_batch_tune_set(4, 8, 16, 0, 32, 512) == 9      # run
    assert L.spaghetty_batch_tune_set(0, 0, 0, 0, 0, 0) == 0          # clear


def test_tma_candidates_replay_rank6():
    """Every TMA candidate the tuner can force for a sample of rank-6 perms
    (the merges of six folded dims into five map dims) replays correctly."""
    from spaghetty_gb300.autotune import candidates, clear
    from spaghetty_gb300.workloads import TRIPLES_SORT6
    L = lib()
    rnd = random.Random(11)
    perms = list(TRIPLES_SORT6[:6]) + [tuple(rnd.sample(range(1, 7), 6)) for _ in range(6)]
    tried = 0
    try:
        for dims in [(4, 6, 4, 6, 4, 6), (6, 4, 8, 2, 6, 4)]:
            for perm in perms:
                for op in (0, 1):
                    _, cands = candidates(dims, perm, op)
                    for box, nt, ept, st in cands:
                        if st < 12:
                            continue
                        rc = L.spaghetty_tune_set(6, int_array(dims), int_array(perm), op,
                                                  int_array(box), nt, ept, st)
                        if rc:
                            continue
                        vrc, _ = verify(dims, perm, op)
                        assert vrc == 0, (dims, perm, op, box, nt, ept, st)
                        tried += 1
                    clear()
    finally:
        clear()
    assert tried > 0


def test_batch_own_launch_options():
    """SPAGHETTY_OPT_BATCH_OWN_MIN takes element counts >= 0 (0: every sort
    stays on the persistent kernel's work list); SPAGHETTY_OPT_BATCH_OWN_KINDS
    takes 0 or 1.  Other values are rejected and leave the setting alone."""
    L = lib()
    own_min, own_kinds = 5, 6
    try:
        assert L.spaghetty_set_option(own_min, -1) == 9          # SPAGHETTY_ERR_CONFIG
        assert L.spaghetty_set_option(own_kinds, 2) == 9
        assert L.spaghetty_set_option(own_kinds, -1) == 9
        assert L.spaghetty_set_option(own_min, 0) == 0
        assert L.spaghetty_set_option(own_min, 1 << 20) == 0
        assert L.spaghetty_set_option(own_kinds, 1) == 0
        assert L.spaghetty_set_option(99, 0) == 9
    finally:
        L.spaghetty_set_option(own_min, 1 << 24)
        L.spaghetty_set_option(own_kinds, 0)


@pytest.mark.parametrize("name", ["spaghetty_sort_fused", "spaghetty_sortacc_fused"])
def test_fused_entry_validation(name):
    """The fused entries check their arguments before any launch: rank
    (1..6), term count (1..16), null arrays, permutations, and the memory
    space of the buffers (device memory only; host arrays are refused)."""
    fn = getattr(lib(), name)
    dbl = ctypes.c_double
    u = np.zeros(24)
    s = np.zeros(24)
    srcs = (ctypes.c_void_p * 2)(u.ctypes.data, u.ctypes.data)
    dims = int_array([2, 3, 4] * 2)
    perms = int_array([3, 2, 1, 1, 3, 2])
    fac = (dbl * 2)(1.0, -0.5)
    out = ctypes.c_void_p(s.ctypes.data)
    assert fn(0, 2, srcs, dims, perms, fac, out, None) == 1           # SPAGHETTY_ERR_RANK
    assert fn(7, 2, srcs, dims, perms, fac, out, None) == 1
    assert fn(3, 0, srcs, dims, perms, fac, out, None) == 9           # SPAGHETTY_ERR_CONFIG
    assert fn(3, 17, srcs, dims, perms, fac, out, None) == 9
    assert fn(3, 2, None, dims, perms, fac, out, None) == 5           # SPAGHETTY_ERR_NULL
    assert fn(3, 2, srcs, dims, int_array([3, 2, 4, 1, 3, 2]), fac, out, None) == 2   # ERR_PERM
    assert fn(3, 2, srcs, int_array([2, 0, 4] * 2), perms, fac, out, None) == 0       # empty
    assert fn(3, 2, srcs, dims, perms, fac, out, None) == 8           # host arrays: ERR_MEMSPACE
    assert np.all(s == 0.0)


C_CALLER = r"""
#include <stdio.h>
#include "spaghetty_gb300.h"
int main(void) {
    int dims[4] = {30, 30, 30, 30}, perm[4] = {4, 3, 2, 1}, bad[4] = {1, 1, 2, 3}, two = 2;
    spaghetty_plan_info info;
    int64_t st[4];
    double u[16] = {0}, s[16] = {0}, f = 1.0;
    int rq = spaghetty_plan_query(4, dims, perm, 0, &info);
    int rv = spaghetty_plan_verify(4, dims, perm, 1, 152, st);
    int rs = tce_sort_4_status(u, s, &two, &two, &two, &two, &bad[0], &bad[1], &bad[2], &bad[3], &f);
    printf("%d %d %d %d %s\n", rq, info.kind, rv, rs, spaghetty_version());
    return (rq == SPAGHETTY_OK && rv == SPAGHETTY_OK && rs == SPAGHETTY_ERR_PERM) ? 0 : 1;
}
"""


def test_c_program_links_and_calls_the_library(tmp_path):
    """A C caller compiled against include/spaghetty_gb300.h and linked with
    the shared library (as NWChem's link line does) plans, replays a plan and
    gets the reference's bad-permutation status, with no GPU."""
    import shutil
    import subprocess
    if not shutil.which("gcc"):
        pytest.skip("no C compiler")
    src = tmp_path / "caller.c"
    src.write_text(C_CALLER)
    exe = tmp_path / "caller"
    libdir = os.path.dirname(LIB_PATH)
    subprocess.check_call(["gcc", "-std=c99", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe),
                           "-L", libdir, "-lspaghetty_gb300", "-Wl,-rpath," + libdir])
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.split()[3] == "2" and "spaghetty_gb300" in r.stdout
