"""Host replay of the batched kernel's plans (spaghetty_batch_verify, no GPU):
the work list the persistent kernel would get for a batch -- every sort's
job record, its work units and every box through the kernel's own index
functions -- is in bounds and writes every output element exactly once from
the input element the permutation maps to it (trunk/old_sort.f:54-58), for
the batched workload's own mixes (reduced in size), every bucket rule the
autotuner can install, and other SM counts."""
import ctypes
import random

import numpy as np
import pytest

from spaghetty_gb300._lib import BatchEntry, lib
from spaghetty_gb300.workloads import batched_mix


def entries(mix):
    arr = (BatchEntry * len(mix))()
    for e, m in zip(arr, mix):
        e.rank = len(m["dims"])
        for q, d in enumerate(m["dims"]):
            e.dims[q] = d
        for q, p in enumerate(m["perm"]):
            e.perm[q] = p
        e.factor = m["factor"]
        e.acc_factor = 1.0 if m.get("acc") else 0.0
    return arr


def verify(mix, sms=152):
    st = (ctypes.c_int64 * 4)()
    rc = lib().spaghetty_batch_verify(ctypes.cast(entries(mix), ctypes.c_void_p), len(mix), sms, st)
    return rc, list(st)


def test_small_tile_mix():
    mix = batched_mix(4096, seed=2024, ext4=(4, 12), ext6=(3, 6))
    rc, (jobs, units, boxes, elems) = verify(mix)
    assert rc == 0
    assert jobs == len(mix) and elems == sum(int(np.prod(m["dims"])) for m in mix)
    assert units >= jobs and boxes >= units


def test_reduced_configuration_mix():
    """A seeded slice of the batched configuration's own mix (extents 8-40
    and 6-20), its 6-D sorts capped at 12 per extent to keep the replay
    short."""
    mix = batched_mix(96, seed=2024, ext4=(8, 40), ext6=(6, 12))
    rc, st = verify(mix)
    assert rc == 0 and st[0] == 96


@pytest.mark.parametrize("sms", [1, 16, 152, 304])
def test_unit_sizes_follow_the_sm_count(sms):
    mix = batched_mix(64, seed=7, ext4=(8, 24), ext6=(4, 9))
    rc, st = verify(mix, sms)
    assert rc == 0 and st[0] == 64


@pytest.mark.parametrize("rule", [(8, 8, 256), (16, 64, 1024), (64, 16, 512), (32, 32, 1024)])
def test_every_bucket_rule_shape(rule):
    L = lib()
    mix = batched_mix(48, seed=11, ext4=(5, 33), ext6=(3, 9))
    try:
        for rank, lo, hi in [(4, 1, 64), (6, 1, 32)]:
            assert L.spaghetty_batch_tune_set(rank, lo, hi, *rule) == 0
        rc, st = verify(mix)
        assert rc == 0 and st[0] == 48
    finally:
        L.spaghetty_batch_tune_set(0, 0, 0, 0, 0, 0)
        L.spaghetty_tune_load(ctypes.c_char_p(lib_tune_file().encode()))


def lib_tune_file():
    import os
    from spaghetty_gb300._lib import LIB_PATH
    return os.path.join(os.path.dirname(LIB_PATH), "tune_cache.txt")


def test_odd_shapes_and_unit_dims():
    rnd = random.Random(5)
    mix = []
    for _ in range(40):
        r = rnd.choice([2, 3, 4, 5, 6])
        dims = tuple(rnd.choice([1, 1, 2, 3, 7, 13, 17, 31]) for _ in range(r))
        perm = list(range(1, r + 1))
        rnd.shuffle(perm)
        mix.append({"dims": dims, "perm": tuple(perm), "factor": rnd.uniform(-2, 2),
                    "acc": rnd.random() < 0.5})
    rc, st = verify(mix)
    assert rc == 0


def test_bad_entry_is_named():
    mix = batched_mix(8, seed=3, ext4=(4, 8), ext6=(3, 4))
    mix[5] = dict(mix[5], perm=(1,) * len(mix[5]["dims"]))
    rc, _ = verify(mix)
    assert rc == 2                                  # SPAGHETTY_ERR_PERM
    assert lib().spaghetty_batch_bad_index() == 5


def test_python_wrapper():
    from spaghetty_gb300._lib import SpaghettyError
    from spaghetty_gb300.batched import verify_plan
    mix = batched_mix(32, seed=9, ext4=(4, 16), ext6=(3, 6))
    st = verify_plan(mix)
    assert st["jobs"] == 32 and st["elements"] == sum(int(np.prod(m["dims"])) for m in mix)
    bad = list(mix)
    bad[3] = dict(bad[3], dims=(0,) + tuple(bad[3]["dims"][1:]))
    st = verify_plan(bad)                       # an empty tensor is not a job
    assert st["jobs"] == 31
    bad[4] = dict(bad[4], perm=(2,) * len(bad[4]["dims"]))
    with pytest.raises(SpaghettyError):
        verify_plan(bad)
