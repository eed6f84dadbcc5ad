"""The shipped GB300 tune table (spaghetty_gb300/tune_cache.txt) on the CPU:
every entry is a plan the current planner accepts (a stale entry would be
dropped silently and its problem planned by the defaults), and the tuned
plans of the smaller problems replay cleanly through the kernels' index
functions (spaghetty_plan_verify under the tuned override)."""
import os

import numpy as np

from spaghetty_gb300._lib import LIB_PATH, int_array, lib

TABLE = os.path.join(os.path.dirname(LIB_PATH), "tune_cache.txt")


def rows():
    sorts, buckets = [], []
    with open(TABLE) as fh:
        for line in fh:
            if line.startswith("#") or not line.strip():
                continue
            f = line.strip().split("|")
            assert len(f) == 9, line
            assert f[0] == "NVIDIA GB300" and f[1] == "152", line
            if f[2] == "batch":
                buckets.append(tuple(int(x) for x in f[3:]))
                continue
            dims = [int(x) for x in f[2].split(",")]
            perm = [int(x) + 1 for x in f[3].split(",")]
            box = [int(x) for x in f[5].split(",")]
            assert len(dims) == len(perm) == len(box), line
            sorts.append((dims, perm, int(f[4]), box, int(f[6]), int(f[7]), int(f[8])))
    return sorts, buckets


def test_every_entry_is_accepted_and_small_ones_replay():
    L = lib()
    sorts, buckets = rows()
    assert len(sorts) > 500 and len(buckets) >= 1
    replayed = 0
    try:
        for dims, perm, cls, box, threads, ept, stages in sorts:
            rc = L.spaghetty_tune_set(len(dims), int_array(dims), int_array(perm), cls,
                                      int_array(box), threads, ept, stages)
            assert rc == 0, (dims, perm, cls, box, threads, ept, stages, rc)
        for dims, perm, cls, box, threads, ept, stages in sorts:
            if int(np.prod(dims)) > (1 << 20):
                continue
            rc = L.spaghetty_plan_verify(len(dims), int_array(dims), int_array(perm), cls, 152, None)
            assert rc == 0, (dims, perm, cls, box, threads, ept, stages)
            replayed += 1
        assert replayed > 50
        for rank, lo, hi, run_in, run_out, volume in buckets:
            assert L.spaghetty_batch_tune_set(rank, lo, hi, run_in, run_out, volume) == 0
    finally:
        L.spaghetty_tune_set(0, None, None, 0, None, 0, 0, 0)      # drop every override
        L.spaghetty_batch_tune_set(0, 0, 0, 0, 0, 0)
