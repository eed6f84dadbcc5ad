"""Loop-order table for the reference's own C nests -- TEST INFRASTRUCTURE
(the timed CPU baseline of bench.py).

The reference picks, for every permutation, the fastest of its generated
loop orders by timing them all (trunk/generator2.py:581-598 for rank 4;
trunk/generator6.py:19-34,360-386 for the CCSD(T) rank-6 permutations) and
bakes the winners into a dispatch table (trunk/makelib.py:39-62).  This
script does the same on the host it runs on, for the configurations the
benchmark times:

* rank 4: all 24 loop orders for each of the 24 permutations at each size of
  the tce_sort_4 sweep (20^4, 30^4, 50^4, 100^4, (17,29,64,100));
* rank 6: the 54 CCSD(T) permutations at 16^6 (the identity aside), over the loop orders
  oracle/make_ref.py emits for them (up to five each: the two stride-1
  indices innermost in either order, the other four in input or output
  order, and the identity order) -- the full 720-order search per
  permutation would mean compiling 39,600 emitted routines.

Each order is run once to warm up and then timed (best of `reps`) with the
sort form and f = 0.5.  The result, keyed by the host's architecture and
thread count, is written to oracle/ref_loop_orders.json.

    python -m oracle.tune_ref_loops [--reps 3]
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(HERE, "ref_loop_orders.json")

SORT4_DIMS = [(20,) * 4, (30,) * 4, (50,) * 4, (100,) * 4, (17, 29, 64, 100)]


def host_key() -> str:
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return "%s-%dthreads" % (platform.machine(), threads)


def _best(R, perm, dims, u, s, reps):
    best_t, best_lo = None, None
    for lo in R.loops_for(len(dims), perm):
        R.call(perm, lo, u, s, dims, 0.5, 0.0)
        t = min(_timed(R, perm, lo, u, s, dims) for _ in range(reps))
        if best_t is None or t < best_t:
            best_t, best_lo = t, lo
    return best_lo, best_t


def _timed(R, perm, lo, u, s, dims):
    t0 = time.perf_counter()
    R.call(perm, lo, u, s, dims, 0.5, 0.0)
    return time.perf_counter() - t0


def tune(reps: int = 3) -> dict:
    import itertools
    from oracle import refnests as R
    if R.load() is None:
        raise RuntimeError("the reference nests are not built (oracle/make_ref.py)")
    rng = np.random.default_rng(5)
    out = {"host": host_key(), "rank4": {}, "rank6": {}}
    for dims in SORT4_DIMS:
        n = int(np.prod(dims))
        u, s = rng.uniform(-1, 1, n), np.zeros(n)
        key = "x".join(map(str, dims))
        out["rank4"][key] = {}
        for perm in itertools.permutations((1, 2, 3, 4)):
            lo, t = _best(R, perm, dims, u, s, reps)
            out["rank4"][key]["".join(map(str, perm))] = lo
            print(key, perm, lo, "%.2f GB/s" % (16 * n / t / 1e9), flush=True)
    dims = (16,) * 6
    n = 16 ** 6
    u, s = rng.uniform(-1, 1, n), np.zeros(n)
    triples = sorted({p for (r, p, _) in R._index if r == 6 and len(R.loops_for(6, p)) > 1})
    out["rank6"]["16x16x16x16x16x16"] = {}
    for p in triples:
        perm = tuple(int(c) for c in p)
        lo, t = _best(R, perm, dims, u, s, reps)
        out["rank6"]["16x16x16x16x16x16"][p] = lo
        print(dims, p, lo, "%.2f GB/s" % (16 * n / t / 1e9), flush=True)
    return out


def load() -> dict | None:
    """The committed table, if it was tuned on a host like this one."""
    try:
        with open(TABLE) as fh:
            t = json.load(fh)
    except (OSError, ValueError):
        return None
    return t if t.get("host") == host_key() else None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--out", default=TABLE)
    args = ap.parse_args()
    t = tune(args.reps)
    with open(args.out, "w") as fh:
        json.dump(t, fh, indent=1, sort_keys=True)
    print("wrote", args.out, file=sys.stderr)


if __name__ == "__main__":
    main()
