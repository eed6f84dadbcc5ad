"""Brute-force autotuner with a persistent cache.

The reference times every loop order of a permutation and keeps the fastest
(trunk/generator2.py:581-622; "best" and "good within 1.2x" rows), then bakes
the winners into a dispatch table (trunk/makelib.py:39-62, the `knight`
table).  Here the search space is the staging box (how much of each folded
index one CTA moves), the CTA shape (threads x elements per thread) and the
pipeline depth of the tiled kernel; the winners are stored in a JSON cache
keyed by (GPU, folded dims, folded permutation, operation class) and pushed
into the library with spaghetty_tune_set().  Tuning resumes by skipping keys
already in the cache.

CLI:  python -m spaghetty_gb300.autotune --sweep sort4 [--cache FILE]
"""
from __future__ import annotations

import argparse
import ctypes
import itertools
import json
import os
import time
from typing import Sequence

from ._lib import int_array, lib
from .sort import plan

DEFAULT_CACHE = os.environ.get(
    "SPAGHETTY_GB300_TUNE_CACHE",
    os.path.join(os.path.dirname(os.path.abspath(__file__)), "tune_cache.json"))

THREADS = (128, 256, 512)
EPTS = (1, 2, 4, 8)
TMA_THREADS = (128, 256)
TMA_EPTS = (8, 16)
VMAX = 4096
# run targets (contiguous doubles per box row) of the candidate boxes; 24, 40
# and 48 reach boxes that split a 100-long side in halves or thirds
RUNS = (16, 24, 32, 40, 48, 64)


def _split_len(D: int, want: int) -> int:
    if want >= D:
        return D
    want = max(1, want)
    nt = max(1, D // want)
    return -(-D // nt)


def _run(L, D, order):
    r = 1
    for d in order:
        r *= L[d]
        if L[d] < D[d]:
            break
    return r


def _frontier(L, D, order):
    for d in order:
        if L[d] < D[d]:
            return d
    return -1


def greedy_box(D: Sequence[int], P: Sequence[int], trun_in: int, trun_out: int,
               vtarget: int) -> list[int]:
    """The planner's greedy box (plan.cpp choose_box) with free targets."""
    R = len(D)
    L = [1] * R
    in_order = list(range(R - 1, -1, -1))
    out_order = [P[q] for q in range(R - 1, -1, -1)]
    for _ in range(64):
        vol = 1
        for x in L:
            vol *= x
        ri, ro = _run(L, D, in_order), _run(L, D, out_order)
        if ri < trun_in and _frontier(L, D, in_order) >= 0:
            d = _frontier(L, D, in_order)
            need = -(-trun_in * L[d] // ri)
        elif ro < trun_out and _frontier(L, D, out_order) >= 0:
            d = _frontier(L, D, out_order)
            need = -(-trun_out * L[d] // ro)
        else:
            break
        nl = _split_len(D[d], need)
        if vol // L[d] * nl > VMAX:
            nl = max(L[d], VMAX * L[d] // vol)
        if nl <= L[d]:
            break
        L[d] = nl
    for _ in range(64):
        vol = 1
        for x in L:
            vol *= x
        if vol >= vtarget:
            break
        ri, ro = _run(L, D, in_order), _run(L, D, out_order)
        fi, fo = _frontier(L, D, in_order), _frontier(L, D, out_order)
        if fi >= 0 and fo >= 0:
            d = fo if ro <= ri else fi
        else:
            d = fo if fo >= 0 else fi
        if d < 0:
            break
        want = min(L[d] * 2, L[d] * max(2, vtarget // vol))
        nl = _split_len(D[d], want)
        if vol // L[d] * nl > VMAX:
            break
        if nl <= L[d]:
            break
        L[d] = nl
    # at most two partial dims: round others down to divisors
    fi, fo = _frontier(L, D, in_order), _frontier(L, D, out_order)
    for d in range(R):
        if L[d] < D[d] and D[d] % L[d] and d not in (fi, fo):
            x = L[d]
            while x > 1 and D[d] % x:
                x -= 1
            L[d] = x
    return L


def candidates(dims: Sequence[int], perm: Sequence[int], op: int = 0):
    """Candidate (box, threads, ept, stages) for one problem."""
    p = plan(dims, perm, op)
    if p["kind"] == "flat":
        return p, []
    D, P = p["dims"], p["perm"]
    boxes = []
    for ti, to, vt in itertools.product(RUNS, RUNS, (512, 1024, 2048, 4096)):
        b = greedy_box(D, P, ti, to, vt)
        if b not in boxes:
            boxes.append(b)
    out = []
    for b in boxes:
        vol = 1
        for x in b:
            vol *= x
        if vol > VMAX:
            continue
        for nt, ept in itertools.product(THREADS, EPTS):
            cap = nt * ept
            if cap < vol or cap >= 2 * vol + nt:
                continue
            stages = (0,) if (p["kind"] == "direct" or ept < 2) else (0, 2, 3)
            for st in stages:
                out.append((list(b), nt, ept, st))
        # TMA-staged kernel (stages 12/13/14/16 = 2/3/4/6 load stages) on the
        # box with odd partial lengths along both stride-1 dims rounded up to
        # even (the bulk copies move whole 16-byte units there); the library
        # rejects boxes that do not fit the bulk tensor copy rules
        bt = list(b)
        for d in {len(D) - 1, P[len(D) - 1]}:
            if bt[d] % 2 and bt[d] < D[d]:
                bt[d] += 1
        vol_t = 1
        for x in bt:
            vol_t *= x
        if vol_t > VMAX:
            continue
        for nt, ept in itertools.product(TMA_THREADS, TMA_EPTS):
            cap = nt * ept
            if cap < vol_t or cap >= 2 * vol_t + nt:
                continue
            for st in (12, 13, 14, 16):
                if (bt, nt, ept, st) not in out:
                    out.append((bt, nt, ept, st))
    # the warp-shuffle transpose (stages code 20): one tile of the two
    # stride-1 dims per warp, when both are at most 32 long, product <= 128
    R = len(D)
    a, b = R - 1, P[R - 1]
    if a != b and D[a] <= 32 and D[b] <= 32 and D[a] * D[b] <= 128:
        wb = [1] * R
        wb[a], wb[b] = D[a], D[b]
        out.append((wb, 256, -(-D[a] * D[b] // 32), 20))
    return p, out


def _set(dims, perm, op, cfg):
    box, nt, ept, st = cfg
    return lib().spaghetty_tune_set(len(dims), int_array(dims), int_array(perm), op,
                                    int_array(box), nt, ept, st)


def clear():
    lib().spaghetty_tune_set(0, None, None, 0, None, 0, 0, 0)


def time_case(dims, perm, op, reps=5, device=None, flush_bytes=512 << 20, bufs=None):
    """Median kernel time (s) of one sort on device buffers, L2 flushed
    before every launch (so that no launch finds the previous one's tail in
    L2, which would favour some box orders over others) by a read-only pass
    over a scratch buffer, which leaves clean lines behind."""
    import torch
    from .sort import sort_generic
    dev = device or torch.device("cuda", torch.cuda.current_device())
    n = 1
    for d in dims:
        n *= d
    if bufs is None:
        u = torch.rand(n, dtype=torch.float64, device=dev)
        s = torch.rand(n, dtype=torch.float64, device=dev)
    else:
        u, s = bufs
    flush = torch.empty(flush_bytes // 4, dtype=torch.float32, device=dev)
    g = 0.0 if op == 0 else (1.0 if op == 1 else 2.0)
    times = []
    for r in range(reps + 1):
        flush.sum()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        sort_generic(u, s, dims, perm, 0.5, g)
        e1.record()
        e1.synchronize()
        if r:
            times.append(e0.elapsed_time(e1) / 1e3)
    times.sort()
    return times[len(times) // 2]


def gpu_key():
    import torch
    pr = torch.cuda.get_device_properties(torch.cuda.current_device())
    return "%s/%dsm" % (pr.name, pr.multi_processor_count)


def problem_key(p, op):
    cls = 0 if op == 0 else (1 if op == 1 else 2)
    return "%s|%s|%d" % (",".join(map(str, p["dims"])), ",".join(map(str, p["perm"])), cls)


def load_cache(path=DEFAULT_CACHE) -> dict:
    try:
        with open(path) as fh:
            return json.load(fh)
    except Exception:
        return {}


def save_cache(cache: dict, path=DEFAULT_CACHE):
    """Write the JSON cache and, beside it, the line format the C library
    loads by itself (tune_cache.txt next to the shared library)."""
    tmp = path + ".tmp%d" % os.getpid()
    with open(tmp, "w") as fh:
        json.dump(cache, fh, indent=1, sort_keys=True)
    os.replace(tmp, path)
    txt = os.path.splitext(path)[0] + ".txt"
    lines = ["# gpu|sms|folded dims|folded perm (0-based)|op class|box|threads|ept|stages"]
    for gk, ents in sorted(cache.items()):
        name, sms = gk.rsplit("/", 1)
        for key, e in sorted(ents.items()):
            if key.startswith("batch|"):
                if e.get("rule"):
                    _, rank, lo, hi = key.split("|")
                    lines.append("|".join([name, sms.rstrip("sm"), "batch", rank, lo, hi]
                                          + [str(v) for v in e["rule"]]))
                continue
            d, p, cls = key.split("|")
            lines.append("|".join([name, sms.rstrip("sm"), d, p, cls,
                                   ",".join(map(str, e["box"])), str(e["threads"]),
                                   str(e["ept"]), str(e["stages"])]))
    with open(txt + ".tmp", "w") as fh:
        fh.write("\n".join(lines) + "\n")
    os.replace(txt + ".tmp", txt)


def apply_cache(cache: dict | None = None, gpu: str | None = None) -> int:
    """Push every cached winner for this GPU into the library."""
    cache = load_cache() if cache is None else cache
    gpu = gpu or gpu_key()
    nset = 0
    for key, ent in cache.get(gpu, {}).items():
        if key.startswith("batch|"):
            if ent.get("rule"):
                _, rank, lo, hi = key.split("|")
                nset += lib().spaghetty_batch_tune_set(int(rank), int(lo), int(hi), *ent["rule"]) == 0
            continue
        dims_s, perm_s, cls = key.split("|")
        D = [int(x) for x in dims_s.split(",")]
        # the folded problem itself is a valid (dims, perm) call: perm 1-based
        P1 = [int(x) + 1 for x in perm_s.split(",")]
        rc = _set(D, P1, int(cls), (ent["box"], ent["threads"], ent["ept"], ent["stages"]))
        nset += rc == 0
    return nset


def tune(dims, perm, op=0, reps=5, cache=None, verbose=False, force=False, dump=None):
    """Time every candidate for (dims, perm, op); store and apply the best.
    ``dump``: an open text file that receives every candidate's time."""
    import torch
    p, cands = candidates(dims, perm, op)
    if not cands:
        return None
    cache = load_cache() if cache is None else cache
    gk = gpu_key()
    key = problem_key(p, op)
    if not force and key in cache.get(gk, {}):
        return cache[gk][key]
    n = 1
    for d in dims:
        n *= d
    dev = torch.device("cuda", torch.cuda.current_device())
    bufs = (torch.rand(n, dtype=torch.float64, device=dev),
            torch.rand(n, dtype=torch.float64, device=dev))
    clear()
    t_default = time_case(dims, perm, op, reps, bufs=bufs)
    results = []
    for cfg in cands:
        if _set(dims, perm, op, cfg) != 0:
            continue
        try:
            t = time_case(dims, perm, op, reps, bufs=bufs)
        except Exception:
            continue
        results.append((t, cfg))
        if dump is not None:
            dump.write(json.dumps({"dims": list(dims), "perm": list(perm), "op": op, "box": cfg[0],
                                   "threads": cfg[1], "ept": cfg[2], "stages": cfg[3],
                                   "seconds": t}) + "\n")
    if dump is not None:
        dump.write(json.dumps({"dims": list(dims), "perm": list(perm), "op": op, "default": True,
                               "seconds": t_default}) + "\n")
    clear()
    if not results:
        return None
    results.sort(key=lambda r: r[0])
    # confirm: the four fastest and the default again, interleaved, with
    # more repetitions, so that one noisy timing does not pick the winner
    finalists = [cfg for _, cfg in results[:4]] + [None]
    conf = {i: [] for i in range(len(finalists))}
    for _ in range(3):
        for i, cfg in enumerate(finalists):
            clear()
            if cfg is not None and _set(dims, perm, op, cfg) != 0:
                continue
            conf[i].append(time_case(dims, perm, op, reps, bufs=bufs))
    clear()
    med = {i: sorted(v)[len(v) // 2] for i, v in conf.items() if v}
    t_default = med.get(len(finalists) - 1, t_default)
    best_i = min((i for i in med if finalists[i] is not None), key=lambda i: med[i], default=None)
    if best_i is not None:
        results[0] = (med[best_i], finalists[best_i])
    t, (box, nt, ept, st) = results[0]
    if t_default < t:
        # the planner's own default beat every candidate: record it
        d = plan(dims, perm, op)
        if d["kind"] in ("direct", "tiled", "tma", "warp"):
            t, box, nt, ept = t_default, d["box"], d["threads"], d["ept"]
            st = d["stages"] + 10 if d["kind"] == "tma" else (20 if d["kind"] == "warp" else d["stages"])
    bpe = 16 if op == 0 else 24
    best_tma = min((r[0] for r in results if 12 <= r[1][3] < 20), default=None)
    best_other = min((r[0] for r in results if r[1][3] < 12 or r[1][3] == 20), default=None)
    ent = {"box": box, "threads": nt, "ept": ept, "stages": st, "seconds": t,
           "best_tma_gbs": n * bpe / best_tma / 1e9 if best_tma else None,
           "best_other_gbs": n * bpe / best_other / 1e9 if best_other else None,
           "gbs": n * bpe / t / 1e9, "default_seconds": t_default,
           "default_gbs": n * bpe / t_default / 1e9, "candidates": len(results),
           "good": sum(1 for r in results if r[0] < 1.2 * t)}
    if verbose:
        print(json.dumps({"dims": list(dims), "perm": list(perm), "op": op, **ent}), flush=True)
    cache.setdefault(gk, {})[key] = ent
    return ent


# Size buckets of the batched kernel (rank -> inclusive ranges of the largest
# extent) and the candidate tile-shape rules (input run, output run, volume).
BATCH_BUCKETS = {4: [(1, 11), (12, 19), (20, 27), (28, 64)], 6: [(1, 8), (9, 12), (13, 16), (17, 32)]}
BATCH_RULES = [(ti, to, vt) for ti in (8, 16, 32, 64) for to in (8, 16, 32, 64)
               for vt in (256, 512, 1024)]


def _batch_rules_except(cache, gk, skip):
    """Clear every bucket rule, then install the cached winners but `skip`."""
    lib().spaghetty_batch_tune_set(0, 0, 0, 0, 0, 0)
    for key, ent in cache.get(gk, {}).items():
        if key.startswith("batch|") and key != skip and ent.get("rule"):
            _, rank, lo, hi = key.split("|")
            lib().spaghetty_batch_tune_set(int(rank), int(lo), int(hi), *ent["rule"])


def tune_batched(cache, n=4096, seed=2024, budget_bytes=6 << 30, reps=3, verbose=True, force=False,
                 dump=None):
    """Per-size-bucket tile shapes of the persistent batched kernel, tuned on
    the batched configuration's own mix (workloads.batched_mix): for each
    bucket, the jobs of the mix that fall in it (up to budget_bytes) run as
    one batch under every candidate rule; the fastest rule is kept, or none
    when the built-in planner is faster."""
    import torch
    from .batched import Batch
    from .workloads import batched_mix
    dev = torch.device("cuda", torch.cuda.current_device())
    gk = gpu_key()
    mix = batched_mix(n, seed=seed)
    flush = torch.empty((512 << 20) // 4, dtype=torch.float32, device=dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)

    def timed(jobs):
        b = Batch(jobs)
        try:
            ts = []
            for r in range(reps + 1):
                flush.sum()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                b.launch()
                e1.record()
                e1.synchronize()
                if r:
                    ts.append(e0.elapsed_time(e1) / 1e3)
            if b.status() != 0:
                raise RuntimeError("batched status word set")
        finally:
            b.close()
        ts.sort()
        return ts[len(ts) // 2]

    for rank, buckets in BATCH_BUCKETS.items():
        for lo, hi in buckets:
            key = "batch|%d|%d|%d" % (rank, lo, hi)
            if not force and key in cache.get(gk, {}):
                continue
            jobs, used = [], 0
            for m in mix:
                if len(m["dims"]) != rank or not (lo <= max(m["dims"]) <= hi):
                    continue
                k = 1
                for d in m["dims"]:
                    k *= d
                if used + 16 * k > budget_bytes:
                    continue
                u = torch.rand(k, dtype=torch.float64, device=dev, generator=gen) - 0.5
                sb = torch.rand(k, dtype=torch.float64, device=dev, generator=gen) - 0.5
                jobs.append((u, sb, m["dims"], m["perm"], m["factor"], 1.0 if m["acc"] else 0.0))
                used += 16 * k
            if not jobs:
                continue
            _batch_rules_except(cache, gk, key)
            t_default = timed(jobs)
            results = []
            for rule in BATCH_RULES:
                if lib().spaghetty_batch_tune_set(rank, lo, hi, *rule) != 0:
                    continue
                t = timed(jobs)
                results.append((t, rule))
                if dump is not None:
                    dump.write(json.dumps({"batch": [rank, lo, hi], "rule": rule, "seconds": t}) + "\n")
            _batch_rules_except(cache, gk, key)
            results.sort()
            t, rule = results[0]
            ent = {"rule": list(rule) if t < t_default else None, "seconds": min(t, t_default),
                   "default_seconds": t_default, "jobs": len(jobs), "bytes": used,
                   "gbs": used / min(t, t_default) / 1e9, "default_gbs": used / t_default / 1e9}
            cache.setdefault(gk, {})[key] = ent
            if verbose:
                print(json.dumps({"bucket": key, **ent}), flush=True)
            del jobs
            torch.cuda.empty_cache()
    apply_cache(cache, gk)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sweep", default="sort4",
                    choices=["sort4", "sort6-triples", "sort6-sample", "random", "batched", "case"])
    ap.add_argument("--dims", default="100,100,100,100")
    ap.add_argument("--perm", default="4,3,2,1")
    ap.add_argument("--ops", default="0,1")
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--cache", default=DEFAULT_CACHE)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--dump", default=None, help="write every candidate's time to this file")
    args = ap.parse_args()
    from .workloads import PERMS4, SORT4_DIMS, TRIPLES_SORT6
    ops = [int(x) for x in args.ops.split(",")]
    if args.sweep == "sort4":
        probs = [(d, p) for d in SORT4_DIMS for p in PERMS4]
    elif args.sweep == "sort6-triples":
        probs = [((16,) * 6, p) for p in TRIPLES_SORT6]
    elif args.sweep == "random":
        # seeded shapes outside the configurations (the data the planner's
        # default rules are fitted on): rank 4 with extents in [8, 64],
        # rank 6 with extents in [6, 20], random permutations
        import random
        rnd = random.Random(4646)
        probs = []
        for i in range(48):
            r = 4 if i % 2 == 0 else 6
            dims = tuple(rnd.randint(8, 64) if r == 4 else rnd.randint(6, 20) for _ in range(r))
            perm = list(range(1, r + 1))
            while perm == sorted(perm):
                rnd.shuffle(perm)
            probs.append((dims, tuple(perm)))
    elif args.sweep == "sort6-sample":
        # the sort6 configuration's bench sample: triples perms at 16^6 and
        # 20^6, 48 seeded perms at the non-cubic shape
        import random
        from .workloads import PERMS6
        rnd = random.Random(6)
        probs = ([((16,) * 6, p) for p in TRIPLES_SORT6] + [((20,) * 6, p) for p in TRIPLES_SORT6]
                 + [((12, 20, 16, 20, 12, 16), p) for p in rnd.sample(PERMS6, 48)])
    else:
        probs = [(tuple(int(x) for x in args.dims.split(",")),
                  tuple(int(x) for x in args.perm.split(",")))]
    cache = load_cache(args.cache)
    dump = open(args.dump, "w") if args.dump else None
    if args.sweep == "batched":
        t0 = time.time()
        tune_batched(cache, reps=args.reps, force=args.force, dump=dump)
        save_cache(cache, args.cache)
        if dump is not None:
            dump.close()
        print("tuned the batched buckets in %.1fs" % (time.time() - t0))
        return
    t0 = time.time()
    for dims, perm in probs:
        for op in ops:
            tune(dims, perm, op, args.reps, cache, verbose=True, force=args.force, dump=dump)
        save_cache(cache, args.cache)
    if dump is not None:
        dump.close()
    print("tuned %d problems in %.1fs" % (len(probs) * len(ops), time.time() - t0))


if __name__ == "__main__":
    main()
