#!/usr/bin/env python3
"""Benchmark: tce_sort_4 sweep effective GB/s on one GB300 (and replicas).

Workload (one "step"): the tce_sort_4 sweep -- all 24 permutations of a rank-4
FP64 tensor at dims 20^4, 30^4, 50^4, 100^4 (800 MB per tensor) and
(17,29,64,100), factors {1.0, -1.0, 0.5}, sort and sortacc: 720 launches.
Inputs are seeded uniform(-1,1) FP64 resident in HBM.  Each launch is timed
with CUDA events on its stream; before every launch the L2 is flushed
outside the timed events by a read-only pass over a 512 MB scratch buffer,
which leaves the L2 holding clean lines (the previous kernel's dirty lines
are written back during the flush, not during the timed kernel).  value = algorithmic bytes (16
B/element for sort, 24 B/element for sortacc) / summed kernel time.

e2e: the same sweep through the reference-facing C ABI (tce_sort_4 /
tce_sortacc_4) with pinned HOST buffers, wall-clocked per call: each call
copies its input (and, for sortacc, its output) host->device, runs the
kernel, and copies the output back.

--impl reference: the reference's own C loop nests (generated by
trunk/generator2.py, built by oracle/make_ref.py with OpenMP over every host
core), on the best of the 24 loop orders of each permutation and size (the
table oracle/tune_ref_loops.py tunes on the host), timed over a bounded
per-step sample of the same sweep.

Multi-GPU: the sweep has no exchange step, so N ranks run N independent
replicas ("replicas only"); value = all ranks' bytes / max rank time.
"""
from __future__ import annotations

import argparse
import itertools
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "sort4 sweep effective GB/s (24 perms x {20^4,30^4,50^4,100^4,17x29x64x100} x f{1,-1,0.5} x {sort,sortacc}), FP64"
UNIT = "GB/s"
L2_BYTES = 129 * 1024 * 1024
WORKLOAD = ("tce_sort_4 sweep: 24 perms x dims {20^4, 30^4, 50^4, 100^4, (17,29,64,100)} "
            "x f in {1.0,-1.0,0.5} x {sort, sortacc}, FP64 uniform(-1,1)")


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sms, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sms.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sms:
            return None
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sms)}


def sweep_cases():
    from spaghetty_gb300.workloads import PERMS4, SORT4_DIMS, SORT4_FACTORS
    cases = []
    for dims in SORT4_DIMS:
        for perm in PERMS4:
            for f in SORT4_FACTORS:
                for acc in (False, True):
                    cases.append((dims, perm, f, acc))
    return cases


def flush_l2(buf):
    """Evict the L2 before a timed launch: a read-only reduction over `buf`
    (4x the L2), so the L2 is left holding clean lines and the timed kernel
    pays for no write-backs of earlier kernels' data."""
    buf.sum()


def host_lead(torch):
    """Give the host a head start before a run of individually timed
    launches: a ~50 ms GPU sleep (torch.cuda._sleep, a spin on the clock
    that ends by itself) lets it queue launches ahead, so a host-side pause
    (Python's garbage collector, the first plan of a shape) lands while the
    GPU is still busy instead of between an event pair.  Not inside any
    timed pair."""
    torch.cuda._sleep(100_000_000)


def needs_flush(n_elems):
    """Every timed launch starts from a flushed L2: tensors near the L2's size
    (16^6: 134 MB) would otherwise find part of their input there, or pay
    for writing back the previous launch's dirty output lines, and even at
    100^4 the previous launch's tail is in L2."""
    return True


def case_bytes(dims, acc):
    n = 1
    for d in dims:
        n *= d
    return n * (24 if acc else 16)


def traffic_from_profile():
    """dram bytes per launch of the dominant kernel, from the committed ncu
    summary (profiles/tma_sort4_100.md, line 'traffic_bytes_per_launch: X')."""
    path = os.path.join(ROOT, "profiles", "tma_sort4_100.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1])
    except Exception:
        pass
    return None


# ---------------------------------------------------------------------------
def run_ours(args, ws, rank, local):
    import torch
    import spaghetty_gb300 as S
    from spaghetty_gb300._lib import lib, int_array
    import ctypes

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    L = lib()
    cases = sweep_cases()
    sizes = sorted({c[0] for c in cases}, key=lambda d: -int(torch.tensor(d).prod()))
    gen = torch.Generator(device=dev)
    gen.manual_seed(1234 + rank)
    bufs = {}
    for dims in sizes:
        n = 1
        for d in dims:
            n *= d
        u = torch.rand(n, dtype=torch.float64, device=dev, generator=gen) * 2 - 1
        s = torch.rand(n, dtype=torch.float64, device=dev, generator=gen) * 2 - 1
        bufs[dims] = (u, s, n)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)

    def launch(dims, perm, f, acc):
        u, s, n = bufs[dims]
        rc = L.spaghetty_sort_async(4, ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(s.data_ptr()),
                                    int_array(dims), int_array(perm), f, 1.0 if acc else 0.0, sp)
        if rc:
            raise RuntimeError("spaghetty_sort_async failed: %d" % rc)

    def one_step(record):
        evs = []
        if record:
            host_lead(torch)
        for (dims, perm, f, acc) in cases:
            n = bufs[dims][2]
            if needs_flush(n):
                flush_l2(flush)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            launch(dims, perm, f, acc)
            e1.record(stream)
            evs.append((dims, perm, f, acc, e0, e1))
        if record:
            return evs
        return None

    for _ in range(args.warmup):
        one_step(False)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local) if rank == 0 else None
    if sampler:
        sampler.start()
    all_evs = []
    gc.disable()
    w0 = time.perf_counter()
    for _ in range(args.steps):
        all_evs.append(one_step(True))
    torch.cuda.synchronize()
    wall = time.perf_counter() - w0
    gc.enable()
    clocks = sampler.stop() if sampler else None
    if ws > 1:
        torch.distributed.barrier()

    total_ms = 0.0
    total_bytes = 0
    per_size = {}
    detail = {}
    dom_ms, dom_bytes, dom_n = 0.0, 0, 0
    for evs in all_evs:
        for (dims, perm, f, acc, e0, e1) in evs:
            ms = e0.elapsed_time(e1)
            b = case_bytes(dims, acc)
            total_ms += ms
            total_bytes += b
            key = "x".join(map(str, dims))
            a = per_size.setdefault(key, [0.0, 0])
            a[0] += ms
            a[1] += b
            plan = S.plan(dims, perm, 1 if acc else 0)
            dk = (dims, perm, f, acc)
            dd = detail.setdefault(dk, [0.0, 0, plan["kind"]])
            dd[0] += ms
            dd[1] += b
            if dims == (100, 100, 100, 100) and plan["kind"] == "tma" and not acc:
                dom_ms += ms
                dom_bytes += b
                dom_n += 1
    launches = len(cases) * args.steps
    if args.detail and rank == 0:
        with open(args.detail, "w") as fh:
            for (dims, perm, f, acc), (ms, b, kind) in sorted(detail.items()):
                fh.write(json.dumps({"dims": dims, "perm": perm, "f": f, "acc": acc, "kind": kind,
                                     "gbs": round(b / (ms / 1e3) / 1e9, 1)}) + "\n")
    t_rank = total_ms / 1e3
    if ws > 1:
        t = torch.tensor([t_rank], dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_max = float(t[0])
    else:
        t_max = t_rank
    value = total_bytes * ws / t_max / 1e9

    # e2e: same sweep through the C ABI with pinned host buffers (the kernels
    # read and write them in place); the staged variant for comparison
    e2e = None
    if not args.no_e2e:
        # every rank runs the e2e sweep on its own GPU and host buffers; the
        # whole-job value is all ranks' bytes over the slowest rank's time
        e2e = run_e2e(args, cases, torch, L, int_array, ctypes, warm=max(3, args.warmup))
        nbytes, secs = e2e.pop("_bytes"), e2e.pop("_seconds")
        if ws > 1:
            t = torch.tensor([secs], dtype=torch.float64)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            e2e["value"] = round(nbytes * ws / float(t[0]) / 1e9, 2)
            e2e["h2d_bytes_per_step"] *= ws
            e2e["d2h_bytes_per_step"] *= ws
    if rank == 0 and not args.no_e2e:
        # the two alternatives, for comparison only (rank 0): one warm-up sweep each
        L.spaghetty_set_option(1, 0)
        staged = run_e2e(args, cases, torch, L, int_array, ctypes, warm=1)
        L.spaghetty_set_option(1, 1)
        L.spaghetty_set_option(2, 1)
        piped = run_e2e(args, cases, torch, L, int_array, ctypes, warm=1)
        for alt in (staged, piped):
            alt.pop("_bytes")
            alt.pop("_seconds")
        L.spaghetty_set_option(2, 0)
        e2e["staged_copies_value"] = staged["value"]
        e2e["pipelined_slabs_value"] = piped["value"]

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(args.cpu_seconds)

    secondary = None
    if not args.no_secondary and rank == 0:
        del bufs
        torch.cuda.empty_cache()
        secondary = {"sort6": run_sort6(args, dev), "triples_fused": run_fused(args, dev),
                     "autograd": run_autograd(args, dev), "contract": run_contract(args, dev)}
        torch.cuda.empty_cache()
    batched = None
    if not args.no_batched:
        torch.cuda.empty_cache()
        batched = {"config": run_batched(args, dev),
                   "small_tiles": run_batched(args, dev, ext4=(4, 12), ext6=(3, 6))}

    peak, peak_kind = peaks()
    roof = None
    if dom_n:
        achieved = (dom_bytes / dom_n) / ((dom_ms / dom_n) / 1e3) / 1e9
        tr = traffic_from_profile()
        roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": tr,
                "kernel": "spg_tiled_tma, sort (16 B/element), 100^4: every perm planned on the "
                          "TMA-staged kernel, factors 1, -1, 0.5",
                "launches": dom_n,
                "traffic_source": "ncu capture of one launch of the 100^4 perm 4321 sort on its tuned "
                                  "plan (profiles/tma_sort4_100.md), not of this run",
                "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs, burst copy)"}
    breakdown = {k: round(v[1] / (v[0] / 1e3) / 1e9, 1) for k, v in per_size.items()}
    # the identity permutation at each size is a plain streaming copy (the
    # flat kernel): the floor that launch latency and the flush leave there
    floor = {}
    for (dims, perm, f, acc), (ms, b, kind) in detail.items():
        if perm == (1, 2, 3, 4):
            a = floor.setdefault("x".join(map(str, dims)), [0.0, 0])
            a[0] += ms
            a[1] += b
    floor_gbs = {k: round(v[1] / (v[0] / 1e3) / 1e9, 1) for k, v in floor.items()}
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(t_max * 1e3 / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded uniform(-1,1) FP64 in HBM)",
        "config": {"workload": WORKLOAD, "parallelism": "replicas" if ws > 1 else "single",
                   "l2": "flushed before every timed launch (read-only pass over 512 MB, "
                         "leaving clean lines)"},
        "gpu_launches": launches,
        "breakdown_gbs_by_size": breakdown,
        "frac_of_peak_by_size": {k: round(v / peak, 4) for k, v in breakdown.items()},
        "identity_copy_gbs_by_size": floor_gbs,
        "frac_of_identity_copy_by_size": {k: round(breakdown[k] / floor_gbs[k], 4)
                                          for k in breakdown if floor_gbs.get(k)},
        "frac_of_hbm_peak": round(value / ws / peak, 4),
        "roofline": roof,
        "e2e": e2e,
        "cpu_baseline": cpu,
        "batched": batched,
        "secondary": secondary,
        "clocks": clocks,
        "wall_s_timed_region": round(wall, 3),
    }
    return line


def run_e2e(args, cases, torch, L, int_array, ctypes, warm=3):
    host = {}
    for (dims, _, _, _) in cases:
        if dims in host:
            continue
        n = 1
        for d in dims:
            n *= d
        u = (torch.rand(n, dtype=torch.float64) * 2 - 1).pin_memory()
        s = (torch.rand(n, dtype=torch.float64) * 2 - 1).pin_memory()
        host[dims] = (u, s, n)
    fac = ctypes.c_double()
    h2d = d2h = 0
    total_b = 0

    def call(dims, perm, f, acc):
        u, s, n = host[dims]
        fac.value = f
        ints = [ctypes.byref(ctypes.c_int(v)) for v in list(dims) + list(perm)]
        fn = L.tce_sortacc_4_status if acc else L.tce_sort_4_status
        rc = fn(ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(s.data_ptr()), *ints, ctypes.byref(fac))
        if rc:
            raise RuntimeError("tce_sort_4 failed %d" % rc)

    # warm-up: whole sweeps, so that every plan and kernel the timed sweeps
    # use is built and loaded before the clock starts
    for _ in range(warm):
        for (dims, perm, f, acc) in cases:
            call(dims, perm, f, acc)
    steps = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(steps):
        for (dims, perm, f, acc) in cases:
            call(dims, perm, f, acc)
            n = host[dims][2]
            h2d += n * 8 * (2 if acc else 1)
            d2h += n * 8
            total_b += case_bytes(dims, acc)
    dt = time.perf_counter() - t0
    return {"value": round(total_b / dt / 1e9, 2), "unit": UNIT, "_bytes": total_b, "_seconds": dt,
            "h2d_bytes_per_step": h2d // steps, "d2h_bytes_per_step": d2h // steps,
            "steps": steps, "warmup_sweeps": warm,
            "how": "tce_sort_4/tce_sortacc_4 C-ABI calls on pinned host "
                                  "buffers (read and written in place by the kernels over "
                                  "NVLink-C2C), wall clock per sweep"}


# ---------------------------------------------------------------------------
_CPU_STATE = {}


def ref_thread_count() -> int:
    """Host threads the reference's nests run on: every host core, or
    SPAGHETTY_REF_THREADS.  (A launcher such as torchrun starts its ranks
    with OMP_NUM_THREADS=1; the reference runs in rank 0 alone and takes the
    whole host.)"""
    return int(os.environ.get("SPAGHETTY_REF_THREADS", os.cpu_count() or 1))


def _cpu_setup():
    """Build/load the reference nests, pick the loop order of every
    (perm, size) -- from oracle/ref_loop_orders.json when it was tuned on a
    host like this one (all 24 orders timed per perm and size, the
    reference's brute-force method, trunk/generator2.py:581-598), else by
    timing the 24 orders once at 30^4 here -- and make the sweep's buffers."""
    import numpy as np
    from oracle import refnests as R
    from oracle import tune_ref_loops as TR
    from spaghetty_gb300.workloads import PERMS4, SORT4_DIMS
    if _CPU_STATE:
        return _CPU_STATE
    if R.load() is None:
        return None
    R.set_threads(ref_thread_count())
    rng = np.random.default_rng(3)
    table = TR.load()
    best = {}
    if table is not None:
        for dims in SORT4_DIMS:
            row = table["rank4"]["x".join(map(str, dims))]
            for perm in PERMS4:
                best[(dims, perm)] = row["".join(map(str, perm))]
        how = "best of 24 loop orders per (perm, size), from the table tuned on this host type"
    else:
        tdims = (30, 30, 30, 30)
        n = 30 ** 4
        u = rng.uniform(-1, 1, n)
        s = np.zeros(n)
        for perm in PERMS4:
            bt, bl = 1e9, None
            for lo in R.loops_for(4, perm):
                R.call(perm, lo, u, s, tdims, 0.5, 0.0)
                t0 = time.perf_counter()
                R.call(perm, lo, u, s, tdims, 0.5, 0.0)
                dt = time.perf_counter() - t0
                if dt < bt:
                    bt, bl = dt, lo
            for dims in SORT4_DIMS:
                best[(dims, perm)] = bl
        how = "best of 24 loop orders per perm, tuned here at 30^4"
    bufs = {}
    for dims in SORT4_DIMS:
        m = int(np.prod(dims))
        bufs[dims] = (rng.uniform(-1, 1, m), rng.uniform(-1, 1, m))
    _CPU_STATE.update(best=best, bufs=bufs, R=R, how=how, table=table)
    return _CPU_STATE


def cpu_sweep_sample(budget_s: float, threads: int | None = None, start: int = 0):
    """The reference's C loop nests on the host cores (the tuned loop order
    of each perm and size), timed over a bounded sample of the sweep
    starting at case `start`.  Returns (GB/s, cores, description, next)."""
    from spaghetty_gb300.workloads import PERMS4, SORT4_DIMS, SORT4_FACTORS
    st = _cpu_setup()
    if st is None:
        return None
    R, best, bufs = st["R"], st["best"], st["bufs"]
    cores = R.set_threads(threads or ref_thread_count())
    total_b, total_t, calls = 0, 0.0, 0
    # sizes interleaved, so that any bounded prefix weights the sizes as the
    # whole sweep does
    order = [(d, p, f, acc) for p in PERMS4 for f in SORT4_FACTORS for acc in (False, True)
             for d in SORT4_DIMS]
    t_start = time.perf_counter()
    i = start
    while calls < len(order) and time.perf_counter() - t_start <= budget_s:
        dims, perm, f, acc = order[i % len(order)]
        uu, ss = bufs[dims]
        t0 = time.perf_counter()
        R.call(perm, best[(dims, perm)], uu, ss, dims, f, 1.0 if acc else 0.0)
        total_t += time.perf_counter() - t0
        total_b += case_bytes(dims, acc)
        calls += 1
        i += 1
    desc = ("reference generated C nests (trunk/generator2.py emitter, OpenMP over %d host "
            "threads, gcc -O3 -ffp-contract=off), %s; "
            "%d calls of the sweep (24 perms x 5 sizes x f{1,-1,0.5} x sort/sortacc, the five "
            "sizes interleaved, from case %d) within a %.0f s budget"
            % (cores, st["how"], calls, start % len(order), budget_s))
    return total_b / total_t / 1e9, cores, desc, i


def cpu_sort6_baseline(budget_s):
    """The reference's rank-6 C nests (trunk/generator6.py emitter) on the
    host cores at 16^6 for the 54 CCSD(T) perms, sort (f = -0.5) and sortacc
    (f = 1), each perm on its best emitted loop order (the committed table,
    else timed here), over a bounded sample."""
    try:
        import numpy as np
        from oracle import refnests as R
        from oracle import tune_ref_loops as TR
        from spaghetty_gb300.workloads import TRIPLES_SORT6
        if R.load() is None:
            return {"value": None, "unit": UNIT, "error": "reference nests unavailable"}
        R.set_threads(ref_thread_count())
        dims = (16,) * 6
        n = 16 ** 6
        rng = np.random.default_rng(6)
        u, s = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
        table = TR.load()
        best = {}
        for perm in TRIPLES_SORT6:
            key = "".join(map(str, perm))
            if table is not None and key in table["rank6"]["16x16x16x16x16x16"]:
                best[perm] = table["rank6"]["16x16x16x16x16x16"][key]
                continue
            bt = None
            for lo in R.loops_for(6, perm):
                t0 = time.perf_counter()
                R.call(perm, lo, u, s, dims, 0.5, 0.0)
                dt = time.perf_counter() - t0
                if bt is None or dt < bt:
                    bt, best[perm] = dt, lo
        cores = R.set_threads(ref_thread_count())
        total_b, total_t, calls = 0, 0.0, 0
        t_start = time.perf_counter()
        order = [(p, acc) for p in TRIPLES_SORT6 for acc in (False, True)]
        while calls < len(order) and time.perf_counter() - t_start <= budget_s:
            perm, acc = order[calls]
            t0 = time.perf_counter()
            R.call(perm, best[perm], u, s, dims, 1.0 if acc else -0.5, 1.0 if acc else 0.0)
            total_t += time.perf_counter() - t0
            total_b += n * (24 if acc else 16)
            calls += 1
        return {"value": round(total_b / total_t / 1e9, 2), "unit": UNIT, "cores": cores,
                "kind": "reference",
                "sample": "reference generated C nests (trunk/generator6.py emitter, OpenMP over %d "
                          "host threads, gcc -O3 -ffp-contract=off), best of the emitted loop orders "
                          "per perm (%s); %d calls: the 54 CCSD(T) perms at 16^6, sort and sortacc, "
                          "within a %.0f s budget"
                          % (cores, "committed table" if table else "timed here", calls, budget_s)}
    except Exception as e:  # noqa: BLE001
        return {"value": None, "unit": UNIT, "error": str(e)[:200]}


def cpu_baseline(budget_s):
    try:
        r = cpu_sweep_sample(budget_s)
    except Exception as e:  # noqa: BLE001
        return {"value": None, "unit": UNIT, "error": str(e)[:200]}
    if r is None:
        return {"value": None, "unit": UNIT, "error": "reference nests unavailable"}
    v, cores, desc, _ = r
    out = {"value": round(v, 2), "unit": UNIT, "cores": cores, "kind": "reference",
           "sample": desc}
    try:
        out["old_sort"] = old_sort_sample(min(8.0, budget_s / 2))
    except Exception as e:  # noqa: BLE001
        out["old_sort"] = {"value": None, "error": str(e)[:200]}
    return out


def old_sort_sample(budget_s):
    """The Hirata routines themselves (trunk/old_sort.f: old_sort_4 /
    old_sortacc_4, restated in C by the oracle, one host thread as the Fortran
    is serial), timed on the same interleaved sample of the sweep for a
    bounded time: the code NWChem runs when it does not link a tuned
    library."""
    import numpy as np
    from oracle import oracle as O
    from spaghetty_gb300.workloads import PERMS4, SORT4_DIMS
    rng = np.random.default_rng(5)
    bufs = {}
    for dims in SORT4_DIMS:
        m = int(np.prod(dims))
        bufs[dims] = (rng.uniform(-1, 1, m), rng.uniform(-1, 1, m))
    cases = [(d, p, f, a) for p in PERMS4 for f in (1.0, -1.0, 0.5) for a in (False, True)
             for d in SORT4_DIMS]
    tb, tt, k = 0, 0.0, 0
    t_end = time.perf_counter() + budget_s
    while time.perf_counter() < t_end and k < len(cases):
        dims, perm, f, acc = cases[k]
        u, y = bufs[dims]
        t0 = time.perf_counter()
        O.old_sort(u, dims, perm, f, out=y, acc=acc)
        tt += time.perf_counter() - t0
        tb += u.size * (24 if acc else 16)
        k += 1
    return {"value": round(tb / tt / 1e9, 2) if tt else None, "unit": UNIT, "cores": 1,
            "sample": "old_sort_4 / old_sortacc_4 (trunk/old_sort.f:33-95,512-575, the oracle's C "
                      "restatement, -O2 -ffp-contract=off), %d calls of the sweep, sizes interleaved"
                      % k}


def run_reference(args, ws, rank):
    if rank != 0:
        return None
    from oracle import refnests as R
    if R.load() is None:
        return {"impl": "reference", "unavailable": "reference C nests could not be built here"}
    per_step = max(2.0, min(12.0, 150.0 / max(1, args.steps + args.warmup)))
    nxt = 0
    for _ in range(args.warmup):
        _, _, _, nxt = cpu_sweep_sample(per_step, start=nxt)
    vals = []
    t0 = time.perf_counter()
    cores, desc = None, None
    for _ in range(args.steps):
        v, cores, desc, nxt = cpu_sweep_sample(per_step, start=nxt)
        vals.append(v)
    wall = time.perf_counter() - t0
    value = statistics.median(vals)
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 2), "unit": UNIT,
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(wall * 1e3 / args.steps, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded uniform(-1,1) FP64)",
        "config": {"workload": WORKLOAD, "parallelism": "host cores (OpenMP)"},
        "cpu_baseline": {"value": round(value, 2), "unit": UNIT, "cores": cores,
                         "kind": "reference", "sample": desc},
        "e2e": {"value": round(value, 2), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def run_batched(args, dev, ext4=(8, 40), ext6=(6, 20), n=4096, seed=2024):
    """The batched configuration: n uneven sorts (70% rank 4, extents
    uniform in ext4; 30% rank 6, extents uniform in ext6; random perm, factor
    uniform(-1,1), half sortacc) as ONE persistent launch replayed from a CUDA
    graph, against one launch per sort.  Returns tiles/s and GB/s of both."""
    import torch
    from spaghetty_gb300.batched import Batch
    from spaghetty_gb300.workloads import batched_mix
    mix = batched_mix(n, seed=seed, ext4=ext4, ext6=ext6)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    jobs = []
    total_b = 0
    for m in mix:
        k = 1
        for d in m["dims"]:
            k *= d
        u = torch.rand(k, dtype=torch.float64, device=dev, generator=gen) - 0.5
        s = torch.rand(k, dtype=torch.float64, device=dev, generator=gen) - 0.5
        jobs.append((u, s, m["dims"], m["perm"], m["factor"], 1.0 if m["acc"] else 0.0))
        total_b += k * (24 if m["acc"] else 16)
    b = Batch(jobs)
    b.capture()
    stream = torch.cuda.current_stream(dev)

    def timed(fn, reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / 1e3 / reps

    for _ in range(args.warmup):
        b.replay()
        b.launch_plain()
    torch.cuda.synchronize()
    reps = max(1, args.steps)
    t_graph = timed(b.replay, reps)
    t_plain = timed(b.launch_plain, reps)
    st = b.status()
    info = b.info()
    out = {"sorts": n, "ext4": list(ext4), "ext6": list(ext6), "status": st,
           "work_units": info["units"], "bytes_per_launch": total_b,
           "persistent_graph": {"tiles_per_s": round(n / t_graph, 1),
                                "gbs": round(total_b / t_graph / 1e9, 1),
                                "ms": round(t_graph * 1e3, 3), "launches": info["launches"],
                                "sorts_on_work_list": info["jobs"]},
           "one_launch_per_tile": {"tiles_per_s": round(n / t_plain, 1),
                                   "gbs": round(total_b / t_plain / 1e9, 1),
                                   "ms": round(t_plain * 1e3, 3), "launches": n},
           "speedup": round(t_plain / t_graph, 3)}
    b.close()
    del jobs
    torch.cuda.empty_cache()
    return out


def _timed_events(fn, reps, stream):
    import torch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / 1e3 / reps


def run_sort6(args, dev):
    """The tce_sort_6 configuration: all 720 perms at 10^6, 16^6, 20^6 and
    (12,20,16,20,12,16), sort (f = -0.5) and sortacc (f = 1.0), one timed
    launch each after an untimed pass that builds the plans.  Per shape:
    effective GB/s over all perms, its fraction of the HBM peak, the identity
    perm's GB/s (a plain streaming copy: the floor that launch latency leaves
    at that size) and the 54 CCSD(T) perms' GB/s.  L2 flushed (read-only)
    before every timed launch."""
    import torch
    import spaghetty_gb300 as S
    from spaghetty_gb300.workloads import PERMS6, SORT6_DIMS, TRIPLES_SORT6
    triples = set(TRIPLES_SORT6)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    peak, _ = peaks()
    out = {}
    for dims in SORT6_DIMS:
        n = 1
        for d in dims:
            n *= d
        u = torch.rand(n, dtype=torch.float64, device=dev) - 0.5
        y = torch.rand(n, dtype=torch.float64, device=dev) - 0.5
        evs = []
        # events collected and read at the end: the host runs ahead of the
        # GPU (each launch follows a flush), so each pair brackets only its
        # kernel
        for rep in range(2):
            if rep:
                torch.cuda.synchronize()
                gc.disable()
                host_lead(torch)
            for perm in PERMS6:
                for acc in (False, True):
                    if needs_flush(n):
                        flush_l2(flush)
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    S.sort_generic(u, y, dims, perm, 1.0 if acc else -0.5, 1.0 if acc else 0.0)
                    e1.record(stream)
                    if rep:
                        evs.append((perm, acc, e0, e1))
        torch.cuda.synchronize()
        gc.enable()
        acc_b = {"all": [0, 0.0], "triples": [0, 0.0], "identity": [0, 0.0]}
        for perm, acc, e0, e1 in evs:
            t = e0.elapsed_time(e1) / 1e3
            b = n * (24 if acc else 16)
            for k, on in (("all", True), ("triples", perm in triples), ("identity", perm == PERMS6[0])):
                if on:
                    acc_b[k][0] += b
                    acc_b[k][1] += t
        g = {k: v[0] / v[1] / 1e9 for k, v in acc_b.items()}
        if args.detail:
            with open(args.detail, "a") as fh:
                for perm, acc, e0, e1 in evs:
                    t = e0.elapsed_time(e1) / 1e3
                    fh.write(json.dumps({"dims": list(dims), "perm": list(perm), "acc": acc,
                                         "kind": S.plan(dims, perm, int(acc))["kind"],
                                         "gbs": round(n * (24 if acc else 16) / t / 1e9, 1)}) + "\n")
        out["x".join(map(str, dims))] = {
            "gbs": round(g["all"], 1), "frac_of_peak": round(g["all"] / peak, 4),
            "identity_copy_gbs": round(g["identity"], 1),
            "frac_of_identity_copy": round(g["all"] / g["identity"], 4),
            "triples_gbs": round(g["triples"], 1), "launches": len(evs),
            "l2": "flushed before every launch"}
        del u, y
    # the kernels' status word: no bounded wait gave up during the sweep
    from spaghetty_gb300._lib import lib as _lib
    out["device_status"] = int(_lib().spaghetty_device_status())
    if not args.no_cpu:
        out["cpu_baseline_16^6_triples"] = cpu_sort6_baseline(min(20.0, args.cpu_seconds))
    return out


def run_fused(args, dev):
    """The nine triples sortaccs of each group applied to one t3 tile: fused
    (one kernel, t3 read and written once) against nine sortacc launches.
    GB/s counts each path's own algorithmic bytes; speedup is in time."""
    import torch
    import spaghetty_gb300 as S
    from spaghetty_gb300.workloads import TRIPLES_SORTACC6
    stream = torch.cuda.current_stream(dev)
    res = {}
    for ext in (16, 20):
        shape = (ext,) * 6
        n = ext ** 6
        t3 = torch.rand(shape, dtype=torch.float64, device=dev) - 0.5
        srcs = [torch.rand(shape, dtype=torch.float64, device=dev) - 0.5 for _ in range(9)]
        rows = []
        for gi, perms in enumerate(TRIPLES_SORTACC6):
            facs = [1.0 if k % 3 else -1.0 for k in range(9)]

            def fused():
                S.sortacc_fused(t3, srcs, perms, facs)

            def seq():
                for x, p, f in zip(srcs, perms, facs):
                    S.sort_generic(x, t3, shape, p, f, 1.0)

            for _ in range(2):
                fused()
                seq()
            tf = _timed_events(fused, 3, stream)
            ts = _timed_events(seq, 3, stream)
            rows.append({"group": gi, "fused_ms": round(tf * 1e3, 3), "seq_ms": round(ts * 1e3, 3),
                         "fused_gbs": round((16 * n + 8 * n * 9) / tf / 1e9, 1),
                         "seq_gbs": round(9 * 24 * n / ts / 1e9, 1),
                         "speedup": round(ts / tf, 2)})
        res["%d^6" % ext] = rows
        del t3, srcs
    return res


def run_autograd(args, dev):
    """y = sum_k f_k * permute_k(x) over 3 seeded perms and its hand-written
    backward, one fused launch per direction (spaghetty_sort_fused).
    fwd_bwd_gbs counts the algorithmic bytes of the operation as a sort plus
    two sortaccs per direction (2 x 64 B/element); fused_traffic_gbs the
    fused kernels' own (3 reads of the source and one write per direction,
    2 x 32 B/element)."""
    import torch
    from spaghetty_gb300.autograd import permute_sum
    stream = torch.cuda.current_stream(dev)
    res = {}
    for dims, perms in [((24,) * 4, [(4, 3, 2, 1), (2, 4, 1, 3), (3, 1, 4, 2)]),
                        ((12,) * 6, [(6, 5, 4, 3, 2, 1), (2, 6, 1, 5, 4, 3), (4, 3, 6, 2, 1, 5)])]:
        n = 1
        for d in dims:
            n *= d
        x = (torch.rand(dims, dtype=torch.float64, device=dev) - 0.5).requires_grad_(True)
        g = torch.rand(dims, dtype=torch.float64, device=dev)

        def step():
            x.grad = None
            y = permute_sum(x, perms, (0.75, -1.25, 0.3))
            y.backward(g)

        for _ in range(3):
            step()
        t = _timed_events(step, 10, stream)
        res["x".join(map(str, dims))] = {"fwd_bwd_gbs": round(2 * (16 + 2 * 24) * n / t / 1e9, 1),
                                          "fused_traffic_gbs": round(2 * (3 * 8 + 8) * n / t / 1e9, 1),
                                          "ms": round(t * 1e3, 4)}
    return res


def run_contract(args, dev):
    """The macaroni skeleton's CCSD term (ccsd_t2_8: sort 4321, sort 2143,
    dgemm('T','N'), sort 2143) at d^6 index extents: the fused kernel in its
    exact mode (loop_dgemm's bits) and fma mode, against the same chain
    unfused -- three sort launches around cuBLAS's DGEMM (torch.matmul).
    FP64-bound; operands are L2-resident at these sizes, nothing is flushed.
    GFLOP/s counts 2*M*N*K."""
    import torch
    import spaghetty_gb300 as S
    from spaghetty_gb300.contract import contract_4x4
    stream = torch.cuda.current_stream(dev)
    res = {}
    for d in (16, 24, 32):
        d1 = d2 = d3 = d4 = d5 = d6 = d
        M, N, K = d1 * d2, d3 * d4, d5 * d6
        t = torch.rand(d5 * d6 * d1 * d2, dtype=torch.float64, device=dev) - 0.5
        v = torch.rand(d3 * d4 * d5 * d6, dtype=torch.float64, device=dev) - 0.5
        c = torch.empty(d1 * d2 * d3 * d4, dtype=torch.float64, device=dev)
        a_s = torch.empty_like(t)
        b_s = torch.empty_like(v)
        c_s = torch.empty_like(c)
        da, db = (d5, d6, d1, d2), (d3, d4, d5, d6)

        def fused(mode):
            contract_4x4(t, da, (4, 3, 2, 1), v, db, (2, 1, 4, 3), c, (2, 1, 4, 3), mode=mode)

        def unfused():
            S.sort_generic(t, a_s, da, (4, 3, 2, 1), 1.0, 0.0)
            S.sort_generic(v, b_s, db, (2, 1, 4, 3), 1.0, 0.0)
            # c_sort (column-major M x N) = a_sort^T b_sort, i.e. C-order [N][M]
            torch.matmul(b_s.view(N, K), a_s.view(M, K).t(), out=c_s.view(N, M))
            S.sort_generic(c_s, c, (d4, d3, d2, d1), (2, 1, 4, 3), 1.0, 0.0)

        row = {}
        for name, fn in (("fused_exact", lambda: fused("exact")), ("fused_fma", lambda: fused("fma")),
                         ("fused_mma", lambda: fused("mma")), ("unfused_cublas", unfused)):
            for _ in range(3):
                fn()
            tm = _timed_events(fn, 10, stream)
            row[name] = {"ms": round(tm * 1e3, 4), "gflops": round(2.0 * M * N * K / tm / 1e9, 1)}
        row["fma_vs_unfused"] = round(row["unfused_cublas"]["ms"] / row["fused_fma"]["ms"], 2)
        row["exact_vs_unfused"] = round(row["unfused_cublas"]["ms"] / row["fused_exact"]["ms"], 2)
        row["mma_vs_fma"] = round(row["fused_fma"]["ms"] / row["fused_mma"]["ms"], 2)
        res["%d^6" % d] = row
        del t, v, c, a_s, b_s, c_s
    return res


def run_contract_case(args):
    """One fused ccsd_t2_8 contraction at d^6 (profiling workload):
    --contract-case D:MODE (MODE exact or fma)."""
    import torch
    from spaghetty_gb300.contract import contract_4x4
    d_s, mode = args.contract_case.split(":")
    d = int(d_s)
    dev = torch.device("cuda", 0)
    n = d ** 4
    t = torch.rand(n, dtype=torch.float64, device=dev) - 0.5
    v = torch.rand(n, dtype=torch.float64, device=dev) - 0.5
    c = torch.empty(n, dtype=torch.float64, device=dev)
    dims = (d, d, d, d)

    def fn():
        contract_4x4(t, dims, (4, 3, 2, 1), v, dims, (2, 1, 4, 3), c, (2, 1, 4, 3), mode=mode)

    for _ in range(args.warmup):
        fn()
    tm = _timed_events(fn, args.steps, torch.cuda.current_stream(dev))
    print(json.dumps({"contract_case": args.contract_case, "ms": round(tm * 1e3, 4),
                      "gflops": round(2.0 * d ** 6 / tm / 1e9, 1)}), flush=True)


def run_case(args):
    """One sort case, W warm-up + K timed launches (the profiling workload)."""
    import torch
    import spaghetty_gb300 as S
    parts = args.case.split(":")
    dims_s, perm_s, op_s = parts[:3]
    factor = float(parts[3]) if len(parts) > 3 else 0.5
    dims = tuple(int(x) for x in dims_s.split(","))
    perm = tuple(int(x) for x in perm_s.split(","))
    op = int(op_s)
    n = 1
    for d in dims:
        n *= d
    dev = torch.device("cuda", 0)
    u = torch.rand(n, dtype=torch.float64, device=dev)
    s = torch.rand(n, dtype=torch.float64, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    g = 0.0 if op == 0 else 1.0
    times = []
    for r in range(args.warmup + args.steps):
        if needs_flush(n):
            flush_l2(flush)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        S.sort_generic(u, s, dims, perm, factor, g)
        e1.record()
        e1.synchronize()
        if r >= args.warmup:
            times.append(e0.elapsed_time(e1))
    ms = statistics.median(times)
    b = case_bytes(dims, op == 1)
    print(json.dumps({"case": args.case, "ms": round(ms, 4), "gbs": round(b / ms / 1e6, 1),
                      "plan": S.plan(dims, perm, op)}), flush=True)


def run_fused_case(args):
    """One fused triples group (profiling workload): --fused-case GROUP:EXTENT."""
    import torch
    import spaghetty_gb300 as S
    from spaghetty_gb300.workloads import TRIPLES_SORTACC6
    g, ext = (int(x) for x in args.fused_case.split(":"))
    shape = (ext,) * 6
    dev = torch.device("cuda", 0)
    t3 = torch.rand(shape, dtype=torch.float64, device=dev) - 0.5
    srcs = [torch.rand(shape, dtype=torch.float64, device=dev) - 0.5 for _ in range(9)]
    perms = TRIPLES_SORTACC6[g]
    facs = [1.0 if k % 3 else -1.0 for k in range(9)]
    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        S.sortacc_fused(t3, srcs, perms, facs)
    t = _timed_events(lambda: S.sortacc_fused(t3, srcs, perms, facs), max(1, args.steps), stream)
    n = ext ** 6
    print(json.dumps({"fused_case": args.fused_case, "ms": round(t * 1e3, 4),
                      "gbs": round((16 * n + 72 * n) / t / 1e9, 1)}), flush=True)


def run_batched_case(args):
    """A reduced batched mix (profiling workload): --batched-case
    N:E4LO-E4HI:E6LO-E6HI, e.g. 512:8-40:6-12."""
    import torch
    n_s, e4, e6 = args.batched_case.split(":")
    ext4 = tuple(int(x) for x in e4.split("-"))
    ext6 = tuple(int(x) for x in e6.split("-"))
    r = run_batched(args, torch.device("cuda", 0), ext4=ext4, ext6=ext6, n=int(n_s))
    print(json.dumps({"batched_case": args.batched_case, **r}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--batched-case", default=None,
                    help="N:E4LO-E4HI:E6LO-E6HI: time one reduced batched mix")
    ap.add_argument("--fused-case", default=None, help="GROUP:EXTENT: time one fused triples group")
    ap.add_argument("--contract-case", default=None,
                    help="D:MODE: time one fused ccsd_t2_8 contraction at D^6 (MODE exact|fma)")
    ap.add_argument("--case", default=None,
                    help="dims:perm:op[:factor] (op 0 sort, 1 sortacc; factor 0.5): time one case")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-secondary", action="store_true")
    ap.add_argument("--detail", default=None, help="write per-case GB/s (JSON lines) here")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.case:
        run_case(args)
        return
    if args.fused_case:
        run_fused_case(args)
        return
    if args.contract_case:
        run_contract_case(args)
        return
    if args.batched_case:
        run_batched_case(args)
        return
    if args.impl == "reference":
        line = run_reference(args, ws, rank)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    if args.warmup < 3:
        args.warmup = 3
    import torch
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo", init_method="env://")
    line = run_ours(args, ws, rank, local)
    if ws > 1:
        torch.distributed.barrier()        # rank 0's extra sections are done too
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
