"""Batched sorts: one persistent kernel launch over a device work list.

A CCSD(T) sweep issues thousands of uneven tce_sort_4/6 and tce_sortacc_6
calls (the nine sortaccs per triples tile listed in
branches/spaghetty2/ccsd_t_tce_sort_list.txt).  ``Batch`` plans them once,
uploads the work list, and runs them all as one launch
(``spaghetty_batch_launch``), optionally replayed from a CUDA graph.
``launch_plain`` runs the same sorts as one launch each, for comparison.
"""
from __future__ import annotations

import ctypes
from typing import Iterable, Sequence

from ._lib import BatchEntry, SpaghettyError, check, lib

try:
    import torch
except ImportError:
    torch = None


class Batch:
    """Sorts ``(unsorted, sorted, dims, perm, factor, acc_factor)`` on device
    tensors.  The tensors must stay alive while the batch is used; outputs
    must not overlap any other buffer of the batch (inputs may be shared)."""

    def __init__(self, jobs: Iterable[tuple]):
        self._keep = []
        ents = []
        for (u, s, dims, perm, f, g) in jobs:
            e = BatchEntry()
            e.unsorted = u.data_ptr()
            e.sorted = s.data_ptr()
            e.rank = len(dims)
            for q, d in enumerate(dims):
                e.dims[q] = int(d)
            for q, p in enumerate(perm):
                e.perm[q] = int(p)
            e.factor = float(f)
            e.acc_factor = float(g)
            ents.append(e)
            self._keep.append((u, s))
        arr = (BatchEntry * max(1, len(ents)))(*ents)
        self._entries = arr
        h = ctypes.c_void_p()
        rc = lib().spaghetty_batch_create(ctypes.cast(arr, ctypes.c_void_p), len(ents),
                                          ctypes.byref(h))
        if rc:
            bad = lib().spaghetty_batch_bad_index()
            raise SpaghettyError(rc, "batch entry %d" % bad)
        self._h = h
        self._graph = None

    def info(self) -> dict:
        v = (ctypes.c_int64 * 4)()
        check(lib().spaghetty_batch_info(self._h, v), "batch info")
        return {"jobs": v[0], "units": v[1], "bytes": v[2], "smem_bytes": v[3],
                "launches": int(lib().spaghetty_batch_launches(self._h))}

    def _stream(self, stream):
        if stream is None:
            stream = torch.cuda.current_stream().cuda_stream
        return ctypes.c_void_p(int(stream))

    def launch(self, stream=None) -> None:
        """Enqueue the batch: the large sorts (2^24 elements and more by
        default, SPAGHETTY_OPT_BATCH_OWN_MIN) the single-sort planner puts on
        the TMA-staged kernel one launch each, every other sort in ONE
        persistent kernel launch."""
        check(lib().spaghetty_batch_launch(self._h, self._stream(stream)), "batch launch")

    def launch_plain(self, stream=None) -> None:
        """Enqueue the same sorts as one launch each."""
        check(lib().spaghetty_batch_launch_plain(self._h, self._stream(stream)), "batch plain")

    def capture(self):
        """Capture ``launch`` into a CUDA graph; ``replay`` then re-runs it."""
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.launch(s.cuda_stream)          # warm-up outside capture
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        with torch.cuda.graph(g):
            self.launch(torch.cuda.current_stream().cuda_stream)
        self._graph = g
        return g

    def replay(self) -> None:
        if self._graph is None:
            self.capture()
        self._graph.replay()

    def status(self, stream=None) -> int:
        """Synchronise and return the device status (0 = every job ran)."""
        return int(lib().spaghetty_batch_status(self._h, self._stream(stream)))

    def poison(self, index: int) -> None:
        check(lib().spaghetty_batch_poison(self._h, int(index)), "poison")

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().spaghetty_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def verify_plan(specs: Sequence[dict], num_sms: int = 0) -> dict:
    """Host replay of the work list a batch of these sorts would get
    (spaghetty_batch_verify, no GPU needed): specs are dicts with "dims",
    "perm", "factor" and "acc" (or "acc_factor").  Returns the counts of
    jobs, work units, boxes and elements; raises SpaghettyError naming the
    first entry whose plan fails a check."""
    arr = (BatchEntry * max(1, len(specs)))()
    for e, sp in zip(arr, specs):
        e.rank = len(sp["dims"])
        for q, d in enumerate(sp["dims"]):
            e.dims[q] = int(d)
        for q, v in enumerate(sp["perm"]):
            e.perm[q] = int(v)
        e.factor = float(sp.get("factor", 1.0))
        e.acc_factor = float(sp.get("acc_factor", 1.0 if sp.get("acc") else 0.0))
    st = (ctypes.c_int64 * 4)()
    rc = lib().spaghetty_batch_verify(ctypes.cast(arr, ctypes.c_void_p), len(specs), int(num_sms), st)
    if rc:
        raise SpaghettyError(rc, "batch entry %d" % lib().spaghetty_batch_bad_index())
    return {"jobs": st[0], "units": st[1], "boxes": st[2], "elements": st[3]}


def partition(jobs: Sequence[dict], rank: int, world: int) -> list[int]:
    """Indices of the jobs rank `rank` of `world` runs: a greedy
    largest-first assignment by bytes, so replicas get equal traffic.  The
    work list needs no exchange between ranks (every sort is independent)."""
    sizes = []
    for i, j in enumerate(jobs):
        n = 1
        for d in j["dims"]:
            n *= int(d)
        sizes.append((n * (24 if j.get("acc") else 16), i))
    sizes.sort(key=lambda t: (-t[0], t[1]))
    load = [0] * world
    owner = [0] * len(jobs)
    for b, i in sizes:
        r = min(range(world), key=lambda q: (load[q], q))
        owner[i] = r
        load[r] += b
    return [i for i in range(len(jobs)) if owner[i] == rank]
