"""Kernel generator: emits the compiled sm_103a variant set.

The reference generates one Fortran/C loop nest per (permutation, loop order)
and lets a tuner pick the fastest (trunk/generator2.py:48-443 emitters,
trunk/generator2.py:446-629 tuner).  Here the search space is not the loop
order but the shape of the staging box and the CTA that moves it, so the
generator emits, for every arithmetic case (the generated nests'
(factor, acc_factor) cases, trunk/generator2.py:57-130, with the factor split
into 1, -1, +-2^k and any other value), every kernel family
at every (threads, elements-per-thread) point the planner and the autotuner
may pick.  Each output file holds one arithmetic case so that the build can
compile them in parallel; each exposes a table of (kind, op, threads, ept,
function) entries the C-ABI dispatcher searches.
"""
from __future__ import annotations

import os

OPS = {0: "OP_SORT_ONE", 1: "OP_SORT_NEG", 2: "OP_SORT_POW2", 3: "OP_SORT_ANY",
       4: "OP_ACC_ONE", 5: "OP_ACC_NEG", 6: "OP_ACC_POW2", 7: "OP_ACC_ANY", 8: "OP_GEN"}
THREADS = (128, 256, 512)
EPTS = (1, 2, 4, 8)
FLAT_VEC = (1, 2)

HEADER = """// GENERATED by spaghetty_gb300/generator.py -- do not edit.
// Variant table for arithmetic case {opname}.
#include "kernels.cuh"
#include "tma.cuh"
"""
TMA_THREADS = (128, 256)
TMA_EPTS = (8, 16)
TMA_STAGES = (2, 3, 4, 6)
WARP_KS = (1, 2, 3, 4)     # warp-shuffle transpose: registers per lane (tile <= 32*K)


STAGES = (2, 3)


def variants(op: int):
    """(kind, threads, ept, stages, function) for every compiled variant."""
    out = []
    for nt in THREADS:
        for ept in EPTS:
            out.append(("KIND_TILED", nt, ept, 0, "spg_tiled<%d, %d, %s>" % (nt, ept, OPS[op])))
            if ept >= 2:
                for st in STAGES:
                    out.append(("KIND_TILED", nt, ept, st,
                                "spg_tiled_async<%d, %d, %s, %d>" % (nt, ept, OPS[op], st)))
    for nt in THREADS:
        for ept in EPTS:
            out.append(("KIND_DIRECT", nt, ept, 0, "spg_direct<%d, %d, %s>" % (nt, ept, OPS[op])))
    for vec in FLAT_VEC:
        out.append(("KIND_FLAT", 256, vec, 0, "spg_flat<%s, %d>" % (OPS[op], vec)))
    for nt in TMA_THREADS:
        for ept in TMA_EPTS:
            for st in TMA_STAGES:
                out.append(("KIND_TMA", nt, ept, st,
                            "spg_tiled_tma<%d, %d, %s, %d>" % (nt, ept, OPS[op], st)))
    for k in WARP_KS:
        out.append(("KIND_WARP", 256, k, 0, "spg_warp_tr<%s, %d>" % (OPS[op], k)))
    return out


def emit_op(op: int) -> str:
    lines = [HEADER.format(opname=OPS[op])]
    lines.append("static const SpgKernelEntry kEntries[] = {")
    for kind, nt, ept, st, fn in variants(op):
        lines.append("    {%s, %s, %d, %d, %d, (const void *)&%s}," % (kind, OPS[op], nt, ept, st, fn))
    lines.append("};")
    lines.append("const SpgKernelEntry *spg_kernels_op%d(int *n) {" % op)
    lines.append("    *n = (int)(sizeof(kEntries) / sizeof(kEntries[0]));")
    lines.append("    return kEntries;")
    lines.append("}")
    return "\n".join(lines) + "\n"


def emit_all(outdir: str) -> list[str]:
    """Write kernels_op<N>.cu for every arithmetic case; returns the paths
    (files are rewritten only when their text changes)."""
    paths = []
    for op in OPS:
        path = os.path.join(outdir, "kernels_op%d.cu" % op)
        text = emit_op(op)
        old = None
        if os.path.exists(path):
            with open(path) as fh:
                old = fh.read()
        if old != text:
            with open(path, "w") as fh:
                fh.write(text)
        paths.append(path)
    return paths


if __name__ == "__main__":
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc")
    for p in emit_all(here):
        print(p)
