"""The TCE contraction with its operand and result sorts fused
(spaghetty_contract_4x4, ccsd_t2_8 in include/spaghetty_gb300.h).

The reference builds a contraction as sort -> DGEMM('T','N') -> sort
(branches/old/python/macaroni/ccsd_t2_8_skeleton.F:174-184); here one kernel
reads the unsorted operands and writes the sorted result.
"""
from __future__ import annotations

import ctypes
from typing import Sequence

import numpy as np
import torch

from ._lib import check, int_array, lib

MODES = {"exact": 0, "fma": 1, "mma": 2}


def contract_shapes(dims_a: Sequence[int], perm_a: Sequence[int], dims_b: Sequence[int],
                    perm_b: Sequence[int], perm_c: Sequence[int]):
    """(M, N, K, dims of the result) for contract_4x4's arguments."""
    sa = [int(dims_a[p - 1]) for p in perm_a]
    sb = [int(dims_b[p - 1]) for p in perm_b]
    if sa[2:] != sb[2:]:
        raise ValueError("contracted dims differ: %s vs %s" % (sa[2:], sb[2:]))
    cs = [sb[0], sb[1], sa[0], sa[1]]
    return sa[0] * sa[1], sb[0] * sb[1], sa[2] * sa[3], tuple(cs[p - 1] for p in perm_c)


def contract_4x4(a, dims_a, perm_a, b, dims_b, perm_b, c, perm_c, alpha=1.0, factor=1.0,
                 acc_factor=0.0, mode="exact", stream=None):
    """c (=|+=) factor * sort_{perm_c}( sort_{perm_a}(a)[M,K] x sort_{perm_b}(b)[N,K]^T )
    on CUDA FP64 tensors, queued on torch's current stream (or ``stream``).
    ``mode`` "exact" adds the products in k order with every product and sum
    rounded (the skeleton's loop_dgemm bits); "fma" uses fused multiply-adds;
    "mma" FP64 matrix instructions (mma.sync .f64)."""
    _, _, _, dims_c = contract_shapes(dims_a, perm_a, dims_b, perm_b, perm_c)
    for t in (a, b, c):
        if t.dtype != torch.float64 or not t.is_cuda or not t.is_contiguous():
            raise TypeError("operands must be contiguous CUDA FP64 tensors")
    for t, dims, name in ((a, dims_a, "a"), (b, dims_b, "b"), (c, dims_c, "c")):
        n = 1
        for d in dims:
            n *= int(d)
        if t.numel() != n:
            raise ValueError("%s has %d elements, its dims %s need %d" % (name, t.numel(), tuple(dims), n))
    if stream is None:
        stream = torch.cuda.current_stream(c.device).cuda_stream
    rc = lib().spaghetty_contract_4x4(
        ctypes.c_void_p(a.data_ptr()), int_array(dims_a), int_array(perm_a),
        ctypes.c_void_p(b.data_ptr()), int_array(dims_b), int_array(perm_b),
        ctypes.c_void_p(c.data_ptr()), int_array(perm_c), float(alpha), float(factor),
        float(acc_factor), MODES[mode], ctypes.c_void_p(int(stream)))
    check(rc, "contract_4x4")
    return c


def ccsd_t2_8(a_raw, b_raw, c_done, dims: Sequence[int]):
    """The skeleton's subroutine through its C-ABI drop-in: c_done (dims
    (d3,d4,d1,d2)) = sum over (p5,p6) of b_raw (d3,d4,d5,d6) times a_raw
    (d5,d6,d1,d2); host (numpy) or device (torch) buffers, synchronous."""
    d1, d2, d3, d4, d5, d6 = (int(x) for x in dims)
    for t, need, name in ((a_raw, d5 * d6 * d1 * d2, "a_raw"), (b_raw, d3 * d4 * d5 * d6, "b_raw"),
                          (c_done, d1 * d2 * d3 * d4, "c_done")):
        # the C drop-in reads and writes 8 bytes per element from the start
        # of each buffer: anything but contiguous FP64 would run past its end
        if isinstance(t, torch.Tensor):
            if t.dtype != torch.float64 or not t.is_contiguous():
                raise TypeError("%s must be a contiguous FP64 tensor" % name)
        elif getattr(t, "dtype", None) != np.float64 or not t.flags.c_contiguous:
            raise TypeError("%s must be a C-contiguous float64 array" % name)
        n = t.numel() if isinstance(t, torch.Tensor) else t.size
        if n < need:
            raise ValueError("%s has %d elements, the dims need %d" % (name, n, need))

    def ptr(t):
        return ctypes.c_void_p(t.data_ptr() if isinstance(t, torch.Tensor) else t.ctypes.data)

    def iref(v):
        return ctypes.byref(ctypes.c_int(int(v)))

    sizes = [a_raw.size if not isinstance(a_raw, torch.Tensor) else a_raw.numel(),
             b_raw.size if not isinstance(b_raw, torch.Tensor) else b_raw.numel(),
             c_done.size if not isinstance(c_done, torch.Tensor) else c_done.numel()]
    rc = lib().ccsd_t2_8_status(ptr(a_raw), iref(sizes[0]), ptr(b_raw), iref(sizes[1]),
                                ptr(c_done), iref(sizes[2]), iref(d1), iref(d2), iref(d3),
                                iref(d4), iref(d5), iref(d6))
    check(rc, "ccsd_t2_8")
    return c_done
