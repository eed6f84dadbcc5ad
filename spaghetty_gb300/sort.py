"""Python face of the library, mirroring the reference's routines.

``tce_sort_4(unsorted, sorted, a, b, c, d, i, j, k, l, factor)`` and friends
keep the reference's argument order and meaning (trunk/tce_sort4_switch.F:1-8,
branches/spaghetty3/python/tce_sort_hirata.F:62-63,143-144,
branches/spaghetty2/tce_sortacc_hirata.F:49,120): ``unsorted`` has dims
(a,b,c,d) with the LAST index stride-1, the permutation (i,j,k,l) is 1-based,
and ``sorted`` receives dims (d_i, d_j, d_k, d_l).  Buffers may be CUDA
tensors (work is enqueued on torch's current stream), CPU tensors or numpy
arrays (the library stages them through the GPU and returns when done).

``sort`` / ``sortacc`` are the tensor-level forms used by the autograd and
batched layers.  Every call goes through the C ABI; an invalid permutation or
shape raises ``SpaghettyError`` (the reference prints 'something is
wrong...' and returns, trunk/tce_sort4_switch.F:58-60; the C drop-ins keep
that behaviour).
"""
from __future__ import annotations

import ctypes
import math
from typing import Sequence

import numpy as np

from ._lib import SpaghettyError, check, int_array, lib

try:
    import torch
except ImportError:  # torch is optional for numpy-only callers
    torch = None


def _is_cuda_tensor(x) -> bool:
    return torch is not None and isinstance(x, torch.Tensor) and x.is_cuda


def _ptr(x):
    if torch is not None and isinstance(x, torch.Tensor):
        if x.dtype != torch.float64:
            raise TypeError("spaghetty_gb300 sorts FP64 tensors, got %s" % x.dtype)
        if not x.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return ctypes.c_void_p(x.data_ptr())
    if isinstance(x, np.ndarray):
        if x.dtype != np.float64:
            raise TypeError("spaghetty_gb300 sorts FP64 arrays, got %s" % x.dtype)
        if not x.flags.c_contiguous:
            raise ValueError("array must be C-contiguous")
        return ctypes.c_void_p(x.ctypes.data)
    raise TypeError("expected a torch.Tensor or numpy.ndarray")


def _numel(x) -> int:
    return int(x.numel()) if (torch is not None and isinstance(x, torch.Tensor)) else int(x.size)


# ctypes int arrays of the (dims, perm) tuples seen so far: building them is
# a large part of a small call's host time
_ARRAYS: dict = {}


def _int_array_cached(vals):
    key = tuple(int(v) for v in vals)
    a = _ARRAYS.get(key)
    if a is None:
        if len(_ARRAYS) > 4096:
            _ARRAYS.clear()
        a = _ARRAYS[key] = int_array(key)
    return a


def _raw_stream(dev_index: int) -> int:
    """torch's current stream on the device, as a cudaStream_t value."""
    get = getattr(torch._C, "_cuda_getCurrentRawStream", None)
    if get is not None:
        return int(get(dev_index))
    return int(torch.cuda.current_stream(dev_index).cuda_stream)


def sort_generic(unsorted, sorted, dims: Sequence[int], perm: Sequence[int],
                 factor: float, acc_factor: float = 0.0, stream=None) -> None:
    """Two-factor form of the generated nests (trunk/generator2.py:57-130):
    acc_factor 0 -> sort, 1 -> sortacc, else sorted = g*sorted + f*unsorted."""
    rank = len(dims)
    if len(perm) != rank:
        raise ValueError("dims and perm differ in length")
    n = math.prod(int(d) for d in dims) if rank else 0
    for t in (unsorted, sorted):
        if _numel(t) != n:
            raise ValueError("buffer holds %d elements, dims need %d" % (_numel(t), n))
    d = _int_array_cached(dims)
    p = _int_array_cached(perm)
    L = lib()
    if _is_cuda_tensor(unsorted) and _is_cuda_tensor(sorted):
        # the library runs on the device that holds the tensors
        if stream is None:
            stream = _raw_stream(unsorted.device.index)
        rc = L.spaghetty_sort_async(rank, _ptr(unsorted), _ptr(sorted), d, p, float(factor),
                                    float(acc_factor), ctypes.c_void_p(int(stream)))
    else:
        if _is_cuda_tensor(unsorted) or _is_cuda_tensor(sorted):
            torch.cuda.current_stream().synchronize()
        rc = L.spaghetty_sort(rank, _ptr(unsorted), _ptr(sorted), d, p,
                              float(factor), float(acc_factor))
    check(rc, "sort rank %d perm %s" % (rank, tuple(perm)))


def _mirror(rank: int, acc: bool):
    def fn(unsorted, sorted, *args):
        if len(args) != 2 * rank + 1:
            raise TypeError("expected %d dims, %d permutation indices and a factor" % (rank, rank))
        dims, perm, factor = args[:rank], args[rank:2 * rank], args[2 * rank]
        sort_generic(unsorted, sorted, dims, perm, factor, 1.0 if acc else 0.0)
    fn.__name__ = "tce_sort%s_%d" % ("acc" if acc else "", rank)
    fn.__doc__ = ("Mirror of %s(unsorted, sorted, <%d dims>, <%d perm>, factor); see "
                  "trunk/old_sort.f for the reference arithmetic." % (fn.__name__, rank, rank))
    return fn


tce_sort_2 = _mirror(2, False)
tce_sortacc_2 = _mirror(2, True)
tce_sort_4 = _mirror(4, False)
tce_sortacc_4 = _mirror(4, True)
tce_sort_6 = _mirror(6, False)
tce_sortacc_6 = _mirror(6, True)
tce_sort_8 = _mirror(8, False)
tce_sortacc_8 = _mirror(8, True)


def permuted_shape(shape: Sequence[int], perm: Sequence[int]) -> tuple:
    return tuple(int(shape[p - 1]) for p in perm)


def sort(x, perm: Sequence[int], factor: float = 1.0, out=None):
    """Return factor * x permuted by the 1-based ``perm`` (C order), i.e.
    ``factor * x.permute(p-1)`` materialised contiguously, computed by the
    GPU kernels.  ``x`` is a CUDA FP64 tensor of shape (d1..dr)."""
    shape = tuple(x.shape)
    oshape = permuted_shape(shape, perm)
    if out is None:
        out = torch.empty(oshape, dtype=x.dtype, device=x.device)
    sort_generic(x, out, shape, perm, factor, 0.0)
    return out


def sortacc(x, perm: Sequence[int], out, factor: float = 1.0, acc_factor: float = 1.0):
    """out = acc_factor*out + factor * x.permute(p-1), in place on ``out``."""
    sort_generic(x, out, tuple(x.shape), perm, factor, acc_factor)
    return out


def plan(dims: Sequence[int], perm: Sequence[int], op: int = 0):
    """The planner's folded problem and box for (dims, perm): a dict."""
    from ._lib import PlanInfo
    info = PlanInfo()
    rc = lib().spaghetty_plan_query(len(dims), int_array(dims), int_array(perm), int(op),
                                    ctypes.byref(info))
    check(rc, "plan")
    r = info.rank
    return {
        "kind": ("empty", "flat", "direct", "tiled", "tma", "warp")[info.kind],
        "rank": r,
        "dims": [int(info.dims[q]) for q in range(r)],
        "perm": [int(info.perm[q]) for q in range(r)],
        "box": [int(info.box[q]) for q in range(r)],
        "threads": info.threads, "ept": info.ept, "ntiles": int(info.ntiles),
        "run_in": info.run_in, "run_out": info.run_out,
        "pad": info.pad_period if info.kind != 4 else 0,
        "skew": info.pad_period if info.kind == 4 else 0,
        "masked": bool(info.masked), "stages": info.stages, "smem_bytes": info.smem_bytes,
    }


__all__ = ["tce_sort_2", "tce_sortacc_2", "tce_sort_4", "tce_sortacc_4", "tce_sort_6",
           "tce_sortacc_6", "tce_sort_8", "tce_sortacc_8", "sort", "sortacc", "sort_generic",
           "plan", "permuted_shape", "SpaghettyError"]


# (source shapes, perms, output shape) of fused calls seen so far ->
# (rank, dims array, perms array): validated and built once, since at small
# sizes a fused call's host time is mostly this bookkeeping
_FUSED: dict = {}


def _fused_arrays(shapes, perms, out_shape):
    key = (shapes, perms, out_shape)
    ent = _FUSED.get(key)
    if ent is not None:
        return ent
    rank = len(shapes[0])
    dims, pp = [], []
    for shp, p in zip(shapes, perms):
        if len(shp) != rank or len(p) != rank:
            raise ValueError("every source must have the output's rank")
        if permuted_shape(shp, p) != out_shape:
            raise ValueError("permuted source shape %s != output shape %s"
                             % (permuted_shape(shp, p), out_shape))
        dims += [int(d) for d in shp]
        pp += [int(v) for v in p]
    if len(_FUSED) > 4096:
        _FUSED.clear()
    ent = _FUSED[key] = (rank, int_array(dims), int_array(pp))
    return ent


def _check_fp64_cuda(t, what):
    if t.dtype != torch.float64 or not t.is_contiguous() or not t.is_cuda:
        raise TypeError("%s must be contiguous CUDA FP64 tensors" % what)


def _fused(entry, out, sources, perms, factors, stream):
    n = len(sources)
    if not (len(perms) == n == len(factors)) or n == 0:
        raise ValueError("sources, perms and factors must have one entry per term")
    _check_fp64_cuda(out, "the output")
    seen = None
    for s in sources:
        if s is not seen:
            _check_fp64_cuda(s, "sources")
            seen = s
    rank, dims, pp = _fused_arrays(tuple(tuple(s.shape) for s in sources),
                                   tuple(tuple(p) for p in perms), tuple(out.shape))
    if stream is None:
        stream = _raw_stream(out.device.index)
    src_arr = (ctypes.c_void_p * n)(*[s.data_ptr() for s in sources])
    fac = (ctypes.c_double * n)(*[float(f) for f in factors])
    rc = getattr(lib(), entry)(rank, n, src_arr, dims, pp, fac,
                               ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(int(stream)))
    check(rc, entry)
    return out


def sortacc_fused(out, sources, perms, factors, stream=None):
    """out += sum_k factors[k] * sources[k].permute(perms[k] - 1), added in k
    order with the rounding of consecutive tce_sortacc calls, reading and
    writing ``out`` once (spaghetty_sortacc_fused).  CUDA FP64 tensors; each
    source has its own shape (the dims a tce_sortacc call would pass)."""
    return _fused("spaghetty_sortacc_fused", out, sources, perms, factors, stream)


def sort_fused(out, sources, perms, factors, stream=None):
    """out = sum_k factors[k] * sources[k].permute(perms[k] - 1): the first
    term as tce_sort computes it, the others added in k order as tce_sortacc
    does, without reading ``out`` (spaghetty_sort_fused).  Sources may
    repeat."""
    return _fused("spaghetty_sort_fused", out, sources, perms, factors, stream)
