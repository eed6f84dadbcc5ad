"""ctypes access to the reference's own generated C loop nests -- TEST
INFRASTRUCTURE ONLY (parity cross-check and the timed CPU baseline).

``oracle/_ref/libref_nests.so`` is built by ``oracle/make_ref.py`` from the
reference emitters; it is absent when neither the reference checkout nor the
generated C is available, in which case ``available()`` is False.
"""
from __future__ import annotations

import ctypes
import os
from typing import Sequence

import numpy as np

from . import make_ref

_lib = None
_index: dict | None = None


def load(build: bool = True):
    global _lib, _index
    if _lib is not None:
        return _lib
    path = make_ref.build() if build else (make_ref.LIB if os.path.exists(make_ref.LIB) else None)
    if not path or not os.path.exists(path):
        return None
    L = ctypes.CDLL(path)
    L.ref_count.argtypes = [ctypes.c_int]
    L.ref_count.restype = ctypes.c_int
    L.ref_perm.argtypes = [ctypes.c_int, ctypes.c_int]
    L.ref_perm.restype = ctypes.c_char_p
    L.ref_loop.argtypes = [ctypes.c_int, ctypes.c_int]
    L.ref_loop.restype = ctypes.c_char_p
    dp = ctypes.POINTER(ctypes.c_double)
    L.ref_call.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp,
                           ctypes.POINTER(ctypes.c_int), ctypes.c_double, ctypes.c_double]
    L.ref_call.restype = ctypes.c_int
    if hasattr(L, "ref_set_threads"):
        L.ref_set_threads.argtypes = [ctypes.c_int]
        L.ref_set_threads.restype = None
        L.ref_threads.argtypes = []
        L.ref_threads.restype = ctypes.c_int
    idx = {}
    for rank in (4, 6):
        for i in range(L.ref_count(rank)):
            key = (rank, L.ref_perm(rank, i).decode(), L.ref_loop(rank, i).decode())
            idx[key] = i
    _lib, _index = L, idx
    return L


def available() -> bool:
    try:
        return load() is not None
    except Exception:
        return False


def loops_for(rank: int, perm: Sequence[int]) -> list[str]:
    load()
    p = "".join(str(x) for x in perm)
    return [lo for (r, pp, lo) in _index if r == rank and pp == p]


def call(perm: Sequence[int], loop: str, u: np.ndarray, s: np.ndarray,
         dims: Sequence[int], factor: float, acc_factor: float) -> None:
    """Run trans_<perm>_loop_<loop> (OpenMP form) on flat FP64 buffers."""
    L = load()
    rank = len(dims)
    p = "".join(str(x) for x in perm)
    i = _index[(rank, p, loop)]
    d = (ctypes.c_int * rank)(*dims)
    dp = ctypes.POINTER(ctypes.c_double)
    assert u.dtype == np.float64 and s.dtype == np.float64
    assert u.flags.c_contiguous and s.flags.c_contiguous
    rc = L.ref_call(rank, i, u.ctypes.data_as(dp), s.ctypes.data_as(dp), d,
                    float(factor), float(acc_factor))
    if rc:
        raise ValueError("bad rank")


def set_threads(n: int) -> int:
    """Run the nests on n OpenMP threads (whatever OMP_NUM_THREADS said when
    the process started); returns the count in force."""
    L = load()
    if L is None or not hasattr(L, "ref_set_threads"):
        return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    L.ref_set_threads(int(n))
    return int(L.ref_threads())
