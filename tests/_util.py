"""Shared helpers for the tests (golden fixtures, C-ABI calls on device
buffers, bitwise comparison)."""
from __future__ import annotations

import ctypes
import json
import os

import numpy as np

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


def golden() -> dict:
    with open(os.path.join(HERE, "golden", "golden.json")) as fh:
        return json.load(fh)["cases"]


def parse_key(key: str):
    dims, inp, perm, f, g = key.split("|")
    return (tuple(int(x) for x in dims.split(",")), inp, tuple(int(c) for c in perm),
            float(f), float(g))


def golden_inputs(dims, inp):
    """Regenerate the committed fixtures' inputs (see tests/golden/make_golden.py)."""
    n = int(np.prod(dims))
    if inp == "init_array":
        return O.init_array(dims), np.zeros(n)
    tag = int(inp[len("fixture"):])
    return O.fixture_values(n, 1000 + tag), O.fixture_values(n, 2000 + tag)


def bits_equal(a: np.ndarray, b: np.ndarray) -> bool:
    a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
    b = np.ascontiguousarray(b, dtype=np.float64).reshape(-1)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def first_mismatch(a, b):
    a = np.asarray(a).reshape(-1)
    b = np.asarray(b).reshape(-1)
    idx = np.nonzero(a.view(np.uint64) != b.view(np.uint64))[0]
    if idx.size == 0:
        return None
    i = int(idx[0])
    return i, float(a[i]), float(b[i]), int(idx.size)


def cref(v: int):
    return ctypes.byref(ctypes.c_int(int(v)))


def call_dropin(name: str, u_ptr: int, s_ptr: int, dims, perm, factor: float):
    """Call tce_sort_<r>/tce_sortacc_<r> (void, Fortran-style) through the C ABI."""
    from spaghetty_gb300._lib import lib
    fn = getattr(lib(), name)
    args = [ctypes.c_void_p(u_ptr), ctypes.c_void_p(s_ptr)]
    args += [cref(d) for d in dims] + [cref(p) for p in perm]
    args += [ctypes.byref(ctypes.c_double(float(factor)))]
    return fn(*args)


def call_status(name: str, u_ptr: int, s_ptr: int, dims, perm, factor: float) -> int:
    from spaghetty_gb300._lib import lib
    fn = getattr(lib(), name)
    args = [ctypes.c_void_p(u_ptr), ctypes.c_void_p(s_ptr)]
    args += [cref(d) for d in dims] + [cref(p) for p in perm]
    args += [ctypes.byref(ctypes.c_double(float(factor)))]
    return int(fn(*args))
