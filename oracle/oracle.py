"""Parity oracle -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module, and only as the checker.  The product
library (``spaghetty_gb300``) never calls it and has no CPU fallback.

Two restatements of the reference's sort/sortacc, which must agree bit for bit:

* ``old_sort_*`` / ``old_sortacc_*`` -- ctypes bindings to ``old_sort.c``, a C
  restatement of NWChem's ``trunk/old_sort.f`` (file:line cited in the C
  source), compiled with ``-ffp-contract=off``.
* ``np_sort`` -- the same arithmetic with numpy (one rounded multiply, then one
  rounded add), usable at sizes where the scalar C loop is slow.

Layout convention (trunk/old_sort.f:54-55, trunk/generator2.py:76): the input
``u`` with dims (d1..dr) is a flat buffer whose LAST index is stride-1 (C order
``u[d1]..[dr]``); the output for 1-based permutation p has dims
(d_{p1}..d_{pr}) and equals ``f * u.transpose(p-1)`` in C order.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
SRC_PATH = os.path.join(HERE, "old_sort.c")
SRC_PATHS = [SRC_PATH, os.path.join(HERE, "loop_dgemm.c")]

_lib = None


def build(force: bool = False) -> str:
    """Compile old_sort.c and loop_dgemm.c into liboracle.so (gcc, no FMA
    contraction)."""
    if force or not os.path.exists(LIB_PATH) or (
            os.path.getmtime(LIB_PATH) < max(os.path.getmtime(p) for p in SRC_PATHS)):
        tmp = LIB_PATH + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-std=c99", "-ffp-contract=off",
                               "-fPIC", "-shared"] + SRC_PATHS + ["-o", tmp])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.oracle_sort_generic.argtypes = [ctypes.c_int, dp, dp, ip, ip,
                                          ctypes.c_double, ctypes.c_double]
        L.oracle_sort_generic.restype = ctypes.c_int
        for r, n in ((2, 2), (4, 4), (6, 6)):
            for acc in ("", "acc"):
                fn = getattr(L, "oracle_old_sort%s_%d" % (acc, r))
                fn.argtypes = [dp, dp] + [ip] * (2 * n) + [dp]
                fn.restype = None
        for acc in ("", "acc"):
            fn = getattr(L, "oracle_old_sort%s_8" % acc)
            fn.argtypes = [dp, dp, ip, ip, dp]
            fn.restype = None
        L.oracle_loop_dgemm.argtypes = [ctypes.c_double, ctypes.c_double, dp, dp, dp] + \
            [ctypes.c_int] * 7
        L.oracle_loop_dgemm.restype = ctypes.c_int
        _lib = L
    return _lib


def _dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _iref(v: int):
    return ctypes.byref(ctypes.c_int(int(v)))


def old_sort(u: np.ndarray, dims: Sequence[int], perm: Sequence[int],
             factor: float, out: np.ndarray | None = None,
             acc: bool = False) -> np.ndarray:
    """Call the C restatement of old_sort_r / old_sortacc_r (r = len(dims)).

    ``perm`` is 1-based as in the reference.  For ``acc`` the output buffer
    ``out`` is updated in place (it must hold the prior values)."""
    r = len(dims)
    n = int(np.prod(dims)) if r else 1
    u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
    assert u.size == n
    if out is None:
        out = np.zeros(n, dtype=np.float64)
    flat = out.reshape(-1)
    assert flat.size == n and flat.dtype == np.float64
    L = lib()
    f = ctypes.byref(ctypes.c_double(float(factor)))
    name = "oracle_old_sort%s_%d" % ("acc" if acc else "", r)
    if r in (2, 4, 6):
        args = [_iref(d) for d in dims] + [_iref(p) for p in perm]
        getattr(L, name)(_dptr(u), _dptr(flat), *args, f)
    elif r == 8:
        d = (ctypes.c_int * 8)(*dims)
        p = (ctypes.c_int * 8)(*perm)
        getattr(L, name)(_dptr(u), _dptr(flat), d, p, f)
    else:
        return sort_generic(u, dims, perm, factor, 1.0 if acc else 0.0, out)
    return out


def sort_generic(u: np.ndarray, dims: Sequence[int], perm: Sequence[int],
                 factor: float, acc_factor: float,
                 out: np.ndarray | None = None) -> np.ndarray:
    """Any rank 1..8 with the generated nests' two-factor update
    (trunk/generator2.py:48-130): g=0 sort, g=1 sortacc, else g*y + f*x."""
    r = len(dims)
    n = int(np.prod(dims))
    u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
    if out is None:
        out = np.zeros(n, dtype=np.float64)
    flat = out.reshape(-1)
    d = (ctypes.c_int * r)(*dims)
    p = (ctypes.c_int * r)(*perm)
    rc = lib().oracle_sort_generic(r, _dptr(u), _dptr(flat), d, p,
                                   float(factor), float(acc_factor))
    if rc != 0:
        raise ValueError("oracle rejected rank/permutation")
    return out


def np_sort(u: np.ndarray, dims: Sequence[int], perm: Sequence[int],
            factor: float, acc_factor: float = 0.0,
            out: np.ndarray | None = None) -> np.ndarray:
    """numpy restatement with the same roundings as old_sort/old_sortacc:
    product rounded once, then (sortacc) the sum rounded once.  Returns the
    flat output (C order, output dims (d_{p1}..d_{pr}))."""
    dims = tuple(int(d) for d in dims)
    axes = tuple(int(p) - 1 for p in perm)
    x = np.asarray(u, dtype=np.float64).reshape(dims)
    prod = np.multiply(x, np.float64(factor)).transpose(axes).reshape(-1)
    if acc_factor == 0.0:
        return np.ascontiguousarray(prod)
    assert out is not None
    y = np.asarray(out, dtype=np.float64).reshape(-1)
    if acc_factor == 1.0:
        return np.add(y, prod)
    return np.add(np.multiply(y, np.float64(acc_factor)), prod)


def np_permuted(u: np.ndarray, dims: Sequence[int], perm: Sequence[int]) -> np.ndarray:
    """The index map of old_sort_r alone (trunk/old_sort.f:54-58: element ia
    of the input goes to position ib of the output): the input's elements in
    output order, flat C order over (d_{p1}..d_{pr}), no arithmetic.  With
    it, a sort is ``np.multiply(T, f)`` and a sortacc ``np.add(y,
    np.multiply(T, f))`` -- np_sort's roundings -- so the full-size tests
    permute once per permutation and reuse the result for every factor."""
    dims = tuple(int(d) for d in dims)
    axes = tuple(int(p) - 1 for p in perm)
    x = np.asarray(u, dtype=np.float64).reshape(dims)
    return np.ascontiguousarray(x.transpose(axes)).reshape(-1)


def loop_dgemm(alpha: float, beta: float, a: np.ndarray, b: np.ndarray, c: np.ndarray,
               row_a: int, col_a: int, row_b: int, col_b: int, row_c: int, col_c: int,
               case: int) -> np.ndarray:
    """The skeleton's reference DGEMM (loop_dgemm.c, restating
    branches/old/python/macaroni/ccsd_t2_8_skeleton.F:214-292) on flat
    column-major buffers; updates ``c`` in place and returns it."""
    a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
    b = np.ascontiguousarray(b, dtype=np.float64).reshape(-1)
    flat = c.reshape(-1)
    assert flat.dtype == np.float64 and flat.flags.c_contiguous
    rc = lib().oracle_loop_dgemm(float(alpha), float(beta), _dptr(a), _dptr(b), _dptr(flat),
                                 row_a, col_a, row_b, col_b, row_c, col_c, case)
    if rc != 0:
        raise ValueError("loop_dgemm: shapes do not match case %d" % case)
    return c


def contract_4x4(a: np.ndarray, dims_a: Sequence[int], perm_a: Sequence[int],
                 b: np.ndarray, dims_b: Sequence[int], perm_b: Sequence[int],
                 perm_c: Sequence[int], alpha: float = 1.0, factor: float = 1.0,
                 acc_factor: float = 0.0, out: np.ndarray | None = None) -> np.ndarray:
    """The skeleton's sort -> DGEMM('T','N') -> sort chain
    (ccsd_t2_8_skeleton.F:174-184) with loop_dgemm case 3 as the DGEMM, on a
    zeroed c_sort with beta = 1: a_sort = sort(a, perm_a) read as the
    column-major K x M matrix, b_sort = sort(b, perm_b) as K x N, c_sort
    (M x N column-major, i.e. C-order dims (SB0,SB1,SA0,SA1)) =
    Sum_k (alpha*a)*b, then the result sort (factor, acc_factor) into
    ``out``.  Returns the flat result."""
    sa = [int(dims_a[p - 1]) for p in perm_a]
    sb = [int(dims_b[p - 1]) for p in perm_b]
    assert sa[2:] == sb[2:], "contracted dims differ"
    M, N, K = sa[0] * sa[1], sb[0] * sb[1], sa[2] * sa[3]
    a_sort = sort_generic(a, dims_a, perm_a, 1.0, 0.0)
    b_sort = sort_generic(b, dims_b, perm_b, 1.0, 0.0)
    c_sort = np.zeros(M * N)
    loop_dgemm(alpha, 1.0, a_sort, b_sort, c_sort, K, M, K, N, M, N, 3)
    cs = (sb[0], sb[1], sa[0], sa[1])
    if out is None:
        out = np.zeros(M * N)
    return sort_generic(c_sort, cs, perm_c, factor, acc_factor, out)


def init_array(dims: Sequence[int]) -> np.ndarray:
    """Integer-valued fixture of trunk/tester_futil.F:139-185 (init_4d_array /
    init_6d_array): x(i,j,k,l) = i + j*a + k*a*b + l*a*b*c over the Fortran
    (column-major) array x(a,b,c,d), 1-based.  Returned as the flat buffer the
    routines see."""
    dims = [int(d) for d in dims]
    # x(i,j,k,l) at flat position m = (i-1) + a(j-1) + ab(k-1) + abc(l-1) is
    # i + ja + kab + labc = m + (1 + a + ab + abc): a ramp with that offset
    # (and likewise for rank 6).
    n = int(np.prod(dims))
    const = 0
    scale = 1
    for d in dims:
        const += scale
        scale *= d
    return np.arange(n, dtype=np.float64) + float(const)


def seeded_uniform(n: int, seed: int) -> np.ndarray:
    """Seeded uniform(-1,1) FP64 values (numpy PCG64)."""
    return np.random.Generator(np.random.PCG64(seed)).uniform(-1.0, 1.0, n)


def fixture_values(n: int, seed: int) -> np.ndarray:
    """Platform-independent uniform[-1,1) values for committed fixtures:
    splitmix64 (Steele, Lea & Flood, OOPSLA 2014) of (seed, i), top 53 bits
    scaled to [0,2) and shifted by -1 -- every step exact in binary64."""
    with np.errstate(over="ignore"):
        x = (np.arange(n, dtype=np.uint64) + np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15))
        x = x + np.uint64(0x9E3779B97F4A7C15)
        z = x
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    k = (z >> np.uint64(11)).astype(np.float64)
    return k * (2.0 ** -52) - 1.0


def digest(a: np.ndarray) -> str:
    """SHA-256 of the FP64 bytes (little-endian), the fixture comparison key."""
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()
