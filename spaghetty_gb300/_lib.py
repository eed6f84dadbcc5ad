"""ctypes binding of the in-tree C-ABI library (include/spaghetty_gb300.h).

The library is the product: there is no Python or CPU fallback.  If the
shared object is missing, ``lib()`` raises -- build it with
``python -m spaghetty_gb300.build`` (or ``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes
import os
import threading

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libspaghetty_gb300.so")

_lib = None
_lock = threading.Lock()

c_int_p = ctypes.POINTER(ctypes.c_int)
c_double_p = ctypes.POINTER(ctypes.c_double)


class PlanInfo(ctypes.Structure):
    """Mirror of spaghetty_plan_info."""
    _fields_ = [
        ("kind", ctypes.c_int),
        ("rank", ctypes.c_int),
        ("dims", ctypes.c_int64 * 8),
        ("perm", ctypes.c_int * 8),
        ("box", ctypes.c_int * 8),
        ("threads", ctypes.c_int),
        ("ept", ctypes.c_int),
        ("ntiles", ctypes.c_int64),
        ("run_in", ctypes.c_int),
        ("run_out", ctypes.c_int),
        ("pad_period", ctypes.c_int),
        ("masked", ctypes.c_int),
        ("grid", ctypes.c_int),
        ("vec", ctypes.c_int),
        ("stages", ctypes.c_int),
        ("smem_bytes", ctypes.c_int),
    ]


class BatchEntry(ctypes.Structure):
    """Mirror of spaghetty_batch_entry."""
    _fields_ = [
        ("unsorted", ctypes.c_void_p),
        ("sorted", ctypes.c_void_p),
        ("rank", ctypes.c_int),
        ("dims", ctypes.c_int * 8),
        ("perm", ctypes.c_int * 8),
        ("factor", ctypes.c_double),
        ("acc_factor", ctypes.c_double),
    ]


# Every function the header declares, with its ctypes prototype.
_R4 = [ctypes.c_void_p, ctypes.c_void_p] + [c_int_p] * 8 + [c_double_p]
_R6 = [ctypes.c_void_p, ctypes.c_void_p] + [c_int_p] * 12 + [c_double_p]
_R8 = [ctypes.c_void_p, ctypes.c_void_p] + [c_int_p] * 16 + [c_double_p]
_R2 = [ctypes.c_void_p, ctypes.c_void_p] + [c_int_p] * 4 + [c_double_p]
# ccsd_t2_8(a_raw, size_a, b_raw, size_b, c_done, size_c, dim1..dim6)
_T2_8 = [ctypes.c_void_p, c_int_p, ctypes.c_void_p, c_int_p, ctypes.c_void_p, c_int_p] + [c_int_p] * 6

c_int64_p = ctypes.POINTER(ctypes.c_int64)
_R4_I8 = [ctypes.c_void_p, ctypes.c_void_p] + [c_int64_p] * 8 + [c_double_p]
_R6_I8 = [ctypes.c_void_p, ctypes.c_void_p] + [c_int64_p] * 12 + [c_double_p]

PROTOTYPES = {
    "tce_sort_4_i8": (None, _R4_I8), "tce_sort_4_i8_": (None, _R4_I8),
    "tce_sortacc_4_i8": (None, _R4_I8), "tce_sortacc_4_i8_": (None, _R4_I8),
    "tce_sort_6_i8": (None, _R6_I8), "tce_sort_6_i8_": (None, _R6_I8),
    "tce_sortacc_6_i8": (None, _R6_I8), "tce_sortacc_6_i8_": (None, _R6_I8),
    "tce_sort_2": (None, _R2), "tce_sort_2_": (None, _R2),
    "tce_sortacc_2": (None, _R2), "tce_sortacc_2_": (None, _R2),
    "tce_sort_4": (None, _R4), "tce_sort_4_": (None, _R4),
    "tce_sortacc_4": (None, _R4), "tce_sortacc_4_": (None, _R4),
    "tce_sort_6": (None, _R6), "tce_sort_6_": (None, _R6),
    "tce_sortacc_6": (None, _R6), "tce_sortacc_6_": (None, _R6),
    "tce_sort_8": (None, _R8), "tce_sort_8_": (None, _R8),
    "tce_sortacc_8": (None, _R8), "tce_sortacc_8_": (None, _R8),
    "tce_sort_4_status": (ctypes.c_int, _R4), "tce_sortacc_4_status": (ctypes.c_int, _R4),
    "tce_sort_6_status": (ctypes.c_int, _R6), "tce_sortacc_6_status": (ctypes.c_int, _R6),
    "spaghetty_sort_async": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                            c_int_p, c_int_p, ctypes.c_double,
                                            ctypes.c_double, ctypes.c_void_p]),
    "spaghetty_sort": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                      c_int_p, c_int_p, ctypes.c_double, ctypes.c_double]),
    "spaghetty_last_error": (ctypes.c_int, []),
    "spaghetty_last_cuda_error": (ctypes.c_int, []),
    "spaghetty_last_cuda_error_string": (ctypes.c_char_p, []),
    "spaghetty_device_status": (ctypes.c_int, []),
    "spaghetty_set_option": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "spaghetty_error_string": (ctypes.c_char_p, [ctypes.c_int]),
    "spaghetty_plan_query": (ctypes.c_int, [ctypes.c_int, c_int_p, c_int_p, ctypes.c_int,
                                            ctypes.POINTER(PlanInfo)]),
    "spaghetty_tune_set": (ctypes.c_int, [ctypes.c_int, c_int_p, c_int_p, ctypes.c_int,
                                          c_int_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "spaghetty_plan_verify": (ctypes.c_int, [ctypes.c_int, c_int_p, c_int_p, ctypes.c_int,
                                             ctypes.c_int, ctypes.POINTER(ctypes.c_int64)]),
    "spaghetty_tune_load": (ctypes.c_int, [ctypes.c_char_p]),
    "spaghetty_batch_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int,
                                              ctypes.POINTER(ctypes.c_void_p)]),
    "spaghetty_batch_bad_index": (ctypes.c_int, []),
    "spaghetty_batch_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "spaghetty_batch_launch_plain": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "spaghetty_batch_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "spaghetty_batch_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]),
    "spaghetty_batch_poison": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "spaghetty_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "spaghetty_batch_tune_set": (ctypes.c_int, [ctypes.c_int] * 6),
    "spaghetty_batch_verify": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                              ctypes.POINTER(ctypes.c_int64)]),
    "spaghetty_batch_launches": (ctypes.c_int, [ctypes.c_void_p]),
    "spaghetty_sortacc_fused": (ctypes.c_int, [ctypes.c_int, ctypes.c_int,
                                               ctypes.POINTER(ctypes.c_void_p), c_int_p, c_int_p,
                                               ctypes.POINTER(ctypes.c_double), ctypes.c_void_p,
                                               ctypes.c_void_p]),
    "spaghetty_sort_fused": (ctypes.c_int, [ctypes.c_int, ctypes.c_int,
                                            ctypes.POINTER(ctypes.c_void_p), c_int_p, c_int_p,
                                            ctypes.POINTER(ctypes.c_double), ctypes.c_void_p,
                                            ctypes.c_void_p]),
    "spaghetty_sort_batch_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "spaghetty_contract_4x4": (ctypes.c_int, [ctypes.c_void_p, c_int_p, c_int_p, ctypes.c_void_p,
                                              c_int_p, c_int_p, ctypes.c_void_p, c_int_p,
                                              ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                              ctypes.c_int, ctypes.c_void_p]),
    "spaghetty_contract_last_error": (ctypes.c_int, []),
    "spaghetty_contract_verify": (ctypes.c_int, [c_int_p, c_int_p, c_int_p, c_int_p, c_int_p,
                                                 ctypes.POINTER(ctypes.c_int64)]),
    "ccsd_t2_8": (None, _T2_8), "ccsd_t2_8_": (None, _T2_8),
    "ccsd_t2_8_status": (ctypes.c_int, _T2_8),
    "spaghetty_selftest": (ctypes.c_int, []),
    "spaghetty_version": (ctypes.c_char_p, []),
}


class SpaghettyError(RuntimeError):
    def __init__(self, code: int, where: str = ""):
        self.code = code
        msg = lib().spaghetty_error_string(code).decode()
        if code == 7:   # SPAGHETTY_ERR_CUDA: name the CUDA error behind it
            self.cuda_error = lib().spaghetty_last_cuda_error()
            msg += " [%s, %d]" % (lib().spaghetty_last_cuda_error_string().decode(), self.cuda_error)
        super().__init__("%s%s (code %d)" % (where + ": " if where else "", msg, code))


def lib():
    """Load the C-ABI library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(
                    "spaghetty_gb300: %s is missing; build it with "
                    "`python -m spaghetty_gb300.build`" % LIB_PATH)
            L = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in PROTOTYPES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(code: int, where: str = "") -> None:
    if code != 0:
        raise SpaghettyError(code, where)


def int_array(vals):
    vals = [int(v) for v in vals]
    return (ctypes.c_int * max(1, len(vals)))(*vals)
