"""spaghetty_gb300 -- GB300-native (sm_103a) NWChem TCE tensor sorts.

FP64 tensor permutations ``tce_sort_{2,4,6,8}`` and their accumulate forms,
bit-identical to the reference loop nests of jeffhammond/spaghetty
(trunk/old_sort.f, trunk/generator2.py, trunk/generator6.py), computed by
hand-written CUDA kernels behind a C ABI (include/spaghetty_gb300.h).
"""
from ._lib import LIB_PATH, SpaghettyError, lib
from .sort import (permuted_shape, plan, sort, sort_fused, sort_generic, sortacc, sortacc_fused,
                   tce_sort_2,
                   tce_sort_4,
                   tce_sort_6, tce_sort_8, tce_sortacc_2, tce_sortacc_4, tce_sortacc_6,
                   tce_sortacc_8)

from .contract import ccsd_t2_8, contract_4x4

__all__ = ["LIB_PATH", "SpaghettyError", "lib", "sort", "sortacc", "sortacc_fused", "sort_fused",
           "sort_generic", "plan",
           "permuted_shape", "tce_sort_2", "tce_sortacc_2", "tce_sort_4", "tce_sortacc_4",
           "tce_sort_6", "tce_sortacc_6", "tce_sort_8", "tce_sortacc_8", "contract_4x4",
           "ccsd_t2_8"]
