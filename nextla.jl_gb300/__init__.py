"""GB300 (sm_103a) implementation of NextLA.jl's recursive triangular solve /
multiply (`unified_rectrxm!`, src/rectrxm.jl).

The compute path is the C-ABI library ``libnextla_gb300.so`` (declared in
include/nextla_gb300.h); this package holds its sources (``csrc/``), its build
(``build.py``), the ctypes binding (``_lib.py``) and the host-side mirror of the
reference's Julia API (``rectrxm.py``).  The directory name is not a Python
identifier, so callers load it by path with :func:`load_package` in
``__graft_entry__``.
"""

from . import _lib
from ._lib import NLAArgumentError, NLAError
from .rectrxm import (GEMM_ADD_, GEMM_SUB_, LeftLowerTRMM_, LeftLowerTRSM_, LeftUpperTRMM_, LeftUpperTRSM_,
                      getrf2_trsm_, lauum_offdiag_trmm_,
                      RightLowerTRMM_, RightLowerTRSM_, RightUpperTRMM_, RightUpperTRSM_, device_status,
                      matmul_, matmul_mixed_, residual_, scale_, split_point, trmm, trsm, unified_rec,
                      unified_rectrxm_, unified_rectrxm_host_, unified_rectrxm_mixed_,
                      unified_rectrxm_mixed_host_)

__all__ = [
    "unified_rectrxm_", "unified_rec", "split_point", "matmul_", "scale_", "GEMM_ADD_", "GEMM_SUB_",
    "LeftLowerTRSM_", "LeftUpperTRSM_", "RightLowerTRSM_", "RightUpperTRSM_",
    "LeftLowerTRMM_", "LeftUpperTRMM_", "RightLowerTRMM_", "RightUpperTRMM_",
    "NLAError", "NLAArgumentError", "load_library", "unified_rectrxm_mixed_", "matmul_mixed_", "device_status",
    "residual_", "trsm", "trmm", "unified_rectrxm_host_", "unified_rectrxm_mixed_host_", "getrf2_trsm_",
    "lauum_offdiag_trmm_",
]


def load_library():
    """Load libnextla_gb300.so (raises ImportError when it is not built)."""
    return _lib.load()
