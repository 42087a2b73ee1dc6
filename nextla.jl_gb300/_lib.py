"""ctypes binding of ``libnextla_gb300.so`` (the C ABI in include/nextla_gb300.h).

The library is the only compute path: if it cannot be loaded, every entry
point raises.  There is no CPU fallback.
"""

from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnextla_gb300.so")

NLA_F16, NLA_F32, NLA_F64, NLA_C32, NLA_C64 = 0, 1, 2, 3, 4
NLA_OK = 0
NLA_ERR_ARG = -1
NLA_ERR_DTYPE = -2
NLA_ERR_UNSUPPORTED = -3
NLA_ERR_WORKSPACE = -4
NLA_ERR_TIMEOUT = -5
NLA_ERR_NOMEM = -6
NLA_ERR_CUDA_BASE = -100

# Every symbol declared in include/nextla_gb300.h, with its ctypes signature.
_i32, _i64, _d, _c, _p, _sz = (ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_char, ctypes.c_void_p,
                               ctypes.c_size_t)
SIGNATURES = {
    "nla_version": ([], _i32),
    "nla_last_error": ([], ctypes.c_char_p),
    "nla_trxm": ([_c, _c, _c, _d, _c, _i32, _i64, _i64, _p, _i64, _p, _i64, _p], _i32),
    "nla_trxm_ex": ([_c, _c, _c, _d, _c, _i32, _i64, _i64, _p, _i64, _p, _i64, _i64, _i64, _p], _i32),
    "nla_diag_block": ([_c, _c, _c, _i32, _i32, _i64, _i64, _p, _i64, _p, _i64, _p], _i32),
    "nla_gemm_update": ([_i32, _i32, _i32, _i64, _i64, _i64, _d, _p, _i64, _p, _i64, _p, _i64, _p], _i32),
    "nla_scale": ([_i32, _i64, _i64, _d, _p, _i64, _p], _i32),
    "nla_host_alloc": ([_sz, ctypes.POINTER(_p)], _i32),
    "nla_host_free": ([_p], _i32),
    "nla_scale_complex": ([_i32, _i64, _i64, _d, _d, _p, _i64, _p], _i32),
    "nla_trxm_complex": ([_c, _c, _c, _d, _d, _c, _i32, _i64, _i64, _p, _i64, _p, _i64, _p], _i32),
    "nla_trace_enable": ([_i32], _i32),
    "nla_trace_summary": ([_i32, ctypes.POINTER(_i64), ctypes.POINTER(_d), ctypes.POINTER(_d), ctypes.POINTER(_d)],
                          _i32),
}

NLA_LOWP_BF16, NLA_LOWP_F16 = 0, 1
NLA_RESIDUAL_FP64, NLA_RESIDUAL_SPLIT, NLA_RESIDUAL_DD = 0, 1, 2


class MixedOpts(ctypes.Structure):
    """nla_mixed_opts of include/nextla_gb300.h."""

    _fields_ = [("lowp", ctypes.c_int), ("split_terms", ctypes.c_int), ("sweeps", ctypes.c_int),
                ("residual", ctypes.c_int), ("cutoff", ctypes.c_int64), ("corr_out", ctypes.POINTER(ctypes.c_double))]


SIGNATURES.update({
    "nla_trxm_mixed": ([_c, _c, _c, _d, _c, _i64, _i64, _p, _i64, _p, _i64, ctypes.POINTER(MixedOpts), _p], _i32),
    "nla_gemm_update_mixed": ([_i32, _i32, _i64, _i64, _i64, _d, _p, _i64, _p, _i64, _p, _i64, _i32, _i32, _p],
                              _i32),
    "nla_device_status": ([_p], _i32),
    "nla_set_wait_limit_ns": ([ctypes.c_uint64], _i32),
    "nla_trxm_residual": ([_c, _c, _c, _d, _i64, _i64, _p, _i64, _p, _i64, _p, _i64, _p, _i64, _i32, _p], _i32),
    "nla_gemm_update_mixed_noalloc": ([_i32, _i32, _i64, _i64, _i64, _d, _p, _i64, _p, _i64, _p, _i64, _i32, _i32,
                                       _p], _i32),
})
NLA_NOALLOC_SCRATCH_BYTES = 64 << 20

class BatchDesc(ctypes.Structure):
    """nla_batch_desc of include/nextla_gb300.h."""

    _fields_ = [("n", ctypes.c_int64), ("m", ctypes.c_int64), ("a_off", ctypes.c_int64), ("lda", ctypes.c_int64),
                ("b_off", ctypes.c_int64), ("ldb", ctypes.c_int64)]


class BatchTuning(ctypes.Structure):
    """nla_batch_tuning of include/nextla_gb300.h: per size bucket, the leaf
    order of the recursion and the widest block of right-hand sides."""

    _fields_ = [("cutoff", ctypes.c_int * 6), ("cols", ctypes.c_int * 6)]


NLA_BATCH_BUCKETS = 6
NLA_BATCH_GRAPH, NLA_BATCH_PERSISTENT, NLA_BATCH_LOOP = 0, 1, 2

SIGNATURES.update({
    "nla_batch_plan_create": ([ctypes.POINTER(_p), _i32, _c, _c, _i64, ctypes.POINTER(BatchDesc),
                               ctypes.POINTER(_i32)], _i32),
    "nla_batch_plan_create_tuned": ([ctypes.POINTER(_p), _i32, _c, _c, _i64, ctypes.POINTER(BatchDesc),
                                     ctypes.POINTER(BatchTuning)], _i32),
    "nla_batch_plan_info": ([_p, ctypes.POINTER(_i64), ctypes.POINTER(_i64), ctypes.POINTER(_d)], _i32),
    "nla_batch_solve": ([_p, _d, _p, _p, _i32, _p], _i32),
    "nla_batch_plan_destroy": ([_p], _i32),
    "nla_batch_solve_mixed": ([_p, _d, _p, _p, _i32, _p], _i32),
    "nla_batch_solve_mixed_ex": ([_p, _d, _p, _p, _i32, _i32, _p], _i32),
})

SIGNATURES["nla_trxm_diag"] = ([_c, _c, _c, _c, _d, _c, _i32, _i64, _i64, _p, _i64, _p, _i64, _p], _i32)
SIGNATURES["nla_measure_pipes"] = ([ctypes.POINTER(_d), ctypes.POINTER(_d), ctypes.POINTER(_d), _p], _i32)
SIGNATURES["nla_trxm_mixed_diag"] = ([_c, _c, _c, _c, _d, _c, _i64, _i64, _p, _i64, _p, _i64, ctypes.POINTER(MixedOpts),
                                      _p], _i32)
SIGNATURES["nla_trxm_host"] = ([_c, _c, _c, _d, _c, _i32, _i64, _i64, _p, _i64, _p, _i64, _p, _i64, _p, _i64, _p,
                                 _i64, _i32, _p], _i32)
SIGNATURES["nla_trxm_mixed_host"] = ([_c, _c, _c, _d, _c, _i64, _i64, _p, _i64, _p, _i64, _p, _i64, _p, _i64, _p,
                                       _i64, ctypes.POINTER(MixedOpts), _i32, _p], _i32)


def measure_pipes(stream=None) -> dict:
    """{'dfma', 'dmma', 'ffma'}: measured TFLOP/s of those pipes on this GPU."""
    a, b, c = _d(), _d(), _d()
    check(load().nla_measure_pipes(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), stream))
    return {"dfma": a.value, "dmma": b.value, "ffma": c.value}


def host_empty(numel, dtype):
    """A 1-D CPU tensor of `numel` elements of torch `dtype` in page-locked
    memory from nla_host_alloc (cudaHostAlloc), freed with the tensor; reshape
    it to the layout the host-buffer entry points are given."""
    import weakref

    import numpy as np
    import torch

    es = torch.empty((), dtype=dtype).element_size()
    nbytes = max(int(numel) * es, 1)
    p = _p()
    check(load().nla_host_alloc(nbytes, ctypes.byref(p)))
    arr = np.frombuffer((ctypes.c_byte * nbytes).from_address(p.value), dtype=np.uint8)
    weakref.finalize(arr, load().nla_host_free, ctypes.c_void_p(p.value))
    return torch.from_numpy(arr).view(dtype)[: int(numel)]


KERNEL_CLASSES = ["leaf_solve", "leaf_mult", "gemm_simt", "gemm_umma", "split", "scale", "residual", "batched",
                  "copy_in", "copy_out"]

_lib = None
_lock = threading.Lock()


class NLAError(RuntimeError):
    """A negative status from the library, with its message."""

    def __init__(self, code: int, msg: str):
        super().__init__("%s (status %d)" % (msg or "nextla_gb300 error", code))
        self.code = code


class NLAArgumentError(NLAError, ValueError):
    """Invalid arguments (the reference would have fallen through silently)."""


def load(path: str | None = None):
    """Load the library (built in-tree by build.py) and declare signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise ImportError("libnextla_gb300.so is not built (run nextla.jl_gb300/build.py or "
                              "__graft_entry__.build())")
        L = ctypes.CDLL(p)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
        return _lib


def check(rc: int) -> None:
    if rc == NLA_OK:
        return
    msg = load().nla_last_error()
    msg = msg.decode() if msg else ""
    if rc in (NLA_ERR_ARG, NLA_ERR_DTYPE):
        raise NLAArgumentError(rc, msg)
    raise NLAError(rc, msg)


def trace_enable(on: bool) -> None:
    check(load().nla_trace_enable(1 if on else 0))


def trace_summary() -> dict:
    """{kernel class: (launches, device ms, algorithmic flops, bytes)} of the
    launches recorded since trace_enable(True)."""
    L = load()
    out = {}
    for k, name in enumerate(KERNEL_CLASSES):
        n, ms, fl, by = _i64(), _d(), _d(), _d()
        check(L.nla_trace_summary(k, ctypes.byref(n), ctypes.byref(ms), ctypes.byref(fl), ctypes.byref(by)))
        if n.value:
            out[name] = (n.value, ms.value, fl.value, by.value)
    return out


def ch(c: str):
    return ctypes.c_char(c.encode() if isinstance(c, str) else c)
