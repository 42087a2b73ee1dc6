"""Batched solve of many independent, unevenly sized triangular systems
(no counterpart in the reference, which handles one system per
``unified_rectrxm!`` call, src/rectrxm.jl:43-76).

A :class:`BatchPlan` describes the systems by offsets into two device pools
(column-major A_i and B_i); :meth:`BatchPlan.solve` runs one persistent
kernel over all of them, replayed from a CUDA graph.
"""

from __future__ import annotations

import ctypes

from . import _lib
from .rectrxm import _dtype_code, _stream

MODES = {"graph": _lib.NLA_BATCH_GRAPH, "persistent": _lib.NLA_BATCH_PERSISTENT, "loop": _lib.NLA_BATCH_LOOP}


def bucket_of(n: int) -> int:
    """Size bucket b of a system of order n: 16*2^b <= n < 32*2^b (last bucket open)."""
    b, hi = 0, 32
    while b < _lib.NLA_BATCH_BUCKETS - 1 and n >= hi:
        b += 1
        hi *= 2
    return b


class BatchPlan:
    """Plan for solving op(A_i) X_i = alpha B_i, i = 1..count (side 'L').

    ``systems`` is a sequence of (n, m, a_off, lda, b_off, ldb) with offsets
    in elements into the A and B pools.  The plan runs unified_rec's recursion
    (src/rectrxm.jl:101-198) for each system on the host and uploads its
    leaves and update tiles as a node queue.  Per size bucket, ``cutoff``
    gives the leaf order (16, 32 or 64) and ``cols`` the widest block of
    right-hand sides (16, 32, 64 or 128); ``cols_per_item`` is an older name
    for ``cols``.  None takes the library defaults (see :mod:`tune` for tuned
    values)."""

    def __init__(self, dtype, uplo, trans, systems, cols_per_item=None, *, cutoff=None, cols=None):
        import torch

        self.dtype = dtype
        code = {torch.float16: _lib.NLA_F16, torch.float32: _lib.NLA_F32, torch.float64: _lib.NLA_F64}.get(dtype)
        if code is None:
            raise ValueError("batched solves take Float16, Float32 or Float64, got %s" % dtype)
        arr = (_lib.BatchDesc * max(len(systems), 1))()
        for i, s in enumerate(systems):
            arr[i] = _lib.BatchDesc(*[int(v) for v in s])
        cols = cols if cols is not None else cols_per_item
        self._plan = ctypes.c_void_p()
        L = _lib.load()
        if cutoff is None and cols is None:
            _lib.check(L.nla_batch_plan_create(ctypes.byref(self._plan), code, _lib.ch(uplo), _lib.ch(trans),
                                               len(systems), arr, None))
        else:
            t = _lib.BatchTuning()
            for b in range(_lib.NLA_BATCH_BUCKETS):
                t.cutoff[b] = int(cutoff[b]) if cutoff is not None else 64
                t.cols[b] = int(cols[b]) if cols is not None else (64 if code == _lib.NLA_F64 else 128)
            _lib.check(L.nla_batch_plan_create_tuned(ctypes.byref(self._plan), code, _lib.ch(uplo),
                                                     _lib.ch(trans), len(systems), arr, ctypes.byref(t)))
        self.count = len(systems)

    def info(self):
        """(queued nodes, persistent CTAs, total n^2 m flops)."""
        items, grid, flops = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_double()
        _lib.check(_lib.load().nla_batch_plan_info(self._plan, ctypes.byref(items), ctypes.byref(grid),
                                                   ctypes.byref(flops)))
        return items.value, grid.value, flops.value

    def solve(self, alpha, A_pool, B_pool, mode="graph"):
        """Solve every system in place in B_pool (1-D device tensors)."""
        if A_pool.dtype != self.dtype or B_pool.dtype != self.dtype:
            raise ValueError("pool element type does not match the plan")
        if not (A_pool.is_cuda and B_pool.is_cuda):
            raise ValueError("pools must be CUDA tensors")
        _lib.check(_lib.load().nla_batch_solve(self._plan, float(alpha), A_pool.data_ptr(), B_pool.data_ptr(),
                                               MODES[mode], _stream(B_pool)))
        return B_pool

    def solve_mixed(self, alpha, A_pool, B_pool, sweeps=2, residual="split"):
        """Mixed-precision form of a Float64 batch: Float32 solves refined by
        ``sweeps`` Float64-accurate residuals (nla_batch_solve_mixed_ex),
        formed on the tensor cores from exact BF16 slice products
        (``residual`` 'split') or on the FP64 pipe ('fp64'); X replaces B."""
        import torch

        if self.dtype != torch.float64 or A_pool.dtype != torch.float64 or B_pool.dtype != torch.float64:
            raise ValueError("the mixed batch form needs a Float64 plan and Float64 pools")
        if not (A_pool.is_cuda and B_pool.is_cuda):
            raise ValueError("pools must be CUDA tensors")
        code = {"split": _lib.NLA_RESIDUAL_SPLIT, "fp64": _lib.NLA_RESIDUAL_FP64}[residual]
        _lib.check(_lib.load().nla_batch_solve_mixed_ex(self._plan, float(alpha), A_pool.data_ptr(),
                                                        B_pool.data_ptr(), int(sweeps), code, _stream(B_pool)))
        return B_pool

    def close(self):
        if self._plan:
            _lib.load().nla_batch_plan_destroy(self._plan)
            self._plan = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def uneven_sizes(count=10000, n_lo=16, n_hi=1024, m_hi=128, seed=7):
    """n_i log-uniform in [n_lo, n_hi] (rounded), m_i uniform in {1..m_hi}
    (numpy PCG64 with the given seed)."""
    import numpy as np

    rng = np.random.default_rng(seed)
    n = np.rint(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi), count))).astype(np.int64)
    n = np.clip(n, n_lo, n_hi)
    m = rng.integers(1, m_hi + 1, count)
    return n, m


def make_batch(n, m, dtype, device, seed=7, uplo="L"):
    """Device pools for systems of orders n[i] with m[i] right-hand sides:
    A_i with off-diagonals N(0,1)/sqrt(n_i) in the named triangle (the other
    triangle holds unreferenced values) and diagonal 2 + |N(0,1)|; B_i
    uniform on [-1, 1].  torch's Philox generator, seeded, on the device.
    Returns (A_pool, B_pool, systems)."""
    import numpy as np
    import torch

    n = np.asarray(n, dtype=np.int64)
    m = np.asarray(m, dtype=np.int64)
    a_off = np.concatenate([[0], np.cumsum(n * n)[:-1]])
    b_off = np.concatenate([[0], np.cumsum(n * m)[:-1]])
    g = torch.Generator(device=device).manual_seed(seed)
    A = torch.randn(int((n * n).sum()), generator=g, device=device, dtype=torch.float64)
    B = torch.rand(int((n * m).sum()), generator=g, device=device, dtype=torch.float64).mul_(2).sub_(1)
    # scale the off-diagonal entries of each system by 1/sqrt(n_i)
    scale = torch.from_numpy(np.repeat(1.0 / np.sqrt(n), n * n)).to(device)
    A.mul_(scale)
    del scale
    # diagonals: 2 + |N(0,1)|
    diag_idx = np.concatenate([a_off[i] + np.arange(n[i]) * (n[i] + 1) for i in range(len(n))])
    d = torch.randn(len(diag_idx), generator=g, device=device, dtype=torch.float64).abs_().add_(2.0)
    A[torch.from_numpy(diag_idx).to(device)] = d
    systems = [(int(n[i]), int(m[i]), int(a_off[i]), int(n[i]), int(b_off[i]), int(n[i])) for i in range(len(n))]
    return A.to(dtype), B.to(dtype), systems
