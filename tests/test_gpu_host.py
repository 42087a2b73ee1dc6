"""Host-buffer entry points (nla_trxm_host, nla_trxm_mixed_host).

They run the same kernels on the same operands in the same order as the
device-resident calls, with the copies in and out pipelined around them, so
their results must be bit-identical to nla_trxm / nla_trxm_mixed on the same
inputs: for every side / uplo / trans / func, every element type, in place
and out of place, from page-locked and pageable host memory, with padded
leading dimensions, and for every number of pipelined levels.  One case per
form is also checked against the oracle (relative error < 1e-13).
"""

import itertools
import os

import numpy as np
import pytest

from gpu_util import to_dev, to_host, torch_dtype

pytestmark = pytest.mark.gpu


def _host(X, dtype, ld=None, pin=False):
    """Column-major CPU tensor view of X (shape (r, c), strides (1, ld))."""
    import torch

    X = np.asarray(X)
    r, c = X.shape
    ld = ld or max(r, 1)
    buf = torch.zeros((max(c, 1), ld), dtype=torch_dtype(dtype))
    if pin:
        buf = buf.pin_memory()
    if r and c:
        buf[:c, :r] = torch.from_numpy(np.ascontiguousarray(X.T.astype(dtype)))
    return buf.T[:r, :c]


def _np(Xh):
    return Xh.numpy().astype(np.float64)


def _device_plain(pkg, cuda, side, uplo, trans, alpha, func, A, B, dtype):
    import torch

    Ad, Bd = to_dev(A, dtype, cuda), to_dev(B, dtype, cuda)
    pkg.unified_rectrxm_(side, uplo, trans, alpha, func, Ad, Bd, native=True)
    torch.cuda.synchronize()
    return to_host(Bd)


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.float16])
def test_plain_host_matches_device(pkg, workloads, cuda, dtype):
    n, m = (600, 70) if dtype != np.float16 else (300, 40)
    for k, (side, uplo, trans, func) in enumerate(itertools.product("LR", "LU", "NT", "SM")):
        A, B = workloads.problem(n, m, side, uplo, seed=100 + k)
        ref = _device_plain(pkg, cuda, side, uplo, trans, 0.75, func, A, B, dtype)
        for levels in (1, 3, 6):
            Ah, Bh = _host(A, dtype, pin=True), _host(B, dtype, pin=True)
            Xh = _host(np.zeros_like(B), dtype, pin=True)
            pkg.unified_rectrxm_host_(side, uplo, trans, 0.75, func, Ah, Bh, X=Xh, host_levels=levels)
            assert np.array_equal(_np(Xh), ref, equal_nan=True), (side, uplo, trans, func, levels)
            assert np.array_equal(_np(Bh), np.asarray(B).astype(dtype).astype(np.float64))  # B is only read


@pytest.mark.parametrize("terms", [7, 3])
def test_mixed_host_matches_device(pkg, workloads, cuda, terms):
    import torch

    n, m = 1100, 90
    for k, (side, uplo, trans, func) in enumerate(itertools.product("LR", "LU", "NT", "SM")):
        A, B = workloads.problem(n, m, side, uplo, seed=200 + k)
        Ad, Bd = to_dev(A, np.float64, cuda), to_dev(B, np.float64, cuda)
        pkg.unified_rectrxm_mixed_(side, uplo, trans, 0.5, func, Ad, Bd, split_terms=terms, sweeps=0)
        torch.cuda.synchronize()
        ref = to_host(Bd)
        for levels in (2, 4):
            Ah, Bh = _host(A, np.float64, pin=True), _host(B, np.float64, pin=True)
            Xh = _host(np.zeros_like(B), np.float64, pin=True)
            pkg.unified_rectrxm_mixed_host_(side, uplo, trans, 0.5, func, Ah, Bh, X=Xh, split_terms=terms,
                                            sweeps=0, host_levels=levels)
            assert np.array_equal(_np(Xh), ref), (terms, side, uplo, trans, func, levels)


def test_mixed_host_refinement(pkg, workloads, cuda):
    """Sweeps > 0 take the copy-all, solve, copy-out form."""
    import torch

    n, m = 900, 50
    for k, (side, uplo, trans) in enumerate(itertools.product("LR", "LU", "NT")):
        A, B = workloads.problem(n, m, side, uplo, seed=300 + k)
        Ad, Bd = to_dev(A, np.float64, cuda), to_dev(B, np.float64, cuda)
        pkg.unified_rectrxm_mixed_(side, uplo, trans, 1.5, "S", Ad, Bd, split_terms=3, sweeps=2)
        torch.cuda.synchronize()
        Ah, Bh = _host(A, np.float64), _host(B, np.float64)
        Xh = pkg.unified_rectrxm_mixed_host_(side, uplo, trans, 1.5, "S", Ah, Bh, split_terms=3, sweeps=2)
        assert Xh is Bh
        assert np.array_equal(_np(Bh), to_host(Bd)), (side, uplo, trans)


def test_host_in_place_padded_pageable(pkg, oracle, workloads, cuda):
    """In place (X = B), pageable host memory, padded leading dimensions on
    the host and on the device; against the device call and the oracle."""
    import torch

    n, m = 777, 61
    nthreads = os.cpu_count() or 1
    for k, (side, uplo, trans, func) in enumerate(itertools.product("LR", "LU", "NT", "SM")):
        A, B = workloads.problem(n, m, side, uplo, seed=400 + k)
        rows, cols = B.shape
        ref = _device_plain(pkg, cuda, side, uplo, trans, -2.0, func, A, B, np.float64)
        Ah, Bh = _host(A, np.float64, ld=n + 3), _host(B, np.float64, ld=rows + 5)
        A_dev = to_dev(np.zeros((n, n)), np.float64, cuda, ld=n + 7)
        B_dev = to_dev(np.zeros((rows, cols)), np.float64, cuda, ld=rows + 9)
        pkg.unified_rectrxm_host_(side, uplo, trans, -2.0, func, Ah, Bh, A_dev=A_dev, B_dev=B_dev)
        X = _np(Bh)
        assert np.array_equal(X, ref), (side, uplo, trans, func)
        torch.cuda.synchronize()
        assert np.array_equal(to_host(B_dev), ref)
        want = oracle.rectrxm(side, uplo, trans, -2.0, func, A, B, nthreads=nthreads)
        assert oracle.rel_err(X, want) < 1e-13, (side, uplo, trans, func)


def test_host_empty_and_argument_errors(pkg, cuda):
    import torch

    Ah = _host(np.zeros((0, 0)), np.float64)
    Bh = _host(np.zeros((0, 5)), np.float64)
    pkg.unified_rectrxm_host_("L", "L", "N", 1.0, "S", Ah, Bh)  # nothing to do
    A = _host(np.eye(8), np.float64)
    B = _host(np.ones((8, 3)), np.float64)
    with pytest.raises(ValueError):
        pkg.unified_rectrxm_host_("X", "L", "N", 1.0, "S", A, B)
    with pytest.raises(ValueError):  # a device tensor where a host one is expected
        pkg.unified_rectrxm_host_("L", "L", "N", 1.0, "S", A, B.to(cuda))
    with pytest.raises(ValueError):  # X of the wrong shape
        pkg.unified_rectrxm_host_("L", "L", "N", 1.0, "S", A, B, X=_host(np.ones((8, 4)), np.float64))
    torch.cuda.synchronize()
