"""Complex element types (ComplexF32, ComplexF64) on the plain path against
the oracle's complex restatement and BLAS ztrsm/ztrmm (ctrsm/ctrmm).

The reference's unified_rec takes only real element types
(src/rectrxm.jl:101) though its base-case docstrings list complex ones
(src/trsm.jl:180-183); these tests hold the GPU path to the reference's real
contract (test/unified_rectrxm.jl:42, test/trsm.jl:55): relative Frobenius
error below 1e-14 (ComplexF64) and 1e-5 (ComplexF32), against the oracle and
against BLAS, over every side, uplo and trans ('C' is the Adjoint), both
functions, a complex alpha, and sizes that recurse.
"""

import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {np.complex128: 1e-14, np.complex64: 1e-5}


def _pair(rng, n, m, side, uplo):
    Z = (rng.random((n, n)) + 1.0) + 1j * (rng.random((n, n)) - 0.5)
    A = (np.tril(Z) if uplo == "L" else np.triu(Z)) + 10.0 * np.eye(n)
    shape = (n, m) if side == "L" else (m, n)
    B = (rng.random(shape) + 1.0) + 1j * (rng.random(shape) - 0.5)
    return np.asfortranarray(A), np.asfortranarray(B)


def _dev(X, dt, dev):
    import torch

    t = torch.from_numpy(np.ascontiguousarray(np.asarray(X, dtype=dt).T)).to(dev)
    return t.T  # column-major view


@pytest.mark.parametrize("dt", [np.complex128, np.complex64])
@pytest.mark.parametrize("native", [True, False])
def test_complex_sweep(pkg, oracle, cuda, dt, native):
    import torch

    rng = np.random.default_rng(31)
    alpha = 0.5 - 0.25j
    for n, m, side, uplo, trans, func in itertools.product([16, 100, 300], [1, 9, 40], "LR", "LU", "NTC", "SM"):
        A, B = _pair(rng, n, m, side, uplo)
        Ad, Bd = _dev(A, dt, cuda), _dev(B, dt, cuda)
        pkg.unified_rectrxm_(side, uplo, trans, alpha, func, Ad, Bd, native=native)
        torch.cuda.synchronize()
        X = Bd.cpu().numpy()
        ref = oracle.rectrxm_complex(side, uplo, trans, alpha, func, A.astype(dt), B.astype(dt))
        assert oracle.rel_err(X, ref) < TOL[dt], (n, m, side, uplo, trans, func)
        blas = oracle.blas_rectrxm(side, uplo, trans, alpha, func, A.astype(dt), B.astype(dt))
        assert oracle.rel_err(X, blas) < TOL[dt], (n, m, side, uplo, trans, func)


def test_complex_larger_and_adjoint_differs(pkg, oracle, cuda):
    """n = 1000 (several recursion levels with 128-row leaves): 'C' is the
    conjugate transpose, so its result differs from 'T' and matches BLAS."""
    import torch

    rng = np.random.default_rng(32)
    n, m = 1000, 64
    A, B = _pair(rng, n, m, "L", "U")
    out = {}
    for trans in "TC":
        Ad, Bd = _dev(A, np.complex128, cuda), _dev(B, np.complex128, cuda)
        pkg.unified_rectrxm_("L", "U", trans, 1.0 + 0.5j, "S", Ad, Bd, native=True)
        torch.cuda.synchronize()
        out[trans] = Bd.cpu().numpy()
        blas = oracle.blas_rectrxm("L", "U", trans, 1.0 + 0.5j, "S", A, B)
        assert oracle.rel_err(out[trans], blas) < 1e-14, trans
    assert oracle.rel_err(out["T"], out["C"]) > 1e-3


def test_complex_unit_diagonal_and_host_buffers(pkg, oracle, cuda):
    """trsm() with diag 'U' (the diagonal never read: NaNs there) and the
    host-buffer entry point, both on ComplexF64."""
    import torch

    rng = np.random.default_rng(33)
    n, m = 300, 17
    A, B = _pair(rng, n, m, "L", "L")
    A = np.asfortranarray(np.tril(A, -1) / n + 10.0 * np.eye(n))  # well conditioned with a unit diagonal too
    An = A.copy()
    An[np.diag_indices(n)] = np.nan
    Ad, Bd = _dev(An, np.complex128, cuda), _dev(B, np.complex128, cuda)
    pkg.trsm("L", "L", "C", "U", Ad, Bd, 2.0)
    torch.cuda.synchronize()
    Au = A.copy()
    Au[np.diag_indices(n)] = 1.0
    ref = oracle.blas_rectrxm("L", "L", "C", 2.0, "S", Au, B)
    assert oracle.rel_err(Bd.cpu().numpy(), ref) < 1e-14

    ref = oracle.blas_rectrxm("L", "L", "C", 0.5, "M", A, B)
    Ah = torch.from_numpy(np.array(A.T)).T  # copies: the call writes its result into B's memory
    Bh = torch.from_numpy(np.array(B.T)).T
    X = pkg.unified_rectrxm_host_("L", "L", "C", 0.5, "M", Ah, Bh)
    assert oracle.rel_err(np.asarray(X), ref) < 1e-14


def test_complex_rejected_where_real_only(pkg, cuda):
    import ctypes

    import torch

    from nextla_gb300 import _lib, batched

    A = torch.eye(8, dtype=torch.complex128, device=cuda)
    B = torch.ones(8, 2, dtype=torch.complex128, device=cuda)
    with pytest.raises(ValueError):
        pkg.unified_rectrxm_mixed_("L", "L", "N", 1.0, "S", A, B)
    with pytest.raises(ValueError):
        batched.BatchPlan(torch.complex128, "L", "N", [(8, 2, 0, 8, 0, 8)])
    plan = ctypes.c_void_p()
    d = (_lib.BatchDesc * 1)(_lib.BatchDesc(8, 2, 0, 8, 0, 8))
    with pytest.raises(_lib.NLAError):  # the C ABI refuses it too
        _lib.check(_lib.load().nla_batch_plan_create(ctypes.byref(plan), _lib.NLA_C64, b"L", b"N", 1, d, None))
