"""FP64-accurate residual R = alpha*B - op(A) X on the tensor cores.

The split residual stages op(A) and X as 7 BF16 slices and accumulates slice
products exactly; its error bound is about 2^-50 * (|op(A)| |X|) per entry
(the fixed-point rounding of the smallest slice pairs), far below the FP64
rounding of a DGEMM.  Checked against exact rational arithmetic on sampled
columns, bit for bit on integer data, and against torch FP64 for all forms.
"""

import itertools
from fractions import Fraction

import numpy as np
import pytest

from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu


def _residual(pkg, cuda, side, uplo, trans, alpha, A, X, B, mode="split"):
    import torch

    Ad, Xd, Bd = (to_dev(M, np.float64, cuda) for M in (A, X, B))
    Rd = to_dev(np.zeros_like(B), np.float64, cuda)
    pkg.residual_(side, uplo, trans, alpha, Ad, Xd, Bd, Rd, residual=mode)
    pkg.device_status(Rd)
    torch.cuda.synchronize()
    return to_host(Rd)


def _op(A, uplo, trans):
    T = np.tril(A) if uplo == "L" else np.triu(A)
    return T.T if trans == "T" else T


@pytest.mark.parametrize("side", ["L", "R"])
def test_residual_exact_on_integers(pkg, cuda, side):
    rng = np.random.default_rng(4)
    n, m = 300, 45
    for uplo, trans in itertools.product("LU", "NT"):
        A = rng.integers(-1000, 1001, (n, n)).astype(np.float64)
        X = rng.integers(-1000, 1001, (n, m) if side == "L" else (m, n)).astype(np.float64)
        B = rng.integers(-1000, 1001, X.shape).astype(np.float64)
        opA = _op(A, uplo, trans)
        ref = 2.0 * B - (opA @ X if side == "L" else X @ opA)  # exact: all values < 2^53
        R = _residual(pkg, cuda, side, uplo, trans, 2.0, A, X, B)
        np.testing.assert_array_equal(R, ref)


@pytest.mark.parametrize("mode", ["split", "dd"])
def test_residual_against_rationals(pkg, workloads, cuda, mode):
    """Full 53-bit data: entry error <= 2^-48 * (|op(A)| |X|) + ulp(R); the
    double-double mode with a nearly cancelling right-hand side is checked
    to 4 ulps of the exact residual itself."""
    n, m = 256, 3
    A, _ = workloads.problem(n, m, "L", "L", seed=12)
    X = np.random.default_rng(5).standard_normal((n, m))
    L = np.tril(A)
    B = np.random.default_rng(6).standard_normal((n, m))
    if mode == "dd":
        B = L @ X + 1e-12 * B  # the residual is ~1e-12 of the terms
    R = _residual(pkg, cuda, "L", "L", "N", 1.0, A, X, B, mode=mode)
    for j in range(m):
        for i in range(n):
            exact = Fraction(B[i, j]) - sum((Fraction(L[i, k]) * Fraction(X[k, j]) for k in range(i + 1)), Fraction(0))
            if mode == "dd":
                bound = 4 * np.spacing(abs(float(exact)))
            else:
                bound = 2.0 ** -48 * float(np.abs(L[i, : i + 1]) @ np.abs(X[: i + 1, j])) + np.spacing(abs(float(exact)))
            assert abs(float(Fraction(R[i, j]) - exact)) <= bound, (i, j)


@pytest.mark.parametrize("side,uplo,trans", list(itertools.product("LR", "LU", "NT")))
def test_residual_all_forms_vs_fp64(pkg, workloads, cuda, side, uplo, trans):
    import torch

    n, m = 1000, 77
    A, _ = workloads.problem(n, m, side, uplo, seed=8)
    rng = np.random.default_rng(9)
    X = rng.standard_normal((n, m) if side == "L" else (m, n))
    B = rng.standard_normal(X.shape)
    opA = _op(A, uplo, trans)
    prod = opA @ X if side == "L" else X @ opA
    ref = -0.5 * B - prod
    scale = np.abs(opA) @ np.abs(X) if side == "L" else np.abs(X) @ np.abs(opA)
    for mode in ("split", "fp64", "dd"):
        R = _residual(pkg, cuda, side, uplo, trans, -0.5, A, X, B, mode=mode)
        assert np.max(np.abs(R - ref) / scale) < 1e-13, mode
