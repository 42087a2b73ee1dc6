"""Seeded synthetic inputs with the shapes and value distributions of the
benchmark configurations (no public data set exists for this path).

All generators use numpy's PCG64 ``default_rng(seed)`` and return column-major
(Fortran-ordered) float64 arrays; callers cast to the element type they test.

  triangular(n, uplo, seed): off-diagonal entries N(0,1)/sqrt(n) in the named
      triangle, diagonal 2 + |N(0,1)|, zeros elsewhere;
  rhs(rows, cols, seed): uniform on [-1, 1];
  reference_test_pair(...): the construction of the reference's own tests
      (test/unified_rectrxm.jl:20-27): tri(rand + 1) + 10 I and rand + 1.
"""

from __future__ import annotations

import numpy as np


def triangular(n: int, uplo: str = "L", seed: int = 0, rng=None) -> np.ndarray:
    rng = np.random.default_rng(seed) if rng is None else rng
    Z = rng.standard_normal((n, n)) / np.sqrt(max(n, 1))
    d = 2.0 + np.abs(rng.standard_normal(n))
    T = np.tril(Z, -1) if uplo == "L" else np.triu(Z, 1)
    T[np.diag_indices(n)] = d
    return np.asfortranarray(T)


def rhs(rows: int, cols: int, seed: int = 0, rng=None) -> np.ndarray:
    rng = np.random.default_rng(seed) if rng is None else rng
    return np.asfortranarray(rng.uniform(-1.0, 1.0, (rows, cols)))


def problem(n: int, m: int, side: str = "L", uplo: str = "L", seed: int = 0):
    """A (n x n triangular) and B (n x m for side L, m x n for side R) drawn
    from one generator, A first."""
    rng = np.random.default_rng(seed)
    A = triangular(n, uplo, rng=rng)
    B = rhs(n, m, rng=rng) if side == "L" else rhs(m, n, rng=rng)
    return A, B


def reference_test_pair(n: int, m: int, side: str, uplo: str, rng) -> tuple:
    """A and B as built by test/unified_rectrxm.jl:20-27."""
    R = rng.random((n, n)) + 1.0
    A = (np.tril(R) if uplo == "L" else np.triu(R)) + 10.0 * np.eye(n)
    B = rng.random((n, m)) + 1.0 if side == "L" else rng.random((m, n)) + 1.0
    return np.asfortranarray(A), np.asfortranarray(B)


def config0():
    """Plain FP64 TRSM L/L/N: A 1024 x 1024 lower, B 1024 x 256, seed 0."""
    return problem(1024, 256, "L", "L", seed=0)


def cond1_lower(A) -> float:
    """1-norm condition number estimate of a lower-triangular matrix (LAPACK
    dtrcon through scipy)."""
    from scipy.linalg import lapack

    rc, info = lapack.dtrcon(A, norm="1", uplo="L", diag="N")
    if info != 0:
        raise ValueError("dtrcon failed (info %d)" % info)
    return float("inf") if rc == 0 else 1.0 / rc


def conditioned(n: int, target: float, seed: int = 0, rtol: float = 0.25):
    """Lower-triangular A with off-diagonals N(0,1)/sqrt(n) and diagonal
    c * (2 + |N(0,1)|), the scale c chosen by bisection on log(c) so that the
    dtrcon 1-norm estimate of cond(A) is within a factor 10**rtol of target.
    Returns (A, c, cond)."""
    rng = np.random.default_rng(seed)
    A = np.asfortranarray(np.tril(rng.standard_normal((n, n)) / np.sqrt(max(n, 1)), -1))
    d = 2.0 + np.abs(rng.standard_normal(n))
    idx = np.diag_indices(n)

    def cond_at(c):
        A[idx] = c * d
        return cond1_lower(A)

    lo, hi = np.log(1e-3), np.log(1e3)  # cond decreases as c grows
    c = 1.0
    k = cond_at(c)
    for _ in range(60):
        if abs(np.log10(k) - np.log10(target)) <= rtol:
            break
        if k > target:
            lo = np.log(c)
        else:
            hi = np.log(c)
        c = float(np.exp(0.5 * (lo + hi)))
        k = cond_at(c)
    return A, c, k
