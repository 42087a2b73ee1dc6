"""Generate the golden fixtures in this directory.

  kat.npz      exact known-answer cases: small integer triangular systems whose
               diagonals are powers of two, so every solve and multiply of the
               reference algorithm is exact in Float16, Float32 and Float64.
               Expected outputs are computed with exact rational arithmetic
               (fractions), independently of any implementation.  All 8
               (side, uplo, trans in {N, T}) x {S, M} forms, n in {5, 16, 33},
               alpha in {1, 0.5, -2}.
  config0.npz  the plain Float64 solve on the 1024 x 1024 / 1024 x 256 seed-0
               workload: the oracle's solution for the first 8 right-hand
               sides and checksums of the whole solution.

Run from the repository root:  python tests/golden/make_golden.py
"""

from __future__ import annotations

import itertools
import os
import sys
from fractions import Fraction

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def _tri_int(n, uplo, rng):
    T = rng.integers(-3, 4, size=(n, n)).astype(np.float64)
    T = np.tril(T, -1) if uplo == "L" else np.triu(T, 1)
    d = rng.choice([1.0, -1.0, 2.0, -2.0, 4.0, -4.0], size=n)
    T[np.diag_indices(n)] = d
    return T


def _frac_mat(X):
    return [[Fraction(float(v)) for v in row] for row in X]


def _frac_mul(P, Q):
    n, k, m = len(P), len(Q), len(Q[0])
    return [[sum((P[i][t] * Q[t][j] for t in range(k)), Fraction(0)) for j in range(m)] for i in range(n)]


def _to_np(F):
    return np.array([[float(v) for v in row] for row in F], dtype=np.float64)


def make_kat():
    rng = np.random.default_rng(20250101)
    cases = {}
    idx = 0
    for n, side, uplo, trans, func, alpha in itertools.product([5, 16, 33], "LR", "LU", "NT", "SM", [1.0, 0.5, -2.0]):
        A = _tri_int(n, uplo, rng)
        m = 3
        opA = A.T if trans == "T" else A
        Xi = rng.integers(-4, 5, size=(n, m) if side == "L" else (m, n)).astype(np.float64)
        FA, FX = _frac_mat(opA), _frac_mat(Xi)
        prod = _frac_mul(FA, FX) if side == "L" else _frac_mul(FX, FA)
        if func == "S":
            # B = op(A) Xi (or Xi op(A)), so solving op(A) X = alpha B gives alpha * Xi.
            B = _to_np(prod)
            expect = alpha * Xi
        else:
            B = Xi
            expect = alpha * _to_np(prod)
        key = "c%03d" % idx
        cases[key + "_A"] = A
        cases[key + "_B"] = B
        cases[key + "_X"] = expect
        cases[key + "_meta"] = np.array([ord(side), ord(uplo), ord(trans), ord(func), alpha, n, m])
        idx += 1
    np.savez_compressed(os.path.join(HERE, "kat.npz"), **cases)
    return idx


def make_config0():
    import __graft_entry__ as graft

    import importlib

    orc = graft.load_oracle()
    graft.load_package()
    wl = importlib.import_module("nextla_gb300.workloads")
    A, B = wl.config0()
    X = orc.rectrxm("L", "L", "N", 1.0, "S", A, B, nthreads=os.cpu_count() or 1)
    np.savez_compressed(os.path.join(HERE, "config0.npz"), X_first8=X[:, :8], col_sums=X.sum(axis=0),
                        fro=np.array([np.linalg.norm(X)]))


if __name__ == "__main__":
    print("kat cases:", make_kat())
    make_config0()
    print("config0 written")
