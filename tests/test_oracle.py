"""The oracle is pinned before it is trusted: it must meet the reference's own
test contract against BLAS (test/unified_rectrxm.jl:8-43, test/trsm.jl:55-111)
and reproduce exact known-answer cases (tests/golden/kat.npz)."""

import itertools
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("func", ["S", "M"])
@pytest.mark.parametrize("side", ["L", "R"])
def test_reference_contract_f64(oracle, workloads, side, func):
    """The 432-case sweep of test/unified_rectrxm.jl:10-16 (here 216 per
    side/func pair, plus n = 300 and 600, which recurse for solves too):
    relative Frobenius error vs BLAS < 1e-14."""
    rng = np.random.default_rng(7)
    for n, m, uplo, trans in itertools.product([16, 32, 128, 256, 300, 600], [1, 8, 64], "LU", "NTC"):
        A, B = workloads.reference_test_pair(n, m, side, uplo, rng)
        X = oracle.rectrxm(side, uplo, trans, 1.0, func, A, B)
        ref = oracle.blas_rectrxm(side, uplo, trans, 1.0, func, A, B)
        assert oracle.rel_err(X, ref) < 1e-14, (n, m, uplo, trans)


@pytest.mark.parametrize("side,uplo", [("L", "L"), ("L", "U"), ("R", "L"), ("R", "U")])
def test_reference_contract_f32_leaves(oracle, side, uplo):
    """test/trsm.jl:57-111: Float32 base-case solves vs BLAS, tolerance 1e-5."""
    rng = np.random.default_rng(11)
    for n, m in itertools.product([16, 32, 128, 256], [1, 8, 64]):
        R = rng.random((n, n), dtype=np.float32) + 1
        A = (np.tril(R) if uplo == "L" else np.triu(R)) + np.float32(10) * np.eye(n, dtype=np.float32)
        B = (rng.random((n, m), dtype=np.float32) if side == "L" else rng.random((m, n), dtype=np.float32)) + 1
        X = oracle.leaf("S", side, uplo, A, B)
        ref = oracle.blas_rectrxm(side, uplo, "N", 1.0, "S", A, B)
        assert X.dtype == np.float32
        assert oracle.rel_err(X, ref) < 1e-5


def _kat_cases():
    z = np.load(os.path.join(GOLDEN, "kat.npz"))
    keys = sorted({k.split("_")[0] for k in z.files})
    for k in keys:
        meta = z[k + "_meta"]
        yield k, chr(int(meta[0])), chr(int(meta[1])), chr(int(meta[2])), chr(int(meta[3])), float(meta[4]), \
            z[k + "_A"], z[k + "_B"], z[k + "_X"]


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.float16])
def test_known_answers_exact(oracle, dtype):
    """Integer systems with power-of-two diagonals are exact in every element
    type; the oracle must reproduce the rational-arithmetic answers bit for bit."""
    count = 0
    for key, side, uplo, trans, func, alpha, A, B, X in _kat_cases():
        got = oracle.rectrxm(side, uplo, trans, alpha, func, A.astype(dtype), B.astype(dtype), thresholds=(8, 4))
        np.testing.assert_array_equal(got.astype(np.float64), X, err_msg=key)
        count += 1
    assert count == 144


def test_config0_fixture(oracle, workloads):
    z = np.load(os.path.join(GOLDEN, "config0.npz"))
    A, B = workloads.config0()
    X = oracle.rectrxm("L", "L", "N", 1.0, "S", A, B, nthreads=4)
    np.testing.assert_array_equal(X[:, :8], z["X_first8"])
    np.testing.assert_array_equal(X.sum(axis=0), z["col_sums"])
    # The solution is accurate: small backward error against float64 BLAS.
    assert oracle.rel_err(X, oracle.blas_rectrxm("L", "L", "N", 1.0, "S", A, B)) < 1e-13


def test_threads_do_not_change_results(oracle, workloads):
    for side in "LR":
        A, B = workloads.problem(700, 37, side, "U", seed=3)
        one = oracle.rectrxm(side, "U", "T", 0.5, "S", A, B, nthreads=1)
        many = oracle.rectrxm(side, "U", "T", 0.5, "S", A, B, nthreads=5)
        np.testing.assert_array_equal(one, many)


def test_split_point(oracle, pkg):
    for n in list(range(1, 600)) + [1023, 1024, 1025, 12288, 16384, 16385]:
        expect = n // 2 if (n & (n - 1)) == 0 else 1 << (n.bit_length() - 1)
        assert oracle.split_point(n) == expect
        assert pkg.split_point(n) == expect


def test_float16_rounds_every_operation(oracle):
    """The Float16 form rounds after every operation (Julia Float16 semantics):
    a product that is exact in Float32 but not in Float16 must be rounded."""
    A = np.array([[1.0]], dtype=np.float16)
    B = np.array([[1.0 + 2.0 ** -10]], dtype=np.float16)
    # alpha * b = 3 * (1 + 2^-10) = 3.0029296875 -> Float16 spacing at 3 is 2^-9
    X = oracle.rectrxm("L", "L", "N", 3.0, "M", A, B)
    assert float(X[0, 0]) == float(np.float16(3.0 * (1.0 + 2.0 ** -10)))


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-14), (np.complex64, 1e-5)])
def test_complex_contract(oracle, dtype, tol):
    """The complex restatement meets the reference's real contract against
    BLAS ztrsm/ztrmm (ctrsm/ctrmm) for every side, uplo, trans (with 'C' the
    conjugate transpose) and both functions, with a complex alpha."""
    rng = np.random.default_rng(13)
    for n, m, side, uplo, trans, func in itertools.product([16, 300], [1, 9], "LR", "LU", "NTC", "SM"):
        Z = (rng.random((n, n)) + 1) + 1j * (rng.random((n, n)) - 0.5)
        A = (np.tril(Z) if uplo == "L" else np.triu(Z)) + 10 * np.eye(n)
        shape = (n, m) if side == "L" else (m, n)
        B = rng.random(shape) + 1j * rng.random(shape)
        X = oracle.rectrxm_complex(side, uplo, trans, 0.5 - 0.25j, func, A.astype(dtype), B.astype(dtype),
                                   nthreads=4)
        assert X.dtype == dtype
        ref = oracle.blas_rectrxm(side, uplo, trans, 0.5 - 0.25j, func, A.astype(dtype), B.astype(dtype))
        assert oracle.rel_err(X, ref) < tol, (n, m, side, uplo, trans, func)
    # 'C' conjugates: it differs from 'T' on complex data
    A = np.tril(rng.random((6, 6)) + 1j * rng.random((6, 6))) + 5 * np.eye(6)
    B = rng.random((6, 2)) + 0j
    assert oracle.rel_err(oracle.rectrxm_complex("L", "L", "T", 1, "M", A, B),
                          oracle.rectrxm_complex("L", "L", "C", 1, "M", A, B)) > 1e-3
