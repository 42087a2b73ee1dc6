"""GPU parity of the plain (dtype-preserving) path against the oracle.

Tolerances (relative Frobenius error, ||X - X_ref||_F / ||X_ref||_F):
  Float64  1e-14 against the oracle and against BLAS (the reference's own
           bound, test/unified_rectrxm.jl:8);
  Float32  1e-5 (test/trsm.jl:55);
  Float16  the GPU result must be within 2x (+1e-3) of the reference
           algorithm's own Float16 error against the Float64 answer, and below
           1e-2; the GPU accumulates Float16 products in Float32, the reference
           in Float16.
Exact known-answer cases must match bit for bit in every element type.
"""

import itertools
import os

import numpy as np
import pytest

from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL = {np.float64: 1e-14, np.float32: 1e-5}


def _run(pkg, dev, side, uplo, trans, alpha, func, A, B, dtype, native, thresholds=None, lda=None, ldb=None):
    import torch

    Ad = to_dev(A, dtype, dev, ld=lda)
    Bd = to_dev(B, dtype, dev, ld=ldb)
    pkg.unified_rectrxm_(side, uplo, trans, alpha, func, Ad, Bd, native=native, thresholds=thresholds)
    torch.cuda.synchronize()
    return to_host(Bd)


@pytest.mark.parametrize("native", [False, True])
@pytest.mark.parametrize("func", ["S", "M"])
def test_reference_sweep_f64(pkg, oracle, workloads, cuda, func, native):
    """test/unified_rectrxm.jl:10-44: n in {16,32,128,256}, m in {1,8,64}, all
    side/uplo/trans, Float64, alpha = 1; plus n = 300 and 600 so that solves
    recurse too.  Checked against BLAS (the reference's oracle) and the oracle."""
    rng = np.random.default_rng(2)
    for n, m, side, uplo, trans in itertools.product([16, 32, 128, 256, 300, 600], [1, 8, 64], "LR", "LU", "NTC"):
        A, B = workloads.reference_test_pair(n, m, side, uplo, rng)
        X = _run(pkg, cuda, side, uplo, trans, 1.0, func, A, B, np.float64, native)
        ref = oracle.blas_rectrxm(side, uplo, trans, 1.0, func, A, B)
        assert oracle.rel_err(X, ref) < 1e-14, (n, m, side, uplo, trans)
        orc = oracle.rectrxm(side, uplo, trans, 1.0, func, A, B)
        assert oracle.rel_err(X, orc) < 1e-14, (n, m, side, uplo, trans)


@pytest.mark.parametrize("func", ["S", "M"])
def test_reference_sweep_f32(pkg, oracle, workloads, cuda, func):
    rng = np.random.default_rng(3)
    for n, m, side, uplo, trans in itertools.product([16, 32, 128, 256, 300], [1, 8, 64], "LR", "LU", "NT"):
        A, B = workloads.reference_test_pair(n, m, side, uplo, rng)
        A32, B32 = A.astype(np.float32), B.astype(np.float32)
        X = _run(pkg, cuda, side, uplo, trans, 1.0, func, A32, B32, np.float32, True)
        ref = oracle.blas_rectrxm(side, uplo, trans, 1.0, func, A32, B32)
        assert oracle.rel_err(X, ref) < 1e-5, (n, m, side, uplo, trans)


@pytest.mark.parametrize("side,uplo", [("L", "L"), ("L", "U"), ("R", "L"), ("R", "U")])
def test_base_case_kernels_f32(pkg, oracle, cuda, side, uplo):
    """test/trsm.jl:57-111 through the base-case entry points."""
    import torch

    fn = getattr(pkg, {"LL": "LeftLowerTRSM_", "LU": "LeftUpperTRSM_", "RL": "RightLowerTRSM_",
                       "RU": "RightUpperTRSM_"}[side + uplo])
    rng = np.random.default_rng(5)
    for n, m in itertools.product([16, 32, 128, 256], [1, 8, 64]):
        R = rng.random((n, n), dtype=np.float32) + 1
        A = (np.tril(R) if uplo == "L" else np.triu(R)) + np.float32(10) * np.eye(n, dtype=np.float32)
        B = (rng.random((n, m), dtype=np.float32) if side == "L" else rng.random((m, n), dtype=np.float32)) + 1
        Ad, Bd = to_dev(A, np.float32, cuda), to_dev(B, np.float32, cuda)
        fn(Ad, Bd)
        torch.cuda.synchronize()
        ref = oracle.blas_rectrxm(side, uplo, "N", 1.0, "S", A, B)
        assert oracle.rel_err(to_host(Bd), ref) < 1e-5


def _kat_cases():
    z = np.load(os.path.join(GOLDEN, "kat.npz"))
    for k in sorted({k.split("_")[0] for k in z.files}):
        meta = z[k + "_meta"]
        yield (k, chr(int(meta[0])), chr(int(meta[1])), chr(int(meta[2])), chr(int(meta[3])), float(meta[4]),
               z[k + "_A"], z[k + "_B"], z[k + "_X"])


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.float16])
@pytest.mark.parametrize("native", [False, True])
def test_known_answers_exact(pkg, cuda, dtype, native):
    for key, side, uplo, trans, func, alpha, A, B, X in _kat_cases():
        got = _run(pkg, cuda, side, uplo, trans, alpha, func, A, B, dtype, native, thresholds=(8, 4))
        np.testing.assert_array_equal(got, X, err_msg=key)


def test_config0(pkg, oracle, workloads, cuda):
    """Plain FP64 TRSM L/L/N, A 1024^2, B 1024 x 256, seed 0, vs the golden
    oracle columns and the full oracle solution; backward error O(1)."""
    z = np.load(os.path.join(GOLDEN, "config0.npz"))
    A, B = workloads.config0()
    X = _run(pkg, cuda, "L", "L", "N", 1.0, "S", A, B, np.float64, True)
    assert oracle.rel_err(X[:, :8], z["X_first8"]) < 1e-14
    ref = oracle.rectrxm("L", "L", "N", 1.0, "S", A, B, nthreads=os.cpu_count() or 1)
    assert oracle.rel_err(X, ref) < 1e-14
    assert oracle.backward_error("L", "L", "N", 1.0, A, X, B) < 1.0


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_recursive_sizes_all_forms(pkg, oracle, workloads, cuda, dtype):
    """Non-power-of-two and multi-level recursion, all 8 side/uplo/trans forms
    for solve and multiply, alpha = 0.5 and -2, default cut-offs and the
    reference's (256, 16)."""
    nthreads = os.cpu_count() or 1
    for n, m, side, uplo, trans, func in itertools.product([257, 1000, 2048], [33], "LR", "LU", "NT", "SM"):
        A, B = workloads.problem(n, m, side, uplo, seed=n + m)
        alpha = 0.5 if trans == "N" else -2.0
        ref = oracle.rectrxm(side, uplo, trans, alpha, func, A.astype(dtype), B.astype(dtype), nthreads=nthreads)
        for thr in (None, (256, 16)):
            X = _run(pkg, cuda, side, uplo, trans, alpha, func, A, B, dtype, True, thresholds=thr)
            assert oracle.rel_err(X, ref) < TOL[dtype] * (10 if dtype == np.float64 else 1), (n, side, uplo, trans,
                                                                                                func, thr)


def test_float16(pkg, oracle, workloads, cuda):
    for n, side, uplo, trans, func in itertools.product([64, 300, 1024], "LR", "LU", "NT", "SM"):
        A, B = workloads.problem(n, 24, side, uplo, seed=n)
        A16, B16 = A.astype(np.float16), B.astype(np.float16)
        exact = oracle.rectrxm(side, uplo, trans, 0.5, func, A16.astype(np.float64), B16.astype(np.float64))
        ref16 = oracle.rectrxm(side, uplo, trans, 0.5, func, A16, B16)
        X = _run(pkg, cuda, side, uplo, trans, 0.5, func, A16, B16, np.float16, True)
        e_gpu = oracle.rel_err(X, exact)
        e_ref = oracle.rel_err(ref16, exact)
        assert e_gpu < 1e-2 and e_gpu <= 2 * e_ref + 1e-3, (n, side, uplo, trans, func, e_gpu, e_ref)


def test_unreferenced_triangle_is_never_read(pkg, workloads, cuda):
    """Only the uplo triangle is read: NaNs in the other one change nothing."""
    for side, uplo, trans, func in itertools.product("LR", "LU", "NT", "SM"):
        A, B = workloads.problem(700, 9, side, uplo, seed=5)
        clean = _run(pkg, cuda, side, uplo, trans, 1.0, func, A, B, np.float64, True)
        dirty = A.copy()
        if uplo == "L":
            dirty[np.triu_indices(700, 1)] = np.nan
        else:
            dirty[np.tril_indices(700, -1)] = np.nan
        got = _run(pkg, cuda, side, uplo, trans, 1.0, func, dirty, B, np.float64, True)
        np.testing.assert_array_equal(got, clean)


def test_strided_views(pkg, oracle, workloads, cuda):
    """A and B embedded in larger arrays (leading dimension > rows)."""
    for side, func in itertools.product("LR", "SM"):
        A, B = workloads.problem(300, 20, side, "L", seed=9)
        ref = oracle.rectrxm(side, "L", "T", 0.5, func, A, B)
        X = _run(pkg, cuda, side, "L", "T", 0.5, func, A, B, np.float64, True, lda=333, ldb=B.shape[0] + 7)
        assert oracle.rel_err(X, ref) < 1e-14
        X = _run(pkg, cuda, side, "L", "T", 0.5, func, A, B, np.float64, False, lda=333, ldb=B.shape[0] + 7)
        assert oracle.rel_err(X, ref) < 1e-14


def test_transposed_view_of_A(pkg, oracle, workloads, cuda):
    """A passed as a transposed tensor view (Julia: Transpose(A) as the argument)."""
    import torch

    A, B = workloads.problem(400, 10, "L", "U", seed=4)
    ref = oracle.rectrxm("L", "L", "N", 1.0, "S", A.T.copy(order="F"), B)
    for native in (False, True):
        Ad = to_dev(A, np.float64, cuda).T  # lower-triangular view of an upper parent
        Bd = to_dev(B, np.float64, cuda)
        pkg.unified_rectrxm_("L", "L", "N", 1.0, "S", Ad, Bd, native=native)
        torch.cuda.synchronize()
        assert oracle.rel_err(to_host(Bd), ref) < 1e-14


def test_empty_and_single(pkg, oracle, cuda):
    import torch

    for n, m in [(0, 5), (5, 0), (1, 1), (1, 7)]:
        A = np.full((n, n), 2.0)
        B = np.ones((n, m))
        for func in "SM":
            X = _run(pkg, cuda, "L", "L", "N", 3.0, func, A, B, np.float64, True)
            if n and m:
                np.testing.assert_array_equal(X, oracle.rectrxm("L", "L", "N", 3.0, func, A, B))
    torch.cuda.synchronize()


def test_gemm_update_matches_oracle(pkg, oracle, cuda):
    import torch

    rng = np.random.default_rng(8)
    for dtype, (N, R, M), t1, t2 in itertools.product([np.float64, np.float32], [(129, 65, 33), (256, 300, 70)],
                                                      [False, True], [False, True]):
        C = rng.uniform(-1, 1, (N, M))
        X1 = rng.uniform(-1, 1, (R, N) if t1 else (N, R))
        X2 = rng.uniform(-1, 1, (M, R) if t2 else (R, M))
        ref = oracle.matmul(C.astype(dtype), X1.astype(dtype), X2.astype(dtype), -1.0, t1=t1, t2=t2)
        Cd = to_dev(C, dtype, cuda)
        a = to_dev(X1, dtype, cuda)
        b = to_dev(X2, dtype, cuda)
        pkg.GEMM_SUB_(Cd, a.T if t1 else a, b.T if t2 else b)
        torch.cuda.synchronize()
        assert oracle.rel_err(to_host(Cd), ref) < TOL[dtype]


@pytest.mark.parametrize("side,uplo", [("L", "L"), ("L", "U"), ("R", "L"), ("R", "U")])
def test_f64_leaf_one_rhs_per_thread(pkg, oracle, workloads, cuda, side, uplo):
    """Float64 diagonal blocks of up to 128 rows with at least 1024 right-hand
    sides take the one-right-hand-side-per-thread kernel (left-looking 32-row
    panels): partial panels, a partial last CTA (1100 = 8 x 128 + 76), both
    transposes, against the oracle and BLAS at the Float64 bound."""
    for n, trans in itertools.product([1, 5, 31, 32, 33, 100, 128], "NT"):
        A, B = workloads.problem(n, 1100, side, uplo, seed=n)
        X = _run(pkg, cuda, side, uplo, trans, 0.5, "S", A, B, np.float64, True)
        ref = oracle.rectrxm(side, uplo, trans, 0.5, "S", A, B)
        assert oracle.rel_err(X, ref) < 1e-14, (n, side, uplo, trans)
        assert oracle.rel_err(X, oracle.blas_rectrxm(side, uplo, trans, 0.5, "S", A, B)) < 1e-14


def test_f64_leaf_one_rhs_per_thread_exact(pkg, cuda):
    """Integer systems with power-of-two diagonals are solved exactly by every
    operation order: the one-right-hand-side-per-thread kernel must return the
    integers bit for bit."""
    import torch

    rng = np.random.default_rng(11)
    for n in (64, 100, 128):
        L = np.tril(rng.integers(-3, 4, (n, n)), -1).astype(np.int64)
        L[np.diag_indices(n)] = 2 ** rng.integers(0, 3, n)
        X = rng.integers(-8, 9, (n, 1100)).astype(np.int64)
        B = L @ X
        Ad = to_dev(L.astype(np.float64), np.float64, cuda)
        Bd = to_dev(B.astype(np.float64), np.float64, cuda)
        pkg.unified_rectrxm_("L", "L", "N", 1.0, "S", Ad, Bd, native=True)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(to_host(Bd), X.astype(np.float64))


@pytest.mark.parametrize("cw", [56, 64, 96, 112, 128])
def test_f64_leaf_columns_per_cta(pkg, oracle, workloads, cuda, cw, monkeypatch):
    """Every width of the one-right-hand-side-per-thread leaf (NLA_LEAF_CW
    pins it; by default the fewest columns per CTA that fit one wave): exact
    integer solves bit for bit, and a random system with a partial last CTA
    against BLAS at the Float64 bound."""
    import torch

    monkeypatch.setenv("NLA_LEAF_CW", str(cw))
    rng = np.random.default_rng(cw)
    for n in (37, 128):
        L = np.tril(rng.integers(-3, 4, (n, n)), -1).astype(np.int64)
        L[np.diag_indices(n)] = 2 ** rng.integers(0, 3, n)
        X = rng.integers(-8, 9, (n, 1100)).astype(np.int64)
        Ad = to_dev(L.astype(np.float64), np.float64, cuda)
        Bd = to_dev((L @ X).astype(np.float64), np.float64, cuda)
        pkg.unified_rectrxm_("L", "L", "N", 1.0, "S", Ad, Bd, native=True)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(to_host(Bd), X.astype(np.float64))
    for side, trans in itertools.product("LR", "NT"):
        A, B = workloads.problem(128, 1237, side, "U", seed=cw)
        X = _run(pkg, cuda, side, "U", trans, -1.5, "S", A, B, np.float64, True)
        assert oracle.rel_err(X, oracle.blas_rectrxm(side, "U", trans, -1.5, "S", A, B)) < 1e-14, (cw, side, trans)


@pytest.mark.parametrize("func", ["S", "M"])
def test_trsm_trmm_wrappers_with_diag(pkg, oracle, workloads, cuda, func):
    """trsm()/trmm() (src/trsm.jl:186-204, src/trmm.jl:430-448) through the
    recursion: every side/uplo/transa, diag 'N' and 'U' (unit diagonal, never
    read: the stored diagonal is NaN), n from one base case to a recursive
    300, against BLAS at the Float64 bound."""
    import torch

    fn = pkg.trsm if func == "S" else pkg.trmm
    for n, m, side, uplo, transa, diag in itertools.product([17, 300], [9], "LR", "LU", "NT", "NU"):
        A, B = workloads.problem(n, m, side, uplo, seed=n + (diag == "U"))
        An = A.copy()
        if diag == "U":
            An[np.diag_indices(n)] = np.nan
        Ad, Bd = to_dev(An, np.float64, cuda), to_dev(B, np.float64, cuda)
        fn(side, uplo, transa, diag, Ad, Bd, 0.5)
        torch.cuda.synchronize()
        Aref = A.copy()
        if diag == "U":
            Aref[np.diag_indices(n)] = 1.0
        ref = oracle.blas_rectrxm(side, uplo, transa, 0.5, func, Aref, B)
        got = to_host(Bd)
        assert np.isfinite(got).all(), (n, side, uplo, transa, diag)
        assert oracle.rel_err(got, ref) < 1e-14, (n, side, uplo, transa, diag)
