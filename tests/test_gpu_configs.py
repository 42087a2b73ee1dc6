"""GPU parity at the sizes the benchmark configurations are quoted on, checked
against the oracle (the reference algorithm restated on the CPU) on sampled
right-hand sides.

Columns of B are independent for side 'L' and rows for side 'R', and the
oracle computes each one with the same arithmetic whether it is alone or in
the full matrix, so a sample of columns (rows) solved by the oracle is the
oracle's answer for those columns (rows) of the full problem.

Tolerances (relative Frobenius error over the sample):
  plain Float64                        1e-14 against the oracle
                                       (test/unified_rectrxm.jl:42);
  plain Float32                        1e-5 (test/trsm.jl:55);
  mixed Float64, exact 7-slice updates 1e-13 against the Float64 oracle, and
                                       a backward error at most 2x that of the
                                       plain Float64 solve of the same inputs;
  mixed Float64, 3-term BF16 split     1e-6 against the Float64 oracle (24
                                       bits of operand per term set);
  Float16 TRSM                         within 2x (+1e-3) of the reference
                                       algorithm's own Float16 error against
                                       the Float64 answer, and below 1e-2;
  batched                              Float64 1e-13, Float32 1e-5, mixed
                                       Float64 (two sweeps) 1e-13.
"""

import itertools
import os

import numpy as np
import pytest

from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1
_PROBLEMS = {}


def _problem(n, side, uplo, seed):
    """A (n x n, named triangle: off-diagonals N(0,1)/sqrt(n), diagonal
    2 + |N(0,1)|) and B (n x n, uniform on [-1, 1]) as in the configuration,
    numpy PCG64 with the given seed; cached per (n, uplo, seed)."""
    key = (n, uplo, seed)
    if key not in _PROBLEMS:
        if any(k[0] != n for k in _PROBLEMS):
            _PROBLEMS.clear()
        rng = np.random.default_rng(seed)
        Z = rng.standard_normal((n, n)) / np.sqrt(n)
        A = np.tril(Z, -1) if uplo == "L" else np.triu(Z, 1)
        del Z
        A[np.diag_indices(n)] = 2.0 + np.abs(rng.standard_normal(n))
        B = rng.uniform(-1.0, 1.0, (n, n))
        _PROBLEMS[key] = (np.asfortranarray(A), np.asfortranarray(B))
    return _PROBLEMS[key]


def _sample(side, B, idx):
    return np.asfortranarray(B[:, idx] if side == "L" else B[idx, :])


def _oracle_sample(oracle, side, uplo, trans, alpha, func, A, B, idx, dtype):
    return oracle.rectrxm(side, uplo, trans, alpha, func, A.astype(dtype), _sample(side, B, idx).astype(dtype),
                          nthreads=THREADS)


# ---------------------------------------------------------------------------
# Configuration 1: plain, dtype-preserving TRSM and TRMM over all 8
# side/uplo/trans forms, alpha = 0.5, B n x n.
# ---------------------------------------------------------------------------
CONFIG1 = [(4096, dt, func, side, uplo, trans) for dt, func, side, uplo, trans in
           itertools.product(["f64", "f32"], "SM", "LR", "LU", "NT")]
CONFIG1 += [(8192, "f32", "S", "L", "L", "N"), (8192, "f32", "M", "R", "U", "T"), (8192, "f64", "S", "L", "U", "T"),
            (16384, "f32", "S", "R", "L", "N"), (16384, "f32", "M", "L", "L", "T"),
            (16384, "f64", "S", "L", "L", "N")]


@pytest.mark.parametrize("n,dt,func,side,uplo,trans", CONFIG1)
def test_config1_plain(pkg, oracle, cuda, n, dt, func, side, uplo, trans):
    import torch

    dtype = {"f64": np.float64, "f32": np.float32}[dt]
    tol = {"f64": 1e-14, "f32": 1e-5}[dt]
    A, B = _problem(n, side, uplo, seed=1)
    Ad, Bd = to_dev(A, dtype, cuda), to_dev(B, dtype, cuda)
    pkg.unified_rectrxm_(side, uplo, trans, 0.5, func, Ad, Bd, native=True)
    torch.cuda.synchronize()
    idx = np.random.default_rng(n).choice(n, 16, replace=False)
    X = to_host(Bd[:, idx] if side == "L" else Bd[idx, :])
    del Ad, Bd
    ref = _oracle_sample(oracle, side, uplo, trans, 0.5, func, A, B, idx, dtype)
    assert oracle.rel_err(X, ref) < tol


# ---------------------------------------------------------------------------
# Configuration 2 (the benchmark's headline): Float64 TRSM L/L/N, n = m =
# 16384, seed 0, mixed form with exact 7-slice BF16 updates and no sweep.
# ---------------------------------------------------------------------------
def test_config2_headline_exact7(pkg, oracle, cuda):
    import torch

    import bench

    n = m = 16384
    A_h, B_h = bench.make_inputs(n, m)  # the benchmark's own seed-0 inputs
    A = torch.from_numpy(np.ascontiguousarray(A_h.T)).to(cuda).T
    B0 = torch.from_numpy(np.ascontiguousarray(B_h.T)).to(cuda).T
    X = torch.empty_like(B0.T).T
    X.copy_(B0)
    pkg.unified_rectrxm_mixed_("L", "L", "N", 1.0, "S", A, X, split_terms=7, sweeps=0)
    pkg.device_status(X)
    P = torch.empty_like(B0.T).T
    P.copy_(B0)
    pkg.unified_rectrxm_("L", "L", "N", 1.0, "S", A, P, native=True)
    torch.cuda.synchronize()
    idx = np.arange(0, m, m // 64)
    ref = oracle.rectrxm("L", "L", "N", 1.0, "S", A_h, np.asfortranarray(B_h[:, idx]), nthreads=THREADS)
    assert oracle.rel_err(to_host(X[:, idx]), ref) < 1e-13

    # Backward errors on the same columns, residuals in double-double.
    cols = torch.from_numpy(idx).to(cuda)
    an = float(torch.tril(A).abs().sum(dim=1).max())

    def berr(Y):
        Ys = Y[:, cols].contiguous().T.contiguous().T
        Bs = B0[:, cols].contiguous().T.contiguous().T
        R = torch.empty_like(Ys.T).T
        pkg.residual_("L", "L", "N", 1.0, A, Ys, Bs, R, residual="dd")
        torch.cuda.synchronize()
        return float(R.abs().sum(dim=1).max()) / (an * float(Ys.abs().sum(dim=1).max()) * n * 2.0 ** -53)

    b_mixed, b_plain = berr(X), berr(P)
    assert b_mixed <= 2.0 * b_plain, (b_mixed, b_plain)


# ---------------------------------------------------------------------------
# Configuration 3: mixed TRMM R/U/T n = 12288 with a 3-term BF16 split, and a
# Float16 TRSM n = 8192, m = 4096 on the FP16 tensor path.
# ---------------------------------------------------------------------------
def test_config3_trmm_bf16x3(pkg, oracle, cuda):
    import torch

    n = 12288
    A_h, B_h = _problem(n, "R", "U", seed=3)
    A = torch.from_numpy(np.ascontiguousarray(A_h.T)).to(cuda).T
    X = torch.from_numpy(np.ascontiguousarray(B_h.T)).to(cuda).T
    pkg.unified_rectrxm_mixed_("R", "U", "T", 1.0, "M", A, X, lowp="bf16", split_terms=3)
    pkg.device_status(X)
    idx = np.random.default_rng(12).choice(n, 16, replace=False)
    got = to_host(X[idx, :])
    del A, X
    ref = _oracle_sample(oracle, "R", "U", "T", 1.0, "M", A_h, B_h, idx, np.float64)
    assert oracle.rel_err(got, ref) < 1e-6


def test_config3_trsm_f16(pkg, oracle, cuda):
    import torch

    n, m = 8192, 4096
    rng = np.random.default_rng(4)
    T = np.tril(rng.standard_normal((n, n)) / np.sqrt(n), -1)
    T[np.diag_indices(n)] = 2.0 + np.abs(rng.standard_normal(n))
    A16 = np.asfortranarray(T.astype(np.float16))
    del T
    B16 = np.asfortranarray(rng.uniform(-1, 1, (n, m)).astype(np.float16))
    Ad, Bd = to_dev(A16, np.float16, cuda), to_dev(B16, np.float16, cuda)
    pkg.unified_rectrxm_("L", "L", "N", 1.0, "S", Ad, Bd, native=True)
    torch.cuda.synchronize()
    idx = np.random.default_rng(13).choice(m, 16, replace=False)
    got = to_host(Bd[:, idx])
    del Ad, Bd
    exact = oracle.blas_rectrxm("L", "L", "N", 1.0, "S", A16.astype(np.float64),
                                np.asfortranarray(B16[:, idx].astype(np.float64)))
    ref16 = oracle.rectrxm("L", "L", "N", 1.0, "S", A16, np.asfortranarray(B16[:, idx]), nthreads=THREADS)
    e_gpu, e_ref = oracle.rel_err(got, exact), oracle.rel_err(ref16, exact)
    assert e_gpu < 2 * e_ref + 1e-3 and e_gpu < 1e-2, (e_gpu, e_ref)


# ---------------------------------------------------------------------------
# Configuration 4: the full batch of 10,000 uneven systems, seed 7, in
# Float32, Float64 and mixed Float64 (two refinement sweeps); about nine
# sampled systems from each size bucket against the oracle.
# ---------------------------------------------------------------------------
def _bucket_sample(n, per_bucket, seed):
    from nextla_gb300 import batched

    rng = np.random.default_rng(seed)
    b = np.array([batched.bucket_of(int(v)) for v in n])
    pick = []
    for k in range(6):
        ids = np.flatnonzero(b == k)
        pick += list(rng.choice(ids, min(per_bucket, len(ids)), replace=False))
    return sorted(int(i) for i in pick)


def _system(A_pool, B_pool, s):
    n, m, a_off, lda, b_off, ldb = s
    A = A_pool[a_off:a_off + n * n].reshape(n, n).T.detach().cpu().numpy().astype(np.float64)
    B = B_pool[b_off:b_off + n * m].reshape(m, n).T.detach().cpu().numpy().astype(np.float64)
    return A, B


@pytest.mark.parametrize("form", ["f32", "f64", "mixed"])
def test_config4_full_batch(pkg, oracle, cuda, form):
    import torch

    from nextla_gb300 import batched

    dtype = torch.float32 if form == "f32" else torch.float64
    n, m = batched.uneven_sizes(count=10000, seed=7)
    A, B0, systems = batched.make_batch(n, m, dtype, cuda, seed=7)
    plan = batched.BatchPlan(dtype, "L", "N", systems)
    B = B0.clone()
    if form == "mixed":
        plan.solve_mixed(1.0, A, B, sweeps=2)
    else:
        plan.solve(1.0, A, B, mode="graph")
    pkg.device_status(B)
    plan.close()
    np_dt = np.float32 if form == "f32" else np.float64
    tol = 1e-5 if form == "f32" else 1e-13
    picks = _bucket_sample(n, 9, seed=70)
    assert len(picks) >= 50
    for i in picks:
        Ai, Bi = _system(A, B0, systems[i])
        ref = oracle.rectrxm("L", "L", "N", 1.0, "S", Ai.astype(np_dt), Bi.astype(np_dt))
        _, Xi = _system(A, B, systems[i])
        assert oracle.rel_err(Xi, ref) < tol, (i, systems[i][:2])
