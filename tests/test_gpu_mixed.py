"""Mixed-precision form against FP64 references.

Bounds (relative Frobenius error against the FP64 oracle's answer, on
well-conditioned seeded systems):
  no refinement, BF16 x3 or FP16 x2 slices:   < 1e-5
  with 2 refinement sweeps:                   < 1e-13 (plain FP64 level), and
                                              backward error within 2x of the
                                              plain FP64 path's (+1e-3)
  multiply (no refinement), BF16 x3:          < 1e-5
"""

import itertools
import os

import numpy as np
import pytest

from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu


def _mixed(pkg, cuda, side, uplo, trans, alpha, func, A, B, **kw):
    import torch

    Ad, Bd = to_dev(A, np.float64, cuda), to_dev(B, np.float64, cuda)
    out = pkg.unified_rectrxm_mixed_(side, uplo, trans, alpha, func, Ad, Bd, **kw)
    pkg.device_status(Bd)
    torch.cuda.synchronize()
    if isinstance(out, tuple):
        return to_host(Bd), out[1]
    return to_host(Bd)


@pytest.mark.parametrize("lowp,terms", [("bf16", 3), ("f16", 2)])
def test_mixed_solve_all_forms(pkg, oracle, workloads, cuda, lowp, terms):
    nthreads = os.cpu_count() or 1
    for n, side, uplo, trans in itertools.product([300, 1000], "LR", "LU", "NT"):
        A, B = workloads.problem(n, 40, side, uplo, seed=n + 1)
        ref = oracle.rectrxm(side, uplo, trans, 0.5, "S", A, B, nthreads=nthreads)
        X0 = _mixed(pkg, cuda, side, uplo, trans, 0.5, "S", A, B, lowp=lowp, split_terms=terms, sweeps=0, cutoff=64)
        assert oracle.rel_err(X0, ref) < 1e-5, (n, side, uplo, trans)
        X2 = _mixed(pkg, cuda, side, uplo, trans, 0.5, "S", A, B, lowp=lowp, split_terms=terms, sweeps=2,
                    cutoff=64)
        assert oracle.rel_err(X2, ref) < 1e-13, (n, side, uplo, trans)


def test_refinement_matches_plain_backward_error(pkg, oracle, workloads, cuda):
    import torch

    n, m = 2048, 64
    A, B = workloads.problem(n, m, "L", "L", seed=21)
    X, corr = _mixed(pkg, cuda, "L", "L", "N", 1.0, "S", A, B, sweeps=3, corrections=True, residual="split")
    Ad, Bd = to_dev(A, np.float64, cuda), to_dev(B, np.float64, cuda)
    pkg.unified_rectrxm_("L", "L", "N", 1.0, "S", Ad, Bd, native=True)
    torch.cuda.synchronize()
    Xp = to_host(Bd)
    be_mixed = oracle.backward_error("L", "L", "N", 1.0, A, X, B)
    be_plain = oracle.backward_error("L", "L", "N", 1.0, A, Xp, B)
    assert be_mixed <= 2 * be_plain + 1e-3, (be_mixed, be_plain)
    assert corr[0] < 1e-5 and corr[-1] < corr[0], corr


@pytest.mark.parametrize("side,uplo,trans", [("R", "U", "T"), ("L", "L", "N"), ("L", "U", "T"), ("R", "L", "N")])
def test_mixed_multiply(pkg, oracle, workloads, cuda, side, uplo, trans):
    A, B = workloads.problem(777, 50, side, uplo, seed=3)
    ref = oracle.rectrxm(side, uplo, trans, -2.0, "M", A, B, nthreads=os.cpu_count() or 1)
    X = _mixed(pkg, cuda, side, uplo, trans, -2.0, "M", A, B, split_terms=3)
    assert oracle.rel_err(X, ref) < 1e-5


def test_mixed_rejects_bad_options(pkg, cuda):
    import torch

    A = to_dev(np.eye(4), np.float64, cuda)
    B = to_dev(np.ones((4, 2)), np.float64, cuda)
    with pytest.raises(ValueError):
        pkg.unified_rectrxm_mixed_("L", "L", "N", 1.0, "S", A, B, split_terms=5)
    with pytest.raises(ValueError):
        pkg.unified_rectrxm_mixed_("L", "L", "N", 1.0, "S", A.float(), B.float())
    torch.cuda.synchronize()


def test_exact_updates_without_refinement(pkg, oracle, workloads, cuda):
    """split_terms = 7: FP64-accurate updates, FP64 leaves, no refinement."""
    for side, uplo, trans in [("L", "L", "N"), ("R", "U", "T"), ("L", "U", "T"), ("R", "L", "N")]:
        A, B = workloads.problem(1500, 60, side, uplo, seed=17)
        ref = oracle.rectrxm(side, uplo, trans, 1.0, "S", A, B, nthreads=os.cpu_count() or 1)
        X = _mixed(pkg, cuda, side, uplo, trans, 1.0, "S", A, B, split_terms=7, sweeps=0)
        assert oracle.rel_err(X, ref) < 1e-13


@pytest.mark.parametrize("residual", ["split", "fp64"])
def test_refinement_residual_modes(pkg, oracle, workloads, cuda, residual):
    for side, uplo, trans in [("L", "L", "N"), ("R", "U", "T"), ("R", "L", "T"), ("L", "U", "N")]:
        A, B = workloads.problem(900, 50, side, uplo, seed=23)
        ref = oracle.rectrxm(side, uplo, trans, 0.5, "S", A, B, nthreads=os.cpu_count() or 1)
        X = _mixed(pkg, cuda, side, uplo, trans, 0.5, "S", A, B, split_terms=2, sweeps=3, residual=residual)
        assert oracle.rel_err(X, ref) < 1e-14, (side, uplo, trans)


@pytest.mark.parametrize("diag", ["N", "U"])
def test_inverse_leaves_match_substitution(pkg, oracle, workloads, cuda, diag, monkeypatch):
    """Exact 7-slice solves apply each leaf block through its FP64 inverse on
    the tensor cores (X := inv(T) X).  Over every side, uplo and trans,
    sizes with ragged leaves (n = 1, 65, 1000, 1500) and a unit diagonal,
    the result matches the substitution leaves (NLA_MIXED_INV_LEAF=0) and
    the oracle at the Float64 tolerance."""
    import torch

    nthreads = os.cpu_count() or 1
    for k, (n, side, uplo, trans) in enumerate(itertools.product([1, 65, 1000], "LR", "LU", "NT")):
        A, B = workloads.problem(n, 37, side, uplo, seed=300 + k)
        if diag == "U":
            A = np.array(A) / max(n, 1)  # well conditioned with a unit diagonal too
            A[np.diag_indices(n)] = 1.0  # what the unit solve assumes; the device copy gets NaNs there
        out = {}
        for inv in ("1", "0"):
            monkeypatch.setenv("NLA_MIXED_INV_LEAF", inv)
            An = np.array(A)
            if diag == "U":
                An[np.diag_indices(n)] = np.nan
            Ad, Bd = to_dev(An, np.float64, cuda), to_dev(B, np.float64, cuda)
            pkg.trsm(side, uplo, trans, diag, Ad, Bd, 0.5, mixed=True)
            pkg.device_status(Bd)
            torch.cuda.synchronize()
            out[inv] = to_host(Bd)
        ref = oracle.rectrxm(side, uplo, trans, 0.5, "S", A, B, nthreads=nthreads)
        assert np.isfinite(out["1"]).all(), (n, side, uplo, trans)
        assert oracle.rel_err(out["1"], ref) < 1e-13, (n, side, uplo, trans)
        assert oracle.rel_err(out["1"], out["0"]) < 1e-13, (n, side, uplo, trans)


def test_leaf_pairs_match_separate_leaves(pkg, oracle, workloads, cuda, monkeypatch):
    """A recursion node whose two halves are both leaves runs as one launch
    (leaf, update, leaf: leaf_pair_kernel).  Over every side, uplo and trans,
    nodes of 64 + 1, 64 + 36 and 64 + 64 rows and the nodes inside n = 1000,
    with right-hand-side counts that leave a partial block of 128, the result
    matches the separate launches (NLA_LEAF_PAIR=0) to a few rounding errors
    and the oracle at the Float64 tolerance.  A NaN or an infinity in B
    spreads over its own right-hand side only, as in the separate launches."""
    import torch

    nthreads = os.cpu_count() or 1
    cases = [(65, 37), (100, 300), (128, 129), (1000, 257)]
    for k, ((n, m), side, uplo, trans) in enumerate(itertools.product(cases, "LR", "LU", "NT")):
        A, B = workloads.problem(n, m, side, uplo, seed=500 + k)
        out = {}
        for pair in ("1", "0"):
            monkeypatch.setenv("NLA_LEAF_PAIR", pair)
            Ad, Bd = to_dev(A, np.float64, cuda), to_dev(B, np.float64, cuda)
            pkg.trsm(side, uplo, trans, "N", Ad, Bd, -1.5, mixed=True)
            pkg.device_status(Bd)
            torch.cuda.synchronize()
            out[pair] = to_host(Bd)
        ref = oracle.rectrxm(side, uplo, trans, -1.5, "S", A, B, nthreads=nthreads)
        assert np.isfinite(out["1"]).all(), (n, m, side, uplo, trans)
        assert oracle.rel_err(out["1"], ref) < 1e-13, (n, m, side, uplo, trans)
        assert oracle.rel_err(out["1"], out["0"]) < 1e-14, (n, m, side, uplo, trans)

    n, m = 100, 300
    for side in "LR":
        A, B = workloads.problem(n, m, side, "L", seed=77)
        B = np.array(B)
        if side == "L":
            B[5, 3], B[70, 200] = np.nan, np.inf
        else:
            B[3, 5], B[200, 70] = np.nan, np.inf
        out = {}
        for pair in ("1", "0"):
            monkeypatch.setenv("NLA_LEAF_PAIR", pair)
            Ad, Bd = to_dev(A, np.float64, cuda), to_dev(B, np.float64, cuda)
            pkg.trsm(side, "L", "N", "N", Ad, Bd, 1.0, mixed=True)
            pkg.device_status(Bd)
            torch.cuda.synchronize()
            out[pair] = to_host(Bd)
        bad = ~np.isfinite(out["0"])
        assert bad.any(), side
        assert np.array_equal(bad, ~np.isfinite(out["1"])), side
        rhs_axis = 0 if side == "L" else 1  # right-hand sides are B's columns (L) or rows (R)
        touched = bad.any(axis=rhs_axis)
        assert touched.sum() == 2, side
        good = out["0"][:, ~touched] if side == "L" else out["0"][~touched, :]
        good1 = out["1"][:, ~touched] if side == "L" else out["1"][~touched, :]
        assert oracle.rel_err(good1, good) < 1e-14, side
