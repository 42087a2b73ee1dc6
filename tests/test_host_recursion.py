"""Host-side logic of the Python mirror, checked on the CPU.

The mirror's recursion (unified_rec) only slices views and calls the base
cases and the updates.  Backing those calls with the oracle's own base-case and
matmul routines on numpy views must reproduce the oracle's full recursion bit
for bit, which pins the split points, the forward/backward orderings, the
choice of GEMM operands and the alpha placement."""

import itertools

import numpy as np
import pytest


@pytest.fixture()
def cpu_backed(pkg, oracle, monkeypatch):
    rt = pkg.rectrxm
    calls = {"leaf": 0, "gemm": 0, "scale": 0}

    def diag_block(func, side, uplo, A, B):
        B[...] = oracle.leaf(func, side, uplo, np.asarray(A), np.asarray(B))
        calls["leaf"] += 1
        return B

    def matmul(output, input1, input2, alpha=1.0):
        output[...] = oracle.matmul(np.asarray(output), np.asarray(input1), np.asarray(input2), alpha)
        calls["gemm"] += 1
        return output

    def scale(B, alpha):
        if B.dtype == np.float64:
            B[...] = alpha * B
        else:
            B[...] = (np.float64(alpha) * B.astype(np.float64)).astype(B.dtype)
        calls["scale"] += 1
        return B

    monkeypatch.setattr(rt, "_diag_block", diag_block)
    monkeypatch.setattr(rt, "matmul_", matmul)
    monkeypatch.setattr(rt, "scale_", scale)
    return rt, calls


def _call(rt, side, uplo, trans, alpha, func, A, B, thresholds):
    """unified_rectrxm_'s non-native path without the CUDA-only checks."""
    n = A.shape[0]
    threshold = thresholds[1]
    if trans in ("T", "C"):
        A = A.T
        uplo = "U" if uplo == "L" else "L"
    if func == "S":
        threshold = thresholds[0]
        rt.scale_(B, alpha)
    rt.unified_rec(func, side, uplo, A, n, B, threshold)
    if func == "M":
        rt.scale_(B, alpha)
    return B


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_mirror_recursion_matches_oracle(cpu_backed, oracle, workloads, dtype):
    rt, calls = cpu_backed
    for n, side, uplo, trans, func in itertools.product([37, 64, 100], "LR", "LU", "NT", "SM"):
        A, B = workloads.problem(n, 5, side, uplo, seed=n)
        A = A.astype(dtype)
        B = B.astype(dtype)
        expect = oracle.rectrxm(side, uplo, trans, 0.5, func, A, B, thresholds=(16, 8))
        got = _call(rt, side, uplo, trans, 0.5, func, A.copy(order="F"), B.copy(order="F"), (16, 8))
        np.testing.assert_array_equal(got, expect)
    assert calls["leaf"] > 0 and calls["gemm"] > 0


def test_mirror_launch_counts(cpu_backed, workloads):
    """n = 1024 with the reference's thresholds: 4 solve leaves + 3 updates,
    64 multiply leaves + 63 updates (src/rectrxm.jl:52,63)."""
    rt, calls = cpu_backed
    A, B = workloads.problem(1024, 1, "L", "L", seed=1)
    _call(rt, "L", "L", "N", 1.0, "S", A, B.copy(order="F"), (256, 16))
    assert (calls["leaf"], calls["gemm"]) == (4, 3)
    calls.update(leaf=0, gemm=0)
    _call(rt, "L", "L", "N", 1.0, "M", A, B.copy(order="F"), (256, 16))
    assert (calls["leaf"], calls["gemm"]) == (64, 63)
