"""The package's own callers of the path, run through it on the GPU.

getrf2! (src/lu.jl:277) solves A[1:n1, n1+1:end] with the unit lower triangle
of A[1:n1, 1:n1] by BLAS.trsm!('L', 'L', 'N', 'U').  The diagonal of that
block holds U's diagonal, so the unit-diagonal flag must keep it unread.

The blocked LAUUM (src/lauum.jl:110 for upper, :162 for lower) multiplies
each off-diagonal panel by the transposed diagonal block.

Both operate on views of one device array.  Checked against scipy/numpy in
Float64 (relative error < 1e-13, plain and with exact tensor-core updates,
``mixed=True``) and Float32 (< 1e-5), with every element outside the updated
panel unchanged bit for bit.
"""

import numpy as np
import pytest

from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype,tol,mixed", [(np.float64, 1e-13, False), (np.float32, 1e-5, False),
                                             (np.float64, 1e-13, True)])
@pytest.mark.parametrize("n,n1", [(700, 350), (513, 256), (64, 31)])
def test_getrf2_trsm(pkg, cuda, dtype, tol, mixed, n, n1):
    import torch
    from scipy.linalg import solve_triangular

    rng = np.random.default_rng(n + n1)
    A = rng.standard_normal((n, n))
    # The leading block as getrf2! leaves it: a unit lower L (strict part
    # small enough to keep the solve well conditioned) under U's diagonal.
    A[:n1, :n1] = np.tril(A[:n1, :n1], -1) / np.sqrt(n1) + np.triu(A[:n1, :n1])
    A[np.arange(n1), np.arange(n1)] = rng.uniform(5.0, 9.0, n1)  # U's diagonal: never read
    Ad = to_dev(A, dtype, cuda)
    before = to_host(Ad)
    pkg.getrf2_trsm_(Ad, n1, mixed=mixed)
    torch.cuda.synchronize()
    got = to_host(Ad)
    Af = before
    L11 = np.tril(Af[:n1, :n1], -1) + np.eye(n1)
    want = solve_triangular(L11, Af[:n1, n1:], lower=True, unit_diagonal=True)
    rel = np.linalg.norm(got[:n1, n1:] - want) / np.linalg.norm(want)
    assert rel < tol, rel
    mask = np.ones_like(got, dtype=bool)
    mask[:n1, n1:] = False
    assert np.array_equal(got[mask], before[mask])


@pytest.mark.parametrize("dtype,tol,mixed", [(np.float64, 1e-13, False), (np.float32, 1e-5, False),
                                             (np.float64, 1e-13, True)])
@pytest.mark.parametrize("uplo", ["U", "L"])
def test_lauum_offdiag_trmm(pkg, cuda, dtype, tol, mixed, uplo):
    import torch

    n, ib = 600, 128
    rng = np.random.default_rng(7 if uplo == "U" else 8)
    T = np.triu(rng.standard_normal((n, n))) if uplo == "U" else np.tril(rng.standard_normal((n, n)))
    for i in range(0, n, ib):
        b = min(ib, n - i)
        Ad = to_dev(T, dtype, cuda)
        before = to_host(Ad)
        pkg.lauum_offdiag_trmm_(uplo, Ad, i, b, mixed=mixed)
        torch.cuda.synchronize()
        got = to_host(Ad)
        blk = before[i:i + b, i:i + b]
        if uplo == "U":
            want = before[:i, i:i + b] @ blk.T
            panel = (slice(0, i), slice(i, i + b))
        else:
            want = blk.T @ before[i:i + b, :i]
            panel = (slice(i, i + b), slice(0, i))
        if i > 0:
            rel = np.linalg.norm(got[panel] - want) / np.linalg.norm(want)
            assert rel < tol, (i, rel)
        mask = np.ones_like(got, dtype=bool)
        mask[panel] = False
        assert np.array_equal(got[mask], before[mask]), i
