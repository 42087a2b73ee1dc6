"""Tensor-core (tcgen05) update kernel against torch references.

Float16 plain path: the update must equal the FP32 product of the Float16
inputs rounded once to Float16 (relative error < 2e-3, i.e. about 2 Float16
ulps).  Mixed path: the error against an FP64 product must fall with the
number of slices: BF16 (8-bit slices) 1/2/3 terms < 6e-2 / 1e-3 / 2e-5,
FP16 (11-bit slices) < 1.2e-2 / 2e-5 / 2e-5 (FP32 accumulation bounds the last);
the operands' rows are scaled by exp(2 N(0,1)), so transposed operands carry
that range along K, inside one row's power-of-two scale.
"""

import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _col_major(t):
    return t.T.contiguous().T


def _rel(x, ref):
    import torch

    return float(torch.linalg.norm((x - ref).double()) / torch.linalg.norm(ref.double()))


def test_umma_f16_update_small(pkg, cuda):
    import torch

    g = torch.Generator(device=cuda).manual_seed(0)
    for (N, R, M), t1, t2 in itertools.product([(128, 64, 128), (300, 200, 257), (1024, 512, 640)], [False, True],
                                               [False, True]):
        C = _col_major(torch.rand(N, M, device=cuda, generator=g).half())
        A = _col_major(torch.rand(R, N, device=cuda, generator=g).half()) if t1 else \
            _col_major(torch.rand(N, R, device=cuda, generator=g).half())
        B = _col_major(torch.rand(M, R, device=cuda, generator=g).half()) if t2 else \
            _col_major(torch.rand(R, M, device=cuda, generator=g).half())
        opA = A.T if t1 else A
        opB = B.T if t2 else B
        ref = (C.float() - opA.float() @ opB.float()).half()
        pkg.GEMM_SUB_(C, opA, opB)
        pkg.device_status(C)
        assert _rel(C, ref) < 2e-3, (N, R, M, t1, t2)


@pytest.mark.parametrize("lowp", ["bf16", "f16"])
def test_mixed_update_error_falls_with_terms(pkg, cuda, lowp):
    import torch

    g = torch.Generator(device=cuda).manual_seed(1)
    bounds = {"bf16": [6e-2, 1e-3, 2e-5], "f16": [1.2e-2, 2e-5, 2e-5]}[lowp]
    for (N, R, M), t1 in itertools.product([(256, 300, 130), (700, 1024, 515)], [False, True]):
        C0 = _col_major(torch.randn(N, M, device=cuda, generator=g, dtype=torch.float64))
        A = torch.randn(R if t1 else N, N if t1 else R, device=cuda, generator=g, dtype=torch.float64)
        A = _col_major(A * torch.exp(2 * torch.randn(A.shape[0], 1, device=cuda, generator=g, dtype=torch.float64)))
        B = _col_major(torch.randn(R, M, device=cuda, generator=g, dtype=torch.float64))
        opA = A.T if t1 else A
        prod = opA @ B
        ref = C0 - prod
        errs = []
        for S in (1, 2, 3):
            C = C0.clone().T.contiguous().T
            pkg.matmul_mixed_(C, opA, B, -1.0, lowp=lowp, split_terms=S)
            pkg.device_status(C)
            # error relative to the size of the product
            errs.append(float(torch.linalg.norm(C - ref) / torch.linalg.norm(prod)))
        for S, (e, b) in enumerate(zip(errs, bounds), 1):
            assert e < b, (lowp, N, R, M, t1, S, errs)
        assert errs[1] < errs[0]


def test_mixed_update_exact_for_short_integers(pkg, cuda):
    """Products of values with at most 8 significant bits are exact with one
    BF16 slice when the sum fits FP32: the result must be bit-exact."""
    import torch

    g = torch.Generator(device=cuda).manual_seed(2)
    N, R, M = 256, 128, 256
    A = _col_major(torch.randint(-100, 101, (N, R), device=cuda, generator=g).double())
    B = _col_major(torch.randint(-100, 101, (R, M), device=cuda, generator=g).double())
    C = _col_major(torch.zeros(N, M, device=cuda, dtype=torch.float64))
    ref = A @ B
    pkg.matmul_mixed_(C, A, B, 1.0, lowp="bf16", split_terms=2)
    pkg.device_status(C)
    assert torch.equal(C, ref)


def test_mixed_update_nonfinite_rows_give_nan(pkg, cuda):
    import torch

    N, R, M = 128, 64, 128
    A = _col_major(torch.ones(N, R, device=cuda, dtype=torch.float64))
    A[5, 3] = float("inf")
    B = _col_major(torch.ones(R, M, device=cuda, dtype=torch.float64))
    C = _col_major(torch.zeros(N, M, device=cuda, dtype=torch.float64))
    pkg.matmul_mixed_(C, A, B, 1.0)
    pkg.device_status(C)
    assert torch.isnan(C[5]).all()
    assert torch.isfinite(C[:5]).all() and torch.isfinite(C[6:]).all()
    assert float(C[0, 0]) == 64.0


def test_exact_update_is_fp64_accurate(pkg, cuda):
    """7 BF16 slices with exact slice products: error below FP64 GEMM level."""
    import torch

    g = torch.Generator(device=cuda).manual_seed(3)
    for (N, R, M), t1 in itertools.product([(256, 300, 130), (700, 2500, 515)], [False, True]):
        C0 = _col_major(torch.randn(N, M, device=cuda, generator=g, dtype=torch.float64))
        A = torch.randn(R if t1 else N, N if t1 else R, device=cuda, generator=g, dtype=torch.float64)
        A = _col_major(A * torch.exp(torch.randn(A.shape[0], 1, device=cuda, generator=g, dtype=torch.float64)))
        B = _col_major(torch.randn(R, M, device=cuda, generator=g, dtype=torch.float64))
        opA = A.T if t1 else A
        C = C0.clone().T.contiguous().T
        pkg.matmul_mixed_(C, opA, B, -1.0, split_terms=7)
        pkg.device_status(C)
        scale = opA.abs() @ B.abs()
        err = ((C - (C0 - opA @ B)).abs() / scale).max().item()
        assert err < 1e-14, (N, R, M, t1, err)


def test_exact_update_bit_exact_on_integers(pkg, cuda):
    import torch

    g = torch.Generator(device=cuda).manual_seed(4)
    N, R, M = 384, 1500, 200
    A = _col_major(torch.randint(-3000, 3001, (N, R), device=cuda, generator=g).double())
    B = _col_major(torch.randint(-3000, 3001, (R, M), device=cuda, generator=g).double())
    C = _col_major(torch.randint(-10, 11, (N, M), device=cuda, generator=g).double())
    ref = C + A @ B
    pkg.matmul_mixed_(C, A, B, 1.0, split_terms=7)
    pkg.device_status(C)
    assert torch.equal(C, ref)


@pytest.mark.parametrize("terms", [7, 3])
def test_fused_staging_matches_separate(pkg, cuda, terms, monkeypatch):
    """Updates with K <= 256 stage both operands in one launch
    (stage_pair_kernel).  Its slices and row exponents equal those of the
    separate exponent scan and split; the row bounds differ at most in the
    order of a float sum.  So the updates agree bit for bit on the fast path,
    and on the exact path to the last bit (the fixed point's scale can shift
    when a row bound sits at a power of two).  Both operand layouts, ragged
    sizes, K from one 64-wide tile to 256 (and 1024, staged separately both
    times), a zero row and a zero column."""
    import torch

    g = torch.Generator(device=cuda).manual_seed(17)
    shapes = [(129, 64, 300), (257, 100, 64), (200, 256, 130), (131, 1024, 70)]
    for (N, R, M), t1, t2 in itertools.product(shapes, [False, True], [False, True]):
        A = torch.randn(R if t1 else N, N if t1 else R, device=cuda, generator=g, dtype=torch.float64)
        B = torch.randn(M if t2 else R, R if t2 else M, device=cuda, generator=g, dtype=torch.float64)
        A = _col_major(A)
        B = _col_major(B)
        opA, opB = (A.T if t1 else A), (B.T if t2 else B)
        opA[3].zero_()
        opB[:, 5].zero_()
        C0 = _col_major(torch.randn(N, M, device=cuda, generator=g, dtype=torch.float64))
        out = []
        for fused in ("1", "0"):
            monkeypatch.setenv("NLA_STAGE_FUSED", fused)
            C = C0.clone().T.contiguous().T
            pkg.matmul_mixed_(C, opA, opB, -1.0, split_terms=terms)
            pkg.device_status(C)
            out.append(C)
        if terms == 3:
            assert torch.equal(out[0], out[1]), (N, R, M, t1, t2)
        else:
            scale = (opA.abs() @ opB.abs()).clamp_min(1e-300)
            assert ((out[0] - out[1]).abs() / scale).max().item() < 1e-15, (N, R, M, t1, t2)


def test_exact_short_k_group_table(pkg, cuda, monkeypatch):
    """Updates with K <= 256 use the coupled kernel's short-K table: the pairs
    of one weight share a TMEM accumulator (at most 4 pairs x 256 products
    of at most 2^14 stay exact in FP32).  Integers come out bit for bit;
    random data is FP64-accurate and agrees with the 16-group table to the
    last bit of the fixed point (the tables round the low-weight chunks at
    different points)."""
    import torch

    g = torch.Generator(device=cuda).manual_seed(23)
    for N, R, M in [(200, 256, 130), (130, 64, 300), (129, 100, 129)]:
        A = _col_major(torch.randint(-3000, 3001, (N, R), device=cuda, generator=g).double())
        B = _col_major(torch.randint(-3000, 3001, (R, M), device=cuda, generator=g).double())
        C = _col_major(torch.randint(-10, 11, (N, M), device=cuda, generator=g).double())
        ref = C + A @ B
        pkg.matmul_mixed_(C, A, B, 1.0, split_terms=7)
        pkg.device_status(C)
        assert torch.equal(C, ref), (N, R, M)
    for (N, R, M), t1 in itertools.product([(256, 256, 200), (300, 128, 140), (140, 64, 256)], [False, True]):
        A = torch.randn(R if t1 else N, N if t1 else R, device=cuda, generator=g, dtype=torch.float64)
        A = _col_major(A * torch.exp(torch.randn(A.shape[0], 1, device=cuda, generator=g, dtype=torch.float64)))
        B = _col_major(torch.randn(R, M, device=cuda, generator=g, dtype=torch.float64))
        opA = A.T if t1 else A
        C0 = _col_major(torch.randn(N, M, device=cuda, generator=g, dtype=torch.float64))
        out = []
        for merged in ("1", "0"):
            monkeypatch.setenv("NLA_EXACT_MERGED", merged)
            C = C0.clone().T.contiguous().T
            pkg.matmul_mixed_(C, opA, B, -1.0, split_terms=7)
            pkg.device_status(C)
            out.append(C)
        scale = opA.abs() @ B.abs()
        err = ((out[0] - (C0 - opA @ B)).abs() / scale).max().item()
        assert err < 1e-14, (N, R, M, t1, err)
        assert ((out[0] - out[1]).abs() / scale).max().item() < 1e-15, (N, R, M, t1)


def test_exact_finish_pass_matches_epilogue(pkg, cuda, monkeypatch):
    """Plain exact updates leave their fixed-point sums in the workspace and
    exact_finish_kernel applies them to C; NLA_EXACT_FINISH=0 applies them in
    the exact kernel's epilogue.  Same arithmetic, so the results agree bit
    for bit: ragged shapes, both operand layouts, alpha other than +-1, a
    non-finite row of A and a non-finite column of B (NaN out)."""
    import torch

    g = torch.Generator(device=cuda).manual_seed(29)
    for (N, R, M), t1 in itertools.product([(257, 300, 130), (128, 1500, 77), (64, 64, 1000)], [False, True]):
        A = torch.randn(R if t1 else N, N if t1 else R, device=cuda, generator=g, dtype=torch.float64)
        B = _col_major(torch.randn(R, M, device=cuda, generator=g, dtype=torch.float64))
        A = _col_major(A)
        opA = A.T if t1 else A
        opA[1, 2] = float("inf")
        B[3, 4] = float("nan")
        C0 = _col_major(torch.randn(N, M, device=cuda, generator=g, dtype=torch.float64))
        out = []
        for fin in ("1", "0"):
            monkeypatch.setenv("NLA_EXACT_FINISH", fin)
            C = C0.clone().T.contiguous().T
            pkg.matmul_mixed_(C, opA, B, 0.75, split_terms=7)
            pkg.device_status(C)
            out.append(C)
        assert torch.isnan(out[0][1]).all() and torch.isnan(out[0][:, 4]).all()
        assert torch.equal(out[0].nan_to_num(7.0), out[1].nan_to_num(7.0)), (N, R, M, t1)
