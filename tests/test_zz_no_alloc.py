"""nla_gemm_update_mixed_noalloc: the mixed-precision update for callers that
cannot let a library allocate device memory (a framework that owns all
device memory, a fixed memory budget, a latency-critical loop).

It stages its operands in a static device array of the library instead of
the pooled workspace.  Checked through the C ABI against the allocating entry
point nla_gemm_update_mixed on two calls in a row (same kernels, so the
results must agree to the suite's Float64 tolerance, relative error 1e-14),
that a request larger than the array is refused, and that repeated calls leave
the device's free memory unchanged.  This file is collected last so that a
run stopping at its first failure has already run every other test; it also
passes alone in a fresh process.
"""

import ctypes

import pytest

pytestmark = pytest.mark.gpu


def _col_major(t):
    return t.T.contiguous().T


def _call(lib, fn_name, C, A, B, alpha, lowp, terms):
    import torch

    fn = getattr(lib, fn_name)
    N, R = A.shape
    M = B.shape[1]
    stream = torch.cuda.current_stream().cuda_stream
    return fn(0, 0, N, R, M, ctypes.c_double(alpha), A.data_ptr(), A.stride(1), B.data_ptr(), B.stride(1),
              C.data_ptr(), C.stride(1), lowp, terms, ctypes.c_void_p(stream))


@pytest.mark.parametrize("lowp,terms", [(0, 3), (1, 2), (0, 7)])
def test_noalloc_matches_allocating_update(lib, cuda, lowp, terms):
    import torch

    g = torch.Generator(device=cuda).manual_seed(7 + terms)
    # Calls in a row with different shapes; the last has R <= 256, which
    # stages both operands in one fused kernel that writes every byte it reads
    # from the array, right after a larger call has left its contents there.
    for (N, R, M) in [(300, 257, 129), (640, 512, 384), (300, 200, 129)]:
        A = _col_major(torch.randn(N, R, generator=g, device=cuda, dtype=torch.float64))
        B = _col_major(torch.randn(R, M, generator=g, device=cuda, dtype=torch.float64))
        C0 = _col_major(torch.randn(N, M, generator=g, device=cuda, dtype=torch.float64))
        C_ref, C_new = C0.clone().T.contiguous().T, C0.clone().T.contiguous().T
        assert _call(lib, "nla_gemm_update_mixed", C_ref, A, B, -1.0, lowp, terms) == 0
        assert _call(lib, "nla_gemm_update_mixed_noalloc", C_new, A, B, -1.0, lowp, terms) == 0
        assert lib.nla_device_status(None) == 0
        rel = float(torch.linalg.norm(C_new - C_ref) / torch.linalg.norm(C_ref))
        assert rel <= 1e-14, (N, R, M, rel)


def test_noalloc_refuses_oversized_and_allocates_nothing(lib, cuda):
    import torch

    g = torch.Generator(device=cuda).manual_seed(3)
    # 2048 x 4096 x 2048 with 3 slices needs more staging than the static array holds.
    A = _col_major(torch.randn(2048, 4096, generator=g, device=cuda, dtype=torch.float64))
    B = _col_major(torch.randn(4096, 2048, generator=g, device=cuda, dtype=torch.float64))
    C = _col_major(torch.zeros(2048, 2048, device=cuda, dtype=torch.float64))
    assert _call(lib, "nla_gemm_update_mixed_noalloc", C, A, B, 1.0, 0, 3) == -4  # NLA_ERR_WORKSPACE
    assert b"static scratch" in lib.nla_last_error()
    assert float(C.abs().max()) == 0.0  # nothing was written

    A = _col_major(torch.randn(512, 512, generator=g, device=cuda, dtype=torch.float64))
    B = _col_major(torch.randn(512, 512, generator=g, device=cuda, dtype=torch.float64))
    C = _col_major(torch.zeros(512, 512, device=cuda, dtype=torch.float64))
    assert _call(lib, "nla_gemm_update_mixed_noalloc", C, A, B, 1.0, 0, 3) == 0  # first call sets up
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _call(lib, "nla_gemm_update_mixed_noalloc", C, A, B, 1.0, 0, 3) == 0
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
    assert lib.nla_device_status(None) == 0
