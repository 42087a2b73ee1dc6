// The mixed-precision off-diagonal update without any device allocation.
//
// nla_gemm_update_mixed stages its operands (BF16/FP16 slices, exponents and
// row bounds) in a workspace drawn from a stream-ordered pool, which may call
// cudaMallocAsync.  Some callers cannot let a library allocate: a host
// framework that owns all device memory through its own allocator, a process
// held to a fixed device-memory budget, or a latency-critical loop that cannot
// absorb an allocation.  nla_gemm_update_mixed_noalloc does the same update
// with its staging in one statically sized device array that the library
// defines, so it never allocates.
//
// The array is a file-scope __device__ object: every GPU that loads the
// library holds it (NLA_NOALLOC_SCRATCH_BYTES) until the process exits.  Host
// code cannot use the array's name as a device address, so the first call on
// each device looks the address up with cudaGetSymbolAddress (with that
// device current) and caches it.  All calls share the array and it keeps the
// previous call's contents: the staging kernels write every byte they read
// (exponents and bounds are cleared with cudaMemsetAsync first), and calls
// whose executions overlap on the GPU (different streams, or different host
// threads without ordering) race on it.  The cached address belongs to the
// device's context at the first call: resetting the device (cudaDeviceReset)
// after that is not supported, as for the library's other per-device state
// (the copy streams of the host-buffer entry points).
#include <mutex>

#include "nla_common.cuh"

namespace nla {
namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[NLA_NOALLOC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_scratch_mu;
void* g_scratch_ptr[MAX_DEVICES] = {};

// Device address of the scratch array on the current device (set up once per
// device, with that device current).
int scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  if (dev < 0 || dev >= MAX_DEVICES) return fail(NLA_ERR_UNSUPPORTED, "device index out of range");
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(scratch)");
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return NLA_OK;
}

}  // namespace
}  // namespace nla

using namespace nla;

extern "C" int nla_gemm_update_mixed_noalloc(int trans1, int trans2, int64_t N, int64_t R, int64_t M, double alpha,
                                             const double* in1, int64_t ld1, const double* in2, int64_t ld2,
                                             double* out, int64_t ldo, int lowp, int split_terms, void* stream) {
  clear_error();
  if (N < 0 || R < 0 || M < 0) return fail(NLA_ERR_ARG, "N, R and M must be non-negative");
  if (lowp != NLA_LOWP_BF16 && lowp != NLA_LOWP_F16) return fail(NLA_ERR_ARG, "lowp must be BF16 or F16");
  if (!(split_terms >= 1 && split_terms <= 3) && split_terms != EXACT_SLICES)
    return fail(NLA_ERR_ARG, "split_terms must be 1, 2, 3 or 7");
  NLA_TRY(check_matrix("in1", in1, trans1 ? R : N, trans1 ? N : R, ld1));
  NLA_TRY(check_matrix("in2", in2, trans2 ? M : R, trans2 ? R : M, ld2));
  NLA_TRY(check_matrix("out", out, N, M, ldo));
  if (N == 0 || M == 0 || R == 0) return NLA_OK;
  const size_t need = sliced_workspace_bytes(N, M, R, split_terms);
  if (need > (size_t)NLA_NOALLOC_SCRATCH_BYTES)
    return fail(NLA_ERR_WORKSPACE, "update needs " + std::to_string(need) + " bytes of staging; the static scratch holds " +
                                       std::to_string((size_t)NLA_NOALLOC_SCRATCH_BYTES));
  void* scratch = nullptr;
  NLA_TRY(scratch_address(&scratch));
  Mat A{const_cast<double*>(in1), ld1, trans1 ? 1 : 0};
  Mat B{const_cast<double*>(in2), ld2, trans2 ? 1 : 0};
  Mat C{out, ldo, 0};
  return launch_sliced_gemm(N, M, R, alpha, A, B, C, NLA_F64, NLA_F64, split_terms, lowp == NLA_LOWP_BF16, scratch,
                            (size_t)NLA_NOALLOC_SCRATCH_BYTES, (cudaStream_t)stream);
}
