// Throughput of the arithmetic pipes the plain paths run on, measured on the
// current GPU: FP64 fused multiply-add on CUDA cores (DFMA), the FP64 matrix
// instruction mma.sync m8n8k4 (DMMA), and FP32 FMA (FFMA).  Each probe runs
// independent dependency chains on every SM slot for a fixed iteration count
// and is timed with CUDA events; the results are the rooflines of the FP64
// and FP32 diagonal-block and update kernels.
#include <cudaTypedefs.h>

#include "nla_common.cuh"
#include "nla_umma.cuh"

namespace nla {
namespace {

constexpr int PROBE_THREADS = 256;

__global__ void __launch_bounds__(PROBE_THREADS) dfma_probe(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void __launch_bounds__(PROBE_THREADS) ffma_probe(float* out, int iters, float a, float b) {
  float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
    x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void __launch_bounds__(PROBE_THREADS) dmma_probe(double* out, int iters) {
  const double a = 1.0 + threadIdx.x * 1e-3, b = 1.0 - threadIdx.x * 1e-3;
  double c[4][2] = {};
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                   : "+d"(c[j][0]), "+d"(c[j][1])
                   : "d"(a), "d"(b));
  }
  double s = 0;
  for (int j = 0; j < 4; ++j) s += c[j][0] + c[j][1];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// ---------------------------------------------------------------------------
// Tensor-core feed probes (nla_measure_tensor_feed): what the tcgen05 MMAs
// and the TMA loads that feed them sustain per SM, separately and together.
// One CTA per SM, operands from a 4 MiB (L2-resident) buffer of zeros.
// ---------------------------------------------------------------------------
__device__ int g_probe_error = 0;
constexpr int FEED_BOX = 16384;  // one 128-row x 128-byte box (64 BF16 of K)

// MMAs only: 128 x 128 x 16 BF16 MMAs from one A and one B tile resident in
// shared memory, issued back to back by one thread.
__global__ void __launch_bounds__(128, 1) feed_mma_kernel(int iters) {
  extern __shared__ __align__(1024) unsigned char sm_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)sm_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* bar = (uint64_t*)(base + 2 * FEED_BOX);
  uint32_t* slot = (uint32_t*)(bar + 1);
  __shared__ volatile int s_abort;
  for (int i = threadIdx.x; i < 2 * FEED_BOX / 4; i += blockDim.x) ((uint32_t*)base)[i] = 0;
  if (threadIdx.x == 0) {
    s_abort = 0;
    umma::mbar_init(umma::smem_u32(bar), 1);
    umma::fence_barrier_init();
  }
  const int warp = threadIdx.x >> 5;
  if (warp == 1) umma::tmem_alloc(umma::smem_u32(slot), 128);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *slot;
  if (threadIdx.x == 32) {
    const uint32_t idesc = umma::idesc_f16(128, 128, true);
    const uint32_t a0 = umma::smem_u32(base), b0 = a0 + FEED_BOX;
    for (int it = 0; it < iters; ++it)
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)
        umma::mma_f16(tmem, umma::desc_kmajor_sw128(a0 + kk * 32), umma::desc_kmajor_sw128(b0 + kk * 32), idesc,
                      (it > 0 || kk > 0) ? 1u : 0u);
    umma::mma_commit(umma::smem_u32(bar));
    umma::mbar_wait(umma::smem_u32(bar), 0, &s_abort, &g_probe_error, 1, false);
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    umma::fence_after_sync();
    umma::tmem_dealloc(tmem, 128);
  }
}

// TMA loads into a ring of FEED_STAGES stages of two boxes, refilled as soon
// as a stage lands (WITH_MMA = false), or released by four MMAs on the stage
// (WITH_MMA = true, the exact kernels' main loop without their epilogue).
// With PRODUCERS = 2 the A and the B box of a stage are issued by two warps.
constexpr int FEED_STAGES = 6;
template <int PRODUCERS, bool WITH_MMA>
__global__ void __launch_bounds__(128, 1) feed_pipe_kernel(const __grid_constant__ CUtensorMap map, int iters,
                                                            int rows_total) {
  extern __shared__ __align__(1024) unsigned char sm_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)sm_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(base + FEED_STAGES * 2 * FEED_BOX);
  uint64_t* empty = full + FEED_STAGES;
  uint64_t* drain = empty + FEED_STAGES;
  uint32_t* slot = (uint32_t*)(drain + 1);
  __shared__ volatile int s_abort;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int s = 0; s < FEED_STAGES; ++s) {
      umma::mbar_init(umma::smem_u32(&full[s]), PRODUCERS);
      umma::mbar_init(umma::smem_u32(&empty[s]), 1);
    }
    umma::mbar_init(umma::smem_u32(drain), 1);
    umma::fence_barrier_init();
  }
  if (WITH_MMA && warp == 1) umma::tmem_alloc(umma::smem_u32(slot), 256);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = WITH_MMA ? *slot : 0u;
  const bool producer = warp == 0 || (PRODUCERS == 2 && warp == 2);
  if (producer && lane == 0) {
    for (int it = 0; it < iters; ++it) {
      const int s = it % FEED_STAGES;
      const uint32_t round = (uint32_t)(it / FEED_STAGES);
      if (WITH_MMA) {
        if (!umma::mbar_wait(umma::smem_u32(&empty[s]), (round & 1u) ^ 1u, &s_abort, &g_probe_error, 2)) break;
      } else if (it >= FEED_STAGES) {
        if (!umma::mbar_wait(umma::smem_u32(&full[s]), (round - 1) & 1u, &s_abort, &g_probe_error, 3)) break;
      }
      const uint32_t fb = umma::smem_u32(&full[s]);
      const int y = ((blockIdx.x * 5 + it * 2) * 128) % rows_total;
      unsigned char* st = base + s * 2 * FEED_BOX;
      if (PRODUCERS == 1) {
        umma::mbar_arrive_expect_tx(fb, 2 * FEED_BOX);
        umma::tma_load_2d(umma::smem_u32(st), &map, fb, 0, y);
        umma::tma_load_2d(umma::smem_u32(st + FEED_BOX), &map, fb, 0, (y + 128) % rows_total);
      } else {
        umma::mbar_arrive_expect_tx(fb, FEED_BOX);
        const int half = warp == 0 ? 0 : 1;
        umma::tma_load_2d(umma::smem_u32(st + half * FEED_BOX), &map, fb, 0, (y + half * 128) % rows_total);
      }
    }
    if (!WITH_MMA) {
      // Wait for the last loads of every stage before the CTA exits.
      for (int s = 0; s < FEED_STAGES && s < iters; ++s) {
        const int last = s + ((iters - 1 - s) / FEED_STAGES) * FEED_STAGES;
        if (!umma::mbar_wait(umma::smem_u32(&full[s]), (uint32_t)(last / FEED_STAGES) & 1u, &s_abort,
                             &g_probe_error, 4))
          break;
      }
    }
  } else if (WITH_MMA && warp == 1 && lane == 0) {
    const uint32_t idesc = umma::idesc_f16(128, 128, true);
    for (int it = 0; it < iters; ++it) {
      const int s = it % FEED_STAGES;
      if (!umma::mbar_wait(umma::smem_u32(&full[s]), (uint32_t)(it / FEED_STAGES) & 1u, &s_abort, &g_probe_error, 5))
        break;
      umma::fence_after_sync();
      const uint32_t a0 = umma::smem_u32(base + s * 2 * FEED_BOX), b0 = a0 + FEED_BOX;
      const uint32_t d = tmem + (uint32_t)(((it >> 4) & 1) * 128);
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)
        umma::mma_f16(d, umma::desc_kmajor_sw128(a0 + kk * 32), umma::desc_kmajor_sw128(b0 + kk * 32), idesc,
                      ((it & 15) > 0 || kk > 0) ? 1u : 0u);
      umma::mma_commit(umma::smem_u32(&empty[s]));
    }
    umma::mma_commit(umma::smem_u32(drain));
    umma::mbar_wait(umma::smem_u32(drain), 0, &s_abort, &g_probe_error, 6, false);
  }
  umma::fence_before_sync();
  __syncthreads();
  if (WITH_MMA && warp == 1) {
    umma::fence_after_sync();
    umma::tmem_dealloc(tmem, 256);
  }
}

}  // namespace
}  // namespace nla

using namespace nla;

extern "C" int nla_measure_pipes(double* dfma_tflops, double* dmma_tflops, double* ffma_tflops, void* stream) {
  clear_error();
  cudaStream_t s = (cudaStream_t)stream;
  const int blocks = num_sms() * 8;
  double* buf = nullptr;
  cudaError_t e = cudaMallocAsync(&buf, sizeof(double) * blocks * PROBE_THREADS, s);
  if (e != cudaSuccess) return cuda_status(e, "probe buffer");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto time_it = [&](auto launch, double flops, double* out) -> int {
    launch();  // warm-up
    cudaEventRecord(e0, s);
    launch();
    cudaEventRecord(e1, s);
    cudaError_t r = cudaEventSynchronize(e1);
    if (r != cudaSuccess) return cuda_status(r, "probe");
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (out) *out = flops / (ms * 1e-3) / 1e12;
    return NLA_OK;
  };
  const double threads = (double)blocks * PROBE_THREADS;
  int rc = time_it([&] { dfma_probe<<<blocks, PROBE_THREADS, 0, s>>>(buf, 4096, 0.999, 1e-3); },
                   2.0 * 8 * 4096 * threads, dfma_tflops);
  if (rc == NLA_OK)
    rc = time_it([&] { dmma_probe<<<blocks, PROBE_THREADS, 0, s>>>(buf, 1024); },
                 512.0 * 4 * 1024 * (threads / 32), dmma_tflops);
  if (rc == NLA_OK)
    rc = time_it([&] { ffma_probe<<<blocks, PROBE_THREADS, 0, s>>>(reinterpret_cast<float*>(buf), 65536, 0.999f,
                                                                     1e-3f); },
                 2.0 * 8 * 65536 * threads, ffma_tflops);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(buf, s);
  if (rc == NLA_OK) {
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e, "probe kernels");
  }
  return rc;
}

extern "C" int nla_measure_tensor_feed(double* mma_tflops, double* tma_gbs_1, double* tma_gbs_2,
                                       double* pipe_tflops_1, double* pipe_tflops_2, void* stream) {
  clear_error();
  cudaStream_t s = (cudaStream_t)stream;
  const int sms = num_sms();
  PFN_cuTensorMapEncodeTiled_v12000 enc = nullptr;
  {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return fail(NLA_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available from the driver");
    enc = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  const int rows = 128 * 256;  // 32768 rows of 128 bytes: 4 MiB
  void* buf = nullptr;
  cudaError_t e = cudaMallocAsync(&buf, (size_t)rows * 128, s);
  if (e != cudaSuccess) return cuda_status(e, "feed probe buffer");
  cudaMemsetAsync(buf, 0, (size_t)rows * 128, s);
  CUtensorMap map;
  cuuint64_t dims[2] = {64, (cuuint64_t)rows};
  cuuint64_t strides[1] = {128};
  cuuint32_t box[2] = {64, 128};
  cuuint32_t es[2] = {1, 1};
  if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, buf, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
          CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
      CUDA_SUCCESS) {
    cudaFreeAsync(buf, s);
    return fail(NLA_ERR_UNSUPPORTED, "feed probe tensor map");
  }
  const int mma_smem = 1024 + 2 * FEED_BOX + 64;
  const int pipe_smem = 1024 + FEED_STAGES * 2 * FEED_BOX + 256;
  cudaFuncSetAttribute(feed_mma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, mma_smem);
  cudaFuncSetAttribute(feed_pipe_kernel<1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, pipe_smem);
  cudaFuncSetAttribute(feed_pipe_kernel<2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, pipe_smem);
  cudaFuncSetAttribute(feed_pipe_kernel<1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, pipe_smem);
  cudaFuncSetAttribute(feed_pipe_kernel<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, pipe_smem);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int rc = NLA_OK;
  auto time_it = [&](auto launch, double work, double* out) {
    if (rc != NLA_OK) return;
    launch();  // warm-up
    cudaEventRecord(e0, s);
    launch();
    cudaEventRecord(e1, s);
    cudaError_t r = cudaEventSynchronize(e1);
    if (r == cudaSuccess) r = cudaGetLastError();
    if (r != cudaSuccess) {
      rc = cuda_status(r, "feed probe");
      return;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (out) *out = work / (ms * 1e-3);
  };
  const int iters = 4096;
  const double mma_flops = 2.0 * 128 * 128 * 64 * (double)iters * sms;  // per stage: 4 MMAs of K = 16
  const double bytes_per_sm = 2.0 * FEED_BOX * iters;
  time_it([&] { feed_mma_kernel<<<sms, 128, mma_smem, s>>>(iters); }, mma_flops / 1e12, mma_tflops);
  time_it([&] { feed_pipe_kernel<1, false><<<sms, 128, pipe_smem, s>>>(map, iters, rows); }, bytes_per_sm / 1e9,
          tma_gbs_1);
  time_it([&] { feed_pipe_kernel<2, false><<<sms, 128, pipe_smem, s>>>(map, iters, rows); }, bytes_per_sm / 1e9,
          tma_gbs_2);
  time_it([&] { feed_pipe_kernel<1, true><<<sms, 128, pipe_smem, s>>>(map, iters, rows); }, mma_flops / 1e12,
          pipe_tflops_1);
  time_it([&] { feed_pipe_kernel<2, true><<<sms, 128, pipe_smem, s>>>(map, iters, rows); }, mma_flops / 1e12,
          pipe_tflops_2);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(buf, s);
  int derr = 0;
  cudaMemcpyFromSymbol(&derr, g_probe_error, sizeof(int));
  if (rc == NLA_OK && derr != 0) {
    const int zero = 0;
    cudaMemcpyToSymbol(g_probe_error, &zero, sizeof(int));
    return fail(NLA_ERR_TIMEOUT, "feed probe: a bounded wait gave up");
  }
  return rc;
}

