// Throughput of the arithmetic pipes the plain paths run on, measured on the
// current GPU: FP64 fused multiply-add on CUDA cores (DFMA), the FP64 matrix
// instruction mma.sync m8n8k4 (DMMA), and FP32 FMA (FFMA).  Each probe runs
// independent dependency chains on every SM slot for a fixed iteration count
// and is timed with CUDA events; the results are the rooflines of the FP64
// and FP32 diagonal-block and update kernels.
#include "nla_common.cuh"

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


