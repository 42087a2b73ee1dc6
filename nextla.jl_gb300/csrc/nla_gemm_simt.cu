// Dtype-preserving off-diagonal update on CUDA cores:
//   C (N x M) += alpha * op(A) (N x K) * op(B) (K x M)
// Replaces matmul! (src/matmul.jl:5-66).  Float64 runs on the DFMA pipe
// (measured on GB300: DFMA 1.20 TFLOP/s, DMMA m8n8k4 1.05 TFLOP/s, so the
// FP64 "tensor" path is slower than plain DFMA there); Float32 runs on FFMA;
// Float16 accumulates in Float32 (the tensor-core path for Float16 lives in
// nla_umma.cu).
//
// Tiling: 256 threads as 16 x 16; each thread owns a (2V) x (2V) block made
// of two V-wide strips in each direction, so shared-memory reads are V-wide
// vectors and global stores of a column are 16V contiguous elements.
// Tiles are double-buffered in shared memory with a register prefetch of the
// next K slab.  Operand loads are layout-aware: threads run along whichever
// index is contiguous in memory for op(A) = A or A^T.
#include "nla_common.cuh"

namespace nla {
namespace {

template <typename Tc, int V> struct Vec;
template <> struct Vec<float, 4> {
  using type = float4;
  __device__ static void unpack(const float4& v, float* o) { o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w; }
};
template <> struct Vec<double, 2> {
  using type = double2;
  __device__ static void unpack(const double2& v, double* o) { o[0] = v.x; o[1] = v.y; }
};

template <typename T, int V, int BK>
__global__ void __launch_bounds__(256) gemm_simt_kernel(int64_t N, int64_t M, int64_t K, double alpha,
                                                        const T* __restrict__ A, int64_t lda, int tA,
                                                        const T* __restrict__ B, int64_t ldb, int tB, T* C,
                                                        int64_t ldc) {
  using Tc = typename Elem<T>::compute;
  constexpr int BM = 32 * V;  // = BN
  constexpr int BN = 32 * V;
  constexpr int LA = BM * BK / 256;
  constexpr int LB = BK * BN / 256;
  __shared__ __align__(16) Tc As[2][BK][BM];
  __shared__ __align__(16) Tc Bs[2][BK][BN];

  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int64_t row0 = (int64_t)blockIdx.x * BM;
  const int64_t col0 = (int64_t)blockIdx.y * BN;

  Tc ra[LA], rb[LB];
  auto load_tiles = [&](int64_t k0) {
#pragma unroll
    for (int e = 0; e < LA; ++e) {
      int l = tid + 256 * e;
      int i, k;
      if (!tA) { i = l % BM; k = l / BM; } else { k = l % BK; i = l / BK; }
      int64_t gi = row0 + i, gk = k0 + k;
      ra[e] = (gi < N && gk < K) ? Elem<T>::load(A + mat_off(gi, gk, lda, tA)) : Tc(0);
    }
#pragma unroll
    for (int e = 0; e < LB; ++e) {
      int l = tid + 256 * e;
      int k, j;
      if (!tB) { k = l % BK; j = l / BK; } else { j = l % BN; k = l / BN; }
      int64_t gk = k0 + k, gj = col0 + j;
      rb[e] = (gk < K && gj < M) ? Elem<T>::load(B + mat_off(gk, gj, ldb, tB)) : Tc(0);
    }
  };
  auto store_tiles = [&](int buf) {
#pragma unroll
    for (int e = 0; e < LA; ++e) {
      int l = tid + 256 * e;
      int i, k;
      if (!tA) { i = l % BM; k = l / BM; } else { k = l % BK; i = l / BK; }
      As[buf][k][i] = ra[e];
    }
#pragma unroll
    for (int e = 0; e < LB; ++e) {
      int l = tid + 256 * e;
      int k, j;
      if (!tB) { k = l % BK; j = l / BK; } else { j = l % BN; k = l / BN; }
      Bs[buf][k][j] = rb[e];
    }
  };

  Tc acc[2 * V][2 * V];
#pragma unroll
  for (int r = 0; r < 2 * V; ++r)
#pragma unroll
    for (int c = 0; c < 2 * V; ++c) acc[r][c] = Tc(0);

  const int64_t nk = (K + BK - 1) / BK;
  if (nk > 0) {
    load_tiles(0);
    store_tiles(0);
  }
  __syncthreads();
  for (int64_t kt = 0; kt < nk; ++kt) {
    const int cur = (int)(kt & 1);
    if (kt + 1 < nk) load_tiles((kt + 1) * BK);
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      Tc a[2 * V], b[2 * V];
      using VT = typename Vec<Tc, V>::type;
      Vec<Tc, V>::unpack(*reinterpret_cast<const VT*>(&As[cur][k][V * tx]), a);
      Vec<Tc, V>::unpack(*reinterpret_cast<const VT*>(&As[cur][k][16 * V + V * tx]), a + V);
      Vec<Tc, V>::unpack(*reinterpret_cast<const VT*>(&Bs[cur][k][V * ty]), b);
      Vec<Tc, V>::unpack(*reinterpret_cast<const VT*>(&Bs[cur][k][16 * V + V * ty]), b + V);
#pragma unroll
      for (int r = 0; r < 2 * V; ++r)
#pragma unroll
        for (int c = 0; c < 2 * V; ++c) acc[r][c] = fma(a[r], b[c], acc[r][c]);
    }
    if (kt + 1 < nk) store_tiles(cur ^ 1);
    __syncthreads();
  }

  const Tc al = (Tc)alpha;
#pragma unroll
  for (int c = 0; c < 2 * V; ++c) {
    int64_t j = col0 + (c < V ? V * ty + c : 16 * V + V * ty + (c - V));
    if (j >= M) continue;
#pragma unroll
    for (int r = 0; r < 2 * V; ++r) {
      int64_t i = row0 + (r < V ? V * tx + r : 16 * V + V * tx + (r - V));
      if (i >= N) continue;
      T* p = C + i + j * ldc;
      Elem<T>::store(p, fma(al, acc[r][c], Elem<T>::load(p)));
    }
  }
}

template <typename T, int V, int BK>
int launch_simt(int64_t N, int64_t M, int64_t K, double alpha, const Mat& A, const Mat& B, const Mat& C,
                cudaStream_t s) {
  constexpr int BM = 32 * V;
  int64_t gx = (N + BM - 1) / BM, gy = (M + BM - 1) / BM;
  if (gx > 2147483647LL || gy > 65535) return fail(NLA_ERR_UNSUPPORTED, "gemm: matrix too large for one launch");
  TraceScope trace(NLA_K_GEMM_SIMT, s, 2.0 * (double)N * (double)M * (double)K,
                   (double)sizeof(T) * ((double)N * K + (double)K * M + 2.0 * (double)N * M));
  gemm_simt_kernel<T, V, BK><<<dim3((unsigned)gx, (unsigned)gy), 256, 0, s>>>(
      N, M, K, alpha, static_cast<const T*>(A.p), A.ld, A.t, static_cast<const T*>(B.p), B.ld, B.t,
      static_cast<T*>(C.p), C.ld);
  NLA_CHECK_LAUNCH("gemm_simt_kernel");
  return NLA_OK;
}

}  // namespace

int launch_gemm_simt(int dtype, int64_t N, int64_t M, int64_t K, double alpha, const Mat& A, const Mat& B,
                     const Mat& C, cudaStream_t s) {
  if (N <= 0 || M <= 0) return NLA_OK;
  if (C.t) return fail(NLA_ERR_UNSUPPORTED, "gemm: transposed output view");
  switch (dtype) {
    case NLA_F64: return launch_simt<double, 2, 16>(N, M, K, alpha, A, B, C, s);
    case NLA_F32: return launch_simt<float, 4, 8>(N, M, K, alpha, A, B, C, s);
    case NLA_F16: return launch_simt<__half, 4, 8>(N, M, K, alpha, A, B, C, s);
    default: return fail(NLA_ERR_DTYPE, "gemm: unknown dtype");
  }
}

}  // namespace nla
