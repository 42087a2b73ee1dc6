// Complex element types (ComplexF32, ComplexF64) for the plain path: the
// diagonal-block solve and multiply, the off-diagonal update and the alpha
// scaling that the recursion of unified_rec (src/rectrxm.jl:101-198) calls.
//
// The reference's unified_rec is restricted to real element types
// (src/rectrxm.jl:101), though its base-case docstrings list complex ones
// (src/trsm.jl:180-183).  These kernels run the same recursion on complex
// data: trans 'T' reads A transposed, 'C' reads its conjugate transpose (the
// Adjoint wrapper), and the arithmetic is ordinary complex arithmetic, every
// product formed with fused multiply-adds of the real parts and every
// quotient with Smith's algorithm (R. L. Smith, "Algorithm 116: Complex
// division", CACM 5(8), 1962).
//
// Values are interleaved (re, im) pairs, column-major, as Julia and torch
// store them.  All kernels work on the canonical lower-left problem of the
// real diagonal-block kernels: side 'R' becomes side 'L' on transposed
// views, uplo 'U' becomes lower by reversing the block's index order.
#include <mutex>

#include "nla_common.cuh"

namespace nla {
namespace cx {

template <typename R>
struct alignas(2 * sizeof(R)) cpx {
  R re, im;
};

template <typename R> __device__ __forceinline__ cpx<R> mk(R a, R b) { return cpx<R>{a, b}; }
template <typename R> __device__ __forceinline__ cpx<R> zero() { return cpx<R>{R(0), R(0)}; }
template <typename R> __device__ __forceinline__ cpx<R> conj_if(cpx<R> a, bool c) { return c ? mk(a.re, -a.im) : a; }
// c + a b
template <typename R> __device__ __forceinline__ cpx<R> fma_c(cpx<R> a, cpx<R> b, cpx<R> c) {
  return mk(fma(a.re, b.re, fma(-a.im, b.im, c.re)), fma(a.re, b.im, fma(a.im, b.re, c.im)));
}
// c - a b
template <typename R> __device__ __forceinline__ cpx<R> fms_c(cpx<R> a, cpx<R> b, cpx<R> c) {
  return mk(fma(-a.re, b.re, fma(a.im, b.im, c.re)), fma(-a.re, b.im, fma(-a.im, b.re, c.im)));
}
// a / b, Smith's algorithm.
template <typename R> __device__ __forceinline__ cpx<R> div(cpx<R> a, cpx<R> b) {
  if (fabs(b.re) >= fabs(b.im)) {
    const R t = b.im / b.re, den = b.re + b.im * t;
    return mk((a.re + a.im * t) / den, (a.im - a.re * t) / den);
  }
  const R t = b.re / b.im, den = b.im + b.re * t;
  return mk((a.re * t + a.im) / den, (a.im * t - a.re) / den);
}

// Canonical-coordinate views (see the file comment): element (i, k) of the
// canonical lower triangle and (i, c) of the right-hand sides.
struct View {
  const void* A;
  int64_t lda;
  int tA, conj, rev, unit;
  void* B;
  int64_t ldb;
  int tB;
  int n;
  int64_t m;
};

template <typename R>
__device__ __forceinline__ cpx<R> a_get(const View& v, int i, int k) {
  const int r = v.rev ? v.n - 1 - i : i, c = v.rev ? v.n - 1 - k : k;
  const cpx<R>* A = static_cast<const cpx<R>*>(v.A);
  return conj_if(A[mat_off(r, c, v.lda, v.tA)], v.conj != 0);
}
template <typename R>
__device__ __forceinline__ cpx<R>* b_ptr(const View& v, int i, int64_t col) {
  const int r = v.rev ? v.n - 1 - i : i;
  return static_cast<cpx<R>*>(v.B) + mat_off(r, col, v.ldb, v.tB);
}

constexpr int LEAF_COLS = 64;   // right-hand sides per CTA, one per thread
constexpr int LEAF_PANEL = 32;  // rows of the triangle staged at a time

// Diagonal-block solve X := L^{-1} X (func 'S') or multiply X := L X ('M')
// for LEAF_COLS right-hand sides per CTA, one per thread.  The CTA's block of
// X lives in shared memory (column per thread: conflict-free); the rows of L
// are staged LEAF_PANEL at a time and read as broadcasts.
// Solve: x_r = (b_r - sum_{k<r} l_rk x_k) / l_rr, rows in increasing order.
// Multiply: x_r = sum_{k<=r} l_rk b_k with k increasing (the reference's
// order, src/trmm.jl:90-94), rows from the last so that each b_k is still
// the old value when read.
template <typename R, bool SOLVE>
__global__ void __launch_bounds__(LEAF_COLS) cplx_leaf_kernel(View v) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cpx<R>* X = reinterpret_cast<cpx<R>*>(smem_raw);  // n x LEAF_COLS
  cpx<R>* Lp = X + (size_t)v.n * LEAF_COLS;          // LEAF_PANEL x n
  const int t = threadIdx.x, n = v.n;
  const int64_t col = (int64_t)blockIdx.x * LEAF_COLS + t;
  const bool live = col < v.m;
  for (int r = 0; r < n; ++r) X[r * LEAF_COLS + t] = live ? *b_ptr<R>(v, r, col) : zero<R>();
  const int npanels = (n + LEAF_PANEL - 1) / LEAF_PANEL;
  for (int pi = 0; pi < npanels; ++pi) {
    const int p = SOLVE ? pi : npanels - 1 - pi;
    const int p0 = p * LEAF_PANEL, pw = min(LEAF_PANEL, n - p0);
    __syncthreads();
    // Rows p0 .. p0 + pw of L, columns 0 .. p0 + pw (k <= r; the diagonal
    // is taken as 1 for a unit-diagonal view).
    for (int idx = t; idx < pw * (p0 + pw); idx += LEAF_COLS) {
      const int i = idx / (p0 + pw), k = idx % (p0 + pw);
      const int r = p0 + i;
      cpx<R> val = zero<R>();
      if (k < r) val = a_get<R>(v, r, k);
      else if (k == r) val = v.unit ? mk(R(1), R(0)) : a_get<R>(v, r, k);
      Lp[i * n + k] = val;
    }
    __syncthreads();
    for (int ii = 0; ii < pw; ++ii) {
      const int i = SOLVE ? ii : pw - 1 - ii;
      const int r = p0 + i;
      const cpx<R>* l = Lp + i * n;
      if (SOLVE) {
        cpx<R> x = X[r * LEAF_COLS + t];
        for (int k = 0; k < r; ++k) x = fms_c(l[k], X[k * LEAF_COLS + t], x);
        X[r * LEAF_COLS + t] = div(x, l[r]);
      } else {
        cpx<R> x = zero<R>();
        for (int k = 0; k <= r; ++k) x = fma_c(l[k], X[k * LEAF_COLS + t], x);
        X[r * LEAF_COLS + t] = x;
      }
    }
  }
  if (live)
    for (int r = 0; r < n; ++r) *b_ptr<R>(v, r, col) = X[r * LEAF_COLS + t];
}

// C (N x M) += alpha * op(A) (N x K) * op(B) (K x M), alpha real (+-1 in
// the recursion).  64 x 64 tiles, 256 threads, each a 4 x 4 register tile;
// K in chunks of 16 staged in shared memory; conjugation applied as the
// operands are staged.
constexpr int GT = 64, GK = 16;
template <typename R>
__global__ void __launch_bounds__(256) cplx_gemm_kernel(int64_t N, int64_t M, int64_t K, R alpha, const cpx<R>* A,
                                                        int64_t lda, int tA, int cA, const cpx<R>* B, int64_t ldb,
                                                        int tB, int cB, cpx<R>* C, int64_t ldc) {
  __shared__ cpx<R> As[GK][GT + 1], Bs[GK][GT + 1];
  const int t = threadIdx.x, tr = t % 16, tc = t / 16;
  const int64_t i0 = (int64_t)blockIdx.x * GT, j0 = (int64_t)blockIdx.y * GT;
  cpx<R> acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = zero<R>();
  for (int64_t k0 = 0; k0 < K; k0 += GK) {
    for (int idx = t; idx < GK * GT; idx += 256) {
      // op(A)(i, k): threads along i for a plain view, along k for a transposed one.
      int i, k;
      if (!tA) { i = idx % GT; k = idx / GT; }
      else { k = idx % GK; i = idx / GK; }
      const int64_t gi = i0 + i, gk = k0 + k;
      As[k][i] = gi < N && gk < K ? conj_if(A[mat_off(gi, gk, lda, tA)], cA != 0) : zero<R>();
      int j, kb;
      if (!tB) { kb = idx % GK; j = idx / GK; }
      else { j = idx % GT; kb = idx / GT; }
      const int64_t gj = j0 + j, gkb = k0 + kb;
      Bs[kb][j] = gj < M && gkb < K ? conj_if(B[mat_off(gkb, gj, ldb, tB)], cB != 0) : zero<R>();
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < GK; ++k) {
      cpx<R> av[4], bv[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) av[a] = As[k][tr + 16 * a];
#pragma unroll
      for (int b = 0; b < 4; ++b) bv[b] = Bs[k][tc + 16 * b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = fma_c(av[a], bv[b], acc[a][b]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int64_t i = i0 + tr + 16 * a;
    if (i >= N) continue;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int64_t j = j0 + tc + 16 * b;
      if (j >= M) continue;
      cpx<R>* p = C + i + j * ldc;
      const cpx<R> c = *p;
      *p = mk(fma(alpha, acc[a][b].re, c.re), fma(alpha, acc[a][b].im, c.im));
    }
  }
}

// B .= alpha .* B with the product formed in ComplexF64 and rounded to the
// element type (src/rectrxm.jl:64, :72).
template <typename R>
__global__ void cplx_scale_kernel(int64_t rows, int64_t cols, double are, double aim, cpx<R>* B, int64_t ldb, int tB) {
  const int64_t total = rows * cols;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t i, j;
    if (!tB) { i = idx % rows; j = idx / rows; }
    else { j = idx % cols; i = idx / cols; }
    cpx<R>* p = B + mat_off(i, j, ldb, tB);
    const double br = (double)p->re, bi = (double)p->im;
    *p = mk((R)(are * br - aim * bi), (R)(are * bi + aim * br));
  }
}

template <typename R, bool SOLVE>
int launch_leaf_r(const View& v, cudaStream_t s) {
  const size_t smem = ((size_t)v.n * LEAF_COLS + (size_t)LEAF_PANEL * v.n) * sizeof(cpx<R>);
  if (smem > 200 * 1024) return fail(NLA_ERR_UNSUPPORTED, "complex diag block: block too large");
  const int64_t grid = (v.m + LEAF_COLS - 1) / LEAF_COLS;
  if (grid > 2147483647LL) return fail(NLA_ERR_UNSUPPORTED, "complex diag block: too many right-hand sides");
  static std::once_flag once;
  static cudaError_t st = cudaSuccess;
  std::call_once(once, [] {
    st = cudaFuncSetAttribute(cplx_leaf_kernel<R, SOLVE>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  });
  if (st != cudaSuccess) return cuda_status(st, "cudaFuncSetAttribute(cplx_leaf_kernel)");
  TraceScope trace(SOLVE ? NLA_K_LEAF_SOLVE : NLA_K_LEAF_MULT, s, 4.0 * (double)v.n * v.n * (double)v.m,
                   (double)sizeof(cpx<R>) * ((double)v.n * (v.n + 1) / 2 + 2.0 * (double)v.n * v.m));
  cplx_leaf_kernel<R, SOLVE><<<(unsigned)grid, LEAF_COLS, smem, s>>>(v);
  NLA_CHECK_LAUNCH("cplx_leaf_kernel");
  return NLA_OK;
}

}  // namespace cx

bool is_complex(int dtype) { return dtype == NLA_C32 || dtype == NLA_C64; }

constexpr int64_t CPLX_LEAF_MAX = 128;  // rows of a complex diagonal block held in shared memory

int launch_leaf_complex(char func, char side, char uplo, int dtype, int64_t n, int64_t m, const Mat& A, const Mat& B,
                        cudaStream_t s, bool unit) {
  if (n <= 0 || m <= 0) return NLA_OK;
  if (n > 1024) return fail(NLA_ERR_ARG, "diag block: n must be <= 1024");
  if (B.t) return fail(NLA_ERR_UNSUPPORTED, "diag block: transposed B view");
  if (n > CPLX_LEAF_MAX) {
    // A larger block (the reference's 256-row solve leaves, or a direct
    // nla_diag_block call) runs the recursion itself down to blocks that fit.
    RecPlan c{func, side, uplo, dtype, m, CPLX_LEAF_MAX, s, GEMM_PLAIN, 1, false};
    c.unit = unit;
    return recurse(c, A, n, B);
  }
  cx::View v;
  v.A = A.p;
  v.lda = A.ld;
  v.tA = A.t;
  v.conj = A.c;
  v.B = B.p;
  v.ldb = B.ld;
  v.tB = 0;
  v.unit = unit ? 1 : 0;
  v.n = (int)n;
  v.m = m;
  if (side == 'R') {  // X op(A) = B  <=>  op(A)^T X^T = B^T (no conjugation added)
    v.tA = !v.tA;
    v.tB = 1;
    uplo = uplo == 'L' ? 'U' : 'L';
  }
  v.rev = uplo == 'U';
  if (dtype == NLA_C64)
    return func == 'S' ? cx::launch_leaf_r<double, true>(v, s) : cx::launch_leaf_r<double, false>(v, s);
  return func == 'S' ? cx::launch_leaf_r<float, true>(v, s) : cx::launch_leaf_r<float, false>(v, s);
}

int launch_gemm_complex(int dtype, int64_t N, int64_t M, int64_t K, double alpha, const Mat& A, const Mat& B,
                        const Mat& C, cudaStream_t s) {
  if (N <= 0 || M <= 0) return NLA_OK;
  if (C.t) return fail(NLA_ERR_UNSUPPORTED, "gemm: transposed output view");
  const int64_t gx = (N + cx::GT - 1) / cx::GT, gy = (M + cx::GT - 1) / cx::GT;
  if (gx > 2147483647LL || gy > 65535) return fail(NLA_ERR_UNSUPPORTED, "gemm: matrix too large for one launch");
  const size_t es = dtype == NLA_C64 ? 16 : 8;
  TraceScope trace(NLA_K_GEMM_SIMT, s, 8.0 * (double)N * (double)M * (double)K,
                   (double)es * ((double)N * K + (double)K * M + 2.0 * (double)N * M));
  if (dtype == NLA_C64)
    cx::cplx_gemm_kernel<double><<<dim3((unsigned)gx, (unsigned)gy), 256, 0, s>>>(
        N, M, K, alpha, static_cast<const cx::cpx<double>*>(A.p), A.ld, A.t, A.c,
        static_cast<const cx::cpx<double>*>(B.p), B.ld, B.t, B.c, static_cast<cx::cpx<double>*>(C.p), C.ld);
  else
    cx::cplx_gemm_kernel<float><<<dim3((unsigned)gx, (unsigned)gy), 256, 0, s>>>(
        N, M, K, (float)alpha, static_cast<const cx::cpx<float>*>(A.p), A.ld, A.t, A.c,
        static_cast<const cx::cpx<float>*>(B.p), B.ld, B.t, B.c, static_cast<cx::cpx<float>*>(C.p), C.ld);
  NLA_CHECK_LAUNCH("cplx_gemm_kernel");
  return NLA_OK;
}

int launch_scale_complex(int dtype, int64_t rows, int64_t cols, double alpha_re, double alpha_im, const Mat& B,
                         cudaStream_t s) {
  if (rows <= 0 || cols <= 0 || (alpha_re == 1.0 && alpha_im == 0.0)) return NLA_OK;
  const int64_t total = rows * cols;
  int64_t blocks = (total + 255) / 256;
  const int64_t cap = (int64_t)num_sms() * 8;
  if (blocks > cap) blocks = cap;
  TraceScope trace(NLA_K_SCALE, s, 6.0 * (double)total, 2.0 * (double)total * (double)dtype_size(dtype));
  if (dtype == NLA_C64)
    cx::cplx_scale_kernel<double><<<(unsigned)blocks, 256, 0, s>>>(rows, cols, alpha_re, alpha_im,
                                                                    static_cast<cx::cpx<double>*>(B.p), B.ld, B.t);
  else
    cx::cplx_scale_kernel<float><<<(unsigned)blocks, 256, 0, s>>>(rows, cols, alpha_re, alpha_im,
                                                                   static_cast<cx::cpx<float>*>(B.p), B.ld, B.t);
  NLA_CHECK_LAUNCH("cplx_scale_kernel");
  return NLA_OK;
}

}  // namespace nla
