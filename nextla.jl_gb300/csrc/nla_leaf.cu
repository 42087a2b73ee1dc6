// Base cases of the recursion on one diagonal block (n <= 1024):
//   func 'S': the triangular solve of LeftLowerTRSM! ... RightUpperTRSM!
//             (src/trsm.jl:5-150);
//   func 'M': the triangular multiply of LeftLowerTRMM! ... RightUpperTRMM!
//             (src/trmm.jl:43-389).
//
// All eight (func, side, uplo) forms map onto one canonical problem, a
// LOWER triangle applied from the LEFT:
//   side 'R' becomes side 'L' on transposed operands (X op(A) = B  <=>
//   op(A)^T X^T = B^T), which flips uplo;
//   uplo 'U' becomes lower by reversing the index order of the block
//   (i -> n-1-i on rows and columns of A and on the rows of B).
// Both are pure index maps, so no data is copied.
//
// One CTA of 128 threads (a warp-group) owns CW right-hand sides.  The CTA
// stages its n x CW block of B in shared memory in the compute type and works
// down the diagonal in 32-row panels:
//   solve:    the panel's 32 x 32 triangle is solved by one warp per group of
//             columns, one row per lane, each solved value broadcast to the
//             lanes below with __shfl_sync; reciprocals of the diagonal are
//             formed once per CTA, not once per right-hand side; the rows
//             below the panel are then updated from a 128 x 32 slab of A
//             staged through shared memory with coalesced loads;
//   multiply: each thread forms one output row as a dot product with
//             increasing k (the reference's order, src/trmm.jl:90-94), reading
//             A through the same staged slabs and B from shared memory, and
//             writes it straight to global memory (B was fully staged first,
//             so the in-place update has no hazard).
// Float16 blocks are computed in Float32 and rounded once when stored.
#include <mutex>

#include "nla_common.cuh"

namespace nla {
namespace {

constexpr int LEAF_THREADS = 128;
constexpr int PANEL = 32;
constexpr int SLAB_PAD = PANEL + 1;

struct LeafArgs {
  const void* A;
  int64_t lda;
  int tA;
  void* B;
  int64_t ldb;
  int tB;
  int rev;
  int n;
  int64_t m;
};

template <typename T>
__device__ __forceinline__ int64_t a_off(const LeafArgs& g, int i, int j) {
  int mi = g.rev ? g.n - 1 - i : i, mj = g.rev ? g.n - 1 - j : j;
  return mat_off(mi, mj, g.lda, g.tA);
}

template <typename T>
__device__ __forceinline__ int64_t b_off(const LeafArgs& g, int i, int64_t c) {
  int mi = g.rev ? g.n - 1 - i : i;
  return mat_off(mi, c, g.ldb, g.tB);
}

// Stage Acan(r0 + t, k0 + kk), t < rows <= ROWS, kk < cols, into slab[t][kk] (zero
// outside, and zero where keep(t, kk) is false).  Threads run along the index
// that is contiguous in memory.
template <int ROWS, typename T, typename Tc, typename Keep>
__device__ __forceinline__ void stage_slab(const LeafArgs& g, Tc* slab, int r0, int rows, int k0, int cols,
                                           Keep keep) {
  const T* A = static_cast<const T*>(g.A);
  for (int idx = threadIdx.x; idx < ROWS * PANEL; idx += LEAF_THREADS) {
    int t, kk;
    if (!g.tA) { t = idx % ROWS; kk = idx / ROWS; }
    else { kk = idx % PANEL; t = idx / PANEL; }
    Tc v = Tc(0);
    if (t < rows && kk < cols && keep(r0 + t, k0 + kk)) v = Elem<T>::load(A + a_off<T>(g, r0 + t, k0 + kk));
    slab[t * SLAB_PAD + kk] = v;
  }
}

template <typename T, typename Tc, int CW>
__device__ __forceinline__ void load_block(const LeafArgs& g, Tc* X, int64_t c0, int ncols) {
  const T* B = static_cast<const T*>(g.B);
  const int total = g.n * CW;
  for (int idx = threadIdx.x; idx < total; idx += LEAF_THREADS) {
    int i, c;
    if (!g.tB) { i = idx % g.n; c = idx / g.n; }
    else { c = idx % CW; i = idx / CW; }
    X[i * CW + c] = c < ncols ? Elem<T>::load(B + b_off<T>(g, i, c0 + c)) : Tc(0);
  }
}

template <typename T, typename Tc, int CW>
__device__ __forceinline__ void store_block(const LeafArgs& g, const Tc* X, int64_t c0, int ncols) {
  T* B = static_cast<T*>(g.B);
  const int total = g.n * CW;
  for (int idx = threadIdx.x; idx < total; idx += LEAF_THREADS) {
    int i, c;
    if (!g.tB) { i = idx % g.n; c = idx / g.n; }
    else { c = idx % CW; i = idx / CW; }
    if (c < ncols) Elem<T>::store(B + b_off<T>(g, i, c0 + c), X[i * CW + c]);
  }
}

// Canonical lower-left solve: X := L^{-1} X for CW columns.
template <typename T, int CW>
__global__ void __launch_bounds__(LEAF_THREADS) leaf_solve_kernel(LeafArgs g) {
  using Tc = typename Elem<T>::compute;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Tc* X = reinterpret_cast<Tc*>(smem_raw);            // n x CW
  Tc* inv_d = X + (size_t)g.n * CW;                   // n
  Tc* slab = inv_d + g.n;                             // 128 x 33
  Tc* diag = slab + LEAF_THREADS * SLAB_PAD;          // 32 x 33

  const int64_t c0 = (int64_t)blockIdx.x * CW;
  const int ncols = (int)(g.m - c0 < CW ? g.m - c0 : CW);
  const int n = g.n;
  const T* A = static_cast<const T*>(g.A);

  load_block<T, Tc, CW>(g, X, c0, ncols);
  for (int i = threadIdx.x; i < n; i += LEAF_THREADS) inv_d[i] = Tc(1) / Elem<T>::load(A + a_off<T>(g, i, i));
  __syncthreads();

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int CPW = CW / 4;  // columns per warp
  for (int p0 = 0; p0 < n; p0 += PANEL) {
    const int pw = min(PANEL, n - p0);
    // Strictly-lower part of the panel's diagonal block.
    stage_slab<PANEL, T>(g, diag, p0, pw, p0, pw, [](int i, int j) { return j < i; });
    __syncthreads();

    Tc x[CPW];
#pragma unroll
    for (int q = 0; q < CPW; ++q) x[q] = lane < pw ? X[(p0 + lane) * CW + warp + 4 * q] : Tc(0);
    for (int i = 0; i < pw; ++i) {
      const Tc lij = diag[lane * SLAB_PAD + i];
      const Tc inv = inv_d[p0 + i];
#pragma unroll
      for (int q = 0; q < CPW; ++q) {
        if (lane == i) x[q] *= inv;
        const Tc xi = __shfl_sync(0xffffffffu, x[q], i);
        if (lane > i) x[q] = fma(-lij, xi, x[q]);
      }
    }
    if (lane < pw) {
#pragma unroll
      for (int q = 0; q < CPW; ++q) X[(p0 + lane) * CW + warp + 4 * q] = x[q];
    }
    __syncthreads();

    // Rows below the panel: X[r, :] -= A[r, panel] * X[panel, :].
    for (int r0 = p0 + pw; r0 < n; r0 += LEAF_THREADS) {
      const int rows = min(LEAF_THREADS, n - r0);
      stage_slab<LEAF_THREADS, T>(g, slab, r0, rows, p0, pw, [](int, int) { return true; });
      __syncthreads();
      const int t = threadIdx.x;
      if (t < rows) {
        Tc acc[CW];
#pragma unroll
        for (int c = 0; c < CW; ++c) acc[c] = Tc(0);
        for (int kk = 0; kk < pw; ++kk) {
          const Tc a = slab[t * SLAB_PAD + kk];
          const Tc* xr = X + (p0 + kk) * CW;
#pragma unroll
          for (int c = 0; c < CW; ++c) acc[c] = fma(a, xr[c], acc[c]);
        }
        Tc* xo = X + (r0 + t) * CW;
#pragma unroll
        for (int c = 0; c < CW; ++c) xo[c] -= acc[c];
      }
      __syncthreads();
    }
  }
  store_block<T, Tc, CW>(g, X, c0, ncols);
}

// Canonical lower-left multiply: X := L X for CW columns.
template <typename T, int CW>
__global__ void __launch_bounds__(LEAF_THREADS) leaf_mult_kernel(LeafArgs g) {
  using Tc = typename Elem<T>::compute;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Tc* X = reinterpret_cast<Tc*>(smem_raw);  // n x CW (original B)
  Tc* slab = X + (size_t)g.n * CW;          // 128 x 33

  const int64_t c0 = (int64_t)blockIdx.x * CW;
  const int ncols = (int)(g.m - c0 < CW ? g.m - c0 : CW);
  const int n = g.n;
  T* Bp = static_cast<T*>(g.B);

  load_block<T, Tc, CW>(g, X, c0, ncols);
  __syncthreads();

  for (int r0 = 0; r0 < n; r0 += LEAF_THREADS) {
    const int rows = min(LEAF_THREADS, n - r0);
    const int kmax = min(n, r0 + rows);  // k <= r
    const int t = threadIdx.x;
    const int r = r0 + t;
    Tc acc[CW];
#pragma unroll
    for (int c = 0; c < CW; ++c) acc[c] = Tc(0);
    for (int k0 = 0; k0 < kmax; k0 += PANEL) {
      const int kw = min(PANEL, kmax - k0);
      stage_slab<LEAF_THREADS, T>(g, slab, r0, rows, k0, kw, [](int i, int j) { return j <= i; });
      __syncthreads();
      if (t < rows) {
        for (int kk = 0; kk < kw; ++kk) {
          const Tc a = slab[t * SLAB_PAD + kk];
          const Tc* xr = X + (k0 + kk) * CW;
#pragma unroll
          for (int c = 0; c < CW; ++c) acc[c] = fma(a, xr[c], acc[c]);
        }
      }
      __syncthreads();
    }
    if (t < rows) {
#pragma unroll
      for (int c = 0; c < CW; ++c)
        if (c < ncols) Elem<T>::store(Bp + b_off<T>(g, r, c0 + c), acc[c]);
    }
  }
}

template <typename T, int CW>
size_t leaf_smem(char func, int n) {
  using Tc = typename Elem<T>::compute;
  size_t elems = (size_t)n * CW + (size_t)LEAF_THREADS * SLAB_PAD;
  if (func == 'S') elems += (size_t)n + (size_t)PANEL * SLAB_PAD;
  return elems * sizeof(Tc);
}

template <typename T, int CW>
int leaf_smem_attr() {
  static std::once_flag once;
  static cudaError_t st = cudaSuccess;
  std::call_once(once, [] {
    st = cudaFuncSetAttribute(leaf_solve_kernel<T, CW>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (st == cudaSuccess)
      st = cudaFuncSetAttribute(leaf_mult_kernel<T, CW>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  });
  return st == cudaSuccess ? NLA_OK : cuda_status(st, "cudaFuncSetAttribute(leaf kernels)");
}

template <typename T, int CW>
int launch_leaf_t(char func, const LeafArgs& g, cudaStream_t s) {
  const size_t smem = leaf_smem<T, CW>(func, g.n);
  const int64_t grid = (g.m + CW - 1) / CW;
  if (grid > 2147483647LL) return fail(NLA_ERR_UNSUPPORTED, "leaf: too many right-hand sides");
  if (smem > 200 * 1024) return fail(NLA_ERR_UNSUPPORTED, "leaf: shared memory plan too large");
  NLA_TRY((leaf_smem_attr<T, CW>()));
  // n^2 m flops per solve or multiply (the benchmark's convention); bytes:
  // the triangle once plus B read and written.
  TraceScope trace(func == 'S' ? NLA_K_LEAF_SOLVE : NLA_K_LEAF_MULT, s, (double)g.n * g.n * (double)g.m,
                   (double)sizeof(T) * ((double)g.n * (g.n + 1) / 2 + 2.0 * (double)g.n * g.m));
  if (func == 'S')
    leaf_solve_kernel<T, CW><<<(unsigned)grid, LEAF_THREADS, smem, s>>>(g);
  else
    leaf_mult_kernel<T, CW><<<(unsigned)grid, LEAF_THREADS, smem, s>>>(g);
  NLA_CHECK_LAUNCH(func == 'S' ? "leaf_solve_kernel" : "leaf_mult_kernel");
  return NLA_OK;
}

}  // namespace

int launch_leaf(char func, char side, char uplo, int dtype, int64_t n, int64_t m, const Mat& A, const Mat& B,
                cudaStream_t s) {
  if (n <= 0 || m <= 0) return NLA_OK;
  if (n > 1024) return fail(NLA_ERR_ARG, "diag block: n must be <= 1024");
  if (B.t) return fail(NLA_ERR_UNSUPPORTED, "diag block: transposed B view");
  LeafArgs g;
  g.A = A.p;
  g.lda = A.ld;
  g.tA = A.t;
  g.B = B.p;
  g.ldb = B.ld;
  g.tB = 0;
  g.n = (int)n;
  g.m = m;
  if (side == 'R') {  // X op(A) = B  <=>  op(A)^T X^T = B^T
    g.tA = !g.tA;
    g.tB = 1;
    uplo = uplo == 'L' ? 'U' : 'L';
  }
  g.rev = uplo == 'U';
  switch (dtype) {
    case NLA_F64:
      return n <= 512 ? launch_leaf_t<double, 16>(func, g, s) : launch_leaf_t<double, 8>(func, g, s);
    case NLA_F32:
      return n <= 512 ? launch_leaf_t<float, 32>(func, g, s) : launch_leaf_t<float, 16>(func, g, s);
    case NLA_F16:
      return n <= 512 ? launch_leaf_t<__half, 32>(func, g, s) : launch_leaf_t<__half, 16>(func, g, s);
    default: return fail(NLA_ERR_DTYPE, "diag block: unknown dtype");
  }
}

}  // namespace nla
