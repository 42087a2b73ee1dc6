// Base cases of the recursion on one diagonal block (n <= 1024):
//   func 'S': the triangular solve of LeftLowerTRSM! ... RightUpperTRSM!
//             (src/trsm.jl:5-150);
//   func 'M': the triangular multiply of LeftLowerTRMM! ... RightUpperTRMM!
//             (src/trmm.jl:43-389).
// The shared device code and the canonical-form mapping are in nla_leaf.cuh.
//   multiply: each thread forms one output row as a dot product with
//             increasing k (the reference's order, src/trmm.jl:90-94), reading
//             A through staged slabs and B from shared memory, and writes it
//             straight to global memory (B was fully staged first, so the
//             in-place update has no hazard).
#include <mutex>

#include <cstdlib>

#include "nla_leaf.cuh"

namespace nla {
namespace {

using namespace leafdev;

template <typename T, int CW>
__global__ void __launch_bounds__(LEAF_THREADS) leaf_solve_kernel(LeafArgs g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int64_t c0 = (int64_t)blockIdx.x * CW;
  const int ncols = (int)(g.m - c0 < CW ? g.m - c0 : CW);
  solve_block<T, CW>(g, c0, ncols, smem_raw, typename Elem<T>::compute(1));
}

// Wide blocks of right-hand sides, one per thread in the panel solves.
template <typename T, int CW>
__global__ void __launch_bounds__(LEAF_THREADS) leaf_solve_wide_kernel(LeafArgs g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int64_t c0 = (int64_t)blockIdx.x * CW;
  const int ncols = (int)(g.m - c0 < CW ? g.m - c0 : CW);
  solve_block_wide<T, CW>(g, c0, ncols, smem_raw, typename Elem<T>::compute(1));
}

template <int HALVES, int CW>
__global__ void __launch_bounds__(CW * HALVES, 1) leaf_solve_cols_kernel(LeafArgs g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int64_t c0 = (int64_t)blockIdx.x * CW;
  const int ncols = (int)(g.m - c0 < CW ? g.m - c0 : CW);
  solve_cols_f64<HALVES, CW>(g, c0, ncols, smem_raw, 1.0);
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

  constexpr int CT = CW / 4;
  const int tr = threadIdx.x & 31, tc = threadIdx.x >> 5;
  for (int r0 = 0; r0 < n; r0 += LEAF_THREADS) {
    const int rows = min(LEAF_THREADS, n - r0);
    const int kmax = min(n, r0 + rows);  // k <= r
    Tc acc[4][CT];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int c = 0; c < CT; ++c) acc[i][c] = Tc(0);
    for (int k0 = 0; k0 < kmax; k0 += PANEL) {
      const int kw = min(PANEL, kmax - k0);
      const bool unit = g.unit != 0;
      stage_slab<LEAF_THREADS, T>(g, slab, r0, rows, k0, kw, [unit](int i, int j) { return unit ? j < i : j <= i; });
      __syncthreads();
      tile_product<Tc, CW>(slab, X + (size_t)k0 * CW, kw, rows, acc);
      __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = tr + 32 * i;
      if (r < rows) {
#pragma unroll
        for (int c = 0; c < CT; ++c)
          if (tc * CT + c < ncols) {
            // A unit diagonal contributes the row's own value of X.
            const Tc v = g.unit ? acc[i][c] + X[(size_t)(r0 + r) * CW + tc * CT + c] : acc[i][c];
            Elem<T>::store(Bp + b_off<T>(g, r0 + r, c0 + tc * CT + c), v);
          }
      }
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

template <typename T, int CW>
int launch_leaf_wide(const LeafArgs& g, cudaStream_t s) {
  using Tc = typename Elem<T>::compute;
  const size_t smem = leaf_solve_smem_elems(g.n, CW) * sizeof(Tc);
  const int64_t grid = (g.m + CW - 1) / CW;
  if (smem > 200 * 1024) return fail(NLA_ERR_UNSUPPORTED, "leaf: shared memory plan too large");
  static std::once_flag once;
  static cudaError_t st = cudaSuccess;
  std::call_once(once, [] {
    st = cudaFuncSetAttribute(leaf_solve_wide_kernel<T, CW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              200 * 1024);
  });
  if (st != cudaSuccess) return cuda_status(st, "cudaFuncSetAttribute(leaf_solve_wide_kernel)");
  TraceScope trace(NLA_K_LEAF_SOLVE, s, (double)g.n * g.n * (double)g.m,
                   (double)sizeof(T) * ((double)g.n * (g.n + 1) / 2 + 2.0 * (double)g.n * g.m));
  leaf_solve_wide_kernel<T, CW><<<(unsigned)grid, LEAF_THREADS, smem, s>>>(g);
  NLA_CHECK_LAUNCH("leaf_solve_wide_kernel");
  return NLA_OK;
}

// Threads per right-hand side of the Float64 column-per-thread leaf:
// NLA_LEAF_COLS = 0 (use the panel-parallel kernels), 1 or 2 (default 2).
int leaf_cols_mode() {
  static const int mode = [] {
    const char* v = getenv("NLA_LEAF_COLS");
    if (v && (v[0] == '0' || v[0] == '1' || v[0] == '2') && v[1] == 0) return v[0] - '0';
    return 2;
  }();
  return mode;
}

template <int HALVES, int CW>
int launch_leaf_cols(const LeafArgs& g, cudaStream_t s) {
  const size_t smem = leaf_cols_smem_elems(g.n, HALVES, CW) * sizeof(double);
  const int64_t grid = (g.m + CW - 1) / CW;
  if (g.n > COLS_MAX_N || smem > 200 * 1024) return fail(NLA_ERR_UNSUPPORTED, "leaf: shared memory plan too large");
  if (grid > 2147483647LL) return fail(NLA_ERR_UNSUPPORTED, "leaf: too many right-hand sides");
  static std::once_flag once;
  static cudaError_t st = cudaSuccess;
  std::call_once(once, [] {
    st = cudaFuncSetAttribute(leaf_solve_cols_kernel<HALVES, CW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              200 * 1024);
  });
  if (st != cudaSuccess) return cuda_status(st, "cudaFuncSetAttribute(leaf_solve_cols_kernel)");
  TraceScope trace(NLA_K_LEAF_SOLVE, s, (double)g.n * g.n * (double)g.m,
                   8.0 * ((double)g.n * (g.n + 1) / 2 + 2.0 * (double)g.n * g.m));
  leaf_solve_cols_kernel<HALVES, CW><<<(unsigned)grid, CW * HALVES, smem, s>>>(g);
  NLA_CHECK_LAUNCH("leaf_solve_cols_kernel");
  return NLA_OK;
}

// Right-hand sides per CTA of the two-threads-per-column leaf: the fewest of
// 128, 112, 96 and 64 that keep every CTA in one wave of one CTA per SM
// (NLA_LEAF_CW forces one of them).
int leaf_cols_width(int64_t m) {
  const char* v = getenv("NLA_LEAF_CW");  // read per launch, so tests can pin each width
  const int forced = v ? atoi(v) : 0;
  if (forced == 128 || forced == 112 || forced == 96 || forced == 64 || forced == 56) return forced;
  const int64_t sms = num_sms();
  for (int cw : {64, 96, 112})
    if ((m + cw - 1) / cw <= sms) return cw;
  return 128;
}

int launch_leaf_cols2(const LeafArgs& g, cudaStream_t s) {
  switch (leaf_cols_width(g.m)) {
    case 56: return launch_leaf_cols<2, 56>(g, s);
    case 64: return launch_leaf_cols<2, 64>(g, s);
    case 96: return launch_leaf_cols<2, 96>(g, s);
    case 112: return launch_leaf_cols<2, 112>(g, s);
    default: return launch_leaf_cols<2, 128>(g, s);
  }
}

// Wide solve blocks: the widest of 128/64/32 right-hand sides whose block
// fits 128 KiB of shared memory and still gives two CTAs per SM; 0 when the
// row-parallel kernel is the better choice (few right-hand sides).
int wide_cols(int64_t n, int64_t m, size_t elem) {
  if (m < 32) return 0;
  const int64_t want = 2 * (int64_t)num_sms();
  for (int cw : {128, 64, 32}) {
    if ((size_t)n * cw * elem > 128 * 1024) continue;
    if ((m + cw - 1) / cw >= want || cw == 32) return cw;
  }
  return 0;
}

template <typename T>
int launch_solve_wide(const LeafArgs& g, int cw, cudaStream_t s) {
  switch (cw) {
    case 128: return launch_leaf_wide<T, 128>(g, s);
    case 64: return launch_leaf_wide<T, 64>(g, s);
    default: return launch_leaf_wide<T, 32>(g, s);
  }
}

// Float64 register tiles wider than 32 columns do not fit the register file
// without spilling, so Float64 uses 32-column blocks.
template <>
int launch_solve_wide<double>(const LeafArgs& g, int, cudaStream_t s) {
  return launch_leaf_wide<double, 32>(g, s);
}

}  // namespace

int launch_leaf(char func, char side, char uplo, int dtype, int64_t n, int64_t m, const Mat& A, const Mat& B,
                cudaStream_t s, bool unit) {
  if (is_complex(dtype)) return launch_leaf_complex(func, side, uplo, dtype, n, m, A, B, s, unit);
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
  g.unit = unit ? 1 : 0;
  g.n = (int)n;
  g.m = m;
  if (side == 'R') {  // X op(A) = B  <=>  op(A)^T X^T = B^T
    g.tA = !g.tA;
    g.tB = 1;
    uplo = uplo == 'L' ? 'U' : 'L';
  }
  g.rev = uplo == 'U';
  if (func == 'S') {
    // Float64 blocks of up to 128 rows with enough right-hand sides to fill
    // the GPU: one right-hand side per thread, or two threads per right-hand
    // side (NLA_LEAF_COLS=0 selects the panel-parallel kernels instead).
    if (dtype == NLA_F64 && n <= COLS_MAX_N && m >= 8 * LEAF_THREADS && leaf_cols_mode() != 0)
      return leaf_cols_mode() == 1 ? launch_leaf_cols<1, LEAF_THREADS>(g, s) : launch_leaf_cols2(g, s);
    const int cw = wide_cols(n, m, dtype == NLA_F64 ? 8 : 4);
    if (cw) {
      switch (dtype) {
        case NLA_F64: return launch_solve_wide<double>(g, cw, s);
        case NLA_F32: return launch_solve_wide<float>(g, cw, s);
        case NLA_F16: return launch_solve_wide<__half>(g, cw, s);
        default: break;
      }
    }
  }
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
