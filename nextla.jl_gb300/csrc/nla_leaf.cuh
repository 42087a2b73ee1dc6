// Diagonal-block solve / multiply building blocks shared by the base-case
// kernels (nla_leaf.cu) and the persistent batched solver (nla_batched.cu).
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
// down the diagonal in 32-row panels: the panel's 32 x 32 triangle is solved
// by one warp per group of columns, one row per lane, each solved value
// broadcast to the lanes below with __shfl_sync; reciprocals of the diagonal
// are formed once per CTA, not once per right-hand side; the rows below the
// panel are then updated from a 128 x 32 slab of A staged through shared
// memory with coalesced loads.  Float16 blocks are computed in Float32 and
// rounded once when stored.
#pragma once

#include <type_traits>

#include "nla_common.cuh"

namespace nla {
namespace leafdev {

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
  int unit;  // unit diagonal: the diagonal of A is taken as 1 and not read
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

// With BATCH > 1 the loads are issued in batches of BATCH per thread before
// any is used, so that a CTA that is alone on its SM keeps many requests in
// flight; kernels with several CTAs per SM use BATCH = 1 (fewer registers).
template <typename T, typename Tc, int CW, int BATCH = 1>
__device__ __forceinline__ void load_block(const LeafArgs& g, Tc* X, int64_t c0, int ncols, Tc alpha = Tc(1)) {
  const T* B = static_cast<const T*>(g.B);
  const int total = g.n * CW;
  for (int base = threadIdx.x; base < total; base += LEAF_THREADS * BATCH) {
    Tc v[BATCH];
#pragma unroll
    for (int u = 0; u < BATCH; ++u) {
      const int idx = base + u * LEAF_THREADS;
      int i, c;
      if (!g.tB) { i = idx % g.n; c = idx / g.n; }
      else { c = idx % CW; i = idx / CW; }
      v[u] = idx < total && c < ncols ? alpha * Elem<T>::load(B + b_off<T>(g, i, c0 + c)) : Tc(0);
    }
#pragma unroll
    for (int u = 0; u < BATCH; ++u) {
      const int idx = base + u * LEAF_THREADS;
      int i, c;
      if (!g.tB) { i = idx % g.n; c = idx / g.n; }
      else { c = idx % CW; i = idx / CW; }
      if (idx < total) X[i * CW + c] = v[u];
    }
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

// acc[i][c] += sum_kk slab[tr + 32 i][kk] * Xp[kk, tc * CW/4 + c] for
// kk < pw: LEAF_THREADS threads as 32 row lanes (tr) x 4 column groups (tc,
// one warp each, so the X reads are warp-wide broadcasts).  Each k step reads
// 4 slab values and CW/4 values of X for 4 * CW/4 fused multiply-adds.  Row
// slots past `rows` multiply zeros of the slab: skipping them (with
// predicates or per-slot-count copies of the body) measured slower in the
// persistent batched solver, whose CTAs see every chunk height.
template <typename Tc, int CW>
__device__ __forceinline__ void tile_product(const Tc* __restrict__ slab, const Tc* __restrict__ Xp, int pw,
                                             int rows, Tc (&acc)[4][CW / 4]) {
  (void)rows;
  constexpr int CT = CW / 4;
  const int tr = threadIdx.x & 31, tc = threadIdx.x >> 5;
  for (int kk = 0; kk < pw; ++kk) {
    Tc a[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) a[i] = slab[(tr + 32 * i) * SLAB_PAD + kk];
    Tc xv[CT];
    const Tc* xr = Xp + kk * CW + tc * CT;
#pragma unroll
    for (int c = 0; c < CT; ++c) xv[c] = xr[c];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int c = 0; c < CT; ++c) acc[i][c] = fma(a[i], xv[c], acc[i][c]);
  }
}

// Xo[r, :] -= sum_kk slab[r][kk] * Xp[kk, :] for r < rows, kk < pw.
template <typename Tc, int CW>
__device__ __forceinline__ void trailing_update(const Tc* __restrict__ slab, const Tc* __restrict__ Xp,
                                                Tc* __restrict__ Xo, int rows, int pw) {
  constexpr int CT = CW / 4;
  const int tr = threadIdx.x & 31, tc = threadIdx.x >> 5;
  Tc acc[4][CT];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int c = 0; c < CT; ++c) acc[i][c] = Tc(0);
  tile_product<Tc, CW>(slab, Xp, pw, rows, acc);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = tr + 32 * i;
    if (r < rows) {
      Tc* xo = Xo + r * CW + tc * CT;
#pragma unroll
      for (int c = 0; c < CT; ++c) xo[c] -= acc[i][c];
    }
  }
}

// Canonical lower-left solve: X := L^{-1} (alpha X) for the CW columns
// starting at c0 (ncols of them valid), run by one CTA of LEAF_THREADS.
// smem holds leaf_solve_smem_elems(n, CW) compute-type elements.
template <typename T, int CW>
__device__ __forceinline__ void solve_block(const LeafArgs& g, int64_t c0, int ncols, unsigned char* smem_raw,
                                            typename Elem<T>::compute alpha) {
  using Tc = typename Elem<T>::compute;
  Tc* X = reinterpret_cast<Tc*>(smem_raw);            // n x CW
  Tc* inv_d = X + (size_t)g.n * CW;                   // n
  Tc* slab = inv_d + g.n;                             // 128 x 33
  Tc* diag = slab + LEAF_THREADS * SLAB_PAD;          // 32 x 33
  const int n = g.n;
  const T* A = static_cast<const T*>(g.A);

  load_block<T, Tc, CW>(g, X, c0, ncols, alpha);
  for (int i = threadIdx.x; i < n; i += LEAF_THREADS)
    inv_d[i] = g.unit ? Tc(1) : Tc(1) / Elem<T>::load(A + a_off<T>(g, i, i));
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

    // Rows below the panel: X[r, :] -= A[r, panel] * X[panel, :], as a
    // register-tiled product: thread (tr, tc) owns rows r0 + tr + 32 i
    // (i < 4) and the CW/4 columns of column group tc (its warp), so each
    // k step reads 4 slab values and one broadcast vector of X for 4 * CW/4
    // fused multiply-adds.
    for (int r0 = p0 + pw; r0 < n; r0 += LEAF_THREADS) {
      const int rows = min(LEAF_THREADS, n - r0);
      stage_slab<LEAF_THREADS, T>(g, slab, r0, rows, p0, pw, [](int, int) { return true; });
      __syncthreads();
      trailing_update<Tc, CW>(slab, X + (size_t)p0 * CW, X + (size_t)r0 * CW, rows, pw);
      __syncthreads();
    }
  }
  __syncthreads();
  store_block<T, Tc, CW>(g, X, c0, ncols);
}

// Xo[r, :] -= sum_kk slab[r][kk] * Xp[kk, :] for r < rows, kk < pw, for wide
// column blocks: LEAF_THREADS threads as RG row groups x (LEAF_THREADS / RG)
// column groups, each thread a 4-row x CT-column register tile (rows strided
// by RG so that slab reads are conflict-free).  rows <= 4 * RG.
template <typename Tc, int CW, int RG, int SLOTS>
__device__ __forceinline__ void trailing_update_wide_n(const Tc* __restrict__ slab, const Tc* __restrict__ Xp,
                                                       Tc* __restrict__ Xo, int rows, int pw) {
  constexpr int CG = LEAF_THREADS / RG;
  constexpr int CT = CW / CG;
  const int tr = threadIdx.x % RG, tc = threadIdx.x / RG;
  Tc acc[SLOTS][CT];
#pragma unroll
  for (int i = 0; i < SLOTS; ++i)
#pragma unroll
    for (int c = 0; c < CT; ++c) acc[i][c] = Tc(0);
  for (int kk = 0; kk < pw; ++kk) {
    Tc a[SLOTS];
#pragma unroll
    for (int i = 0; i < SLOTS; ++i) a[i] = slab[(tr + RG * i) * SLAB_PAD + kk];
    const Tc* xr = Xp + kk * CW + tc * CT;
#pragma unroll
    for (int c = 0; c < CT; ++c) {
      const Tc xv = xr[c];
#pragma unroll
      for (int i = 0; i < SLOTS; ++i) acc[i][c] = fma(a[i], xv, acc[i][c]);
    }
  }
#pragma unroll
  for (int i = 0; i < SLOTS; ++i) {
    const int r = tr + RG * i;
    if (r < rows) {
      Tc* xo = Xo + r * CW + tc * CT;
#pragma unroll
      for (int c = 0; c < CT; ++c) xo[c] -= acc[i][c];
    }
  }
}

// Float64: row slots with RG * i >= rows hold no row of the chunk and are
// skipped (the slot count is a compile-time constant of the body), which pays
// on the 2-FMA-per-clock DFMA pipe.  Float32 keeps the single full-height
// body, which measured faster there.
template <typename Tc, int CW, int RG>
__device__ __forceinline__ void trailing_update_wide(const Tc* __restrict__ slab, const Tc* __restrict__ Xp,
                                                     Tc* __restrict__ Xo, int rows, int pw) {
  if constexpr (!std::is_same<Tc, double>::value) {
    trailing_update_wide_n<Tc, CW, RG, 4>(slab, Xp, Xo, rows, pw);
    return;
  }
  switch ((rows + RG - 1) / RG) {
    case 1: trailing_update_wide_n<Tc, CW, RG, 1>(slab, Xp, Xo, rows, pw); break;
    case 2: trailing_update_wide_n<Tc, CW, RG, 2>(slab, Xp, Xo, rows, pw); break;
    case 3: trailing_update_wide_n<Tc, CW, RG, 3>(slab, Xp, Xo, rows, pw); break;
    default: trailing_update_wide_n<Tc, CW, RG, 4>(slab, Xp, Xo, rows, pw); break;
  }
}

// Canonical lower-left solve for wide column blocks (CW in {16, 32, 64, 128}):
// the same panels as solve_block, but each panel's 32 x 32 triangle is solved
// with one right-hand side per thread (threads < CW), fully unrolled over the
// panel's values in registers, so every lane does useful work and no value
// has to cross lanes.
template <typename T, int CW>
__device__ __forceinline__ void solve_block_wide(const LeafArgs& g, int64_t c0, int ncols, unsigned char* smem_raw,
                                                 typename Elem<T>::compute alpha) {
  using Tc = typename Elem<T>::compute;
  constexpr int RG = CW >= 128 ? 16 : 32;  // row groups of the trailing update
  constexpr int CHUNK = 4 * RG;            // rows per trailing-update pass
  Tc* X = reinterpret_cast<Tc*>(smem_raw);            // n x CW
  Tc* inv_d = X + (size_t)g.n * CW;                   // n
  Tc* slab = inv_d + g.n;                             // 128 x 33
  Tc* diag = slab + LEAF_THREADS * SLAB_PAD;          // 32 x 33
  const int n = g.n;
  const T* A = static_cast<const T*>(g.A);

  load_block<T, Tc, CW>(g, X, c0, ncols, alpha);
  for (int i = threadIdx.x; i < n; i += LEAF_THREADS)
    inv_d[i] = g.unit ? Tc(1) : Tc(1) / Elem<T>::load(A + a_off<T>(g, i, i));
  __syncthreads();

  const int t = threadIdx.x;
  for (int p0 = 0; p0 < n; p0 += PANEL) {
    const int pw = min(PANEL, n - p0);
    stage_slab<PANEL, T>(g, diag, p0, pw, p0, pw, [](int i, int j) { return j < i; });
    __syncthreads();
    // The panel's serial chains run on CW threads.  In Float64 the warps
    // that take them rotate with the panel and the CTA so that co-resident
    // CTAs spread this FP64 work over all four SM sub-partitions.
    const int rot = std::is_same<Tc, double>::value ? 32 * (int)((p0 / PANEL + blockIdx.x) % (LEAF_THREADS / 32)) : 0;
    const int tt = (t - rot + LEAF_THREADS) % LEAF_THREADS;
    if (tt < CW) {
      // Right-looking: x_j is subtracted from every later row as soon as it
      // is known.  Each row sees the same FMAs in the same order (j
      // increasing) as a row-by-row dot product, so the bits are the same,
      // and the dependent chain is one FMA and one multiply per row.
      Tc y[PANEL];
#pragma unroll
      for (int r = 0; r < PANEL; ++r) y[r] = r < pw ? X[(p0 + r) * CW + tt] : Tc(0);
#pragma unroll
      for (int j = 0; j < PANEL; ++j) {
        if (j < pw) {
          const Tc xj = y[j] * inv_d[p0 + j];
          X[(p0 + j) * CW + tt] = xj;
#pragma unroll
          for (int r = j + 1; r < PANEL; ++r) y[r] = fma(-diag[r * SLAB_PAD + j], xj, y[r]);
        }
      }
    }
    __syncthreads();
    for (int r0 = p0 + pw; r0 < n; r0 += CHUNK) {
      const int rows = min(CHUNK, n - r0);
      stage_slab<CHUNK, T>(g, slab, r0, rows, p0, pw, [](int, int) { return true; });
      __syncthreads();
      trailing_update_wide<Tc, CW, RG>(slab, X + (size_t)p0 * CW, X + (size_t)r0 * CW, rows, pw);
      __syncthreads();
    }
  }
  __syncthreads();
  store_block<T, Tc, CW>(g, X, c0, ncols);
}

// Float64 solve with one right-hand side per thread, for n <= COLS_MAX_N and
// CW columns per CTA.  GB300 issues FP64 at two fused multiply-adds per clock
// per SM, and measured time is proportional to the FP64 warp instructions an
// SM issues, whichever sub-partitions issue them (8 warps of independent FMA
// chains take 8/7 of the time of 7).  So a solve over m columns is fastest
// with the fewest columns per CTA that still fit one CTA per SM: 112 for
// m = 16384 (147 CTAs) instead of 128 (128 CTAs, 24 SMs idle).
//
// The kernel works left-looking over 32-row panels.  Each thread keeps its
// panel's 32 values in registers, y, and does two steps:
//   1. Subtract the already solved rows of its column,
//      y -= A[p0:p0+32, 0:p0] x[0:p0]. These are 32 independent FMA chains.
//   2. Solve the panel's triangle column by column, so that y_i gets its
//      update as soon as x_j is known.
// Each thread does n(n-1)/2 FMAs in total. The A rows of the panel are staged
// once per panel in shared memory and read as warp-wide broadcasts. X stays in
// shared memory, one column per thread, so accesses are conflict-free.
constexpr int COLS_MAX_N = 128;
constexpr int LOAD_BATCH = 16;  // loads in flight per thread (one CTA per SM)

// HALVES = 2 runs two threads per right-hand side (256 per CTA): the halves
// split the already-solved rows of each panel's update, so that every SM
// sub-partition has two warps issuing FMAs in that phase; half 1 hands its
// partial sums over through shared memory and half 0 solves the triangle.
__host__ __device__ constexpr size_t leaf_cols_smem_elems(int n, int halves, int cw = LEAF_THREADS) {
  return (size_t)n * cw + (size_t)PANEL * COLS_MAX_N + (size_t)n + (halves > 1 ? (size_t)PANEL * cw : 0);
}

template <int HALVES, int CW>
__device__ __forceinline__ void solve_cols_f64(const LeafArgs& g, int64_t c0, int ncols, unsigned char* smem_raw,
                                               double alpha) {
  static_assert(CW % 8 == 0 && CW <= LEAF_THREADS, "right-hand sides per CTA");
  constexpr int NT = CW * HALVES;  // threads per CTA
  const int n = g.n;
  double* X = reinterpret_cast<double*>(smem_raw);  // n x CW
  double* L = X + (size_t)n * CW;                   // PANEL x COLS_MAX_N: rows p0.., columns 0..
  double* inv_d = L + PANEL * COLS_MAX_N;           // n
  double* Y1 = inv_d + n;                           // PANEL x CW partial sums of half 1
  const double* A = static_cast<const double*>(g.A);
  const double* Bp = static_cast<const double*>(g.B);
  const int t = threadIdx.x, c = t % CW, h = t / CW;

  // Block of B (times alpha), LOAD_BATCH loads in flight per thread.
  const int total = n * CW;
  for (int base = t; base < total; base += NT * LOAD_BATCH) {
    double v[LOAD_BATCH];
#pragma unroll
    for (int u = 0; u < LOAD_BATCH; ++u) {
      const int idx = base + u * NT;
      int i, cc;
      if (!g.tB) { i = idx % n; cc = idx / n; }
      else { cc = idx % CW; i = idx / CW; }
      v[u] = idx < total && cc < ncols ? alpha * Bp[b_off<double>(g, i, c0 + cc)] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < LOAD_BATCH; ++u) {
      const int idx = base + u * NT;
      int i, cc;
      if (!g.tB) { i = idx % n; cc = idx / n; }
      else { cc = idx % CW; i = idx / CW; }
      if (idx < total) X[i * CW + cc] = v[u];
    }
  }
  for (int i = t; i < n; i += NT) inv_d[i] = g.unit ? 1.0 : 1.0 / A[a_off<double>(g, i, i)];
  for (int p0 = 0; p0 < n; p0 += PANEL) {
    const int pw = min(PANEL, n - p0);
    // Columns of A staged for the panel's rows: through the diagonal, rounded
    // up to even for the paired loads (the extra column is zero).
    const int kw = (p0 + pw + 1) & ~1;
    __syncthreads();  // previous panel done with L and Y1 (and X, inv_d ready)
    // Stage A[p0 + i][k], i < PANEL, k < kw; zero on and above the diagonal
    // and below the block.  Threads run along the index contiguous in memory.
    for (int base = t; base < PANEL * kw; base += NT * LOAD_BATCH) {
      double v[LOAD_BATCH];
#pragma unroll
      for (int u = 0; u < LOAD_BATCH; ++u) {
        const int idx = base + u * NT;
        int i, k;
        if (!g.tA) { i = idx % PANEL; k = idx / PANEL; }
        else { k = idx % kw; i = idx / kw; }
        v[u] = idx < PANEL * kw && i < pw && k < p0 + i ? A[a_off<double>(g, p0 + i, k)] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < LOAD_BATCH; ++u) {
        const int idx = base + u * NT;
        int i, k;
        if (!g.tA) { i = idx % PANEL; k = idx / PANEL; }
        else { k = idx % kw; i = idx / kw; }
        if (idx < PANEL * kw) L[i * COLS_MAX_N + k] = v[u];
      }
    }
    __syncthreads();
    double y[PANEL];
#pragma unroll
    for (int i = 0; i < PANEL; ++i) y[i] = h == 0 && i < pw ? X[(p0 + i) * CW + c] : 0.0;
    // Already-solved rows: half h takes k in [h p0 / HALVES, (h+1) p0 / HALVES)
    // (p0 is a multiple of 32, so both ranges have even bounds).  Two k per
    // step with one 16-byte broadcast load of A per row; the two FMAs into
    // each y[i] of a step are PANEL instructions apart.
    const int ka = h * (p0 / HALVES), kb = (h + 1) * (p0 / HALVES);
    for (int k = ka; k < kb; k += 2) {
      const double xk0 = X[k * CW + c], xk1 = X[(k + 1) * CW + c];
      double2 a[PANEL];
#pragma unroll
      for (int i = 0; i < PANEL; ++i) a[i] = *reinterpret_cast<const double2*>(&L[i * COLS_MAX_N + k]);
#pragma unroll
      for (int i = 0; i < PANEL; ++i) y[i] = fma(-a[i].x, xk0, y[i]);
#pragma unroll
      for (int i = 0; i < PANEL; ++i) y[i] = fma(-a[i].y, xk1, y[i]);
    }
    if constexpr (HALVES > 1) {
      if (h == 1) {
#pragma unroll
        for (int i = 0; i < PANEL; ++i) Y1[i * CW + c] = y[i];
      }
      __syncthreads();
      if (h == 0) {
#pragma unroll
        for (int i = 0; i < PANEL; ++i) y[i] += Y1[i * CW + c];
      }
    }
    if (h == 0) {
      if (pw == PANEL) {
        // Full panel: the triangle two columns at a time (x_j, then x_{j+1},
        // then one paired load and two FMAs for each row below).
#pragma unroll
        for (int jj = 0; jj < PANEL / 2; ++jj) {
          const int j = 2 * jj;
          const double xj = y[j] * inv_d[p0 + j];
          const double xj1 = fma(-L[(j + 1) * COLS_MAX_N + p0 + j], xj, y[j + 1]) * inv_d[p0 + j + 1];
          y[j] = xj;
          y[j + 1] = xj1;
#pragma unroll
          for (int i = j + 2; i < PANEL; ++i) {
            const double2 a = *reinterpret_cast<const double2*>(&L[i * COLS_MAX_N + p0 + j]);
            y[i] = fma(-a.x, xj, y[i]);
            y[i] = fma(-a.y, xj1, y[i]);
          }
        }
      } else {
#pragma unroll
        for (int j = 0; j < PANEL; ++j) {
          if (j < pw) {
            const double xj = y[j] * inv_d[p0 + j];
            y[j] = xj;
#pragma unroll
            for (int i = j + 1; i < PANEL; ++i) y[i] = fma(-L[i * COLS_MAX_N + p0 + j], xj, y[i]);
          }
        }
      }
#pragma unroll
      for (int i = 0; i < PANEL; ++i)
        if (i < pw) X[(p0 + i) * CW + c] = y[i];
    }
  }
  __syncthreads();
  double* Bo = static_cast<double*>(g.B);
  for (int idx = t; idx < total; idx += NT) {
    int i, cc;
    if (!g.tB) { i = idx % n; cc = idx / n; }
    else { cc = idx % CW; i = idx / CW; }
    if (cc < ncols) Bo[b_off<double>(g, i, c0 + cc)] = X[i * CW + cc];
  }
}

__host__ __device__ constexpr size_t leaf_solve_smem_elems(int n, int CW) {
  return (size_t)n * CW + (size_t)n + (size_t)LEAF_THREADS * SLAB_PAD + (size_t)PANEL * SLAB_PAD;
}

}  // namespace leafdev
}  // namespace nla
