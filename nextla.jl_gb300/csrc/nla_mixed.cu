// Mixed-precision form of the recursive triangular solve / multiply: an FP64
// answer for Float64 inputs, with the off-diagonal updates done on the tensor
// cores from BF16 or FP16 operand slices (nla_umma.cu) and the diagonal
// blocks in FP64 (nla_leaf.cu).  For solves, iterative refinement
//     R = alpha*B - op(A) X   (FP64 residual)
//     op(A) D = R             (same mixed solver)
//     X += D
// wins back the accuracy the split loses.
#include <cmath>
#include <cstdlib>
#include <algorithm>
#include <climits>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "nla_common.cuh"
#include "nla_split7.cuh"
#include "nla_umma.cuh"

namespace nla {
namespace {

// Second stream-ordered pool (per device and stream) for the refinement
// buffers, separate from the update kernels' staging workspace.
struct Buf {
  void* p = nullptr;
  size_t n = 0;
};
std::mutex g_buf_mu;
std::unordered_map<uint64_t, Buf> g_bufs;

int refine_buffers(cudaStream_t s, size_t bytes, void** out) {
  int dev = 0;
  cudaGetDevice(&dev);
  const uint64_t key = ((uint64_t)(uint32_t)dev << 48) ^ (uint64_t)reinterpret_cast<uintptr_t>(s);
  std::lock_guard<std::mutex> lk(g_buf_mu);
  Buf& b = g_bufs[key];
  if (b.n < bytes) {
    if (b.p) cudaFreeAsync(b.p, s);
    b.p = nullptr;
    b.n = 0;
    cudaError_t e = cudaMallocAsync(&b.p, bytes, s);
    if (e != cudaSuccess) {
      b.p = nullptr;
      return cuda_status(e, "refinement buffers");
    }
    b.n = bytes;
  }
  *out = b.p;
  return NLA_OK;
}

// dst = src on rows x cols column-major views.
__global__ void copy_kernel(int64_t rows, int64_t cols, const double* __restrict__ src, int64_t lds,
                            double* __restrict__ dst, int64_t ldd) {
  const int64_t total = rows * cols;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx % rows, j = idx / rows;
    dst[i + j * ldd] = src[i + j * lds];
  }
}

// R = B0 - R.
__global__ void residual_kernel(int64_t rows, int64_t cols, const double* __restrict__ B0, int64_t ldb0,
                                double* __restrict__ R, int64_t ldr) {
  const int64_t total = rows * cols;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx % rows, j = idx / rows;
    R[i + j * ldr] = B0[i + j * ldb0] - R[i + j * ldr];
  }
}

// X += D, and the largest |D| and |X| (as ordered bit patterns of non-negative
// doubles) into amax[0], amax[1].
__global__ void correct_kernel(int64_t rows, int64_t cols, const double* __restrict__ D, int64_t ldd,
                               double* __restrict__ X, int64_t ldx, unsigned long long* amax) {
  double md = 0.0, mx = 0.0;
  const int64_t total = rows * cols;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx % rows, j = idx / rows;
    const double d = D[i + j * ldd];
    const double x = X[i + j * ldx] + d;
    X[i + j * ldx] = x;
    md = fmax(md, fabs(d));
    mx = fmax(mx, fabs(x));
  }
  for (int o = 16; o > 0; o >>= 1) {
    md = fmax(md, __shfl_xor_sync(0xffffffffu, md, o));
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  if ((threadIdx.x & 31) == 0 && amax) {
    atomicMax(&amax[0], (unsigned long long)__double_as_longlong(md));
    atomicMax(&amax[1], (unsigned long long)__double_as_longlong(mx));
  }
}

__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  const double bp = s - a;
  e = (a - (s - bp)) + (b - bp);
}

// R = alpha*B - op(A) X (left) or alpha*B - X op(A) (right), accumulated in
// double-double (exact products by fma, error-free sums) and rounded once;
// op(A) is the `lower` (after the transpose flip) triangle of A or A^T.
__global__ void dd_residual_kernel(int64_t rows, int64_t cols, int64_t n, const double* __restrict__ A, int64_t lda,
                                   int tA, int lower, int left, const double* __restrict__ X, int64_t ldx,
                                   const double* __restrict__ B, int64_t ldb, double alpha, double* __restrict__ R,
                                   int64_t ldr) {
  const int64_t total = rows * cols;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx % rows, j = idx / rows;
    double hi = 0.0, lo = 0.0;
    // left:  sum over k of op(A)(i,k) X(k,j), k in the triangle of row i
    // right: sum over k of X(i,k) op(A)(k,j), k in the triangle of column j
    const int64_t piv = left ? i : j;
    int64_t k0, k1;
    if (left) { k0 = lower ? 0 : piv; k1 = lower ? piv + 1 : n; }
    else { k0 = lower ? piv : 0; k1 = lower ? n : piv + 1; }
    for (int64_t k = k0; k < k1; ++k) {
      double a, x;
      if (left) {
        a = tA ? A[k + i * lda] : A[i + k * lda];
        x = X[k + j * ldx];
      } else {
        a = tA ? A[j + k * lda] : A[k + j * lda];
        x = X[i + k * ldx];
      }
      const double p = a * x;
      const double pe = fma(a, x, -p);
      double e;
      two_sum(hi, p, hi, e);
      lo += e + pe;
    }
    const double b = B[i + j * ldb];
    const double q = alpha * b;
    const double qe = fma(alpha, b, -q);
    double r, e2;
    two_sum(q, -hi, r, e2);
    R[i + j * ldr] = r + ((e2 + qe) - lo);
  }
}

unsigned grid_for(int64_t total) {
  int64_t blocks = (total + 255) / 256;
  const int64_t cap = (int64_t)num_sms() * 8;
  return (unsigned)(blocks < cap ? (blocks > 0 ? blocks : 1) : cap);
}

// FP64 diagonal blocks of the mixed recursion: 64 rows.  The FP64 leaf is
// bound by GB300's FP64 pipe (2 FMA per clock per SM), so halving it from 128
// moves half of its work onto the tensor cores as one more level of short
// exact updates; with the fused staging, the short-K group table and the
// finishing pass those cost less than the leaf time they save.
int default_mixed_cutoff() {
  const char* v = std::getenv("NLA_MIXED_CUTOFF");
  if (v && *v) {
    long x = std::atol(v);
    if (x > 0) return (int)(x > 1024 ? 1024 : x);
  }
  return 64;
}

}  // namespace

// ---------------------------------------------------------------------------
// Leaves of a mixed exact solve through their inverses.  GB300 runs FP64 FMAs
// at 2 per clock per SM, so the substitution leaf (n^2 m / 2 FMAs per block)
// is a large share of a solve whose updates run on the tensor cores.  Here
// each leaf block T (at most 64 rows) is inverted once in FP64, and the leaf
// becomes X := inv(T) X, an exact 7-slice product on the tensor cores
// rounded once per element.  (X + (inv(T) - I) X, the form a general
// accumulating update would give, loses digits to cancellation when T's
// diagonal is large: x ~ b / d from b - (1 - 1/d) b.)  Where both halves of
// a recursion node are leaves, leaf_pair_kernel runs the two leaves and the
// update between them in one launch.
// ---------------------------------------------------------------------------
namespace {

constexpr int INV_MAX = 1900;  // leaves per launch (the table rides in the kernel parameters)

struct LeafInvArgs {
  const double* A;  // leaf j's block starts at A + k[j] * (lda + 1)
  int64_t lda;
  int tA, upper, unit;
  double* W;  // slot first_slot + j at W + (first_slot + j) * 64 * 64, leading dimension 64
  int first_slot;
  int count;
  int k[INV_MAX];
  int nl[INV_MAX];
};

// One CTA per leaf.  The block is read in canonical lower orientation (an
// upper block with its indices reversed), the inverse formed column by
// column by right-looking substitution (four threads per column, in one
// warp, rows split by residue mod 4), and written back in the block's own
// orientation.
constexpr int INV_SMEM = (2 * LEAF_INV_N * (LEAF_INV_N + 1) + LEAF_INV_N) * (int)sizeof(double);

__global__ void __launch_bounds__(256) leaf_inverse_kernel(const __grid_constant__ LeafInvArgs g) {
  extern __shared__ double inv_smem[];
  auto T = reinterpret_cast<double (*)[LEAF_INV_N + 1]>(inv_smem);
  auto S = reinterpret_cast<double (*)[LEAF_INV_N + 1]>(inv_smem + LEAF_INV_N * (LEAF_INV_N + 1));
  double* dinv = inv_smem + 2 * LEAF_INV_N * (LEAF_INV_N + 1);
  const int b = blockIdx.x, t = threadIdx.x, n = g.nl[b];
  const double* Ab = g.A + (int64_t)g.k[b] * (g.lda + 1);
  for (int idx = t; idx < n * n; idx += blockDim.x) {
    const int i = idx % n, j = idx / n;
    double v = 0.0;
    if (j <= i) {
      const int ri = g.upper ? n - 1 - i : i, rj = g.upper ? n - 1 - j : j;
      v = g.tA ? Ab[rj + (int64_t)ri * g.lda] : Ab[ri + (int64_t)rj * g.lda];
    }
    T[i][j] = v;
    S[i][j] = i == j ? 1.0 : 0.0;
  }
  __syncthreads();
  if (t < n) dinv[t] = g.unit ? 1.0 : 1.0 / T[t][t];
  __syncthreads();
  const int j = t >> 2, rg = t & 3;
  for (int i = 0; i < n; ++i) {
    double x = 0.0;
    if (j < n && i >= j) x = S[i][j] * dinv[i];
    __syncwarp();
    if (j < n && i >= j) {
      if (rg == (i & 3)) S[i][j] = x;
      for (int r = i + 1 + ((rg - i - 1) & 3); r < n; r += 4) S[r][j] -= T[r][i] * x;
    }
    __syncwarp();
  }
  __syncthreads();
  double* W = g.W + (int64_t)(g.first_slot + b) * LEAF_INV_N * LEAF_INV_N;
  for (int idx = t; idx < n * n; idx += blockDim.x) {
    const int i = idx % n, jj = idx / n;
    const double v = jj <= i ? S[i][jj] : 0.0;
    const int ri = g.upper ? n - 1 - i : i, rj = g.upper ? n - 1 - jj : jj;
    W[ri + (int64_t)rj * LEAF_INV_N] = v;
  }
}

// X := W X (side L, X n x m) or X W (side R, X m x n) for one leaf, W the
// leaf's FP64 inverse (n <= 64), in one kernel: each CTA takes 128
// right-hand sides (M of the MMA: D^T = X^T W^T), loads its block of X and
// W, scales every right-hand side and every row of W by a power of two,
// splits both into 7 BF16 digit slices in shared memory (nla_split7.cuh),
// multiplies the 28 slice pairs with p + q <= 6 on the tensor cores (one
// FP32 TMEM accumulator per weight p + q, exact: 7 x 64 x 2^14 < 2^24),
// combines the weights exactly in int64 and writes the result over X with one
// rounding.  Each CTA reads and writes only its own right-hand sides.
constexpr int LP_COLS = 128;                            // right-hand sides per CTA
constexpr int LP_THREADS = 512;                         // 16 warps: load, split, drain; one thread issues MMAs
constexpr int LP_A_BYTES = split7::SLICES * LP_COLS * 128;   // X^T slices: 128 rows x 64 K
constexpr int LP_B_BYTES = split7::SLICES * LEAF_INV_N * 128;  // W slices: 64 rows x 64 K
constexpr int LP_SMEM = LP_A_BYTES + LP_B_BYTES + 1024 + 8192;

// Shared memory of the leaf product kernels.  Thread t holds, for every
// product, rows k = 16 (t / 128) + u (u < 16) of right-hand side t % 128 and
// row t % 64 of the W operand at k = 8 (t / 64) + u (u < 8); the drain gives
// it output rows 16 (t / 128) + c of right-hand side t % 128, the same
// positions, so one product's result is the next one's right-hand sides
// without an exchange.
struct LpShared {
  uint8_t* sA;         // 7 slices of the right-hand sides: 128 rows x 64 K
  uint8_t* sB;         // 7 slices of W: 64 rows x 64 K
  int* xpart;          // [4][128] exponent-field maxima of the right-hand sides
  int* wpart;          // [8][64] of W's rows
  int* ex_s;           // [128] scale exponents of the right-hand sides
  int* ew_s;           // [64] of W's rows
  uint64_t* bar;       // MMA completion
  uint32_t* tmem_slot;
};

__device__ __forceinline__ LpShared lp_shared(uint8_t* raw) {
  LpShared s;
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(raw) + 1023) & ~uintptr_t(1023));
  s.sA = smem;
  s.sB = smem + LP_A_BYTES;
  s.xpart = reinterpret_cast<int*>(s.sB + LP_B_BYTES);
  s.wpart = s.xpart + 4 * LP_COLS;
  s.ex_s = s.wpart + 8 * LEAF_INV_N;
  s.ew_s = s.ex_s + LP_COLS;
  s.bar = reinterpret_cast<uint64_t*>(s.ew_s + LEAF_INV_N);
  s.tmem_slot = reinterpret_cast<uint32_t*>(s.bar + 1);
  return s;
}

// The scale exponents (per right-hand side and per row of W) and the 7
// digit slices of one product's operands, ending with the slices visible to
// the tensor cores.  Every thread of the CTA takes part.
__device__ __forceinline__ void lp_stage(const LpShared& s, const double (&vx)[16], const double (&vw)[8]) {
  using namespace split7;
  const int t = threadIdx.x;
  const int jr = t & (LP_COLS - 1), xp = t >> 7;
  const int wi = t & (LEAF_INV_N - 1), wp = t >> 6;
  int bx = 0, bw = 0;
#pragma unroll
  for (int u = 0; u < 16; ++u) bx = max(bx, exp_field(vx[u]));
#pragma unroll
  for (int u = 0; u < 8; ++u) bw = max(bw, exp_field(vw[u]));
  s.xpart[xp * LP_COLS + jr] = bx;
  s.wpart[wp * LEAF_INV_N + wi] = bw;
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  if (t < LP_COLS) {
    s.ex_s[t] =
        scale_exp(max(max(s.xpart[t], s.xpart[LP_COLS + t]), max(s.xpart[2 * LP_COLS + t], s.xpart[3 * LP_COLS + t])));
  } else if (t < LP_COLS + LEAF_INV_N) {
    const int i = t - LP_COLS;
    int m8 = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) m8 = max(m8, s.wpart[q * LEAF_INV_N + i]);
    s.ew_s[i] = scale_exp(m8);
  }
  __syncthreads();
  {
    const int ex = s.ex_s[jr], ew = s.ew_s[wi];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      long long y[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) y[u] = fixed56(vx[c * 8 + u], ex);
      store_chunks(s.sA, LP_COLS * 128, jr, xp * 2 + c, y);
    }
    long long y[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) y[u] = fixed56(vw[u], ew);
    store_chunks(s.sB, LEAF_INV_N * 128, wi, wp, y);
  }
  // The tensor cores read shared memory through the async proxy.
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
}

// The 28 slice pairs with p + q <= 6 (weight w = p + q into accumulator w,
// TMEM columns 64 w ..), issued by one thread, with their completion
// committed to s.bar.  W's slices lie one after another in shared memory and
// the accumulators side by side in TMEM, so slice p of the right-hand sides
// meets W's slices q = 0 .. 6 - p in MMAs as wide as N = 256 allows: rows
// 64 q of the stacked slices feed accumulator p + q.  That is 10 MMAs per
// 16-wide K step instead of 28, each reading the right-hand-side slice from
// shared memory once (the 28 narrow MMAs were bound by shared-memory reads).
// The accumulators hold exact integers, so the order of the sums is free.
__device__ __forceinline__ void lp_issue(const LpShared& s, uint32_t tmem) {
  using namespace split7;
  const uint32_t a0 = umma::smem_u32(s.sA), b0 = umma::smem_u32(s.sB);
#pragma unroll 1
  for (int p = 0; p < SLICES; ++p) {
    const int rows = LEAF_INV_N * (SLICES - p);
#pragma unroll 1
    for (int r0 = 0; r0 < rows; r0 += 256) {
      const int nn = min(256, rows - r0);
      const uint32_t idesc = umma::idesc_f16(LP_COLS, nn, true);
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)
        umma::mma_f16(tmem + (uint32_t)(p * LEAF_INV_N + r0), umma::desc_kmajor_sw128(a0 + p * LP_COLS * 128 + kk * 32),
                      umma::desc_kmajor_sw128(b0 + r0 * 128 + kk * 32), idesc, (p > 0 || kk > 0) ? 1u : 0u);
    }
  }
  umma::mma_commit(umma::smem_u32(s.bar));
}

// Waits for the products committed in phase `parity`, with one answer for
// the whole CTA.  After a wait that gave up, thread 0 lets the MMAs finish
// (a drain with the default limit) so that the tensor memory can be
// released.
__device__ __forceinline__ bool lp_wait(const LpShared& s, uint32_t parity, volatile int* abort, int* err,
                                        int site) {
  __syncwarp();
  bool ok = __all_sync(0xffffffffu, umma::mbar_wait(umma::smem_u32(s.bar), parity, abort, err, site));
  umma::fence_after_sync();
  ok = __syncthreads_and(ok ? 1 : 0) != 0;
  if (!ok && threadIdx.x == 0) umma::mbar_wait(umma::smem_u32(s.bar), parity, abort, err, site + 1, false);
  return ok;
}

// Drain: right-hand side t % 128 (the warp's TMEM lane quarter), output rows
// 16 (t / 128) + c.  One block of K: S = H 2^18 + round(L 2^-6), with
// H = sum_{w<4} T_w 2^(24 - 8 w) and L = sum_{4<=w<7} T_w 2^(48 - 8 w); the
// product is S 2^(e_x + e_w - 58).  L is rounded first and H 2^18 added as
// the exact integer sum_{w<4} T_w 2^(42 - 8 w), which keeps one int64 per
// element live.
__device__ __forceinline__ void lp_drain(uint32_t tmem, long long (&tot)[16]) {
  using namespace split7;
  const int warp = threadIdx.x >> 5;
  const uint32_t tq = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)((warp >> 2) * 16);
#pragma unroll
  for (int c = 0; c < 16; ++c) tot[c] = 0;
#pragma unroll
  for (int w = 4; w < SLICES; ++w) {
    uint32_t rr[16];
    umma::tmem_ld16(tq + (uint32_t)(w * LEAF_INV_N), rr);
#pragma unroll
    for (int c = 0; c < 16; ++c) tot[c] += (long long)__float2int_rn(__uint_as_float(rr[c])) << (48 - 8 * w);
  }
#pragma unroll
  for (int c = 0; c < 16; ++c) tot[c] = (tot[c] + (1ll << 5)) >> 6;
#pragma unroll
  for (int w = 0; w < 4; ++w) {
    uint32_t rr[16];
    umma::tmem_ld16(tq + (uint32_t)(w * LEAF_INV_N), rr);
#pragma unroll
    for (int c = 0; c < 16; ++c) tot[c] += (long long)__float2int_rn(__uint_as_float(rr[c])) << (42 - 8 * w);
  }
}

// One element of a product from its int64 sum and the operands' scale
// exponents (NaN when either operand held a non-finite value).
__device__ __forceinline__ double lp_value(long long tot, int ex, int ew) {
  using namespace split7;
  return ex == NONFINITE || ew == NONFINITE ? __longlong_as_double(0x7ff8000000000000ll)
                                            : scaled_i64_to_f64(tot, ex + ew - 58);
}

struct LeafProdArgs {
  const double* W;  // column-major, leading dimension LEAF_INV_N
  double* X;
  int64_t ldx;
  int64_t m;
  int n;
  int side_r;
  int* err;
};

__global__ void __launch_bounds__(LP_THREADS, 1) leaf_product_kernel(const LeafProdArgs a) {
  extern __shared__ uint8_t lp_smem_raw[];
  const LpShared s = lp_shared(lp_smem_raw);
  __shared__ volatile int s_abort;

  const int t = threadIdx.x, warp = t >> 5, n = a.n;
  const int64_t j0 = (int64_t)blockIdx.x * LP_COLS;
  // Element (k, j) of the right-hand sides (k < n, j < m) and (i, k) of the
  // W operand (W itself for side L, W^T for side R).
  auto xat = [&](int k, int64_t j) -> int64_t { return a.side_r ? j + (int64_t)k * a.ldx : k + j * a.ldx; };
  auto wat = [&](int i, int k) -> int { return a.side_r ? k + i * LEAF_INV_N : i + k * LEAF_INV_N; };

  if (t == 0) {
    s_abort = 0;
    umma::mbar_init(umma::smem_u32(s.bar), 1);
    umma::fence_barrier_init();
  }
  if (warp == 0) umma::tmem_alloc(umma::smem_u32(s.tmem_slot), 512);

  const int jr = t & (LP_COLS - 1), xp = t >> 7;
  const int wi = t & (LEAF_INV_N - 1), wp = t >> 6;
  const int64_t j = j0 + jr;
  double vx[16], vw[8];
#pragma unroll
  for (int u = 0; u < 16; ++u) {
    const int k = xp * 16 + u;
    vx[u] = k < n && j < a.m ? a.X[xat(k, j)] : 0.0;
  }
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int k = wp * 8 + u;
    vw[u] = wi < n && k < n ? a.W[wat(wi, k)] : 0.0;
  }
  lp_stage(s, vx, vw);
  const uint32_t tmem = *s.tmem_slot;
  if (t == 0) lp_issue(s, tmem);
  if (lp_wait(s, 0u, &s_abort, a.err, 41)) {
    long long tot[16];
    lp_drain(tmem, tot);
    const int ex = s.ex_s[jr];
    if (j < a.m) {
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        const int i = xp * 16 + c;
        if (i < n) a.X[xat(i, j)] = lp_value(tot[c], ex, s.ew_s[i]);
      }
    }
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    umma::fence_after_sync();
    umma::tmem_dealloc(tmem, 512);
  }
}

// Two sibling leaves of the recursion and the update between them in one
// kernel: for the node of n <= 128 rows whose halves f (solved first) and s
// are both leaves,
//     X_f := W_f X_f,   C := X_s - G X_f,   X_s := W_s C
// with G the node's off-diagonal block (A21 or A12 of the recursion's update,
// read through the caller's strides).  Each step is the exact 7-slice product
// of leaf_product_kernel, rounded once per element as in the separate
// launches (the update's result is X_s - round(G X_f)); X_f and C stay in
// registers between the steps, in the positions the next step loads them
// from.  This replaces a leaf launch, the update's staging, product and
// finishing launches and the second leaf launch of every such node.
struct LeafPairArgs {
  const double* Wf;  // inverses of the two leaves, column-major, leading dimension LEAF_INV_N
  const double* Ws;
  const double* G;   // G(i, k) = G[i * gsi + k * gsk], i < ns, k < nf
  int64_t gsi, gsk;
  double* Xf;        // the halves' right-hand sides: element (k, j) at k + j ldx (side L) or j + k ldx (side R)
  double* Xs;
  int64_t ldx;
  int64_t m;
  int nf, ns;
  int* err;
};

// Side L: a block of right-hand sides (rows k < 64 of the CTA's 128
// columns; column j at X + j ldx) passes through a shared-memory tile, so
// that global loads and stores run along the contiguous rows (a thread's own
// 16 rows of one column would touch 32 cache lines per warp instruction).
// Row r of the tile is right-hand side r, padded to LP_TP doubles.
constexpr int LP_TP = 65;
static_assert(LP_COLS * LP_TP * 8 <= LP_A_BYTES, "the staging tile lives in the slice buffer");

// Asynchronous copy of the block into the tile: warp w takes columns w + 16 q
// (q < 8), lane l rows l and l + 32; rows >= nk and columns >= m read as 0.
__device__ __forceinline__ void lp_tile_fetch(double* tile, const double* X, int64_t ldx, int64_t j0, int64_t m,
                                              int nk) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll 1
  for (int q = 0; q < 8; ++q) {
    const int r = warp + 16 * q;
    const int64_t j = j0 + r;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int k = lane + 32 * h;
      const bool in = j < m && k < nk;
      const double* src = in ? X + k + j * ldx : X;
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(umma::smem_u32(tile + r * LP_TP + k)),
                   "l"(src), "r"(in ? 8 : 0)
                   : "memory");
    }
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
}

__device__ __forceinline__ void lp_tile_arrived() {
  asm volatile("cp.async.wait_all;" ::: "memory");
  __syncthreads();
}

// Stores rows k < nk of the tile's columns j < m back to X (after a barrier
// that follows the tile's writes).
__device__ __forceinline__ void lp_tile_store(const double* tile, double* X, int64_t ldx, int64_t j0, int64_t m,
                                              int nk) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int r = warp + 16 * q;
    const int64_t j = j0 + r;
    if (j >= m) break;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int k = lane + 32 * h;
      if (k < nk) X[k + j * ldx] = tile[r * LP_TP + k];
    }
  }
}

template <bool SIDE_R>
__global__ void __launch_bounds__(LP_THREADS, 1) leaf_pair_kernel(const LeafPairArgs a) {
  extern __shared__ uint8_t lp_smem_raw[];
  const LpShared s = lp_shared(lp_smem_raw);
  __shared__ volatile int s_abort;

  const int t = threadIdx.x, warp = t >> 5;
  const int jr = t & (LP_COLS - 1), xp = t >> 7;
  const int wi = t & (LEAF_INV_N - 1), wp = t >> 6;
  const int64_t j0 = (int64_t)blockIdx.x * LP_COLS;
  const int64_t j = j0 + jr;
  const bool jin = j < a.m;
  // Side R: X(k, j) at j + k ldx, so a thread's loads and stores are already
  // coalesced across the warp (consecutive j); side L goes through `tile`.
  double* tile = reinterpret_cast<double*>(s.sA);
  double* trow = tile + jr * LP_TP + xp * 16;
  auto wat = [&](int i, int k) -> int { return SIDE_R ? k + i * LEAF_INV_N : i + k * LEAF_INV_N; };

  if (t == 0) {
    s_abort = 0;
    umma::mbar_init(umma::smem_u32(s.bar), 1);
    umma::fence_barrier_init();
  }
  if (warp == 0) umma::tmem_alloc(umma::smem_u32(s.tmem_slot), 512);

  // The first product's operands: X_f and W_f.
  double vx[16], vw[8];
  if constexpr (!SIDE_R) lp_tile_fetch(tile, a.Xf, a.ldx, j0, a.m, a.nf);
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int k = wp * 8 + u;
    vw[u] = wi < a.nf && k < a.nf ? a.Wf[wat(wi, k)] : 0.0;
  }
  if constexpr (!SIDE_R) {
    lp_tile_arrived();
#pragma unroll
    for (int u = 0; u < 16; ++u) vx[u] = trow[u];
  } else {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int k = xp * 16 + u;
      vx[u] = k < a.nf && jin ? a.Xf[j + k * a.ldx] : 0.0;
    }
  }
  uint32_t tmem = 0;

  // Step 0: X_f := W_f X_f;  step 1: C := X_s - G X_f;  step 2: X_s := W_s C.
  // One body for the three steps, so that its code is fetched once and hits
  // the instruction cache in the later steps.
#pragma unroll 1
  for (int st = 0; st < 3; ++st) {
    lp_stage(s, vx, vw);
    if (st == 0) tmem = *s.tmem_slot;
    if (t == 0) lp_issue(s, tmem);
    if (st == 0) {
      // G's block, in flight during the products.
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int k = wp * 8 + u;
        vw[u] = wi < a.ns && k < a.nf ? a.G[wi * a.gsi + k * a.gsk] : 0.0;
      }
    } else if (st == 1 && !SIDE_R) {
      // X_s's block into L2 while the products run (one 128-byte line per
      // thread); it comes into the tile once they are done.
      const int r = t >> 2, k = (t & 3) * 16;
      if (j0 + r < a.m && k < a.ns) asm volatile("prefetch.global.L2 [%0];" ::"l"(a.Xs + k + (j0 + r) * a.ldx));
    }
    if (!lp_wait(s, (uint32_t)(st & 1), &s_abort, a.err, 43)) break;
    if (st == 1 && !SIDE_R) lp_tile_fetch(tile, a.Xs, a.ldx, j0, a.m, a.ns);
    long long tot[16];
    lp_drain(tmem, tot);
    const int ex = s.ex_s[jr];
    const int nout = st == 0 ? a.nf : a.ns;
    if (st == 1 && !SIDE_R) lp_tile_arrived();
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      const int i = xp * 16 + c;
      double v = 0.0;
      if (i < nout) {
        v = lp_value(tot[c], ex, s.ew_s[i]);
        if (st == 1) v = (SIDE_R ? (jin ? a.Xs[j + i * a.ldx] : 0.0) : trow[c]) - v;
      }
      vx[c] = v;
    }
    if (st != 1) {
      double* Xo = st == 0 ? a.Xf : a.Xs;
      if constexpr (!SIDE_R) {
#pragma unroll
        for (int c = 0; c < 16; ++c) trow[c] = vx[c];
        __syncthreads();
        lp_tile_store(tile, Xo, a.ldx, j0, a.m, nout);
      } else if (jin) {
#pragma unroll
        for (int c = 0; c < 16; ++c)
          if (xp * 16 + c < nout) Xo[j + (xp * 16 + c) * a.ldx] = vx[c];
      }
    } else {
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int k = wp * 8 + u;
        vw[u] = wi < a.ns && k < a.ns ? a.Ws[wat(wi, k)] : 0.0;
      }
    }
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    umma::fence_after_sync();
    umma::tmem_dealloc(tmem, 512);
  }
}

std::mutex g_inv_mu;
std::unordered_map<uint64_t, Buf> g_inv_bufs;

// The inverses' slots, one buffer per (device, stream), grown on demand.
int inverse_buffer(cudaStream_t s, size_t bytes, double** out) {
  int dev = 0;
  cudaGetDevice(&dev);
  const uint64_t key = ((uint64_t)(uint32_t)dev << 48) ^ (uint64_t)reinterpret_cast<uintptr_t>(s);
  std::lock_guard<std::mutex> lk(g_inv_mu);
  Buf& b = g_inv_bufs[key];
  if (b.n < bytes) {
    if (b.p) cudaFreeAsync(b.p, s);
    b.p = nullptr;
    b.n = 0;
    cudaError_t e = cudaMallocAsync(&b.p, bytes, s);
    if (e != cudaSuccess) {
      b.p = nullptr;
      return cuda_status(e, "leaf inverse buffer");
    }
    b.n = bytes;
  }
  *out = static_cast<double*>(b.p);
  return NLA_OK;
}

void collect_leaves(int64_t k, int64_t n, int64_t thr, std::vector<int64_t>* ks, std::vector<int>* ns) {
  if (n <= thr) {
    ks->push_back(k);
    ns->push_back((int)n);
    return;
  }
  const int64_t mid = split_point(n);
  collect_leaves(k, mid, thr, ks, ns);
  collect_leaves(k + mid, n - mid, thr, ks, ns);
}

int launch_inverses(const RecPlan& c, const double* A, int64_t lda, int tA, const std::vector<int64_t>& ks,
                    const std::vector<int>& ns, double* W, int first) {
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    attr = cudaFuncSetAttribute(leaf_inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, INV_SMEM);
  });
  if (attr != cudaSuccess) return cuda_status(attr, "cudaFuncSetAttribute(leaf_inverse_kernel)");
  TraceScope trace(NLA_K_LEAF_SOLVE, c.s, 0.0, 0.0);
  for (size_t j0 = 0; j0 < ks.size(); j0 += INV_MAX) {
    LeafInvArgs g{};
    g.A = A;
    g.lda = lda;
    g.tA = tA;
    g.upper = c.uplo == 'U';
    g.unit = c.unit ? 1 : 0;
    g.W = W;
    g.first_slot = first + (int)j0;
    g.count = (int)std::min<size_t>(INV_MAX, ks.size() - j0);
    for (int j = 0; j < g.count; ++j) {
      g.k[j] = (int)ks[j0 + j];
      g.nl[j] = ns[j0 + j];
    }
    leaf_inverse_kernel<<<(unsigned)g.count, 256, INV_SMEM, c.s>>>(g);
    NLA_CHECK_LAUNCH("leaf_inverse_kernel");
    if (j0 > 0) trace_kernels(1);
  }
  return NLA_OK;
}

}  // namespace

bool leaf_inverses_wanted(const RecPlan& c) {
  if (c.mode != GEMM_MIXED || c.S != EXACT_SLICES || !c.bf16 || c.func != 'S' || c.dtype != NLA_F64) return false;
  if (c.threshold > LEAF_INV_N) return false;
  const char* v = std::getenv("NLA_MIXED_INV_LEAF");
  return !(v && v[0] == '0');
}

int leaf_inverses_upfront(const RecPlan& c, const Mat& A, int64_t n, LeafInverses* out) {
  out->a_base = static_cast<const double*>(A.p);
  out->lda = A.ld;
  out->err = device_error_word();
  if (!out->err) return fail(NLA_ERR_UNSUPPORTED, "leaf inverses: no device error word");
  out->k.clear();
  std::vector<int> ns;
  collect_leaves(0, n, c.threshold, &out->k, &ns);
  if (n > INT32_MAX) return fail(NLA_ERR_UNSUPPORTED, "leaf inverses: n too large");
  NLA_TRY(inverse_buffer(c.s, out->k.size() * LEAF_INV_N * LEAF_INV_N * sizeof(double), &out->w));
  return launch_inverses(c, out->a_base, A.ld, A.t, out->k, ns, out->w, 0);
}

namespace {

// Slot of the inverse of the leaf whose diagonal block starts at row k of the
// solve's A.
int leaf_slot(const LeafInverses& L, int64_t k, int64_t* slot) {
  const auto it = std::lower_bound(L.k.begin(), L.k.end(), k);
  if (L.a_base == nullptr || it == L.k.end() || *it != k)
    return fail(NLA_ERR_ARG, "leaf inverses: no inverse for this block");
  *slot = it - L.k.begin();
  return NLA_OK;
}

// The shared-memory opt-in of one leaf product kernel, once per process
// (one flag per kernel: the template argument is the kernel itself).
template <auto Kernel>
int allow_smem(const char* name) {
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] { attr = cudaFuncSetAttribute(Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, LP_SMEM); });
  return attr == cudaSuccess ? NLA_OK : cuda_status(attr, name);
}

}  // namespace

int leaf_inverse_apply(const RecPlan& c, const Mat& A, int64_t n, const Mat& B) {
  if (n <= 0 || c.m <= 0) return NLA_OK;
  const LeafInverses& L = *c.inv;
  int64_t slot = 0;
  NLA_TRY(leaf_slot(L, (static_cast<const double*>(A.p) - L.a_base) / (L.lda + 1), &slot));
  // X := inv(T) X  (side L)  or  X inv(T)  (side R), one kernel.
  NLA_TRY(allow_smem<leaf_product_kernel>("cudaFuncSetAttribute(leaf_product_kernel)"));
  if (B.t) return fail(NLA_ERR_UNSUPPORTED, "leaf product: transposed B view");
  LeafProdArgs g{L.w + slot * LEAF_INV_N * LEAF_INV_N, static_cast<double*>(B.p), B.ld, c.m, (int)n,
                 c.side == 'R' ? 1 : 0, L.err};
  const int64_t grid = (c.m + LP_COLS - 1) / LP_COLS;
  if (grid > 2147483647LL) return fail(NLA_ERR_UNSUPPORTED, "leaf product: too many right-hand sides");
  TraceScope trace(NLA_K_LEAF_SOLVE, c.s, 2.0 * (double)n * n * (double)c.m, 16.0 * (double)n * (double)c.m);
  leaf_product_kernel<<<(unsigned)grid, LP_THREADS, LP_SMEM, c.s>>>(g);
  NLA_CHECK_LAUNCH("leaf_product_kernel");
  return NLA_OK;
}

bool leaf_pair_wanted(const RecPlan& c, int64_t n) {
  if (!c.inv || c.func != 'S' || n <= c.threshold) return false;
  const int64_t mid = split_point(n);
  if (mid > c.threshold || n - mid > c.threshold) return false;
  const char* v = std::getenv("NLA_LEAF_PAIR");
  return !(v && v[0] == '0');
}

int leaf_pair_apply(const RecPlan& c, const Mat& A, int64_t n, const Mat& B) {
  if (c.m <= 0) return NLA_OK;
  const LeafInverses& L = *c.inv;
  if (B.t) return fail(NLA_ERR_UNSUPPORTED, "leaf pair: transposed B view");
  // The halves in the recursion's order (src/rectrxm.jl:104-124): f is solved
  // first, then s is updated from it and solved.
  const int64_t mid = split_point(n), rem = n - mid;
  const bool fwd = rec_forward(c), R = c.side == 'R';
  const int64_t of = fwd ? 0 : mid, nf = fwd ? mid : rem, os = fwd ? mid : 0, ns = fwd ? rem : mid;
  const double* Ap = static_cast<const double*>(A.p);
  const int64_t k0 = (Ap - L.a_base) / (L.lda + 1);
  int64_t slot_f = 0, slot_s = 0;
  NLA_TRY(leaf_slot(L, k0 + of, &slot_f));
  NLA_TRY(leaf_slot(L, k0 + os, &slot_s));
  NLA_TRY(R ? allow_smem<leaf_pair_kernel<true>>("cudaFuncSetAttribute(leaf_pair_kernel)")
            : allow_smem<leaf_pair_kernel<false>>("cudaFuncSetAttribute(leaf_pair_kernel)"));
  LeafPairArgs g{};
  g.Wf = L.w + slot_f * LEAF_INV_N * LEAF_INV_N;
  g.Ws = L.w + slot_s * LEAF_INV_N * LEAF_INV_N;
  // G(i, k) = op(A)(os + i, of + k) for side L (B_s -= A_sf X_f) and
  // op(A)(of + k, os + i) for side R (X_s -= X_f A_fs), read through A's view.
  if (!R) {
    g.G = Ap + mat_off(os, of, A.ld, A.t);
    g.gsi = A.t ? A.ld : 1;
    g.gsk = A.t ? 1 : A.ld;
  } else {
    g.G = Ap + mat_off(of, os, A.ld, A.t);
    g.gsi = A.t ? 1 : A.ld;
    g.gsk = A.t ? A.ld : 1;
  }
  double* Bp = static_cast<double*>(B.p);
  g.Xf = Bp + (R ? of * B.ld : of);
  g.Xs = Bp + (R ? os * B.ld : os);
  g.ldx = B.ld;
  g.m = c.m;
  g.nf = (int)nf;
  g.ns = (int)ns;
  g.err = L.err;
  const int64_t grid = (c.m + LP_COLS - 1) / LP_COLS;
  if (grid > 2147483647LL) return fail(NLA_ERR_UNSUPPORTED, "leaf pair: too many right-hand sides");
  TraceScope trace(NLA_K_LEAF_SOLVE, c.s, 2.0 * (double)(nf * nf + ns * ns + nf * ns) * (double)c.m,
                   8.0 * (double)(2 * n + ns) * (double)c.m);
  if (R) leaf_pair_kernel<true><<<(unsigned)grid, LP_THREADS, LP_SMEM, c.s>>>(g);
  else leaf_pair_kernel<false><<<(unsigned)grid, LP_THREADS, LP_SMEM, c.s>>>(g);
  NLA_CHECK_LAUNCH("leaf_pair_kernel");
  return NLA_OK;
}

// Stage the strict triangle of op(A) as the row operand of the residual
// product: op(A) itself for side L, op(A)^T for side R.
int stage_triangle(const Mat& Am, int64_t n, char side, char uplo, void* buf, Staged* out, cudaStream_t s) {
  if (side == 'L') return stage_operand(Am, n, n, NLA_F64, EXACT_SLICES, true, uplo == 'L' ? 3 : 4, buf, out, s);
  return stage_operand(transposed(Am), n, n, NLA_F64, EXACT_SLICES, true, uplo == 'L' ? 4 : 3, buf, out, s);
}

// R -= op(A) X (side L) or X op(A) (side R): exact slice products for the
// strict triangle (As, staged by stage_triangle); the diagonal term and the
// subtraction are folded into the exact kernel's epilogue (one rounding).
int split_residual(const Mat& Am, const Staged& As, char side, int64_t n, int64_t m, const Mat& Xm, const Mat& Rm,
                   void* xbuf, Staged* Xs, cudaStream_t s) {
  // The epilogue subtracts the exact strict-triangle product and the FP64
  // diagonal term from R (= alpha*B on entry) and rounds once.
  const ResidualTerm term{static_cast<const double*>(Xm.p), Xm.ld, static_cast<const double*>(Am.p), Am.ld + 1};
  if (side == 'L') {  // op(A) (n x n) times X (n x m): B-operand rows are X's columns
    NLA_TRY(stage_operand(transposed(Xm), m, n, NLA_F64, EXACT_SLICES, true, 0, xbuf, Xs, s, false));
    return launch_exact_gemm(As, *Xs, -1.0, Rm, false, s, &term);
  }
  // (X op(A))^T = op(A)^T X^T: B-operand rows are X's rows; written transposed
  NLA_TRY(stage_operand(Xm, m, n, NLA_F64, EXACT_SLICES, true, 0, xbuf, Xs, s, false));
  return launch_exact_gemm(As, *Xs, -1.0, Rm, true, s, &term);
}

int mixed_plan(char side, char uplo, char trans, char func, int64_t n, int64_t m, const void* A, int64_t lda,
               const void* B, int64_t ldb, const nla_mixed_opts* o, cudaStream_t s, RecPlan* c, int* a_trans,
               nla_mixed_opts* out) {
  NLA_TRY(check_flags(side, uplo, trans, func, NLA_F64));
  if (n < 0 || m < 0) return fail(NLA_ERR_ARG, "n and m must be non-negative");
  NLA_TRY(check_matrix("A", A, n, n, lda));
  const int64_t rows = side == 'L' ? n : m, cols = side == 'L' ? m : n;
  NLA_TRY(check_matrix("B", B, rows, cols, ldb));
  nla_mixed_opts opts{NLA_LOWP_BF16, 3, 2, NLA_RESIDUAL_SPLIT, 0, nullptr};
  if (o) opts = *o;
  if (opts.lowp != NLA_LOWP_BF16 && opts.lowp != NLA_LOWP_F16) return fail(NLA_ERR_ARG, "lowp must be BF16 or F16");
  if (!(opts.split_terms >= 1 && opts.split_terms <= 3) && opts.split_terms != EXACT_SLICES)
    return fail(NLA_ERR_ARG, "split_terms must be 1, 2, 3 or 7");
  if (opts.split_terms == EXACT_SLICES && opts.lowp != NLA_LOWP_BF16)
    return fail(NLA_ERR_ARG, "exact (7-term) updates use BF16 slices");
  if (opts.sweeps < 0 || opts.sweeps > 8) return fail(NLA_ERR_ARG, "sweeps must be in 0..8");
  if (opts.residual != NLA_RESIDUAL_FP64 && opts.residual != NLA_RESIDUAL_SPLIT)
    return fail(NLA_ERR_ARG, "unknown residual mode");
  *out = opts;
  *a_trans = 0;
  if (trans == 'T' || trans == 'C') {  // src/rectrxm.jl:56-59
    *a_trans = 1;
    uplo = uplo == 'L' ? 'U' : 'L';
  }
  *c = RecPlan{func, side, uplo, NLA_F64, m, opts.cutoff > 0 ? (opts.cutoff > 1024 ? 1024 : opts.cutoff)
                                                             : default_mixed_cutoff(),
               s, GEMM_MIXED, opts.split_terms, opts.lowp == NLA_LOWP_BF16};
  if (n == 0 || m == 0) return NLA_OK;
  // Size the staging workspace once for the largest update (the top split).
  const int64_t mid = split_point(n), rem = n - mid;
  const int64_t big = mid > rem ? mid : rem;
  void* ws = nullptr;
  if (n > c->threshold) NLA_TRY(workspace_get(s, sliced_workspace_bytes(big, m, big, opts.split_terms), &ws));
  return NLA_OK;
}

int trxm_mixed_impl(char side, char uplo, char trans, double alpha, char func, int64_t n, int64_t m,
                    const double* A, int64_t lda, double* B, int64_t ldb, const nla_mixed_opts* o,
                    cudaStream_t s, bool unit) {
  RecPlan mixed{};
  nla_mixed_opts opts{};
  int at = 0;
  NLA_TRY(mixed_plan(side, uplo, trans, func, n, m, A, lda, B, ldb, o, s, &mixed, &at, &opts));
  // A unit diagonal reaches only the FP64 diagonal blocks (the updates never
  // read the diagonal); the refinement's residual would need it too.
  if (unit && func == 'S' && opts.sweeps > 0)
    return fail(NLA_ERR_UNSUPPORTED, "unit-diagonal mixed solves take no refinement sweeps");
  mixed.unit = unit;
  if (n == 0 || m == 0) return NLA_OK;
  uplo = mixed.uplo;
  const int64_t rows = side == 'L' ? n : m, cols = side == 'L' ? m : n;
  const Mat Am{const_cast<double*>(A), lda, at};
  const Mat Bm{B, ldb, 0};

  if (func == 'M') {
    NLA_TRY(recurse(mixed, Am, n, Bm));
    return launch_scale(NLA_F64, rows, cols, alpha, Bm, s);  // src/rectrxm.jl:72
  }
  LeafInverses inv;
  if (leaf_inverses_wanted(mixed)) {
    NLA_TRY(leaf_inverses_upfront(mixed, Am, n, &inv));
    mixed.inv = &inv;
  }

  NLA_TRY(launch_scale(NLA_F64, rows, cols, alpha, Bm, s));  // src/rectrxm.jl:64
  if (opts.sweeps == 0) return recurse(mixed, Am, n, Bm);

  // Refinement needs alpha*B (B0), a residual/correction buffer (R), two
  // device words for the correction norms and, for the split residual, op(A)
  // staged once (it does not change between sweeps) and X staged per sweep.
  const size_t elems = (size_t)rows * (size_t)cols;
  const bool split = opts.residual == NLA_RESIDUAL_SPLIT;
  const size_t a_stage = split ? staged_bytes(n, n, EXACT_SLICES) : 0;
  const size_t x_stage = split ? staged_bytes(m, n, EXACT_SLICES) : 0;
  void* buf = nullptr;
  NLA_TRY(refine_buffers(s, 2 * elems * sizeof(double) + 2048 + a_stage + x_stage, &buf));
  double* B0 = static_cast<double*>(buf);
  double* R = B0 + elems;
  unsigned long long* amax = reinterpret_cast<unsigned long long*>(R + elems);
  uint8_t* stage_base = reinterpret_cast<uint8_t*>(buf) + ((2 * elems * sizeof(double) + 256 + 1023) & ~(size_t)1023);
  const unsigned grid = grid_for((int64_t)elems);
  {
    TraceScope t(NLA_K_RESIDUAL, s, 0.0, 16.0 * (double)elems);
    copy_kernel<<<grid, 256, 0, s>>>(rows, cols, B, ldb, B0, rows);
    NLA_CHECK_LAUNCH("copy_kernel");
  }
  NLA_TRY(recurse(mixed, Am, n, Bm));  // X0

  // op(A) as the left operand (side L: op(A) X) or the right one (side R:
  // X op(A), staged as op(A)^T); only its triangle is staged.
  // The strict triangle is staged (its rows then carry no diagonal, whose
  // size would coarsen the row scale); the diagonal term is applied in FP64.
  Staged As{}, Xs{};
  if (split) NLA_TRY(stage_triangle(Am, n, side, uplo, stage_base, &As, s));
  RecPlan resid{'M', side, uplo, NLA_F64, m, 128, s, GEMM_PLAIN, 1, false};
  Mat Rm{R, rows, 0};
  for (int k = 0; k < opts.sweeps; ++k) {
    if (split) {
      {
        TraceScope t(NLA_K_RESIDUAL, s, 0.0, 16.0 * (double)elems);
        copy_kernel<<<grid, 256, 0, s>>>(rows, cols, B0, rows, R, rows);
        NLA_CHECK_LAUNCH("copy_kernel");
      }
      NLA_TRY(split_residual(Am, As, side, n, m, Bm, Rm, stage_base + a_stage, &Xs, s));
    } else {
      {
        TraceScope t(NLA_K_RESIDUAL, s, 0.0, 16.0 * (double)elems);
        copy_kernel<<<grid, 256, 0, s>>>(rows, cols, B, ldb, R, rows);
        NLA_CHECK_LAUNCH("copy_kernel");
      }
      NLA_TRY(recurse(resid, Am, n, Rm));  // R = op(A) X (or X op(A)) on the FP64 pipe
      {
        TraceScope t(NLA_K_RESIDUAL, s, (double)elems, 24.0 * (double)elems);
        residual_kernel<<<grid, 256, 0, s>>>(rows, cols, B0, rows, R, rows);
        NLA_CHECK_LAUNCH("residual_kernel");
      }
    }
    NLA_TRY(recurse(mixed, Am, n, Rm));  // D
    {
      TraceScope t(NLA_K_RESIDUAL, s, (double)elems, 24.0 * (double)elems);
      if (opts.corr_out) cudaMemsetAsync(amax, 0, 2 * sizeof(unsigned long long), s);
      correct_kernel<<<grid, 256, 0, s>>>(rows, cols, R, rows, B, ldb, opts.corr_out ? amax : nullptr);
      NLA_CHECK_LAUNCH("correct_kernel");
    }
    if (opts.corr_out) {
      unsigned long long h[2] = {0, 0};
      cudaError_t e = cudaMemcpyAsync(h, amax, sizeof(h), cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return cuda_status(e, "correction norms");
      const double md = __builtin_bit_cast(double, h[0]), mx = __builtin_bit_cast(double, h[1]);
      opts.corr_out[k] = mx > 0 ? md / mx : md;
    }
  }
  return NLA_OK;
}

// R = alpha*B - op(A) X (side L) or alpha*B - X op(A) (side R), FP64-accurate.
int residual_impl(char side, char uplo, char trans, double alpha, int64_t n, int64_t m, const double* A, int64_t lda,
                  const double* X, int64_t ldx, const double* B, int64_t ldb, double* R, int64_t ldr, int mode,
                  cudaStream_t s) {
  NLA_TRY(check_flags(side, uplo, trans, 'M', NLA_F64));
  if (n < 0 || m < 0) return fail(NLA_ERR_ARG, "n and m must be non-negative");
  const int64_t rows = side == 'L' ? n : m, cols = side == 'L' ? m : n;
  NLA_TRY(check_matrix("A", A, n, n, lda));
  NLA_TRY(check_matrix("X", X, rows, cols, ldx));
  NLA_TRY(check_matrix("B", B, rows, cols, ldb));
  NLA_TRY(check_matrix("R", R, rows, cols, ldr));
  if (mode != NLA_RESIDUAL_FP64 && mode != NLA_RESIDUAL_SPLIT && mode != NLA_RESIDUAL_DD)
    return fail(NLA_ERR_ARG, "unknown residual mode");
  if (rows == 0 || cols == 0) return NLA_OK;
  Mat Am{const_cast<double*>(A), lda, 0};
  if (trans == 'T' || trans == 'C') {
    Am.t = 1;
    uplo = uplo == 'L' ? 'U' : 'L';
  }
  const Mat Xm{const_cast<double*>(X), ldx, 0}, Rm{R, ldr, 0};
  const size_t elems = (size_t)rows * (size_t)cols;
  const unsigned grid = grid_for((int64_t)elems);
  if (mode == NLA_RESIDUAL_DD) {
    TraceScope t(NLA_K_RESIDUAL, s, 2.0 * (double)n * (double)elems / 2.0, 8.0 * (double)elems * 4.0);
    dd_residual_kernel<<<grid_for((int64_t)elems), 256, 0, s>>>(rows, cols, n, A, lda, Am.t, uplo == 'L',
                                                                side == 'L', X, ldx, B, ldb, alpha, R, ldr);
    NLA_CHECK_LAUNCH("dd_residual_kernel");
    return NLA_OK;
  }
  if (mode == NLA_RESIDUAL_SPLIT) {
    const size_t a_stage = staged_bytes(n, n, EXACT_SLICES), x_stage = staged_bytes(m, n, EXACT_SLICES);
    void* buf = nullptr;
    NLA_TRY(refine_buffers(s, a_stage + x_stage + 1024, &buf));
    uint8_t* base = static_cast<uint8_t*>(buf);
    copy_kernel<<<grid, 256, 0, s>>>(rows, cols, B, ldb, R, ldr);
    NLA_CHECK_LAUNCH("copy_kernel");
    NLA_TRY(launch_scale(NLA_F64, rows, cols, alpha, Rm, s));
    Staged As{}, Xs{};
    NLA_TRY(stage_triangle(Am, n, side, uplo, base, &As, s));
    return split_residual(Am, As, side, n, m, Xm, Rm, base + a_stage, &Xs, s);
  }
  // FP64 pipe: R = op(A) X by the plain recursion, then R = alpha*B - R.
  void* buf = nullptr;
  NLA_TRY(refine_buffers(s, elems * sizeof(double), &buf));
  double* B0 = static_cast<double*>(buf);
  copy_kernel<<<grid, 256, 0, s>>>(rows, cols, B, ldb, B0, rows);
  copy_kernel<<<grid, 256, 0, s>>>(rows, cols, X, ldx, R, ldr);
  NLA_CHECK_LAUNCH("copy_kernel");
  const Mat B0m{B0, rows, 0};
  NLA_TRY(launch_scale(NLA_F64, rows, cols, alpha, B0m, s));
  RecPlan resid{'M', side, uplo, NLA_F64, m, 128, s, GEMM_PLAIN, 1, false};
  NLA_TRY(recurse(resid, Am, n, Rm));
  residual_kernel<<<grid, 256, 0, s>>>(rows, cols, B0, rows, R, ldr);
  NLA_CHECK_LAUNCH("residual_kernel");
  return NLA_OK;
}

}  // namespace nla

using namespace nla;

extern "C" {

int nla_trxm_mixed(char side, char uplo, char trans, double alpha, char func, int64_t n, int64_t m,
                   const double* A, int64_t lda, double* B, int64_t ldb, const nla_mixed_opts* opts, void* stream) {
  clear_error();
  return trxm_mixed_impl(side, uplo, trans, alpha, func, n, m, A, lda, B, ldb, opts, (cudaStream_t)stream);
}

int nla_trxm_mixed_diag(char side, char uplo, char trans, char diag, double alpha, char func, int64_t n, int64_t m,
                        const double* A, int64_t lda, double* B, int64_t ldb, const nla_mixed_opts* opts,
                        void* stream) {
  clear_error();
  if (diag != 'N' && diag != 'U') return fail(NLA_ERR_ARG, std::string("diag must be 'N' or 'U', got '") + diag + "'");
  return trxm_mixed_impl(side, uplo, trans, alpha, func, n, m, A, lda, B, ldb, opts, (cudaStream_t)stream,
                         diag == 'U');
}

int nla_gemm_update_mixed(int trans1, int trans2, int64_t N, int64_t R, int64_t M, double alpha, const double* in1,
                          int64_t ld1, const double* in2, int64_t ld2, double* out, int64_t ldo, int lowp,
                          int split_terms, void* stream) {
  clear_error();
  if (N < 0 || R < 0 || M < 0) return fail(NLA_ERR_ARG, "N, R and M must be non-negative");
  if (lowp != NLA_LOWP_BF16 && lowp != NLA_LOWP_F16) return fail(NLA_ERR_ARG, "lowp must be BF16 or F16");
  if (!(split_terms >= 1 && split_terms <= 3) && split_terms != EXACT_SLICES)
    return fail(NLA_ERR_ARG, "split_terms must be 1, 2, 3 or 7");
  NLA_TRY(check_matrix("in1", in1, trans1 ? R : N, trans1 ? N : R, ld1));
  NLA_TRY(check_matrix("in2", in2, trans2 ? M : R, trans2 ? R : M, ld2));
  NLA_TRY(check_matrix("out", out, N, M, ldo));
  Mat A{const_cast<double*>(in1), ld1, trans1 ? 1 : 0};
  Mat B{const_cast<double*>(in2), ld2, trans2 ? 1 : 0};
  Mat C{out, ldo, 0};
  return launch_sliced_gemm(N, M, R, alpha, A, B, C, NLA_F64, NLA_F64, split_terms, lowp == NLA_LOWP_BF16, nullptr,
                            0, (cudaStream_t)stream);
}

int nla_trxm_residual(char side, char uplo, char trans, double alpha, int64_t n, int64_t m, const double* A,
                      int64_t lda, const double* X, int64_t ldx, const double* B, int64_t ldb, double* R,
                      int64_t ldr, int residual, void* stream) {
  clear_error();
  return residual_impl(side, uplo, trans, alpha, n, m, A, lda, X, ldx, B, ldb, R, ldr, residual,
                       (cudaStream_t)stream);
}

int nla_device_status(void* stream) {
  clear_error();
  return device_status((cudaStream_t)stream);
}

int nla_set_wait_limit_ns(uint64_t ns) {
  clear_error();
  return set_wait_limit(ns);
}

}  // extern "C"
