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
// rounded once per element.  (X + (inv(T) - I) X, which needs no overwrite,
// loses digits to cancellation when T's diagonal is large: x ~ b / d from
// b - (1 - 1/d) b.)
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
  using namespace split7;
  extern __shared__ uint8_t lp_smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(lp_smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* sA = smem;
  uint8_t* sB = smem + LP_A_BYTES;
  int* xpart = reinterpret_cast<int*>(sB + LP_B_BYTES);  // [4][128] exponent-field maxima of X
  int* wpart = xpart + 4 * LP_COLS;                        // [8][64] of W
  int* ex_s = wpart + 8 * LEAF_INV_N;                      // [128] scale exponents of the right-hand sides
  int* ew_s = ex_s + LP_COLS;                              // [64] of W's rows
  uint64_t* mma_bar = reinterpret_cast<uint64_t*>(ew_s + LEAF_INV_N);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mma_bar + 1);
  __shared__ volatile int s_abort;

  const int t = threadIdx.x, warp = t >> 5, lane = t & 31, n = a.n;
  const int64_t j0 = (int64_t)blockIdx.x * LP_COLS;
  // Element (k, j) of the right-hand sides (k < n, j < m) and (i, k) of the
  // W operand (W itself for side L, W^T for side R).
  auto xat = [&](int k, int64_t j) -> int64_t { return a.side_r ? j + (int64_t)k * a.ldx : k + j * a.ldx; };
  auto wat = [&](int i, int k) -> int { return a.side_r ? k + i * LEAF_INV_N : i + k * LEAF_INV_N; };

  if (t == 0) {
    s_abort = 0;
    umma::mbar_init(umma::smem_u32(mma_bar), 1);
    umma::fence_barrier_init();
  }
  if (warp == 0) umma::tmem_alloc(umma::smem_u32(tmem_slot), 512);

  // Loads: right-hand side jr = t % 128 with k = 16 (t / 128) .. + 16; row
  // i = t % 64 of W with k = 8 (t / 64) .. + 8.
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
  int bx = 0, bw = 0;
#pragma unroll
  for (int u = 0; u < 16; ++u) bx = max(bx, exp_field(vx[u]));
#pragma unroll
  for (int u = 0; u < 8; ++u) bw = max(bw, exp_field(vw[u]));
  xpart[xp * LP_COLS + jr] = bx;
  wpart[wp * LEAF_INV_N + wi] = bw;
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  if (t < LP_COLS) {
    ex_s[t] = scale_exp(max(max(xpart[t], xpart[LP_COLS + t]), max(xpart[2 * LP_COLS + t], xpart[3 * LP_COLS + t])));
  } else if (t < LP_COLS + LEAF_INV_N) {
    const int i = t - LP_COLS;
    int m8 = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) m8 = max(m8, wpart[q * LEAF_INV_N + i]);
    ew_s[i] = scale_exp(m8);
  }
  __syncthreads();
  {
    const int ex = ex_s[jr], ew = ew_s[wi];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      long long y[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) y[u] = fixed56(vx[c * 8 + u], ex);
      store_chunks(sA, LP_COLS * 128, jr, xp * 2 + c, y);
    }
    long long y[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) y[u] = fixed56(vw[u], ew);
    store_chunks(sB, LEAF_INV_N * 128, wi, wp, y);
  }
  // The tensor cores read shared memory through the async proxy.
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  if (t == 0) {
    const uint32_t idesc = umma::idesc_f16(LP_COLS, LEAF_INV_N, true);
    const uint32_t a0 = umma::smem_u32(sA), b0 = umma::smem_u32(sB);
#pragma unroll 1
    for (int w = 0; w < SLICES; ++w)
      for (int p = 0; p <= w; ++p) {
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
          umma::mma_f16(tmem + (uint32_t)(w * LEAF_INV_N), umma::desc_kmajor_sw128(a0 + p * LP_COLS * 128 + kk * 32),
                        umma::desc_kmajor_sw128(b0 + (w - p) * LEAF_INV_N * 128 + kk * 32), idesc,
                        (p > 0 || kk > 0) ? 1u : 0u);
      }
    umma::mma_commit(umma::smem_u32(mma_bar));
  }
  __syncwarp();
  bool ok = __all_sync(0xffffffffu, umma::mbar_wait(umma::smem_u32(mma_bar), 0u, &s_abort, a.err, 41));
  umma::fence_after_sync();
  if (!ok && t == 0) {
    // Let the MMAs finish (a drain with the default limit) before the tensor
    // memory is released.
    umma::mbar_wait(umma::smem_u32(mma_bar), 0u, &s_abort, a.err, 42, false);
  }
  if (ok) {
    // Drain: right-hand side q * 32 + lane (the warp's TMEM lane quarter),
    // output rows h * 16 .. + 16.  One block of K: S = H 2^18 + round(L 2^-6)
    // (H = sum_{w<4} T_w 2^(24 - 8 w), L = sum_{4<=w<7} T_w 2^(48 - 8 w)),
    // and the product is S 2^(e_x + e_w - 58).
    const int q = warp & 3, h = warp >> 2;
    const int jd = q * 32 + lane;
    const int64_t jj = j0 + jd;
    const uint32_t tq = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(h * 16);
    long long S[16], L[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) S[c] = L[c] = 0;
#pragma unroll
    for (int w = 0; w < SLICES; ++w) {
      uint32_t rr[16];
      umma::tmem_ld16(tq + (uint32_t)(w * LEAF_INV_N), rr);
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        const long long v = (long long)__float2int_rn(__uint_as_float(rr[c]));
        if (w < 4) S[c] += v << (24 - 8 * w);
        else L[c] += v << (48 - 8 * w);
      }
    }
    const int ex = ex_s[jd];
    if (jj < a.m) {
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        const int i = h * 16 + c;
        if (i < n) {
          const int ew = ew_s[i];
          const long long tot = (S[c] << 18) + ((L[c] + (1ll << 5)) >> 6);
          a.X[xat(i, jj)] = ex == NONFINITE || ew == NONFINITE ? __longlong_as_double(0x7ff8000000000000ll)
                                                               : scaled_i64_to_f64(tot, ex + ew - 58);
        }
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
  }
  return NLA_OK;
}

}  // namespace

bool leaf_inverses_wanted(const RecPlan& c) {
  if (c.mode != GEMM_MIXED || c.S != EXACT_SLICES || !c.bf16 || c.func != 'S' || c.dtype != NLA_F64) return false;
  if (c.threshold > LEAF_INV_N) return false;
  // The leaf overwrites X from the finishing pass (NLA_EXACT_FINISH=0 removes it).
  const char* f = std::getenv("NLA_EXACT_FINISH");
  if (f && f[0] == '0') return false;
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

int leaf_inverse_apply(const RecPlan& c, const Mat& A, int64_t n, const Mat& B) {
  if (n <= 0 || c.m <= 0) return NLA_OK;
  const LeafInverses& L = *c.inv;
  const int64_t k = (static_cast<const double*>(A.p) - L.a_base) / (L.lda + 1);
  const auto it = std::lower_bound(L.k.begin(), L.k.end(), k);
  if (L.a_base == nullptr || it == L.k.end() || *it != k)
    return fail(NLA_ERR_ARG, "leaf inverses: no inverse for this block");
  const int64_t slot = it - L.k.begin();
  // X := inv(T) X  (side L)  or  X inv(T)  (side R), one kernel.
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    attr = cudaFuncSetAttribute(leaf_product_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, LP_SMEM);
  });
  if (attr != cudaSuccess) return cuda_status(attr, "cudaFuncSetAttribute(leaf_product_kernel)");
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
