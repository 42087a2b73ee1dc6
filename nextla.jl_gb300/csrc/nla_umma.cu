// Off-diagonal update on the 5th-generation tensor cores (tcgen05) of sm_103a.
//
//   C (M x N) += alpha * op(A) (M x K) * op(B) (K x N)
//
// The operands are first "staged": each is written as S slices of 16-bit
// values (BF16 or FP16) in a K-major layout padded to the tile grid, with one
// power-of-two exponent per row of op(A) and per column of op(B):
//     x = 2^e * sum_p s_p * 2^(-beta p),   s_p integers, |s_p| <= 2^(beta-1)
// (beta = 8 for BF16 slices, 11 for FP16).  The split is done with integer
// arithmetic on the FP64 bit pattern, so it issues no FP64 instruction.
// A Float16 operand of the plain Float16 path is staged as one unscaled slice.
//
// The GEMM kernel (one 128 x 128 output tile per CTA, 6 warps):
//   warp 0      TMA producer: per 64-wide K block, one 128 x 64 box per slice
//               of each operand (128-byte swizzle) into a multi-stage ring;
//   warp 1      allocates TMEM, and one elected lane issues tcgen05.mma for
//               every slice pair (p, q) kept by the split, accumulating pairs
//               of equal weight p + q in the same FP32 TMEM accumulator;
//   warps 2-5   epilogue: tcgen05.ld of the accumulators, combination of the
//               weights in FP32, and the update of C (one FP64 operation per
//               element for FP64 outputs; the power-of-two scale is applied
//               to the exponent bits).
// Every mbarrier wait is bounded; on expiry the kernel records an error word
// that nla_device_status() reports, releases its TMEM and returns.
#include <cudaTypedefs.h>

#include <cstdlib>
#include <cstring>
#include <atomic>
#include <mutex>
#include <type_traits>
#include <unordered_map>

#include "nla_common.cuh"
#include "nla_split7.cuh"
#include "nla_umma.cuh"

namespace nla {

__device__ int g_device_error = 0;

namespace {

constexpr int BM = 128;
constexpr int BN = 128;
constexpr int BK = 64;                     // 64 16-bit elements = one 128-byte swizzle row
constexpr int TILE_BYTES = BM * BK * 2;    // 16 KiB per slice tile (BN == BM)
constexpr int GEMM_THREADS = 224;  // A producer, MMA, 4 epilogue warps, B producer
constexpr int MAX_PAIRS = 16;
constexpr int MAX_ACC = 4;
constexpr int SENTINEL_EXP = -2139062144;  // 0x80808080: "no element seen"
constexpr int NONFINITE_EXP = 0x7fffffff;

enum Epi { EPI_F64 = 0, EPI_F16 = 1 };

struct GemmParams {
  int M, N;
  int num_kb;
  int tiles_m, tiles_n;
  int a_rows, b_rows;  // padded rows of the operands (multiples of 128)
  int sa, sb;          // slices of A and B loaded per stage
  int stages;
  int stage_bytes;
  int npairs;
  int8_t pair_a[MAX_PAIRS], pair_b[MAX_PAIRS], pair_acc[MAX_PAIRS], pair_first[MAX_PAIRS];
  int nacc;
  float acc_w[MAX_ACC];
  uint32_t tmem_cols;
  uint32_t idesc;
  void* C;
  int64_t ldc;
  double alpha;
  const int* ea;
  const int* eb;
  int exp_bias;
  int producers;  // TMA-issuing warps: 2 (A and B apart) or 1 (warp 0 loads both)
};

__device__ __forceinline__ double scaled_double(float v, int e) {
  const uint32_t fb = __float_as_uint(v);
  if ((fb << 1) == 0) return __longlong_as_double((unsigned long long)(fb >> 31) << 63);
  const int E = (int)((fb >> 23) & 0xFF);
  const int de = E - 127 + 1023 + e;
  if (E == 0 || E == 255 || de <= 0 || de >= 2047) return ldexp((double)v, e);
  const unsigned long long db = ((unsigned long long)(fb >> 31) << 63) | ((unsigned long long)de << 52) |
                                ((unsigned long long)(fb & 0x7FFFFFu) << 29);
  return __longlong_as_double(db);
}

template <int EPI>
__global__ void __launch_bounds__(GEMM_THREADS, 1)
    umma_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                     const GemmParams p) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)p.stages * p.stage_bytes);
  uint64_t* fullA = bars;  // the A producer's (or, with one producer, both operands') loads of each stage
  uint64_t* fullB = bars + p.stages;  // the B producer's loads
  uint64_t* empty = bars + 2 * p.stages;
  uint64_t* accf = bars + 3 * p.stages;
  uint64_t* drain = accf + 1;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
  __shared__ volatile int s_abort;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  // Grouped rasterisation: 8 row tiles per group keep a wave's operands in L2.
  const int group = 8;
  const int per_group = group * p.tiles_n;
  const int g = blockIdx.x / per_group;
  const int first_m = g * group;
  const int gsize = min(p.tiles_m - first_m, group);
  const int local = blockIdx.x % per_group;
  const int tm = first_m + local % gsize;
  const int tn = local / gsize;
  const int m0 = tm * BM, n0 = tn * BN;

  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int s = 0; s < p.stages; ++s) {
      umma::mbar_init(umma::smem_u32(&fullA[s]), 1);
      umma::mbar_init(umma::smem_u32(&fullB[s]), 1);
      umma::mbar_init(umma::smem_u32(&empty[s]), 1);
    }
    umma::mbar_init(umma::smem_u32(accf), 1);
    umma::mbar_init(umma::smem_u32(drain), 1);
    umma::fence_barrier_init();
    umma::prefetch_tmap(&tmA);
    umma::prefetch_tmap(&tmB);
  }
  if (warp == 1) umma::tmem_alloc(umma::smem_u32(tmem_slot), p.tmem_cols);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 || warp == GEMM_THREADS / 32 - 1) {
    // Producers: warp 0 loads the A slices and the last warp the B slices
    // (p.producers = 2), or warp 0 loads both (1).  One issuing thread is
    // limited to about 110 GB/s of TMA tile loads per SM, two reach about
    // 175 GB/s.  Each producer arrives on its own full barrier of a stage.
    const bool is_a = warp == 0;
    const bool both = p.producers == 1;
    if (lane == 0 && (is_a || !both)) {
      uint64_t* own = is_a ? fullA : fullB;
      int kb = 0;
      for (; kb < p.num_kb; ++kb) {
        const int s = kb % p.stages;
        const uint32_t round = (uint32_t)(kb / p.stages);
        if (!umma::mbar_wait(umma::smem_u32(&empty[s]), (round & 1u) ^ 1u, &s_abort, &g_device_error, 1)) break;
        const uint32_t fb = umma::smem_u32(&own[s]);
        uint8_t* st = smem + (size_t)s * p.stage_bytes;
        umma::mbar_arrive_expect_tx(fb, (uint32_t)(((both ? p.sa + p.sb : is_a ? p.sa : p.sb)) * TILE_BYTES));
        if (is_a)
          for (int sl = 0; sl < p.sa; ++sl)
            umma::tma_load_2d(umma::smem_u32(st + sl * TILE_BYTES), &tmA, fb, kb * BK, m0 * p.sa + sl * BM);
        if (!is_a || both)
          for (int sl = 0; sl < p.sb; ++sl)
            umma::tma_load_2d(umma::smem_u32(st + (p.sa + sl) * TILE_BYTES), &tmB, fb, kb * BK, n0 * p.sb + sl * BN);
      }
      umma::producer_quiesce(own, p.stages, kb, &s_abort, &g_device_error, 5);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      bool ok = true;
      for (int kb = 0; kb < p.num_kb; ++kb) {
        const int s = kb % p.stages;
        const uint32_t round = (uint32_t)(kb / p.stages);
        if (!umma::mbar_wait(umma::smem_u32(&fullA[s]), round & 1u, &s_abort, &g_device_error, 2) ||
            (p.producers == 2 && !umma::mbar_wait(umma::smem_u32(&fullB[s]), round & 1u, &s_abort, &g_device_error, 2))) {
          ok = false;
          break;
        }
        umma::fence_after_sync();
        const uint32_t st = umma::smem_u32(smem + (size_t)s * p.stage_bytes);
        for (int pr = 0; pr < p.npairs; ++pr) {
          const uint32_t a0 = st + p.pair_a[pr] * TILE_BYTES;
          const uint32_t b0 = st + (p.sa + p.pair_b[pr]) * TILE_BYTES;
          const uint32_t d = tmem + (uint32_t)(p.pair_acc[pr] * BN);
#pragma unroll
          for (int kk = 0; kk < BK / 16; ++kk) {
            const uint32_t acc = (kb > 0 || kk > 0 || !p.pair_first[pr]) ? 1u : 0u;
            umma::mma_f16(d, umma::desc_kmajor_sw128(a0 + kk * 32), umma::desc_kmajor_sw128(b0 + kk * 32), p.idesc,
                          acc);
          }
        }
        umma::mma_commit(umma::smem_u32(&empty[s]));
      }
      if (ok) umma::mma_commit(umma::smem_u32(accf));
      // Before TMEM is released every issued MMA must have finished.
      umma::mma_commit(umma::smem_u32(drain));
      umma::mbar_wait(umma::smem_u32(drain), 0, &s_abort, &g_device_error, 3, false);
    }
  } else {
    // Epilogue warps 2..5 own TMEM lane quadrants (warp % 4).
    const int q = warp & 3;
    const int row = q * 32 + lane;
    const int i = m0 + row;
    // tcgen05.ld is warp-collective: the lanes act on one shared verdict.
    const bool ok = __all_sync(0xffffffffu, umma::mbar_wait(umma::smem_u32(accf), 0, &s_abort, &g_device_error, 4));
    umma::fence_after_sync();
    if (ok) {
      const uint32_t tq = tmem + ((uint32_t)(q * 32) << 16);
      int ei = 0;
      bool row_nan = false;
      if (EPI == EPI_F64 && p.ea != nullptr && i < p.M) {
        ei = p.ea[i];
        row_nan = ei == NONFINITE_EXP;
        ei = max(ei, -4000);
      }
      for (int c0 = 0; c0 < BN; c0 += 16) {
        float v[16];
        uint32_t r[16];
        umma::tmem_ld16(tq + (uint32_t)c0, r);
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
        for (int a = 1; a < p.nacc; ++a) {
          umma::tmem_ld16(tq + (uint32_t)(a * BN + c0), r);
          const float w = p.acc_w[a];
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] = fmaf(__uint_as_float(r[j]), w, v[j]);
        }
        if (i < p.M) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int col = n0 + c0 + j;
            if (col >= p.N) continue;
            if (EPI == EPI_F64) {
              double* cp = static_cast<double*>(p.C) + i + (int64_t)col * p.ldc;
              int ej = p.eb != nullptr ? p.eb[col] : 0;
              if (row_nan || ej == NONFINITE_EXP) {
                *cp = __longlong_as_double(0x7ff8000000000000ull);
              } else {
                const double d = scaled_double(v[j], ei + max(ej, -4000) + p.exp_bias);
                *cp = fma(p.alpha, d, *cp);
              }
            } else {
              __half* cp = static_cast<__half*>(p.C) + i + (int64_t)col * p.ldc;
              *cp = __float2half_rn(fmaf((float)p.alpha, v[j], __half2float(*cp)));
            }
          }
        }
      }
    }
  }

  umma::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    umma::fence_after_sync();
    umma::tmem_dealloc(tmem, p.tmem_cols);
  }
}

// ---------------------------------------------------------------------------
// Exact-accumulation update (the FP64 residual of refinement).
//
// Operands are staged as S = 7 BF16 slices of integers |s| <= 128, so one
// slice pair's products are exact and their FP32 sum over a chunk of <= 1024
// values (|sum| <= 2^24) is exact in TMEM.  K is walked in 1024-value chunks
// (outer loop, so all CTAs of a wave share a small working set in L2) and,
// inside each chunk, every slice pair accumulates into one of two TMEM
// buffers (double-buffered); eight
// epilogue warps drain each chunk, convert it to integers and add it, shifted
// by the pair's weight 2^(-8(p+q)), into 64-bit fixed-point accumulators held
// in registers.  FP64 arithmetic is used once per output element, for the
// final C += alpha * 2^e * acc.  A tile's K range is clipped to where both
// operands can be non-zero, so a triangular operand (staged with zeros
// outside its triangle) costs only its triangle.
// ---------------------------------------------------------------------------

constexpr int EX_THREADS = 352;  // A producer, MMA, B producer, 8 epilogue warps
constexpr int EX_CHUNK = 16;     // k-blocks per exact chunk (1024 values)
constexpr int EX_SLICES = 7;
constexpr int EX_MAX_PAIRS = 28;
constexpr int EX_STAGES = 6;  // 192 KiB of stages (seven measured no faster)
constexpr int EX_STAGE_BYTES = 2 * TILE_BYTES;
constexpr int EX_DYN_SMEM = EX_STAGES * EX_STAGE_BYTES + 1024 + 256;
static_assert(EX_DYN_SMEM + 16 <= 232448, "exact kernel shared memory above the per-block limit");

struct ExactParams {
  int M, N, K;
  int tiles_m, tiles_n;
  int a_rows, b_rows;
  int npairs;
  int8_t pa[EX_MAX_PAIRS], pb[EX_MAX_PAIRS];
  int tri_a, tri_b;  // staged triangle of each operand (see in_tri)
  int trans_out;     // write the product transposed: element (i, j) to C[j + i*ldc]
  const float* nrm_a;  // per-row slice-magnitude sums of A (headroom of the fixed point)
  // Residual epilogue (when res_x is set): C := C - P - d_i * X(pos), with
  // d_i = res_d[i * res_dstride] and X at the position of C's element.
  const double* res_x;
  int64_t res_ldx;
  const double* res_d;
  int64_t res_dstride;
  void* C;
  int64_t ldc;
  double alpha;
  const int* ea;
  const int* eb;
  int merged;  // coupled kernel: short-K group table (pairs of one weight share an accumulator)
  // When set, the kernel writes its fixed-point sums to P (element (i, j) at
  // P[i + j * ldp]) and exact_finish_kernel applies them to C.
  long long* P;
  int64_t ldp;
};

// K range of the staged triangle that meets rows [r0, r0 + span).
__device__ __forceinline__ void tri_k_range(int tri, int r0, int span, int K, int& lo, int& hi) {
  lo = 0;
  hi = K - 1;
  if (tri == 1 || tri == 3) hi = min(K - 1, r0 + span - 1);
  else if (tri == 2 || tri == 4) lo = r0;
}

__device__ __forceinline__ double scale_pow2(double d, int e) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const int E = (int)((b >> 52) & 0x7FF);
  const int ne = E + e;
  if (E == 0 || E == 0x7FF || ne <= 0 || ne >= 2047) return ldexp(d, e);
  return __longlong_as_double((long long)((b & ~(0x7FFull << 52)) | ((unsigned long long)ne << 52)));
}

__device__ __forceinline__ void two_sum_dev(double a, double b, double& s, double& e) {
  s = a + b;
  const double bp = s - a;
  e = (a - (s - bp)) + (b - bp);
}

// Fixed point of an output row of the exact kernels: LSB 2^-Lb in units of
// 2^(ea+eb).  Every partial sum is bounded by nrm_a[i] * (1/2 + 2^-8), so Lb
// keeps it below 2^61 while giving short or small rows the finest resolution.
__device__ __forceinline__ int exact_row_lb(const ExactParams& p, int i) {
  int Lb = 60;
  if (i < p.M) {
    const float bound = p.nrm_a[i] * (0.5f + 0.00390625f) * 1.001f;
    if (bound > 0.0f) Lb = 61 - (int)ceilf(log2f(bound));
    Lb = min(max(Lb, 0), 77);
  }
  return Lb;
}

// Adds one exact FP32 chunk sum (64 TMEM columns of this thread's lane at ta)
// into the int64 fixed point, shifted by sh (rounded half up when sh < 0).
// The chunk sums are integers below 2^24 in magnitude, so each converts to an
// int32 v exactly.  When every lane of the warp has sh >= 0, v * 2^sh is built
// from 32-bit shifts: low word v << sh (0 once sh >= 32), high word the
// funnel shift of (sign(v) : v) by min(sh, 32), shifted on by sh - 32.  When
// every lane has -24 <= sh < 0 the rounded shift stays in 32 bits.  Both give
// the same bits as the 64-bit expression of the general case.
__device__ __forceinline__ uint32_t shl_clamped(uint32_t a, uint32_t s) {
  uint32_t d;
  asm("shl.b32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(s));  // shifts of 32 or more give 0
  return d;
}

#ifndef NLA_DRAIN_COLS
#define NLA_DRAIN_COLS 16
#endif
constexpr int DRAIN_COLS = NLA_DRAIN_COLS;  // TMEM columns per load-and-wait
__device__ __forceinline__ void drain_load(uint32_t ta, uint32_t* r) {
  if constexpr (DRAIN_COLS == 32) umma::tmem_ld32(ta, r);
  else umma::tmem_ld16(ta, r);
}

__device__ __forceinline__ void exact_drain(long long (&acc)[64], uint32_t ta, int sh) {
  if (__all_sync(0xffffffffu, sh >= 0)) {
    const uint32_t s_lo = (uint32_t)sh, s_hi = (uint32_t)max(sh - 32, 0);
#pragma unroll
    for (int j0 = 0; j0 < 64; j0 += DRAIN_COLS) {
      uint32_t r[DRAIN_COLS];
      drain_load(ta + (uint32_t)j0, r);
#pragma unroll
      for (int j = 0; j < DRAIN_COLS; ++j) {
        const int v = __float2int_rn(__uint_as_float(r[j]));
        const uint32_t lo = shl_clamped((uint32_t)v, s_lo);
        const uint32_t hi = __funnelshift_lc((uint32_t)v, (uint32_t)(v >> 31), s_lo) << s_hi;
        acc[j0 + j] += (long long)(((unsigned long long)hi << 32) | lo);
      }
    }
  } else if (__all_sync(0xffffffffu, sh < 0 && sh >= -24)) {
    const int n = -sh, bias = 1 << (n - 1);
#pragma unroll
    for (int j0 = 0; j0 < 64; j0 += 16) {
      uint32_t r[16];
      umma::tmem_ld16(ta + (uint32_t)j0, r);
#pragma unroll
      for (int j = 0; j < 16; ++j) acc[j0 + j] += (long long)((__float2int_rn(__uint_as_float(r[j])) + bias) >> n);
    }
  } else {
#pragma unroll
    for (int j0 = 0; j0 < 64; j0 += 16) {
      uint32_t r[16];
      umma::tmem_ld16(ta + (uint32_t)j0, r);
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const long long v = (long long)__float2int_rn(__uint_as_float(r[j]));
        acc[j0 + j] += sh >= 0 ? (v << sh) : ((v + (1ll << (-sh - 1))) >> (-sh));
      }
    }
  }
}

// The fixed-point sums of output row i and the 64 columns from c0, written
// to P as they are: 64 independent stores, no loads and no FP64 work, so
// the CTA ends (and the next tile starts on its SM) as soon as they are
// issued.  exact_finish_kernel applies them to C.
__device__ __forceinline__ void exact_store_fixed(const ExactParams& p, const long long (&acc)[64], int i, int c0) {
  if (i >= p.M) return;
  long long* P = p.P + i;
#pragma unroll
  for (int j = 0; j < 64; ++j)
    if (c0 + j < p.N) P[(int64_t)(c0 + j) * p.ldp] = acc[j];
}

// C += alpha * P for the fixed-point sums an exact kernel left in P: the
// same arithmetic as exact_store, over all M x N elements at full occupancy
// (a drain warp doing it in the exact kernel spent about 40 us per 128 x 128
// tile on the latency of its loads and its FP64 conversions, with the
// tensor cores of its SM idle).
constexpr int FINISH_COLS = 16;  // columns per CTA of exact_finish_kernel
__global__ void __launch_bounds__(256) exact_finish_kernel(const ExactParams p) {
  // Thread: one row; CTA: 256 rows x FINISH_COLS columns (coalesced along
  // the rows, eight columns of loads in flight per thread).
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i >= p.M) return;
  const int ei = p.ea[i];
  const bool row_nan = ei == NONFINITE_EXP;
  const int er = max(ei, -4000) - exact_row_lb(p, i);
  const int64_t cbase = (int64_t)blockIdx.y * FINISH_COLS;
#pragma unroll
  for (int c0 = 0; c0 < FINISH_COLS; c0 += 8) {
    long long v[8];
    double cv[8];
    int ej[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int64_t col = cbase + c0 + c;
      const bool in = col < p.N;
      v[c] = in ? p.P[(int64_t)i + col * p.ldp] : 0;
      cv[c] = in ? static_cast<const double*>(p.C)[(int64_t)i + col * p.ldc] : 0.0;
      ej[c] = in ? p.eb[col] : 0;
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int64_t col = cbase + c0 + c;
      if (col >= p.N) continue;
      double out = __longlong_as_double(0x7ff8000000000000ll);
      // The sum as FP64 by integer operations (the same rounding as a
      // conversion followed by an exact scaling), which leaves the FMA as
      // the only work on GB300's FP64 pipe (2 operations per clock per SM).
      if (!row_nan && ej[c] != NONFINITE_EXP)
        out = fma(p.alpha, split7::scaled_i64_to_f64(v[c], er + max(ej[c], -4000)), cv[c]);
      static_cast<double*>(p.C)[(int64_t)i + col * p.ldc] = out;
    }
  }
}

// C update of the exact kernels for output row i and the 64 columns from c0:
// C += alpha * P, or the residual form C := C - P - d_i x (P exact in acc,
// formed with error-free transformations and rounded once).
__device__ __forceinline__ void exact_store(const ExactParams& p, const long long (&acc)[64], int i, int c0, int Lb) {
  if (i >= p.M) return;
  int ei = p.ea[i];
  const bool row_nan = ei == NONFINITE_EXP;
  ei = max(ei, -4000);
#pragma unroll
  for (int j = 0; j < 64; ++j) {
    const int col = c0 + j;
    if (col >= p.N) continue;
    double* cp = static_cast<double*>(p.C) +
                 (p.trans_out ? (int64_t)col + (int64_t)i * p.ldc : (int64_t)i + (int64_t)col * p.ldc);
    const int ej = p.eb[col];
    if (row_nan || ej == NONFINITE_EXP) {
      *cp = __longlong_as_double(0x7ff8000000000000ull);
    } else if (p.res_x == nullptr) {
      const double d = scale_pow2(__ll2double_rn(acc[j]), ei + max(ej, -4000) - Lb);
      *cp = fma(p.alpha, d, *cp);
    } else {
      const int e = ei + max(ej, -4000) - Lb;
      const double hi_u = __ll2double_rn(acc[j]);
      const double lo_u = __ll2double_rn(acc[j] - (long long)hi_u);
      const double s_hi = scale_pow2(hi_u, e), s_lo = scale_pow2(lo_u, e);
      const double dg = p.res_d[(int64_t)i * p.res_dstride];
      const double xv = p.res_x[p.trans_out ? (int64_t)col + (int64_t)i * p.res_ldx
                                            : (int64_t)i + (int64_t)col * p.res_ldx];
      const double pr = dg * xv;
      const double pe = fma(dg, xv, -pr);
      double t1, e1, t2, e2;
      two_sum_dev(*cp, -s_hi, t1, e1);
      two_sum_dev(t1, -pr, t2, e2);
      *cp = t2 + (((e1 + e2) - pe) - s_lo);
    }
  }
}

// Pair by pair: each stage holds one A slice tile and one B slice tile
// (32 KiB), and every slice pair has its own accumulator drain.
__global__ void __launch_bounds__(EX_THREADS, 1)
    umma_exact_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                      const ExactParams p) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* fullA = reinterpret_cast<uint64_t*>(smem + EX_STAGES * EX_STAGE_BYTES);  // A producer's loads
  uint64_t* fullB = fullA + EX_STAGES;                                                // B producer's loads
  uint64_t* empty = fullB + EX_STAGES;
  uint64_t* cfull = empty + EX_STAGES;
  uint64_t* cempty = cfull + 2;
  uint64_t* drain = cempty + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
  __shared__ volatile int s_abort;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // Output tiles are rasterised in groups of 8 tile rows for L2 reuse.
  const int cid = (int)blockIdx.x;
  constexpr int group = 8;
  const int per_group = group * p.tiles_n;
  const int g = cid / per_group;
  const int first_m = g * group;
  const int gsize = min(p.tiles_m - first_m, group);
  const int local = cid % per_group;
  const int m0 = (first_m + local % gsize) * BM, n0 = (local / gsize) * BN;

  int alo, ahi, blo, bhi;
  tri_k_range(p.tri_a, m0, BM, p.K, alo, ahi);
  tri_k_range(p.tri_b, n0, BN, p.K, blo, bhi);
  const int klo = max(alo, blo), khi = min(ahi, bhi);
  const int kb0 = klo / BK;
  const int kb1 = khi >= klo ? khi / BK + 1 : kb0;  // empty range when the triangles miss each other

  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int s = 0; s < EX_STAGES; ++s) {
      umma::mbar_init(umma::smem_u32(&fullA[s]), 1);
      umma::mbar_init(umma::smem_u32(&fullB[s]), 1);
      umma::mbar_init(umma::smem_u32(&empty[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      umma::mbar_init(umma::smem_u32(&cfull[b]), 1);
      umma::mbar_init(umma::smem_u32(&cempty[b]), 8);
    }
    umma::mbar_init(umma::smem_u32(drain), 1);
    umma::fence_barrier_init();
  }
  if (warp == 1) umma::tmem_alloc(umma::smem_u32(tmem_slot), 256);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  bool ok = true;

  if (warp == 0 || warp == 2) {
    // Two producers, one per operand: a thread issues TMA tile loads at a
    // limited rate (about 110 GB/s per SM measured with 16 KiB boxes), and two
    // issuing warps reach about 175 GB/s.  Each arrives on its own full
    // barrier of a stage for its 16 KiB.
    const bool is_a = warp == 0;
    if (lane == 0) {
      uint64_t* own = is_a ? fullA : fullB;
      int it = 0;
      for (int cc = kb0 / EX_CHUNK; cc * EX_CHUNK < kb1 && ok; ++cc) {
        const int c0 = max(kb0, cc * EX_CHUNK), c1 = min(kb1, (cc + 1) * EX_CHUNK);
        if (c0 >= c1) continue;  // empty K range (the operands' triangles miss each other)
        for (int pr = 0; pr < p.npairs && ok; ++pr) {
          for (int kb = c0; kb < c1; ++kb, ++it) {
            const int s = it % EX_STAGES;
            const uint32_t round = (uint32_t)(it / EX_STAGES);
            if (!umma::mbar_wait(umma::smem_u32(&empty[s]), (round & 1u) ^ 1u, &s_abort, &g_device_error, 11)) {
              ok = false;
              break;
            }
            const uint32_t fb = umma::smem_u32(&own[s]);
            umma::mbar_arrive_expect_tx(fb, (uint32_t)TILE_BYTES);
            uint8_t* st = smem + s * EX_STAGE_BYTES;
            if (is_a)
              umma::tma_load_2d(umma::smem_u32(st), &tmA, fb, kb * BK, m0 * EX_SLICES + p.pa[pr] * BM);
            else
              umma::tma_load_2d(umma::smem_u32(st + TILE_BYTES), &tmB, fb, kb * BK, n0 * EX_SLICES + p.pb[pr] * BN);
          }
        }
      }
      umma::producer_quiesce(own, EX_STAGES, it, &s_abort, &g_device_error, 16);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = umma::idesc_f16(BM, BN, true), idesc2 = umma::idesc_f16(BM, 2 * BN, true);
      int it = 0, ch = 0;
      for (int cc = kb0 / EX_CHUNK; cc * EX_CHUNK < kb1 && ok; ++cc) {
        const int c0 = max(kb0, cc * EX_CHUNK), c1 = min(kb1, (cc + 1) * EX_CHUNK);
        if (c0 >= c1) continue;
        for (int pr = 0; pr < p.npairs && ok; ++pr, ++ch) {
          const int b = ch & 1;
          const uint32_t use = (uint32_t)(ch >> 1);
          if (!umma::mbar_wait(umma::smem_u32(&cempty[b]), (use & 1u) ^ 1u, &s_abort, &g_device_error, 12)) {
            ok = false;
            break;
          }
          umma::fence_after_sync();
          for (int kb = c0; kb < c1; ++kb, ++it) {
            const int s = it % EX_STAGES;
            const uint32_t round = (uint32_t)(it / EX_STAGES);
            if (!umma::mbar_wait(umma::smem_u32(&fullA[s]), round & 1u, &s_abort, &g_device_error, 13) ||
                !umma::mbar_wait(umma::smem_u32(&fullB[s]), round & 1u, &s_abort, &g_device_error, 13)) {
              ok = false;
              break;
            }
            umma::fence_after_sync();
            const uint32_t a0 = umma::smem_u32(smem + s * EX_STAGE_BYTES);
            const uint32_t b0 = a0 + TILE_BYTES;
#pragma unroll
            for (int kk = 0; kk < BK / 16; ++kk)
              umma::mma_f16(tmem + (uint32_t)(b * BN), umma::desc_kmajor_sw128(a0 + kk * 32),
                            umma::desc_kmajor_sw128(b0 + kk * 32), idesc, (kb > c0 || kk > 0) ? 1u : 0u);
            umma::mma_commit(umma::smem_u32(&empty[s]));
          }
          if (ok) umma::mma_commit(umma::smem_u32(&cfull[b]));
        }
      }
      umma::mma_commit(umma::smem_u32(drain));
      umma::mbar_wait(umma::smem_u32(drain), 0, &s_abort, &g_device_error, 14, false);
    }
  } else {
    const int q = warp & 3;
    const int h = (warp - 3) >> 2;  // column half: 0 (warps 3-6) or 1 (warps 7-10)
    const int row = q * 32 + lane;
    const int i = m0 + row;
    long long acc[64];
#pragma unroll
    for (int j = 0; j < 64; ++j) acc[j] = 0;
    const int Lb = exact_row_lb(p, i);
    int ch = 0;
    for (int cc = kb0 / EX_CHUNK; cc * EX_CHUNK < kb1 && ok; ++cc) {
      if (max(kb0, cc * EX_CHUNK) >= min(kb1, (cc + 1) * EX_CHUNK)) continue;
      for (int pr = 0; pr < p.npairs && ok; ++pr, ++ch) {
        const int sh = Lb - 8 * (p.pa[pr] + p.pb[pr] + 2);
        const int b = ch & 1;
        const uint32_t use = (uint32_t)(ch >> 1);
        ok = __all_sync(0xffffffffu,
                        umma::mbar_wait(umma::smem_u32(&cfull[b]), use & 1u, &s_abort, &g_device_error, 15));
        if (!ok) break;
        umma::fence_after_sync();
        exact_drain(acc, tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * BN + h * 64), sh);
        umma::fence_before_sync();
        __syncwarp();
        if (lane == 0) umma::mbar_arrive(umma::smem_u32(&cempty[b]));
      }
    }
    if (ok) {
      if (p.P) exact_store_fixed(p, acc, i, n0 + h * 64);
      else exact_store(p, acc, i, n0 + h * 64, Lb);
    }
  }

  umma::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    umma::fence_after_sync();
    umma::tmem_dealloc(tmem, 256);
  }
}

// ---------------------------------------------------------------------------
// Exact kernel with coupled pairs.  The 28 slice pairs (A_a, B_b), a + b <= 6,
// are walked as 16 groups: for each A slice a, the B slices b = 0, 2, 4, 6
// each with its successor b + 1 while b + 1 <= 6 - a.  A group's stage holds
// A_a and B_b, B_b+1 (one 256-row box: the staging puts the slices of a tile
// next to each other), 48 KiB in all, and feeds two adjacent accumulators
// (weights a + b and a + b + 1) with one MMA of N = 256.  A pair costs 24 KiB
// of tile loads instead of 32 (the TMA feed bounds these kernels, about
// 100-120 GB/s per SM), and 12 KiB of shared-memory operand reads per 16-wide
// K step instead of 16 (two N = 128 MMAs that shared one B tile, the earlier
// form, read close to the 128 B per clock that shared memory delivers).
// Each group's two accumulators take half of a 256-column TMEM buffer; two
// buffers fill the 512 columns.  Updates with K <= 256 use a second table
// (below) in which the pairs of one weight share an accumulator.  Plain
// updates store the tile's fixed-point sums for exact_finish_kernel;
// residuals apply them here (exact_store).
// Warps: 0 loads A, 1 issues the MMAs, 2 loads B, 3-10 drain.
// ---------------------------------------------------------------------------
constexpr int CP_STAGES = 4;
constexpr int CP_STAGE_BYTES = 3 * TILE_BYTES;
constexpr int CP_DYN_SMEM = CP_STAGES * CP_STAGE_BYTES + 1024 + 256;
constexpr int CP_GROUPS = 16;
static_assert(CP_DYN_SMEM + 16 <= 232448, "coupled exact kernel shared memory above the per-block limit");

// Group tables.  A group is drained as one or two accumulators (d0, d1) of
// weights w0, w1; it is filled by segments, each one K loop of one slice
// pair (A_q, B_p) into d0 or d1, or of the coupled pairs (A_q, B_p) -> d0
// and (A_q, B_p+1) -> d1 that share the A_q tile (the entries name B's slice
// first: the pair set is symmetric, so p and q range as in (A_p, B_q)).  A
// segment's init bits mark the first write into each accumulator (its MMAs
// start with enable_input_d 0); a coupled segment's two bits are equal.
//   segment: p | q << 4 | coupled << 8 | dst << 9 | init0 << 10 | init1 << 11
//   group:   first segment | segment count << 8 | w0 << 12 | w1 << 16 (15: no d1)
constexpr uint16_t cp_seg(int p, int q, int two, int dst, int i0, int i1) {
  return (uint16_t)(p | q << 4 | two << 8 | dst << 9 | i0 << 10 | i1 << 11);
}
constexpr uint32_t cp_grp(int first, int count, int w0, int w1) {
  return (uint32_t)(first | count << 8 | w0 << 12 | w1 << 16);
}
constexpr int CP_MERGED_MAX_K = 256;  // 4 pairs x 256 products of at most 2^14: 2^24
constexpr int CP_GROUPS_MERGED = 5;
__constant__ uint16_t c_cp_segs[CP_GROUPS + 19] = {
    // Default: 16 groups of one segment, q-major, p = 0, 2, 4, ... (a
    // coupled segment also takes p + 1 while p + 1 <= 6 - q).
    cp_seg(0, 0, 1, 0, 1, 1), cp_seg(2, 0, 1, 0, 1, 1), cp_seg(4, 0, 1, 0, 1, 1), cp_seg(6, 0, 0, 0, 1, 0),
    cp_seg(0, 1, 1, 0, 1, 1), cp_seg(2, 1, 1, 0, 1, 1), cp_seg(4, 1, 1, 0, 1, 1),
    cp_seg(0, 2, 1, 0, 1, 1), cp_seg(2, 2, 1, 0, 1, 1), cp_seg(4, 2, 0, 0, 1, 0),
    cp_seg(0, 3, 1, 0, 1, 1), cp_seg(2, 3, 1, 0, 1, 1),
    cp_seg(0, 4, 1, 0, 1, 1), cp_seg(2, 4, 0, 0, 1, 0),
    cp_seg(0, 5, 1, 0, 1, 1),
    cp_seg(0, 6, 0, 0, 1, 0),
    // Short K (at most CP_MERGED_MAX_K): the pairs of one weight share an
    // accumulator, at most 4 pairs each, so 5 groups (9 drains) replace 16
    // groups (28 drains) with the same 28 pair products.
    cp_seg(0, 0, 1, 0, 1, 1), cp_seg(0, 1, 0, 1, 0, 0),                              // w 0 | 1
    cp_seg(0, 2, 1, 0, 1, 1), cp_seg(1, 1, 1, 0, 0, 0), cp_seg(2, 0, 1, 0, 0, 0),
    cp_seg(0, 3, 0, 1, 0, 0),                                                         // w 2 | 3
    cp_seg(0, 4, 1, 0, 1, 1), cp_seg(1, 3, 1, 0, 0, 0), cp_seg(2, 2, 1, 0, 0, 0),   // w 4 | 5
    cp_seg(3, 1, 1, 0, 1, 1), cp_seg(4, 0, 1, 0, 0, 0), cp_seg(0, 5, 0, 1, 0, 0),   // w 4 | 5
    cp_seg(0, 6, 0, 0, 1, 0), cp_seg(1, 5, 0, 0, 0, 0), cp_seg(2, 4, 0, 0, 0, 0), cp_seg(3, 3, 0, 0, 0, 0),
    cp_seg(4, 2, 0, 1, 0, 1), cp_seg(5, 1, 0, 1, 0, 0), cp_seg(6, 0, 0, 1, 0, 0)};  // w 6 | 6
__constant__ uint32_t c_cp_grps[CP_GROUPS + CP_GROUPS_MERGED] = {
    cp_grp(0, 1, 0, 1),   cp_grp(1, 1, 2, 3),   cp_grp(2, 1, 4, 5),   cp_grp(3, 1, 6, 15),
    cp_grp(4, 1, 1, 2),   cp_grp(5, 1, 3, 4),   cp_grp(6, 1, 5, 6),
    cp_grp(7, 1, 2, 3),   cp_grp(8, 1, 4, 5),   cp_grp(9, 1, 6, 15),
    cp_grp(10, 1, 3, 4),  cp_grp(11, 1, 5, 6),
    cp_grp(12, 1, 4, 5),  cp_grp(13, 1, 6, 15),
    cp_grp(14, 1, 5, 6),
    cp_grp(15, 1, 6, 15),
    cp_grp(16, 2, 0, 1),  cp_grp(18, 4, 2, 3),  cp_grp(22, 3, 4, 5),  cp_grp(25, 3, 4, 5),
    cp_grp(28, 7, 6, 6)};

struct CpSeg {
  int p, q;
  bool two, init0, init1;
  int dst;
};
__device__ __forceinline__ CpSeg cp_seg_at(int i) {
  const int v = c_cp_segs[i];
  return CpSeg{v & 15, (v >> 4) & 15, ((v >> 8) & 1) != 0, ((v >> 10) & 1) != 0, ((v >> 11) & 1) != 0,
               (v >> 9) & 1};
}

__global__ void __launch_bounds__(EX_THREADS, 1)
    umma_exact_coupled_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                              const __grid_constant__ CUtensorMap tmB2, const ExactParams p) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* fullA = reinterpret_cast<uint64_t*>(smem + CP_STAGES * CP_STAGE_BYTES);  // A producer's loads
  uint64_t* fullB = fullA + CP_STAGES;                                                // B producer's loads
  uint64_t* empty = fullB + CP_STAGES;
  uint64_t* cfull = empty + CP_STAGES;
  uint64_t* cempty = cfull + 2;
  uint64_t* drain = cempty + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
  __shared__ volatile int s_abort;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int group = 8;
  const int per_group = group * p.tiles_n;
  const int gr = blockIdx.x / per_group;
  const int first_m = gr * group;
  const int gsize = min(p.tiles_m - first_m, group);
  const int local = blockIdx.x % per_group;
  const int m0 = (first_m + local % gsize) * BM, n0 = (local / gsize) * BN;
  int alo, ahi, blo, bhi;
  tri_k_range(p.tri_a, m0, BM, p.K, alo, ahi);
  tri_k_range(p.tri_b, n0, BN, p.K, blo, bhi);
  const int klo = max(alo, blo), khi = min(ahi, bhi);
  const int kb0 = klo / BK;
  const int kb1 = khi >= klo ? khi / BK + 1 : kb0;  // empty range when the triangles miss each other

  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int s = 0; s < CP_STAGES; ++s) {
      umma::mbar_init(umma::smem_u32(&fullA[s]), 1);
      umma::mbar_init(umma::smem_u32(&fullB[s]), 1);
      umma::mbar_init(umma::smem_u32(&empty[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      umma::mbar_init(umma::smem_u32(&cfull[b]), 1);
      umma::mbar_init(umma::smem_u32(&cempty[b]), 8);
    }
    umma::mbar_init(umma::smem_u32(drain), 1);
    umma::fence_barrier_init();
  }
  if (warp == 1) umma::tmem_alloc(umma::smem_u32(tmem_slot), 512);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  bool ok = true;

  const int g0 = p.merged ? CP_GROUPS : 0, g1 = p.merged ? CP_GROUPS + CP_GROUPS_MERGED : CP_GROUPS;
  if (warp == 0 || warp == 2) {
    const bool is_a = warp == 0;
    if (lane == 0) {
      uint64_t* own = is_a ? fullA : fullB;
      int it = 0;
      for (int cc = kb0 / EX_CHUNK; cc * EX_CHUNK < kb1 && ok; ++cc) {
        const int c0 = max(kb0, cc * EX_CHUNK), c1 = min(kb1, (cc + 1) * EX_CHUNK);
        if (c0 >= c1) continue;
        for (int g = g0; g < g1 && ok; ++g) {
          const uint32_t gv = c_cp_grps[g];
          const int s0 = gv & 255, ns = (gv >> 8) & 15;
          for (int si = s0; si < s0 + ns && ok; ++si) {
            const CpSeg sg = cp_seg_at(si);
            for (int kb = c0; kb < c1; ++kb, ++it) {
              const int s = it % CP_STAGES;
              const uint32_t round = (uint32_t)(it / CP_STAGES);
              if (!umma::mbar_wait(umma::smem_u32(&empty[s]), (round & 1u) ^ 1u, &s_abort, &g_device_error, 31)) {
                ok = false;
                break;
              }
              const uint32_t fb = umma::smem_u32(&own[s]);
              uint8_t* st = smem + s * CP_STAGE_BYTES;
              // Staged rows: slice sl of the tile at row r0 starts at r0 * 7 + sl * 128,
              // so B_p and B_p+1 are one 256-row box.  A segment (p, q) takes
              // A's slice q against B's slice p (and p + 1).
              if (is_a) {
                umma::mbar_arrive_expect_tx(fb, (uint32_t)TILE_BYTES);
                umma::tma_load_2d(umma::smem_u32(st), &tmA, fb, kb * BK, m0 * EX_SLICES + sg.q * BM);
              } else {
                umma::mbar_arrive_expect_tx(fb, (uint32_t)((sg.two ? 2 : 1) * TILE_BYTES));
                umma::tma_load_2d(umma::smem_u32(st + TILE_BYTES), sg.two ? &tmB2 : &tmB, fb, kb * BK,
                                  n0 * EX_SLICES + sg.p * BN);
              }
            }
          }
        }
      }
      umma::producer_quiesce(own, CP_STAGES, it, &s_abort, &g_device_error, 36);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = umma::idesc_f16(BM, BN, true), idesc2 = umma::idesc_f16(BM, 2 * BN, true);
      int it = 0, ch = 0;
      for (int cc = kb0 / EX_CHUNK; cc * EX_CHUNK < kb1 && ok; ++cc) {
        const int c0 = max(kb0, cc * EX_CHUNK), c1 = min(kb1, (cc + 1) * EX_CHUNK);
        if (c0 >= c1) continue;
        for (int g = g0; g < g1 && ok; ++g, ++ch) {
          const uint32_t gv = c_cp_grps[g];
          const int s0 = gv & 255, ns = (gv >> 8) & 15;
          const int b = ch & 1;
          if (!umma::mbar_wait(umma::smem_u32(&cempty[b]), ((uint32_t)(ch >> 1) & 1u) ^ 1u, &s_abort,
                               &g_device_error, 32)) {
            ok = false;
            break;
          }
          umma::fence_after_sync();
          const uint32_t d0 = tmem + (uint32_t)(b * 2 * BN), d1 = d0 + (uint32_t)BN;
          for (int si = s0; si < s0 + ns && ok; ++si) {
            const CpSeg sg = cp_seg_at(si);
            // The first MMA of a segment starts an accumulator the segment
            // initialises and adds to one an earlier segment started.  A
            // coupled segment is one MMA of N = 256 into both accumulators
            // (adjacent in TMEM), against B's two slices (adjacent in shared
            // memory); its two accumulators start together (init0 == init1
            // for every coupled segment of the tables).
            const uint32_t first0 = sg.two ? (sg.init0 ? 0u : 1u) : (sg.dst ? (sg.init1 ? 0u : 1u) : (sg.init0 ? 0u : 1u));
            const uint32_t dA = sg.two ? d0 : (sg.dst ? d1 : d0);
            const uint32_t id = sg.two ? idesc2 : idesc;
            for (int kb = c0; kb < c1; ++kb, ++it) {
              const int s = it % CP_STAGES;
              if (!umma::mbar_wait(umma::smem_u32(&fullA[s]), (uint32_t)(it / CP_STAGES) & 1u, &s_abort,
                                   &g_device_error, 33) ||
                  !umma::mbar_wait(umma::smem_u32(&fullB[s]), (uint32_t)(it / CP_STAGES) & 1u, &s_abort,
                                   &g_device_error, 33)) {
                ok = false;
                break;
              }
              umma::fence_after_sync();
              const uint32_t a0 = umma::smem_u32(smem + s * CP_STAGE_BYTES), b0 = a0 + TILE_BYTES;
#pragma unroll
              for (int kk = 0; kk < BK / 16; ++kk)
                umma::mma_f16(dA, umma::desc_kmajor_sw128(a0 + kk * 32), umma::desc_kmajor_sw128(b0 + kk * 32), id,
                              (kb > c0 || kk > 0) ? 1u : first0);
              umma::mma_commit(umma::smem_u32(&empty[s]));
            }
          }
          if (ok) umma::mma_commit(umma::smem_u32(&cfull[b]));
        }
      }
      umma::mma_commit(umma::smem_u32(drain));
      umma::mbar_wait(umma::smem_u32(drain), 0, &s_abort, &g_device_error, 34, false);
    }
  } else {
    const int q = warp & 3;
    const int h = (warp - 3) >> 2;  // column half: 0 (warps 3-6) or 1 (warps 7-10)
    const int i = m0 + q * 32 + lane;
    long long acc[64];
#pragma unroll
    for (int j = 0; j < 64; ++j) acc[j] = 0;
    const int Lb = exact_row_lb(p, i);
    int ch = 0;
    for (int cc = kb0 / EX_CHUNK; cc * EX_CHUNK < kb1 && ok; ++cc) {
      if (max(kb0, cc * EX_CHUNK) >= min(kb1, (cc + 1) * EX_CHUNK)) continue;
      for (int g = g0; g < g1 && ok; ++g, ++ch) {
        const uint32_t gv = c_cp_grps[g];
        const int w0 = (gv >> 12) & 15, w1 = (gv >> 16) & 15;
        const int b = ch & 1;
        ok = __all_sync(0xffffffffu, umma::mbar_wait(umma::smem_u32(&cfull[b]), (uint32_t)(ch >> 1) & 1u, &s_abort,
                                                     &g_device_error, 35));
        if (!ok) break;
        umma::fence_after_sync();
        const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * 2 * BN + h * 64);
        exact_drain(acc, ta, Lb - 8 * (w0 + 2));
        if (w1 != 15) exact_drain(acc, ta + (uint32_t)BN, Lb - 8 * (w1 + 2));
        umma::fence_before_sync();
        __syncwarp();
        if (lane == 0) umma::mbar_arrive(umma::smem_u32(&cempty[b]));
      }
    }
    if (ok) {
      if (p.P) exact_store_fixed(p, acc, i, n0 + h * 64);
      else exact_store(p, acc, i, n0 + h * 64, Lb);
    }
  }

  umma::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    umma::fence_after_sync();
    umma::tmem_dealloc(tmem, 512);
  }
}

// ---------------------------------------------------------------------------
// Staging kernels.
// ---------------------------------------------------------------------------

template <typename T> __device__ __forceinline__ double to_double(T x);
template <> __device__ __forceinline__ double to_double<double>(double x) { return x; }
template <> __device__ __forceinline__ double to_double<__half>(__half x) { return (double)__half2float(x); }

// frexp-style exponent of |x| plus one (so that x * 2^-e lies in [0.25, 0.5)
// for the largest element), from the bit pattern.
__device__ __forceinline__ int exp_of(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int biased = (int)((b >> 52) & 0x7FF);
  const unsigned long long mant = b & ((1ull << 52) - 1);
  if (biased == 0x7FF) return NONFINITE_EXP;
  if (biased == 0) return mant == 0 ? SENTINEL_EXP : -1021;
  return biased - 1022 + 1;
}

// Whether (i, k) lies in the staged part: everything (tri 0), k <= i (1),
// k >= i (2), k < i (3) or k > i (4).
__device__ __forceinline__ bool in_tri(int tri, int64_t i, int64_t k) {
  switch (tri) {
    case 1: return k <= i;
    case 2: return k >= i;
    case 3: return k < i;
    case 4: return k > i;
    default: return true;
  }
}

// Per-row maximum exponent of a rows x cols view (op(X) = X or X^T), one
// 64 x 64 tile per CTA, reduced into e[] with atomicMax.  Exponents of zeros
// (SENTINEL_EXP) sort below every finite one and non-finite values
// (NONFINITE_EXP) above, so a plain maximum carries both.  Each thread first
// reduces its own elements of a row; with K contiguous (t = 1) a warp owns a
// row and reduces it with one warp-wide max, so no shared-memory atomics
// collide.
template <typename T>
__global__ void __launch_bounds__(256) row_exp_kernel(const T* __restrict__ X, int64_t ld, int t, int64_t rows,
                                                      int64_t cols, int tri, int* __restrict__ e) {
  __shared__ int se[64];
  if (threadIdx.x < 64) se[threadIdx.x] = SENTINEL_EXP;
  __syncthreads();
  const int64_t i0 = (int64_t)blockIdx.x * 64, k0 = (int64_t)blockIdx.y * 64;
  auto ex_at = [&](int i, int k) -> int {
    const int64_t gi = i0 + i, gk = k0 + k;
    if (gi < rows && gk < cols && in_tri(tri, gi, gk)) return exp_of(to_double(X[mat_off(gi, gk, ld, t)]));
    return SENTINEL_EXP;
  };
  // The loops are unrolled so that every load of a thread is in flight at
  // once (the kernel is bound by memory-level parallelism).
  if (t) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int m[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) m[r] = max(ex_at(warp + 8 * r, lane), ex_at(warp + 8 * r, lane + 32));
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int v = __reduce_max_sync(0xffffffffu, m[r]);
      if (lane == 0) se[warp + 8 * r] = v;
    }
  } else {
    const int i = threadIdx.x & 63;
    int m = SENTINEL_EXP;
#pragma unroll
    for (int k = threadIdx.x >> 6, j = 0; j < 16; k += 4, ++j) m = max(m, ex_at(i, k));
    atomicMax(&se[i], m);
  }
  __syncthreads();
  if (threadIdx.x < 64 && i0 + threadIdx.x < rows && se[threadIdx.x] != SENTINEL_EXP)
    atomicMax(&e[i0 + threadIdx.x], se[threadIdx.x]);
}

// Two slice values (small integers held exactly in floats) packed for one
// 32-bit store.  A BF16 slice value has at most 8 significant bits, so its
// BF16 pattern is the upper half of its float pattern.
template <typename S> __device__ __forceinline__ uint32_t pack_slices(float a, float b);
template <> __device__ __forceinline__ uint32_t pack_slices<__nv_bfloat16>(float a, float b) {
  return (__float_as_uint(a) >> 16) | (__float_as_uint(b) & 0xFFFF0000u);
}
template <> __device__ __forceinline__ uint32_t pack_slices<__half>(float a, float b) {
  return (uint32_t)__half_as_ushort(__float2half_rn(a)) | ((uint32_t)__half_as_ushort(__float2half_rn(b)) << 16);
}

// Two adjacent slice values packed for one 32-bit store.
template <typename S> __device__ __forceinline__ uint32_t pack2(S a, S b) {
  return (uint32_t)__builtin_bit_cast(uint16_t, a) | ((uint32_t)__builtin_bit_cast(uint16_t, b) << 16);
}

// x * 2^(62 - ex) rounded to an integer (0 for zeros, non-finite values and
// rows without a finite element), from the FP64 bit pattern.
__device__ __forceinline__ long long fixed_of(double x, int ex) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int biased = (int)((b >> 52) & 0x7FF);
  const unsigned long long mant = b & ((1ull << 52) - 1);
  long long Y = 0;
  if (biased != 0x7FF && ex != NONFINITE_EXP && ex != SENTINEL_EXP && (biased != 0 || mant != 0)) {
    const unsigned long long m = biased ? (mant | (1ull << 52)) : mant;
    const int eb = biased ? biased : 1;
    const int sh = eb - 1013 - ex;  // Y = m * 2^sh = x * 2^(62 - ex)
    if (sh >= 0) Y = (long long)(m << sh);
    else if (sh > -63) Y = (long long)((m + (1ull << (-sh - 1))) >> (-sh));
    if (b >> 63) Y = -Y;
  }
  return Y;
}

// Split a rows x cols view into NS K-major slices of type Sl (rows padded to
// rows_pad, K padded to cols_pad, zeros in the padding and outside the staged
// triangle).  Layout: the slices of one 128-row tile are adjacent, row
// (t * NS + sl) * 128 + r holding row t * 128 + r of slice sl, so that one
// TMA box of 256 rows brings slices sl and sl + 1 of a tile.  The slices are the integers s_p of
//   x = 2^e[row] * sum_p s_p 2^(-beta p),  beta = 8 (BF16) or 11 (FP16),
// peeled from the top of the 63-bit fixed-point value with round-to-nearest
// so that |s_p| <= 2^(beta-1).  NS = 0 stages the element itself (a Float16
// operand of the plain path).  The slice count and width are compile-time
// constants, so every shift is an immediate; each thread produces two
// adjacent K values and writes them with one 32-bit store per slice.
// When nrm is not null, nrm[row] accumulates sum_k sum_p |s_p| 2^(-beta p),
// which bounds every partial sum of slice products along that row (in units
// of the row's scale 2^e) for a partner whose elements are below 1/2.
// Loads of one 32 x 64 tile (rows i0.., K k0..) of a rows x cols view: eight
// per thread, all in flight before any is used (the staging kernels are bound
// by memory-level parallelism, not by their integer work).  Zeros outside
// the view and outside the staged triangle.
template <typename T>
__device__ __forceinline__ void load_tile(const T* __restrict__ X, int64_t ld, int t, int64_t rows, int64_t cols,
                                          int tri, int64_t i0, int64_t k0, double (&v)[8]) {
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int idx = threadIdx.x + 256 * j;
    int i, k;
    if (!t) { i = idx & 31; k = idx >> 5; } else { k = idx & 63; i = idx >> 6; }
    const int64_t gi = i0 + i, gk = k0 + k;
    v[j] = (gi < rows && gk < cols && in_tri(tri, gi, gk)) ? to_double(X[mat_off(gi, gk, ld, t)]) : 0.0;
  }
}

__device__ __forceinline__ void store_tile(double (*tile)[65], int t, const double (&v)[8]) {
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int idx = threadIdx.x + 256 * j;
    int i, k;
    if (!t) { i = idx & 31; k = idx >> 5; } else { k = idx & 63; i = idx >> 6; }
    tile[i][k] = v[j];
  }
}

// Split the 32 x 64 tile in `tile` (rows i0.., K k0..) into NS K-major slices
// of type Sl.  Layout: the slices of one 128-row tile are adjacent, row
// (t * NS + sl) * 128 + r holding row t * 128 + r of slice sl, so that one
// TMA box of 256 rows brings slices sl and sl + 1 of a tile.  The slices are
// the integers s_p of
//   x = 2^ex[row] * sum_p s_p 2^(-beta p),  beta = 8 (BF16) or 11 (FP16),
// with |s_p| <= 2^(beta-1).  NS = 0 stages the element itself (a Float16
// operand of the plain path).  The slice count and width are compile-time
// constants, so every shift is an immediate; each thread produces two
// adjacent K values and writes them with one 32-bit store per slice.  Warp w
// handles rows w, w + 8, w + 16 and w + 24; mag[r] returns, for the r-th of
// them, sum_k sum_p |s_p| 2^(-beta p) over the tile (on every lane).
template <typename Sl, int NS>
__device__ __forceinline__ void split_tile(const double (*tile)[65], int64_t i0, int64_t k0, int64_t rows,
                                           const int* ex_rows, Sl* __restrict__ out, int64_t cols_pad,
                                           float (&mag)[4], bool with_mag) {
  constexpr int BETA = std::is_same<Sl, __nv_bfloat16>::value ? 8 : 11;
  constexpr int NSL = NS == 0 ? 1 : NS;
  // One row per warp and pass (idx >> 5 is warp-uniform), two K values per lane.
#pragma unroll
  for (int pass = 0; pass < 4; ++pass) {
    const int idx = threadIdx.x + 256 * pass;
    const int i = idx >> 5, k = (idx & 31) * 2;
    const int64_t gi = i0 + i, gk = k0 + k;
    uint32_t* o = reinterpret_cast<uint32_t*>(out + ((gi >> 7) * NSL * 128 + (gi & 127)) * cols_pad + gk);
    mag[pass] = 0.0f;
    if constexpr (NS == 0) {
      *o = pack2<Sl>((Sl)(float)tile[i][k], (Sl)(float)tile[i][k + 1]);
    } else {
      const int ex = gi < rows ? ex_rows[i] : SENTINEL_EXP;
      // Balanced digits by bias: with Z = Y + sum_p 2^(beta-1) 2^(sigma_p)
      // + 2^(sigma_last - 1) and sigma_p = 62 - beta (p + 1), the digit
      // s_p = ((Z >> sigma_p) mod 2^beta) - 2^(beta-1) (the top digit keeps
      // all high bits) lies in [-2^(beta-1), 2^(beta-1)), and sum_p s_p
      // 2^(sigma_p) is Y rounded half up at 2^(sigma_last).  Each digit is a
      // constant shift and mask; |Y| < 2^61 keeps Z inside 64 bits.
      constexpr long long BIAS = [] {
        long long b = 1ll << (62 - BETA * NS - 1);
        for (int p = 0; p < NS; ++p) b += 1ll << (62 - BETA * (p + 1) + BETA - 1);
        return b;
      }();
      const long long z0 = fixed_of(tile[i][k], ex) + BIAS, z1 = fixed_of(tile[i][k + 1], ex) + BIAS;
      float m = 0.0f;
#pragma unroll
      for (int sl = 0; sl < NS; ++sl) {
        const int sigma = 62 - BETA * (sl + 1);
        constexpr int HALF = 1 << (BETA - 1);
        const int d0 = sl == 0 ? (int)(z0 >> sigma) - HALF : (int)((unsigned long long)z0 >> sigma & (2 * HALF - 1)) - HALF;
        const int d1 = sl == 0 ? (int)(z1 >> sigma) - HALF : (int)((unsigned long long)z1 >> sigma & (2 * HALF - 1)) - HALF;
        // Small integers as floats without a conversion instruction: the
        // integer added to the bit pattern of 1.5 * 2^23 lands in the
        // mantissa's last place.
        const float f0 = __int_as_float(0x4B400000 + d0) - 12582912.0f;
        const float f1 = __int_as_float(0x4B400000 + d1) - 12582912.0f;
        o[sl * (128 * cols_pad / 2)] = pack_slices<Sl>(f0, f1);
        // 2^(-beta (sl + 1)) built from its exponent bits (exact).
        if (with_mag) m += (fabsf(f0) + fabsf(f1)) * __int_as_float((127 - BETA * (sl + 1)) << 23);
      }
      if (with_mag)  // uniform over the launch
        for (int off = 16; off > 0; off >>= 1) m += __shfl_xor_sync(0xffffffffu, m, off);
      mag[pass] = m;
    }
  }
}

// Split a rows x cols view into NS K-major slices of type Sl (rows padded to
// rows_pad, K padded to cols_pad, zeros in the padding and outside the staged
// triangle), one 32 x 64 tile per CTA, with the row exponents e[] from
// row_exp_kernel.  When nrm is not null, nrm[row] accumulates
// sum_k sum_p |s_p| 2^(-beta p), which bounds every partial sum of slice
// products along that row (in units of the row's scale 2^e) for a partner
// whose elements are below 1/2.
template <typename T, typename Sl, int NS>
__global__ void __launch_bounds__(256) split_kernel(const T* __restrict__ X, int64_t ld, int t, int64_t rows,
                                                    int64_t cols, int tri, const int* __restrict__ e,
                                                    Sl* __restrict__ out, int64_t rows_pad, int64_t cols_pad,
                                                    float* __restrict__ nrm) {
  __shared__ double tile[32][65];
  const int64_t i0 = (int64_t)blockIdx.x * 32, k0 = (int64_t)blockIdx.y * 64;
  (void)rows_pad;
  double v[8];
  load_tile(X, ld, t, rows, cols, tri, i0, k0, v);
  store_tile(tile, t, v);
  __syncthreads();
  float mag[4];
  split_tile<Sl, NS>(tile, i0, k0, rows, e ? e + i0 : nullptr, out, cols_pad, mag, nrm != nullptr);
  if (NS != 0 && nrm && (threadIdx.x & 31) == 0) {
#pragma unroll
    for (int pass = 0; pass < 4; ++pass) {
      const int64_t gi = i0 + (threadIdx.x >> 5) + 8 * pass;
      if (gi < rows && mag[pass] > 0.0f) atomicAdd(&nrm[gi], mag[pass]);
    }
  }
}

// One operand of a fused staging launch.
struct StageJob {
  const double* X;
  int64_t ld;
  int t;
  int64_t rows, cols;
  int tri;
  int* e;
  void* out;
  int64_t cols_pad;
  float* nrm;
  int blocks;  // 32-row blocks: rows_pad / 32
};

// Both operands of one update staged by one launch, for short K: a CTA takes
// 32 rows of one operand, finds their exponents over the whole K range (the
// same maximum row_exp_kernel takes), then splits them tile by tile as
// split_kernel does (the second pass reads from L2), and writes e[] and
// nrm[] itself, so no memsets, no atomics and one launch replace the eight
// stream operations of two separately staged operands.
template <typename Sl, int NS>
__global__ void __launch_bounds__(256, 4) stage_pair_kernel(const StageJob a, const StageJob b) {
  __shared__ double tile[2][32][65];
  __shared__ int sred[8][32];
  __shared__ int sexp[32];
  const bool first = (int)blockIdx.x < a.blocks;
  const StageJob j = first ? a : b;
  const int64_t i0 = (int64_t)(first ? blockIdx.x : blockIdx.x - a.blocks) * 32;
  const int64_t ktiles = j.cols_pad / 64;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  // Pass 1: row exponents.  With t = 0 a thread's eight values lie in row
  // `lane`; with t = 1 in rows (threadIdx.x >> 6) + 4 q, q = 0..7.
  int m[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) m[q] = SENTINEL_EXP;
  for (int64_t kt = 0; kt < ktiles; ++kt) {
    double v[8];
    load_tile(j.X, j.ld, j.t, j.rows, j.cols, j.tri, i0, kt * 64, v);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int ex = exp_of(v[q]);  // zeros (and the padding) give SENTINEL_EXP
      if (j.t) m[q] = max(m[q], ex);
      else m[0] = max(m[0], ex);
    }
  }
  if (!j.t) {
    sred[warp][lane] = m[0];
  } else {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int r = __reduce_max_sync(0xffffffffu, m[q]);
      if (lane == 0) sred[warp][q] = r;  // rows (warp >> 1) + 4 q
    }
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int r = threadIdx.x;
    int mx = SENTINEL_EXP;
    if (!j.t) {
#pragma unroll
      for (int w = 0; w < 8; ++w) mx = max(mx, sred[w][r]);
    } else {
      const int g = r & 3, q = r >> 2;  // row r = g + 4 q, read by warps 2g and 2g + 1
      mx = max(sred[2 * g][q], sred[2 * g + 1][q]);
    }
    sexp[r] = mx;
    if (i0 + r < j.rows) j.e[i0 + r] = mx;
    else j.e[i0 + r] = SENTINEL_EXP;
  }
  __syncthreads();

  // Pass 2: the split, two tile buffers so that one barrier per tile orders
  // both the tile's writes before its reads and the previous reads before
  // the next writes.
  float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  Sl* out = static_cast<Sl*>(j.out);
  for (int64_t kt = 0; kt < ktiles; ++kt) {
    double v[8];
    load_tile(j.X, j.ld, j.t, j.rows, j.cols, j.tri, i0, kt * 64, v);
    store_tile(tile[kt & 1], j.t, v);
    __syncthreads();
    float mag[4];
    split_tile<Sl, NS>(tile[kt & 1], i0, kt * 64, j.rows, sexp, out, j.cols_pad, mag, j.nrm != nullptr);
#pragma unroll
    for (int pass = 0; pass < 4; ++pass) acc[pass] += mag[pass];
  }
  if (lane == 0 && j.nrm) {
#pragma unroll
    for (int pass = 0; pass < 4; ++pass) j.nrm[i0 + warp + 8 * pass] = i0 + warp + 8 * pass < j.rows ? acc[pass] : 0.0f;
  }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

int make_map(CUtensorMap* map, const void* base, bool bf16, uint64_t cols_pad, uint64_t total_rows,
             uint32_t box_rows = BM) {
  auto fn = encode_fn();
  if (!fn) return fail(NLA_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available from the driver");
  if ((reinterpret_cast<uintptr_t>(base) & 15) != 0) return fail(NLA_ERR_ARG, "staged operand is not 16-byte aligned");
  cuuint64_t dims[2] = {cols_pad, total_rows};
  cuuint64_t strides[1] = {cols_pad * 2};
  cuuint32_t box[2] = {BK, box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2,
                  const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(NLA_ERR_ARG, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return NLA_OK;
}

// Stream-ordered, grow-only workspace per (device, stream).
struct Pool {
  void* ptr = nullptr;
  size_t size = 0;
};
std::mutex g_pool_mu;
std::unordered_map<uint64_t, Pool> g_pools;

int64_t pad_to(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

// Raise the dynamic shared-memory limit of one kernel instantiation (once per
// process; a single GPU is used).  The limit must leave room for the kernel's
// static shared memory, so it is set to what the launches actually use.
constexpr int GEMM_DYN_SMEM = 200 * 1024;

// TMA-issuing warps of the fast tensor-core kernel (NLA_GEMM_PRODUCERS = 1
// or 2, default 2; read once).
int gemm_producers() {
  static const int n = [] {
    const char* v = getenv("NLA_GEMM_PRODUCERS");
    return v && v[0] == '1' && v[1] == 0 ? 1 : 2;
  }();
  return n;
}

template <int EPI>
int ensure_gemm_smem() {
  static std::once_flag once;
  static cudaError_t status = cudaSuccess;
  std::call_once(once, [] {
    status = cudaFuncSetAttribute(umma_gemm_kernel<EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, GEMM_DYN_SMEM);
  });
  return status == cudaSuccess ? NLA_OK : cuda_status(status, "cudaFuncSetAttribute(umma_gemm_kernel)");
}

int ensure_exact_smem() {
  static std::once_flag once;
  static cudaError_t status = cudaSuccess;
  std::call_once(once, [] {
    status = cudaFuncSetAttribute(umma_exact_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, EX_DYN_SMEM);
  });
  return status == cudaSuccess ? NLA_OK : cuda_status(status, "cudaFuncSetAttribute(umma_exact_kernel)");
}

// Exact-kernel variant (NLA_EXACT_KERNEL, read once): "coupled" (pairs
// sharing a B tile, the default) or "pairs" (pair by pair).
bool exact_coupled() {
  static const bool on = [] {
    const char* e = getenv("NLA_EXACT_KERNEL");
    return !(e && !strcmp(e, "pairs"));
  }();
  return on;
}

// Fixed-point sums applied to C by exact_finish_kernel (NLA_EXACT_FINISH=0
// applies them in the exact kernel's epilogue instead; read per launch).
bool exact_finish_enabled() {
  const char* v = getenv("NLA_EXACT_FINISH");
  return !(v && v[0] == '0');
}

// Short-K group table of the coupled kernel (NLA_EXACT_MERGED=0 turns it
// off; read per launch, so that tests can compare both tables).
bool exact_merged_enabled() {
  const char* v = getenv("NLA_EXACT_MERGED");
  return !(v && v[0] == '0');
}

int launch_exact_coupled(const ExactParams& params, const Staged& A, const Staged& B, cudaStream_t s) {
  ExactParams p = params;
  p.merged = A.K_pad <= CP_MERGED_MAX_K && exact_merged_enabled() ? 1 : 0;
  CUtensorMap mA, mB, mB2;
  NLA_TRY(make_map(&mA, A.slices, true, (uint64_t)A.K_pad, (uint64_t)(EX_SLICES * A.rows_pad)));
  NLA_TRY(make_map(&mB, B.slices, true, (uint64_t)B.K_pad, (uint64_t)(EX_SLICES * B.rows_pad)));
  NLA_TRY(make_map(&mB2, B.slices, true, (uint64_t)B.K_pad, (uint64_t)(EX_SLICES * B.rows_pad), 2 * BN));
  static std::once_flag once;
  static cudaError_t st = cudaSuccess;
  std::call_once(once, [] {
    st = cudaFuncSetAttribute(umma_exact_coupled_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, CP_DYN_SMEM);
  });
  if (st != cudaSuccess) return cuda_status(st, "cudaFuncSetAttribute(umma_exact_coupled_kernel)");
  const int64_t grid = (int64_t)p.tiles_m * p.tiles_n;
  if (grid > 2147483647LL) return fail(NLA_ERR_UNSUPPORTED, "too many output tiles");
  umma_exact_coupled_kernel<<<(unsigned)grid, EX_THREADS, CP_DYN_SMEM, s>>>(mA, mB, mB2, p);
  NLA_CHECK_LAUNCH("umma_exact_coupled_kernel");
  return NLA_OK;
}

int launch_exact_pairs(const ExactParams& p, const Staged& A, const Staged& B, cudaStream_t s) {
  CUtensorMap mA, mB;
  NLA_TRY(make_map(&mA, A.slices, true, (uint64_t)A.K_pad, (uint64_t)(EX_SLICES * A.rows_pad)));
  NLA_TRY(make_map(&mB, B.slices, true, (uint64_t)B.K_pad, (uint64_t)(EX_SLICES * B.rows_pad)));
  NLA_TRY(ensure_exact_smem());
  const int64_t grid = (int64_t)p.tiles_m * p.tiles_n;
  if (grid > 2147483647LL) return fail(NLA_ERR_UNSUPPORTED, "too many output tiles");
  umma_exact_kernel<<<(unsigned)grid, EX_THREADS, EX_DYN_SMEM, s>>>(mA, mB, p);
  NLA_CHECK_LAUNCH("umma_exact_kernel");
  return NLA_OK;
}

}  // namespace

int workspace_get(cudaStream_t s, size_t bytes, void** out) {
  int dev = 0;
  cudaGetDevice(&dev);
  const uint64_t key = ((uint64_t)(uint32_t)dev << 48) ^ (uint64_t)reinterpret_cast<uintptr_t>(s);
  std::lock_guard<std::mutex> lk(g_pool_mu);
  Pool& p = g_pools[key];
  if (p.size < bytes) {
    if (p.ptr) cudaFreeAsync(p.ptr, s);
    p.ptr = nullptr;
    p.size = 0;
    size_t want = bytes + bytes / 8 + (1 << 20);
    cudaError_t e = cudaMallocAsync(&p.ptr, want, s);
    if (e != cudaSuccess) {
      p.ptr = nullptr;
      return cuda_status(e, "workspace allocation");
    }
    p.size = want;
  }
  *out = p.ptr;
  return NLA_OK;
}

size_t staged_bytes(int64_t rows, int64_t K, int S) {
  const int64_t Rp = pad_to(rows, BM), Kp = pad_to(K, BK);
  size_t b = (size_t)S * (size_t)Rp * (size_t)Kp * 2;
  b = (b + 1023) & ~(size_t)1023;
  b += ((size_t)Rp * sizeof(int) + 1023) & ~(size_t)1023;
  b += ((size_t)Rp * sizeof(float) + 1023) & ~(size_t)1023;
  return b;
}

// The layout of a staged operand in `buf` (see staged_bytes).
void staged_layout(void* buf, int64_t rows, int64_t K, int S, bool bf16, bool copy, int tri, Staged* out) {
  const int64_t Rp = pad_to(rows, BM), Kp = pad_to(K, BK);
  uint8_t* w = static_cast<uint8_t*>(buf);
  out->slices = w;
  out->e = reinterpret_cast<int*>(w + (((size_t)S * Rp * Kp * 2 + 1023) & ~(size_t)1023));
  out->nrm = reinterpret_cast<float*>(reinterpret_cast<uint8_t*>(out->e) +
                                      (((size_t)Rp * sizeof(int) + 1023) & ~(size_t)1023));
  out->rows = rows;
  out->rows_pad = Rp;
  out->K = K;
  out->K_pad = Kp;
  out->S = S;
  out->bf16 = copy ? false : bf16;
  out->tri = tri;
  out->scaled = !copy;
}

int stage_operand(const Mat& X, int64_t rows, int64_t K, int in_dtype, int S, bool bf16, int tri, void* buf,
                  Staged* out, cudaStream_t s, bool want_nrm) {
  const bool copy = in_dtype == NLA_F16;
  const int beta = bf16 ? 8 : 11;
  if (copy) S = 1;
  if (S < 1 || 62 - beta * S < 1) return fail(NLA_ERR_ARG, "too many slices for the slice width");
  const int64_t Rp = pad_to(rows, BM), Kp = pad_to(K, BK);
  staged_layout(buf, rows, K, S, bf16, copy, tri, out);
  TraceScope trace(NLA_K_SPLIT, s, 0.0,
                   (double)rows * (double)K * (double)dtype_size(in_dtype) * (copy ? 1 : 2) + (double)S * Rp * Kp * 2);
  const dim3 gs((unsigned)(Rp / 32), (unsigned)(Kp / 64));
  if (copy) {
    split_kernel<__half, __half, 0><<<gs, 256, 0, s>>>((const __half*)X.p, X.ld, X.t, rows, K, tri, nullptr,
                                                       (__half*)out->slices, Rp, Kp, nullptr);
    NLA_CHECK_LAUNCH("split_kernel");
    return NLA_OK;
  }
  cudaMemsetAsync(out->e, 0x80, (size_t)Rp * sizeof(int), s);
  // The row-magnitude sums bound the exact kernel's fixed point for its A
  // operand; nothing reads them for a B operand or in the fast mode.
  if (want_nrm) cudaMemsetAsync(out->nrm, 0, (size_t)Rp * sizeof(float), s);
  else out->nrm = nullptr;
  const dim3 ge((unsigned)((rows + 63) / 64), (unsigned)((K + 63) / 64));
  row_exp_kernel<double><<<ge, 256, 0, s>>>((const double*)X.p, X.ld, X.t, rows, K, tri, out->e);
  NLA_CHECK_LAUNCH("row_exp_kernel");
  const double* xp = static_cast<const double*>(X.p);
  if (bf16) {
    auto* o = static_cast<__nv_bfloat16*>(out->slices);
    switch (S) {
      case 1: split_kernel<double, __nv_bfloat16, 1><<<gs, 256, 0, s>>>(xp, X.ld, X.t, rows, K, tri, out->e, o, Rp, Kp, out->nrm); break;
      case 2: split_kernel<double, __nv_bfloat16, 2><<<gs, 256, 0, s>>>(xp, X.ld, X.t, rows, K, tri, out->e, o, Rp, Kp, out->nrm); break;
      case 3: split_kernel<double, __nv_bfloat16, 3><<<gs, 256, 0, s>>>(xp, X.ld, X.t, rows, K, tri, out->e, o, Rp, Kp, out->nrm); break;
      case EXACT_SLICES: split_kernel<double, __nv_bfloat16, EXACT_SLICES><<<gs, 256, 0, s>>>(xp, X.ld, X.t, rows, K, tri, out->e, o, Rp, Kp, out->nrm); break;
      default: return fail(NLA_ERR_ARG, "BF16 slices: 1, 2, 3 or 7 terms");
    }
  } else {
    auto* o = static_cast<__half*>(out->slices);
    switch (S) {
      case 1: split_kernel<double, __half, 1><<<gs, 256, 0, s>>>(xp, X.ld, X.t, rows, K, tri, out->e, o, Rp, Kp, out->nrm); break;
      case 2: split_kernel<double, __half, 2><<<gs, 256, 0, s>>>(xp, X.ld, X.t, rows, K, tri, out->e, o, Rp, Kp, out->nrm); break;
      case 3: split_kernel<double, __half, 3><<<gs, 256, 0, s>>>(xp, X.ld, X.t, rows, K, tri, out->e, o, Rp, Kp, out->nrm); break;
      default: return fail(NLA_ERR_ARG, "FP16 slices: 1, 2 or 3 terms");
    }
  }
  NLA_CHECK_LAUNCH("split_kernel");
  trace_kernels(1);  // row_exp_kernel and split_kernel
  return NLA_OK;
}

// Fused staging of both operands of one Float64 update (stage_pair_kernel)
// for K up to FUSED_STAGE_MAX_K; NLA_STAGE_FUSED=0 turns it off (read per
// update, so that tests can compare both paths in one process).
constexpr int64_t FUSED_STAGE_MAX_K = 256;  // measured: slower than the separate kernels from K = 512
bool stage_fused_enabled() {
  const char* v = getenv("NLA_STAGE_FUSED");
  return !(v && v[0] == '0');
}

int stage_pair(const Mat& A, int64_t M, const Mat& Bt, int64_t N, int64_t K, int S, bool bf16, void* bufA,
               void* bufB, Staged* As, Staged* Bs, cudaStream_t s) {
  staged_layout(bufA, M, K, S, bf16, false, 0, As);
  staged_layout(bufB, N, K, S, bf16, false, 0, Bs);
  auto job = [](const Mat& X, const Staged& st) {
    StageJob j{};
    j.X = static_cast<const double*>(X.p);
    j.ld = X.ld;
    j.t = X.t;
    j.rows = st.rows;
    j.cols = st.K;
    j.tri = 0;
    j.e = st.e;
    j.out = st.slices;
    j.cols_pad = st.K_pad;
    j.nrm = st.nrm;
    j.blocks = (int)(st.rows_pad / 32);
    return j;
  };
  StageJob ja = job(A, *As), jb = job(Bt, *Bs);
  jb.nrm = nullptr;  // only the A operand's row-magnitude sums are read (exact kernel)
  Bs->nrm = nullptr;
  if (S != EXACT_SLICES) {
    ja.nrm = nullptr;
    As->nrm = nullptr;
  }
  const int64_t grid = (int64_t)ja.blocks + jb.blocks;
  if (grid > 2147483647LL) return fail(NLA_ERR_UNSUPPORTED, "operand too large");
  TraceScope trace(NLA_K_SPLIT, s, 0.0,
                   (double)(M + N) * (double)K * 16.0 + (double)S * (As->rows_pad + Bs->rows_pad) * As->K_pad * 2);
  if (bf16) {
    switch (S) {
      case 1: stage_pair_kernel<__nv_bfloat16, 1><<<(unsigned)grid, 256, 0, s>>>(ja, jb); break;
      case 2: stage_pair_kernel<__nv_bfloat16, 2><<<(unsigned)grid, 256, 0, s>>>(ja, jb); break;
      case 3: stage_pair_kernel<__nv_bfloat16, 3><<<(unsigned)grid, 256, 0, s>>>(ja, jb); break;
      case EXACT_SLICES: stage_pair_kernel<__nv_bfloat16, EXACT_SLICES><<<(unsigned)grid, 256, 0, s>>>(ja, jb); break;
      default: return fail(NLA_ERR_ARG, "BF16 slices: 1, 2, 3 or 7 terms");
    }
  } else {
    switch (S) {
      case 1: stage_pair_kernel<__half, 1><<<(unsigned)grid, 256, 0, s>>>(ja, jb); break;
      case 2: stage_pair_kernel<__half, 2><<<(unsigned)grid, 256, 0, s>>>(ja, jb); break;
      case 3: stage_pair_kernel<__half, 3><<<(unsigned)grid, 256, 0, s>>>(ja, jb); break;
      default: return fail(NLA_ERR_ARG, "FP16 slices: 1, 2 or 3 terms");
    }
  }
  NLA_CHECK_LAUNCH("stage_pair_kernel");
  return NLA_OK;
}

// Exact updates also hold their fixed-point sums, rows padded to 128.
size_t fixed_sums_bytes(int64_t M, int64_t N) { return (size_t)pad_to(M, BM) * (size_t)N * sizeof(long long); }

size_t sliced_workspace_bytes(int64_t M, int64_t N, int64_t K, int S) {
  return staged_bytes(M, K, S) + staged_bytes(N, K, S) + 1024 + (S == EXACT_SLICES ? fixed_sums_bytes(M, N) : 0);
}

// One tensor-core update.  in_dtype is NLA_F64 (split into S slices of BF16
// or FP16) or NLA_F16 (S = 1, staged as is).  out_dtype is NLA_F64 or NLA_F16.
int launch_sliced_gemm(int64_t M, int64_t N, int64_t K, double alpha, const Mat& A, const Mat& B, const Mat& C,
                       int in_dtype, int out_dtype, int S, bool bf16, void* ws, size_t ws_bytes, cudaStream_t s) {
  if (M <= 0 || N <= 0 || K <= 0) return NLA_OK;
  if (C.t) return fail(NLA_ERR_UNSUPPORTED, "tensor-core update: transposed output view");
  const bool copy = in_dtype == NLA_F16;
  if (copy) S = 1;
  if (S == EXACT_SLICES && !copy) {
    // Exact slice products (FP64-accurate update).
    if (!bf16) return fail(NLA_ERR_ARG, "exact updates use BF16 slices");
    if (out_dtype != NLA_F64) return fail(NLA_ERR_DTYPE, "exact updates produce Float64");
    const size_t sa = staged_bytes(M, K, S), sb = staged_bytes(N, K, S), need = sa + sb + 1024;
    void* base = ws;
    if (base == nullptr) {
      NLA_TRY(workspace_get(s, need + fixed_sums_bytes(M, N), &base));
      ws_bytes = need + fixed_sums_bytes(M, N);
    } else if (ws_bytes < need) {
      return fail(NLA_ERR_WORKSPACE, "workspace too small for the exact update");
    }
    // The fixed-point sums follow the staged operands when the workspace has
    // room for them (a caller's fixed workspace may not).
    long long* fixed = ws_bytes >= need + fixed_sums_bytes(M, N)
                           ? reinterpret_cast<long long*>(static_cast<uint8_t*>(base) + ((sa + sb + 1023) & ~(size_t)1023))
                           : nullptr;
    Staged As, Bs;
    if (K <= FUSED_STAGE_MAX_K && stage_fused_enabled()) {
      NLA_TRY(stage_pair(A, M, transposed(B), N, K, S, true, base, static_cast<uint8_t*>(base) + sa, &As, &Bs, s));
    } else {
      NLA_TRY(stage_operand(A, M, K, NLA_F64, S, true, 0, base, &As, s));
      NLA_TRY(stage_operand(transposed(B), N, K, NLA_F64, S, true, 0, static_cast<uint8_t*>(base) + sa, &Bs, s,
                            false));
    }
    return launch_exact_gemm(As, Bs, alpha, C, false, s, nullptr, fixed);
  }
  if (S < 1 || S > 3) return fail(NLA_ERR_ARG, "split terms must be 1, 2, 3 or 7");
  const int beta = bf16 ? 8 : 11;
  const int64_t Mp = pad_to(M, BM), Np = pad_to(N, BN), Kp = pad_to(K, BK);
  if (S * Mp > 0xFFFFFFFFLL || S * Np > 0xFFFFFFFFLL) return fail(NLA_ERR_UNSUPPORTED, "operand too large");
  const size_t need = sliced_workspace_bytes(M, N, K, S);
  void* base = ws;
  if (base == nullptr) {
    NLA_TRY(workspace_get(s, need, &base));
  } else if (ws_bytes < need) {
    return fail(NLA_ERR_WORKSPACE, "workspace too small for the tensor-core update");
  }
  Staged As, Bs;
  // N x K view: row j is column j of op(B)
  if (!copy && K <= FUSED_STAGE_MAX_K && stage_fused_enabled()) {
    NLA_TRY(stage_pair(A, M, transposed(B), N, K, S, bf16, base, static_cast<uint8_t*>(base) + staged_bytes(M, K, S),
                       &As, &Bs, s));
  } else {
    NLA_TRY(stage_operand(A, M, K, in_dtype, S, bf16, 0, base, &As, s, false));
    NLA_TRY(stage_operand(transposed(B), N, K, in_dtype, S, bf16, 0,
                          static_cast<uint8_t*>(base) + staged_bytes(M, K, S), &Bs, s, false));
  }

  const bool use_bf16 = As.bf16;
  CUtensorMap mA, mB;
  NLA_TRY(make_map(&mA, As.slices, use_bf16, (uint64_t)Kp, (uint64_t)(S * Mp)));
  NLA_TRY(make_map(&mB, Bs.slices, use_bf16, (uint64_t)Kp, (uint64_t)(S * Np)));

  GemmParams p{};
  p.M = (int)M;
  p.N = (int)N;
  p.num_kb = (int)(Kp / BK);
  p.tiles_m = (int)(Mp / BM);
  p.tiles_n = (int)(Np / BN);
  p.a_rows = (int)Mp;
  p.b_rows = (int)Np;
  p.sa = S;
  p.sb = S;
  p.producers = gemm_producers();
  p.stage_bytes = 2 * S * TILE_BYTES;
  p.stages = (GEMM_DYN_SMEM - 1024 - 256) / p.stage_bytes;
  if (p.stages > 6) p.stages = 6;
  // Slice pairs (a, b) with a + b <= S - 1 (0-based), grouped by weight.
  p.npairs = 0;
  p.nacc = S;
  for (int t = 0; t < S; ++t) {
    p.acc_w[t] = ldexpf(1.0f, -beta * t);
    for (int a = 0; a <= t; ++a) {
      const int b = t - a;
      p.pair_a[p.npairs] = (int8_t)a;
      p.pair_b[p.npairs] = (int8_t)b;
      p.pair_acc[p.npairs] = (int8_t)t;
      p.pair_first[p.npairs] = (int8_t)(a == 0);
      ++p.npairs;
    }
  }
  uint32_t cols = 32;
  while (cols < (uint32_t)(p.nacc * BN)) cols <<= 1;
  p.tmem_cols = cols;
  p.idesc = umma::idesc_f16(BM, BN, use_bf16);
  p.C = C.p;
  p.ldc = C.ld;
  p.alpha = alpha;
  p.ea = copy ? nullptr : As.e;
  p.eb = copy ? nullptr : Bs.e;
  p.exp_bias = copy ? 0 : -2 * beta;

  const int smem = p.stages * p.stage_bytes + 1024 + 256;
  const int64_t grid = (int64_t)p.tiles_m * p.tiles_n;
  if (grid > 2147483647LL) return fail(NLA_ERR_UNSUPPORTED, "too many output tiles");
  const double pair_flops = 2.0 * (double)M * (double)N * (double)K;
  TraceScope trace(NLA_K_GEMM_UMMA, s, pair_flops * p.npairs,
                   (double)S * (Mp + Np) * Kp * 2 + 2.0 * (double)M * N * (double)dtype_size(out_dtype));
  if (smem > GEMM_DYN_SMEM) return fail(NLA_ERR_UNSUPPORTED, "tensor-core update: shared memory plan too large");
  if (out_dtype == NLA_F64) {
    NLA_TRY(ensure_gemm_smem<EPI_F64>());
    umma_gemm_kernel<EPI_F64><<<(unsigned)grid, GEMM_THREADS, smem, s>>>(mA, mB, p);
  } else if (out_dtype == NLA_F16) {
    NLA_TRY(ensure_gemm_smem<EPI_F16>());
    umma_gemm_kernel<EPI_F16><<<(unsigned)grid, GEMM_THREADS, smem, s>>>(mA, mB, p);
  } else {
    return fail(NLA_ERR_DTYPE, "tensor-core update: unsupported output type");
  }
  NLA_CHECK_LAUNCH("umma_gemm_kernel");
  return NLA_OK;
}

// C (M x N, FP64) += alpha * A * B^T from two operands staged with
// EX_SLICES BF16 slices (A: M rows, B: N rows, same K).
int launch_exact_gemm(const Staged& A, const Staged& B, double alpha, const Mat& C, bool trans_out,
                      cudaStream_t s, const ResidualTerm* res, long long* fixed_buf) {
  const int64_t M = A.rows, N = B.rows, K = A.K;
  if (M <= 0 || N <= 0 || K <= 0) return NLA_OK;
  if (B.K != K || A.S != EX_SLICES || B.S != EX_SLICES || !A.bf16 || !B.bf16 || !A.scaled || !B.scaled)
    return fail(NLA_ERR_ARG, "exact update: operands not staged for it");
  if (C.t) return fail(NLA_ERR_UNSUPPORTED, "exact update: transposed output view");
  if (K > (1LL << 30)) return fail(NLA_ERR_UNSUPPORTED, "exact update: K too large");
  ExactParams p{};
  p.M = (int)M;
  p.N = (int)N;
  p.K = (int)K;
  p.tiles_m = (int)(A.rows_pad / BM);
  p.tiles_n = (int)(B.rows_pad / BN);
  p.a_rows = (int)A.rows_pad;
  p.b_rows = (int)B.rows_pad;
  p.npairs = 0;
  for (int t = 0; t < EX_SLICES; ++t)
    for (int a = 0; a <= t; ++a) {
      p.pa[p.npairs] = (int8_t)a;
      p.pb[p.npairs] = (int8_t)(t - a);
      ++p.npairs;
    }
  p.tri_a = A.tri;
  p.tri_b = B.tri;
  p.trans_out = trans_out ? 1 : 0;
  p.nrm_a = A.nrm;
  if (res) {
    p.res_x = res->x;
    p.res_ldx = res->ldx;
    p.res_d = res->d;
    p.res_dstride = res->dstride;
  }
  p.C = C.p;
  p.ldc = C.ld;
  p.alpha = alpha;
  p.ea = A.e;
  p.eb = B.e;
  // Executed flops of the slice pairs: 2 M N K per pair, half of that when
  // one operand is a staged triangle (its tiles' K ranges are clipped).
  const double tri_frac = (A.tri != 0 || B.tri != 0) ? 0.5 : 1.0;
  TraceScope trace(NLA_K_GEMM_UMMA, s, 2.0 * (double)M * N * (double)K * p.npairs * tri_frac,
                   (double)EX_SLICES * (A.rows_pad + B.rows_pad) * A.K_pad * 2 + 16.0 * (double)M * N);
  // Plain updates leave their fixed-point sums in fixed_buf (A.rows_pad x N)
  // for exact_finish_kernel; residuals and transposed outputs are applied by
  // the exact kernel itself.
  if (fixed_buf && !res && !trans_out && exact_finish_enabled() && (N + FINISH_COLS - 1) / FINISH_COLS <= 65535) {
    p.P = fixed_buf;
    p.ldp = A.rows_pad;
  }
  const int rc = exact_coupled() ? launch_exact_coupled(p, A, B, s) : launch_exact_pairs(p, A, B, s);
  if (rc != NLA_OK || !p.P) return rc;
  const int64_t gy = (N + FINISH_COLS - 1) / FINISH_COLS;
  exact_finish_kernel<<<dim3((unsigned)((M + 255) / 256), (unsigned)gy), 256, 0, s>>>(p);
  NLA_CHECK_LAUNCH("exact_finish_kernel");
  trace_kernels(1);  // the exact kernel and its finishing pass
  return NLA_OK;
}

namespace {
std::atomic<uint64_t> g_wait_limit_host{umma::WAIT_LIMIT_NS};
}

int set_wait_limit(uint64_t ns) {
  const uint64_t v = ns == 0 ? umma::WAIT_LIMIT_NS : ns;
  const cudaError_t e = cudaMemcpyToSymbol(umma::g_wait_limit_ns, &v, sizeof(v));
  if (e != cudaSuccess) return cuda_status(e, "set wait limit");
  g_wait_limit_host.store(v);
  return NLA_OK;
}

uint64_t wait_limit_ns() { return g_wait_limit_host.load(); }

// Reads and clears the device error word after synchronising the stream.
int* device_error_word() {
  void* p = nullptr;
  return cudaGetSymbolAddress(&p, g_device_error) == cudaSuccess ? static_cast<int*>(p) : nullptr;
}

int device_status(cudaStream_t s) {
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(e, "stream synchronize");
  int v = 0;
  e = cudaMemcpyFromSymbol(&v, g_device_error, sizeof(int));
  if (e != cudaSuccess) return cuda_status(e, "read device status");
  if (v != 0) {
    int zero = 0;
    cudaMemcpyToSymbol(g_device_error, &zero, sizeof(int));
  }
  const int vb = batch_device_error();
  if (v != 0) return fail(NLA_ERR_TIMEOUT, "a bounded device-side wait gave up (site " + std::to_string(v) + ")");
  if (vb != 0)
    return fail(NLA_ERR_TIMEOUT, "a batched dependency wait gave up (site " + std::to_string(vb) + ")");
  return NLA_OK;
}

}  // namespace nla
