// Exact 7-slice splitting of Float64 values into BF16 digit slices, with
// integer arithmetic on the bit patterns (no FP64 instruction), shared by
// the kernels that stage their own operands in shared memory for tcgen05.mma
// (the batched residual and the leaf products of the mixed solve).
//
// A row (or column) of values is scaled by 2^-e, e from its largest exponent
// field, so that every |v 2^-e| < 1/2; y = round(v 2^(56 - e)) is then a
// 56-bit fixed-point integer and its seven balanced 8-bit digits,
// y = sum_p d_p 2^(8 (6 - p)) with |d_p| <= 128, are exact in BF16.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace nla {
namespace split7 {

constexpr int SLICES = 7;
constexpr int NONFINITE = 0x7FFFFFFF;  // scale exponent of a row or column holding Inf or NaN

// Biased exponent field of a double.
__device__ __forceinline__ int exp_field(double v) { return (__double2hiint(v) >> 20) & 0x7FF; }

// Scale exponent e of a row or column from the largest biased exponent of
// its elements: |v| < 2^(e - 1) for all of them (0 when all are zero or
// subnormal, NONFINITE when one is Inf or NaN).
__device__ __forceinline__ int scale_exp(int bmax) {
  return bmax == 0x7FF ? NONFINITE : (bmax == 0 ? 0 : bmax - 1021);
}

// y = round(v 2^(56 - e)) from the bits of v (|v| < 2^(e - 1), so |y| < 2^55;
// subnormals, Inf and NaN give 0).
__device__ __forceinline__ long long fixed56(double v, int e) {
  const long long b = __double_as_longlong(v);
  const int be = (int)((b >> 52) & 0x7FF);
  if (be == 0 || be == 0x7FF || e == NONFINITE) return 0;
  const long long m = (b & 0xFFFFFFFFFFFFFll) | (1ll << 52);
  const int s = be - 1019 - e;  // y = m 2^s, s <= 2
  const long long y = s >= 0 ? (m << s) : (s > -62 ? ((m + (1ll << (-s - 1))) >> (-s)) : 0ll);
  return b < 0 ? -y : y;
}

// FP32 bit pattern of byte `sel` of w minus 128, an exact small integer:
// 0x4B4000uu is 2^23 + 2^22 + uu as a float.
__device__ __forceinline__ uint32_t digit_f32(uint32_t w, uint32_t sel) {
  return __float_as_uint(__uint_as_float(__byte_perm(w, 0x4B4000u, 0x6540u + sel)) - 12583040.0f);
}

// 8 values (k = 8 j .. 8 j + 7 of a row), as fixed-point integers y, stored
// as 7 BF16 slices of one 16-byte chunk each.  The balanced digits are the
// bytes of y + 0x0080808080808080 minus 128 (the top digit: bits 48 and up),
// so no carries need propagating; an integer |d| <= 256 is exact in BF16,
// which is the upper half of its FP32 pattern.
__device__ __forceinline__ void store_chunks(uint8_t* base, int slice_bytes, int row, int j, const long long (&y)[8]) {
  uint32_t lo[8], hi[8];
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const unsigned long long o = (unsigned long long)y[u] + 0x0080808080808080ull;
    lo[u] = (uint32_t)o;
    hi[u] = (uint32_t)(o >> 32);
  }
  const int off = row * 128 + ((j ^ (row & 7)) << 4);
#pragma unroll
  for (int p = 0; p < SLICES; ++p) {
    uint32_t f[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      if (p == 0) f[u] = __float_as_uint(__uint_as_float(0x4B400000u | (hi[u] >> 16)) - 12583040.0f);
      else if (p <= 2) f[u] = digit_f32(hi[u], (uint32_t)(2 - p));
      else f[u] = digit_f32(lo[u], (uint32_t)(6 - p));
    }
    uint4 q;
    q.x = __byte_perm(f[0], f[1], 0x7632);
    q.y = __byte_perm(f[2], f[3], 0x7632);
    q.z = __byte_perm(f[4], f[5], 0x7632);
    q.w = __byte_perm(f[6], f[7], 0x7632);
    *reinterpret_cast<uint4*>(base + p * slice_bytes + off) = q;
  }
}

// The out-of-range case of scaled_i64_to_f64, out of line: inlined, ldexp's
// code at every call site crowded the instruction cache of the kernels that
// convert many elements in straight-line code.
static __device__ __noinline__ double scaled_i64_to_f64_ldexp(long long v, int s) { return ldexp((double)v, s); }

// (double)v * 2^s rounded to nearest even, with integer operations only (the
// FP64 pipe runs 2 operations per clock per SM on GB300, and a conversion plus
// ldexp per output element made it the busiest pipe of the kernels that write
// these products); results outside the normal range go through ldexp.
__device__ __forceinline__ double scaled_i64_to_f64(long long v, int s) {
  if (v == 0) return 0.0;
  const unsigned long long sign = v < 0 ? (1ull << 63) : 0ull;
  const unsigned long long u = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
  int msb = 63 - __clzll((long long)u);
  unsigned long long m;
  if (msb > 52) {
    const int sh = msb - 52;
    const unsigned long long rem = u & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    m = u >> sh;
    if (rem > half || (rem == half && (m & 1ull))) ++m;
    if (m >> 53) {
      m >>= 1;
      ++msb;
    }
  } else {
    m = u << (52 - msb);
  }
  const int biased = msb + s + 1023;
  if (biased <= 0 || biased >= 2047) return scaled_i64_to_f64_ldexp(v, s);
  return __longlong_as_double((long long)(sign | ((unsigned long long)biased << 52) | (m & 0xFFFFFFFFFFFFFull)));
}

}  // namespace split7
}  // namespace nla
