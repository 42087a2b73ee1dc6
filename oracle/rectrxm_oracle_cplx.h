/*
 * Complex element-type specialisation of the CPU oracle (ComplexF64,
 * ComplexF32).  Included twice by rectrxm_oracle.c with
 *   SUF     - name suffix (c64, c32)
 *   RND(x)  - round a double to the real element type and back
 *
 * Matrices are column-major arrays of complex values stored as interleaved
 * (re, im) doubles.  The algorithm is the one of the real oracle
 * (unified_rectrxm!, src/rectrxm.jl:43-198; src/trsm.jl, src/trmm.jl,
 * src/matmul.jl) with Julia's complex arithmetic on every operation: a
 * product is (ar br - ai bi, ar bi + ai br), each real multiply and add
 * rounded; a quotient uses Smith's algorithm (R. L. Smith, "Algorithm 116:
 * Complex division", CACM 5(8), 1962).  trans 'C' reads the conjugate of A
 * (Adjoint), 'T' its plain transpose.  The reference's unified_rec accepts
 * only real element types (src/rectrxm.jl:101) though its docstrings list
 * complex ones (src/trsm.jl:180-183): this restatement is the algorithm the
 * reference would run on them.
 *
 * This is test infrastructure: it is the parity checker, never the product.
 */

#define OC_CAT2(a, b) a##_##b
#define OC_CAT(a, b) OC_CAT2(a, b)
#define FN(name) OC_CAT(name, SUF)

static inline cz FN(mul)(cz a, cz b) {
  cz r;
  r.re = RND(RND(a.re * b.re) - RND(a.im * b.im));
  r.im = RND(RND(a.re * b.im) + RND(a.im * b.re));
  return r;
}
static inline cz FN(add)(cz a, cz b) {
  cz r;
  r.re = RND(a.re + b.re);
  r.im = RND(a.im + b.im);
  return r;
}
static inline cz FN(sub2)(cz a, cz b) {
  cz r;
  r.re = RND(a.re - b.re);
  r.im = RND(a.im - b.im);
  return r;
}
static inline cz FN(div)(cz a, cz b) {
  cz r;
  if (fabs(b.re) >= fabs(b.im)) {
    const double t = RND(b.im / b.re), den = RND(b.re + RND(b.im * t));
    r.re = RND(RND(a.re + RND(a.im * t)) / den);
    r.im = RND(RND(a.im - RND(a.re * t)) / den);
  } else {
    const double t = RND(b.re / b.im), den = RND(b.im + RND(b.re * t));
    r.re = RND(RND(RND(a.re * t) + a.im) / den);
    r.im = RND(RND(RND(a.im * t) - a.re) / den);
  }
  return r;
}

/* matmul!, src/matmul.jl:5-66: 32-wide partial sums in the element type,
 * then out += alpha * partial with alpha = +-1 (exact). */
static void FN(matmul)(zview out, zview in1, zview in2, int64_t N, int64_t R, int64_t M, double alpha) {
  for (int64_t J = 0; J < M; ++J)
    for (int64_t I = 0; I < N; ++I) {
      cz outval = {0.0, 0.0};
      for (int64_t t = 0; t < R; t += 32) {
        const int64_t kend = t + 32 < R ? t + 32 : R;
        cz tmp = {0.0, 0.0};
        for (int64_t k = t; k < kend; ++k) tmp = FN(add)(tmp, FN(mul)(zget(in1, I, k), zget(in2, k, J)));
        outval = FN(add)(outval, tmp);
      }
      cz o = zget(out, I, J);
      cz prod = {alpha * outval.re, alpha * outval.im};
      zset(out, I, J, FN(add)(o, prod));
    }
}

static void FN(leaf)(char func, char side, char uplo, zview A, int64_t n, zview B, int64_t m) {
  if (func == 'S') {
    /* src/trsm.jl:5-150: x = b / d, then x -= (a / d) x_i in the kernels' order. */
    const int lower = uplo == 'L';
    if (side == 'L') {
      for (int64_t c = 0; c < m; ++c) {
        for (int64_t r = 0; r < n; ++r) zset(B, r, c, FN(div)(zget(B, r, c), zget(A, r, r)));
        for (int64_t s = 0; s < n; ++s) {
          const int64_t i = lower ? s : n - 1 - s;
          const cz xi = zget(B, i, c);
          for (int64_t r = lower ? i + 1 : 0; lower ? r < n : r < i; ++r) {
            const cz a = FN(div)(zget(A, r, i), zget(A, r, r));
            zset(B, r, c, FN(sub2)(zget(B, r, c), FN(mul)(a, xi)));
          }
        }
      }
    } else {
      for (int64_t row = 0; row < m; ++row) {
        for (int64_t c = 0; c < n; ++c) zset(B, row, c, FN(div)(zget(B, row, c), zget(A, c, c)));
        for (int64_t s = 0; s < n; ++s) {
          const int64_t i = lower ? n - 1 - s : s;
          const cz xi = zget(B, row, i);
          for (int64_t c = lower ? 0 : i + 1; lower ? c < i : c < n; ++c) {
            const cz a = FN(div)(zget(A, i, c), zget(A, c, c));
            zset(B, row, c, FN(sub2)(zget(B, row, c), FN(mul)(xi, a)));
          }
        }
      }
    }
  } else {
    /* src/trmm.jl:43-312: sums in increasing k from zero, from the old B. */
    const int upper = uplo == 'U';
    cz* buf = (cz*)malloc(sizeof(cz) * (size_t)(n > 0 ? n : 1));
    if (side == 'L') {
      for (int64_t j = 0; j < m; ++j) {
        for (int64_t i = 0; i < n; ++i) {
          cz o = {0.0, 0.0};
          for (int64_t k = upper ? i : 0; k < (upper ? n : i + 1); ++k) o = FN(add)(o, FN(mul)(zget(A, i, k), zget(B, k, j)));
          buf[i] = o;
        }
        for (int64_t i = 0; i < n; ++i) zset(B, i, j, buf[i]);
      }
    } else {
      for (int64_t i = 0; i < m; ++i) {
        for (int64_t j = 0; j < n; ++j) {
          cz o = {0.0, 0.0};
          for (int64_t k = upper ? 0 : j; k < (upper ? j + 1 : n); ++k) o = FN(add)(o, FN(mul)(zget(B, i, k), zget(A, k, j)));
          buf[j] = o;
        }
        for (int64_t j = 0; j < n; ++j) zset(B, i, j, buf[j]);
      }
    }
    free(buf);
  }
}

/* unified_rec, src/rectrxm.jl:101-198, with the GEMM updates of :162-194. */
static void FN(rec)(char func, char side, char uplo, zview A, int64_t n, zview B, int64_t m, int64_t threshold) {
  if (n <= threshold) {
    FN(leaf)(func, side, uplo, A, n, B, m);
    return;
  }
  const int64_t mid = split_point(n), rem = n - mid;
  zview A11 = zsub(A, 0, 0), A22 = zsub(A, mid, mid), A21 = zsub(A, mid, 0), A12 = zsub(A, 0, mid);
  zview B1 = zsub(B, 0, 0);
  zview B2 = side == 'L' ? zsub(B, mid, 0) : zsub(B, 0, mid);
  const int forward = (side == 'L' && uplo == 'L' && func == 'S') || (side == 'R' && uplo == 'U' && func == 'S') ||
                      (side == 'L' && uplo == 'U' && func == 'M') || (side == 'R' && uplo == 'L' && func == 'M');
  if (forward) {
    FN(rec)(func, side, uplo, A11, mid, B1, m, threshold);
    if (side == 'L') {
      if (func == 'S') FN(matmul)(B2, A21, B1, rem, mid, m, -1.0);
      else FN(matmul)(B1, A12, B2, mid, rem, m, 1.0);
    } else {
      if (func == 'S') FN(matmul)(B2, B1, A12, m, mid, rem, -1.0);
      else FN(matmul)(B1, B2, A21, m, rem, mid, 1.0);
    }
    FN(rec)(func, side, uplo, A22, rem, B2, m, threshold);
  } else {
    FN(rec)(func, side, uplo, A22, rem, B2, m, threshold);
    if (side == 'L') {
      if (func == 'S') FN(matmul)(B1, A12, B2, mid, rem, m, -1.0);
      else FN(matmul)(B2, A21, B1, rem, mid, m, 1.0);
    } else {
      if (func == 'S') FN(matmul)(B1, B2, A21, m, rem, mid, -1.0);
      else FN(matmul)(B2, B1, A12, m, mid, rem, 1.0);
    }
    FN(rec)(func, side, uplo, A11, mid, B1, m, threshold);
  }
}

/* B .= alpha .* B (src/rectrxm.jl:64, :72): the product in ComplexF64,
 * stored back in the element type. */
static void FN(scale)(zview B, int64_t rows, int64_t cols, cz alpha) {
  for (int64_t j = 0; j < cols; ++j)
    for (int64_t i = 0; i < rows; ++i) {
      const cz b = zget(B, i, j);
      cz r;
      r.re = RND(alpha.re * b.re - alpha.im * b.im);
      r.im = RND(alpha.re * b.im + alpha.im * b.re);
      zset(B, i, j, r);
    }
}

static void FN(rectrxm)(char side, char uplo, char trans, cz alpha, char func, zview A, int64_t n, zview B,
                        int64_t m, int64_t thr_s, int64_t thr_m) {
  int64_t threshold = thr_m;
  if (trans == 'T' || trans == 'C') { /* src/rectrxm.jl:56-59: Transpose / Adjoint */
    A.t = !A.t;
    A.c = trans == 'C';
    uplo = uplo == 'L' ? 'U' : 'L';
  }
  const int64_t rows = side == 'L' ? n : m, cols = side == 'L' ? m : n;
  if (func == 'S') {
    threshold = thr_s;
    FN(scale)(B, rows, cols, alpha);
  }
  FN(rec)(func, side, uplo, A, n, B, m, threshold);
  if (func == 'M') FN(scale)(B, rows, cols, alpha);
}

#undef FN
#undef OC_CAT
#undef OC_CAT2
