/*
 * One element-type specialisation of the CPU oracle for NextLA.jl's recursive
 * triangular solve / multiply.  Included three times by rectrxm_oracle.c with
 *   SUF     - name suffix (f64, f32, f16)
 *   RND(x)  - round a double to the element type and back (identity for f64)
 *
 * Every arithmetic operation is done in double and immediately rounded with
 * RND, which reproduces IEEE arithmetic in the element type (double has more
 * than 2p+2 significand bits for p = 11 and p = 24, so the double rounding is
 * innocuous).  Products and sums are never fused (built with
 * -ffp-contract=off).
 *
 * This is test infrastructure: it is the parity checker, never the product.
 */

#define OR_CAT2(a, b) a##_##b
#define OR_CAT(a, b) OR_CAT2(a, b)
#define FN(name) OR_CAT(name, SUF)

/* matmul! kernel, src/matmul.jl:5-66.
 * out[I,J] += alpha * sum_k in1[I,k] * in2[k,J], where the sum is built from
 * partial sums over 32-wide K tiles (src/matmul.jl:23-58, TILE_DIM = 32 at
 * src/matmul.jl:3) accumulated in the output element type, and the final
 * update promotes to Float64 because alpha is a Float64 (src/matmul.jl:64). */
static void FN(matmul)(view out, view in1, view in2, int64_t N, int64_t R, int64_t M, double alpha) {
  /* Columns of the output are processed in blocks of up to JB so that each
   * operand element is reused from cache; every output element still sees
   * exactly the reference's sequence of operations. */
  enum { JB = 8 };
  if (N <= 0 || M <= 0) return;
  double* outval = (double*)malloc(sizeof(double) * (size_t)N * JB);
  double* tmp = (double*)malloc(sizeof(double) * (size_t)N * JB);
  if (!outval || !tmp) {
    free(outval);
    free(tmp);
    return;
  }
  for (int64_t J0 = 0; J0 < M; J0 += JB) {
    const int64_t nj = M - J0 < JB ? M - J0 : JB;
    for (int64_t x = 0; x < N * nj; ++x) outval[x] = 0.0;
    for (int64_t t = 0; t < R; t += 32) {
      const int64_t kend = t + 32 < R ? t + 32 : R;
      for (int64_t x = 0; x < N * nj; ++x) tmp[x] = 0.0;
      for (int64_t k = t; k < kend; ++k) {
        for (int64_t j = 0; j < nj; ++j) {
          const double b = *at(in2, k, J0 + j);
          double* tj = tmp + j * N;
          for (int64_t I = 0; I < N; ++I) tj[I] = RND(tj[I] + RND(*at(in1, I, k) * b));
        }
      }
      for (int64_t x = 0; x < N * nj; ++x) outval[x] = RND(outval[x] + tmp[x]);
    }
    for (int64_t j = 0; j < nj; ++j) {
      for (int64_t I = 0; I < N; ++I) {
        double* o = at(out, I, J0 + j);
        double prod = alpha * outval[j * N + I]; /* Float64 product */
        double sum = *o + prod;                  /* Float64 sum */
        *o = RND(sum);                           /* stored back in eltype(output) */
      }
    }
  }
  free(outval);
  free(tmp);
}

/* GEMM_SUB!(X, Y, Z): X -= Y*Z, src/matmul.jl:76-81. */
static void FN(gemm_sub)(view X, int64_t xr, int64_t xc, view Y, view Z, int64_t zr) {
  FN(matmul)(X, Y, Z, xr, zr, xc, -1.0);
}

/* GEMM_ADD!(X, Y, Z): Z += X*Y, src/matmul.jl:69-74.  xr = size(X,1),
 * yr = size(Y,1), yc = size(Y,2). */
static void FN(gemm_add)(view X, int64_t xr, view Y, int64_t yr, int64_t yc, view Z) {
  FN(matmul)(Z, X, Y, xr, yr, yc, 1.0);
}

/* lower_left_kernel via LeftLowerTRSM!, src/trsm.jl:5-33 and :128-132.
 * The wrapper passes Transpose(A), so the kernel's A[i,row] is A[row,i].
 * x_r = b_r / d_r, then for i = 1..n, for r > i: x_r -= (A[r,i]/d_r) * x_i. */
static void FN(trsm_left_lower)(view A, view B, int64_t n, int64_t m) {
  for (int64_t c = 0; c < m; ++c) {
    for (int64_t r = 0; r < n; ++r) *at(B, r, c) = RND(*at(B, r, c) / *at(A, r, r));
    for (int64_t i = 0; i < n; ++i) {
      double xi = *at(B, i, c);
      for (int64_t r = i + 1; r < n; ++r) {
        double a = RND(*at(A, r, i) / *at(A, r, r));
        double* x = at(B, r, c);
        *x = RND(*x - RND(a * xi));
      }
    }
  }
}

/* upper_left_kernel via LeftUpperTRSM!, src/trsm.jl:36-64 and :134-138.
 * x_r = b_r / d_r, then for i = n..1, for r < i: x_r -= (A[r,i]/d_r) * x_i. */
static void FN(trsm_left_upper)(view A, view B, int64_t n, int64_t m) {
  for (int64_t c = 0; c < m; ++c) {
    for (int64_t r = 0; r < n; ++r) *at(B, r, c) = RND(*at(B, r, c) / *at(A, r, r));
    for (int64_t i = n - 1; i >= 0; --i) {
      double xi = *at(B, i, c);
      for (int64_t r = 0; r < i; ++r) {
        double a = RND(*at(A, r, i) / *at(A, r, r));
        double* x = at(B, r, c);
        *x = RND(*x - RND(a * xi));
      }
    }
  }
}

/* right_lower_kernel via RightLowerTRSM!, src/trsm.jl:67-95 and :140-144.
 * B is rows x n; per row: x_c = b_c / d_c, then for i = n..1, for c < i:
 * x_c -= x_i * (A[i,c]/d_c). */
static void FN(trsm_right_lower)(view A, view B, int64_t n, int64_t rows) {
  for (int64_t row = 0; row < rows; ++row) {
    for (int64_t c = 0; c < n; ++c) *at(B, row, c) = RND(*at(B, row, c) / *at(A, c, c));
    for (int64_t i = n - 1; i >= 0; --i) {
      double xi = *at(B, row, i);
      for (int64_t c = 0; c < i; ++c) {
        double a = RND(*at(A, i, c) / *at(A, c, c));
        double* x = at(B, row, c);
        *x = RND(*x - RND(xi * a));
      }
    }
  }
}

/* right_upper_kernel via RightUpperTRSM!, src/trsm.jl:98-126 and :146-150.
 * The wrapper passes Transpose(A), so the kernel's A[col,i] is A[i,col].
 * Per row: x_c = b_c / d_c, then for i = 1..n, for c > i: x_c -= x_i * (A[i,c]/d_c). */
static void FN(trsm_right_upper)(view A, view B, int64_t n, int64_t rows) {
  for (int64_t row = 0; row < rows; ++row) {
    for (int64_t c = 0; c < n; ++c) *at(B, row, c) = RND(*at(B, row, c) / *at(A, c, c));
    for (int64_t i = 0; i < n; ++i) {
      double xi = *at(B, row, i);
      for (int64_t c = i + 1; c < n; ++c) {
        double a = RND(*at(A, i, c) / *at(A, c, c));
        double* x = at(B, row, c);
        *x = RND(*x - RND(xi * a));
      }
    }
  }
}

/* LeftLowerTRMM_kernel! / LeftUpperTRMM_kernel!, src/trmm.jl:43-109 and
 * :116-180: B[i,j] := sum_{k<=i} A[i,k] B[k,j]  (lower) or
 * sum_{k>=i} A[i,k] B[k,j] (upper), summed in increasing k from zero in the
 * element type (src/trmm.jl:90-94, :163-167).  All new values are formed from
 * the old B before any is written (the kernels stage B in shared memory). */
static void FN(trmm_left)(int upper, view A, view B, int64_t n, int64_t m, double* col) {
  for (int64_t j = 0; j < m; ++j) {
    for (int64_t i = 0; i < n; ++i) {
      double out = 0.0;
      int64_t k0 = upper ? i : 0, k1 = upper ? n : i + 1;
      for (int64_t k = k0; k < k1; ++k) out = RND(out + RND(*at(A, i, k) * *at(B, k, j)));
      col[i] = out;
    }
    for (int64_t i = 0; i < n; ++i) *at(B, i, j) = col[i];
  }
}

/* RightLowerTRMM_kernel! / RightUpperTRMM_kernel!, src/trmm.jl:189-250 and
 * :252-312: B[i,j] := sum_{k>=j} B[i,k] A[k,j] (lower) or
 * sum_{k<=j} B[i,k] A[k,j] (upper), summed in increasing k
 * (src/trmm.jl:232-236, :295-299). */
static void FN(trmm_right)(int upper, view A, view B, int64_t n, int64_t rows, double* rowbuf) {
  for (int64_t i = 0; i < rows; ++i) {
    for (int64_t j = 0; j < n; ++j) {
      double out = 0.0;
      int64_t k0 = upper ? 0 : j, k1 = upper ? j + 1 : n;
      for (int64_t k = k0; k < k1; ++k) out = RND(out + RND(*at(B, i, k) * *at(A, k, j)));
      rowbuf[j] = out;
    }
    for (int64_t j = 0; j < n; ++j) *at(B, i, j) = rowbuf[j];
  }
}

/* Base-case dispatch of unified_rec, src/rectrxm.jl:103-126.  B is n x m for
 * side L and m x n for side R. */
static void FN(leaf)(char func, char side, char uplo, view A, int64_t n, view B, int64_t m, double* buf) {
  if (func == 'S') {
    if (side == 'L' && uplo == 'L') FN(trsm_left_lower)(A, B, n, m);
    else if (side == 'L' && uplo == 'U') FN(trsm_left_upper)(A, B, n, m);
    else if (side == 'R' && uplo == 'L') FN(trsm_right_lower)(A, B, n, m);
    else FN(trsm_right_upper)(A, B, n, m);
  } else {
    if (side == 'L') FN(trmm_left)(uplo == 'U', A, B, n, m, buf);
    else FN(trmm_right)(uplo == 'U', A, B, n, m, buf);
  }
}

/* unified_rec, src/rectrxm.jl:101-198. */
static void FN(rec)(char func, char side, char uplo, view A, int64_t n, view B, int64_t m, int64_t threshold,
                    double* buf) {
  if (n <= threshold) {
    FN(leaf)(func, side, uplo, A, n, B, m, buf);
    return;
  }
  int64_t mid = split_point(n); /* src/rectrxm.jl:129-133 */
  int64_t rem = n - mid;
  view A11 = sub(A, 0, 0), A22 = sub(A, mid, mid), A21 = sub(A, mid, 0), A12 = sub(A, 0, mid);
  view B1 = sub(B, 0, 0);
  view B2 = side == 'L' ? sub(B, mid, 0) : sub(B, 0, mid);
  int forward = (side == 'L' && uplo == 'L' && func == 'S') || (side == 'R' && uplo == 'U' && func == 'S') ||
                (side == 'L' && uplo == 'U' && func == 'M') || (side == 'R' && uplo == 'L' && func == 'M');
  if (forward) { /* src/rectrxm.jl:153-176 */
    FN(rec)(func, side, uplo, A11, mid, B1, m, threshold, buf);
    if (side == 'L') {
      if (func == 'S') FN(gemm_sub)(B2, rem, m, A21, B1, mid);   /* B2 -= A21*B1 */
      else FN(gemm_add)(A12, mid, B2, rem, m, B1);              /* B1 += A12*B2 */
    } else {
      if (func == 'S') FN(gemm_sub)(B2, m, rem, B1, A12, mid);   /* B2 -= B1*A12 */
      else FN(gemm_add)(B2, m, A21, rem, mid, B1);              /* B1 += B2*A21 */
    }
    FN(rec)(func, side, uplo, A22, rem, B2, m, threshold, buf);
  } else { /* src/rectrxm.jl:177-197 */
    FN(rec)(func, side, uplo, A22, rem, B2, m, threshold, buf);
    if (side == 'L') {
      if (func == 'S') FN(gemm_sub)(B1, mid, m, A12, B2, rem);   /* B1 -= A12*B2 */
      else FN(gemm_add)(A21, rem, B1, mid, m, B2);              /* B2 += A21*B1 */
    } else {
      if (func == 'S') FN(gemm_sub)(B1, m, mid, B2, A21, rem);   /* B1 -= B2*A21 */
      else FN(gemm_add)(B1, m, A12, mid, rem, B2);              /* B2 += B1*A12 */
    }
    FN(rec)(func, side, uplo, A11, mid, B1, m, threshold, buf);
  }
}

/* B .= alpha .* B, src/rectrxm.jl:64 and :72: Float64 product stored back in
 * the element type. */
static void FN(scale)(view B, int64_t rows, int64_t cols, double alpha) {
  for (int64_t j = 0; j < cols; ++j)
    for (int64_t i = 0; i < rows; ++i) {
      double* b = at(B, i, j);
      *b = RND(alpha * *b);
    }
}

/* unified_rectrxm!, src/rectrxm.jl:43-76, on one block of B (all of B, or a
 * block of independent columns for side L / rows for side R). */
static void FN(rectrxm)(char side, char uplo, char trans, double alpha, char func, view A, int64_t n, view B,
                        int64_t m, int64_t thr_s, int64_t thr_m) {
  int64_t threshold = thr_m; /* src/rectrxm.jl:52 */
  if (trans == 'T' || trans == 'C') { /* src/rectrxm.jl:56-59; real data: 'C' == 'T' */
    A.t = !A.t;
    uplo = uplo == 'L' ? 'U' : 'L';
  }
  int64_t rows = side == 'L' ? n : m, cols = side == 'L' ? m : n;
  if (func == 'S') { /* src/rectrxm.jl:62-65 */
    threshold = thr_s;
    FN(scale)(B, rows, cols, alpha);
  }
  double* buf = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  FN(rec)(func, side, uplo, A, n, B, m, threshold, buf);
  free(buf);
  if (func == 'M') FN(scale)(B, rows, cols, alpha); /* src/rectrxm.jl:71-73 */
}

#undef FN
#undef OR_CAT
#undef OR_CAT2
