/*
 * CPU oracle for NextLA.jl's recursive triangular solve / multiply
 * (`unified_rectrxm!`, src/rectrxm.jl:43-198, with the base-case kernels of
 * src/trsm.jl and src/trmm.jl and the GEMM update of src/matmul.jl).
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates the reference algorithm in
 * plain C so that the GPU library can be checked against it; it is imported
 * only by the tests, by the smoke check and by the CPU-baseline leg of the
 * benchmark.  The product library never links or calls it.
 *
 * Matrices are column-major arrays of double.  Element types narrower than
 * double (Float32, Float16) are emulated by rounding after every operation,
 * so the double arrays always hold values representable in the element type.
 *
 * Parity pinning: the reference ships no golden vectors.  Its own tests
 * (test/unified_rectrxm.jl:10-44, test/trsm.jl:57-111) compare against BLAS
 * trsm!/trmm! with relative Frobenius error < 1e-14 (Float64) and < 1e-5
 * (Float32); the test suite checks this oracle against the same contract and
 * against exact rational solutions of small integer systems.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>

/* A strided column-major view; element (i,j) is p[i + j*ld], or p[j + i*ld]
 * when t is set (a Transpose/Adjoint wrapper of a real matrix). */
typedef struct {
  double* p;
  int64_t ld;
  int t;
} view;

static inline double* at(view v, int64_t i, int64_t j) { return v.t ? &v.p[j + i * v.ld] : &v.p[i + j * v.ld]; }

/* view(v, i0+1:end, j0+1:end) */
static inline view sub(view v, int64_t i0, int64_t j0) {
  view r = v;
  r.p = at(v, i0, j0);
  return r;
}

/* src/rectrxm.jl:129-133: n/2 when log2(n) is an integer, otherwise the
 * largest power of two below n. */
static int64_t split_point(int64_t n) {
  int64_t p = 1;
  while (p * 2 <= n) p *= 2;
  return p == n ? n / 2 : p;
}

#define SUF f64
#define RND(x) (x)
#include "rectrxm_oracle_impl.h"
#undef SUF
#undef RND

#define SUF f32
#define RND(x) ((double)(float)(x))
#include "rectrxm_oracle_impl.h"
#undef SUF
#undef RND

#define SUF f16
#define RND(x) ((double)(_Float16)(x))
#include "rectrxm_oracle_impl.h"
#undef SUF
#undef RND

/* Complex matrices: interleaved (re, im) doubles, column-major; element
 * (i, j) at p[2 (i + j ld)], or p[2 (j + i ld)] when t is set; c reads the
 * conjugate (an Adjoint view). */
typedef struct {
  double re, im;
} cz;
typedef struct {
  double* p;
  int64_t ld;
  int t, c;
} zview;

static inline double* zat(zview v, int64_t i, int64_t j) { return v.p + 2 * (v.t ? j + i * v.ld : i + j * v.ld); }
static inline cz zget(zview v, int64_t i, int64_t j) {
  const double* q = zat(v, i, j);
  cz r = {q[0], v.c ? -q[1] : q[1]};
  return r;
}
static inline void zset(zview v, int64_t i, int64_t j, cz x) {
  double* q = zat(v, i, j);
  q[0] = x.re;
  q[1] = x.im;
}
static inline zview zsub(zview v, int64_t i0, int64_t j0) {
  zview r = v;
  r.p = zat(v, i0, j0);
  return r;
}

#define SUF c64
#define RND(x) (x)
#include "rectrxm_oracle_cplx.h"
#undef SUF
#undef RND

#define SUF c32
#define RND(x) ((double)(float)(x))
#include "rectrxm_oracle_cplx.h"
#undef SUF
#undef RND

/* dtype codes: 0 = Float16, 1 = Float32, 2 = Float64, 3 = ComplexF32,
 * 4 = ComplexF64 (same as the library). */

typedef struct {
  char side, uplo, trans, func;
  double alpha;
  int dtype;
  view A;
  int64_t n;
  view B;
  int64_t m;
  int64_t thr_s, thr_m;
} job;

static void run_job(const job* j) {
  if (j->m <= 0) return;
  switch (j->dtype) {
    case 0: rectrxm_f16(j->side, j->uplo, j->trans, j->alpha, j->func, j->A, j->n, j->B, j->m, j->thr_s, j->thr_m); break;
    case 1: rectrxm_f32(j->side, j->uplo, j->trans, j->alpha, j->func, j->A, j->n, j->B, j->m, j->thr_s, j->thr_m); break;
    default: rectrxm_f64(j->side, j->uplo, j->trans, j->alpha, j->func, j->A, j->n, j->B, j->m, j->thr_s, j->thr_m); break;
  }
}

static void* job_thread(void* arg) {
  run_job((const job*)arg);
  return NULL;
}

/*
 * unified_rectrxm!(side, uplo, trans, alpha, func, A, B) on column-major
 * double arrays.  A is n x n (lda >= n); B is n x m for side 'L' and m x n for
 * side 'R' (ldb >= rows).  thr_s / thr_m are the recursion thresholds (the
 * reference uses 256 and 16, src/rectrxm.jl:52,63).  nthreads > 1 splits the
 * independent right-hand sides (columns for side 'L', rows for side 'R')
 * into contiguous blocks solved concurrently; each block runs the same
 * arithmetic as the single-threaded call.  Returns 0, or -1 on bad input.
 */
int oracle_rectrxm(char side, char uplo, char trans, double alpha, char func, int dtype, int64_t n, int64_t m,
                   double* A, int64_t lda, double* B, int64_t ldb, int64_t thr_s, int64_t thr_m, int nthreads) {
  if (n < 0 || m < 0 || lda < (n > 1 ? n : 1) || thr_s < 1 || thr_m < 1) return -1;
  int64_t rows = side == 'L' ? n : m;
  if (ldb < (rows > 1 ? rows : 1)) return -1;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > m) nthreads = (int)(m > 0 ? m : 1);
  job* jobs = (job*)calloc((size_t)nthreads, sizeof(job));
  pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
  if (!jobs || !th) {
    free(jobs);
    free(th);
    return -1;
  }
  view Av = {A, lda, 0};
  int64_t start = 0;
  for (int t = 0; t < nthreads; ++t) {
    int64_t cnt = m / nthreads + (t < m % nthreads ? 1 : 0);
    view Bv = {B, ldb, 0};
    Bv = side == 'L' ? sub(Bv, 0, start) : sub(Bv, start, 0);
    job j = {side, uplo, trans, func, alpha, dtype, Av, n, Bv, cnt, thr_s, thr_m};
    jobs[t] = j;
    start += cnt;
  }
  char* started = (char*)calloc((size_t)nthreads, 1);
  for (int t = 1; t < nthreads; ++t) {
    if (started && pthread_create(&th[t], NULL, job_thread, &jobs[t]) == 0)
      started[t] = 1;
    else
      run_job(&jobs[t]); /* no thread available: run it here */
  }
  run_job(&jobs[0]);
  for (int t = 1; t < nthreads; ++t)
    if (started && started[t]) pthread_join(th[t], NULL);
  free(started);
  free(jobs);
  free(th);
  return 0;
}

/* matmul!(out, in1, in2, N, R, M, alpha) of src/matmul.jl:5-66 with optional
 * transposed operand views (t1, t2).  out is N x M (ldo), op(in1) N x R,
 * op(in2) R x M. */
int oracle_matmul(int dtype, int64_t N, int64_t R, int64_t M, double alpha, double* out, int64_t ldo, double* in1,
                  int64_t ld1, int t1, double* in2, int64_t ld2, int t2) {
  if (N < 0 || R < 0 || M < 0) return -1;
  view o = {out, ldo, 0}, a = {in1, ld1, t1}, b = {in2, ld2, t2};
  switch (dtype) {
    case 0: matmul_f16(o, a, b, N, R, M, alpha); break;
    case 1: matmul_f32(o, a, b, N, R, M, alpha); break;
    default: matmul_f64(o, a, b, N, R, M, alpha); break;
  }
  return 0;
}

/* One base-case call (LeftLowerTRSM! ... RightUpperTRMM!) on op(A) = A or
 * A^T (tA).  B is n x m (side 'L') or m x n (side 'R'). */
int oracle_leaf(char func, char side, char uplo, int dtype, int64_t n, int64_t m, double* A, int64_t lda, int tA,
                double* B, int64_t ldb) {
  if (n < 0 || m < 0) return -1;
  view a = {A, lda, tA}, b = {B, ldb, 0};
  double* buf = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  if (!buf) return -1;
  switch (dtype) {
    case 0: leaf_f16(func, side, uplo, a, n, b, m, buf); break;
    case 1: leaf_f32(func, side, uplo, a, n, b, m, buf); break;
    default: leaf_f64(func, side, uplo, a, n, b, m, buf); break;
  }
  free(buf);
  return 0;
}

/* The recursion's split point (src/rectrxm.jl:129-133), exported so the
 * host-side planner can be checked against it. */
int64_t oracle_split_point(int64_t n) { return split_point(n); }

/* unified_rectrxm! on complex column-major arrays (interleaved re, im
 * doubles), dtype 3 (ComplexF32, values rounded to float after every
 * operation) or 4 (ComplexF64), alpha = alpha_re + i alpha_im.  Arguments as
 * for oracle_rectrxm; the right-hand sides are split over nthreads. */
typedef struct {
  char side, uplo, trans, func;
  cz alpha;
  int dtype;
  zview A;
  int64_t n;
  zview B;
  int64_t m;
  int64_t thr_s, thr_m;
} zjob;

static void* zjob_thread(void* arg) {
  const zjob* j = (const zjob*)arg;
  if (j->m <= 0) return NULL;
  if (j->dtype == 3)
    rectrxm_c32(j->side, j->uplo, j->trans, j->alpha, j->func, j->A, j->n, j->B, j->m, j->thr_s, j->thr_m);
  else
    rectrxm_c64(j->side, j->uplo, j->trans, j->alpha, j->func, j->A, j->n, j->B, j->m, j->thr_s, j->thr_m);
  return NULL;
}

int oracle_rectrxm_cplx(char side, char uplo, char trans, double alpha_re, double alpha_im, char func, int dtype,
                        int64_t n, int64_t m, double* A, int64_t lda, double* B, int64_t ldb, int64_t thr_s,
                        int64_t thr_m, int nthreads) {
  if (n < 0 || m < 0 || lda < (n > 1 ? n : 1) || thr_s < 1 || thr_m < 1 || (dtype != 3 && dtype != 4)) return -1;
  int64_t rows = side == 'L' ? n : m;
  if (ldb < (rows > 1 ? rows : 1)) return -1;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > m) nthreads = (int)(m > 0 ? m : 1);
  zjob* jobs = (zjob*)calloc((size_t)nthreads, sizeof(zjob));
  pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
  char* started = (char*)calloc((size_t)nthreads, 1);
  if (!jobs || !th || !started) {
    free(jobs);
    free(th);
    free(started);
    return -1;
  }
  zview Av = {A, lda, 0, 0};
  int64_t start = 0;
  for (int t = 0; t < nthreads; ++t) {
    int64_t cnt = m / nthreads + (t < m % nthreads ? 1 : 0);
    zview Bv = {B, ldb, 0, 0};
    Bv = side == 'L' ? zsub(Bv, 0, start) : zsub(Bv, start, 0);
    zjob j = {side, uplo, trans, func, {alpha_re, alpha_im}, dtype, Av, n, Bv, cnt, thr_s, thr_m};
    jobs[t] = j;
    start += cnt;
  }
  for (int t = 1; t < nthreads; ++t) {
    if (pthread_create(&th[t], NULL, zjob_thread, &jobs[t]) == 0)
      started[t] = 1;
    else
      zjob_thread(&jobs[t]);
  }
  zjob_thread(&jobs[0]);
  for (int t = 1; t < nthreads; ++t)
    if (started[t]) pthread_join(th[t], NULL);
  free(started);
  free(jobs);
  free(th);
  return 0;
}
