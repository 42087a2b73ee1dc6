/*
 * nextla_gb300.h - C ABI of the GB300 (sm_103a) implementation of NextLA.jl's
 * recursive triangular solve / multiply.
 *
 * Conventions shared by every entry point:
 *  - Matrices are column-major with an explicit leading dimension, as Julia
 *    stores them; element (i,j) of X is X[i + j*ldx].  A transposed operand is
 *    passed as the untransposed parent with a transpose flag, which is how a
 *    Julia `Transpose(A)` view or a strided SubArray reaches the library.
 *  - All pointers are device pointers owned by the caller, except where a
 *    comment says "host".  Nothing is freed or retained by the library.
 *  - Work is enqueued on `stream` (a cudaStream_t; NULL is the legacy default
 *    stream) and runs asynchronously; the caller synchronises, as the
 *    reference's callers do (test/unified_rectrxm.jl:34).
 *  - Every call returns NLA_OK (0) or a negative status; nla_last_error()
 *    then describes the failure for the calling thread.
 *  - Character flags are the reference's: side 'L'/'R', uplo 'L'/'U',
 *    trans 'N'/'T'/'C' ('C' equals 'T' for real data), func 'S' (solve,
 *    TRSM) / 'M' (multiply, TRMM).  Unlike the reference, which silently
 *    falls through to a default branch on an unknown character
 *    (src/rectrxm.jl:104-124), unknown characters are rejected with
 *    NLA_ERR_ARG.
 */
#ifndef NEXTLA_GB300_H
#define NEXTLA_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define NLA_API __attribute__((visibility("default")))
#else
#define NLA_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Element types (Float16, Float32, Float64; ComplexF32, ComplexF64 stored as
 * interleaved (re, im) pairs, as Julia and torch store them).  The complex
 * types run the plain path (nla_trxm, nla_trxm_ex, nla_trxm_diag,
 * nla_trxm_complex, nla_diag_block, nla_gemm_update, nla_scale and the
 * host-buffer nla_trxm_host); the mixed, batched and no-allocation forms are
 * real only. */
#define NLA_F16 0
#define NLA_F32 1
#define NLA_F64 2
#define NLA_C32 3
#define NLA_C64 4

/* Status codes. */
#define NLA_OK 0
#define NLA_ERR_ARG -1         /* bad flag, size, leading dimension or null pointer */
#define NLA_ERR_DTYPE -2       /* element type not supported by this entry point */
#define NLA_ERR_UNSUPPORTED -3 /* valid request this build does not implement */
#define NLA_ERR_WORKSPACE -4   /* caller-provided workspace too small */
#define NLA_ERR_TIMEOUT -5     /* a bounded device-side wait gave up */
#define NLA_ERR_NOMEM -6       /* device allocation failed */
#define NLA_ERR_CUDA_BASE -100 /* NLA_ERR_CUDA_BASE - cudaError_t for CUDA errors */

/* Library version (major*10000 + minor*100 + patch). */
NLA_API int nla_version(void);

/* Description of the last failure on the calling thread ("" if none). */
NLA_API const char* nla_last_error(void);

/*
 * unified_rectrxm!(side, uplo, trans, alpha, func, A, B)
 * Replaces src/rectrxm.jl:43-76 (with the recursion unified_rec,
 * src/rectrxm.jl:101-198) for one GPU.  The whole recursion runs in native
 * host code; each base case and each off-diagonal update is one kernel launch.
 *   func 'S': solve op(A) X = alpha B (side 'L') or X op(A) = alpha B ('R');
 *   func 'M': B := alpha op(A) B ('L') or alpha B op(A) ('R').
 * A is n x n (only the `uplo` triangle is read, diagonal non-unit); B is
 * n x m for side 'L' and m x n for side 'R'; the result overwrites B.
 * dtype is NLA_F16, NLA_F32, NLA_F64, NLA_C32 or NLA_C64 and applies to A
 * and B.  trans 'T' takes A's transpose, 'C' its conjugate transpose (the
 * Adjoint wrapper; the same as 'T' for real types).
 * The recursion cut-offs are the library's tuned defaults (environment
 * NLA_TRXM_CUTOFF_S / NLA_TRXM_CUTOFF_M override them; complex diagonal
 * blocks are at most 128).
 */
NLA_API int nla_trxm(char side, char uplo, char trans, double alpha, char func, int dtype, int64_t n, int64_t m,
             const void* A, int64_t lda, void* B, int64_t ldb, void* stream);

/*
 * nla_trxm for complex element types with a complex alpha = alpha_re +
 * i alpha_im (dtype NLA_C32 or NLA_C64).  The reference's unified_rec accepts
 * only real element types (src/rectrxm.jl:101) though its base-case
 * docstrings list complex ones (src/trsm.jl:180-183); this runs the same
 * recursion on complex data.
 */
NLA_API int nla_trxm_complex(char side, char uplo, char trans, double alpha_re, double alpha_im, char func, int dtype,
                             int64_t n, int64_t m, const void* A, int64_t lda, void* B, int64_t ldb, void* stream);

/*
 * nla_trxm with explicit recursion cut-offs for solve and multiply (the
 * reference's are 256 and 16, src/rectrxm.jl:52,63).  A cut-off <= 0 selects
 * the default.  Solve cut-offs above 1024 are clamped to 1024.
 */
NLA_API int nla_trxm_ex(char side, char uplo, char trans, double alpha, char func, int dtype, int64_t n, int64_t m,
                const void* A, int64_t lda, void* B, int64_t ldb, int64_t cutoff_s, int64_t cutoff_m, void* stream);

/*
 * nla_trxm with a unit-diagonal option: diag 'U' takes the diagonal of A as
 * ones and never reads it; 'N' is nla_trxm.  Backs the trsm()/trmm() wrappers
 * (src/trsm.jl:186-204, src/trmm.jl:430-448), which take a diag argument the
 * reference accepts but does not apply; here the wrappers run the recursion,
 * so they also honour transa and any n.
 */
NLA_API int nla_trxm_diag(char side, char uplo, char trans, char diag, double alpha, char func, int dtype, int64_t n,
                          int64_t m, const void* A, int64_t lda, void* B, int64_t ldb, void* stream);

/*
 * One base case of the recursion on a diagonal block.
 * Replaces LeftLowerTRSM!/LeftUpperTRSM!/RightLowerTRSM!/RightUpperTRSM!
 * (src/trsm.jl:128-150, kernels :5-126) for func 'S' and
 * LeftLowerTRMM!/LeftUpperTRMM!/RightLowerTRMM!/RightUpperTRMM!
 * (src/trmm.jl:332-389, kernels :43-312) for func 'M'.
 * op(A) = A (transA 0) or A^T (transA 1) is the n x n triangle named by uplo
 * (the reference passes Transpose views here); for complex types bit 1 of
 * transA conjugates A's elements (3: the conjugate transpose); B is n x m
 * (side 'L') or
 * m x n (side 'R').  No alpha: the reference's base cases have none.
 * n <= 1024 (the reference's shared buffers hold 1024 entries,
 * src/trsm.jl:10-12).
 */
NLA_API int nla_diag_block(char func, char side, char uplo, int transA, int dtype, int64_t n, int64_t m, const void* A,
                   int64_t lda, void* B, int64_t ldb, void* stream);

/*
 * The off-diagonal update: out (N x M) += alpha * op(in1) (N x R) * op(in2) (R x M).
 * Replaces matmul! (src/matmul.jl:5-66) as launched by GEMM_ADD!
 * (src/matmul.jl:69-74, alpha = +1) and GEMM_SUB! (src/matmul.jl:76-81,
 * alpha = -1).  trans1/trans2 select op() = transpose (1) or identity (0),
 * matching matmul!'s transA/transB arguments for real data; for complex
 * types bit 1 also conjugates the operand (3: conjugate transpose).  Float16 inputs
 * accumulate in Float32 (the reference accumulates in Float16).
 * `out` must not overlap `in1` or `in2`.
 */
NLA_API int nla_gemm_update(int dtype, int trans1, int trans2, int64_t N, int64_t R, int64_t M, double alpha,
                    const void* in1, int64_t ld1, const void* in2, int64_t ld2, void* out, int64_t ldo, void* stream);

/*
 * B .= alpha .* B (src/rectrxm.jl:64,72): each element is multiplied by alpha
 * in Float64 and rounded back to the element type, as Julia's promotion does.
 */
NLA_API int nla_scale(int dtype, int64_t rows, int64_t cols, double alpha, void* B, int64_t ldb, void* stream);

/* nla_scale for complex types with a complex alpha (the product in
 * ComplexF64, rounded to the element type). */
NLA_API int nla_scale_complex(int dtype, int64_t rows, int64_t cols, double alpha_re, double alpha_im, void* B,
                              int64_t ldb, void* stream);

/*
 * Page-locked host memory for the host-buffer entry points (no counterpart in
 * the reference; a Julia caller would use CUDA.jl's pinned buffers):
 * nla_host_alloc returns `bytes` of page-locked, 256-byte aligned host memory
 * (cudaHostAlloc), nla_host_free releases it.  Copies from and to it run at
 * the copy engines' rate without staging.
 */
NLA_API int nla_host_alloc(size_t bytes, void** out);
NLA_API int nla_host_free(void* p);

/*
 * Mixed-precision form (no counterpart in the reference): the FP64 answer of
 * unified_rectrxm! for Float64 A and B, with the off-diagonal updates on the
 * tcgen05 tensor cores.  Each update operand is split into `split_terms`
 * BF16 (lowp NLA_LOWP_BF16) or FP16 (NLA_LOWP_F16) slices with one
 * power-of-two scale per row / column, slice products accumulate in FP32, and
 * the diagonal blocks (size `cutoff`, default 64) are solved or multiplied in
 * FP64.  Solves then run `sweeps` refinement sweeps: R = alpha*B - op(A) X with
 * an FP64-accurate residual product (`residual`), op(A) D = R with the same
 * mixed solver, X += D.  If corr_out is not
 * NULL it receives max|D| / max|X| of each sweep (host array of `sweeps`
 * doubles; the call then synchronises the stream).  Multiplies (func 'M')
 * ignore `sweeps`.  Inputs must be finite.
 */
#define NLA_LOWP_BF16 0
#define NLA_LOWP_F16 1
#define NLA_RESIDUAL_FP64 0  /* residual product on the FP64 pipe (DFMA) */
#define NLA_RESIDUAL_SPLIT 1 /* residual product from 7 BF16 slices per operand with
                                exact FP32 chunk sums and 64-bit integer accumulation */
#define NLA_RESIDUAL_DD 2    /* nla_trxm_residual only: double-double accumulation on
                                the FP64 pipe, rounded once (for measuring errors) */
typedef struct {
  int lowp;          /* NLA_LOWP_BF16 or NLA_LOWP_F16 */
  int split_terms;   /* 1, 2 or 3 slices per operand; 7 = exact BF16 slice products (FP64-accurate updates) */
  int sweeps;        /* refinement sweeps for solves, 0..8 */
  int residual;      /* how the residual product is formed */
  int64_t cutoff;    /* FP64 diagonal block size; <= 0 selects the default */
  double* corr_out;  /* host, `sweeps` entries, or NULL */
} nla_mixed_opts;
NLA_API int nla_trxm_mixed(char side, char uplo, char trans, double alpha, char func, int64_t n, int64_t m,
                           const double* A, int64_t lda, double* B, int64_t ldb, const nla_mixed_opts* opts,
                           void* stream);

/*
 * nla_trxm_mixed with a unit-diagonal option, as nla_trxm_diag is to
 * nla_trxm: diag 'U' takes the diagonal of A as ones and never reads it (the
 * recursive LU's solve with its unit lower factor, BLAS.trsm!('L', 'L', 'N',
 * 'U') at src/lu.jl:277, whose diagonal holds U's).  Unit-diagonal solves
 * take no refinement sweeps (NLA_ERR_UNSUPPORTED): use the exact 7-term
 * updates, whose solves need none.
 */
NLA_API int nla_trxm_mixed_diag(char side, char uplo, char trans, char diag, double alpha, char func, int64_t n,
                                int64_t m, const double* A, int64_t lda, double* B, int64_t ldb,
                                const nla_mixed_opts* opts, void* stream);

/*
 * Host-buffer forms of nla_trxm and nla_trxm_mixed: what a Julia caller does
 * with host arrays around unified_rectrxm! (CuArray(A), CuArray(B), the call,
 * copyto!(B, dB); src/rectrxm.jl:43-76), as one call.
 *
 * A_host and B_host are column-major host arrays (page-locked for the copies
 * to overlap); A_dev and B_dev are caller-owned device arrays of the same
 * shapes with leading dimensions lda_dev and ldb_dev.  The result goes to
 * the host array X_host of B's shape (X_host == B_host with ldx == ldb is
 * the reference's in-place form); B_dev holds it too.  B_host is only read
 * and must not overlap X_host otherwise.  The top `host_levels` levels of the
 * recursion (<= 0: the library default, 3) are split into blocks: each block
 * of A and of B is copied to the device on a copy stream just before the
 * recursion first touches it, and each block of the result is copied back
 * on a second copy stream as soon as it is final, so copies overlap the
 * solve.  Only the diagonal blocks and the off-diagonal blocks of the
 * `uplo` triangle that the recursion reads are copied; the rest of A_dev is
 * left as it was.  Refinement sweeps (nla_trxm_mixed with sweeps > 0) need
 * all of the first solution, so that form copies in, solves and copies out
 * without overlap.  The results are bit-identical to nla_trxm /
 * nla_trxm_mixed on A_dev and B_dev.  Asynchronous on `stream`: B_host holds
 * the result once the stream has been synchronised.
 */
NLA_API int nla_trxm_host(char side, char uplo, char trans, double alpha, char func, int dtype, int64_t n, int64_t m,
                          const void* A_host, int64_t lda, const void* B_host, int64_t ldb, void* X_host,
                          int64_t ldx, void* A_dev, int64_t lda_dev, void* B_dev, int64_t ldb_dev, int host_levels,
                          void* stream);
NLA_API int nla_trxm_mixed_host(char side, char uplo, char trans, double alpha, char func, int64_t n, int64_t m,
                                const double* A_host, int64_t lda, const double* B_host, int64_t ldb, double* X_host,
                                int64_t ldx, double* A_dev, int64_t lda_dev, double* B_dev, int64_t ldb_dev,
                                const nla_mixed_opts* opts, int host_levels, void* stream);

/*
 * One mixed-precision off-diagonal update (no counterpart in the reference;
 * the mixed form of matmul!, src/matmul.jl:5-66): out (N x M, FP64) +=
 * alpha * op(in1) (N x R) * op(in2) (R x M) from `split_terms` BF16/FP16
 * slices per operand on the tensor cores (1-3: FP32 accumulation; 7: BF16
 * only, exact slice products accumulated in 64-bit integers, FP64-accurate).
 */
NLA_API int nla_gemm_update_mixed(int trans1, int trans2, int64_t N, int64_t R, int64_t M, double alpha,
                                  const double* in1, int64_t ld1, const double* in2, int64_t ld2, double* out,
                                  int64_t ldo, int lowp, int split_terms, void* stream);

/*
 * The residual of a solve, FP64-accurate (no counterpart in the reference):
 * R = alpha*B - op(A) X (side 'L') or alpha*B - X op(A) (side 'R'), with A
 * n x n triangular (uplo, trans as for nla_trxm) and X, B, R of B's shape.
 * `residual` selects NLA_RESIDUAL_SPLIT (tensor cores, exact slice products),
 * NLA_RESIDUAL_FP64 (FP64 pipe) or NLA_RESIDUAL_DD (double-double, rounded
 * once: the reference value for backward errors).  R must not overlap X or B.
 */
NLA_API int nla_trxm_residual(char side, char uplo, char trans, double alpha, int64_t n, int64_t m, const double* A,
                              int64_t lda, const double* X, int64_t ldx, const double* B, int64_t ldb, double* R,
                              int64_t ldr, int residual, void* stream);

/*
 * nla_gemm_update_mixed without any device allocation.  No counterpart in the
 * reference (which allocates nothing itself but has no mixed form).
 * Some callers cannot let a library call cudaMalloc: a host framework that
 * owns all device memory through its own allocator, a process held to a fixed
 * device-memory budget, or a latency-critical loop that cannot absorb an
 * allocation.  This entry point stages its operands in a static device array
 * of NLA_NOALLOC_SCRATCH_BYTES that the library defines (held by every GPU
 * that loads the library until the process exits) instead of the pooled
 * workspace.  Updates whose staging would exceed that size fail with
 * NLA_ERR_WORKSPACE: with 3 slices, for example, about (N + M) * R <= 11e6
 * once N, M are rounded up to 128 and R to 64.  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress); make that first
 * call before any stream capture; the address is cached per device, so
 * resetting the device after that first call is not supported.  All calls
 * share the array: calls that overlap on the GPU (concurrent streams or
 * unordered host threads) race.
 */
#define NLA_NOALLOC_SCRATCH_BYTES (64ll << 20)
NLA_API int nla_gemm_update_mixed_noalloc(int trans1, int trans2, int64_t N, int64_t R, int64_t M, double alpha,
                                          const double* in1, int64_t ld1, const double* in2, int64_t ld2,
                                          double* out, int64_t ldo, int lowp, int split_terms, void* stream);

/*
 * Synchronises `stream` and reports (then clears) the device-side error word
 * that the tensor-core kernels raise when a bounded wait gives up:
 * NLA_OK or NLA_ERR_TIMEOUT.
 */
NLA_API int nla_device_status(void* stream);

/*
 * Give-up limit, in nanoseconds, of the waits between the roles of a
 * tensor-core kernel on the current device (TMA producer, MMA issuer,
 * accumulator drain); 0 restores the default of 2 s.  No counterpart in the
 * reference, which has no bounded waits.  A wait past the limit makes the
 * kernel stop, wait for its own in-flight loads and tensor-core work with the
 * default limit, release its tensor memory and return; nla_device_status then
 * reports NLA_ERR_TIMEOUT.  A limit below 1 ms makes nearly every wait that
 * does not complete at once give up: that is how the tests drive this path.
 * Takes effect for kernels launched after it returns.
 */
NLA_API int nla_set_wait_limit_ns(uint64_t ns);

/*
 * Batched solve of independent, unevenly sized systems (no counterpart in the
 * reference, which solves one system per unified_rectrxm! call,
 * src/rectrxm.jl:43-76).  Every system i solves op(A_i) X_i = alpha B_i
 * (side 'L', the batch's uplo and trans) in place in B_i, with A_i n_i x n_i
 * (n_i <= 1024) at A_pool + a_off elements and B_i n_i x m_i at
 * B_pool + b_off elements, column-major with leading dimensions lda, ldb.
 * A plan runs the recursion of unified_rec (src/rectrxm.jl:101-198) for every
 * system and block of right-hand sides (a group) on the host, down to leaves
 * of at most `cutoff` rows, and uploads its pieces as a queue of nodes: leaf
 * solves and update tiles (one per leaf the recursion's GEMM updates, with
 * the K range of the half solved first).  The queue is ordered by a
 * list-scheduling simulation over the persistent CTAs; nodes wait on
 * per-group and per-leaf counters for the nodes they depend on, each wait
 * bounded (nla_set_wait_limit_ns; nla_device_status reports one that gave
 * up).  Per size bucket b (16*2^b <= n < 32*2^b, the last bucket open above)
 * `tuning` gives the leaf order (16, 32 or 64) and the widest block of
 * right-hand sides (16, 32, 64 or 128); NULL takes defaults.  With
 * nla_batch_plan_create, `cols_per_item` gives only the block widths.  The
 * plan owns device memory until destroyed; one plan must not be used from
 * two streams at once.  nla_batch_plan_info reports the number of nodes.
 * Modes of nla_batch_solve:
 *   NLA_BATCH_GRAPH       one persistent kernel, captured once into a CUDA
 *                         graph (re-captured when alpha or the pools change)
 *                         and replayed;
 *   NLA_BATCH_PERSISTENT  the same kernel launched directly;
 *   NLA_BATCH_LOOP        one nla_trxm recursion per system (the baseline).
 */
typedef struct {
  int64_t n, m;
  int64_t a_off, lda;
  int64_t b_off, ldb;
} nla_batch_desc;
#define NLA_BATCH_BUCKETS 6
typedef struct {
  int cutoff[NLA_BATCH_BUCKETS]; /* leaf order per size bucket: 16, 32 or 64 */
  int cols[NLA_BATCH_BUCKETS];   /* widest block of right-hand sides: 16, 32, 64 or 128 */
} nla_batch_tuning;
#define NLA_BATCH_GRAPH 0
#define NLA_BATCH_PERSISTENT 1
#define NLA_BATCH_LOOP 2
typedef struct nla_batch_plan_s* nla_batch_plan;
NLA_API int nla_batch_plan_create(nla_batch_plan* plan, int dtype, char uplo, char trans, int64_t count,
                                  const nla_batch_desc* descs, const int* cols_per_item);
NLA_API int nla_batch_plan_create_tuned(nla_batch_plan* plan, int dtype, char uplo, char trans, int64_t count,
                                        const nla_batch_desc* descs, const nla_batch_tuning* tuning);
NLA_API int nla_batch_plan_info(nla_batch_plan plan, int64_t* items, int64_t* grid, double* flops);
NLA_API int nla_batch_solve(nla_batch_plan plan, double alpha, const void* A_pool, void* B_pool, int mode,
                            void* stream);
NLA_API int nla_batch_plan_destroy(nla_batch_plan plan);

/*
 * Mixed-precision form of a Float64 batch (plan created with NLA_F64; no
 * counterpart in the reference).  Every system is solved in Float32 (A_i and
 * alpha B_i rounded to Float32) and then refined `sweeps` times (0..8):
 * R_i = alpha B_i - op(A_i) X_i, a Float32 solve of op(A_i) D_i = R_i,
 * X_i += D_i.  X_i (Float64) replaces B_i.  The residual is Float64-accurate:
 * with `residual` NLA_RESIDUAL_SPLIT (the default of nla_batch_solve_mixed)
 * op(A_i) X_i is formed on the tcgen05 tensor cores from seven BF16 slices of
 * every 64-wide block of each row and column, the slice products summed
 * exactly; with NLA_RESIDUAL_FP64 on the FP64 pipe.  The elements of A and B
 * must be finite and lie in the Float32 range.  The plan allocates Float32
 * copies of the pools, a Float64 residual buffer and the residual's tile list
 * on first use and keeps them until destroyed.
 */
NLA_API int nla_batch_solve_mixed(nla_batch_plan plan, double alpha, const void* A_pool, void* B_pool, int sweeps,
                                  void* stream);
NLA_API int nla_batch_solve_mixed_ex(nla_batch_plan plan, double alpha, const void* A_pool, void* B_pool, int sweeps,
                                     int residual, void* stream);

/*
 * Measured throughput (TFLOP/s) of the pipes the plain paths use on the
 * current GPU (no counterpart in the reference): FP64 FMA on CUDA cores,
 * FP64 mma.sync m8n8k4, FP32 FMA.  Any output pointer may be NULL.  Runs a
 * few milliseconds of probe kernels on `stream` and synchronises it.
 */
NLA_API int nla_measure_pipes(double* dfma_tflops, double* dmma_tflops, double* ffma_tflops, void* stream);

/*
 * Kernel tracing (no counterpart in the reference, which has no tracing).
 * nla_trace_enable(1) clears earlier records and starts recording; every
 * library operation launched afterwards (one kernel, or a few that belong
 * together, such as an update and its finishing pass) is bracketed by CUDA
 * events on its stream together with its algorithmic flops and bytes.
 * nla_trace_enable(0) stops recording.  nla_trace_summary() waits for the
 * recorded events and returns, for one kernel class, the number of kernel
 * launches (copies count one each), their summed device time in milliseconds
 * and their summed algorithmic flops and bytes.  Do not trace work that is
 * being captured into a CUDA graph.
 */
#define NLA_K_LEAF_SOLVE 0 /* diagonal-block solve */
#define NLA_K_LEAF_MULT 1  /* diagonal-block multiply */
#define NLA_K_GEMM_SIMT 2  /* off-diagonal update on CUDA cores */
#define NLA_K_GEMM_UMMA 3  /* off-diagonal update on tcgen05 tensor cores */
#define NLA_K_SPLIT 4      /* operand split / staging for the tensor-core update */
#define NLA_K_SCALE 5      /* alpha scaling and element-wise passes */
#define NLA_K_RESIDUAL 6   /* residual and correction passes of refinement */
#define NLA_K_BATCHED 7    /* persistent batched solve */
#define NLA_K_COPY_IN 8    /* host-to-device block copies of the host-buffer entry points (bytes, no flops) */
#define NLA_K_COPY_OUT 9   /* device-to-host block copies of the host-buffer entry points */
#define NLA_K_COUNT 10
NLA_API int nla_trace_enable(int on);
NLA_API int nla_trace_summary(int kernel_class, int64_t* launches, double* ms, double* flops, double* bytes);

#ifdef __cplusplus
}
#endif

#endif /* NEXTLA_GB300_H */
