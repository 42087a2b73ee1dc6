// Shared definitions of the GB300 triangular solve / multiply library.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/nextla_gb300.h"

namespace nla {

// ---------------------------------------------------------------------------
// Status reporting (thread-local message, negative codes).
// ---------------------------------------------------------------------------
void set_error(const std::string& msg);
void clear_error();
int fail(int code, const std::string& msg);
int cuda_status(cudaError_t e, const char* where);

#define NLA_CHECK_LAUNCH(where)                          \
  do {                                                   \
    cudaError_t e_ = cudaGetLastError();                 \
    if (e_ != cudaSuccess) return ::nla::cuda_status(e_, where); \
  } while (0)

#define NLA_TRY(expr)          \
  do {                         \
    int rc_ = (expr);          \
    if (rc_ != NLA_OK) return rc_; \
  } while (0)

// ---------------------------------------------------------------------------
// Matrix views.  A column-major parent with leading dimension ld; element
// (i,j) of the view is p[i + j*ld], or p[j + i*ld] when t is set (the
// library's form of a Julia Transpose/Adjoint wrapper of a real matrix).
// ---------------------------------------------------------------------------
struct Mat {
  void* p;
  int64_t ld;
  int t;
  int c = 0;  // complex types: read the conjugate of every element (an Adjoint view with t set)
};

inline size_t dtype_size(int dtype) {
  return dtype == NLA_C64 ? 16 : dtype == NLA_F64 || dtype == NLA_C32 ? 8 : dtype == NLA_F32 ? 4 : 2;
}

// Element offset of (i, j) in a view.
__host__ __device__ inline int64_t mat_off(int64_t i, int64_t j, int64_t ld, int t) {
  return t ? j + i * ld : i + j * ld;
}

// view(X, i0+1:end, j0+1:end)
inline Mat sub(const Mat& v, int64_t i0, int64_t j0, int dtype) {
  Mat r = v;
  r.p = static_cast<char*>(v.p) + mat_off(i0, j0, v.ld, v.t) * (int64_t)dtype_size(dtype);
  return r;
}

inline Mat transposed(const Mat& v) {
  Mat r = v;
  r.t = !v.t;
  return r;
}

// Element conversions between storage and compute types.
template <typename T> struct Elem;
template <> struct Elem<double> {
  using compute = double;
  __device__ static double load(const double* p) { return *p; }
  __device__ static void store(double* p, double v) { *p = v; }
  __device__ static void store_d(double* p, double v) { *p = v; }
};
template <> struct Elem<float> {
  using compute = float;
  __device__ static float load(const float* p) { return *p; }
  __device__ static void store(float* p, float v) { *p = v; }
  __device__ static void store_d(float* p, double v) { *p = (float)v; }
};
template <> struct Elem<__half> {
  using compute = float;
  __device__ static float load(const __half* p) { return __half2float(*p); }
  __device__ static void store(__half* p, float v) { *p = __float2half_rn(v); }
  __device__ static void store_d(__half* p, double v) { *p = __double2half(v); }
};

// ---------------------------------------------------------------------------
// Kernel tracing: when enabled (nla_trace_enable), each traced launch is
// bracketed by CUDA events on its stream and its algorithmic flops and bytes
// are recorded, so callers can measure per-kernel durations live.
// ---------------------------------------------------------------------------
void trace_begin(int kclass, cudaStream_t s, double flops, double bytes, void** handle);
void trace_end(void* handle, cudaStream_t s);
// Counts `extra` more kernel launches in the innermost recording scope of
// this thread (a scope counts one launch unless told otherwise).
void trace_kernels(int extra);

struct TraceScope {
  void* h = nullptr;
  cudaStream_t s;
  TraceScope(int kclass, cudaStream_t st, double flops, double bytes) : s(st) {
    trace_begin(kclass, st, flops, bytes, &h);
  }
  ~TraceScope() {
    if (h) trace_end(h, s);
  }
};

// ---------------------------------------------------------------------------
// Kernel launchers (defined in the .cu files).
// ---------------------------------------------------------------------------

// out (N x M) += alpha * op(A) (N x K) * op(B) (K x M), plain dtype-preserving path.
int launch_gemm(int dtype, int64_t N, int64_t M, int64_t K, double alpha, const Mat& A, const Mat& B, const Mat& C,
                cudaStream_t s);

// Base case on a diagonal block: func 'S' (solve) or 'M' (multiply).
int launch_leaf(char func, char side, char uplo, int dtype, int64_t n, int64_t m, const Mat& A, const Mat& B,
                cudaStream_t s, bool unit = false);

// B .= alpha .* B on a rows x cols view.
int launch_scale(int dtype, int64_t rows, int64_t cols, double alpha, const Mat& B, cudaStream_t s);

// Complex element types (nla_complex.cu): the same three pieces, with
// conjugated views (Mat::c) and a complex alpha for the scaling.
bool is_complex(int dtype);
int launch_leaf_complex(char func, char side, char uplo, int dtype, int64_t n, int64_t m, const Mat& A, const Mat& B,
                        cudaStream_t s, bool unit);
int launch_gemm_complex(int dtype, int64_t N, int64_t M, int64_t K, double alpha, const Mat& A, const Mat& B,
                        const Mat& C, cudaStream_t s);
int launch_scale_complex(int dtype, int64_t rows, int64_t cols, double alpha_re, double alpha_im, const Mat& B,
                         cudaStream_t s);

// Tensor-core update on staged slices (nla_umma.cu).  C (M x N) += alpha *
// op(A) (M x K) * op(B) (K x N); in_dtype NLA_F64 (split into S BF16/FP16
// slices) or NLA_F16 (one unscaled slice); out_dtype NLA_F64 or NLA_F16.
int launch_sliced_gemm(int64_t M, int64_t N, int64_t K, double alpha, const Mat& A, const Mat& B, const Mat& C,
                       int in_dtype, int out_dtype, int S, bool bf16, void* ws, size_t ws_bytes, cudaStream_t s);
size_t sliced_workspace_bytes(int64_t M, int64_t N, int64_t K, int S);

// An operand staged for the tensor cores: S K-major 16-bit slices of a
// rows x K view (padded to rows_pad x K_pad) and one exponent per row.
struct Staged {
  void* slices;
  int* e;
  float* nrm;  // per row: sum over k and slices of |s_p| 2^(-beta p)
  int64_t rows, rows_pad, K, K_pad;
  int S;
  bool bf16;
  bool scaled;
  int tri;  // 0 full, 1 k <= row, 2 k >= row, 3 k < row, 4 k > row
};
size_t staged_bytes(int64_t rows, int64_t K, int S);
// want_nrm: also the row-magnitude sums the exact kernel reads for its A
// operand (nrm is null in *out otherwise).
int stage_operand(const Mat& X, int64_t rows, int64_t K, int in_dtype, int S, bool bf16, int tri, void* buf,
                  Staged* out, cudaStream_t s, bool want_nrm = true);
// The diagonal term and final rounding of a residual computed by the exact
// update: C := C - P - d_i * X(pos), with d_i = d[i * dstride] (i the row of
// the staged A operand) and X at the position of C's element.
struct ResidualTerm {
  const double* x;
  int64_t ldx;
  const double* d;
  int64_t dstride;
};

// C (M x N, FP64) += alpha * A * B^T with exact slice-pair accumulation; both
// operands staged with 7 BF16 slices.  With trans_out the product is added
// to C^T (C is N x M).  With res, the epilogue instead forms a residual
// (alpha is then -1 implicitly), rounding once.
// fixed_buf (A.rows_pad x N int64, or null) lets a plain update leave its
// fixed-point sums there for a separate finishing pass over C.
int launch_exact_gemm(const Staged& A, const Staged& B, double alpha, const Mat& C, bool trans_out,
                      cudaStream_t s, const ResidualTerm* res = nullptr, long long* fixed_buf = nullptr);
constexpr int EXACT_SLICES = 7;
int workspace_get(cudaStream_t s, size_t bytes, void** out);
int device_status(cudaStream_t s);
int* device_error_word();  // device address of the error word nla_device_status reads (null on failure)
int set_wait_limit(uint64_t ns);
uint64_t wait_limit_ns();  // the limit last set (default 2 s), for kernels that take it as a parameter
int batch_device_error();  // the batched kernel's error word (read and cleared), or 0

// Inverses of the diagonal blocks (leaves) of a mixed solve's recursion,
// W = inv(T) for each leaf block T (lower or upper as the recursion sees it),
// one 64 x 64 slot each in w, slot j for the j-th leaf offset in k (relative
// to a_base).  A leaf is then X := W X on the tensor cores with the exact
// slice products.  The device path inverts every leaf before the recursion;
// the host-buffer path, where A arrives block by block, inverts the leaves of
// each block when the block arrives.
constexpr int LEAF_INV_N = 64;
struct LeafInverses {
  const double* a_base = nullptr;  // A (or the block) as the recursion indexes it
  int64_t lda = 0;
  double* w = nullptr;
  std::vector<int64_t> k;  // leaf offsets, increasing
  int* err = nullptr;  // the device error word of the bounded waits
};

// The recursion of unified_rec (src/rectrxm.jl:101-198) with a choice of
// update kernel.
enum GemmMode { GEMM_PLAIN = 0, GEMM_MIXED = 1 };
struct RecPlan {
  char func, side, uplo;
  int dtype;
  int64_t m;
  int64_t threshold;
  cudaStream_t s;
  int mode;
  int S;
  bool bf16;
  bool unit = false;  // unit diagonal
  const LeafInverses* inv = nullptr;  // leaves through their inverses (mixed exact solves)
};
int recurse(const RecPlan& c, const Mat& A, int64_t n, const Mat& B);
// Mixed exact solves: whether the leaves go through inverses (a 7-slice solve
// with leaves of at most LEAF_INV_N rows, unless NLA_MIXED_INV_LEAF=0), the
// inversion of every leaf of the n x n block A (one launch), and the leaf.
bool leaf_inverses_wanted(const RecPlan& c);
int leaf_inverses_upfront(const RecPlan& c, const Mat& A, int64_t n, LeafInverses* out);
int leaf_inverse_apply(const RecPlan& c, const Mat& A, int64_t n, const Mat& B);
// A recursion node whose two halves are both leaves, solved with the update
// between them in one launch (nla_mixed.cu).
bool leaf_pair_wanted(const RecPlan& c, int64_t n);
int leaf_pair_apply(const RecPlan& c, const Mat& A, int64_t n, const Mat& B);
// Launches inside the scope are traced under kernel class kclass (the leaf
// products of a mixed solve run the update kernels but are leaf work).
struct TraceClassScope {
  int prev;
  explicit TraceClassScope(int kclass);
  ~TraceClassScope();
};
// One node of the recursion: which half goes first, which off-diagonal block
// the update between the halves reads, and that update.
bool rec_forward(const RecPlan& c);
bool rec_update_reads_a21(const RecPlan& c);
int rec_update(const RecPlan& c, const Mat& A, int64_t n, const Mat& B);
// The plain recursion behind nla_trxm / nla_trxm_ex / nla_trxm_diag, and its
// argument checks and plan (a_trans: A is used transposed).
int trxm_plan(char side, char uplo, char trans, char func, int dtype, int64_t n, int64_t m, const void* A,
              int64_t lda, const void* B, int64_t ldb, int64_t cutoff_s, int64_t cutoff_m, cudaStream_t s, bool unit,
              RecPlan* c, int* a_trans);
int trxm_impl(char side, char uplo, char trans, double alpha, char func, int dtype, int64_t n, int64_t m,
              const void* A, int64_t lda, void* B, int64_t ldb, int64_t cutoff_s, int64_t cutoff_m, cudaStream_t s,
              bool unit = false, double alpha_im = 0.0);
// The mixed-precision recursion behind nla_trxm_mixed, and its checks and plan
// (which also sizes the update workspace on stream s).
int mixed_plan(char side, char uplo, char trans, char func, int64_t n, int64_t m, const void* A, int64_t lda,
               const void* B, int64_t ldb, const nla_mixed_opts* o, cudaStream_t s, RecPlan* c, int* a_trans,
               nla_mixed_opts* out);
int trxm_mixed_impl(char side, char uplo, char trans, double alpha, char func, int64_t n, int64_t m,
                    const double* A, int64_t lda, double* B, int64_t ldb, const nla_mixed_opts* o, cudaStream_t s,
                    bool unit = false);
int64_t split_point(int64_t n);
int check_flags(char side, char uplo, char trans, char func, int dtype);
int check_matrix(const char* name, const void* p, int64_t rows, int64_t cols, int64_t ld);

int num_sms();

}  // namespace nla
