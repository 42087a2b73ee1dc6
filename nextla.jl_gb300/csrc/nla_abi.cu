// C ABI entry points and the native host recursion of unified_rectrxm!.
//
// nla_trxm mirrors src/rectrxm.jl:43-198: the trans flag becomes a transposed
// view of A with uplo flipped (src/rectrxm.jl:56-59), alpha scales B before a
// solve (:62-65) and after a multiply (:71-73), and the recursion splits at
// n/2 for powers of two and at the largest power of two below n otherwise
// (:129-133), with the forward (A11 -> GEMM -> A22) or backward ordering of
// :153-197.  Each base case is one launch of the diagonal-block kernel and
// each update one launch of the GEMM kernel, all on the caller's stream.
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "nla_common.cuh"

namespace nla {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }
int fail(int code, const std::string& msg) {
  set_error(msg);
  return code;
}
int cuda_status(cudaError_t e, const char* where) {
  set_error(std::string(where) + ": " + cudaGetErrorString(e));
  return NLA_ERR_CUDA_BASE - (int)e;
}

// ---------------------------------------------------------------------------
// Tracing.
// ---------------------------------------------------------------------------
namespace {
struct TraceRec {
  int kclass;
  cudaEvent_t e0, e1;
  double flops, bytes;
  int kernels;       // kernel launches inside the scope
  TraceRec* parent;  // the scope open around this one on the same thread
};
std::mutex g_trace_mu;
std::atomic<bool> g_trace_on{false};
std::vector<TraceRec*> g_trace;
std::vector<cudaEvent_t> g_event_pool;

cudaEvent_t pooled_event() {
  if (!g_event_pool.empty()) {
    cudaEvent_t e = g_event_pool.back();
    g_event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void clear_trace_locked() {
  for (TraceRec* r : g_trace) {
    g_event_pool.push_back(r->e0);
    g_event_pool.push_back(r->e1);
    delete r;
  }
  g_trace.clear();
}
}  // namespace

namespace {
thread_local int t_trace_class = -1;  // TraceClassScope's override, or -1
thread_local TraceRec* t_trace_open = nullptr;  // innermost recording scope of this thread
}

TraceClassScope::TraceClassScope(int kclass) : prev(t_trace_class) { t_trace_class = kclass; }
TraceClassScope::~TraceClassScope() { t_trace_class = prev; }

void trace_begin(int kclass, cudaStream_t s, double flops, double bytes, void** handle) {
  *handle = nullptr;
  if (!g_trace_on.load(std::memory_order_relaxed)) return;
  if (t_trace_class >= 0) kclass = t_trace_class;
  std::lock_guard<std::mutex> lk(g_trace_mu);
  TraceRec* r = new TraceRec{kclass, pooled_event(), pooled_event(), flops, bytes, 1, t_trace_open};
  cudaEventRecord(r->e0, s);
  g_trace.push_back(r);
  t_trace_open = r;
  *handle = r;
}

void trace_end(void* handle, cudaStream_t s) {
  TraceRec* r = static_cast<TraceRec*>(handle);
  cudaEventRecord(r->e1, s);
  if (t_trace_open == r) t_trace_open = r->parent;
}

void trace_kernels(int extra) {
  if (!t_trace_open) return;
  std::lock_guard<std::mutex> lk(g_trace_mu);
  t_trace_open->kernels += extra;
}

int num_sms() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

// ---------------------------------------------------------------------------
// Alpha scaling: B .= alpha .* B with the product formed in Float64 and
// rounded back to the element type (src/rectrxm.jl:64,72).  When alpha is
// exactly representable in Float32 the Float32 product of a Float32/Float16
// element is already the correctly rounded result, so no FP64 operation is
// issued (GB300 runs FP64 at 1/64 of the FP32 rate).
// ---------------------------------------------------------------------------
template <typename T, typename Tm>
__global__ void scale_kernel(int64_t rows, int64_t cols, Tm alpha, T* B, int64_t ldb, int tB) {
  const int64_t total = rows * cols;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t i, j;
    if (!tB) { i = idx % rows; j = idx / rows; }
    else { j = idx % cols; i = idx / cols; }
    T* p = B + mat_off(i, j, ldb, tB);
    Tm v = (Tm)Elem<T>::load(p) * alpha;
    if constexpr (sizeof(Tm) == 8) Elem<T>::store_d(p, (double)v);  // one rounding from the Float64 product
    else Elem<T>::store(p, v);
  }
}

int launch_scale(int dtype, int64_t rows, int64_t cols, double alpha, const Mat& B, cudaStream_t s) {
  if (is_complex(dtype)) return launch_scale_complex(dtype, rows, cols, alpha, 0.0, B, s);
  if (rows <= 0 || cols <= 0 || alpha == 1.0) return NLA_OK;
  const int64_t total = rows * cols;
  int64_t blocks = (total + 255) / 256;
  const int64_t cap = (int64_t)num_sms() * 8;
  if (blocks > cap) blocks = cap;
  const bool f32_exact = (double)(float)alpha == alpha;
  TraceScope trace(NLA_K_SCALE, s, (double)total, 2.0 * (double)total * (double)dtype_size(dtype));
  switch (dtype) {
    case NLA_F64:
      scale_kernel<double, double><<<(unsigned)blocks, 256, 0, s>>>(rows, cols, alpha, (double*)B.p, B.ld, B.t);
      break;
    case NLA_F32:
      if (f32_exact)
        scale_kernel<float, float><<<(unsigned)blocks, 256, 0, s>>>(rows, cols, (float)alpha, (float*)B.p, B.ld, B.t);
      else
        scale_kernel<float, double><<<(unsigned)blocks, 256, 0, s>>>(rows, cols, alpha, (float*)B.p, B.ld, B.t);
      break;
    case NLA_F16:
      if (f32_exact)
        scale_kernel<__half, float><<<(unsigned)blocks, 256, 0, s>>>(rows, cols, (float)alpha, (__half*)B.p, B.ld,
                                                                      B.t);
      else
        scale_kernel<__half, double><<<(unsigned)blocks, 256, 0, s>>>(rows, cols, alpha, (__half*)B.p, B.ld, B.t);
      break;
    default: return fail(NLA_ERR_DTYPE, "scale: unknown dtype");
  }
  NLA_CHECK_LAUNCH("scale_kernel");
  return NLA_OK;
}

int launch_gemm_simt(int dtype, int64_t N, int64_t M, int64_t K, double alpha, const Mat& A, const Mat& B,
                     const Mat& C, cudaStream_t s);

static bool umma_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("NLA_DISABLE_UMMA");
    return !(v && *v && *v != '0');
  }();
  return on;
}

// Float16 updates large enough to fill 128 x 128 tiles run on the tensor
// cores (FP32 accumulation); everything else on CUDA cores.
int launch_gemm(int dtype, int64_t N, int64_t M, int64_t K, double alpha, const Mat& A, const Mat& B, const Mat& C,
                cudaStream_t s) {
  if (is_complex(dtype)) return launch_gemm_complex(dtype, N, M, K, alpha, A, B, C, s);
  if (dtype == NLA_F16 && umma_enabled() && N >= 128 && M >= 128 && K >= 64)
    return launch_sliced_gemm(N, M, K, alpha, A, B, C, NLA_F16, NLA_F16, 1, false, nullptr, 0, s);
  return launch_gemm_simt(dtype, N, M, K, alpha, A, B, C, s);
}

static int launch_update(const RecPlan& c, int64_t N, int64_t M, int64_t K, double alpha, const Mat& A,
                         const Mat& B, const Mat& C) {
  if (c.mode == GEMM_MIXED)
    return launch_sliced_gemm(N, M, K, alpha, A, B, C, NLA_F64, NLA_F64, c.S, c.bf16, nullptr, 0, c.s);
  return launch_gemm(c.dtype, N, M, K, alpha, A, B, C, c.s);
}

// ---------------------------------------------------------------------------
// Argument checks.
// ---------------------------------------------------------------------------
static bool valid_side(char c) { return c == 'L' || c == 'R'; }
static bool valid_uplo(char c) { return c == 'L' || c == 'U'; }
static bool valid_trans(char c) { return c == 'N' || c == 'T' || c == 'C'; }
static bool valid_func(char c) { return c == 'S' || c == 'M'; }
static bool valid_dtype(int d) {
  return d == NLA_F16 || d == NLA_F32 || d == NLA_F64 || d == NLA_C32 || d == NLA_C64;
}

int check_flags(char side, char uplo, char trans, char func, int dtype) {
  if (!valid_side(side)) return fail(NLA_ERR_ARG, std::string("side must be 'L' or 'R', got '") + side + "'");
  if (!valid_uplo(uplo)) return fail(NLA_ERR_ARG, std::string("uplo must be 'L' or 'U', got '") + uplo + "'");
  if (!valid_trans(trans))
    return fail(NLA_ERR_ARG, std::string("transpose must be 'N', 'T' or 'C', got '") + trans + "'");
  if (!valid_func(func)) return fail(NLA_ERR_ARG, std::string("func must be 'S' or 'M', got '") + func + "'");
  if (!valid_dtype(dtype)) return fail(NLA_ERR_DTYPE, "dtype must be NLA_F16, NLA_F32, NLA_F64, NLA_C32 or NLA_C64");
  return NLA_OK;
}

int check_matrix(const char* name, const void* p, int64_t rows, int64_t cols, int64_t ld) {
  if (rows < 0 || cols < 0) return fail(NLA_ERR_ARG, std::string(name) + ": negative dimension");
  const int64_t need = rows > 1 ? rows : 1;
  if (ld < need) return fail(NLA_ERR_ARG, std::string(name) + ": leading dimension smaller than the row count");
  if (rows > 0 && cols > 0 && p == nullptr) return fail(NLA_ERR_ARG, std::string(name) + ": null pointer");
  return NLA_OK;
}

// src/rectrxm.jl:129-133
int64_t split_point(int64_t n) {
  int64_t p = 1;
  while (p * 2 <= n) p *= 2;
  return p == n ? n / 2 : p;
}

// ---------------------------------------------------------------------------
// Recursion (unified_rec, src/rectrxm.jl:101-198).
// ---------------------------------------------------------------------------
// The first half (A11, B1) is processed first in these four cases
// (src/rectrxm.jl:104-124); otherwise the second half (A22, B2) is.
bool rec_forward(const RecPlan& c) {
  const bool S = c.func == 'S', L = c.side == 'L';
  return (L && c.uplo == 'L' && S) || (!L && c.uplo == 'U' && S) || (L && c.uplo == 'U' && !S) ||
         (!L && c.uplo == 'L' && !S);
}

// Whether the update between the halves reads A21 (else A12).
bool rec_update_reads_a21(const RecPlan& c) {
  return rec_forward(c) != (c.side == 'R') != (c.func == 'M');
}

// The update between the two halves of one recursion node on the n x n
// diagonal block A and its rows (side 'L') or columns ('R') of B.  A solve
// writes the half processed second from the one solved first; a multiply
// adds into the half processed first from the other.
int rec_update(const RecPlan& c, const Mat& A, int64_t n, const Mat& B) {
  const int64_t mid = split_point(n), rem = n - mid;
  const int d = c.dtype;
  const Mat A21 = sub(A, mid, 0, d), A12 = sub(A, 0, mid, d);
  const Mat B1 = B, B2 = c.side == 'L' ? sub(B, mid, 0, d) : sub(B, 0, mid, d);
  const bool S = c.func == 'S', L = c.side == 'L';
  const int64_t m = c.m;
  if (rec_forward(c)) {
    if (L) {
      if (S) return launch_update(c, rem, m, mid, -1.0, A21, B1, B2);  // B2 -= A21*B1
      return launch_update(c, mid, m, rem, 1.0, A12, B2, B1);          // B1 += A12*B2
    }
    if (S) return launch_update(c, m, rem, mid, -1.0, B1, A12, B2);  // B2 -= B1*A12
    return launch_update(c, m, mid, rem, 1.0, B2, A21, B1);          // B1 += B2*A21
  }
  if (L) {
    if (S) return launch_update(c, mid, m, rem, -1.0, A12, B2, B1);  // B1 -= A12*B2
    return launch_update(c, rem, m, mid, 1.0, A21, B1, B2);          // B2 += A21*B1
  }
  if (S) return launch_update(c, m, mid, rem, -1.0, B2, A21, B1);  // B1 -= B2*A21
  return launch_update(c, m, rem, mid, 1.0, B1, A12, B2);          // B2 += B1*A12
}

int recurse(const RecPlan& c, const Mat& A, int64_t n, const Mat& B) {
  if (c.inv && leaf_pair_wanted(c, n)) return leaf_pair_apply(c, A, n, B);
  if (n <= c.threshold) {
    if (c.inv) return leaf_inverse_apply(c, A, n, B);
    return launch_leaf(c.func, c.side, c.uplo, c.dtype, n, c.m, A, B, c.s, c.unit);
  }
  const int64_t mid = split_point(n), rem = n - mid;
  const int d = c.dtype;
  const Mat A11 = A, A22 = sub(A, mid, mid, d);
  const Mat B1 = B, B2 = c.side == 'L' ? sub(B, mid, 0, d) : sub(B, 0, mid, d);
  if (rec_forward(c)) {
    NLA_TRY(recurse(c, A11, mid, B1));
    NLA_TRY(rec_update(c, A, n, B));
    return recurse(c, A22, rem, B2);
  }
  NLA_TRY(recurse(c, A22, rem, B2));
  NLA_TRY(rec_update(c, A, n, B));
  return recurse(c, A11, mid, B1);
}

static int64_t env_cutoff(const char* name, int64_t dflt) {
  const char* v = std::getenv(name);
  if (!v || !*v) return dflt;
  long long x = std::atoll(v);
  return x > 0 ? (int64_t)x : dflt;
}

int64_t default_cutoff(char func, int dtype) {
  if (func == 'S') return env_cutoff("NLA_TRXM_CUTOFF_S", 256);
  (void)dtype;
  return env_cutoff("NLA_TRXM_CUTOFF_M", 128);
}

int trxm_plan(char side, char uplo, char trans, char func, int dtype, int64_t n, int64_t m, const void* A,
              int64_t lda, const void* B, int64_t ldb, int64_t cutoff_s, int64_t cutoff_m, cudaStream_t s, bool unit,
              RecPlan* c, int* a_trans) {
  NLA_TRY(check_flags(side, uplo, trans, func, dtype));
  if (n < 0 || m < 0) return fail(NLA_ERR_ARG, "n and m must be non-negative");
  NLA_TRY(check_matrix("A", A, n, n, lda));
  NLA_TRY(check_matrix("B", B, side == 'L' ? n : m, side == 'L' ? m : n, ldb));
  *a_trans = 0;
  if (trans == 'T' || trans == 'C') {  // src/rectrxm.jl:56-59
    *a_trans = 1;
    uplo = uplo == 'L' ? 'U' : 'L';
  }
  *c = RecPlan{func, side, uplo, dtype, m, 0, s, GEMM_PLAIN, 1, false};
  c->unit = unit;
  const int64_t cut = func == 'S' ? (cutoff_s > 0 ? cutoff_s : default_cutoff('S', dtype))
                                  : (cutoff_m > 0 ? cutoff_m : default_cutoff('M', dtype));
  // Complex diagonal blocks hold their rows of right-hand sides and a panel
  // of the triangle in shared memory: at most 128 rows.
  const int64_t cap = is_complex(dtype) ? 128 : 1024;
  c->threshold = cut > cap ? cap : cut;
  return NLA_OK;
}

int trxm_impl(char side, char uplo, char trans, double alpha, char func, int dtype, int64_t n, int64_t m,
              const void* A, int64_t lda, void* B, int64_t ldb, int64_t cutoff_s, int64_t cutoff_m, cudaStream_t s,
              bool unit, double alpha_im) {
  RecPlan c{};
  int at = 0;
  NLA_TRY(trxm_plan(side, uplo, trans, func, dtype, n, m, A, lda, B, ldb, cutoff_s, cutoff_m, s, unit, &c, &at));
  if (alpha_im != 0.0 && !is_complex(dtype)) return fail(NLA_ERR_DTYPE, "a complex alpha needs a complex dtype");
  if (n == 0 || m == 0) return NLA_OK;
  Mat Am{const_cast<void*>(A), lda, at};
  Am.c = trans == 'C' && is_complex(dtype);  // Adjoint(A), src/rectrxm.jl:56-59
  const Mat Bm{B, ldb, 0};
  const int64_t rows = side == 'L' ? n : m, cols = side == 'L' ? m : n;
  auto scale = [&]() {
    return is_complex(dtype) ? launch_scale_complex(dtype, rows, cols, alpha, alpha_im, Bm, s)
                             : launch_scale(dtype, rows, cols, alpha, Bm, s);
  };
  if (func == 'S') NLA_TRY(scale());  // src/rectrxm.jl:64
  NLA_TRY(recurse(c, Am, n, Bm));
  if (func == 'M') NLA_TRY(scale());  // src/rectrxm.jl:72
  return NLA_OK;
}

}  // namespace nla

using namespace nla;

extern "C" {

int nla_version(void) { return 100; }

int nla_trace_enable(int on) {
  clear_error();
  std::lock_guard<std::mutex> lk(g_trace_mu);
  if (on) clear_trace_locked();
  g_trace_on.store(on != 0);
  return NLA_OK;
}

int nla_trace_summary(int kernel_class, int64_t* launches, double* ms, double* flops, double* bytes) {
  clear_error();
  if (kernel_class < 0 || kernel_class >= NLA_K_COUNT) return fail(NLA_ERR_ARG, "unknown kernel class");
  std::lock_guard<std::mutex> lk(g_trace_mu);
  int64_t n = 0;
  double t = 0, f = 0, b = 0;
  for (TraceRec* r : g_trace) {
    if (r->kclass != kernel_class) continue;
    cudaError_t e = cudaEventSynchronize(r->e1);
    if (e != cudaSuccess) return cuda_status(e, "nla_trace_summary");
    float x = 0;
    e = cudaEventElapsedTime(&x, r->e0, r->e1);
    if (e != cudaSuccess) return cuda_status(e, "nla_trace_summary");
    n += r->kernels;
    t += x;
    f += r->flops;
    b += r->bytes;
  }
  if (launches) *launches = n;
  if (ms) *ms = t;
  if (flops) *flops = f;
  if (bytes) *bytes = b;
  return NLA_OK;
}

const char* nla_last_error(void) { return g_last_error.c_str(); }

int nla_trxm(char side, char uplo, char trans, double alpha, char func, int dtype, int64_t n, int64_t m,
             const void* A, int64_t lda, void* B, int64_t ldb, void* stream) {
  clear_error();
  return trxm_impl(side, uplo, trans, alpha, func, dtype, n, m, A, lda, B, ldb, 0, 0, (cudaStream_t)stream);
}

int nla_trxm_complex(char side, char uplo, char trans, double alpha_re, double alpha_im, char func, int dtype,
                     int64_t n, int64_t m, const void* A, int64_t lda, void* B, int64_t ldb, void* stream) {
  clear_error();
  if (!is_complex(dtype)) return fail(NLA_ERR_DTYPE, "nla_trxm_complex: dtype must be NLA_C32 or NLA_C64");
  return trxm_impl(side, uplo, trans, alpha_re, func, dtype, n, m, A, lda, B, ldb, 0, 0, (cudaStream_t)stream, false,
                   alpha_im);
}

int nla_trxm_ex(char side, char uplo, char trans, double alpha, char func, int dtype, int64_t n, int64_t m,
                const void* A, int64_t lda, void* B, int64_t ldb, int64_t cutoff_s, int64_t cutoff_m, void* stream) {
  clear_error();
  return trxm_impl(side, uplo, trans, alpha, func, dtype, n, m, A, lda, B, ldb, cutoff_s, cutoff_m,
                   (cudaStream_t)stream);
}

int nla_trxm_diag(char side, char uplo, char trans, char diag, double alpha, char func, int dtype, int64_t n,
                  int64_t m, const void* A, int64_t lda, void* B, int64_t ldb, void* stream) {
  clear_error();
  if (diag != 'N' && diag != 'U') return fail(NLA_ERR_ARG, std::string("diag must be 'N' or 'U', got '") + diag + "'");
  return trxm_impl(side, uplo, trans, alpha, func, dtype, n, m, A, lda, B, ldb, 0, 0, (cudaStream_t)stream,
                   diag == 'U');
}

int nla_diag_block(char func, char side, char uplo, int transA, int dtype, int64_t n, int64_t m, const void* A,
                   int64_t lda, void* B, int64_t ldb, void* stream) {
  clear_error();
  NLA_TRY(check_flags(side, uplo, 'N', func, dtype));
  if (n < 0 || m < 0) return fail(NLA_ERR_ARG, "n and m must be non-negative");
  if (n > 1024) return fail(NLA_ERR_ARG, "diag block: n must be <= 1024");
  NLA_TRY(check_matrix("A", A, n, n, lda));
  NLA_TRY(check_matrix("B", B, side == 'L' ? n : m, side == 'L' ? m : n, ldb));
  Mat Am{const_cast<void*>(A), lda, transA & 1};
  Am.c = (transA & 2) && is_complex(dtype);
  Mat Bm{B, ldb, 0};
  return launch_leaf(func, side, uplo, dtype, n, m, Am, Bm, (cudaStream_t)stream);
}

int nla_gemm_update(int dtype, int trans1, int trans2, int64_t N, int64_t R, int64_t M, double alpha,
                    const void* in1, int64_t ld1, const void* in2, int64_t ld2, void* out, int64_t ldo, void* stream) {
  clear_error();
  if (!valid_dtype(dtype)) return fail(NLA_ERR_DTYPE, "dtype must be NLA_F16, NLA_F32, NLA_F64, NLA_C32 or NLA_C64");
  if (N < 0 || R < 0 || M < 0) return fail(NLA_ERR_ARG, "N, R and M must be non-negative");
  const int t1 = trans1 & 1, t2 = trans2 & 1;
  NLA_TRY(check_matrix("in1", in1, t1 ? R : N, t1 ? N : R, ld1));
  NLA_TRY(check_matrix("in2", in2, t2 ? M : R, t2 ? R : M, ld2));
  NLA_TRY(check_matrix("out", out, N, M, ldo));
  Mat A{const_cast<void*>(in1), ld1, t1};
  Mat B{const_cast<void*>(in2), ld2, t2};
  A.c = (trans1 & 2) && is_complex(dtype);
  B.c = (trans2 & 2) && is_complex(dtype);
  Mat C{out, ldo, 0};
  return launch_gemm(dtype, N, M, R, alpha, A, B, C, (cudaStream_t)stream);
}

int nla_scale(int dtype, int64_t rows, int64_t cols, double alpha, void* B, int64_t ldb, void* stream) {
  clear_error();
  if (!valid_dtype(dtype)) return fail(NLA_ERR_DTYPE, "dtype must be NLA_F16, NLA_F32, NLA_F64, NLA_C32 or NLA_C64");
  NLA_TRY(check_matrix("B", B, rows, cols, ldb));
  Mat Bm{B, ldb, 0};
  return launch_scale(dtype, rows, cols, alpha, Bm, (cudaStream_t)stream);
}

int nla_scale_complex(int dtype, int64_t rows, int64_t cols, double alpha_re, double alpha_im, void* B, int64_t ldb,
                      void* stream) {
  clear_error();
  if (!is_complex(dtype)) return fail(NLA_ERR_DTYPE, "nla_scale_complex: dtype must be NLA_C32 or NLA_C64");
  NLA_TRY(check_matrix("B", B, rows, cols, ldb));
  Mat Bm{B, ldb, 0};
  return launch_scale_complex(dtype, rows, cols, alpha_re, alpha_im, Bm, (cudaStream_t)stream);
}

}  // extern "C"
