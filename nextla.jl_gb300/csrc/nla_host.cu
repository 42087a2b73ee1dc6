// Host-buffer entry points (nla_trxm_host, nla_trxm_mixed_host).
//
// A Julia caller with host arrays wraps unified_rectrxm! (src/rectrxm.jl:43-76)
// in CuArray(A), CuArray(B) and copyto!(B, dB): copy everything in, solve,
// copy everything out.  Here the top levels of the recursion (unified_rec,
// src/rectrxm.jl:101-198) are walked on the host and split into blocks along
// the diagonal.  Each block of A and of B is copied in on a copy stream just
// before the recursion first touches it, and each block of the result is
// copied out on a second copy stream as soon as it is final.  The compute
// stream (the caller's) and the copy streams are ordered by events only, so
// the copies run under the solve.  Below the staged levels the device
// recursion runs unchanged, and every kernel sees the same operands in the
// same order as in nla_trxm / nla_trxm_mixed: the results are bit-identical.
#include <cstdlib>
#include <mutex>
#include <vector>

#include "nla_common.cuh"

namespace nla {
namespace {

constexpr int HOST_LEVELS_DEFAULT = 3;
constexpr int HOST_LEVELS_MAX = 12;
constexpr int MAX_DEVICES = 64;

// Two non-blocking copy streams per device (host to device, device to host),
// created on first use and kept for the life of the process.
struct CopyStreams {
  cudaStream_t in = nullptr, out = nullptr;
};
std::mutex g_host_mu;  // one host-buffer call enqueues at a time
CopyStreams g_copy[MAX_DEVICES];

int copy_streams(CopyStreams* out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "copy streams");
  if (dev < 0 || dev >= MAX_DEVICES) return fail(NLA_ERR_UNSUPPORTED, "device index out of range");
  CopyStreams& c = g_copy[dev];
  if (!c.in) {
    cudaStream_t a = nullptr, b = nullptr;
    e = cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      if (a) cudaStreamDestroy(a);
      return cuda_status(e, "copy streams");
    }
    c.in = a;
    c.out = b;
  }
  *out = c;
  return NLA_OK;
}

// One block of B's rows (side 'L') or columns ('R'): [k, k + len).
struct BlockB {
  int64_t k, len;
  bool in, out;
};

struct HostRun {
  RecPlan c;  // device recursion; c.s is the caller's (compute) stream
  double alpha;
  bool scale;  // apply alpha per block (off when the device call scales)
  size_t es;
  const char* Ah;
  int64_t ldah;
  char* Ad;
  int64_t ldad;
  int at;  // A is used transposed
  int conj = 0;  // complex types: and conjugated (trans 'C')
  const char* Bh;
  int64_t ldbh;
  char* Xh;
  int64_t ldxh;
  char* Bd;
  int64_t ldbd;
  cudaStream_t in = nullptr, out = nullptr;
  std::vector<BlockB> blocks;
  std::vector<cudaEvent_t> ev;
  ~HostRun() {
    for (cudaEvent_t e : ev) cudaEventDestroy(e);  // released once their work completes
  }
};

// Everything enqueued on `from` so far completes before `to` goes on.
int order(HostRun& h, cudaStream_t from, cudaStream_t to) {
  cudaEvent_t e = nullptr;
  cudaError_t r = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  if (r != cudaSuccess) return cuda_status(r, "host copy events");
  h.ev.push_back(e);
  r = cudaEventRecord(e, from);
  if (r == cudaSuccess) r = cudaStreamWaitEvent(to, e, 0);
  return r == cudaSuccess ? NLA_OK : cuda_status(r, "host copy ordering");
}

Mat a_view(const HostRun& h, int64_t i, int64_t j) {
  Mat A{h.Ad, h.ldad, h.at};
  A.c = h.conj;
  return sub(A, i, j, h.c.dtype);
}

Mat b_view(const HostRun& h, int64_t k) {
  const Mat B{h.Bd, h.ldbd, 0};
  return h.c.side == 'L' ? sub(B, k, 0, h.c.dtype) : sub(B, 0, k, h.c.dtype);
}

// Block (i, j), r x q, of A as the recursion indexes it: its stored block is
// copied to the device, and the compute stream waits for it.
int copy_a(HostRun& h, int64_t i, int64_t j, int64_t r, int64_t q) {
  if (r <= 0 || q <= 0) return NLA_OK;
  const int64_t si = h.at ? j : i, sj = h.at ? i : j, sr = h.at ? q : r, sq = h.at ? r : q;
  const size_t es = h.es;
  TraceScope trace(NLA_K_COPY_IN, h.in, 0.0, (double)sr * (double)sq * (double)es);
  cudaError_t e = cudaMemcpy2DAsync(h.Ad + (size_t)(si + sj * h.ldad) * es, (size_t)h.ldad * es,
                                    h.Ah + (size_t)(si + sj * h.ldah) * es, (size_t)h.ldah * es, (size_t)sr * es,
                                    (size_t)sq, cudaMemcpyHostToDevice, h.in);
  if (e != cudaSuccess) return cuda_status(e, "copy of A to the device");
  return order(h, h.in, h.c.s);
}

// The rows (side 'L') or columns ('R') of one block of B: a strided copy.
cudaError_t copy_b(const HostRun& h, const BlockB& b, bool to_device) {
  const size_t es = h.es;
  const bool L = h.c.side == 'L';
  const size_t width = (size_t)(L ? b.len : h.c.m) * es, height = (size_t)(L ? h.c.m : b.len);
  char* d = h.Bd + (size_t)(L ? b.k : b.k * h.ldbd) * es;
  TraceScope trace(to_device ? NLA_K_COPY_IN : NLA_K_COPY_OUT, to_device ? h.in : h.out, 0.0,
                   (double)width * (double)height);
  if (to_device)
    return cudaMemcpy2DAsync(d, (size_t)h.ldbd * es, h.Bh + (size_t)(L ? b.k : b.k * h.ldbh) * es,
                             (size_t)h.ldbh * es, width, height, cudaMemcpyHostToDevice, h.in);
  return cudaMemcpy2DAsync(h.Xh + (size_t)(L ? b.k : b.k * h.ldxh) * es, (size_t)h.ldxh * es, d, (size_t)h.ldbd * es,
                           width, height, cudaMemcpyDeviceToHost, h.out);
}

int scale_block(const HostRun& h, const BlockB& b) {
  const bool L = h.c.side == 'L';
  return launch_scale(h.c.dtype, L ? b.len : h.c.m, L ? h.c.m : b.len, h.alpha, b_view(h, b.k), h.c.s);
}

// The blocks of B in [k, k + len) not yet on the device are copied in; the
// compute stream waits for each and, for a solve, scales it by alpha
// (src/rectrxm.jl:64).
int acquire_b(HostRun& h, int64_t k, int64_t len) {
  for (BlockB& b : h.blocks) {
    if (b.k < k || b.k >= k + len || b.in) continue;
    cudaError_t e = copy_b(h, b, true);
    if (e != cudaSuccess) return cuda_status(e, "copy of B to the device");
    NLA_TRY(order(h, h.in, h.c.s));
    if (h.scale && h.c.func == 'S') NLA_TRY(scale_block(h, b));
    b.in = true;
  }
  return NLA_OK;
}

// The blocks of B in [k, k + len) are final: for a multiply they are scaled
// by alpha (src/rectrxm.jl:72), then copied out once the compute stream has
// written them.
int release_b(HostRun& h, int64_t k, int64_t len) {
  bool any = false;
  for (BlockB& b : h.blocks) {
    if (b.k < k || b.k >= k + len || b.out) continue;
    if (h.scale && h.c.func == 'M') NLA_TRY(scale_block(h, b));
    any = true;
  }
  if (!any) return NLA_OK;
  NLA_TRY(order(h, h.c.s, h.out));
  for (BlockB& b : h.blocks) {
    if (b.k < k || b.k >= k + len || b.out) continue;
    cudaError_t e = copy_b(h, b, false);
    if (e != cudaSuccess) return cuda_status(e, "copy of the result to the host");
    b.out = true;
  }
  return NLA_OK;
}

// Where the staged walk stops: after `levels` levels, at a leaf, or at a node
// whose two leaves and update run as one launch (the device-resident solve
// runs that node the same way, and its results match bit for bit).
bool walk_stops(const RecPlan& c, int64_t n, int levels) {
  return levels == 0 || n <= c.threshold || leaf_pair_wanted(c, n);
}

// The blocks of B: the diagonal blocks where the staged walk stops.
void plan_blocks(const RecPlan& c, int64_t k, int64_t n, int levels, std::vector<BlockB>* out) {
  if (walk_stops(c, n, levels)) {
    out->push_back(BlockB{k, n, false, false});
    return;
  }
  const int64_t mid = split_point(n);
  plan_blocks(c, k, mid, levels - 1, out);
  plan_blocks(c, k + mid, n - mid, levels - 1, out);
}

// The recursion over the diagonal block [k, k + n) with its copies.  With
// `emit`, the blocks of B it finishes are copied out.  A solve finishes each
// block at the end of its own recursion.  A multiply finishes the half it
// processes first only with the update after it, so that half is copied out
// after the update.
int staged(HostRun& h, int64_t k, int64_t n, int levels, bool emit) {
  const RecPlan& c = h.c;
  if (walk_stops(c, n, levels)) {
    NLA_TRY(copy_a(h, k, k, n, n));
    NLA_TRY(acquire_b(h, k, n));
    // The block's leaves through their inverses: all of them inverted in one
    // launch once the block is on the device.
    if (c.inv) NLA_TRY(leaf_inverses_upfront(c, a_view(h, k, k), n, const_cast<LeafInverses*>(c.inv)));
    NLA_TRY(recurse(c, a_view(h, k, k), n, b_view(h, k)));
    return emit ? release_b(h, k, n) : NLA_OK;
  }
  const int64_t mid = split_point(n), rem = n - mid;
  const bool fwd = rec_forward(c), mult = c.func == 'M';
  const int64_t k1 = fwd ? k : k + mid, n1 = fwd ? mid : rem;  // the half processed first
  const int64_t k2 = fwd ? k + mid : k, n2 = fwd ? rem : mid;  // and second
  NLA_TRY(staged(h, k1, n1, levels - 1, emit && !mult));
  if (rec_update_reads_a21(c)) NLA_TRY(copy_a(h, k + mid, k, rem, mid));
  else NLA_TRY(copy_a(h, k, k + mid, mid, rem));
  NLA_TRY(acquire_b(h, k2, n2));
  NLA_TRY(rec_update(c, a_view(h, k, k), n, b_view(h, k)));
  if (emit && mult) NLA_TRY(release_b(h, k1, n1));
  return staged(h, k2, n2, levels - 1, emit);
}

int host_levels(int requested) {
  int v = requested;
  if (v <= 0) {
    const char* e = std::getenv("NLA_HOST_LEVELS");
    v = (e && *e) ? std::atoi(e) : HOST_LEVELS_DEFAULT;
  }
  if (v < 0) v = 0;
  return v > HOST_LEVELS_MAX ? HOST_LEVELS_MAX : v;
}

// Negative sizes are left to the plan's checks.
int check_host_args(int64_t n, int64_t m, char side, const void* X, int64_t ldx, const void* Ad, int64_t lda_dev,
                    const void* Bd, int64_t ldb_dev) {
  const int64_t rows = side == 'L' ? n : m, cols = side == 'L' ? m : n;
  NLA_TRY(check_matrix("X_host", X, rows, cols, ldx));
  NLA_TRY(check_matrix("A_dev", Ad, n, n, lda_dev));
  return check_matrix("B_dev", Bd, rows, cols, ldb_dev);
}

// Common driver.  `whole` copies all of A and B in, runs `device_call` on
// the device arrays and copies the result out (for the refinement sweeps,
// which need the whole first solution); otherwise the staged walk.
template <typename F>
int host_run(HostRun& h, int64_t n, int levels, bool whole, F&& device_call) {
  std::lock_guard<std::mutex> lk(g_host_mu);
  CopyStreams cs;
  NLA_TRY(copy_streams(&cs));
  h.in = cs.in;
  h.out = cs.out;
  cudaStream_t s = h.c.s;
  NLA_TRY(order(h, s, h.in));  // the device arrays are free once earlier work on s is done
  NLA_TRY(order(h, s, h.out));
  if (whole) {
    h.scale = false;
    h.blocks.push_back(BlockB{0, n, false, false});
    NLA_TRY(copy_a(h, 0, 0, n, n));
    NLA_TRY(acquire_b(h, 0, n));
    NLA_TRY(device_call());
  } else {
    plan_blocks(h.c, 0, n, levels, &h.blocks);
    NLA_TRY(staged(h, 0, n, levels, true));
  }
  NLA_TRY(release_b(h, 0, n));  // whatever the walk has not copied out yet
  return order(h, h.out, s);
}

}  // namespace
}  // namespace nla

using namespace nla;

extern "C" {

int nla_host_alloc(size_t bytes, void** out) {
  clear_error();
  if (!out) return fail(NLA_ERR_ARG, "nla_host_alloc: null output pointer");
  *out = nullptr;
  if (bytes == 0) return NLA_OK;
  const cudaError_t e = cudaHostAlloc(out, bytes, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    *out = nullptr;
    return e == cudaErrorMemoryAllocation ? fail(NLA_ERR_NOMEM, "nla_host_alloc: out of page-locked memory")
                                          : cuda_status(e, "cudaHostAlloc");
  }
  return NLA_OK;
}

int nla_host_free(void* p) {
  clear_error();
  if (!p) return NLA_OK;
  const cudaError_t e = cudaFreeHost(p);
  return e == cudaSuccess ? NLA_OK : cuda_status(e, "cudaFreeHost");
}

int nla_trxm_host(char side, char uplo, char trans, double alpha, char func, int dtype, int64_t n, int64_t m,
                  const void* A_host, int64_t lda, const void* B_host, int64_t ldb, void* X_host, int64_t ldx,
                  void* A_dev, int64_t lda_dev, void* B_dev, int64_t ldb_dev, int levels, void* stream) {
  clear_error();
  HostRun h{};
  int at = 0;
  NLA_TRY(check_flags(side, uplo, trans, func, dtype));
  NLA_TRY(check_host_args(n, m, side, X_host, ldx, A_dev, lda_dev, B_dev, ldb_dev));
  NLA_TRY(trxm_plan(side, uplo, trans, func, dtype, n, m, A_host, lda, B_host, ldb, 0, 0, (cudaStream_t)stream,
                    false, &h.c, &at));
  if (n == 0 || m == 0) return NLA_OK;
  h.alpha = alpha;
  h.scale = true;
  h.es = dtype_size(dtype);
  h.Ah = static_cast<const char*>(A_host);
  h.ldah = lda;
  h.Ad = static_cast<char*>(A_dev);
  h.ldad = lda_dev;
  h.at = at;
  h.conj = trans == 'C' && is_complex(dtype);
  h.Bh = static_cast<const char*>(B_host);
  h.ldbh = ldb;
  h.Xh = static_cast<char*>(X_host);
  h.ldxh = ldx;
  h.Bd = static_cast<char*>(B_dev);
  h.ldbd = ldb_dev;
  return host_run(h, n, host_levels(levels), false, [] { return NLA_OK; });
}

int nla_trxm_mixed_host(char side, char uplo, char trans, double alpha, char func, int64_t n, int64_t m,
                        const double* A_host, int64_t lda, const double* B_host, int64_t ldb, double* X_host,
                        int64_t ldx, double* A_dev, int64_t lda_dev, double* B_dev, int64_t ldb_dev,
                        const nla_mixed_opts* opts, int levels, void* stream) {
  clear_error();
  HostRun h{};
  int at = 0;
  nla_mixed_opts o{};
  cudaStream_t s = (cudaStream_t)stream;
  NLA_TRY(check_flags(side, uplo, trans, func, NLA_F64));
  NLA_TRY(check_host_args(n, m, side, X_host, ldx, A_dev, lda_dev, B_dev, ldb_dev));
  NLA_TRY(mixed_plan(side, uplo, trans, func, n, m, A_host, lda, B_host, ldb, opts, s, &h.c, &at, &o));
  if (n == 0 || m == 0) return NLA_OK;
  h.alpha = alpha;
  h.scale = true;
  h.es = sizeof(double);
  h.Ah = reinterpret_cast<const char*>(A_host);
  h.ldah = lda;
  h.Ad = reinterpret_cast<char*>(A_dev);
  h.ldad = lda_dev;
  h.at = at;
  h.Bh = reinterpret_cast<const char*>(B_host);
  h.ldbh = ldb;
  h.Xh = reinterpret_cast<char*>(X_host);
  h.ldxh = ldx;
  h.Bd = reinterpret_cast<char*>(B_dev);
  h.ldbd = ldb_dev;
  const bool whole = func == 'S' && o.sweeps > 0;
  // The staged walk brings A in block by block, so the leaves of each block
  // are inverted when the block arrives (the whole-array form inverts them
  // all inside trxm_mixed_impl).
  LeafInverses blockinv;
  if (!whole && leaf_inverses_wanted(h.c)) h.c.inv = &blockinv;
  return host_run(h, n, host_levels(levels), whole, [&] {
    return trxm_mixed_impl(side, uplo, trans, alpha, func, n, m, A_dev, lda_dev, B_dev, ldb_dev, &o, s);
  });
}

}  // extern "C"
