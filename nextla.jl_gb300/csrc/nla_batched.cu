// Batched solve of many independent, unevenly sized triangular systems
// op(A_i) X_i = alpha B_i (side L) in one persistent launch.
//
// The reference solves one system per unified_rectrxm! call
// (src/rectrxm.jl:43-76); a batch of thousands of small systems then costs
// thousands of recursions and launches.  Here a plan turns the batch into
// work items, one per (system, block of right-hand sides), sorted by cost
// (largest first); a persistent kernel of one warp-group CTA per SM slot
// pulls items from a device counter and solves each with the diagonal-block
// solver of nla_leaf.cuh (systems are at most 1024, the base case's limit).
// Items are independent, so no CTA ever waits on another.  The number of
// right-hand sides per item is chosen per size bucket (tuned by the host
// side and passed in).  The counter reset and the kernel are captured once
// into a CUDA graph and replayed.
#include <algorithm>
#include <mutex>
#include <vector>

#include "nla_leaf.cuh"

struct nla_batch_plan_s {
  int dtype;
  int tA, rev;
  int64_t count;
  int nitems;
  int n_max;
  int cw_max;
  size_t smem;
  int grid;
  void* d_descs;
  void* d_items;
  int* d_counter;
  std::vector<nla_batch_desc> h_descs;
  // Graph cache (valid for one alpha / pool pair).
  cudaStream_t cap_stream;
  cudaGraphExec_t exec;
  double g_alpha;
  const void* g_A;
  void* g_B;
  double flops;
  // Mixed-precision form (Float64 plans): pool extents in elements and the
  // plan-owned Float32 pools and Float64 residual buffer (allocated on first
  // use).
  int64_t a_elems, b_elems;
  float* a32;
  float* x32;
  double* r64;
};

namespace nla {
namespace {

using namespace leafdev;

struct BatchItem {
  int sys;
  int c0;
  int cw;
  int pad;
};

struct BatchArgs {
  const nla_batch_desc* descs;
  const BatchItem* items;
  int nitems;
  int* counter;
  const void* A;
  void* B;
  int tA, rev;
  double alpha;
};

template <typename T>
__global__ void __launch_bounds__(LEAF_THREADS) batched_solve_kernel(BatchArgs a) {
  using Tc = typename Elem<T>::compute;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(a.counter, 1);
    __syncthreads();
    const int it = s_item;
    __syncthreads();
    if (it >= a.nitems) break;
    const BatchItem w = a.items[it];
    const nla_batch_desc d = a.descs[w.sys];
    LeafArgs g;
    g.A = static_cast<const T*>(a.A) + d.a_off;
    g.lda = d.lda;
    g.tA = a.tA;
    g.B = static_cast<T*>(a.B) + d.b_off;
    g.ldb = d.ldb;
    g.tB = 0;
    g.rev = a.rev;
    g.unit = 0;
    g.n = (int)d.n;
    g.m = d.m;
    const int ncols = (int)(d.m - w.c0 < w.cw ? d.m - w.c0 : w.cw);
    const Tc al = (Tc)a.alpha;
    if (w.cw == 8) solve_block<T, 8>(g, w.c0, ncols, smem_raw, al);
    else if (w.cw == 16) solve_block<T, 16>(g, w.c0, ncols, smem_raw, al);
    else solve_block<T, 32>(g, w.c0, ncols, smem_raw, al);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Mixed-precision batch (Float32 solves, Float64 residuals).  Every kernel
// below works on the plan's items, one CTA per item, so only the systems'
// own elements of the caller's pools are read or written.
// ---------------------------------------------------------------------------
enum MapOp { MAP_INIT = 0, MAP_SET = 1, MAP_ADD = 2 };

struct MapArgs {
  const nla_batch_desc* descs;
  const BatchItem* items;
  const double* A64;
  float* A32;
  double* B64;
  double* R64;
  float* X32;
  double alpha;
  int op;
};

// MAP_INIT: R = alpha B (Float64), X32 = (float) R, and (first item of each
// system) A32 = (float) A over the n x n block; MAP_SET: B = (double) X32;
// MAP_ADD: B += (double) X32.  Elements are the item's n x ncols block.
__global__ void __launch_bounds__(256) batched_map_kernel(MapArgs a) {
  const BatchItem w = a.items[blockIdx.x];
  const nla_batch_desc d = a.descs[w.sys];
  const int n = (int)d.n;
  const int ncols = (int)(d.m - w.c0 < w.cw ? d.m - w.c0 : w.cw);
  const int total = n * ncols;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int64_t o = d.b_off + (int64_t)(idx % n) + (int64_t)(w.c0 + idx / n) * d.ldb;
    if (a.op == MAP_INIT) {
      const double r = a.alpha * a.B64[o];
      a.R64[o] = r;
      a.X32[o] = (float)r;
    } else if (a.op == MAP_SET) {
      a.B64[o] = (double)a.X32[o];
    } else {
      a.B64[o] += (double)a.X32[o];
    }
  }
  if (a.op == MAP_INIT && w.c0 == 0) {
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
      const int64_t o = d.a_off + (int64_t)(idx % n) + (int64_t)(idx / n) * d.lda;
      a.A32[o] = (float)a.A64[o];
    }
  }
}

struct ResidualArgs {
  const nla_batch_desc* descs;
  const BatchItem* items;
  const double* A64;
  const double* X64;  // current solution (the caller's B pool)
  const double* R64;  // alpha B
  float* D32;         // out: the residual, rounded to Float32
  int tA, rev;
};

// D32 = (float)(R - L X) on one 128-row band of an item's n x ncols block,
// L the canonical lower triangle (diagonal included) of op(A).  A band is
// its own CTA (blockIdx.y), and the X rows it needs are streamed through
// shared memory 32 at a time, so a CTA holds about 45 KB and several run per
// SM (the update is bound by the 2-FMA-per-clock DFMA rate, and one CTA per
// SM leaves it waiting on shared memory).  Each panel is formed with the
// register-tiled product of the diagonal-block kernels, summing in Float64.
constexpr int RES_PANEL_ELEMS = PANEL * 32 + LEAF_THREADS * SLAB_PAD;  // X panel (CW <= 32) + slab

template <int CW>
__device__ __forceinline__ void residual_band(const ResidualArgs& a, const BatchItem& w, const nla_batch_desc& d,
                                              int r0, double* smem) {
  LeafArgs g;
  g.A = a.A64 + d.a_off;
  g.lda = d.lda;
  g.tA = a.tA;
  g.B = const_cast<double*>(a.X64) + d.b_off;
  g.ldb = d.ldb;
  g.tB = 0;
  g.rev = a.rev;
  g.unit = 0;
  g.n = (int)d.n;
  g.m = d.m;
  const int ncols = (int)(d.m - w.c0 < CW ? d.m - w.c0 : CW);
  const int rows = min(LEAF_THREADS, g.n - r0);
  const int kmax = r0 + rows;  // k <= r
  double* Xs = smem;                 // PANEL x CW
  double* slab = smem + PANEL * 32;  // 128 x 33
  constexpr int CT = CW / 4;
  const int tr = threadIdx.x & 31, tc = threadIdx.x >> 5;
  double acc[4][CT];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int c = 0; c < CT; ++c) acc[i][c] = 0.0;
  const double* X = a.X64 + d.b_off;
  for (int k0 = 0; k0 < kmax; k0 += PANEL) {
    const int kw = min(PANEL, kmax - k0);
    // X rows k0 .. k0 + kw of the item's columns (threads along the rows,
    // which are contiguous in memory).
    for (int idx = threadIdx.x; idx < PANEL * CW; idx += LEAF_THREADS) {
      const int k = idx % PANEL, c = idx / PANEL;
      Xs[k * CW + c] = k < kw && c < ncols ? X[b_off<double>(g, k0 + k, w.c0 + c)] : 0.0;
    }
    stage_slab<LEAF_THREADS, double>(g, slab, r0, rows, k0, kw, [](int i, int j) { return j <= i; });
    __syncthreads();
    tile_product<double, CW>(slab, Xs, kw, rows, acc);
    __syncthreads();
  }
  const double* R = a.R64 + d.b_off;
  float* D = a.D32 + d.b_off;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = tr + 32 * i;
    if (r < rows) {
#pragma unroll
      for (int c = 0; c < CT; ++c) {
        const int col = tc * CT + c;
        if (col < ncols) {
          const int64_t o = b_off<double>(g, r0 + r, w.c0 + col);
          D[o] = (float)(R[o] - acc[i][c]);
        }
      }
    }
  }
}

__global__ void __launch_bounds__(LEAF_THREADS) batched_residual_kernel(ResidualArgs a) {
  __shared__ __align__(16) double smem[RES_PANEL_ELEMS];
  const BatchItem w = a.items[blockIdx.x];
  const nla_batch_desc d = a.descs[w.sys];
  const int r0 = (int)blockIdx.y * LEAF_THREADS;
  if (r0 >= d.n) return;
  if (w.cw == 8) residual_band<8>(a, w, d, r0, smem);
  else if (w.cw == 16) residual_band<16>(a, w, d, r0, smem);
  else residual_band<32>(a, w, d, r0, smem);
}

int bucket_of(int64_t n) {
  int b = 0;
  int64_t hi = 32;
  while (b < NLA_BATCH_BUCKETS - 1 && n >= hi) {
    ++b;
    hi *= 2;
  }
  return b;
}

template <typename T>
int launch_batched(nla_batch_plan p, double alpha, const void* A, void* B, cudaStream_t s) {
  BatchArgs a{static_cast<const nla_batch_desc*>(p->d_descs), static_cast<const BatchItem*>(p->d_items), p->nitems,
              p->d_counter, A, B, p->tA, p->rev, alpha};
  batched_solve_kernel<T><<<p->grid, LEAF_THREADS, p->smem, s>>>(a);
  NLA_CHECK_LAUNCH("batched_solve_kernel");
  return NLA_OK;
}

template <typename T>
int batched_smem_attr(size_t smem) {
  static std::once_flag once;
  static cudaError_t st = cudaSuccess;
  std::call_once(once, [] {
    st = cudaFuncSetAttribute(batched_solve_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  });
  if (smem > 200 * 1024) return fail(NLA_ERR_UNSUPPORTED, "batch: shared memory plan too large");
  return st == cudaSuccess ? NLA_OK : cuda_status(st, "cudaFuncSetAttribute(batched_solve_kernel)");
}

template <typename T>
int occupancy(size_t smem, int* blocks) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, batched_solve_kernel<T>, LEAF_THREADS, smem) ==
                 cudaSuccess
             ? NLA_OK
             : fail(NLA_ERR_UNSUPPORTED, "batch: occupancy query failed");
}

int enqueue(nla_batch_plan p, double alpha, const void* A, void* B, cudaStream_t s) {
  cudaMemsetAsync(p->d_counter, 0, sizeof(int), s);
  switch (p->dtype) {
    case NLA_F64: return launch_batched<double>(p, alpha, A, B, s);
    case NLA_F32: return launch_batched<float>(p, alpha, A, B, s);
    default: return launch_batched<__half>(p, alpha, A, B, s);
  }
}

}  // namespace



}  // namespace nla

using namespace nla;

extern "C" {

int nla_batch_plan_create(nla_batch_plan* out, int dtype, char uplo, char trans, int64_t count,
                          const nla_batch_desc* descs, const int* cols_per_item) {
  clear_error();
  if (!out) return fail(NLA_ERR_ARG, "plan pointer is null");
  *out = nullptr;
  NLA_TRY(check_flags('L', uplo, trans, 'S', dtype));
  if (count < 0 || (count > 0 && !descs)) return fail(NLA_ERR_ARG, "bad system count or descriptor array");
  if (count > (int64_t)1 << 30) return fail(NLA_ERR_UNSUPPORTED, "too many systems");
  int cw[NLA_BATCH_BUCKETS] = {8, 16, 16, 16, 16, 16};
  if (dtype != NLA_F64)
    for (int b = 0; b < NLA_BATCH_BUCKETS; ++b) cw[b] = b == 0 ? 16 : 32;
  if (cols_per_item)
    for (int b = 0; b < NLA_BATCH_BUCKETS; ++b) {
      if (cols_per_item[b] != 8 && cols_per_item[b] != 16 && cols_per_item[b] != 32)
        return fail(NLA_ERR_ARG, "cols_per_item entries must be 8, 16 or 32");
      cw[b] = cols_per_item[b];
    }
  nla_batch_plan p = new nla_batch_plan_s();
  p->dtype = dtype;
  p->tA = (trans == 'T' || trans == 'C') ? 1 : 0;
  const char up = p->tA ? (uplo == 'L' ? 'U' : 'L') : uplo;
  p->rev = up == 'U';
  p->count = count;
  p->h_descs.assign(descs, descs + count);
  std::vector<BatchItem> items;
  int bucket_n_max[NLA_BATCH_BUCKETS] = {0, 0, 0, 0, 0, 0};
  p->n_max = 1;
  p->cw_max = 8;
  p->flops = 0;
  p->a_elems = 0;
  p->b_elems = 0;
  p->a32 = nullptr;
  p->x32 = nullptr;
  p->r64 = nullptr;
  for (int64_t i = 0; i < count; ++i) {
    const nla_batch_desc& d = descs[i];
    if (d.n < 0 || d.m < 0 || d.n > 1024 || d.lda < (d.n > 1 ? d.n : 1) || d.ldb < (d.n > 1 ? d.n : 1) ||
        d.a_off < 0 || d.b_off < 0) {
      delete p;
      return fail(NLA_ERR_ARG, "system " + std::to_string(i) + ": bad size, leading dimension or offset");
    }
    if (d.n == 0 || d.m == 0) continue;
    p->a_elems = std::max<int64_t>(p->a_elems, d.a_off + (d.n - 1) * d.lda + d.n);
    p->b_elems = std::max<int64_t>(p->b_elems, d.b_off + (d.m - 1) * d.ldb + d.n);
    const int bk = bucket_of(d.n);
    const int c = cw[bk];
    bucket_n_max[bk] = std::max<int>(bucket_n_max[bk], (int)d.n);
    p->n_max = std::max<int>(p->n_max, (int)d.n);
    p->cw_max = std::max(p->cw_max, c);
    p->flops += (double)d.n * d.n * d.m;
    for (int64_t c0 = 0; c0 < d.m; c0 += c) items.push_back(BatchItem{(int)i, (int)c0, c, 0});
  }
  // Largest items first: the tail of the schedule is made of small items.
  std::stable_sort(items.begin(), items.end(), [&](const BatchItem& x, const BatchItem& y) {
    const double cx = (double)descs[x.sys].n * descs[x.sys].n * std::min<int64_t>(x.cw, descs[x.sys].m - x.c0);
    const double cy = (double)descs[y.sys].n * descs[y.sys].n * std::min<int64_t>(y.cw, descs[y.sys].m - y.c0);
    return cx > cy;
  });
  p->nitems = (int)items.size();
  const size_t esz = dtype == NLA_F64 ? 8 : 4;
  // Shared memory for the largest block any item stages: n_max of a bucket
  // times that bucket's width (narrow items for the large systems keep the
  // plan at two or more CTAs per SM).
  p->smem = 0;
  for (int b = 0; b < NLA_BATCH_BUCKETS; ++b)
    if (bucket_n_max[b] > 0)
      p->smem = std::max(p->smem, leaf_solve_smem_elems(bucket_n_max[b], cw[b]) * esz);
  int rc = NLA_OK;
  int per_sm = 0;
  if (dtype == NLA_F64) rc = batched_smem_attr<double>(p->smem);
  else if (dtype == NLA_F32) rc = batched_smem_attr<float>(p->smem);
  else rc = batched_smem_attr<__half>(p->smem);
  if (rc == NLA_OK) {
    if (dtype == NLA_F64) rc = occupancy<double>(p->smem, &per_sm);
    else if (dtype == NLA_F32) rc = occupancy<float>(p->smem, &per_sm);
    else rc = occupancy<__half>(p->smem, &per_sm);
  }
  if (rc != NLA_OK) {
    delete p;
    return rc;
  }
  p->grid = std::max(1, std::min(p->nitems, num_sms() * std::max(per_sm, 1)));
  cudaError_t e = cudaMalloc(&p->d_descs, sizeof(nla_batch_desc) * (size_t)std::max<int64_t>(count, 1));
  if (e == cudaSuccess) e = cudaMalloc(&p->d_items, sizeof(BatchItem) * (size_t)std::max(p->nitems, 1));
  if (e == cudaSuccess) e = cudaMalloc(&p->d_counter, sizeof(int));
  if (e == cudaSuccess && count > 0)
    e = cudaMemcpy(p->d_descs, descs, sizeof(nla_batch_desc) * (size_t)count, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && p->nitems > 0)
    e = cudaMemcpy(p->d_items, items.data(), sizeof(BatchItem) * items.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    cudaFree(p->d_descs);
    cudaFree(p->d_items);
    cudaFree(p->d_counter);
    delete p;
    return cuda_status(e, "batch plan allocation");
  }
  p->exec = nullptr;
  *out = p;
  return NLA_OK;
}

int nla_batch_plan_info(nla_batch_plan p, int64_t* items, int64_t* grid, double* flops) {
  clear_error();
  if (!p) return fail(NLA_ERR_ARG, "null plan");
  if (items) *items = p->nitems;
  if (grid) *grid = p->grid;
  if (flops) *flops = p->flops;
  return NLA_OK;
}

int nla_batch_solve(nla_batch_plan p, double alpha, const void* A_pool, void* B_pool, int mode, void* stream) {
  clear_error();
  if (!p) return fail(NLA_ERR_ARG, "null plan");
  if (p->nitems == 0) return NLA_OK;
  if (!A_pool || !B_pool) return fail(NLA_ERR_ARG, "null pool pointer");
  cudaStream_t s = (cudaStream_t)stream;
  if (mode == NLA_BATCH_LOOP) {
    // One recursion (and its launches) per system, as one unified_rectrxm!
    // call per system would do: the baseline the persistent launch replaces.
    const char uplo = p->rev ^ p->tA ? 'U' : 'L';
    const char trans = p->tA ? 'T' : 'N';
    const size_t esz = dtype_size(p->dtype);
    for (const nla_batch_desc& d : p->h_descs) {
      if (d.n == 0 || d.m == 0) continue;
      NLA_TRY(trxm_impl('L', uplo, trans, alpha, 'S', p->dtype, d.n, d.m,
                        static_cast<const char*>(A_pool) + d.a_off * esz, d.lda,
                        static_cast<char*>(B_pool) + d.b_off * esz, d.ldb, 0, 0, s));
    }
    return NLA_OK;
  }
  TraceScope trace(NLA_K_BATCHED, s, p->flops, 0.0);
  if (mode == NLA_BATCH_PERSISTENT) return enqueue(p, alpha, A_pool, B_pool, s);
  if (mode != NLA_BATCH_GRAPH) return fail(NLA_ERR_ARG, "unknown batch mode");
  if (!p->exec || p->g_alpha != alpha || p->g_A != A_pool || p->g_B != B_pool) {
    if (p->exec) {
      cudaGraphExecDestroy(p->exec);
      p->exec = nullptr;
    }
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(p->cap_stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_status(e, "batch graph capture");
    int rc = enqueue(p, alpha, A_pool, B_pool, p->cap_stream);
    e = cudaStreamEndCapture(p->cap_stream, &graph);
    if (rc != NLA_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) return cuda_status(e, "batch graph capture");
    e = cudaGraphInstantiate(&p->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      p->exec = nullptr;
      return cuda_status(e, "batch graph instantiate");
    }
    p->g_alpha = alpha;
    p->g_A = A_pool;
    p->g_B = B_pool;
  }
  cudaError_t e = cudaGraphLaunch(p->exec, s);
  return e == cudaSuccess ? NLA_OK : cuda_status(e, "batch graph launch");
}

int nla_batch_solve_mixed(nla_batch_plan p, double alpha, const void* A_pool, void* B_pool, int sweeps,
                          void* stream) {
  clear_error();
  if (!p) return fail(NLA_ERR_ARG, "null plan");
  if (p->dtype != NLA_F64) return fail(NLA_ERR_DTYPE, "mixed batch: the plan must be Float64");
  if (sweeps < 0 || sweeps > 8) return fail(NLA_ERR_ARG, "mixed batch: sweeps must be 0..8");
  if (p->nitems == 0) return NLA_OK;
  if (!A_pool || !B_pool) return fail(NLA_ERR_ARG, "null pool pointer");
  cudaStream_t s = (cudaStream_t)stream;
  if (!p->a32) {
    cudaError_t e = cudaMalloc(&p->a32, sizeof(float) * (size_t)p->a_elems);
    if (e == cudaSuccess) e = cudaMalloc(&p->x32, sizeof(float) * (size_t)p->b_elems);
    if (e == cudaSuccess) e = cudaMalloc(&p->r64, sizeof(double) * (size_t)p->b_elems);
    if (e != cudaSuccess) {
      cudaFree(p->a32);
      cudaFree(p->x32);
      cudaFree(p->r64);
      p->a32 = nullptr;
      p->x32 = nullptr;
      p->r64 = nullptr;
      return cuda_status(e, "mixed batch buffers");
    }
  }
  NLA_TRY(batched_smem_attr<float>(p->smem));
  const auto* descs = static_cast<const nla_batch_desc*>(p->d_descs);
  const auto* items = static_cast<const BatchItem*>(p->d_items);
  double* B64 = static_cast<double*>(B_pool);
  const double* A64 = static_cast<const double*>(A_pool);
  TraceScope trace(NLA_K_BATCHED, s, p->flops, 0.0);
  MapArgs m{descs, items, A64, p->a32, B64, p->r64, p->x32, alpha, MAP_INIT};
  batched_map_kernel<<<p->nitems, 256, 0, s>>>(m);
  NLA_CHECK_LAUNCH("batched_map_kernel");
  auto solve32 = [&]() -> int {
    cudaMemsetAsync(p->d_counter, 0, sizeof(int), s);
    return launch_batched<float>(p, 1.0, p->a32, p->x32, s);
  };
  NLA_TRY(solve32());
  m.op = MAP_SET;
  batched_map_kernel<<<p->nitems, 256, 0, s>>>(m);
  NLA_CHECK_LAUNCH("batched_map_kernel");
  const ResidualArgs r{descs, items, A64, B64, p->r64, p->x32, p->tA, p->rev};
  for (int k = 0; k < sweeps; ++k) {
    batched_residual_kernel<<<dim3((unsigned)p->nitems, (unsigned)((p->n_max + LEAF_THREADS - 1) / LEAF_THREADS)),
                              LEAF_THREADS, 0, s>>>(r);
    NLA_CHECK_LAUNCH("batched_residual_kernel");
    NLA_TRY(solve32());
    m.op = MAP_ADD;
    batched_map_kernel<<<p->nitems, 256, 0, s>>>(m);
    NLA_CHECK_LAUNCH("batched_map_kernel");
  }
  return NLA_OK;
}

int nla_batch_plan_destroy(nla_batch_plan p) {
  clear_error();
  if (!p) return NLA_OK;
  cudaFree(p->a32);
  cudaFree(p->x32);
  cudaFree(p->r64);
  if (p->exec) cudaGraphExecDestroy(p->exec);
  cudaStreamDestroy(p->cap_stream);
  cudaFree(p->d_descs);
  cudaFree(p->d_items);
  cudaFree(p->d_counter);
  delete p;
  return NLA_OK;
}

}  // extern "C"
