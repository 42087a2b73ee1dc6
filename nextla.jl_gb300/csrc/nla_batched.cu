// Batched solve of many independent, unevenly sized triangular systems
// op(A_i) X_i = alpha B_i (side L) in one persistent launch, as a device
// queue of recursion nodes.
//
// The reference solves one system per unified_rectrxm! call
// (src/rectrxm.jl:43-76), recursing in unified_rec (src/rectrxm.jl:101-198):
// split at mid (:129-133), solve the half that goes first, update the other
// half with one GEMM (:162-194), solve it.  Here the plan runs that recursion
// on the host for every system (and block of right-hand sides, a "group"),
// down to leaves of at most `cutoff` rows, and records its pieces as nodes:
//   LEAF    solve one diagonal block of a group in place;
//   UPDATE  one GEMM tile of the recursion: the rows of one leaf, minus the
//           product of their A block over the K range of the half solved
//           first with the solution of that half.
// Nodes of one group depend on each other exactly as the recursion orders
// them; nodes of different groups are independent.  The plan orders all
// nodes by a list-scheduling simulation over the persistent CTAs (largest
// critical path first), so the updates of one large system spread over many
// CTAs while small systems fill the gaps, and uploads them once.
//
// One persistent kernel (CTAs = SMs x resident CTAs per SM) pulls nodes in
// that order from a device counter.  Before a node runs, its CTA waits for
// its dependencies on two kinds of counters, bounded by %globaltimer:
//   solved[g]       leaves of group g solved so far (leaves finish in order:
//                   a leaf's last update needs every earlier leaf);
//   applied[leaf]   updates applied to a leaf's rows so far (the updates of
//                   one leaf run in the recursion's order, outermost first,
//                   and the leaf runs after all of them).
// The queue order is a topological order of the dependencies and every CTA
// that holds a node is resident, so the waits always end; a wait that runs
// past the limit records an error word (read by nla_device_status) and the
// kernel stops taking nodes.  The counter reset and the kernel are captured
// into a CUDA graph once and replayed.
//
// Alpha is applied where a row of B is first read: by the outermost update
// of each leaf, or by the leaf itself when no update reaches it (the first
// leaf), as alpha * B rounded to the element type (src/rectrxm.jl:64).
#include <algorithm>
#include <mutex>
#include <queue>
#include <vector>

#include "nla_common.cuh"
#include "nla_split7.cuh"
#include "nla_umma.cuh"

namespace nla {
namespace bat {

constexpr int NT = 256;          // threads per CTA
constexpr int MAX_ROWS = 64;     // largest leaf (and update-tile height)
constexpr int ROW_GROUPS = 16;   // 16 row groups x 16 column groups of threads
constexpr int RT = 4;            // rows per thread (strided by ROW_GROUPS)
#ifndef NLA_BATCH_PANEL
#define NLA_BATCH_PANEL 16
#endif
constexpr int PANEL = NLA_BATCH_PANEL;  // triangle panel of a leaf (rows solved one chain per thread)
constexpr int LEAF_PAD = 1;      // row padding of the staged diagonal block

static_assert(NT % MAX_ROWS == 0 && NT % 32 == 0 && NT % 16 == 0, "staging index steps");

enum { NODE_LEAF = 0, NODE_UPDATE = 1 };
enum { FLAG_ALPHA = 1 };

struct Node {
  int group;
  int r0, rows;      // canonical rows of the target leaf
  int k0, kw;        // UPDATE: canonical K range
  int leaf;          // target leaf (index within the group)
  int wait_solved;   // solved leaves of the group needed first
  short wait_applied;  // updates applied to the target leaf needed first
  unsigned char kind, flags;
};
static_assert(sizeof(Node) == 32, "node layout");

struct Group {
  int sys;
  int c0, ncols;  // block of right-hand sides
  int w;          // column template: 16, 32, 64 or 128
  int leaf_base;  // first applied[] counter of the group
  int n;
};

struct Args {
  const nla_batch_desc* descs;
  const Group* groups;
  const Node* nodes;
  int nnodes;
  int* next;       // queue head
  int* solved;     // per group
  int* applied;    // per leaf
  int* abort;      // set when a wait gave up: the CTAs stop taking nodes (reset per launch)
  int* err;        // sticky error word: site of the first wait that gave up
  const void* A;
  void* B;
  int tA, rev;
  double alpha;
  uint64_t limit_ns;
  float alpha_f;      // alpha as a float, and whether that is exact: the float
  int alpha_f_exact;  // product is then the double product rounded once
};

__device__ int g_batch_error = 0;

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void add_release(int* p, int v) {
  asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Waits until *p >= target; false if the limit passed (the error word and
// the abort flag are then set) or another CTA has already aborted.
__device__ bool wait_geq(const int* p, int target, const Args& a, int where) {
  if (ld_acquire(p) >= target) return true;
  const uint64_t t0 = globaltimer();
  unsigned ns = 32;
  for (;;) {
    __nanosleep(ns);
    if (ns < 1024) ns *= 2;
    if (ld_acquire(p) >= target) return true;
    if (*(volatile int*)a.abort) return false;
    if (globaltimer() - t0 > a.limit_ns) {
      atomicCAS(a.err, 0, where);
      atomicExch(a.abort, 1);
      return false;
    }
  }
}

// Loads of the B pool go through L2 (another CTA may have written the rows
// since this SM last cached them); A is read-only.
template <typename T> __device__ __forceinline__ T ldcg(const T* p) { return __ldcg(p); }
template <> __device__ __forceinline__ __half ldcg<__half>(const __half* p) {
  return __ushort_as_half(__ldcg(reinterpret_cast<const unsigned short*>(p)));
}
__device__ __forceinline__ double to_c(double v) { return v; }
__device__ __forceinline__ float to_c(float v) { return v; }
__device__ __forceinline__ float to_c(__half v) { return __half2float(v); }

// alpha * b formed in Float64 and rounded to the element type, as
// B .= alpha .* B does (src/rectrxm.jl:64).
template <typename T> __device__ __forceinline__ typename Elem<T>::compute scaled(T b, double alpha);
template <> __device__ __forceinline__ double scaled<double>(double b, double alpha) { return alpha * b; }
template <> __device__ __forceinline__ float scaled<float>(float b, double alpha) { return (float)(alpha * (double)b); }
// The same for a node's first touch of B, without FP64 work when alpha is a
// float (24 x 24 bits are exact in a double, so one float rounding gives the
// same value).
template <typename T> __device__ __forceinline__ typename Elem<T>::compute scaled_node(T b, const Args& a) {
  return scaled<T>(b, a.alpha);
}
template <> __device__ __forceinline__ float scaled_node<float>(float b, const Args& a) {
  return a.alpha_f_exact ? b * a.alpha_f : scaled<float>(b, a.alpha);
}
template <> __device__ __forceinline__ float scaled<__half>(__half b, double alpha) {
  return __half2float(__double2half(alpha * (double)__half2float(b)));
}

// N consecutive compute-type values from shared memory, read as the widest
// vectors N allows (callers keep p aligned to that width).
template <int N>
__device__ __forceinline__ void lds_vec(const float* p, float (&v)[N]) {
  if constexpr (N % 4 == 0) {
#pragma unroll
    for (int j = 0; j < N; j += 4) {
      const float4 q = *reinterpret_cast<const float4*>(p + j);
      v[j] = q.x;
      v[j + 1] = q.y;
      v[j + 2] = q.z;
      v[j + 3] = q.w;
    }
  } else if constexpr (N % 2 == 0) {
#pragma unroll
    for (int j = 0; j < N; j += 2) {
      const float2 q = *reinterpret_cast<const float2*>(p + j);
      v[j] = q.x;
      v[j + 1] = q.y;
    }
  } else {
#pragma unroll
    for (int j = 0; j < N; ++j) v[j] = p[j];
  }
}
template <int N>
__device__ __forceinline__ void lds_vec(const double* p, double (&v)[N]) {
  if constexpr (N % 2 == 0) {
#pragma unroll
    for (int j = 0; j < N; j += 2) {
      const double2 q = *reinterpret_cast<const double2*>(p + j);
      v[j] = q.x;
      v[j + 1] = q.y;
    }
  } else {
#pragma unroll
    for (int j = 0; j < N; ++j) v[j] = p[j];
  }
}

// RT consecutive values to shared memory as 16-byte vectors (p 16-byte aligned).
__device__ __forceinline__ void sts4(float* p, float a, float b, float c, float d) {
  *reinterpret_cast<float4*>(p) = make_float4(a, b, c, d);
}
__device__ __forceinline__ void sts4(double* p, double a, double b, double c, double d) {
  *reinterpret_cast<double2*>(p) = make_double2(a, b);
  *reinterpret_cast<double2*>(p + 2) = make_double2(c, d);
}

// Element offsets in canonical coordinates: row i / column k of the lower
// triangle applied from the left (rev maps i -> n - 1 - i; tA reads A's
// transpose).
__device__ __forceinline__ int64_t a_at(const nla_batch_desc& d, int tA, int rev, int i, int k) {
  const int64_t r = rev ? d.n - 1 - i : i, c = rev ? d.n - 1 - k : k;
  return d.a_off + (tA ? c + r * d.lda : r + c * d.lda);
}
__device__ __forceinline__ int64_t b_at(const nla_batch_desc& d, int rev, int i, int64_t col) {
  const int64_t r = rev ? d.n - 1 - i : i;
  return d.b_off + r + col * d.ldb;
}

// Shared-memory footprint (compute-type elements) of a node of width W.
__host__ __device__ constexpr int kc_of(int esz) { return esz == 8 ? 16 : 32; }
__host__ __device__ constexpr size_t update_elems(int W, int kc) {
  return (size_t)kc * (MAX_ROWS + 4) + (size_t)kc * (W + 4);
}
__host__ __device__ constexpr size_t leaf_elems(int W) {
  return (size_t)MAX_ROWS * (MAX_ROWS + LEAF_PAD) + (size_t)MAX_ROWS * (W + 4) + MAX_ROWS;
}

// Thread 0 waits for the node's dependencies (acquire loads of the group's
// counters); every thread learns the outcome through *s_ok.  False when a
// wait gave up or another CTA has aborted.  Nodes call it after issuing the
// loads of A, which no other node writes, so that those are in flight
// during the wait.
__device__ __forceinline__ bool node_deps(const Args& a, const Node& nd, volatile int* s_ok) {
  if (threadIdx.x == 0) {
    bool ok = *(volatile int*)a.abort == 0;
    if (ok && nd.kind == NODE_UPDATE && nd.wait_solved > 0) ok = wait_geq(a.solved + nd.group, nd.wait_solved, a, 1);
    if (ok && nd.wait_applied > 0)
      ok = wait_geq(a.applied + a.groups[nd.group].leaf_base + nd.leaf, nd.wait_applied, a, 2);
    *s_ok = ok ? 1 : 0;
  }
  __syncthreads();
  return *s_ok != 0;
}

// ---------------------------------------------------------------------------
// UPDATE: X[r0 + r, c] = base(r, c) - sum_k A[r0 + r, k0 + k] X[k0 + k, c] for
// r < rows, c < ncols, base = alpha B (first touch) or B.  Thread (tr, tc)
// owns rows 4 tr .. 4 tr + 3 and columns tc * CT .. + CT, both read from
// shared memory as vectors (A's 4 values serve 16 lanes of a warp, X's CT
// values are broadcasts).  K is walked in chunks of KC staged in shared
// memory (A k-major, X k-major), the next chunk's elements prefetched into
// registers during the current chunk.
// ---------------------------------------------------------------------------
template <typename T, int W>
__device__ bool run_update(const Args& a, const Node& nd, const Group& g, const nla_batch_desc& d, void* smem,
                           volatile int* s_ok) {
  using Tc = typename Elem<T>::compute;
  constexpr int KC = kc_of(sizeof(Tc));
  constexpr int CT = W / 16;
  constexpr int AP = MAX_ROWS + 4, XP = W + 4;
  constexpr int A_PER = MAX_ROWS * KC / NT, X_PER = KC * W / NT;
  Tc* As = static_cast<Tc*>(smem);  // [KC][AP]
  Tc* Xs = As + KC * AP;             // [KC][XP]
  const T* A = static_cast<const T*>(a.A);
  const T* B = static_cast<const T*>(a.B);
  const int t = threadIdx.x, tr = t % ROW_GROUPS, tc = t / ROW_GROUPS;
  const int rows = nd.rows, ncols = g.ncols;
  const bool warp_cols_live = (tc & ~1) * CT < ncols;  // the warp's first column group

  Tc acc[RT][CT];
#pragma unroll
  for (int i = 0; i < RT; ++i)
#pragma unroll
    for (int c = 0; c < CT; ++c) acc[i][c] = Tc(0);

  // Element (r, k) of a chunk, for this thread's u-th load: A's canonical
  // (r0 + r, k0 + k) and X's (k0 + k, c0 + c) are affine in r, k and c, and
  // (NT being a multiple of 64 and KC) so is u: every load below is a base
  // address plus u times a per-node stride.
  const int64_t sgn = a.rev ? -1 : 1;
  const int64_t dr = sgn * (a.tA ? d.lda : 1), dk = sgn * (a.tA ? 1 : d.lda);
  const int ar = a.tA ? t / KC : t % MAX_ROWS, ak = a.tA ? t % KC : t / MAX_ROWS;
  const int ar_step = a.tA ? NT / KC : 0, ak_step = a.tA ? 0 : NT / MAX_ROWS;
  const int64_t a_step = (int64_t)ar_step * dr + (int64_t)ak_step * dk;
  const int xk = t % KC, xc = t / KC;
  constexpr int XC_STEP = NT / KC;
  const int64_t x_step = (int64_t)XC_STEP * d.ldb;
  const T* A0 = A + a_at(d, a.tA, a.rev, nd.r0, nd.k0) + ar * dr + ak * dk;
  const T* X0 = B + b_at(d, a.rev, nd.k0, g.c0) + sgn * xk + (int64_t)xc * d.ldb;

  Tc pa[A_PER], px[X_PER];
  auto fetch_a = [&](int k0) {
    const int kw = min(KC, nd.k0 + nd.kw - k0);
    const T* pA = A0 + (int64_t)(k0 - nd.k0) * dk;
#pragma unroll
    for (int u = 0; u < A_PER; ++u)
      pa[u] = ar + u * ar_step < rows && ak + u * ak_step < kw ? to_c(pA[u * a_step]) : Tc(0);
  };
  auto fetch_x = [&](int k0) {
    const int kw = min(KC, nd.k0 + nd.kw - k0);
    const T* pX = X0 + (int64_t)(k0 - nd.k0) * sgn;
#pragma unroll
    for (int u = 0; u < X_PER; ++u)
      px[u] = xk < kw && xc + u * XC_STEP < ncols ? to_c(ldcg(pX + u * x_step)) : Tc(0);
  };
  auto stash = [&]() {
#pragma unroll
    for (int u = 0; u < A_PER; ++u) As[(ak + u * ak_step) * AP + ar + u * ar_step] = pa[u];
#pragma unroll
    for (int u = 0; u < X_PER; ++u) Xs[xk * XP + xc + u * XC_STEP] = px[u];
  };

  const int kend = nd.k0 + nd.kw;
  fetch_a(nd.k0);
  if (!node_deps(a, nd, s_ok)) return false;
  fetch_x(nd.k0);
  for (int k0 = nd.k0; k0 < kend; k0 += KC) {
    __syncthreads();  // the previous chunk is no longer read
    stash();
    __syncthreads();
    if (k0 + KC < kend) {
      fetch_a(k0 + KC);
      fetch_x(k0 + KC);
    }
    // A warp holds the columns of two column groups; one whose columns all
    // lie past the group's right-hand sides (a narrow block in a wider
    // template) skips the products.
    const int kw = warp_cols_live ? min(KC, kend - k0) : 0;
#pragma unroll 4
    for (int k = 0; k < kw; ++k) {
      Tc av[RT], xv[CT];
      lds_vec<RT>(As + k * AP + RT * tr, av);
      lds_vec<CT>(Xs + k * XP + tc * CT, xv);
#pragma unroll
      for (int i = 0; i < RT; ++i)
#pragma unroll
        for (int c = 0; c < CT; ++c) acc[i][c] = fma(av[i], xv[c], acc[i][c]);
    }
  }
  // Epilogue: the products go through shared memory (column-major, TP rows)
  // so that the tile of B is read and written along its contiguous rows, all
  // of a thread's loads issued before its first store (a store to the pool
  // may alias a later load of it, which would otherwise wait for it).
  constexpr int TP = MAX_ROWS + 4;
  static_assert(RT == 4 && TP * W <= KC * (AP + XP) + MAX_ROWS * (MAX_ROWS + LEAF_PAD), "tile fits the node's smem");
  // The tile's loads of B are issued first, so that their latency passes
  // while the products go to shared memory.
  constexpr int PER = MAX_ROWS * W / NT, CSTEP = NT / MAX_ROWS;
  const int r = t % MAX_ROWS, cb = t / MAX_ROWS;
  T* const Bt = static_cast<T*>(a.B) + b_at(d, a.rev, nd.r0, g.c0) + sgn * r;
  const bool first = nd.flags & FLAG_ALPHA;
  T bv[PER];
#pragma unroll
  for (int u = 0; u < PER; ++u) {
    const int c = cb + u * CSTEP;
    bv[u] = r < rows && c < ncols ? ldcg(Bt + (int64_t)c * d.ldb) : T(0);
  }
  Tc* Ts = As;
  __syncthreads();  // the last chunk is no longer read
#pragma unroll
  for (int c = 0; c < CT; ++c)
    sts4(Ts + (tc * CT + c) * TP + RT * tr, acc[0][c], acc[1][c], acc[2][c], acc[3][c]);
  __syncthreads();
  // A node-uniform branch: with a select the compiler formed alpha * b (FP64
  // work, slow on this part) for every node.
  if (first) {
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int c = cb + u * CSTEP;
      if (r < rows && c < ncols) Elem<T>::store(Bt + (int64_t)c * d.ldb, scaled_node<T>(bv[u], a) - Ts[c * TP + r]);
    }
  } else {
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int c = cb + u * CSTEP;
      if (r < rows && c < ncols) Elem<T>::store(Bt + (int64_t)c * d.ldb, to_c(bv[u]) - Ts[c * TP + r]);
    }
  }
  return true;
}

// ---------------------------------------------------------------------------
// LEAF: solve the diagonal block rows r0 .. r0 + rows (at most 64) in place.
// The block of A (lower, with the diagonal's reciprocals) and of X are staged
// in shared memory; 16-row panels are solved one right-hand side per thread
// (the panel's values in registers), and each panel's rows below it are then
// updated with the register-tiled product.
// ---------------------------------------------------------------------------
template <typename T, int W>
__device__ bool run_leaf(const Args& a, const Node& nd, const Group& g, const nla_batch_desc& d, void* smem,
                         volatile int* s_ok) {
  using Tc = typename Elem<T>::compute;
  constexpr int LP = MAX_ROWS + LEAF_PAD, XP = W + 4, CT = W / 16;
  Tc* Ls = static_cast<Tc*>(smem);    // [64][LP]: Ls[r][k], k < r, of the block
  Tc* Xs = Ls + MAX_ROWS * LP;        // [64][XP]
  Tc* inv = Xs + MAX_ROWS * XP;       // [64]
  const T* A = static_cast<const T*>(a.A);
  T* B = static_cast<T*>(a.B);
  const int t = threadIdx.x, rows = nd.rows, ncols = g.ncols;
  const bool first = nd.flags & FLAG_ALPHA;

  // Stage the block of A (threads along the index contiguous in memory) and
  // X; offsets are affine in the block's row and column (as in run_update).
  // A's loads are issued before the dependency wait, X's (which other nodes
  // write) after it, and every load before the first store, so that their
  // latencies overlap instead of adding up.
  const int64_t sgn = a.rev ? -1 : 1;
  const int64_t dr = sgn * (a.tA ? d.lda : 1), dk = sgn * (a.tA ? 1 : d.lda);
  const T* A0 = A + a_at(d, a.tA, a.rev, nd.r0, nd.r0);
  constexpr int A_PER = MAX_ROWS * MAX_ROWS / NT, X_PER = MAX_ROWS * W / NT;
  Tc va[A_PER];
  T vx[X_PER];
#pragma unroll
  for (int u = 0; u < A_PER; ++u) {
    const int idx = t + u * NT;
    const int r = a.tA ? idx / MAX_ROWS : idx % MAX_ROWS, k = a.tA ? idx % MAX_ROWS : idx / MAX_ROWS;
    va[u] = r < rows && k <= r ? to_c(A0[r * dr + k * dk]) : Tc(0);
  }
  if (!node_deps(a, nd, s_ok)) return false;
  const T* X0 = B + b_at(d, a.rev, nd.r0, g.c0);
  const int xr = t % MAX_ROWS;  // NT is a multiple of MAX_ROWS: each thread keeps one row of X
#pragma unroll
  for (int u = 0; u < X_PER; ++u) {
    const int c = (t + u * NT) / MAX_ROWS;
    vx[u] = xr < rows && c < ncols ? ldcg(X0 + xr * sgn + (int64_t)c * d.ldb) : T(0);
  }
#pragma unroll
  for (int u = 0; u < A_PER; ++u) {
    const int idx = t + u * NT;
    const int r = a.tA ? idx / MAX_ROWS : idx % MAX_ROWS, k = a.tA ? idx % MAX_ROWS : idx / MAX_ROWS;
    if (r < rows && k < r) Ls[r * LP + k] = va[u];
    else if (r < rows && k == r) inv[r] = Tc(1) / va[u];
  }
  if (first) {  // node-uniform (see the update's epilogue)
#pragma unroll
    for (int u = 0; u < X_PER; ++u) {
      const int c = (t + u * NT) / MAX_ROWS;
      if (xr < rows) Xs[xr * XP + c] = scaled_node<T>(vx[u], a);
    }
  } else {
#pragma unroll
    for (int u = 0; u < X_PER; ++u) {
      const int c = (t + u * NT) / MAX_ROWS;
      if (xr < rows) Xs[xr * XP + c] = to_c(vx[u]);
    }
  }
  __syncthreads();

  const int tr = t % ROW_GROUPS, tc = t / ROW_GROUPS;
  for (int p0 = 0; p0 < rows; p0 += PANEL) {
    const int pw = min(PANEL, rows - p0);
    // The panel's triangle: one right-hand side per thread (warps whose
    // right-hand sides all lie past the group's skip it), right-looking: as
    // soon as x_j is known it is subtracted from every later row.  Each row
    // sees the same FMAs in the same order (j increasing) as a row-by-row
    // dot product, so the bits are the same, but the dependent chain is one
    // FMA and one multiply per row instead of a whole dot product.
    if (t < W && (t & ~31) < ncols) {
      Tc y[PANEL];
#pragma unroll
      for (int i = 0; i < PANEL; ++i) y[i] = i < pw ? Xs[(p0 + i) * XP + t] : Tc(0);
#pragma unroll
      for (int j = 0; j < PANEL; ++j) {
        if (j < pw) {
          const Tc xj = y[j] * inv[p0 + j];
          Xs[(p0 + j) * XP + t] = xj;
#pragma unroll
          for (int r = j + 1; r < PANEL; ++r) y[r] = fma(-Ls[(p0 + r) * LP + p0 + j], xj, y[r]);
        }
      }
    }
    __syncthreads();
    // Rows below the panel: X[r, :] -= L[r, panel] X[panel, :].
    const int rb = p0 + pw;
    if (rb < rows && (tc & ~1) * CT < ncols) {
      Tc acc[RT][CT];
#pragma unroll
      for (int i = 0; i < RT; ++i)
#pragma unroll
        for (int c = 0; c < CT; ++c) acc[i][c] = Tc(0);
      for (int k = 0; k < pw; ++k) {
        Tc xv[CT];
#pragma unroll
        for (int c = 0; c < CT; ++c) xv[c] = Xs[(p0 + k) * XP + tc * CT + c];
#pragma unroll
        for (int i = 0; i < RT; ++i) {
          const int r = rb + tr + ROW_GROUPS * i;
          const Tc av = r < rows ? Ls[r * LP + p0 + k] : Tc(0);
#pragma unroll
          for (int c = 0; c < CT; ++c) acc[i][c] = fma(av, xv[c], acc[i][c]);
        }
      }
#pragma unroll
      for (int i = 0; i < RT; ++i) {
        const int r = rb + tr + ROW_GROUPS * i;
        if (r < rows) {
#pragma unroll
          for (int c = 0; c < CT; ++c) Xs[r * XP + tc * CT + c] -= acc[i][c];
        }
      }
    }
    __syncthreads();
  }
  T* Xw = B + b_at(d, a.rev, nd.r0, g.c0);
  for (int idx = t; idx < MAX_ROWS * W; idx += NT) {
    const int r = idx % MAX_ROWS, c = idx / MAX_ROWS;
    if (r < rows && c < ncols) Elem<T>::store(Xw + r * sgn + (int64_t)c * d.ldb, Xs[r * XP + c]);
  }
  return true;
}

template <typename T, int W>
__device__ __forceinline__ bool run_node(const Args& a, const Node& nd, const Group& g, const nla_batch_desc& d,
                                         void* smem, volatile int* s_ok) {
  if (nd.kind == NODE_LEAF) return run_leaf<T, W>(a, nd, g, d, smem, s_ok);
  return run_update<T, W>(a, nd, g, d, smem, s_ok);
}

template <typename T>
__global__ void __launch_bounds__(NT, 2) batched_node_kernel(Args a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_idx;
  __shared__ volatile int s_ok;
  for (;;) {
    if (threadIdx.x == 0) s_idx = atomicAdd(a.next, 1);
    __syncthreads();
    const int idx = s_idx;
    if (idx >= a.nnodes) break;
    const Node nd = a.nodes[idx];
    const Group g = a.groups[nd.group];
    const nla_batch_desc d = a.descs[g.sys];
    // Float64 groups are at most 64 wide (the plan splits wider blocks): a
    // 128-wide Float64 tile would not fit the register budget of two CTAs
    // per SM, and the FP64 pipe is saturated at 64.
    bool ok = false;
    switch (g.w) {
      case 16: ok = run_node<T, 16>(a, nd, g, d, smem_raw, &s_ok); break;
      case 32: ok = run_node<T, 32>(a, nd, g, d, smem_raw, &s_ok); break;
      case 64: ok = run_node<T, 64>(a, nd, g, d, smem_raw, &s_ok); break;
      default:
        if constexpr (sizeof(typename Elem<T>::compute) == 4) ok = run_node<T, 128>(a, nd, g, d, smem_raw, &s_ok);
        break;
    }
    if (!ok) break;  // a dependency did not arrive in time (the same on every thread)
    __syncthreads();  // every thread's stores of this node are issued
    if (threadIdx.x == 0) {
      __threadfence();
      if (nd.kind == NODE_LEAF) add_release(a.solved + nd.group, 1);
      else add_release(a.applied + g.leaf_base + nd.leaf, 1);
    }
  }
}

size_t node_smem_bytes(int dtype, int w_max) {
  const int esz = dtype == NLA_F64 ? 8 : 4;
  return std::max(update_elems(w_max, kc_of(esz)), leaf_elems(w_max)) * esz;
}

// ---------------------------------------------------------------------------
// Mixed-precision batch (Float32 solves, Float64 residuals), on the plan's
// groups: one CTA per group (map) or per (group, 64-row band) (residual).
// ---------------------------------------------------------------------------
enum MapOp { MAP_INIT = 0, MAP_SET = 1, MAP_ADD = 2 };

struct MapArgs {
  const nla_batch_desc* descs;
  const Group* groups;
  const double* A64;
  float* A32;
  double* B64;
  double* R64;
  float* X32;
  double alpha;
  int op;
};

// MAP_INIT: R = alpha B (Float64), X32 = (float) R, and (first group of each
// system) A32 = (float) A over the n x n block; MAP_SET: B = (double) X32;
// MAP_ADD: B += (double) X32.
__global__ void __launch_bounds__(256) batched_map_kernel(MapArgs a) {
  const Group g = a.groups[blockIdx.x];
  const nla_batch_desc d = a.descs[g.sys];
  const int n = (int)d.n;
  const int total = n * g.ncols;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int64_t o = d.b_off + (int64_t)(idx % n) + (int64_t)(g.c0 + idx / n) * d.ldb;
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
  if (a.op == MAP_INIT && g.c0 == 0) {
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
      const int64_t o = d.a_off + (int64_t)(idx % n) + (int64_t)(idx / n) * d.lda;
      a.A32[o] = (float)a.A64[o];
    }
  }
}

struct ResidualArgs {
  const nla_batch_desc* descs;
  const Group* groups;
  const double* A64;
  const double* X64;  // current solution (the caller's B pool)
  const double* R64;  // alpha B
  float* D32;         // out: the residual, rounded to Float32
  int tA, rev;
};

// D32 = (float)(R - L X) on one 64-row band of a group, L the canonical lower
// triangle (diagonal included) of op(A), summed in Float64 with the
// register-tiled product of the UPDATE nodes.
template <int W>
__device__ void residual_band(const ResidualArgs& a, const Group& g, const nla_batch_desc& d, int r0, double* smem) {
  constexpr int KC = 16, CT = W / 16, AP = MAX_ROWS + 4, XP = W + 4;
  double* As = smem;
  double* Xs = smem + KC * AP;
  const int t = threadIdx.x, tr = t % ROW_GROUPS, tc = t / ROW_GROUPS;
  const int rows = min(MAX_ROWS, (int)d.n - r0), ncols = g.ncols;
  const int kend = r0 + rows;  // k <= r
  double acc[RT][CT];
#pragma unroll
  for (int i = 0; i < RT; ++i)
#pragma unroll
    for (int c = 0; c < CT; ++c) acc[i][c] = 0.0;
  for (int k0 = 0; k0 < kend; k0 += KC) {
    const int kw = min(KC, kend - k0);
    __syncthreads();
    for (int idx = t; idx < MAX_ROWS * KC; idx += NT) {
      int r, k;
      if (!a.tA) { r = idx % MAX_ROWS; k = idx / MAX_ROWS; }
      else { k = idx % KC; r = idx / KC; }
      As[k * AP + r] = r < rows && k < kw && k0 + k <= r0 + r ? a.A64[a_at(d, a.tA, a.rev, r0 + r, k0 + k)] : 0.0;
    }
    for (int idx = t; idx < KC * W; idx += NT) {
      const int k = idx % KC, c = idx / KC;
      Xs[k * XP + c] = k < kw && c < ncols ? a.X64[b_at(d, a.rev, k0 + k, g.c0 + c)] : 0.0;
    }
    __syncthreads();
    for (int k = 0; k < kw; ++k) {
      double av[RT], xv[CT];
#pragma unroll
      for (int i = 0; i < RT; ++i) av[i] = As[k * AP + tr + ROW_GROUPS * i];
#pragma unroll
      for (int c = 0; c < CT; ++c) xv[c] = Xs[k * XP + tc * CT + c];
#pragma unroll
      for (int i = 0; i < RT; ++i)
#pragma unroll
        for (int c = 0; c < CT; ++c) acc[i][c] = fma(av[i], xv[c], acc[i][c]);
    }
  }
#pragma unroll
  for (int i = 0; i < RT; ++i) {
    const int r = tr + ROW_GROUPS * i;
    if (r >= rows) continue;
#pragma unroll
    for (int c = 0; c < CT; ++c) {
      const int col = tc * CT + c;
      if (col < ncols) {
        const int64_t o = b_at(d, a.rev, r0 + r, g.c0 + col);
        a.D32[o] = (float)(a.R64[o] - acc[i][c]);
      }
    }
  }
}

__global__ void __launch_bounds__(NT) batched_residual_kernel(ResidualArgs a) {
  __shared__ __align__(16) double smem[16 * (MAX_ROWS + 4) + 16 * (128 + 4)];
  const Group g = a.groups[blockIdx.x];
  const nla_batch_desc d = a.descs[g.sys];
  const int r0 = (int)blockIdx.y * MAX_ROWS;
  if (r0 >= d.n) return;
  switch (g.w) {
    case 16: residual_band<16>(a, g, d, r0, smem); break;
    case 32: residual_band<32>(a, g, d, r0, smem); break;
    case 64: residual_band<64>(a, g, d, r0, smem); break;
    default: residual_band<128>(a, g, d, r0, smem); break;
  }
}


// ---------------------------------------------------------------------------
// Exact residual of a mixed batch on the tensor cores.  One CTA per tile of
// 128 rows x 64 right-hand sides of a group: D32 = (float)(R - L X), with L
// the canonical lower triangle (diagonal included) and X the current
// Float64 solution, L X accumulated exactly enough for Float64 refinement.
//
// Every row of L and every column of X is scaled by its own power of two over
// the tile's K range (largest element in [1/4, 1/2)) and, one 64-wide block
// of K at a time, split into seven balanced 8-bit digits,
// y = round(v 2^(56 - e)) = sum_p d_p 2^(8 (6 - p)), |d_p| <= 128, each
// stored as a BF16 slice in shared memory (K-major, 128-byte swizzle, as
// tcgen05.mma reads it).  The 28 slice pairs (p, q) with p + q <= 6 are
// multiplied on the tensor cores, the pairs of one weight w = p + q into one
// FP32 accumulator in TMEM: 7 x 64 x 2^14 < 2^24, so each block's sums T_w
// are exact integers.  The epilogue warps add each block's
// S = H 2^a + round(L 2^(a - 24)) to an int64 per element, with
// H = sum_{w<4} T_w 2^(24 - 8 w), L = sum_{4<=w<7} T_w 2^(48 - 8 w) and
// a = 18 - ceil(log2(blocks)) (headroom for the tile's blocks), and the tile
// ends with one conversion: L X = acc 2^(e_r + e_c - 40 - a).  The rounding
// of L and the pairs left out (w >= 7) stay below 2^-53 of |l| |x| of the
// row's and column's largest elements per block.  Splitting, combining and
// accumulating are integer work: the FP64 pipe, slow on this part, is used
// once per output element.
// ---------------------------------------------------------------------------
constexpr int XR_ROWS = 128, XR_COLS = 64, XR_KB = 64, XR_SL = 7;
constexpr int XR_THREADS = 512;  // 16 warps: all split and drain; one thread issues the MMAs
constexpr int XR_A_BYTES = XR_SL * XR_ROWS * 128;  // 7 slices x 128 rows x 64 BF16
constexpr int XR_X_BYTES = XR_SL * XR_COLS * 128;  // 7 slices x 64 columns x 64 BF16
constexpr int XR_XRP = XR_KB + 1;                  // row pitch (doubles) of the raw X block, per column
constexpr int XR_XRAW_BYTES = XR_COLS * XR_XRP * 8;
constexpr int XR_SMEM = XR_A_BYTES + XR_X_BYTES + XR_XRAW_BYTES + 1024 + 4096;  // + alignment, exponents, barrier
constexpr int XR_NONFINITE = split7::NONFINITE;  // exponent marker of a row or column holding Inf or NaN
using split7::exp_field;
using split7::fixed56;
using split7::scale_exp;
using split7::store_chunks;

struct ExactTile {
  int group;
  int r0;  // canonical first row
  int c0;  // first right-hand side within the group
  int nkb;  // blocks of K
};

struct ExactResArgs {
  const nla_batch_desc* descs;
  const Group* groups;
  const ExactTile* tiles;
  const double* A64;
  const double* X64;
  const double* R64;
  float* D32;
  int tA, rev;
  int* err;
  const int* row_exp;        // scale exponent of each system row of A's triangle
  const int64_t* row_base;   // first row_exp entry of each system
  const int* col_exp;        // scale exponent of each group column of X
  const int64_t* col_base;   // first col_exp entry of each group
};

// Scale exponents of the rows of A's canonical lower triangles (k <= r), one
// CTA per band of 128 rows of a system, two threads per row.  A does not
// change between sweeps, so this runs once per mixed solve.
struct RowExpArgs {
  const nla_batch_desc* descs;
  const int2* bands;  // (system, first row of the band)
  const int64_t* row_base;
  const double* A64;
  int tA, rev;
  int* out;
};

__global__ void __launch_bounds__(256) batched_row_exp_kernel(RowExpArgs a) {
  __shared__ int part_max[256];
  const int2 b = a.bands[blockIdx.x];
  const nla_batch_desc d = a.descs[b.x];
  const int n = (int)d.n, t = threadIdx.x, row = t & 127, part = t >> 7, r = b.y + row;
  const int64_t dk = (a.rev ? -1 : 1) * (a.tA ? 1 : d.lda);
  int bm = 0;
  if (r < n) {
    const double* arow = a.A64 + a_at(d, a.tA, a.rev, r, 0);
#pragma unroll 8
    for (int k = part; k <= r; k += 2) bm = max(bm, exp_field(__ldg(arow + (int64_t)k * dk)));
  }
  part_max[t] = bm;
  __syncthreads();
  if (t < 128 && r < n) a.out[a.row_base[b.x] + r] = scale_exp(max(part_max[t], part_max[t + 128]));
}

// Scale exponents of the columns of X (over all n rows of the system), one
// CTA per group, a warp per column with its lanes along the column.
struct ColExpArgs {
  const nla_batch_desc* descs;
  const Group* groups;
  const int64_t* col_base;
  const double* X64;
  int rev;
  int* out;
};

__global__ void __launch_bounds__(256) batched_col_exp_kernel(ColExpArgs a) {
  const Group g = a.groups[blockIdx.x];
  const nla_batch_desc d = a.descs[g.sys];
  const int n = (int)d.n, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t sk = a.rev ? -1 : 1;
  for (int c = warp; c < g.ncols; c += 8) {
    const double* xc = a.X64 + b_at(d, a.rev, 0, g.c0 + c);
    int bx = 0;
#pragma unroll 4
    for (int k = lane; k < n; k += 32) bx = max(bx, exp_field(__ldcg(xc + (int64_t)k * sk)));
    bx = __reduce_max_sync(0xffffffffu, bx);
    if (lane == 0) a.out[a.col_base[blockIdx.x] + c] = scale_exp(bx);
  }
}

__global__ void __launch_bounds__(XR_THREADS, 1) batched_exact_residual_kernel(ExactResArgs a) {
  extern __shared__ uint8_t xr_smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(xr_smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* sA = smem;
  uint8_t* sX = smem + XR_A_BYTES;
  double* xraw = reinterpret_cast<double*>(sX + XR_X_BYTES);   // [64 columns][XR_XRP]
  int* ea_s = reinterpret_cast<int*>(xraw + XR_COLS * XR_XRP);  // [128]
  int* eb_s = ea_s + XR_ROWS;                                    // [64]
  uint64_t* mma_bar = reinterpret_cast<uint64_t*>(eb_s + XR_COLS);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mma_bar + 1);
  __shared__ volatile int s_abort;

  const ExactTile tile = a.tiles[blockIdx.x];
  const Group g = a.groups[tile.group];
  const nla_batch_desc d = a.descs[g.sys];
  const int n = (int)d.n, r0 = tile.r0, c0 = tile.c0;
  const int ncols = min(XR_COLS, g.ncols - c0);
  const int kend = min(n, r0 + XR_ROWS);  // k <= row
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int64_t dk = (a.rev ? -1 : 1) * (a.tA ? 1 : d.lda);  // step of canonical k within a row of A
  const int64_t sk = a.rev ? -1 : 1;                          // step of canonical k within a column of X
  const double* xbase = a.X64 + b_at(d, a.rev, 0, g.c0 + c0);  // canonical row 0 of the tile's first column
  // Fixed point of the per-element sums: headroom for the tile's blocks.
  const int lg = tile.nkb > 1 ? 32 - __clz(tile.nkb - 1) : 0;
  const int sa_bits = 18 - lg, sl_bits = 24 - sa_bits;

  if (t == 0) {
    s_abort = 0;
    umma::mbar_init(umma::smem_u32(mma_bar), 1);
    umma::fence_barrier_init();
  }
  if (warp == 0) umma::tmem_alloc(umma::smem_u32(tmem_slot), 512);

  // Scale exponents (per row of A's triangle and per column of X, formed by
  // batched_row_exp_kernel and batched_col_exp_kernel).
  if (t < XR_ROWS) ea_s[t] = r0 + t < n ? a.row_exp[a.row_base[g.sys] + r0 + t] : 0;
  else if (t < XR_ROWS + XR_COLS) {
    const int c = t - XR_ROWS;
    eb_s[c] = c < ncols ? a.col_exp[a.col_base[tile.group] + c0 + c] : 0;
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  // Drain role: rows q * 32 + lane (the warp's TMEM lane quarter), columns
  // h * 16 .. + 16.
  const int q = warp & 3, h = warp >> 2;
  long long acc[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) acc[j] = 0;
  bool ok = true;
  // Split roles: A row t % 128 with the block's k values 16 (t / 128) ..
  // + 16; X column t % 64 with k values 8 (t / 64) .. + 8, read back from the
  // raw block, which threads load along k (thread -> k t % 64, columns
  // t / 64 + 8 j): coalesced.
  const int arow_i = t & 127, apart = t >> 7, ar = r0 + arow_i;
  const double* arow = a.A64 + a_at(d, a.tA, a.rev, min(ar, n - 1), 0);
  const int xk = t & 63, xc8 = t >> 6;

  // One block ahead: the raw X block goes to shared memory by asynchronous
  // copies (zero-filled outside the system), and the first eight values of
  // A into registers, so that both latencies pass during the previous
  // block's MMAs and drain.
  double va[8];
  auto load_ahead = [&](int k0) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int k = k0 + xk, col = xc8 + 8 * j;
      const bool in = k < kend && col < ncols;
      const double* src = in ? xbase + (int64_t)k * sk + (int64_t)col * d.ldb : a.X64;
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(umma::smem_u32(xraw + (xc8 + 8 * j) * XR_XRP + xk)),
                   "l"(src), "r"(in ? 8 : 0)
                   : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int k = k0 + apart * 16 + u;
      va[u] = ar < n && k <= ar ? __ldg(arow + (int64_t)k * dk) : 0.0;
    }
  };
  load_ahead(0);
  int kb = 0;
  for (; kb < tile.nkb && ok; ++kb) {
    const int k0 = kb * XR_KB;
    {
      const int ea = ea_s[arow_i];
#pragma unroll 1
      for (int c = 0; c < 2; ++c) {
        long long y[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) y[u] = fixed56(va[u], ea);
        if (c == 0) {
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int k = k0 + apart * 16 + 8 + u;
            va[u] = ar < n && k <= ar ? __ldg(arow + (int64_t)k * dk) : 0.0;
          }
        }
        store_chunks(sA, XR_ROWS * 128, arow_i, apart * 2 + c, y);
      }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();  // the raw X block is in shared memory
    {
      const int col = t & 63, kc = t >> 6;
      const int eb = eb_s[col];
      long long y[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) y[u] = fixed56(xraw[col * XR_XRP + kc * 8 + u], eb);
      store_chunks(sX, XR_COLS * 128, col, kc, y);
    }
    // The tensor cores read shared memory through the async proxy.
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (t == 0) {
      // Slice p of A against X's slices q = 0 .. 6 - p, stacked in shared
      // memory, into the adjacent accumulators p + q: MMAs up to N = 256
      // wide, 10 per 16-wide K step instead of 28 (exact integer sums, so
      // the order is free).
      const uint32_t a0 = umma::smem_u32(sA), x0 = umma::smem_u32(sX);
#pragma unroll 1
      for (int p = 0; p < XR_SL; ++p) {
        const int rows = XR_COLS * (XR_SL - p);
#pragma unroll 1
        for (int q0 = 0; q0 < rows; q0 += 256) {
          const int nn = min(256, rows - q0);
          const uint32_t idesc = umma::idesc_f16(XR_ROWS, nn, true);
#pragma unroll
          for (int kk = 0; kk < XR_KB / 16; ++kk)
            umma::mma_f16(tmem + (uint32_t)(p * XR_COLS + q0), umma::desc_kmajor_sw128(a0 + p * XR_ROWS * 128 + kk * 32),
                          umma::desc_kmajor_sw128(x0 + q0 * 128 + kk * 32), idesc, (p > 0 || kk > 0) ? 1u : 0u);
        }
      }
      umma::mma_commit(umma::smem_u32(mma_bar));
    }
    __syncwarp();
    if (kb + 1 < tile.nkb) load_ahead(k0 + XR_KB);  // the X split above has read the raw block
    ok = __all_sync(0xffffffffu, umma::mbar_wait(umma::smem_u32(mma_bar), (uint32_t)kb & 1u, &s_abort, a.err, 21));
    umma::fence_after_sync();
    if (ok) {
      const long long lround = 1ll << (sl_bits - 1);
      const uint32_t tq = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(h * 16);
      long long S[16];
      // H: weights 0..3.
#pragma unroll
      for (int j = 0; j < 16; ++j) S[j] = 0;
#pragma unroll
      for (int w = 0; w < 4; ++w) {
        uint32_t rr[16];
        umma::tmem_ld16(tq + (uint32_t)(w * XR_COLS), rr);
#pragma unroll
        for (int j = 0; j < 16; ++j) S[j] += (long long)__float2int_rn(__uint_as_float(rr[j])) << (24 - 8 * w);
      }
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        acc[j] += S[j] << sa_bits;
        S[j] = 0;
      }
      // L: weights 4..6, rounded to the fixed point.
#pragma unroll
      for (int w = 4; w < XR_SL; ++w) {
        uint32_t rr[16];
        umma::tmem_ld16(tq + (uint32_t)(w * XR_COLS), rr);
#pragma unroll
        for (int j = 0; j < 16; ++j) S[j] += (long long)__float2int_rn(__uint_as_float(rr[j])) << (48 - 8 * w);
      }
#pragma unroll
      for (int j = 0; j < 16; ++j) acc[j] += (S[j] + lround) >> sl_bits;
    }
    umma::fence_before_sync();
    __syncthreads();
    ok = ok && !s_abort;
  }
  asm volatile("cp.async.wait_all;" ::: "memory");  // no copy into shared memory outlives the loop
  if (!ok && t == 0 && kb > 0) {
    // A wait gave up: let the tensor cores finish the last block's MMAs (a
    // drain with the default limit) before the tensor memory is released.
    umma::mbar_wait(umma::smem_u32(mma_bar), (uint32_t)(kb - 1) & 1u, &s_abort, a.err, 22, false);
  }

  if (ok) {
    const int row = q * 32 + lane, r = r0 + row;
    if (r < n) {
      const int ea = ea_s[row];
      // All loads before the stores (the pools may alias as far as the
      // compiler knows).
      double rv[16];
      const int64_t rbase = b_at(d, a.rev, r, g.c0 + c0 + h * 16);
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int col = h * 16 + j;
        rv[j] = col < ncols ? a.R64[rbase + (int64_t)j * d.ldb] : 0.0;
      }
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int col = h * 16 + j;
        if (col < ncols) {
          const int eb = eb_s[col];
          const float res = ea == XR_NONFINITE || eb == XR_NONFINITE
                                ? __int_as_float(0x7FC00000)
                                : (float)(rv[j] - split7::scaled_i64_to_f64(acc[j], ea + eb - 40 - sa_bits));
          a.D32[rbase + (int64_t)j * d.ldb] = res;
        }
      }
    }
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    umma::fence_after_sync();
    umma::tmem_dealloc(tmem, 512);
  }
}
}  // namespace bat
}  // namespace nla

// ---------------------------------------------------------------------------
// Host side: the plan.
// ---------------------------------------------------------------------------
struct nla_batch_plan_s {
  int dtype;
  int tA, rev;
  char uplo0, trans0;  // the flags the plan was created with
  nla_batch_plan p32;  // mixed batches: a Float32 plan of the same systems (built on first use)
  int64_t count;
  std::vector<nla_batch_desc> h_descs;
  std::vector<nla::bat::Group> h_groups;
  int ngroups, nleaves, nnodes;
  int n_max;
  int w_max;
  size_t smem;
  int grid;
  double flops;
  void* d_descs;
  void* d_groups;
  void* d_nodes;
  int* d_counters;  // next, abort, then solved[ngroups], then applied[nleaves]
  size_t counter_bytes;
  cudaStream_t cap_stream;
  cudaGraphExec_t exec;
  double g_alpha;
  const void* g_A;
  void* g_B;
  uint64_t g_limit;
  // Mixed-precision form (Float64 plans): pool extents in elements and the
  // plan-owned Float32 pools and Float64 residual buffer (allocated on first
  // use).
  int64_t a_elems, b_elems;
  float* a32;
  float* x32;
  double* r64;
  // Tensor-core residual (built on first use): tiles, row bands, the
  // exponents' indexing and the exponents, in one allocation.
  void* d_xtiles;
  int nxtiles;
  int2* d_bands;
  int nbands;
  int64_t* d_row_base;
  int64_t* d_col_base;
  int* d_row_exp;
  int* d_col_exp;
};

namespace nla {
namespace {

using bat::Group;
using bat::Node;

int bucket_of(int64_t n) {
  int b = 0;
  int64_t hi = 32;
  while (b < NLA_BATCH_BUCKETS - 1 && n >= hi) {
    ++b;
    hi *= 2;
  }
  return b;
}

// Default tuning per size bucket (16 * 2^b <= n < 32 * 2^b), measured on a
// GB300 with the autotuner (tune.py) and used when the caller passes none.
void default_tuning(int dtype, nla_batch_tuning* t) {
  for (int b = 0; b < NLA_BATCH_BUCKETS; ++b) {
    t->cutoff[b] = 64;
    t->cols[b] = dtype == NLA_F64 ? 64 : 128;
  }
}

int check_tuning(const nla_batch_tuning& t) {
  for (int b = 0; b < NLA_BATCH_BUCKETS; ++b) {
    if (t.cutoff[b] != 16 && t.cutoff[b] != 32 && t.cutoff[b] != 64)
      return fail(NLA_ERR_ARG, "batch tuning: cutoff entries must be 16, 32 or 64");
    if (t.cols[b] != 16 && t.cols[b] != 32 && t.cols[b] != 64 && t.cols[b] != 128)
      return fail(NLA_ERR_ARG, "batch tuning: cols entries must be 16, 32, 64 or 128");
  }
  return NLA_OK;
}

struct HostNode {
  Node d;
  double cost;
  double prio;
  int pred[2];  // at most two: the leaf's previous update, the first half's last leaf
  int npred;
};

// Relative cost of a node on one CTA (flop-equivalents): the update tiles
// run near the register-tiled product's rate, the leaves' panel triangles at
// a fraction of it, and every node pays a fixed start-up (staging, waits).
double node_cost(const Node& nd, int w) {
  const double overhead = 40000.0;
  if (nd.kind == bat::NODE_UPDATE) return overhead + 2.0 * nd.rows * (double)nd.kw * w;
  return overhead + 3.0 * (double)nd.rows * nd.rows * w;
}

// The recursion of unified_rec over canonical rows [start, start + len) of
// one group, emitting leaves and update tiles in the recursion's order.
// `first` of a node is its split point measured from the end solved first
// (forward: the reference's mid; backward: len - mid, the reference's
// second half read in reverse).
struct GroupBuilder {
  int gi;
  int cutoff;
  bool rev;
  std::vector<int> leaf_start, leaf_len;  // leaves in solve order
  std::vector<int> chain;                 // updates so far per leaf
  std::vector<int> last_node;             // last node touching each leaf
  std::vector<HostNode>* nodes;
  int group_w;

  void leaves(int start, int len) {
    if (len <= cutoff) {
      leaf_start.push_back(start);
      leaf_len.push_back(len);
      return;
    }
    const int mid = (int)split_point(len);
    const int first = rev ? len - mid : mid;
    leaves(start, first);
    leaves(start + first, len - first);
  }
  int leaf_at(int row) const {
    return (int)(std::upper_bound(leaf_start.begin(), leaf_start.end(), row) - leaf_start.begin()) - 1;
  }
  void link(int from, int to) {
    if (from < 0) return;
    HostNode& t = (*nodes)[to];
    t.pred[t.npred++] = from;
  }
  int add(const Node& nd) {
    HostNode h{};
    h.d = nd;
    h.cost = node_cost(nd, group_w);
    h.npred = 0;
    nodes->push_back(h);
    return (int)nodes->size() - 1;
  }
  void rec(int start, int len) {
    if (len <= cutoff) {
      const int j = leaf_at(start);
      Node nd{};
      nd.group = gi;
      nd.r0 = start;
      nd.rows = len;
      nd.leaf = j;
      nd.kind = bat::NODE_LEAF;
      nd.flags = chain[j] == 0 ? bat::FLAG_ALPHA : 0;
      nd.wait_solved = j;
      nd.wait_applied = (short)chain[j];
      const int id = add(nd);
      link(last_node[j], id);
      last_node[j] = id;
      return;
    }
    const int mid = (int)split_point(len);
    const int first = rev ? len - mid : mid;
    rec(start, first);
    // The update between the halves, one tile per leaf of the second half.
    const int j_first = leaf_at(start + first);
    const int last_solved = j_first - 1;  // the first half's last leaf
    for (int j = j_first; j < (int)leaf_start.size() && leaf_start[j] < start + len; ++j) {
      Node nd{};
      nd.group = gi;
      nd.r0 = leaf_start[j];
      nd.rows = leaf_len[j];
      nd.k0 = start;
      nd.kw = first;
      nd.leaf = j;
      nd.kind = bat::NODE_UPDATE;
      nd.flags = chain[j] == 0 ? bat::FLAG_ALPHA : 0;
      nd.wait_solved = j_first;
      nd.wait_applied = (short)chain[j];
      const int id = add(nd);
      link(last_node[j], id);            // the leaf's previous update
      link(last_node[last_solved], id);  // the first half solved (its last leaf)
      last_node[j] = id;
      chain[j]++;
    }
    rec(start + first, len - first);
  }
};

// List scheduling of the nodes over `workers` CTAs: each free worker takes
// the ready node with the longest remaining path (costs summed to the end of
// its group); the order nodes start in is the queue order.  It is a
// topological order, which the persistent kernel relies on.
std::vector<int> schedule(std::vector<HostNode>& nodes, int workers) {
  const int N = (int)nodes.size();
  // Successor lists (CSR) from the predecessors.
  std::vector<int> first(N + 1, 0), succ;
  for (int i = 0; i < N; ++i)
    for (int q = 0; q < nodes[i].npred; ++q) first[nodes[i].pred[q] + 1]++;
  for (int i = 0; i < N; ++i) first[i + 1] += first[i];
  succ.resize(first[N]);
  {
    std::vector<int> fill(first.begin(), first.end() - 1);
    for (int i = 0; i < N; ++i)
      for (int q = 0; q < nodes[i].npred; ++q) succ[fill[nodes[i].pred[q]]++] = i;
  }
  // Longest path to the end: predecessors were created before their
  // successors, so a reverse sweep sees every successor first.
  std::vector<double> below(N, 0.0);
  for (int i = N - 1; i >= 0; --i) {
    nodes[i].prio = nodes[i].cost + below[i];
    for (int q = 0; q < nodes[i].npred; ++q) below[nodes[i].pred[q]] = std::max(below[nodes[i].pred[q]], nodes[i].prio);
  }
  std::vector<int> preds_left(N);
  std::vector<double> ready_at(N, 0.0);
  using Ready = std::pair<double, int>;  // (priority, node)
  std::priority_queue<Ready> ready;
  using Pending = std::pair<double, int>;  // (ready time, node), earliest first
  std::priority_queue<Pending, std::vector<Pending>, std::greater<Pending>> pending;
  for (int i = 0; i < N; ++i) {
    preds_left[i] = nodes[i].npred;
    if (preds_left[i] == 0) ready.push({nodes[i].prio, i});
  }
  std::priority_queue<double, std::vector<double>, std::greater<double>> free_at;
  for (int w = 0; w < workers; ++w) free_at.push(0.0);
  std::vector<int> order;
  order.reserve(N);
  while ((int)order.size() < N) {
    double t = free_at.top();
    free_at.pop();
    while (!pending.empty() && pending.top().first <= t) {
      ready.push({nodes[pending.top().second].prio, pending.top().second});
      pending.pop();
    }
    if (ready.empty()) {
      // Idle until the next node becomes ready.
      t = pending.top().first;
      while (!pending.empty() && pending.top().first <= t) {
        ready.push({nodes[pending.top().second].prio, pending.top().second});
        pending.pop();
      }
    }
    const int i = ready.top().second;
    ready.pop();
    order.push_back(i);
    const double fin = t + nodes[i].cost;
    free_at.push(fin);
    for (int k = first[i]; k < first[i + 1]; ++k) {
      const int j = succ[k];
      ready_at[j] = std::max(ready_at[j], fin);
      if (--preds_left[j] == 0) pending.push({ready_at[j], j});
    }
  }
  return order;
}

template <typename T>
int node_kernel_setup(size_t smem, int* per_sm) {
  static std::once_flag once;
  static cudaError_t st = cudaSuccess;
  std::call_once(once, [] {
    st = cudaFuncSetAttribute(bat::batched_node_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  });
  if (st != cudaSuccess) return cuda_status(st, "cudaFuncSetAttribute(batched_node_kernel)");
  if (smem > 200 * 1024) return fail(NLA_ERR_UNSUPPORTED, "batch: shared memory plan too large");
  const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, bat::batched_node_kernel<T>, bat::NT,
                                                                      smem);
  return e == cudaSuccess ? NLA_OK : cuda_status(e, "batch: occupancy query");
}

template <typename T>
int launch_nodes(nla_batch_plan p, double alpha, const void* A, void* B, cudaStream_t s) {
  int* c = p->d_counters;  // next, abort, solved[ngroups], applied[nleaves]
  bat::Args a{static_cast<const nla_batch_desc*>(p->d_descs), static_cast<const Group*>(p->d_groups),
              static_cast<const Node*>(p->d_nodes), p->nnodes, c, c + 2, c + 2 + p->ngroups, c + 1, nullptr, A, B,
              p->tA, p->rev, alpha, wait_limit_ns(), (float)alpha, (double)(float)alpha == alpha ? 1 : 0};
  void* errp = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&errp, bat::g_batch_error);
  if (e != cudaSuccess) return cuda_status(e, "batch error word");
  a.err = static_cast<int*>(errp);
  bat::batched_node_kernel<T><<<p->grid, bat::NT, p->smem, s>>>(a);
  NLA_CHECK_LAUNCH("batched_node_kernel");
  return NLA_OK;
}

int enqueue(nla_batch_plan p, double alpha, const void* A, void* B, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(p->d_counters, 0, p->counter_bytes, s);
  if (e != cudaSuccess) return cuda_status(e, "batch counter reset");
  switch (p->dtype) {
    case NLA_F64: return launch_nodes<double>(p, alpha, A, B, s);
    case NLA_F32: return launch_nodes<float>(p, alpha, A, B, s);
    default: return launch_nodes<__half>(p, alpha, A, B, s);
  }
}

int plan_create(nla_batch_plan* out, int dtype, char uplo, char trans, int64_t count, const nla_batch_desc* descs,
                const nla_batch_tuning& tun) {
  if (!out) return fail(NLA_ERR_ARG, "plan pointer is null");
  *out = nullptr;
  NLA_TRY(check_flags('L', uplo, trans, 'S', dtype));
  if (is_complex(dtype)) return fail(NLA_ERR_DTYPE, "batch: real element types only");
  NLA_TRY(check_tuning(tun));
  if (count < 0 || (count > 0 && !descs)) return fail(NLA_ERR_ARG, "bad system count or descriptor array");
  if (count > (int64_t)1 << 24) return fail(NLA_ERR_UNSUPPORTED, "too many systems");
  for (int64_t i = 0; i < count; ++i) {
    const nla_batch_desc& d = descs[i];
    if (d.n < 0 || d.m < 0 || d.n > 1024 || d.lda < (d.n > 1 ? d.n : 1) || d.ldb < (d.n > 1 ? d.n : 1) ||
        d.a_off < 0 || d.b_off < 0)
      return fail(NLA_ERR_ARG, "system " + std::to_string(i) + ": bad size, leading dimension or offset");
  }
  nla_batch_plan p = new nla_batch_plan_s();
  p->dtype = dtype;
  p->uplo0 = uplo;
  p->trans0 = trans;
  p->p32 = nullptr;
  p->tA = (trans == 'T' || trans == 'C') ? 1 : 0;
  const char up = p->tA ? (uplo == 'L' ? 'U' : 'L') : uplo;
  p->rev = up == 'U';
  p->count = count;
  p->h_descs.assign(descs, descs + count);
  p->n_max = 1;
  p->w_max = 16;
  p->flops = 0;
  p->a_elems = p->b_elems = 0;
  p->a32 = p->x32 = nullptr;
  p->r64 = nullptr;
  p->d_xtiles = nullptr;
  p->nxtiles = 0;
  p->d_bands = nullptr;
  p->nbands = 0;
  p->d_row_base = p->d_col_base = nullptr;
  p->d_row_exp = p->d_col_exp = nullptr;
  p->exec = nullptr;
  p->d_descs = p->d_groups = p->d_nodes = nullptr;
  p->d_counters = nullptr;
  p->cap_stream = nullptr;

  std::vector<Group> groups;
  std::vector<HostNode> nodes;
  int leaves_total = 0;
  for (int64_t i = 0; i < count; ++i) {
    const nla_batch_desc& d = descs[i];
    if (d.n == 0 || d.m == 0) continue;
    p->a_elems = std::max<int64_t>(p->a_elems, d.a_off + (d.n - 1) * d.lda + d.n);
    p->b_elems = std::max<int64_t>(p->b_elems, d.b_off + (d.m - 1) * d.ldb + d.n);
    p->n_max = std::max<int>(p->n_max, (int)d.n);
    p->flops += (double)d.n * d.n * d.m;
    const int b = bucket_of(d.n);
    const int wcap = dtype == NLA_F64 ? std::min(tun.cols[b], 64) : tun.cols[b];
    // Balanced blocks of right-hand sides, each at most wcap wide, each run
    // with the narrowest column template that holds it.
    const int64_t nblk = (d.m + wcap - 1) / wcap;
    for (int64_t k = 0; k < nblk; ++k) {
      const int64_t c0 = d.m * k / nblk, c1 = d.m * (k + 1) / nblk;
      Group g{};
      g.sys = (int)i;
      g.c0 = (int)c0;
      g.ncols = (int)(c1 - c0);
      g.w = g.ncols <= 16 ? 16 : g.ncols <= 32 ? 32 : g.ncols <= 64 ? 64 : 128;
      g.leaf_base = leaves_total;
      g.n = (int)d.n;
      p->w_max = std::max(p->w_max, g.w);
      GroupBuilder gb;
      gb.gi = (int)groups.size();
      gb.cutoff = tun.cutoff[b];
      gb.rev = p->rev != 0;
      gb.nodes = &nodes;
      gb.group_w = g.w;
      gb.leaves(0, (int)d.n);
      gb.chain.assign(gb.leaf_start.size(), 0);
      gb.last_node.assign(gb.leaf_start.size(), -1);
      gb.rec(0, (int)d.n);
      leaves_total += (int)gb.leaf_start.size();
      groups.push_back(g);
    }
  }
  if (groups.size() > (size_t)INT32_MAX / 2 || nodes.size() > (size_t)INT32_MAX / 2) {
    delete p;
    return fail(NLA_ERR_UNSUPPORTED, "batch too large");
  }
  p->h_groups = groups;
  p->ngroups = (int)groups.size();
  p->nleaves = leaves_total;
  p->nnodes = (int)nodes.size();
  p->smem = bat::node_smem_bytes(dtype, p->w_max);
  int per_sm = 0, rc;
  if (dtype == NLA_F64) rc = node_kernel_setup<double>(p->smem, &per_sm);
  else if (dtype == NLA_F32) rc = node_kernel_setup<float>(p->smem, &per_sm);
  else rc = node_kernel_setup<__half>(p->smem, &per_sm);
  if (rc != NLA_OK) {
    delete p;
    return rc;
  }
  p->grid = std::max(1, std::min(std::max(p->nnodes, 1), num_sms() * std::max(per_sm, 1)));
  const std::vector<int> order = schedule(nodes, p->grid);
  std::vector<Node> queue(nodes.size());
  for (size_t k = 0; k < order.size(); ++k) queue[k] = nodes[order[k]].d;

  p->counter_bytes = sizeof(int) * (size_t)(2 + p->ngroups + p->nleaves);
  cudaError_t e = cudaMalloc(&p->d_descs, sizeof(nla_batch_desc) * (size_t)std::max<int64_t>(count, 1));
  if (e == cudaSuccess) e = cudaMalloc(&p->d_groups, sizeof(Group) * (size_t)std::max(p->ngroups, 1));
  if (e == cudaSuccess) e = cudaMalloc(&p->d_nodes, sizeof(Node) * (size_t)std::max(p->nnodes, 1));
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&p->d_counters), p->counter_bytes);
  if (e == cudaSuccess && count > 0)
    e = cudaMemcpy(p->d_descs, descs, sizeof(nla_batch_desc) * (size_t)count, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && p->ngroups > 0)
    e = cudaMemcpy(p->d_groups, groups.data(), sizeof(Group) * groups.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && p->nnodes > 0)
    e = cudaMemcpy(p->d_nodes, queue.data(), sizeof(Node) * queue.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    cudaFree(p->d_descs);
    cudaFree(p->d_groups);
    cudaFree(p->d_nodes);
    cudaFree(p->d_counters);
    delete p;
    return cuda_status(e, "batch plan allocation");
  }
  *out = p;
  return NLA_OK;
}

// Tiles of the tensor-core residual: 128 rows x 64 right-hand sides of a
// group, with their blocks of K (k <= row), longest first; the 128-row bands
// of every system for the row exponents; the exponents' indexing; and the
// kernel's shared-memory limit.  One device allocation holds them all.
int exact_residual_setup(nla_batch_plan p) {
  static std::once_flag once;
  static cudaError_t st = cudaSuccess;
  std::call_once(once, [] {
    st = cudaFuncSetAttribute(bat::batched_exact_residual_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              bat::XR_SMEM);
  });
  if (st != cudaSuccess) return cuda_status(st, "cudaFuncSetAttribute(batched_exact_residual_kernel)");
  if (p->d_xtiles) return NLA_OK;
  std::vector<bat::ExactTile> tiles;
  std::vector<int64_t> col_base(p->h_groups.size());
  int64_t ncol = 0;
  for (int gi = 0; gi < (int)p->h_groups.size(); ++gi) {
    const bat::Group& g = p->h_groups[gi];
    col_base[gi] = ncol;
    ncol += g.ncols;
    for (int r0 = 0; r0 < g.n; r0 += bat::XR_ROWS)
      for (int c0 = 0; c0 < g.ncols; c0 += bat::XR_COLS) {
        const int kend = std::min(g.n, r0 + bat::XR_ROWS);
        tiles.push_back(bat::ExactTile{gi, r0, c0, (kend + bat::XR_KB - 1) / bat::XR_KB});
      }
  }
  std::stable_sort(tiles.begin(), tiles.end(),
                   [](const bat::ExactTile& x, const bat::ExactTile& y) { return x.nkb > y.nkb; });
  if (tiles.empty()) return NLA_OK;  // nothing to launch
  std::vector<int2> bands;
  std::vector<int64_t> row_base(p->h_descs.size());
  int64_t nrow = 0;
  for (size_t i = 0; i < p->h_descs.size(); ++i) {
    row_base[i] = nrow;
    nrow += p->h_descs[i].n;
    for (int64_t r0 = 0; r0 < p->h_descs[i].n; r0 += bat::XR_ROWS) bands.push_back(make_int2((int)i, (int)r0));
  }
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t o_bands = up(sizeof(bat::ExactTile) * tiles.size());
  const size_t o_rb = o_bands + up(sizeof(int2) * std::max<size_t>(bands.size(), 1));
  const size_t o_cb = o_rb + up(sizeof(int64_t) * row_base.size());
  const size_t o_re = o_cb + up(sizeof(int64_t) * std::max<size_t>(col_base.size(), 1));
  const size_t o_ce = o_re + up(sizeof(int) * (size_t)std::max<int64_t>(nrow, 1));
  const size_t total = o_ce + up(sizeof(int) * (size_t)std::max<int64_t>(ncol, 1));
  uint8_t* base = nullptr;
  cudaError_t e = cudaMalloc(&base, total);
  if (e == cudaSuccess) e = cudaMemcpy(base, tiles.data(), sizeof(bat::ExactTile) * tiles.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !bands.empty())
    e = cudaMemcpy(base + o_bands, bands.data(), sizeof(int2) * bands.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !row_base.empty())
    e = cudaMemcpy(base + o_rb, row_base.data(), sizeof(int64_t) * row_base.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !col_base.empty())
    e = cudaMemcpy(base + o_cb, col_base.data(), sizeof(int64_t) * col_base.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(base);
    return cuda_status(e, "residual tiles");
  }
  p->d_xtiles = base;
  p->nxtiles = (int)tiles.size();
  p->d_bands = reinterpret_cast<int2*>(base + o_bands);
  p->nbands = (int)bands.size();
  p->d_row_base = reinterpret_cast<int64_t*>(base + o_rb);
  p->d_col_base = reinterpret_cast<int64_t*>(base + o_cb);
  p->d_row_exp = reinterpret_cast<int*>(base + o_re);
  p->d_col_exp = reinterpret_cast<int*>(base + o_ce);
  return NLA_OK;
}

}  // namespace

// Reads (and clears) the batched kernel's error word: the site of the first
// dependency wait that gave up, or 0.
int batch_device_error() {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, bat::g_batch_error, sizeof(int)) != cudaSuccess) return 0;
  if (v != 0) {
    const int zero = 0;
    cudaMemcpyToSymbol(bat::g_batch_error, &zero, sizeof(int));
  }
  return v;
}

}  // namespace nla

using namespace nla;

extern "C" {

int nla_batch_plan_create(nla_batch_plan* out, int dtype, char uplo, char trans, int64_t count,
                          const nla_batch_desc* descs, const int* cols_per_item) {
  clear_error();
  nla_batch_tuning t;
  default_tuning(dtype, &t);
  if (cols_per_item)
    for (int b = 0; b < NLA_BATCH_BUCKETS; ++b) t.cols[b] = cols_per_item[b];
  return plan_create(out, dtype, uplo, trans, count, descs, t);
}

int nla_batch_plan_create_tuned(nla_batch_plan* out, int dtype, char uplo, char trans, int64_t count,
                                const nla_batch_desc* descs, const nla_batch_tuning* tuning) {
  clear_error();
  nla_batch_tuning t;
  default_tuning(dtype, &t);
  if (tuning) t = *tuning;
  return plan_create(out, dtype, uplo, trans, count, descs, t);
}

int nla_batch_plan_info(nla_batch_plan p, int64_t* items, int64_t* grid, double* flops) {
  clear_error();
  if (!p) return fail(NLA_ERR_ARG, "null plan");
  if (items) *items = p->nnodes;
  if (grid) *grid = p->grid;
  if (flops) *flops = p->flops;
  return NLA_OK;
}

int nla_batch_solve(nla_batch_plan p, double alpha, const void* A_pool, void* B_pool, int mode, void* stream) {
  clear_error();
  if (!p) return fail(NLA_ERR_ARG, "null plan");
  if (p->nnodes == 0) return NLA_OK;
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
  if (!p->exec || p->g_alpha != alpha || p->g_A != A_pool || p->g_B != B_pool || p->g_limit != wait_limit_ns()) {
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
    p->g_limit = wait_limit_ns();
  }
  cudaError_t e = cudaGraphLaunch(p->exec, s);
  return e == cudaSuccess ? NLA_OK : cuda_status(e, "batch graph launch");
}

int nla_batch_solve_mixed(nla_batch_plan p, double alpha, const void* A_pool, void* B_pool, int sweeps,
                          void* stream) {
  return nla_batch_solve_mixed_ex(p, alpha, A_pool, B_pool, sweeps, NLA_RESIDUAL_SPLIT, stream);
}

int nla_batch_solve_mixed_ex(nla_batch_plan p, double alpha, const void* A_pool, void* B_pool, int sweeps,
                             int residual, void* stream) {
  clear_error();
  if (residual != NLA_RESIDUAL_SPLIT && residual != NLA_RESIDUAL_FP64)
    return fail(NLA_ERR_ARG, "mixed batch: residual must be NLA_RESIDUAL_SPLIT or NLA_RESIDUAL_FP64");
  if (!p) return fail(NLA_ERR_ARG, "null plan");
  if (p->dtype != NLA_F64) return fail(NLA_ERR_DTYPE, "mixed batch: the plan must be Float64");
  if (sweeps < 0 || sweeps > 8) return fail(NLA_ERR_ARG, "mixed batch: sweeps must be 0..8");
  if (p->nnodes == 0) return NLA_OK;
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
  // The Float32 solves run on a Float32 plan of the same systems: its groups
  // take up to 128 right-hand sides (a Float64 plan's at most 64), so it has
  // fewer, wider nodes; its pools share the Float64 pools' offsets.
  if (!p->p32) {
    nla_batch_tuning t32;
    default_tuning(NLA_F32, &t32);
    NLA_TRY(plan_create(&p->p32, NLA_F32, p->uplo0, p->trans0, p->count, p->h_descs.data(), t32));
  }
  int per_sm = 0;
  NLA_TRY(node_kernel_setup<float>(p->p32->smem, &per_sm));
  const auto* descs = static_cast<const nla_batch_desc*>(p->d_descs);
  const auto* groups = static_cast<const Group*>(p->d_groups);
  double* B64 = static_cast<double*>(B_pool);
  const double* A64 = static_cast<const double*>(A_pool);
  TraceScope trace(NLA_K_BATCHED, s, p->flops, 0.0);
  bat::MapArgs m{descs, groups, A64, p->a32, B64, p->r64, p->x32, alpha, bat::MAP_INIT};
  bat::batched_map_kernel<<<p->ngroups, 256, 0, s>>>(m);
  NLA_CHECK_LAUNCH("batched_map_kernel");
  auto solve32 = [&]() -> int {
    cudaError_t e = cudaMemsetAsync(p->p32->d_counters, 0, p->p32->counter_bytes, s);
    if (e != cudaSuccess) return cuda_status(e, "batch counter reset");
    return launch_nodes<float>(p->p32, 1.0, p->a32, p->x32, s);
  };
  NLA_TRY(solve32());
  m.op = bat::MAP_SET;
  bat::batched_map_kernel<<<p->ngroups, 256, 0, s>>>(m);
  NLA_CHECK_LAUNCH("batched_map_kernel");
  const bat::ResidualArgs r{descs, groups, A64, B64, p->r64, p->x32, p->tA, p->rev};
  if (sweeps > 0 && residual == NLA_RESIDUAL_SPLIT) NLA_TRY(exact_residual_setup(p));
  void* errp = nullptr;
  cudaError_t ee = cudaGetSymbolAddress(&errp, bat::g_batch_error);
  if (ee != cudaSuccess) return cuda_status(ee, "batch error word");
  const bat::ExactResArgs xr{descs,         groups,        static_cast<const bat::ExactTile*>(p->d_xtiles),
                             A64,           B64,           p->r64,
                             p->x32,        p->tA,         p->rev,
                             static_cast<int*>(errp), p->d_row_exp, p->d_row_base,
                             p->d_col_exp,  p->d_col_base};
  if (sweeps > 0 && residual == NLA_RESIDUAL_SPLIT && p->nbands > 0) {
    // Row exponents of A once: A does not change between sweeps.
    const bat::RowExpArgs re{descs, p->d_bands, p->d_row_base, A64, p->tA, p->rev, p->d_row_exp};
    bat::batched_row_exp_kernel<<<(unsigned)p->nbands, 256, 0, s>>>(re);
    NLA_CHECK_LAUNCH("batched_row_exp_kernel");
  }
  const bat::ColExpArgs ce{descs, groups, p->d_col_base, B64, p->rev, p->d_col_exp};
  for (int k = 0; k < sweeps; ++k) {
    if (residual == NLA_RESIDUAL_SPLIT) {
      if (p->nxtiles == 0) return fail(NLA_ERR_UNSUPPORTED, "mixed batch: no residual tiles");
      bat::batched_col_exp_kernel<<<(unsigned)p->ngroups, 256, 0, s>>>(ce);
      NLA_CHECK_LAUNCH("batched_col_exp_kernel");
      bat::batched_exact_residual_kernel<<<(unsigned)p->nxtiles, bat::XR_THREADS, bat::XR_SMEM, s>>>(xr);
      NLA_CHECK_LAUNCH("batched_exact_residual_kernel");
    } else {
      bat::batched_residual_kernel<<<dim3((unsigned)p->ngroups,
                                          (unsigned)((p->n_max + bat::MAX_ROWS - 1) / bat::MAX_ROWS)),
                                     bat::NT, 0, s>>>(r);
      NLA_CHECK_LAUNCH("batched_residual_kernel");
    }
    NLA_TRY(solve32());
    m.op = bat::MAP_ADD;
    bat::batched_map_kernel<<<p->ngroups, 256, 0, s>>>(m);
    NLA_CHECK_LAUNCH("batched_map_kernel");
  }
  return NLA_OK;
}

int nla_batch_plan_destroy(nla_batch_plan p) {
  clear_error();
  if (!p) return NLA_OK;
  if (p->p32) nla_batch_plan_destroy(p->p32);
  cudaFree(p->a32);
  cudaFree(p->x32);
  cudaFree(p->r64);
  cudaFree(p->d_xtiles);
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
  cudaFree(p->d_descs);
  cudaFree(p->d_groups);
  cudaFree(p->d_nodes);
  cudaFree(p->d_counters);
  delete p;
  return NLA_OK;
}

}  // extern "C"
