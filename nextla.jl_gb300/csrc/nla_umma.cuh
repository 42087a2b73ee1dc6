// Inline-PTX building blocks for sm_103a: mbarriers with bounded waits, TMA
// tensor loads, and the tcgen05 (5th-generation tensor core) instructions
// with their shared-memory and instruction descriptors.
#pragma once

#include <cuda.h>
#include <stdint.h>

namespace nla {
namespace umma {

// A bounded wait gives up after this many nanoseconds of %globaltimer.
constexpr uint64_t WAIT_LIMIT_NS = 2000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Limit of the waits that honour aborts (the pipeline waits between the
// roles of a CTA): WAIT_LIMIT_NS unless nla_set_wait_limit_ns changed it.
// The waits that drain a CTA's own in-flight work before it exits always use
// WAIT_LIMIT_NS.
static __device__ uint64_t g_wait_limit_ns = WAIT_LIMIT_NS;

// Wait for the phase with the given parity to complete.  Returns false (and
// raises *abort and the device error word) if the wait runs past the limit
// or another role of the CTA has aborted.  The timer is read every 256 polls,
// or on every poll when the limit is below a millisecond.
// With honor_abort false the wait ignores other roles' aborts (used to drain
// in-flight tensor-core work and TMA loads before the CTA exits).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort, int* err,
                                          int where, bool honor_abort = true) {
  if (mbar_try_wait(bar, parity)) return true;
  // Only a wait that did not complete at once reads the limit.
  const uint64_t limit = honor_abort ? g_wait_limit_ns : WAIT_LIMIT_NS;
  const uint32_t mask = limit < 1000000ull ? 0u : 255u;
  uint64_t t0 = 0;
  for (uint32_t it = 0;; ++it) {
    if (it > 0 && mbar_try_wait(bar, parity)) return true;
    if ((it & mask) == 0) {
      if (honor_abort && *abort) return false;
      const uint64_t now = globaltimer();
      if (it == 0) {
        t0 = now;
      } else if (now - t0 > limit) {
        *abort = 1;
        atomicCAS(err, 0, where);
        return false;
      }
    }
  }
}

// End of a TMA producer's loop: `issued` loads went to stage it % stages in
// round it / stages, each completing one phase of that stage's barrier in
// `own_full` (barriers this producer alone arrives on).  Waits, ignoring
// aborts and with the fixed limit, for the last phase of every stage used, so
// that none of its loads is still writing into this CTA's shared memory when
// the CTA exits (after an abort the consumer may have stopped reading them).
__device__ __forceinline__ void producer_quiesce(const uint64_t* own_full, int stages, int issued,
                                                 volatile int* abort, int* err, int where) {
  for (int s = 0; s < stages && s < issued; ++s) {
    const uint32_t last_round = (uint32_t)((issued - 1 - s) / stages);
    mbar_wait(smem_u32(&own_full[s]), last_round & 1u, abort, err, where, false);
  }
}

// 2-D tiled TMA load into shared memory, completing on an mbarrier.
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int32_t x,
                                            int32_t y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void prefetch_tmap(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// ---- tcgen05 ---------------------------------------------------------------

__device__ __forceinline__ void tmem_alloc(uint32_t slot_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot_smem), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// D[tmem] (+)= A[smem desc] * B[smem desc]^T, kind::f16 (BF16 or FP16 inputs,
// FP32 accumulate), issued by one thread.
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "setp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrive on an mbarrier once all previously issued tcgen05.mma of this thread
// have completed.
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

// 32 lanes x 16 consecutive 32-bit columns; thread t of the warp receives lane
// (quadrant base + t).  Waits for the load before returning.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
}

// 32 consecutive 32-bit TMEM columns of this thread's lane, one wait.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
}

// Shared-memory matrix descriptor for a K-major tile whose rows are 128 bytes
// (64 16-bit elements) written by TMA with 128-byte swizzling: 8-row groups
// are 1024 bytes apart (stride byte offset); the leading byte offset is not
// used by this layout.  The tile base must be 1024-byte aligned; the start
// address may be advanced by 32-byte steps along K inside the 128-byte row.
__device__ __forceinline__ uint64_t desc_kmajor_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address, bits 0-13
  d |= (uint64_t)1 << 16;                    // leading byte offset (16 B, unused)
  d |= (uint64_t)(1024 >> 4) << 32;          // stride byte offset, bits 32-45
  d |= (uint64_t)1 << 46;                    // descriptor version for sm_100 family
  d |= (uint64_t)2 << 61;                    // layout: 128-byte swizzle
  return d;
}

// Instruction descriptor for kind::f16: FP32 accumulator, A and B both BF16
// (bf16 = true) or both FP16, both K-major, shape M x N.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N, bool bf16) {
  return (1u << 4)                            // D format: F32
         | ((bf16 ? 1u : 0u) << 7)            // A format
         | ((bf16 ? 1u : 0u) << 10)           // B format
         | ((uint32_t)(N >> 3) << 17)         // N >> 3, bits 17-22
         | ((uint32_t)(M >> 4) << 24);        // M >> 4, bits 24-28
}

}  // namespace umma
}  // namespace nla
