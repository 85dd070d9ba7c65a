// Thin inline-PTX wrappers for the 5th-generation tensor core (tcgen05),
// tensor memory (TMEM) and mbarriers on sm_100-family GPUs (sm_103a here).
//
// Operand tiles live in shared memory in the canonical K-major layout
// without swizzle: the tile is a grid of "core matrices" of 8 rows x 16
// bytes (each core matrix 128 contiguous bytes, row r at +16 r).  The shared
// memory descriptor gives the distance between core matrices that are
// adjacent along K (leading byte offset) and along M/N (stride byte
// offset).  The instruction descriptor selects the data types, both
// operands K-major, and the M x N shape; the accumulator D is FP32 in TMEM
// (row i of an M = 128 tile in TMEM lane i, column j in TMEM column j).
#pragma once
#include <stdint.h>

namespace lne {
namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared memory matrix descriptor (sm_100 form: version 1 in bits 46-47,
// layout type 0 = no swizzle in bits 61-63).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo_bytes, uint32_t sbo_bytes) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo_bytes >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo_bytes >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor for kind::tf32 with FP32 accumulation, A and B
// K-major, shape M x N.
__host__ __device__ __forceinline__ uint32_t idesc_tf32(int M, int N) {
  uint32_t d = 0;
  d |= 1u << 4;                        // D format: F32
  d |= 2u << 7;                        // A format: TF32
  d |= 2u << 10;                       // B format: TF32
  d |= (uint32_t)(N >> 3) << 17;       // N / 8
  d |= (uint32_t)(M >> 4) << 24;       // M / 16
  return d;
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// Arrive on an mbarrier once every tcgen05 operation this thread issued
// before has completed.
__device__ __forceinline__ void commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Generic-proxy shared memory writes become visible to the tensor core.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// TMEM allocation: one warp, `cols` a power of two >= 32; the base address
// is written to shared memory at `dst`.
__device__ __forceinline__ void tmem_alloc(uint32_t dst_saddr, uint32_t cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_saddr), "r"(cols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}

// 16 consecutive FP32 columns of the TMEM lane owned by this thread
// (warp w reads lanes 32 (w % 4) ..).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// The same load without its wait, so that several loads share one wait: the
// registers may be read only after tmem_wait_ld() and reg_fence16() on them.
__device__ __forceinline__ void tmem_ld16_issue(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
// Orders later uses of r after the preceding (volatile) wait.
__device__ __forceinline__ void reg_fence16(uint32_t (&r)[16]) {
  asm volatile(""
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                 "+r"(r[15]));
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Waits for the phase with the given parity to complete; gives up after
// `max_cycles` SM clock cycles (or within 64 polls of *abort being set) and
// returns false so that the caller can record the timeout.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, long long max_cycles,
                                          const volatile int* abort) {
  const long long t0 = clock64();
  for (uint32_t it = 0;; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred P1;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, P1;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
    // the abort flag is in global memory: look at it every 64 polls
    if (((it & 63u) == 63u && *abort != 0) || clock64() - t0 > max_cycles) return false;
  }
}

// Asynchronous 16-byte global -> shared copy (cp.async, L2 only); bytes of
// the source past `src_bytes` (0..16) are not read and land as zeros.  Both
// addresses 16-byte aligned.
__device__ __forceinline__ void cp_async16(uint32_t dst_saddr, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst_saddr), "l"(src), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// The mbarrier gets one arrival (counted in its expected count) once every
// cp.async this thread issued before has landed.
__device__ __forceinline__ void cp_async_mbar_arrive(uint32_t mbar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
// Arrive and add `bytes` to the transaction count the phase waits for.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes)
               : "memory");
}
// 2-D tiled TMA load of the box at (x, y) (x: innermost, in elements) into
// shared memory; completes `bytes` of the mbarrier's transaction count.
// Out-of-range elements land as zeros.
__device__ __forceinline__ void tma_load_2d(uint32_t dst_saddr, const void* tmap, int x, int y, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst_saddr),
      "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(mbar)
      : "memory");
}
// L2 prefetch of the 2-D box at (x, y) of a tensor map (no shared memory,
// no completion to wait for).
__device__ __forceinline__ void tma_prefetch_2d(const void* tmap, int x, int y) {
  asm volatile("cp.async.bulk.prefetch.tensor.2d.L2.global.tile [%0, {%1, %2}];" ::"l"(
                   reinterpret_cast<uint64_t>(tmap)),
               "r"(x), "r"(y)
               : "memory");
}
// Shared memory descriptor of a K-major operand in the 64-byte swizzle
// layout (what a TMA box with a 64-byte inner extent and SWIZZLE_64B
// writes): 8-row atoms of 64-byte rows, `sbo_bytes` between atoms.
__device__ __forceinline__ uint64_t smem_desc_sw64(uint32_t saddr, uint32_t sbo_bytes) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;  // leading byte offset: unused within one swizzle atom
  d |= (uint64_t)((sbo_bytes >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)4 << 61;  // layout: 64-byte swizzle
  return d;
}
__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}
// Waits until at most N of this thread's committed copy groups are pending.
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// FP32 -> TF32 (round to nearest, ties away), as a float bit pattern.
__device__ __forceinline__ float to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// Byte offset of element (row, k) in a K-major no-swizzle tile whose rows
// hold `kc` 4-byte elements: core matrix (row/8, k/4) at ((row/8)(kc/4) +
// k/4) * 128, row within it at 16 (row % 8), element at 4 (k % 4).
__device__ __forceinline__ uint32_t kmajor_off(uint32_t row, uint32_t k, uint32_t kc) {
  return (((row >> 3) * (kc >> 2) + (k >> 2)) << 7) + ((row & 7u) << 4) + ((k & 3u) << 2);
}

}  // namespace tc
}  // namespace lne
