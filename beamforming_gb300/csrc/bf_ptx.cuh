// bf_ptx.cuh -- inline-PTX building blocks for the sm_103a kernels: mbarriers
// with bounded waits, TMA tensor copies, and the tcgen05 (5th-generation
// tensor core + tensor memory) instructions.
#pragma once

#include <cstdint>
#include <cuda.h>

namespace bf {

// Status codes a kernel writes into its error word (first failure wins).
enum DeviceError : int {
  kDevOk = 0,
  kDevTimeoutFull = 101,      // waiting for a TMA stage
  kDevTimeoutUnpacked = 102,  // waiting for an unpacked operand stage
  kDevTimeoutEmpty = 103,     // waiting for the tensor core to release a stage
  kDevTimeoutAccFull = 104,   // waiting for an accumulator
  kDevTimeoutAccEmpty = 105,  // waiting for the epilogue to drain an accumulator
  kDevBadLaunch = 110,        // launch geometry does not match the kernel's assumptions
};

// A wait gives up after this many nanoseconds of no progress and reports a
// timeout instead of spinning forever.
constexpr uint64_t kWaitTimeoutNs = 1500ull * 1000ull * 1000ull;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// ---------------------------------------------------------------- mbarrier
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// try_wait that lets the hardware suspend the thread until the phase completes
// or `hint_ns` nanoseconds pass, so waiting warps do not take issue slots.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint32_t bar, uint32_t parity, uint32_t hint_ns) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity), "r"(hint_ns)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase with the given parity to complete.  Returns false
// (after recording `code` in *err) when no progress was seen for
// kWaitTimeoutNs, or when another role of the kernel already failed.  The
// hardware ends a suspended try_wait long before the hint, so the error word
// and the clock are read only every kPollCheck polls: reading them on every
// poll took a fifth of the issue slots of the tensor-core kernel.
//
// The clock (%globaltimer) is not trusted alone: a wait expires only after
// kMinTimeoutPolls polls as well (milliseconds of polling; no wait of a working
// pipeline lasts that long), and a clock that steps back restarts the window.
// A time difference taken in unsigned arithmetic across a backward step would
// wrap to ~2^64 and end a healthy wait at once.
constexpr uint32_t kPollCheck = 16;
constexpr uint32_t kMinTimeoutPolls = 4096;
__device__ __forceinline__ bool wait_expired(uint64_t &t0, uint32_t polls) {
  const uint64_t now = globaltimer_ns();
  if (now < t0) {  // the clock stepped back: restart the window
    t0 = now;
    return false;
  }
  return polls >= kMinTimeoutPolls && now - t0 > kWaitTimeoutNs;
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int *err, int code) {
  if (mbar_try_wait(bar, parity)) return true;
  uint64_t t0 = globaltimer_ns();
  for (uint32_t i = 1;; ++i) {
    if (mbar_try_wait_sleep(bar, parity, 200000u)) return true;
    if (i % kPollCheck == 0) {
      if (*reinterpret_cast<volatile int *>(err) != 0) return false;
      if (wait_expired(t0, i)) {
        atomicCAS(err, 0, code);
        return false;
      }
    }
  }
}

// Bounded wait for the error path, which ignores the error word: a role that
// gives up waits with it for the copies it already issued to land before the
// CTA exits (at most kWaitTimeoutNs per barrier).
__device__ __forceinline__ bool mbar_wait_drain(uint32_t bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  uint64_t t0 = globaltimer_ns();
  for (uint32_t i = 1;; ++i) {
    if (mbar_try_wait_sleep(bar, parity, 200000u)) return true;
    if (i % kPollCheck == 0 && wait_expired(t0, i)) return false;
  }
}

// ---------------------------------------------------------------- proxies
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---------------------------------------------------------------- TMA
__device__ __forceinline__ void tma_prefetch_desc(const CUtensorMap *map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// Orders this thread's later tensor-map uses after the map's latest writes
// through the generic proxy (host copies into a problem table that is reused
// from launch to launch), so no stale copy of an earlier map is used.
__device__ __forceinline__ void tensormap_acquire(const CUtensorMap *map) {
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(reinterpret_cast<uint64_t>(map))
               : "memory");
}

__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}

__device__ __forceinline__ uint64_t policy_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, uint32_t bar, int c0, int c1, int c2,
                                            uint64_t policy) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.L2::cache_hint"
      " [%0], [%1, {%3, %4, %5}], [%2], %6;" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(c0), "r"(c1), "r"(c2), "l"(policy)
      : "memory");
}

// ---------------------------------------------------------------- tcgen05
__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, 8-bit float operands, f32 accumulate.
__device__ __forceinline__ void mma_f8f6f4(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                           uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// D[tmem] (+)= A[tmem] * B[smem]^T: the A operand (M rows = TMEM lanes, 4
// E4M3 values per 32-bit column) is read from tensor memory.
__device__ __forceinline__ void mma_f8f6f4_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t b_desc, uint32_t idesc,
                                              uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
      "r"(a_tmem), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// The eight MMAs of one K stage (two 128-byte W boxes, b0 and b1): K step kk
// reads TMEM columns a + 8 kk and box kk / 4 at byte 32 (kk % 4) of its rows
// (descriptor address field in 16 B units).  One asm block and one predicate:
// the issuing thread's instruction stream, not the tensor pipe, is the limit
// at N = 192, so it carries nothing else.
__device__ __forceinline__ void mma_ts_stage8(uint32_t d_tmem, uint32_t a_tmem, uint64_t b0, uint64_t b1,
                                              uint32_t idesc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t.reg .b64 b;\n\t.reg .b32 a;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], [%1], %2, %4, p;\n\t"
      "add.u32 a, %1, 8;\n\tadd.s64 b, %2, 2;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], [a], b, %4, p;\n\t"
      "add.u32 a, %1, 16;\n\tadd.s64 b, %2, 4;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], [a], b, %4, p;\n\t"
      "add.u32 a, %1, 24;\n\tadd.s64 b, %2, 6;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], [a], b, %4, p;\n\t"
      "add.u32 a, %1, 32;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], [a], %3, %4, p;\n\t"
      "add.u32 a, %1, 40;\n\tadd.s64 b, %3, 2;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], [a], b, %4, p;\n\t"
      "add.u32 a, %1, 48;\n\tadd.s64 b, %3, 4;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], [a], b, %4, p;\n\t"
      "add.u32 a, %1, 56;\n\tadd.s64 b, %3, 6;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], [a], b, %4, p;\n\t}" ::"r"(d_tmem),
      "r"(a_tmem), "l"(b0), "l"(b1), "r"(idesc)
      : "memory");
}

// 32 lanes x 32 consecutive 32-bit columns: thread i writes lane (base + i).
__device__ __forceinline__ void tmem_st_32x32b_x32(uint32_t taddr, const uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
      "{%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, "
      "%17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]),
      "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(r[16]), "r"(r[17]),
      "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]), "r"(r[24]), "r"(r[25]),
      "r"(r[26]), "r"(r[27]), "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31])
      : "memory");
}

__device__ __forceinline__ void tmem_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// Arrive once on an mbarrier when every tcgen05 operation this thread issued
// before has completed.
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 32 lanes x 16 consecutive 32-bit columns: thread i gets lane (base + i).
__device__ __forceinline__ void tmem_ld_32x32b_x16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
}

__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Waits for outstanding tcgen05.ld and ties the loaded registers to the wait,
// so no use of them can be scheduled before it.
__device__ __forceinline__ void tmem_ld_wait(uint32_t (&r)[16]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
               :
               : "memory");
}

// Shared-memory matrix descriptor for a K-major operand in the 128-byte
// swizzled layout: rows of 128 bytes, 8-row groups 1024 bytes apart.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((addr >> 4) & 0x3FFFu);        // start address
  d |= static_cast<uint64_t>(1u) << 16;                     // leading byte offset (unused for this layout)
  d |= static_cast<uint64_t>((1024u >> 4) & 0x3FFFu) << 32;  // stride byte offset: next 8-row group
  d |= static_cast<uint64_t>(1u) << 46;                     // descriptor version
  d |= static_cast<uint64_t>(2u) << 61;                     // 128-byte swizzle
  return d;
}

// Shared-memory matrix descriptor for a K-major operand whose rows are 32
// bytes in the 32-byte swizzle the TMA writes (8-row groups of 256 bytes).
__device__ __forceinline__ uint64_t smem_desc_sw32(uint32_t addr) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((addr >> 4) & 0x3FFFu);       // start address
  d |= static_cast<uint64_t>(1u) << 16;                    // leading byte offset (unused for this layout)
  d |= static_cast<uint64_t>((256u >> 4) & 0x3FFFu) << 32;  // stride byte offset: next 8-row group
  d |= static_cast<uint64_t>(1u) << 46;                    // descriptor version
  d |= static_cast<uint64_t>(6u) << 61;                    // 32-byte swizzle
  return d;
}

// Instruction descriptor: kind::f8f6f4, A = B = E4M3, D = F32, both K-major.
__host__ __device__ constexpr uint32_t idesc_e4m3_f32(uint32_t M, uint32_t N) {
  return (1u << 4)              // D format: F32
         | (0u << 7)            // A format: E4M3
         | (0u << 10)           // B format: E4M3
         | ((N >> 3) << 17)     // N / 8
         | ((M >> 4) << 24);    // M / 16
}

}  // namespace bf
