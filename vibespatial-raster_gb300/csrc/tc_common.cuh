// tcgen05 building blocks shared by the split-precision tensor-core kernels
// (conv_tc.cu: 2-D implicit GEMM; gauss_tc.cu: separable Gaussian line
// passes): shared-memory matrix descriptors, the BF16 and F16 MMAs with
// FP32 accumulation, commits, tensor-memory allocation and loads, and the
// bounded mbarrier wait that every role of those kernels uses.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "vsr_internal.cuh"

namespace vsr {
namespace tc {

constexpr int kMmaM = 128;  // MMA M: TMEM lanes of an accumulator
constexpr int kMmaN = 64;   // MMA N: accumulator columns

// --- tcgen05 / descriptor helpers (PTX ISA: tcgen05 family, sm_100a+) ---
// Shared-memory matrix descriptor: start address, leading byte offset,
// stride byte offset (all >> 4), version 1 (bits 46-47), no swizzle.

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major,
// M = kMmaM, N = kMmaN.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(kMmaN >> 3) << 17) |
                            (static_cast<uint32_t>(kMmaM >> 4) << 24);

// The same with A = B = F16 (the two operands of one MMA share a type).
constexpr uint32_t kIdescF16 = (1u << 4) | (static_cast<uint32_t>(kMmaN >> 3) << 17) |
                               (static_cast<uint32_t>(kMmaM >> 4) << 24);

// Shared-memory descriptors are passed as their two 32-bit halves: the low
// word holds the start address (>> 4) and the leading byte offset, so
// stepping an operand is one 32-bit add (addresses stay below 256 KB: the
// start field never carries); the high word (stride byte offset, version)
// is the same for every operand here.
__host__ __device__ constexpr uint32_t desc_lo(uint32_t saddr, uint32_t lbo) {
  return ((saddr & 0x3FFFFu) >> 4) | (((lbo & 0x3FFFFu) >> 4) << 16);
}
constexpr uint32_t kDescHi = (128u >> 4) | (1u << 14);  // SBO = 128 B, version 1 (bit 46)

// The MMA issue loop is latency-bound on one thread: keep it to a handful
// of instructions per MMA.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint32_t a_lo, uint32_t b_lo, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t.reg .b64 da, db;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "mov.b64 da, {%1, %5};\n\t"
      "mov.b64 db, {%2, %5};\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], da, db, %3, p;\n\t}"
      ::"r"(d_tmem), "r"(a_lo), "r"(b_lo), "r"(kIdesc), "r"(accumulate), "r"(kDescHi));
}

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint32_t a_lo, uint32_t b_lo, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t.reg .b64 da, db;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "mov.b64 da, {%1, %5};\n\t"
      "mov.b64 db, {%2, %5};\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], da, db, %3, p;\n\t}"
      ::"r"(d_tmem), "r"(a_lo), "r"(b_lo), "r"(kIdescF16), "r"(accumulate), "r"(kDescHi));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Bulk global -> shared copy completing on ``bar`` (16-byte aligned, size % 16 == 0).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Bounded wait that also gives up once another role has raised ``abort``.
__device__ __forceinline__ bool wait_or_abort(uint64_t* bar, uint32_t parity, volatile int* abort, uint32_t* err,
                                              uint32_t code, uint64_t limit_ns = kWaitLimitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_timer_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (*abort) return false;
    if (global_timer_ns() - t0 > limit_ns) {
      atomicOr(err, code);
      *abort = 1;
      return false;
    }
  }
  return true;
}


__device__ __forceinline__ uint32_t bf16x2_bits(__nv_bfloat162 v) {
  return static_cast<uint32_t>(__bfloat16_as_ushort(v.x)) | (static_cast<uint32_t>(__bfloat16_as_ushort(v.y)) << 16);
}

__device__ __forceinline__ uint32_t f16x2_bits(__half2 v) {
  return static_cast<uint32_t>(__half_as_ushort(__low2half(v))) |
         (static_cast<uint32_t>(__half_as_ushort(__high2half(v))) << 16);
}

// 16 consecutive f32 columns of this warp's 32 TMEM lanes, without the
// wait: issue several, then tmem_wait_ld16() on each before using it.
__device__ __forceinline__ void tmem_ld16_issue(uint32_t taddr, uint32_t r[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
// The wait, with the loaded registers as read-write operands so that no use
// of them is scheduled before it (the first call waits for every load issued;
// later calls return at once).
__device__ __forceinline__ void tmem_wait_ld16(uint32_t r[16]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                 "+r"(r[15])
               :
               : "memory");
}

// 16 consecutive f32 columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace vsr
