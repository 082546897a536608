// Internal helpers shared by the libvsr translation units: error reporting,
// element-type traits, nodata tests, mbarrier / TMA wrappers with bounded
// waits, and tensor-map encoding through the driver entry point.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstdio>
#include <string>

#include "vsr.h"

namespace vsr {

// ---------------------------------------------------------------- errors --
void set_error(const char* fmt, ...);
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);

#define VSR_CUDA_TRY(expr)                                   \
  do {                                                       \
    cudaError_t _e = (expr);                                 \
    if (_e != cudaSuccess) return ::vsr::cuda_fail(_e, #expr); \
  } while (0)

// Device-side error word.  Kernels OR a code into it when a bounded wait
// runs out; the host reads it with vsr_poll_device_error.  The word is a
// file-scope __device__ variable of vsr_api.cu; kernels receive its device
// address (device_error_word(), resolved once per device) as a parameter.
enum DeviceError : uint32_t {
  kDevErrTmaTimeout = VSR_DEVERR_TMA_TIMEOUT,
  kDevErrMmaTimeout = VSR_DEVERR_MMA_TIMEOUT,
  kDevErrQueue = VSR_DEVERR_QUEUE,
  kDevErrPlan = VSR_DEVERR_PLAN,  // a batch launch whose shape differs from its plan's
};
uint32_t* device_error_word();  // nullptr (and error set) on failure

// Wall-clock bound for every spin-wait in a kernel (nanoseconds).
constexpr uint64_t kWaitLimitNs = 2000000000ull;

int sm_count();  // cached per device

// Launch-configuration table chosen by the autotuner (vsr_tuning_set).
int tuning_get(int op);
int horn_config_count();
int batch_config_count();

// ----------------------------------------------------------- dtype traits --
inline size_t dtype_size(int dt) {
  switch (dt) {
    case VSR_U8: return 1;
    case VSR_I16:
    case VSR_U16: return 2;
    case VSR_I32:
    case VSR_F32: return 4;
    case VSR_F64: return 8;
    default: return 0;
  }
}

// Decide how a nodata value is tested in the element type itself.  A value
// that the element type cannot hold exactly never matches any pixel (the
// reference compares the float64 up-cast against float(nodata)), so the
// kind degrades to NONE.  Returns the kind to use.
int resolve_nodata(int dtype, double nodata, int kind, double* as_elem);

template <typename T>
struct NodataTest {
  int kind;  // VSR_NODATA_*
  T value;
  __device__ __forceinline__ bool operator()(T v) const {
    if (kind == VSR_NODATA_VALUE) return v == value;
    if (kind == VSR_NODATA_NAN) return v != v;  // only floats reach here
    return false;
  }
};

// ------------------------------------------------------- device helpers --
__device__ __forceinline__ uint64_t global_timer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait on an mbarrier phase.  Returns false (and ORs ``code`` into
// *err_word) if the phase did not complete within ``limit_ns`` (default
// kWaitLimitNs).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t* err_word,
                                                  uint32_t code, uint64_t limit_ns = kWaitLimitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_timer_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (global_timer_ns() - t0 > limit_ns) {
      atomicOr(err_word, code);
      return false;
    }
  }
  return true;
}

// cp.async (LDGSTS): global -> shared copies that complete per thread
// (commit_group / wait_group); the copying thread sees the data after its
// wait, other threads after a barrier.
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
// 8 bytes, both addresses 8-byte aligned.
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
// 16 bytes, both addresses 16-byte aligned (cached in L2 only).
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
// BYTES (4 or 8) of which the first ``src_bytes`` are read, the rest zero-filled.
template <int BYTES>
__device__ __forceinline__ void cp_async_zfill(void* dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(smem_u32(dst)), "l"(src), "n"(BYTES),
               "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// 2-D tiled TMA load of box (x, y) into shared memory, completing on ``bar``.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// 3-D tiled TMA load of box (x, y, z) into shared memory, completing on ``bar``.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// 2-D tiled TMA store of box (x, y) from shared memory, tracked by the
// thread's bulk async-groups (bulk_commit / bulk_wait_read).  x * element
// size must be a multiple of 16 bytes; the box is clipped at the tensor edge.
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int x, int y, const void* src) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(x), "r"(y), "r"(smem_u32(src))
               : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// Wait until at most N of this thread's committed bulk groups still read
// their shared-memory source.
template <int N>
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}

// Until this thread's committed bulk groups have completed (their writes done).
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Bulk shared -> global copy in this thread's bulk async-group (both
// addresses 16-byte aligned, size a multiple of 16).
__device__ __forceinline__ void bulk_s2g(void* gdst, const void* ssrc, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(reinterpret_cast<uint64_t>(gdst)),
               "r"(smem_u32(ssrc)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// ------------------------------------------------------------ host side --
// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// dependency on libcuda).
int encode_tensor_map_2d(CUtensorMap* map, CUtensorMapDataType type, size_t elem_bytes,
                         const void* base, uint64_t width, uint64_t height, uint64_t pitch_elems,
                         uint32_t box_w, uint32_t box_h);

// 3-D map (x = width, y = height, z = depth planes ``plane_elems`` apart)
// with a box_w x box_h x 1 box.
int encode_tensor_map_3d(CUtensorMap* map, CUtensorMapDataType type, size_t elem_bytes, const void* base,
                         uint64_t width, uint64_t height, uint64_t depth, uint64_t pitch_elems, uint64_t plane_elems,
                         uint32_t box_w, uint32_t box_h);

inline bool aligned(const void* p, size_t a) {
  return (reinterpret_cast<uintptr_t>(p) % a) == 0;
}

}  // namespace vsr
