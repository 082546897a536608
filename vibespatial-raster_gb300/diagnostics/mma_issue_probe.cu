// Diagnostic: cycles per tcgen05.mma (kind::f16, BF16 x BF16 -> FP32, M=128,
// K=16) for N = 16..256, operands resident in shared memory.  One thread per
// CTA issues a chain of MMAs into one accumulator; CTA 0 reports clock64
// cycles per MMA.  Standalone program, not part of libvsr:
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o mma_issue_probe mma_issue_probe.cu
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdio>
#include <cstdint>

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint64_t desc(uint32_t a, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((a & 0x3FFFFu) >> 4) | ((uint64_t)((lbo & 0x3FFFFu) >> 4) << 16) | ((uint64_t)((sbo & 0x3FFFFu) >> 4) << 32) | (1ull << 46);
}
template <int N>
__global__ void __launch_bounds__(128, 1) probe(int iters, float* out, unsigned long long* cyc) {
  extern __shared__ __align__(1024) unsigned char sm[];  // A: 128x16 bf16 (4 KB), B: 256x16 bf16 (8 KB)
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t slot;
  for (int i = threadIdx.x; i < (12 * 1024) / 4; i += 128) reinterpret_cast<uint32_t*>(sm)[i] = 0x3f803f80u;  // bf16 1.0
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&slot)), "r"(256));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&bar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("fence.proxy.async.shared::cta;");
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = slot;
  const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
  const uint32_t base = su32(sm);
  // A: 16 M-groups x 2 K-chunks, M-groups contiguous (SBO 128), K-chunks 2 KB apart (LBO 2048)
  const uint64_t ad = desc(base, 2048, 128);
  // B: N/8 groups x 2 K-chunks at base+4096: SBO 128, LBO N*16
  const uint64_t bd = desc(base + 4096, N * 16, 128);
  unsigned long long t0 = 0, t1 = 0;
  bool ok = true;
  if (threadIdx.x == 0) {
    t0 = clock64();
    for (int i = 0; i < iters; ++i) {
      asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                   ::"r"(tmem), "l"(ad), "l"(bd), "r"(idesc), "r"(i));
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(&bar)) : "memory");
    uint32_t done = 0;
    const unsigned long long lim = clock64() + 4000000000ull;
    while (!done) {
      asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\tselp.u32 %0, 1, 0, p;\n\t}" : "=r"(done) : "r"(su32(&bar)) : "memory");
      if (clock64() > lim) { ok = false; break; }
    }
    t1 = clock64();
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (threadIdx.x < 32) {
    uint32_t r;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];" : "=r"(r) : "r"(tmem));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
    if (threadIdx.x == 0) { out[blockIdx.x] = __uint_as_float(r); cyc[blockIdx.x] = ok ? (t1 - t0) : 0ull; }
  }
  __syncthreads();
  if (threadIdx.x < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256));
}
template <int N> void run(int iters) {
  float* out; unsigned long long* cyc;
  cudaMalloc(&out, 152 * 4); cudaMalloc(&cyc, 152 * 8);
  cudaFuncSetAttribute(probe<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, 13 * 1024);
  probe<N><<<152, 128, 13 * 1024>>>(16, out, cyc);
  cudaEvent_t a, b; cudaEventCreate(&a); cudaEventCreate(&b);
  cudaEventRecord(a);
  probe<N><<<152, 128, 13 * 1024>>>(iters, out, cyc);
  cudaEventRecord(b); cudaEventSynchronize(b);
  float ms; cudaEventElapsedTime(&ms, a, b);
  unsigned long long c[152]; float o[152];
  cudaMemcpy(c, cyc, sizeof(c), cudaMemcpyDeviceToHost); cudaMemcpy(o, out, sizeof(o), cudaMemcpyDeviceToHost);
  printf("N=%3d iters=%d: %.3f ms, %.1f cycles/MMA (clock64 of CTA0), acc[0]=%g, err=%s, TFLOP/s=%.1f\n", N, iters, ms,
         (double)c[0] / iters, o[0], cudaGetErrorString(cudaGetLastError()), 2.0 * 128 * N * 16 * (double)iters * 152 / (ms * 1e-3) / 1e12);
  cudaFree(out); cudaFree(cyc);
}
int main() { run<16>(20000); run<32>(20000); run<64>(20000); run<128>(20000); run<256>(20000); return 0; }
