// vsr_wait_selftest: the bounded mbarrier wait of the kernels, run against a
// barrier that nothing completes, so that its expiry path (error bit, clean
// return) can be tested without a fault or a hang.
#include "vsr_internal.cuh"

namespace vsr {
namespace {

__global__ void wait_selftest_kernel(uint64_t limit_ns, uint32_t* err_word, uint32_t* result) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);  // one arrival expected; none is ever made
  fence_mbar_init();
  const uint64_t t0 = global_timer_ns();
  const bool ok = mbar_wait_bounded(&bar, 0, err_word, kDevErrTmaTimeout, limit_ns);
  const uint64_t dt = global_timer_ns() - t0;
  result[0] = ok ? 0u : 1u;
  result[1] = dt > 0xffffffffull ? 0xffffffffu : static_cast<uint32_t>(dt);
}

}  // namespace
}  // namespace vsr

extern "C" int vsr_wait_selftest(uint64_t limit_ns, uint32_t* result, void* stream) {
  using namespace vsr;
  if (!result) return fail(VSR_ERR_INVALID_ARG, "result must not be NULL");
  if (limit_ns < 1000ull || limit_ns > kWaitLimitNs)
    return fail(VSR_ERR_INVALID_ARG, "limit_ns must be in [1e3, 2e9]");
  uint32_t* err = device_error_word();
  if (!err) return VSR_ERR_CUDA;
  wait_selftest_kernel<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(limit_ns, err, result);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}
