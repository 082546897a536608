// Focal convolution, Gaussian and focal mean entry points.
#include "vsr_internal.cuh"

extern "C" size_t vsr_convolve_workspace_size(int kh, int kw, int precision) {
  (void)precision;
  if (kh <= 0 || kw <= 0) return 0;
  return (static_cast<size_t>(kh) * kw * 8 + 255) & ~size_t(255);
}

extern "C" int vsr_convolve(const void*, int, int64_t, int64_t, int64_t, const double*, int, int,
                            double, int, void*, int, int64_t, int, void*, size_t, void*) {
  return vsr::fail(VSR_ERR_UNSUPPORTED, "vsr_convolve not built yet");
}

extern "C" size_t vsr_gaussian_workspace_size(int kernel_size, int precision) {
  (void)precision;
  return (static_cast<size_t>(kernel_size > 0 ? kernel_size : 1) * 16 + 255) & ~size_t(255);
}

extern "C" int vsr_gaussian(const void*, int, int64_t, int64_t, int64_t, double, int, double, int,
                            void*, int, int64_t, int, void*, size_t, void*) {
  return vsr::fail(VSR_ERR_UNSUPPORTED, "vsr_gaussian not built yet");
}

extern "C" int vsr_focal_mean(const void*, int, int64_t, int64_t, int64_t, int, int, double, int,
                              void*, int, int64_t, void*) {
  return vsr::fail(VSR_ERR_UNSUPPORTED, "vsr_focal_mean not built yet");
}
