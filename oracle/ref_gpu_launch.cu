// Host launchers for the reference's own focal kernels (test infrastructure).
//
// Compiled by oracle/make_ref_gpu.py once per kernel with -DREF_<NAME>, each
// object including one kernel source string that the recipe extracted into
// the git-ignored oracle/_ref/ folder.  The launches use the reference's
// geometry: 16 x 16 thread blocks over a ceil-divided grid and its shared
// memory sizes (src/vibespatial/raster/algebra.py:1943-1958 and 2062-2083
// for the convolution, 2342-2383 slope/aspect, 2700-2760 hillshade,
// 3283-3311 focal statistics).  Every launcher takes device pointers, returns
// a cudaError_t as int and enqueues on ``stream``.
#include <cuda_runtime.h>

#include <cstdint>

namespace {
inline dim3 grid16(int width, int height) { return dim3((width + 15) / 16, (height + 15) / 16, 1); }
}  // namespace

#if defined(REF_CONVOLVE_NORMALIZED)
#include "convolve_normalized.cuh"

extern "C" int ref_convolve_normalized(const double* input, double* output, const double* weights,
                                       const unsigned char* nodata_mask, int width, int height, int kw, int kh,
                                       double nodata_val, void* stream) {
  const int pad_x = kw / 2, pad_y = kh / 2;
  const size_t smem = (static_cast<size_t>(16 + 2 * pad_y) * (16 + 2 * pad_x + 1) + static_cast<size_t>(kh) * kw) * 8 +
                      static_cast<size_t>(16 + 2 * pad_y) * (16 + 2 * pad_x);
  if (smem > 48 * 1024) return static_cast<int>(cudaErrorInvalidValue);  // the reference's default limit
  convolve_normalized<<<grid16(width, height), dim3(16, 16, 1), smem, static_cast<cudaStream_t>(stream)>>>(
      input, output, weights, nodata_mask, width, height, kw, kh, pad_x, pad_y, nodata_val);
  return static_cast<int>(cudaGetLastError());
}
#endif

#if defined(REF_SLOPE_ASPECT)
#include "slope_aspect.cuh"

extern "C" int ref_slope_aspect(const double* dem, double* slope, double* aspect, const unsigned char* nodata_mask,
                                int width, int height, double cell_x, double cell_y, double nodata_val,
                                void* stream) {
  slope_aspect<<<grid16(width, height), dim3(16, 16, 1), 0, static_cast<cudaStream_t>(stream)>>>(
      dem, slope, aspect, nodata_mask, width, height, cell_x, cell_y, nodata_val, slope ? 1 : 0, aspect ? 1 : 0);
  return static_cast<int>(cudaGetLastError());
}
#endif

#if defined(REF_HILLSHADE)
#include "hillshade.cuh"

extern "C" int ref_hillshade(const double* dem, unsigned char* out, const unsigned char* nodata_mask, int width,
                             int height, double cell_x, double cell_y, double z_factor, double zenith_rad,
                             double azimuth_rad, int nodata_out, void* stream) {
  const size_t smem = (16 + 2) * (16 + 2 + 1) * 8;
  hillshade<<<grid16(width, height), dim3(16, 16, 1), smem, static_cast<cudaStream_t>(stream)>>>(
      dem, out, nodata_mask, width, height, cell_x, cell_y, z_factor, zenith_rad, azimuth_rad, nodata_out);
  return static_cast<int>(cudaGetLastError());
}
#endif

#if defined(REF_FOCAL_STATS)
#include "focal_stats.cuh"

extern "C" int ref_focal_stats(const double* input, double* output, const unsigned char* nodata_mask, int width,
                               int height, int radius_x, int radius_y, int stat_type, double nodata_val,
                               void* stream) {
  focal_stats<<<grid16(width, height), dim3(16, 16, 1), 0, static_cast<cudaStream_t>(stream)>>>(
      input, output, nodata_mask, width, height, radius_x, radius_y, stat_type, nodata_val);
  return static_cast<int>(cudaGetLastError());
}
#endif
