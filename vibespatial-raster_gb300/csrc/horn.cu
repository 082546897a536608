// Horn 3x3 terrain kernels: slope, aspect and hillshade fused into one pass.
//
// Replaces the reference's ``slope_aspect`` and ``hillshade`` NVRTC kernels
// (kernels/focal.py:173-283, 303-467) and the float64 up-cast / uint8 mask /
// down-cast passes of their launch glue (algebra.py:2257-2383, 2632-2775).
// The arithmetic is in horn_common.cuh.
//
// Two kernels:
//  * horn_f32_tma  -- float32 rasters with 16-byte aligned rows
//    (horn_tma.cuh; instantiated in horn_tma_all.cu / horn_tma_sub.cu).
//  * horn_generic  -- every other dtype / alignment: one thread per pixel,
//    clamped loads through L1.
#include <type_traits>

#include "horn_common.cuh"

namespace vsr {
namespace horn {

template <int WANT>
int launch_tma_want(int cfg, const CUtensorMap& map, const HornParams& P, float nd_in, float* slope, float* aspect,
                    uint8_t* hs, uint32_t* err, cudaStream_t st);

namespace {

struct PixelOut {
  float slope, aspect;
  uint8_t hs;
};

__device__ __forceinline__ PixelOut horn_pixel(float gx, float gy, const HornParams& P, bool want_s,
                                               bool want_a, bool want_h) {
  PixelOut o;
  const float p = gx * P.inv8cx;
  const float q = gy * P.inv8cy;
  const float s = fmaf(p, p, q * q);
  if (want_s) o.slope = slope_deg(s);
  if (want_a) o.aspect = aspect_deg(p, q);
  if (want_h) o.hs = hillshade_u8(p, q, s, P);
  return o;
}

template <typename T>
struct DiffType { using type = float; };
template <> struct DiffType<double> { using type = double; };
template <> struct DiffType<int32_t> { using type = double; };

template <typename O> __device__ __forceinline__ O nd_out(const HornParams& P);
template <> __device__ __forceinline__ float nd_out<float>(const HornParams& P) { return P.nd_out_f; }
template <> __device__ __forceinline__ double nd_out<double>(const HornParams& P) { return P.nd_out_d; }

template <typename T, typename O>
__global__ void __launch_bounds__(256) horn_generic(const T* __restrict__ src, const HornParams P,
                                                    const NodataTest<T> nd, O* __restrict__ slope,
                                                    O* __restrict__ aspect, uint8_t* __restrict__ hs) {
  using D = typename DiffType<T>::type;
  const int64_t x = static_cast<int64_t>(blockIdx.x) * 32 + threadIdx.x;
  const int64_t y = static_cast<int64_t>(blockIdx.y) * 8 + threadIdx.y;
  if (x >= P.width || y >= P.height) return;
  const int64_t band = blockIdx.z;
  src += band * P.in_band_stride;
  if (slope) slope += band * P.out_band_stride;
  if (aspect) aspect += band * P.out_band_stride;
  if (hs) hs += band * P.hs_band_stride;
  const MaskRule rule = mask_rule(P);
  D v[3][3];
  bool dil = false, ctr = false;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const int64_t yy = min(max(y + r - 1, int64_t(0)), P.height - 1);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int64_t xx = min(max(x + c - 1, int64_t(0)), P.width - 1);
      const T t = __ldg(src + yy * P.in_pitch + xx);
      const bool b = nd(t);
      dil |= b;
      if (r == 1 && c == 1) ctr = b;
      v[r][c] = static_cast<D>(t);
    }
  }
  float gx, gy;
  if constexpr (std::is_same<T, float>::value) {  // float differences may round (see grad_exact)
    gx = grad_exact(v[0][0], v[0][2], v[1][0], v[1][2], v[2][0], v[2][2]);
    gy = grad_exact(v[0][0], v[2][0], v[0][1], v[2][1], v[0][2], v[2][2]);
  } else {  // exact: small integers in float, wider types in double
    gx = static_cast<float>((v[0][2] - v[0][0]) + D(2) * (v[1][2] - v[1][0]) + (v[2][2] - v[2][0]));
    gy = static_cast<float>((v[2][0] - v[0][0]) + D(2) * (v[2][1] - v[0][1]) + (v[2][2] - v[0][2]));
  }
  const PixelOut o = horn_pixel(gx, gy, P, slope != nullptr, aspect != nullptr, hs != nullptr);
  const bool sa_nd = rule.sa_any && (rule.sa_center ? ctr : dil);
  if (slope) slope[y * P.out_pitch + x] = sa_nd ? nd_out<O>(P) : static_cast<O>(o.slope);
  if (aspect) aspect[y * P.out_pitch + x] = sa_nd ? nd_out<O>(P) : static_cast<O>(o.aspect);
  if (hs) hs[y * P.hs_pitch + x] = (rule.hs_any && dil) ? uint8_t(0) : o.hs;
}

template <typename T, typename O>
int launch_generic(const void* src, const HornParams& P, double ndv, void* slope, void* aspect,
                   uint8_t* hs, cudaStream_t st) {
  NodataTest<T> nd{P.nd_kind, static_cast<T>(ndv)};
  dim3 block(32, 8);
  dim3 grid(static_cast<unsigned>((P.width + 31) / 32), static_cast<unsigned>((P.height + 7) / 8),
            static_cast<unsigned>(P.bands));
  if (grid.y > 65535u) return fail(VSR_ERR_UNSUPPORTED, "raster height %lld too large for the generic Horn path", (long long)P.height);
  horn_generic<T, O><<<grid, block, 0, st>>>(static_cast<const T*>(src), P, nd, static_cast<O*>(slope),
                                             static_cast<O*>(aspect), hs);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}

template <typename O>
int dispatch_generic(int dtype, const void* src, const HornParams& P, double ndv, void* slope,
                     void* aspect, uint8_t* hs, cudaStream_t st) {
  switch (dtype) {
    case VSR_F32: return launch_generic<float, O>(src, P, ndv, slope, aspect, hs, st);
    case VSR_F64: return launch_generic<double, O>(src, P, ndv, slope, aspect, hs, st);
    case VSR_U8: return launch_generic<uint8_t, O>(src, P, ndv, slope, aspect, hs, st);
    case VSR_I16: return launch_generic<int16_t, O>(src, P, ndv, slope, aspect, hs, st);
    case VSR_U16: return launch_generic<uint16_t, O>(src, P, ndv, slope, aspect, hs, st);
    case VSR_I32: return launch_generic<int32_t, O>(src, P, ndv, slope, aspect, hs, st);
    default: return fail(VSR_ERR_INVALID_ARG, "unsupported dtype %d", dtype);
  }
}

// Launch configurations of the TMA kernel the autotuner chooses between:
// (output rows per tile, pipeline stages, threads per CTA, CTAs per SM the
// register budget is sized for); launch_tma_want in horn_tma.cuh maps an
// index to its template instance.
struct HornConfig {
  int th, stages, threads, minb;
};
constexpr HornConfig kHornConfigs[] = {{64, 2, 128, 4}, {48, 2, 128, 4}, {32, 2, 128, 4}, {32, 2, 128, 5},
                                       {64, 2, 256, 2}};
constexpr int kNumHornConfigs = sizeof(kHornConfigs) / sizeof(kHornConfigs[0]);

int launch_tma_config(int cfg, const void* src, const HornParams& P, float nd_in, float* slope, float* aspect,
                      uint8_t* hs, cudaStream_t st) {
  CUtensorMap map;
  const int th = kHornConfigs[(cfg >= 0 && cfg < kNumHornConfigs) ? cfg : 0].th;
  const int want = (slope ? kWantSlope : 0) | (aspect ? kWantAspect : 0) | (hs ? kWantHs : 0);
  // the partial output sets run the 64-row shape (horn_tma.cuh)
  const int box_h = (want == 7 ? th : 64) + 2;
  const uint64_t plane = P.bands > 1 ? static_cast<uint64_t>(P.in_band_stride)
                                     : static_cast<uint64_t>(P.in_pitch) * static_cast<uint64_t>(P.height);
  int rc = encode_tensor_map_3d(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, src, P.width, P.height, P.bands, P.in_pitch,
                                plane, kSW, static_cast<uint32_t>(box_h));
  if (rc) return rc;
  uint32_t* err = device_error_word();
  if (!err) return VSR_ERR_CUDA;
  switch (want) {
    case 1: return launch_tma_want<1>(cfg, map, P, nd_in, slope, aspect, hs, err, st);
    case 2: return launch_tma_want<2>(cfg, map, P, nd_in, slope, aspect, hs, err, st);
    case 3: return launch_tma_want<3>(cfg, map, P, nd_in, slope, aspect, hs, err, st);
    case 4: return launch_tma_want<4>(cfg, map, P, nd_in, slope, aspect, hs, err, st);
    case 5: return launch_tma_want<5>(cfg, map, P, nd_in, slope, aspect, hs, err, st);
    case 6: return launch_tma_want<6>(cfg, map, P, nd_in, slope, aspect, hs, err, st);
    default: return launch_tma_want<7>(cfg, map, P, nd_in, slope, aspect, hs, err, st);
  }
}

}  // namespace
}  // namespace horn

int horn_config_count() { return horn::kNumHornConfigs; }

}  // namespace vsr

extern "C" int vsr_horn_fused_bands(const void* dem, int dtype, int bands, int64_t band_stride, int64_t height,
                                    int64_t width, int64_t pitch, double cell_x, double cell_y, double nodata,
                                    int nodata_kind, uint32_t flags, void* slope, void* aspect, int out_dtype,
                                    int64_t out_band_stride, int64_t out_pitch, uint8_t* hillshade,
                                    int64_t hs_band_stride, int64_t hs_pitch, double z_factor, double zenith_rad,
                                    double azimuth_rad, void* stream) {
  using namespace vsr;
  using namespace vsr::horn;
  if (height < 0 || width < 0) return fail(VSR_ERR_INVALID_ARG, "negative raster size");
  if (bands < 1 || bands > 65535) return fail(VSR_ERR_INVALID_ARG, "bands must be in [1, 65535]");
  if (height == 0 || width == 0) return VSR_OK;
  if (!slope && !aspect && !hillshade) return VSR_OK;
  if (!dem) return fail(VSR_ERR_INVALID_ARG, "dem is NULL");
  if (dtype_size(dtype) == 0) return fail(VSR_ERR_INVALID_ARG, "unsupported dtype %d", dtype);
  if (pitch < width) return fail(VSR_ERR_INVALID_ARG, "pitch %lld < width %lld", (long long)pitch, (long long)width);
  if ((slope || aspect) && out_dtype != VSR_F32 && out_dtype != VSR_F64)
    return fail(VSR_ERR_INVALID_ARG, "slope/aspect out_dtype must be VSR_F32 or VSR_F64");
  if ((slope || aspect) && out_pitch < width) return fail(VSR_ERR_INVALID_ARG, "out_pitch < width");
  if (hillshade && hs_pitch < width) return fail(VSR_ERR_INVALID_ARG, "hs_pitch < width");
  if (bands > 1 && (band_stride < pitch * height || ((slope || aspect) && out_band_stride < out_pitch * height) ||
                    (hillshade && hs_band_stride < hs_pitch * height)))
    return fail(VSR_ERR_INVALID_ARG, "band strides smaller than one band");
  if (!(cell_x > 0.0) || !(cell_y > 0.0) || !std::isfinite(cell_x) || !std::isfinite(cell_y))
    return fail(VSR_ERR_INVALID_ARG, "cell sizes must be positive and finite");
  if (nodata_kind < VSR_NODATA_NONE || nodata_kind > VSR_NODATA_NAN)
    return fail(VSR_ERR_INVALID_ARG, "bad nodata_kind %d", nodata_kind);
  const size_t es = dtype_size(dtype);
  const size_t os = (out_dtype == VSR_F64) ? 8 : 4;
  if (!aligned(dem, es)) return fail(VSR_ERR_INVALID_ARG, "dem not aligned to its element size");
  if ((slope && !aligned(slope, os)) || (aspect && !aligned(aspect, os)))
    return fail(VSR_ERR_INVALID_ARG, "slope/aspect not aligned to the output element size");

  HornParams P{};
  P.height = height;
  P.width = width;
  P.in_pitch = pitch;
  P.out_pitch = out_pitch;
  P.hs_pitch = hs_pitch;
  P.bands = bands;
  P.in_band_stride = bands > 1 ? band_stride : 0;
  P.out_band_stride = bands > 1 ? out_band_stride : 0;
  P.hs_band_stride = bands > 1 ? hs_band_stride : 0;
  P.inv8cx = static_cast<float>(1.0 / (8.0 * cell_x));
  P.inv8cy = static_cast<float>(1.0 / (8.0 * cell_y));
  P.zf = static_cast<float>(z_factor);
  P.zf2 = static_cast<float>(z_factor * z_factor);
  P.cos_z = static_cast<float>(std::cos(zenith_rad));
  P.hs_a = static_cast<float>(std::sin(zenith_rad) * std::cos(azimuth_rad) * z_factor);
  P.hs_b = static_cast<float>(std::sin(zenith_rad) * std::sin(azimuth_rad) * z_factor);
  P.nd_out_f = static_cast<float>(nodata);
  P.nd_out_d = nodata;
  P.flags = flags;
  double ndv = 0.0;
  P.nd_kind = resolve_nodata(dtype, nodata, nodata_kind, &ndv);
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  const bool tma_ok = dtype == VSR_F32 && (!(slope || aspect) || out_dtype == VSR_F32) &&
                      aligned(dem, 16) && pitch % 4 == 0 && (!slope || aligned(slope, 16)) &&
                      (!aspect || aligned(aspect, 16)) && (!(slope || aspect) || out_pitch % 4 == 0) &&
                      (!hillshade || (aligned(hillshade, 4) && hs_pitch % 4 == 0)) &&
                      (bands == 1 || (band_stride % 4 == 0 && (!(slope || aspect) || out_band_stride % 4 == 0) &&
                                      (!hillshade || hs_band_stride % 4 == 0))) &&
                      width < (int64_t(1) << 31) && height < (int64_t(1) << 31);
  if (tma_ok)
    return launch_tma_config(tuning_get(VSR_OP_HORN), dem, P, static_cast<float>(ndv),
                             static_cast<float*>(slope), static_cast<float*>(aspect), hillshade, st);
  if ((slope || aspect) && out_dtype == VSR_F64)
    return dispatch_generic<double>(dtype, dem, P, ndv, slope, aspect, hillshade, st);
  return dispatch_generic<float>(dtype, dem, P, ndv, slope, aspect, hillshade, st);
}


extern "C" int vsr_horn_fused(const void* dem, int dtype, int64_t height, int64_t width, int64_t pitch,
                              double cell_x, double cell_y, double nodata, int nodata_kind, uint32_t flags,
                              void* slope, void* aspect, int out_dtype, int64_t out_pitch, uint8_t* hillshade,
                              int64_t hs_pitch, double z_factor, double zenith_rad, double azimuth_rad, void* stream) {
  return vsr_horn_fused_bands(dem, dtype, 1, 0, height, width, pitch, cell_x, cell_y, nodata, nodata_kind, flags,
                              slope, aspect, out_dtype, 0, out_pitch, hillshade, 0, hs_pitch, z_factor, zenith_rad,
                              azimuth_rad, stream);
}
