// Focal statistics other than the mean: min, max, range, std and variety
// (the mean is focal.cu's exact box kernels).
//
// Semantics are the reference CPU functions' (algebra.py:3041-3164, run per
// window by scipy generic_filter with out-of-bounds taps set to the
// placeholder, :3150-3163) rather than its GPU kernel's (kernels/focal.py:
// 666-770, which caps variety at 49 distinct values and does not propagate
// NaN):
//   min / max  nodata taps become +inf / -inf and every tap equal to that
//              placeholder is excluded (valid +-inf data too); a NaN tap
//              makes the result NaN;
//   range      max - min of the valid taps (nodata and NaN excluded);
//   std        population standard deviation of the valid taps; 0.0 for an
//              empty window;
//   variety    number of distinct valid values; 0 for an empty window.
// An empty window gives the raster's nodata value (0.0 when it has none), a
// nodata centre gives the nodata value.
//
// A CTA owns a 64 x 16 output tile and stages its (16 + 2ry) x (64 + 2rx)
// input window into shared memory, converted once to the statistic's type
// (float for 8/16-bit and float32 rasters, double for int32 / float64,
// int32 for the integer std), nodata and out-of-bounds taps already replaced
// by the statistic's placeholder.  min / max / range are separable: a row
// pass reduces each staged row to 64 window rows in shared memory, the
// column pass reduces 2ry+1 of those.  std and variety run over the staged
// window per pixel: std as exact int64 sums for 8/16-bit rasters
// (var = (n sum x^2 - (sum x)^2) / n^2) and two passes in float64 otherwise;
// variety counts the taps with no equal earlier tap.  Bands are blockIdx.z.
#include <cfloat>
#include <cmath>
#include <type_traits>

#include "vsr_internal.cuh"

namespace vsr {
namespace {

constexpr int kFsTX = 64, kFsTY = 16, kFsThreads = 256;
constexpr int kFsMaxRadius = 31;        // window up to 63 x 63
constexpr int kFsMaxVarietyRadius = 7;  // window up to 15 x 15 (225 taps)

struct FsArgs {
  const void* src;
  int dtype;
  int64_t H, W, pitch, band_stride;
  int kind;     // resolved VSR_NODATA_*
  double ndv;   // nodata in the element type (exact)
  int ry, rx;
  double nd_out;  // written for nodata centres and empty windows
  void* dst;
  int out_dtype;
  int64_t out_pitch, out_band_stride;
};

template <typename T>
__device__ __forceinline__ T pos_inf();
template <>
__device__ __forceinline__ float pos_inf<float>() { return __int_as_float(0x7f800000); }
template <>
__device__ __forceinline__ double pos_inf<double>() { return __longlong_as_double(0x7ff0000000000000ll); }
template <typename T>
__device__ __forceinline__ T qnan();
template <>
__device__ __forceinline__ float qnan<float>() { return __int_as_float(0x7fffffff); }
template <>
__device__ __forceinline__ double qnan<double>() { return __longlong_as_double(0x7ff8000000000000ll); }

// NaN-propagating min / max.
__device__ __forceinline__ float min_nan(float a, float b) {
  float r;
  asm("min.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float max_nan(float a, float b) {
  float r;
  asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ double min_nan(double a, double b) { return (a != a || b != b) ? a + b : fmin(a, b); }
__device__ __forceinline__ double max_nan(double a, double b) { return (a != a || b != b) ? a + b : fmax(a, b); }

// Element (band b, index idx) as double, with its nodata test.
__device__ __forceinline__ double fs_load(const FsArgs& a, const char* base, int64_t idx, bool& nodata) {
  double v;
  switch (a.dtype) {
    case VSR_U8: v = __ldg(reinterpret_cast<const uint8_t*>(base) + idx); break;
    case VSR_I16: v = __ldg(reinterpret_cast<const int16_t*>(base) + idx); break;
    case VSR_U16: v = __ldg(reinterpret_cast<const uint16_t*>(base) + idx); break;
    case VSR_I32: v = __ldg(reinterpret_cast<const int32_t*>(base) + idx); break;
    case VSR_F32: v = __ldg(reinterpret_cast<const float*>(base) + idx); break;
    default: v = __ldg(reinterpret_cast<const double*>(base) + idx); break;
  }
  nodata = a.kind == VSR_NODATA_VALUE ? v == a.ndv : (a.kind == VSR_NODATA_NAN ? v != v : false);
  return v;
}

__device__ __forceinline__ int elem_bytes(int dt) {
  return dt == VSR_U8 ? 1 : (dt == VSR_I16 || dt == VSR_U16) ? 2 : (dt == VSR_F64 ? 8 : 4);
}

__device__ __forceinline__ void fs_store(const FsArgs& a, char* obase, int64_t idx, double v) {
  if (a.out_dtype == VSR_F64) reinterpret_cast<double*>(obase)[idx] = v;
  else reinterpret_cast<float*>(obase)[idx] = static_cast<float>(v);
}

// Staged value of one tap for statistic S (placeholder for nodata and
// out-of-bounds taps).
template <typename T, int S>
__device__ __forceinline__ T staged(bool inb, bool nodata, double v) {
  if constexpr (std::is_same<T, int32_t>::value) {
    return (!inb || nodata) ? INT32_MIN : static_cast<int32_t>(v);  // 8/16-bit std
  } else if constexpr (S == VSR_STAT_MIN) {
    return (!inb || nodata) ? pos_inf<T>() : static_cast<T>(v);
  } else if constexpr (S == VSR_STAT_MAX) {
    return (!inb || nodata) ? -pos_inf<T>() : static_cast<T>(v);
  } else {
    return (!inb || nodata) ? qnan<T>() : static_cast<T>(v);  // NaN data stays NaN = excluded
  }
}

template <typename T, int S>
__global__ void __launch_bounds__(kFsThreads) focal_stat_kernel(const FsArgs a) {
  extern __shared__ __align__(16) unsigned char fs_smem[];
  const int SW = kFsTX + 2 * a.rx, SH = kFsTY + 2 * a.ry;
  T* St = reinterpret_cast<T*>(fs_smem);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t x0 = static_cast<int64_t>(blockIdx.x) * kFsTX, y0 = static_cast<int64_t>(blockIdx.y) * kFsTY;
  const char* base = static_cast<const char*>(a.src) + static_cast<int64_t>(blockIdx.z) * a.band_stride * elem_bytes(a.dtype);
  char* obase = static_cast<char*>(a.dst) +
                static_cast<int64_t>(blockIdx.z) * a.out_band_stride * (a.out_dtype == VSR_F64 ? 8 : 4);

  for (int r = warp; r < SH; r += kFsThreads / 32) {
    const int64_t gy = y0 - a.ry + r;
    const bool row_in = gy >= 0 && gy < a.H;
    for (int c = lane; c < SW; c += 32) {
      const int64_t gx = x0 - a.rx + c;
      const bool inb = row_in && gx >= 0 && gx < a.W;
      bool nd = false;
      double v = 0.0;
      if (inb) v = fs_load(a, base, gy * a.pitch + gx, nd);
      St[r * SW + c] = staged<T, S>(inb, nd, v);
    }
  }
  __syncthreads();

  if constexpr (S == VSR_STAT_MIN || S == VSR_STAT_MAX || S == VSR_STAT_RANGE) {
    // Row pass: R0 (min / max / low) and R1 (range high), SH x 64.
    T* R0 = St + SH * SW;
    T* R1 = R0 + SH * kFsTX;
    const int kw = 2 * a.rx + 1;
    for (int r = warp; r < SH; r += kFsThreads / 32) {
      const T* row = St + r * SW;
      for (int c = lane; c < kFsTX; c += 32) {
        T m0 = row[c], m1 = row[c];
        for (int d = 1; d < kw; ++d) {
          const T v = row[c + d];
          if constexpr (S == VSR_STAT_MIN) m0 = min_nan(m0, v);
          else if constexpr (S == VSR_STAT_MAX) m0 = max_nan(m0, v);
          else { m0 = fmin(m0, v); m1 = fmax(m1, v); }  // NaN (excluded) ignored
        }
        R0[r * kFsTX + c] = m0;
        if constexpr (S == VSR_STAT_RANGE) R1[r * kFsTX + c] = m1;
      }
    }
    __syncthreads();
    const int kh = 2 * a.ry + 1;
    for (int r = warp; r < kFsTY; r += kFsThreads / 32) {
      const int64_t y = y0 + r;
      if (y >= a.H) break;
      for (int c = lane; c < kFsTX; c += 32) {
        const int64_t x = x0 + c;
        if (x >= a.W) continue;
        T m0 = R0[r * kFsTX + c], m1 = m0;
        if constexpr (S == VSR_STAT_RANGE) m1 = R1[r * kFsTX + c];
        for (int d = 1; d < kh; ++d) {
          if constexpr (S == VSR_STAT_MIN) m0 = min_nan(m0, R0[(r + d) * kFsTX + c]);
          else if constexpr (S == VSR_STAT_MAX) m0 = max_nan(m0, R0[(r + d) * kFsTX + c]);
          else { m0 = fmin(m0, R0[(r + d) * kFsTX + c]); m1 = fmax(m1, R1[(r + d) * kFsTX + c]); }
        }
        double out;
        if constexpr (S == VSR_STAT_MIN) out = (m0 == pos_inf<T>()) ? a.nd_out : static_cast<double>(m0);
        else if constexpr (S == VSR_STAT_MAX) out = (m0 == -pos_inf<T>()) ? a.nd_out : static_cast<double>(m0);
        else out = (m0 != m0) ? a.nd_out : static_cast<double>(m1) - static_cast<double>(m0);
        bool nd = false;
        fs_load(a, base, y * a.pitch + x, nd);
        fs_store(a, obase, y * a.out_pitch + x, nd ? a.nd_out : out);
      }
    }
  } else {
    const int kh = 2 * a.ry + 1, kw = 2 * a.rx + 1;
    for (int r = warp; r < kFsTY; r += kFsThreads / 32) {
      const int64_t y = y0 + r;
      if (y >= a.H) break;
      for (int c = lane; c < kFsTX; c += 32) {
        const int64_t x = x0 + c;
        if (x >= a.W) continue;
        const T* win = St + r * SW + c;
        double out;
        if constexpr (S == VSR_STAT_STD && std::is_same<T, int32_t>::value) {
          int64_t s = 0, q = 0;
          int n = 0;
          for (int dy = 0; dy < kh; ++dy)
            for (int dx = 0; dx < kw; ++dx) {
              const int32_t v = win[dy * SW + dx];
              if (v == INT32_MIN) continue;
              s += v;
              q += static_cast<int64_t>(v) * v;
              ++n;
            }
          out = n ? sqrt(static_cast<double>(static_cast<int64_t>(n) * q - s * s)) / n : 0.0;
        } else if constexpr (S == VSR_STAT_STD) {
          double s = 0.0;
          int n = 0;
          for (int dy = 0; dy < kh; ++dy)
            for (int dx = 0; dx < kw; ++dx) {
              const double v = win[dy * SW + dx];
              if (v != v) continue;
              s += v;
              ++n;
            }
          double m2 = 0.0;
          if (n) {
            const double mean = s / n;
            for (int dy = 0; dy < kh; ++dy)
              for (int dx = 0; dx < kw; ++dx) {
                const double v = win[dy * SW + dx];
                if (v != v) continue;
                const double d = v - mean;
                m2 = fma(d, d, m2);
              }
          }
          out = n ? sqrt(m2 / n) : 0.0;
        } else {  // variety
          int cnt = 0;
          for (int iy = 0; iy < kh; ++iy)
            for (int ix = 0; ix < kw; ++ix) {
              const T v = win[iy * SW + ix];
              if (v != v) continue;
              bool dup = false;
              for (int jy = 0; jy <= iy && !dup; ++jy) {
                const int jend = jy < iy ? kw : ix;
                for (int jx = 0; jx < jend; ++jx)
                  if (win[jy * SW + jx] == v) { dup = true; break; }
              }
              cnt += !dup;
            }
          out = cnt;
        }
        bool nd = false;
        fs_load(a, base, y * a.pitch + x, nd);
        fs_store(a, obase, y * a.out_pitch + x, nd ? a.nd_out : out);
      }
    }
  }
}

template <typename T, int S>
size_t fs_smem(int ry, int rx) {
  const size_t SW = kFsTX + 2 * rx, SH = kFsTY + 2 * ry;
  size_t b = SW * SH * sizeof(T);
  if (S == VSR_STAT_MIN || S == VSR_STAT_MAX) b += SH * kFsTX * sizeof(T);
  if (S == VSR_STAT_RANGE) b += 2 * SH * kFsTX * sizeof(T);
  return b;
}

template <typename T, int S>
int fs_launch(const FsArgs& a, int bands, cudaStream_t st) {
  const size_t smem = fs_smem<T, S>(a.ry, a.rx);
  auto kern = focal_stat_kernel<T, S>;
  VSR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  const dim3 grid(static_cast<unsigned>((a.W + kFsTX - 1) / kFsTX), static_cast<unsigned>((a.H + kFsTY - 1) / kFsTY),
                  static_cast<unsigned>(bands));
  kern<<<grid, kFsThreads, smem, st>>>(a);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}

template <int S>
int fs_dispatch(const FsArgs& a, int bands, cudaStream_t st) {
  const bool wide = a.dtype == VSR_I32 || a.dtype == VSR_F64;
  if constexpr (S == VSR_STAT_STD) {
    if (a.dtype == VSR_U8 || a.dtype == VSR_I16 || a.dtype == VSR_U16) return fs_launch<int32_t, S>(a, bands, st);
    return fs_launch<double, S>(a, bands, st);
  }
  return wide ? fs_launch<double, S>(a, bands, st) : fs_launch<float, S>(a, bands, st);
}

}  // namespace

int focal_mean_bands_impl(const void* src, int dtype, int bands, int64_t band_stride, int64_t height, int64_t width,
                          int64_t pitch, int radius_y, int radius_x, double nodata, int nodata_kind, void* dst,
                          int out_dtype, int64_t out_band_stride, int64_t out_pitch, void* stream);  // focal.cu

}  // namespace vsr

using namespace vsr;

extern "C" int vsr_focal_stat_bands(const void* src, int dtype, int bands, int64_t band_stride, int64_t height,
                                    int64_t width, int64_t pitch, int stat, int radius_y, int radius_x,
                                    double nodata, int nodata_kind, void* dst, int out_dtype,
                                    int64_t out_band_stride, int64_t out_pitch, void* stream) {
  if (stat == VSR_STAT_MEAN)
    return focal_mean_bands_impl(src, dtype, bands, band_stride, height, width, pitch, radius_y, radius_x, nodata,
                                 nodata_kind, dst, out_dtype, out_band_stride, out_pitch, stream);
  if (stat < VSR_STAT_MIN || stat > VSR_STAT_VARIETY) return fail(VSR_ERR_INVALID_ARG, "unknown focal statistic %d", stat);
  if (bands < 1 || bands > 65535) return fail(VSR_ERR_INVALID_ARG, "bands must be in [1, 65535]");
  if (height < 0 || width < 0) return fail(VSR_ERR_INVALID_ARG, "negative raster size");
  if (height == 0 || width == 0) return VSR_OK;
  if (!src || !dst) return fail(VSR_ERR_INVALID_ARG, "src/dst must not be NULL");
  if (dtype_size(dtype) == 0) return fail(VSR_ERR_INVALID_ARG, "unsupported dtype %d", dtype);
  if (out_dtype != VSR_F32 && out_dtype != VSR_F64) return fail(VSR_ERR_INVALID_ARG, "out_dtype must be VSR_F32 or VSR_F64");
  if (pitch < width || out_pitch < width) return fail(VSR_ERR_INVALID_ARG, "pitch smaller than width");
  if (bands > 1 && (band_stride < pitch * height || out_band_stride < out_pitch * height))
    return fail(VSR_ERR_INVALID_ARG, "band strides smaller than one band");
  if (!aligned(src, dtype_size(dtype)) || !aligned(dst, out_dtype == VSR_F64 ? 8 : 4))
    return fail(VSR_ERR_INVALID_ARG, "src/dst not aligned to their element size");
  if (radius_y < 0 || radius_x < 0) return fail(VSR_ERR_INVALID_ARG, "radius must be non-negative");
  const int rmax = stat == VSR_STAT_VARIETY ? kFsMaxVarietyRadius : kFsMaxRadius;
  if (radius_y > rmax || radius_x > rmax)
    return fail(VSR_ERR_UNSUPPORTED, "focal statistic %d supports radii up to %d", stat, rmax);
  if ((height + kFsTY - 1) / kFsTY > 65535) return fail(VSR_ERR_UNSUPPORTED, "raster taller than %d rows", 65535 * kFsTY);

  FsArgs a{};
  a.src = src;
  a.dtype = dtype;
  a.H = height;
  a.W = width;
  a.pitch = pitch;
  a.band_stride = band_stride;
  a.kind = resolve_nodata(dtype, nodata, nodata_kind, &a.ndv);
  a.ry = radius_y;
  a.rx = radius_x;
  a.nd_out = nodata_kind == VSR_NODATA_NONE ? 0.0 : nodata;
  a.dst = dst;
  a.out_dtype = out_dtype;
  a.out_pitch = out_pitch;
  a.out_band_stride = out_band_stride;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  switch (stat) {
    case VSR_STAT_MIN: return fs_dispatch<VSR_STAT_MIN>(a, bands, st);
    case VSR_STAT_MAX: return fs_dispatch<VSR_STAT_MAX>(a, bands, st);
    case VSR_STAT_STD: return fs_dispatch<VSR_STAT_STD>(a, bands, st);
    case VSR_STAT_RANGE: return fs_dispatch<VSR_STAT_RANGE>(a, bands, st);
    default: return fs_dispatch<VSR_STAT_VARIETY>(a, bands, st);
  }
}

extern "C" int vsr_focal_stat(const void* src, int dtype, int64_t height, int64_t width, int64_t pitch, int stat,
                              int radius_y, int radius_x, double nodata, int nodata_kind, void* dst, int out_dtype,
                              int64_t out_pitch, void* stream) {
  return vsr_focal_stat_bands(src, dtype, 1, 0, height, width, pitch, stat, radius_y, radius_x, nodata, nodata_kind,
                              dst, out_dtype, 0, out_pitch, stream);
}
