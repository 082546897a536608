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

__device__ __forceinline__ void fs_store(const FsArgs& a, char* obase, int64_t idx, double v) {
  if (a.out_dtype == VSR_F64) reinterpret_cast<double*>(obase)[idx] = v;
  else reinterpret_cast<float*>(obase)[idx] = static_cast<float>(v);
}

// Nodata test in the element type itself (the value is exact there).
template <typename TIN>
__device__ __forceinline__ bool is_nd(TIN v, int kind, TIN ndv) {
  if constexpr (std::is_floating_point<TIN>::value)
    return kind == VSR_NODATA_VALUE ? v == ndv : (kind == VSR_NODATA_NAN ? v != v : false);
  else
    return kind == VSR_NODATA_VALUE && v == ndv;
}

// Staged value of one tap for statistic S (placeholder for nodata and
// out-of-bounds taps).
template <typename T, int S, typename TIN>
__device__ __forceinline__ T staged(bool valid, TIN v) {
  if constexpr (std::is_same<T, int32_t>::value) {
    return valid ? static_cast<int32_t>(v) : INT32_MIN;  // 8/16-bit std: INT32_MIN is never a value
  } else if constexpr (S == VSR_STAT_MIN) {
    return valid ? static_cast<T>(v) : pos_inf<T>();
  } else if constexpr (S == VSR_STAT_MAX) {
    return valid ? static_cast<T>(v) : -pos_inf<T>();
  } else {
    return valid ? static_cast<T>(v) : qnan<T>();  // NaN data stays NaN = excluded
  }
}

template <int S, typename T>
struct FsLayout {  // shared-memory carve-up of one CTA (byte offsets)
  static constexpr bool kIntStd = S == VSR_STAT_STD && std::is_same<T, int32_t>::value;
  static constexpr bool kSep = S == VSR_STAT_MIN || S == VSR_STAT_MAX || S == VSR_STAT_RANGE;
  __host__ __device__ static size_t staged(int ry, int rx) {
    return (static_cast<size_t>(kFsTY + 2 * ry) * (kFsTX + 2 * rx) * sizeof(T) + 15) & ~size_t(15);
  }
  __host__ __device__ static size_t rows(int ry) {  // row-pass results, (TY + 2 ry) x TX
    const size_t n = static_cast<size_t>(kFsTY + 2 * ry) * kFsTX;
    if (kIntStd) return n * (4 + 8 + 4);          // sum, sum of squares, count
    if (S == VSR_STAT_RANGE) return 2 * n * sizeof(T);
    if (kSep) return n * sizeof(T);
    return 0;
  }
  __host__ __device__ static size_t total(int ry, int rx) { return staged(ry, rx) + rows(ry) + kFsTY * kFsTX; }
};

// One CTA = a 64 x 16 output tile of one band.  Staging: the tile's window
// in the statistic's type with placeholders applied, and the centre
// pixels' nodata flags.  min / max / range and the 8/16-bit std are
// separable (a row pass into shared memory, a column pass); the float std
// (two float64 passes) and variety run over the staged window per pixel.
template <typename TIN, typename T, int S>
__global__ void __launch_bounds__(kFsThreads) focal_stat_kernel(const FsArgs a) {
  using Lay = FsLayout<S, T>;
  extern __shared__ __align__(16) unsigned char fs_smem[];
  const int ry = a.ry, rx = a.rx;
  const int SW = kFsTX + 2 * rx, SH = kFsTY + 2 * ry;
  T* St = reinterpret_cast<T*>(fs_smem);
  unsigned char* rows = fs_smem + Lay::staged(ry, rx);
  unsigned char* ndc = rows + Lay::rows(ry);  // kFsTY x kFsTX centre nodata flags
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int WARPS = kFsThreads / 32;
  const int64_t x0 = static_cast<int64_t>(blockIdx.x) * kFsTX, y0 = static_cast<int64_t>(blockIdx.y) * kFsTY;
  const TIN* src = static_cast<const TIN*>(a.src) + static_cast<int64_t>(blockIdx.z) * a.band_stride;
  char* obase = static_cast<char*>(a.dst) +
                static_cast<int64_t>(blockIdx.z) * a.out_band_stride * (a.out_dtype == VSR_F64 ? 8 : 4);
  const TIN ndv = static_cast<TIN>(a.ndv);  // exact: resolve_nodata checked it fits the element type
  const int kind = a.kind;
  // columns of the window inside the raster: [c_lo, c_hi)
  const int c_lo = x0 - rx >= 0 ? 0 : static_cast<int>(rx - x0);
  const int64_t chi = a.W - (x0 - rx);
  const int c_hi = chi < SW ? static_cast<int>(chi) : SW;

  for (int r = warp; r < SH; r += WARPS) {
    const int64_t gy = y0 - ry + r;
    const bool row_in = gy >= 0 && gy < a.H;
    const TIN* rowp = src + (row_in ? gy : 0) * a.pitch + (x0 - rx);
    const bool centre_row = r >= ry && r < ry + kFsTY;
    for (int c = lane; c < SW; c += 32) {
      const bool inb = row_in && c >= c_lo && c < c_hi;
      const TIN v = inb ? __ldg(rowp + c) : TIN(0);
      const bool nd = inb && is_nd<TIN>(v, kind, ndv);
      St[r * SW + c] = staged<T, S, TIN>(inb && !nd, v);
      if (centre_row && c >= rx && c < rx + kFsTX) ndc[(r - ry) * kFsTX + (c - rx)] = nd;
    }
  }
  __syncthreads();

  auto out_at = [&](int r, int c, double v) {
    const int64_t y = y0 + r, x = x0 + c;
    fs_store(a, obase, y * a.out_pitch + x, ndc[r * kFsTX + c] ? a.nd_out : v);
  };
  const int nr = static_cast<int>(a.H - y0 < kFsTY ? a.H - y0 : int64_t(kFsTY));  // output rows inside
  const int nc = static_cast<int>(a.W - x0 < kFsTX ? a.W - x0 : int64_t(kFsTX));  // output columns inside
  const int kh = 2 * ry + 1, kw = 2 * rx + 1;

  if constexpr (Lay::kSep) {
    T* R0 = reinterpret_cast<T*>(rows);
    T* R1 = R0 + SH * kFsTX;
    for (int r = warp; r < SH; r += WARPS) {
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
    for (int r = warp; r < nr; r += WARPS)
      for (int c = lane; c < nc; c += 32) {
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
        out_at(r, c, out);
      }
  } else if constexpr (Lay::kIntStd) {
    // exact separable sums: var = (n sum x^2 - (sum x)^2) / n^2
    int32_t* Rs = reinterpret_cast<int32_t*>(rows);
    int64_t* Rq = reinterpret_cast<int64_t*>(rows + static_cast<size_t>(SH) * kFsTX * 4);
    int32_t* Rn = reinterpret_cast<int32_t*>(rows + static_cast<size_t>(SH) * kFsTX * 12);
    for (int r = warp; r < SH; r += WARPS) {
      const int32_t* row = reinterpret_cast<const int32_t*>(St) + r * SW;
      for (int c = lane; c < kFsTX; c += 32) {
        int32_t sm = 0, n = 0;
        int64_t q = 0;
        for (int d = 0; d < kw; ++d) {
          const int32_t v = row[c + d];
          const bool ok = v != INT32_MIN;
          sm += ok ? v : 0;
          q += ok ? static_cast<int64_t>(v) * v : 0;
          n += ok;
        }
        Rs[r * kFsTX + c] = sm;
        Rq[r * kFsTX + c] = q;
        Rn[r * kFsTX + c] = n;
      }
    }
    __syncthreads();
    for (int r = warp; r < nr; r += WARPS)
      for (int c = lane; c < nc; c += 32) {
        int64_t sm = 0, q = 0;
        int32_t n = 0;
        for (int d = 0; d < kh; ++d) {
          sm += Rs[(r + d) * kFsTX + c];
          q += Rq[(r + d) * kFsTX + c];
          n += Rn[(r + d) * kFsTX + c];
        }
        out_at(r, c, n ? sqrt(static_cast<double>(static_cast<int64_t>(n) * q - sm * sm)) / n : 0.0);
      }
  } else {
    for (int r = warp; r < nr; r += WARPS)
      for (int c = lane; c < nc; c += 32) {
        const T* win = St + r * SW + c;
        double out;
        if constexpr (S == VSR_STAT_STD) {
          double sm = 0.0;
          int n = 0;
          for (int dy = 0; dy < kh; ++dy)
            for (int dx = 0; dx < kw; ++dx) {
              const double v = win[dy * SW + dx];
              if (v != v) continue;
              sm += v;
              ++n;
            }
          double m2 = 0.0;
          if (n) {
            const double mean = sm / n;
            for (int dy = 0; dy < kh; ++dy)
              for (int dx = 0; dx < kw; ++dx) {
                const double v = win[dy * SW + dx];
                if (v != v) continue;
                const double d = v - mean;
                m2 = fma(d, d, m2);
              }
          }
          out = n ? sqrt(m2 / n) : 0.0;
        } else {  // variety: taps with no equal earlier tap
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
        out_at(r, c, out);
      }
  }
}

template <typename TIN, typename T, int S>
int fs_launch(const FsArgs& a, int bands, cudaStream_t st) {
  const size_t smem = FsLayout<S, T>::total(a.ry, a.rx);
  auto kern = focal_stat_kernel<TIN, T, S>;
  VSR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  const dim3 grid(static_cast<unsigned>((a.W + kFsTX - 1) / kFsTX), static_cast<unsigned>((a.H + kFsTY - 1) / kFsTY),
                  static_cast<unsigned>(bands));
  kern<<<grid, kFsThreads, smem, st>>>(a);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}

// T: the statistic's type -- float for 8/16-bit and float32 rasters (exact),
// double for int32 / float64, int32 for the 8/16-bit std (exact int sums).
template <int S>
int fs_dispatch(const FsArgs& a, int bands, cudaStream_t st) {
  if constexpr (S == VSR_STAT_STD) {
    switch (a.dtype) {
      case VSR_U8: return fs_launch<uint8_t, int32_t, S>(a, bands, st);
      case VSR_I16: return fs_launch<int16_t, int32_t, S>(a, bands, st);
      case VSR_U16: return fs_launch<uint16_t, int32_t, S>(a, bands, st);
      case VSR_I32: return fs_launch<int32_t, double, S>(a, bands, st);
      case VSR_F32: return fs_launch<float, double, S>(a, bands, st);
      default: return fs_launch<double, double, S>(a, bands, st);
    }
  } else {
    switch (a.dtype) {
      case VSR_U8: return fs_launch<uint8_t, float, S>(a, bands, st);
      case VSR_I16: return fs_launch<int16_t, float, S>(a, bands, st);
      case VSR_U16: return fs_launch<uint16_t, float, S>(a, bands, st);
      case VSR_I32: return fs_launch<int32_t, double, S>(a, bands, st);
      case VSR_F32: return fs_launch<float, float, S>(a, bands, st);
      default: return fs_launch<double, double, S>(a, bands, st);
    }
  }
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
