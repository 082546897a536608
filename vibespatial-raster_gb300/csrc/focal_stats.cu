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
//              empty window (8/16-bit rasters: exact integer sums, and for a
//              float32 output sqrt(n^2 var)/n rounded once to float32 by
//              vsr_std_f32, std_round.h);
//   variety    number of distinct valid values; 0 for an empty window.
// An empty window gives the raster's nodata value (0.0 when it has none), a
// nodata centre gives the nodata value.
//
// For 8/16-bit rasters with square windows of radius <= 4 and rows aligned to
// 4 elements, min / max / range run in fs_warp_kernel and std in fs_warp_std
// (register-resident, below); everything else in focal_stat_kernel:
// a CTA owns a 64 x 16 output tile and stages its (16 + 2ry) x (64 + 2rx)
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
#include "std_round.h"

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
        const int64_t num = static_cast<int64_t>(n) * q - sm * sm;  // n^2 var, exact
        if (a.out_dtype == VSR_F32) {
          // float32 output: sqrt(num)/n correctly rounded without FP64
          const int64_t y = y0 + r, x = x0 + c;
          reinterpret_cast<float*>(obase)[y * a.out_pitch + x] =
              ndc[r * kFsTX + c] ? static_cast<float>(a.nd_out)
                                 : (n ? vsr_std_f32(static_cast<uint64_t>(num), static_cast<uint32_t>(n)) : 0.0f);
        } else {
          out_at(r, c, n ? sqrt(static_cast<double>(num)) / n : 0.0);
        }
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

// ---------------------------------------------- register-resident min / max / range
// 8/16-bit rasters, square (2R+1)^2 windows with R <= 4, rows aligned to 4
// elements: the warp-strip form of the integer focal mean (focal.cu,
// box_warp_int).  A warp owns a 128-column strip, 4 columns per lane (lanes
// 0 and 31 only supply neighbours: 120 output columns per warp); per input
// row each lane loads its 4 elements (prefetched 2R+1 rows ahead), turns
// them into order-preserving keys (int16: bit 15 flipped), invalid taps
// (nodata, outside the raster) made neutral -- 0x10000 for the minimum,
// 0 for the maximum, whose valid keys are v + 1 -- takes R keys from each
// neighbour by shuffles, reduces its 4 horizontal windows, and reduces the
// last 2R+1 rows' results over a register ring (the row loop unrolled by
// 2R+1).  An empty window (minimum key 0x10000 / maximum key 0) or a nodata
// centre gives the nodata value.
constexpr int kFwLanes = 30;
constexpr int kFwCols = 4 * kFwLanes;
constexpr int kFwWarps = 4;
constexpr int kFwStrip = 256;

template <typename T>
struct Fw4 {  // 4 elements in one load
  using type = uint2;
};
template <>
struct Fw4<uint8_t> {
  using type = uint32_t;
};

template <int R, typename T, int S, bool VOUT, bool F64>
__global__ void __launch_bounds__(32 * kFwWarps) fs_warp_kernel(const FsArgs a) {
  static_assert(R >= 1 && R <= 4, "the neighbour exchange covers radii up to 4");
  static_assert(S == VSR_STAT_MIN || S == VSR_STAT_MAX || S == VSR_STAT_RANGE, "min, max or range");
  using V4 = typename Fw4<T>::type;
  constexpr int P = 2 * R + 1;
  constexpr bool kMin = S != VSR_STAT_MAX, kMax = S != VSR_STAT_MIN;
  constexpr uint32_t kFlip = std::is_signed<T>::value ? 0x8000u : 0u;
  constexpr uint32_t kMask = sizeof(T) == 1 ? 0xFFu : 0xFFFFu;
  constexpr uint32_t kNoMin = 0x10000u;
  const int lane = threadIdx.x & 31;
  const int64_t xw = (static_cast<int64_t>(blockIdx.x) * kFwWarps + (threadIdx.x >> 5)) * kFwCols;
  if (xw >= a.W) return;
  const int64_t xs = xw - 4 + 4 * lane;
  const int64_t ys = static_cast<int64_t>(blockIdx.y) * kFwStrip;
  const T* src = static_cast<const T*>(a.src) + static_cast<int64_t>(blockIdx.z) * a.band_stride;
  char* obase = static_cast<char*>(a.dst) +
                static_cast<int64_t>(blockIdx.z) * a.out_band_stride * (a.out_dtype == VSR_F64 ? 8 : 4);
  const int nout = static_cast<int>(a.H - ys < kFwStrip ? a.H - ys : kFwStrip);
  const int nin = nout + 2 * R;
  const bool has_nd = a.kind == VSR_NODATA_VALUE;
  const uint32_t ndk = static_cast<uint32_t>(static_cast<int64_t>(a.ndv)) & kMask;  // nodata's bit pattern
  uint32_t colm = 0u;
#pragma unroll
  for (int e = 0; e < 4; ++e) colm |= static_cast<uint32_t>(xs + e >= 0 && xs + e < a.W) << e;
  const bool ld = xs >= 0 && xs < a.W, whole = xs >= 0 && xs + 4 <= a.W;
  const bool out_lane = lane >= 1 && lane <= kFwLanes;
  const T* rp = src + (ys - R) * a.pitch + xs;
  auto load = [&](int i, const T* p) -> V4 {
    const uint64_t gy = static_cast<uint64_t>(ys - R + i);
    V4 v{};
    if (ld && i < nin && gy < static_cast<uint64_t>(a.H)) {
      if (whole) {
        v = __ldg(reinterpret_cast<const V4*>(p));
      } else {
        uint32_t e[4] = {0u, 0u, 0u, 0u};
        for (int q = 0; q < 4 && xs + q < a.W; ++q)
          e[q] = static_cast<uint32_t>(static_cast<std::make_unsigned_t<T>>(__ldg(p + q)));
        if constexpr (sizeof(T) == 1) v = e[0] | (e[1] << 8) | (e[2] << 16) | (e[3] << 24);
        else v = make_uint2(e[0] | (e[1] << 16), e[2] | (e[3] << 16));
      }
    }
    return v;
  };
  V4 pre[P];
#pragma unroll
  for (int u = 0; u < P; ++u) pre[u] = load(u, rp + u * a.pitch);
  const T* lp = rp + P * a.pitch;
  uint32_t hmn[P][4], hmx[P][4], vm[P];  // per row: horizontal min / max keys, validity bits
#pragma unroll
  for (int u = 0; u < P; ++u) {
    vm[u] = 0u;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      hmn[u][c] = kNoMin;
      hmx[u][c] = 0u;
    }
  }
  int64_t orow = ys * a.out_pitch + xs;
  for (int g0 = 0; g0 < nin; g0 += P) {
#pragma unroll
    for (int u = 0; u < P; ++u) {
      const int i = g0 + u;
      if (i >= nin) break;
      const V4 raw = pre[u];
      pre[u] = load(i + P, lp);
      lp += a.pitch;
      const bool rowin = static_cast<uint64_t>(ys - R + i) < static_cast<uint64_t>(a.H);
      uint32_t e4[4];
      if constexpr (sizeof(T) == 1) {
#pragma unroll
        for (int e = 0; e < 4; ++e) e4[e] = (raw >> (8 * e)) & 0xFFu;
      } else {
        e4[0] = raw.x & 0xFFFFu;
        e4[1] = raw.x >> 16;
        e4[2] = raw.y & 0xFFFFu;
        e4[3] = raw.y >> 16;
      }
      uint32_t kmn[12], kmx[12], m = 0u;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const bool ok = rowin && ((colm >> e) & 1u) && !(has_nd && e4[e] == ndk);
        const uint32_t key = e4[e] ^ kFlip;
        kmn[4 + e] = ok ? key : kNoMin;
        kmx[4 + e] = ok ? key + 1u : 0u;
        m |= static_cast<uint32_t>(ok) << e;
      }
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        if (kMin) {
          kmn[e] = __shfl_up_sync(0xffffffffu, kmn[4 + e], 1);
          kmn[8 + e] = __shfl_down_sync(0xffffffffu, kmn[4 + e], 1);
        }
        if (kMax) {
          kmx[e] = __shfl_up_sync(0xffffffffu, kmx[4 + e], 1);
          kmx[8 + e] = __shfl_down_sync(0xffffffffu, kmx[4 + e], 1);
        }
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        uint32_t a0 = kNoMin, a1 = 0u;
#pragma unroll
        for (int j = 4 + c - R; j <= 4 + c + R; ++j) {
          if (kMin) a0 = min(a0, kmn[j]);
          if (kMax) a1 = max(a1, kmx[j]);
        }
        hmn[u][c] = a0;
        hmx[u][c] = a1;
      }
      vm[u] = m;
      if (i >= 2 * R) {
        if (out_lane) {
          const uint32_t cm = vm[(u + P - R) % P];  // the centre row i - R
          float q[4];
          double qd[4];
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            uint32_t mn = kNoMin, mx = 0u;
#pragma unroll
            for (int t = 0; t < P; ++t) {
              if (kMin) mn = min(mn, hmn[t][c]);
              if (kMax) mx = max(mx, hmx[t][c]);
            }
            const bool empty = kMin ? mn == kNoMin : mx == 0u;
            const bool nd = empty || !((cm >> c) & 1u);
            // keys back to values: undo the flip (int16 sign-extends)
            const float vmn = static_cast<float>(static_cast<T>((mn ^ kFlip) & kMask));
            const float vmx = static_cast<float>(static_cast<T>(((mx - 1u) ^ kFlip) & kMask));
            const float v = S == VSR_STAT_MIN ? vmn : (S == VSR_STAT_MAX ? vmx : vmx - vmn);  // exact
            q[c] = nd ? static_cast<float>(a.nd_out) : v;
            qd[c] = nd ? a.nd_out : static_cast<double>(v);
          }
          if constexpr (F64) {
            double* op = reinterpret_cast<double*>(obase) + orow;
#pragma unroll
            for (int c = 0; c < 4; ++c)
              if (xs + c < a.W) op[c] = qd[c];
          } else {
            float* op = reinterpret_cast<float*>(obase) + orow;
            if (VOUT && xs + 3 < a.W) {
              *reinterpret_cast<float4*>(op) = make_float4(q[0], q[1], q[2], q[3]);
            } else {
#pragma unroll
              for (int c = 0; c < 4; ++c)
                if (xs + c < a.W) op[c] = q[c];
            }
          }
        }
        orow += a.out_pitch;
      }
    }
  }
}

// ---------------------------------------------- register-resident std
// 8/16-bit rasters, square windows with R <= 4, rows aligned to 4 elements.
// Same warp strips; the statistic is shift-invariant, so values enter as
// v' = v (int16: v + 32768 via bit 15) and the sums stay non-negative and
// exact in 32 bits: a packed word (v' in the low bits, a count bit above,
// as in the focal mean) and the two 16-bit halves of v'^2.  Per lane and
// column, running vertical sums over the last 2R+1 rows: the entering row
// added, the leaving one (kept in a shared-memory ring of raw rows, one slot
// column per thread) subtracted; then shuffles and horizontal window sums.  n^2 var = n sum v'^2 -
// (sum v')^2 exactly in 64 bits; a float32 output is sqrt(n^2 var)/n rounded
// once (vsr_std_f32_small), a float64 output the FP64 form of the
// shared-memory kernel.  A nodata centre gives the nodata value.
template <int R, typename T, bool VOUT, bool F64>
__global__ void __launch_bounds__(32 * kFwWarps) fs_warp_std(const FsArgs a) {
  static_assert(R >= 1 && R <= 4, "the neighbour exchange covers radii up to 4");
  using V4 = typename Fw4<T>::type;
  constexpr int P = 2 * R + 1;
  constexpr long long kTaps = static_cast<long long>(P) * P;
  constexpr int kShift = kTaps * 65535ll < (1ll << 22) ? 22 : 23;  // value-sum bits; the count above
  static_assert(kTaps * 65535ll < (1ll << kShift) && kTaps < (1ll << (32 - kShift)), "packed sums overflow");
  constexpr uint32_t kOne = 1u << kShift, kLow = kOne - 1u;
  constexpr uint32_t kFlip = std::is_signed<T>::value ? 0x8000u : 0u;
  constexpr uint32_t kMask = sizeof(T) == 1 ? 0xFFu : 0xFFFFu;
  const int lane = threadIdx.x & 31;
  const int64_t xw = (static_cast<int64_t>(blockIdx.x) * kFwWarps + (threadIdx.x >> 5)) * kFwCols;
  if (xw >= a.W) return;
  const int64_t xs = xw - 4 + 4 * lane;
  const int64_t ys = static_cast<int64_t>(blockIdx.y) * kFwStrip;
  const T* src = static_cast<const T*>(a.src) + static_cast<int64_t>(blockIdx.z) * a.band_stride;
  char* obase = static_cast<char*>(a.dst) +
                static_cast<int64_t>(blockIdx.z) * a.out_band_stride * (F64 ? 8 : 4);
  const int nout = static_cast<int>(a.H - ys < kFwStrip ? a.H - ys : kFwStrip);
  const int nin = nout + 2 * R;
  const bool has_nd = a.kind == VSR_NODATA_VALUE;
  const uint32_t ndk = static_cast<uint32_t>(static_cast<int64_t>(a.ndv)) & kMask;
  uint32_t colm = 0u;
#pragma unroll
  for (int e = 0; e < 4; ++e) colm |= static_cast<uint32_t>(xs + e >= 0 && xs + e < a.W) << e;
  const bool ld = xs >= 0 && xs < a.W, whole = xs >= 0 && xs + 4 <= a.W;
  const bool out_lane = lane >= 1 && lane <= kFwLanes;
  const T* rp = src + (ys - R) * a.pitch + xs;
  auto load = [&](int i, const T* p) -> V4 {
    const uint64_t gy = static_cast<uint64_t>(ys - R + i);
    V4 v{};
    if (ld && i < nin && gy < static_cast<uint64_t>(a.H)) {
      if (whole) {
        v = __ldg(reinterpret_cast<const V4*>(p));
      } else {
        uint32_t e[4] = {0u, 0u, 0u, 0u};
        for (int q = 0; q < 4 && xs + q < a.W; ++q)
          e[q] = static_cast<uint32_t>(static_cast<std::make_unsigned_t<T>>(__ldg(p + q)));
        if constexpr (sizeof(T) == 1) v = e[0] | (e[1] << 8) | (e[2] << 16) | (e[3] << 24);
        else v = make_uint2(e[0] | (e[1] << 16), e[2] | (e[3] << 16));
      }
    }
    return v;
  };
  // a row's 4 elements -> packed words, v'^2 halves, validity bits
  auto prep = [&](const V4 raw, bool rowin, uint32_t pk[4], uint32_t sh[4], uint32_t sl[4]) -> uint32_t {
    uint32_t e4[4];
    if constexpr (sizeof(T) == 1) {
#pragma unroll
      for (int e = 0; e < 4; ++e) e4[e] = (raw >> (8 * e)) & 0xFFu;
    } else {
      e4[0] = raw.x & 0xFFFFu;
      e4[1] = raw.x >> 16;
      e4[2] = raw.y & 0xFFFFu;
      e4[3] = raw.y >> 16;
    }
    uint32_t m = 0u;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const bool ok = rowin && ((colm >> e) & 1u) && !(has_nd && e4[e] == ndk);
      const uint32_t v = e4[e] ^ kFlip, sq = v * v;
      pk[e] = ok ? (v | kOne) : 0u;
      sh[e] = ok ? (sq >> 16) : 0u;
      sl[e] = ok ? (sq & 0xFFFFu) : 0u;
      m |= static_cast<uint32_t>(ok) << e;
    }
    return m;
  };
  // the window's raw rows in a shared-memory ring, one slot column per
  // thread (each thread reads only its own slots: no barrier); the row loop
  // is not unrolled, so the long output code exists once
  __shared__ V4 ring[P][32 * kFwWarps];
  const int t = threadIdx.x;
#pragma unroll
  for (int u = 0; u < P; ++u) ring[u][t] = V4{};
  V4 nxt = load(0, rp);  // one row ahead
  const T* lp = rp + a.pitch;
  uint32_t cs[4] = {0u, 0u, 0u, 0u}, ch[4] = {0u, 0u, 0u, 0u}, cl[4] = {0u, 0u, 0u, 0u};  // column sums
  int64_t orow = ys * a.out_pitch + xs;
  int slot = 0, cslot = P - R;  // ring slots of rows i and i - R
#pragma unroll 1
  for (int i = 0; i < nin; ++i) {
    const V4 rn = nxt;
    nxt = load(i + 1, lp);
    lp += a.pitch;
    const V4 ro = ring[slot][t];  // row i - P, leaving the window
    ring[slot][t] = rn;
    uint32_t pn[4], hn[4], ln[4], po[4], ho[4], lo[4];
    prep(rn, static_cast<uint64_t>(ys - R + i) < static_cast<uint64_t>(a.H), pn, hn, ln);
    prep(ro, i >= P && static_cast<uint64_t>(ys - R + i - P) < static_cast<uint64_t>(a.H), po, ho, lo);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      cs[c] += pn[c] - po[c];
      ch[c] += hn[c] - ho[c];
      cl[c] += ln[c] - lo[c];
    }
    if (i >= 2 * R) {
      // neighbours' column sums, then the horizontal window sums
      uint32_t ws[12], wh[12], wl[12];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        ws[4 + e] = cs[e];
        wh[4 + e] = ch[e];
        wl[4 + e] = cl[e];
        ws[e] = __shfl_up_sync(0xffffffffu, cs[e], 1);
        wh[e] = __shfl_up_sync(0xffffffffu, ch[e], 1);
        wl[e] = __shfl_up_sync(0xffffffffu, cl[e], 1);
        ws[8 + e] = __shfl_down_sync(0xffffffffu, cs[e], 1);
        wh[8 + e] = __shfl_down_sync(0xffffffffu, ch[e], 1);
        wl[8 + e] = __shfl_down_sync(0xffffffffu, cl[e], 1);
      }
      if (out_lane) {
        // the centre row i - R (inside the raster: an output row)
        uint32_t pc[4], hc[4], lc[4];
        const uint32_t cm = prep(ring[cslot][t], true, pc, hc, lc);
        uint32_t s0 = 0u, s1 = 0u, s2 = 0u;
#pragma unroll
        for (int j = 4 - R; j <= 4 + R; ++j) {
          s0 += ws[j];
          s1 += wh[j];
          s2 += wl[j];
        }
        float q[4];
        double qd[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          if (c > 0) {
            s0 += ws[4 + c + R] - ws[3 + c - R];
            s1 += wh[4 + c + R] - wh[3 + c - R];
            s2 += wl[4 + c + R] - wl[3 + c - R];
          }
          const uint32_t cnt = s0 >> kShift, sum = s0 & kLow;
          const uint64_t sq = (static_cast<uint64_t>(s1) << 16) + s2;
          const uint64_t N = static_cast<uint64_t>(cnt) * sq - static_cast<uint64_t>(sum) * sum;  // n^2 var
          const bool ok = (cm >> c) & 1u;  // a valid centre: cnt >= 1
          if constexpr (F64) qd[c] = ok ? sqrt(static_cast<double>(N)) / cnt : a.nd_out;
          else q[c] = ok ? vsr_std_f32_small(N, cnt) : static_cast<float>(a.nd_out);
        }
        if constexpr (F64) {
          double* op = reinterpret_cast<double*>(obase) + orow;
#pragma unroll
          for (int c = 0; c < 4; ++c)
            if (xs + c < a.W) op[c] = qd[c];
        } else {
          float* op = reinterpret_cast<float*>(obase) + orow;
          if (VOUT && xs + 3 < a.W) {
            *reinterpret_cast<float4*>(op) = make_float4(q[0], q[1], q[2], q[3]);
          } else {
#pragma unroll
            for (int c = 0; c < 4; ++c)
              if (xs + c < a.W) op[c] = q[c];
          }
        }
      }
      orow += a.out_pitch;
    }
    slot = slot + 1 == P ? 0 : slot + 1;
    cslot = cslot + 1 == P ? 0 : cslot + 1;
  }
}

template <int R, typename T, int S>
int fs_warp_launch(const FsArgs& a, int bands, cudaStream_t st) {
  const dim3 grid(static_cast<unsigned>((a.W + kFwWarps * kFwCols - 1) / (kFwWarps * kFwCols)),
                  static_cast<unsigned>((a.H + kFwStrip - 1) / kFwStrip), static_cast<unsigned>(bands));
  if (grid.y > 65535u) return -1;
  const bool vout = a.out_dtype == VSR_F32 && aligned(a.dst, 16) && a.out_pitch % 4 == 0 &&
                    (bands == 1 || a.out_band_stride % 4 == 0);
  if constexpr (S == VSR_STAT_STD) {
    if (a.out_dtype == VSR_F64) fs_warp_std<R, T, false, true><<<grid, 32 * kFwWarps, 0, st>>>(a);
    else if (vout) fs_warp_std<R, T, true, false><<<grid, 32 * kFwWarps, 0, st>>>(a);
    else fs_warp_std<R, T, false, false><<<grid, 32 * kFwWarps, 0, st>>>(a);
  } else {
    if (a.out_dtype == VSR_F64) fs_warp_kernel<R, T, S, false, true><<<grid, 32 * kFwWarps, 0, st>>>(a);
    else if (vout) fs_warp_kernel<R, T, S, true, false><<<grid, 32 * kFwWarps, 0, st>>>(a);
    else fs_warp_kernel<R, T, S, false, false><<<grid, 32 * kFwWarps, 0, st>>>(a);
  }
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}

// The register-resident form when it applies (8/16-bit min / max / range /
// std, square window of radius 1..4, rows aligned to 4 elements); -1 otherwise.
template <typename T, int S>
int fs_warp_try(const FsArgs& a, int bands, cudaStream_t st) {
  if (a.ry != a.rx || a.ry < 1 || a.ry > 4) return -1;
  if (!aligned(a.src, 4 * sizeof(T)) || a.pitch % 4 != 0 || (bands > 1 && a.band_stride % 4 != 0)) return -1;
  switch (a.ry) {
    case 1: return fs_warp_launch<1, T, S>(a, bands, st);
    case 2: return fs_warp_launch<2, T, S>(a, bands, st);
    case 3: return fs_warp_launch<3, T, S>(a, bands, st);
    default: return fs_warp_launch<4, T, S>(a, bands, st);
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
    int rc = -1;
    switch (a.dtype) {
      case VSR_U8: rc = fs_warp_try<uint8_t, S>(a, bands, st); break;
      case VSR_I16: rc = fs_warp_try<int16_t, S>(a, bands, st); break;
      case VSR_U16: rc = fs_warp_try<uint16_t, S>(a, bands, st); break;
      default: break;
    }
    if (rc >= 0) return rc;
    switch (a.dtype) {
      case VSR_U8: return fs_launch<uint8_t, int32_t, S>(a, bands, st);
      case VSR_I16: return fs_launch<int16_t, int32_t, S>(a, bands, st);
      case VSR_U16: return fs_launch<uint16_t, int32_t, S>(a, bands, st);
      case VSR_I32: return fs_launch<int32_t, double, S>(a, bands, st);
      case VSR_F32: return fs_launch<float, double, S>(a, bands, st);
      default: return fs_launch<double, double, S>(a, bands, st);
    }
  } else {
    if constexpr (S != VSR_STAT_VARIETY) {
      int rc = -1;
      switch (a.dtype) {
        case VSR_U8: rc = fs_warp_try<uint8_t, S>(a, bands, st); break;
        case VSR_I16: rc = fs_warp_try<int16_t, S>(a, bands, st); break;
        case VSR_U16: rc = fs_warp_try<uint16_t, S>(a, bands, st); break;
        default: break;
      }
      if (rc >= 0) return rc;
    }
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
