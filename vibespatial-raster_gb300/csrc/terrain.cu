// Terrain derivatives on the 3x3 window: TRI, TPI and profile curvature in
// one pass (any subset of the three outputs).
//
// Replaces the reference's ``terrain_derivatives`` NVRTC kernel
// (kernels/focal.py:487-647) and its launch glue (algebra.py:2854-2991): the
// float64 up-cast, the uint8 mask pass and one launch per derivative.  The
// semantics are the reference CPU/GPU ones (algebra.py:3352-3445): window
// z0..z8 (row-major, z4 the centre) with edge replication,
//   TRI  = sum |z_i - z4| / 8                      (Riley et al. 1999)
//   TPI  = z4 - sum z_i / 8
//   curv = -2 (D + E) 100,  D = ((z3 + z5)/2 - z4) / cx^2,
//                           E = ((z1 + z7)/2 - z4) / cy^2   (Zevenbergen & Thorne 1987)
// over the 8 neighbours; border pixels and pixels whose window touches a
// nodata pixel get the output nodata value.
//
// Arithmetic.  The reference computes in float64; GB300's FP64 rate is a
// small fraction of its FP32 rate, so 8/16-bit and float32 DEMs (exact in
// FP32) are evaluated in double-float FP32: every neighbour difference is
// formed error-free (TwoDiff), sums are compensated (TwoSum) and products use
// FMA, so results carry ~44 significant bits -- float64 quality for these
// few-term formulas -- before the single conversion to the output type.
// A formula whose inputs include NaN or +-inf takes the plain float form
// (the special values propagate as in the reference).  int32 and float64
// DEMs are computed in FP64 with the reference's own operation order.
#include <cmath>
#include <type_traits>

#include "vsr_internal.cuh"
#include "df_round.h"
#include "terrain_exact.h"

namespace vsr {
namespace {

constexpr int kDTW = 32, kDTH = 8;  // output tile: 32 x 8 pixels, one per thread
constexpr int kDSW = kDTW + 2, kDSH = kDTH + 2;

struct DerivParams {
  int64_t H, W, pitch, out_pitch;
  int64_t band_stride, out_band_stride;  // band blockIdx.z of a band-first stack
  int nd_kind;      // resolved VSR_NODATA_*
  double nd_in;     // nodata value of the raster (element value, as double)
  double nd_out;    // value written to nodata / border pixels
  double cx2, cy2;                  // cx^2, cy^2 (FP64 path: the reference divides)
  float icx2_hi, icx2_lo, icy2_hi, icy2_lo;  // the same as float pairs
  void *tri, *tpi, *curv;
  int out_dtype;
};

// ---- double-float helpers: value = hi + lo with |lo| <= ulp(hi)/2
struct DF {
  float hi, lo;
};
__device__ __forceinline__ DF two_diff_df(float a, float b) {  // a - b exactly
  const float s = __fsub_rn(a, b);
  const float z = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, z)), -__fadd_rn(b, z))};
}
__device__ __forceinline__ DF two_sum_df(float a, float b) {  // a + b exactly
  const float s = __fadd_rn(a, b);
  const float z = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, z)), __fsub_rn(b, z))};
}
__device__ __forceinline__ DF fast_two_sum_df(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
  const DF s = two_sum_df(a.hi, b.hi);
  return fast_two_sum_df(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ DF df_mul(DF a, DF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum_df(p, e);
}
__device__ __forceinline__ DF df_mul_f(DF a, float c) {
  const float p = __fmul_rn(a.hi, c);
  const float e = __fmaf_rn(a.lo, c, __fmaf_rn(a.hi, c, -p));
  return fast_two_sum_df(p, e);
}
__device__ __forceinline__ DF df_neg(DF a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ DF df_abs(DF a) { return a.hi < 0.0f ? df_neg(a) : a; }
__device__ __forceinline__ DF df_scale(DF a, float p2) { return {a.hi * p2, a.lo * p2}; }  // p2 a power of two

template <typename T>
__device__ __forceinline__ void store_out(void* base, int out_dtype, int64_t i, T v) {
  if (out_dtype == VSR_F64) static_cast<double*>(base)[i] = static_cast<double>(v);
  else static_cast<float*>(base)[i] = static_cast<float>(v);
}
// hi + lo as a double: both floats widened with integer operations
// (vsr_f32_widen), one FP64 add; subnormal or non-finite parts convert in FP64.
__device__ __forceinline__ double df_to_double(float hi, float lo) {
  const uint32_t hb = __float_as_uint(hi), lb = __float_as_uint(lo);
  if (!(vsr_f32_widen_ok(hb) && vsr_f32_widen_ok(lb))) return static_cast<double>(hi) + static_cast<double>(lo);
  uint32_t hh, hl, lh, ll;
  vsr_f32_widen(hb, &hh, &hl);
  vsr_f32_widen(lb, &lh, &ll);
  return __hiloint2double(static_cast<int>(hh), static_cast<int>(hl)) +
         __hiloint2double(static_cast<int>(lh), static_cast<int>(ll));
}

// s 2^e (exact, |s| < 2^31) as the output: float64 bits written directly,
// float32 rounded once.
__device__ __forceinline__ void store_int_scaled(void* base, int out_dtype, int64_t i, int32_t s, int e) {
  const double v = __longlong_as_double(static_cast<long long>(vsr_int_scaled_bits(s, e)));
  if (out_dtype == VSR_F64) static_cast<double*>(base)[i] = v;
  else static_cast<float*>(base)[i] = static_cast<float>(v);
}

__device__ __forceinline__ void store_df(void* base, int out_dtype, int64_t i, DF v) {
  if (out_dtype == VSR_F64) static_cast<double*>(base)[i] = df_to_double(v.hi, v.lo);
  else static_cast<float*>(base)[i] = v.hi + v.lo;
}

// The reference's formulas in the operation order of algebra.py:3394-3412
// (double for FP64 DEMs; float where a window holds NaN or +-inf, whose
// special values propagate the same way in either precision).
template <typename C>
__device__ __forceinline__ C plain_tri(const C z[9]) {
  return (fabs(z[0] - z[4]) + fabs(z[1] - z[4]) + fabs(z[2] - z[4]) + fabs(z[3] - z[4]) + fabs(z[5] - z[4]) +
          fabs(z[6] - z[4]) + fabs(z[7] - z[4]) + fabs(z[8] - z[4])) /
         C(8);
}
template <typename C>
__device__ __forceinline__ C plain_tpi(const C z[9]) {
  return z[4] - (z[0] + z[1] + z[2] + z[3] + z[5] + z[6] + z[7] + z[8]) / C(8);
}
template <typename C>
__device__ __forceinline__ C plain_curv(const C z[9], const DerivParams& P) {
  const C D = ((z[3] + z[5]) / C(2) - z[4]) / static_cast<C>(P.cx2);
  const C E = ((z[1] + z[7]) / C(2) - z[4]) / static_cast<C>(P.cy2);
  return C(-2) * (D + E) * C(100);
}

template <typename T>
__global__ void __launch_bounds__(kDTW * kDTH) terrain_deriv_kernel(const T* __restrict__ src, const DerivParams P) {
  constexpr bool kDF = !std::is_same<T, double>::value && !std::is_same<T, int32_t>::value;
  using C = std::conditional_t<kDF, float, double>;
  __shared__ C tile[kDSH][kDSW + 1];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kDTW + tx;
  const int64_t x0 = static_cast<int64_t>(blockIdx.x) * kDTW, y0 = static_cast<int64_t>(blockIdx.y) * kDTH;
  src += static_cast<int64_t>(blockIdx.z) * P.band_stride;
  // the tile and its 1-pixel halo, coordinates clamped (edge replication)
  for (int i = tid; i < kDSH * kDSW; i += kDTW * kDTH) {
    const int r = i / kDSW, c = i - r * kDSW;
    int64_t gy = y0 - 1 + r, gx = x0 - 1 + c;
    gy = gy < 0 ? 0 : (gy >= P.H ? P.H - 1 : gy);
    gx = gx < 0 ? 0 : (gx >= P.W ? P.W - 1 : gx);
    tile[r][c] = static_cast<C>(__ldg(src + gy * P.pitch + gx));
  }
  __syncthreads();
  const int64_t x = x0 + tx, y = y0 + ty;
  if (x >= P.W || y >= P.H) return;
  const int64_t o = static_cast<int64_t>(blockIdx.z) * P.out_band_stride + y * P.out_pitch + x;
  C z[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) z[k] = tile[ty + k / 3][tx + k % 3];
  bool nd = x == 0 || y == 0 || x == P.W - 1 || y == P.H - 1;
  if (P.nd_kind == VSR_NODATA_VALUE) {
    const C ndv = static_cast<C>(P.nd_in);
#pragma unroll
    for (int k = 0; k < 9; ++k) nd |= z[k] == ndv;
  } else if (P.nd_kind == VSR_NODATA_NAN) {
#pragma unroll
    for (int k = 0; k < 9; ++k) nd |= z[k] != z[k];
  }
  if (nd) {
    if (P.tri) store_out(P.tri, P.out_dtype, o, P.nd_out);
    if (P.tpi) store_out(P.tpi, P.out_dtype, o, P.nd_out);
    if (P.curv) store_out(P.curv, P.out_dtype, o, P.nd_out);
    return;
  }
  // finiteness of the values each formula reads: TRI and TPI all nine,
  // curvature the centre and its four edge neighbours
  bool f5 = true, f9;
#pragma unroll
  for (int k = 1; k < 9; k += 2) f5 &= fabs(z[k]) <= static_cast<C>(3.4e38);
  f5 &= fabs(z[4]) <= static_cast<C>(3.4e38);
  f9 = f5 && fabs(z[0]) <= static_cast<C>(3.4e38) && fabs(z[2]) <= static_cast<C>(3.4e38) &&
       fabs(z[6]) <= static_cast<C>(3.4e38) && fabs(z[8]) <= static_cast<C>(3.4e38);
  if (kDF) {
    // TRI and TPI as exact integers when the window's values share a narrow
    // binade range (terrain_exact.h): the reference's float64 results bit for
    // bit, no double-float arithmetic
    uint32_t bits[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) bits[k] = __float_as_uint(static_cast<float>(z[k]));
    int32_t t8 = 0, p8 = 0;
    int e2 = 0;
    if ((P.tri || P.tpi) && vsr_tt_exact(bits, &t8, &p8, &e2)) {
      if (P.tri) store_int_scaled(P.tri, P.out_dtype, o, t8, e2 - 3);
      if (P.tpi) store_int_scaled(P.tpi, P.out_dtype, o, p8, e2 - 3);
      if (P.curv) {
        if (f5) {
          const float z4 = static_cast<float>(z[4]);
          const DF dw = two_diff_df(static_cast<float>(z[3]), z4), de = two_diff_df(static_cast<float>(z[5]), z4);
          const DF dn = two_diff_df(static_cast<float>(z[1]), z4), ds = two_diff_df(static_cast<float>(z[7]), z4);
          const DF dx = df_scale(df_add(dw, de), 0.5f), dy = df_scale(df_add(dn, ds), 0.5f);
          const DF e = df_add(df_mul(dx, DF{P.icx2_hi, P.icx2_lo}), df_mul(dy, DF{P.icy2_hi, P.icy2_lo}));
          store_df(P.curv, P.out_dtype, o, df_mul_f(e, -200.0f));
        } else {
          store_out(P.curv, P.out_dtype, o, plain_curv(z, P));
        }
      }
      return;
    }
    // error-free neighbour differences d_i = z_i - z4 (i = 0..3, 5..8)
    DF d[8];
#pragma unroll
    for (int k = 0, i = 0; k < 9; ++k)
      if (k != 4) d[i++] = two_diff_df(static_cast<float>(z[k]), static_cast<float>(z[4]));
    if (P.tri) {
      if (f9) {
        DF s = df_abs(d[0]);
#pragma unroll
        for (int i = 1; i < 8; ++i) s = df_add(s, df_abs(d[i]));
        store_df(P.tri, P.out_dtype, o, df_scale(s, 0.125f));
      } else {
        store_out(P.tri, P.out_dtype, o, plain_tri(z));
      }
    }
    if (P.tpi) {
      if (f9) {
        DF s = d[0];
#pragma unroll
        for (int i = 1; i < 8; ++i) s = df_add(s, d[i]);
        store_df(P.tpi, P.out_dtype, o, df_scale(df_neg(s), 0.125f));  // z4 - mean = -(sum d_i) / 8
      } else {
        store_out(P.tpi, P.out_dtype, o, plain_tpi(z));
      }
    }
    if (P.curv) {
      if (f5) {
        // (z3 + z5)/2 - z4 = (d_w + d_e) / 2, (z1 + z7)/2 - z4 = (d_n + d_s) / 2
        const DF dx = df_scale(df_add(d[3], d[4]), 0.5f), dy = df_scale(df_add(d[1], d[6]), 0.5f);
        const DF e = df_add(df_mul(dx, DF{P.icx2_hi, P.icx2_lo}), df_mul(dy, DF{P.icy2_hi, P.icy2_lo}));
        store_df(P.curv, P.out_dtype, o, df_mul_f(e, -200.0f));
      } else {
        store_out(P.curv, P.out_dtype, o, plain_curv(z, P));
      }
    }
    return;
  }
  // FP64 DEMs and int32 DEMs: the reference's formulas in double
  if (P.tri) store_out(P.tri, P.out_dtype, o, plain_tri(z));
  if (P.tpi) store_out(P.tpi, P.out_dtype, o, plain_tpi(z));
  if (P.curv) store_out(P.curv, P.out_dtype, o, plain_curv(z, P));
}

template <typename T>
int launch_deriv(const void* src, const DerivParams& P, int bands, cudaStream_t st) {
  const dim3 grid(static_cast<unsigned>((P.W + kDTW - 1) / kDTW), static_cast<unsigned>((P.H + kDTH - 1) / kDTH),
                  static_cast<unsigned>(bands));
  if (grid.y > 65535u) return fail(VSR_ERR_UNSUPPORTED, "raster too tall for the terrain-derivative grid");
  terrain_deriv_kernel<T><<<grid, dim3(kDTW, kDTH), 0, st>>>(static_cast<const T*>(src), P);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}

}  // namespace
}  // namespace vsr

using namespace vsr;

extern "C" int vsr_terrain_derivatives_bands(const void* dem, int dtype, int bands, int64_t band_stride,
                                             int64_t height, int64_t width, int64_t pitch, double cell_x,
                                             double cell_y, double nodata, int nodata_kind, double nodata_out,
                                             void* tri, void* tpi, void* curvature, int out_dtype,
                                             int64_t out_band_stride, int64_t out_pitch, void* stream) {
  if (height < 0 || width < 0) return fail(VSR_ERR_INVALID_ARG, "negative raster size");
  if (bands < 1 || bands > 65535) return fail(VSR_ERR_INVALID_ARG, "bands must be in [1, 65535]");
  if (height == 0 || width == 0 || (!tri && !tpi && !curvature)) return VSR_OK;
  if (!dem) return fail(VSR_ERR_INVALID_ARG, "dem is NULL");
  const size_t es = dtype_size(dtype);
  if (es == 0) return fail(VSR_ERR_INVALID_ARG, "unsupported dtype %d", dtype);
  if (pitch < width) return fail(VSR_ERR_INVALID_ARG, "pitch %lld < width %lld", (long long)pitch, (long long)width);
  if (out_dtype != VSR_F32 && out_dtype != VSR_F64) return fail(VSR_ERR_INVALID_ARG, "out_dtype must be VSR_F32 or VSR_F64");
  if (out_pitch < width) return fail(VSR_ERR_INVALID_ARG, "out_pitch < width");
  if (bands > 1 && (band_stride < pitch * height || out_band_stride < out_pitch * height))
    return fail(VSR_ERR_INVALID_ARG, "band strides smaller than one band");
  if (!(cell_x > 0.0) || !(cell_y > 0.0) || !std::isfinite(cell_x) || !std::isfinite(cell_y))
    return fail(VSR_ERR_INVALID_ARG, "cell sizes must be positive and finite");
  if (nodata_kind < VSR_NODATA_NONE || nodata_kind > VSR_NODATA_NAN)
    return fail(VSR_ERR_INVALID_ARG, "bad nodata_kind %d", nodata_kind);
  if (!aligned(dem, es)) return fail(VSR_ERR_INVALID_ARG, "dem not aligned to its element size");
  const size_t os = out_dtype == VSR_F64 ? 8 : 4;
  for (void* p : {tri, tpi, curvature})
    if (p && !aligned(p, os)) return fail(VSR_ERR_INVALID_ARG, "outputs not aligned to the output element size");
  DerivParams P{};
  P.H = height;
  P.W = width;
  P.pitch = pitch;
  P.out_pitch = out_pitch;
  P.band_stride = bands > 1 ? band_stride : 0;
  P.out_band_stride = bands > 1 ? out_band_stride : 0;
  P.nd_kind = resolve_nodata(dtype, nodata, nodata_kind, &P.nd_in);
  P.nd_out = nodata_out;
  P.cx2 = cell_x * cell_x;
  P.cy2 = cell_y * cell_y;
  const double icx2 = 1.0 / P.cx2, icy2 = 1.0 / P.cy2;
  P.icx2_hi = static_cast<float>(icx2);
  P.icx2_lo = static_cast<float>(icx2 - static_cast<double>(P.icx2_hi));
  P.icy2_hi = static_cast<float>(icy2);
  P.icy2_lo = static_cast<float>(icy2 - static_cast<double>(P.icy2_hi));
  P.tri = tri;
  P.tpi = tpi;
  P.curv = curvature;
  P.out_dtype = out_dtype;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  switch (dtype) {
    case VSR_U8: return launch_deriv<uint8_t>(dem, P, bands, st);
    case VSR_I16: return launch_deriv<int16_t>(dem, P, bands, st);
    case VSR_U16: return launch_deriv<uint16_t>(dem, P, bands, st);
    case VSR_I32: return launch_deriv<int32_t>(dem, P, bands, st);
    case VSR_F32: return launch_deriv<float>(dem, P, bands, st);
    default: return launch_deriv<double>(dem, P, bands, st);
  }
}

extern "C" int vsr_terrain_derivatives(const void* dem, int dtype, int64_t height, int64_t width, int64_t pitch,
                                       double cell_x, double cell_y, double nodata, int nodata_kind,
                                       double nodata_out, void* tri, void* tpi, void* curvature, int out_dtype,
                                       int64_t out_pitch, void* stream) {
  return vsr_terrain_derivatives_bands(dem, dtype, 1, 0, height, width, pitch, cell_x, cell_y, nodata, nodata_kind,
                                       nodata_out, tri, tpi, curvature, out_dtype, 0, out_pitch, stream);
}
