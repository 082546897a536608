// Horn 3x3 terrain kernels: slope, aspect and hillshade fused into one pass.
//
// Replaces the reference's ``slope_aspect`` and ``hillshade`` NVRTC kernels
// (kernels/focal.py:173-283, 303-467) and the float64 up-cast / uint8 mask /
// down-cast passes of their launch glue (algebra.py:2257-2383, 2632-2775).
//
// Arithmetic (FP32 on CUDA cores):
//   gx = (c - a) + 2 (f - d) + (i - g)      window  a b c
//   gy = (g - a) + 2 (h - b) + (i - c)              d e f
//   p = gx / (8 cell_x), q = gy / (8 cell_y)        g h i
// Differences are formed first: neighbouring elevations are close, so each
// difference is exact (Sterbenz) and the FP32 gradient keeps nearly full
// relative precision even at 4500 m.  1/(8 cell) is formed in FP64 on the
// host.  slope = atan(sqrt(p^2+q^2)) in degrees; aspect =
// (90 - deg(atan2(-q, p))) mod 360 (algebra.py:2240-2243, focal.py:273-279);
// hillshade uses the closed form of cos(zen) cos(slope) + sin(zen) sin(slope)
// cos(az - aspect) with sin/cos(atan r) = r/sqrt(1+r^2), 1/sqrt(1+r^2):
//   hs = (cos zen + sin zen (cos az p' - sin az q')) / sqrt(1 + p'^2 + q'^2)
// with p', q' the z-factor-scaled gradients (focal.py:423-466), clamped to
// [0, 1] and stored as uint8(hs*255 + 0.5) (truncating).
//
// Two kernels:
//  * horn_f32_tma  -- float32 rasters with 16-byte aligned rows.  Persistent
//    CTAs walk 128 x TH output tiles; each tile plus a 4-column / 1-row halo
//    is staged into shared memory by a 2-D TMA load (multi-stage mbarrier
//    pipeline), edge replication is patched in shared memory on border
//    tiles, each lane computes 4 adjacent pixels per row from a rolling
//    3-row register window and writes 128-bit slope/aspect and 32-bit
//    hillshade stores.
//  * horn_generic  -- every other dtype / alignment: one thread per pixel,
//    clamped loads through L1.
#include <mutex>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "vsr_internal.cuh"

namespace vsr {
namespace {

struct HornParams {
  int64_t height, width;
  int64_t in_pitch, out_pitch, hs_pitch;
  float inv8cx, inv8cy;  // 1 / (8 cell) from FP64
  float zf, zf2;
  float cos_z, hs_a, hs_b;  // cos(zen); sin(zen) cos(az) zf; sin(zen) sin(az) zf
  float nd_out_f;   // nodata written to float slope/aspect
  double nd_out_d;  // nodata written to double slope/aspect
  uint32_t flags;
  int nd_kind;      // resolved VSR_NODATA_*
};

// Which masks apply, from the resolved nodata kind and the flags.
struct MaskRule {
  bool sa_any;     // slope/aspect masked at all
  bool sa_center;  // centre-only (reference GPU) instead of 3x3 dilation
  bool hs_any;     // hillshade masked (always 3x3 dilation)
};

__device__ __forceinline__ MaskRule mask_rule(const HornParams& P) {
  MaskRule m;
  m.hs_any = P.nd_kind != VSR_NODATA_NONE;
  m.sa_any = m.hs_any && !(P.nd_kind == VSR_NODATA_NAN && (P.flags & VSR_HORN_SA_NAN_UNMASKED));
  m.sa_center = (P.flags & VSR_HORN_CENTER_ONLY) != 0;
  return m;
}

struct PixelOut {
  float slope, aspect;
  uint8_t hs;
};

// Degree-valued arctangent on t in [0, 1]: t * P(t^2), P the degree-7
// minimax polynomial fitted by csrc/fit_atan.py (max error 2.1e-6 deg in
// float64, 7.6e-6 deg evaluated in float32).
__device__ __forceinline__ float atan_poly_deg(float t) {
  const float u = t * t;
  float p = -0.232309317f;
  p = fmaf(p, u, 1.2526542f);
  p = fmaf(p, u, -3.20353885f);
  p = fmaf(p, u, 5.52457099f);
  p = fmaf(p, u, -7.96905727f);
  p = fmaf(p, u, 11.4285402f);
  p = fmaf(p, u, -19.0966035f);
  p = fmaf(p, u, 57.2957414f);
  return t * p;
}

__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Slope in degrees from s = p^2 + q^2: atan(r), r = sqrt(s), reduced to
// t = min(r, 1/r) with one rsqrt (r = s * rsqrt(s), 1/r = rsqrt(s)).
// s = 0 gives exactly 0; NaN propagates (the select keeps s * rsqrt).
__device__ __forceinline__ float slope_deg(float s) {
  const float rs = rsqrt_approx(s + 1e-30f);
  const bool big = s > 1.0f;
  const float t = big ? rs : s * rs;
  const float a = atan_poly_deg(t);
  return big ? 90.0f - a : a;
}

// Aspect in compass degrees: (90 - atan2(-q, p) in degrees) mod 360.  The
// octant reduction keeps the axes exact (due north 0, east 90, south 180,
// west 270, flat 90 as atan2(-0, +0) = -0 gives).  The min/max are selects
// on a comparison, so a NaN operand lands in t and propagates to the result.
__device__ __forceinline__ float aspect_deg(float p, float q) {
  const float ap = fabsf(p), aq = fabsf(q);
  const bool sw = aq > ap;
  const float mx = sw ? aq : ap, mn = sw ? ap : aq;
  const float t = mn * rcp_approx(mx + 1e-30f);
  float a = atan_poly_deg(t);
  a = sw ? 90.0f - a : a;           // |atan2| folded into [0, 90]
  a = p < 0.0f ? 180.0f - a : a;    // [0, 180]
  // atan2(-q, p) = +a for q <= 0, -a for q > 0; aspect = 90 - atan2
  float asp = fmaf(q > 0.0f ? 1.0f : -1.0f, a, 90.0f);
  return asp < 0.0f ? asp + 360.0f : asp;
}

// Hillshade byte from the unscaled gradient (p, q) and s = p^2 + q^2:
// (cos zen + sin zen (cos az p' - sin az q')) / sqrt(1 + p'^2 + q'^2) with
// p' = zf p, q' = zf q, saturated to [0, 1] (NaN -> 0), uint8(hs*255 + 0.5).
__device__ __forceinline__ uint8_t hillshade_u8(float p, float q, float s, const HornParams& P) {
  const float num = fmaf(P.hs_a, p, fmaf(-P.hs_b, q, P.cos_z));
  const float hs = __saturatef(num * rsqrt_approx(fmaf(P.zf2, s, 1.0f)));
  return static_cast<uint8_t>(__float2uint_rz(fmaf(hs, 255.0f, 0.5f)));
}

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

constexpr int kWantSlope = 1, kWantAspect = 2, kWantHs = 4;

// ---- the same arithmetic on pixel pairs with Blackwell's packed FP32
// instructions (fma/mul/add .f32x2: two IEEE single-precision results per
// instruction, rounded exactly as the scalar forms).  Selects, compares and
// the MUFU approximations stay per element.  The fused kernel is
// instruction-issue bound at about the HBM rate in scalar form; pairing
// halves its FP instruction count.
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sel2(bool c0, bool c1, float2 a, float2 b) {
  return make_float2(c0 ? a.x : b.x, c1 ? a.y : b.y);
}

__device__ __forceinline__ float2 atan_poly_deg2(float2 t) {
  const float2 u = mul2(t, t);
  float2 p = f2(-0.232309317f);
  p = fma2(p, u, f2(1.2526542f));
  p = fma2(p, u, f2(-3.20353885f));
  p = fma2(p, u, f2(5.52457099f));
  p = fma2(p, u, f2(-7.96905727f));
  p = fma2(p, u, f2(11.4285402f));
  p = fma2(p, u, f2(-19.0966035f));
  p = fma2(p, u, f2(57.2957414f));
  return mul2(t, p);
}

__device__ __forceinline__ float2 slope_deg2(float2 s) {
  const float2 sp = add2(s, f2(1e-30f));
  const float2 rs = make_float2(rsqrt_approx(sp.x), rsqrt_approx(sp.y));
  const bool b0 = s.x > 1.0f, b1 = s.y > 1.0f;
  const float2 t = sel2(b0, b1, rs, mul2(s, rs));
  const float2 a = atan_poly_deg2(t);
  return sel2(b0, b1, fma2(a, f2(-1.0f), f2(90.0f)), a);
}

__device__ __forceinline__ float2 aspect_deg2(float2 p, float2 q) {
  const float ap0 = fabsf(p.x), aq0 = fabsf(q.x), ap1 = fabsf(p.y), aq1 = fabsf(q.y);
  const bool w0 = aq0 > ap0, w1 = aq1 > ap1;
  const float2 mx = make_float2(w0 ? aq0 : ap0, w1 ? aq1 : ap1);
  const float2 mn = make_float2(w0 ? ap0 : aq0, w1 ? ap1 : aq1);
  const float2 mxe = add2(mx, f2(1e-30f));
  const float2 t = mul2(mn, make_float2(rcp_approx(mxe.x), rcp_approx(mxe.y)));
  float2 a = atan_poly_deg2(t);
  a = sel2(w0, w1, fma2(a, f2(-1.0f), f2(90.0f)), a);
  a = sel2(p.x < 0.0f, p.y < 0.0f, fma2(a, f2(-1.0f), f2(180.0f)), a);
  const float2 asp = fma2(make_float2(q.x > 0.0f ? 1.0f : -1.0f, q.y > 0.0f ? 1.0f : -1.0f), a, f2(90.0f));
  return sel2(asp.x < 0.0f, asp.y < 0.0f, add2(asp, f2(360.0f)), asp);
}

__device__ __forceinline__ void hillshade_u8_2(float2 p, float2 q, float2 s, const HornParams& P, uint8_t& h0,
                                               uint8_t& h1) {
  const float2 num = fma2(f2(P.hs_a), p, fma2(f2(-P.hs_b), q, f2(P.cos_z)));
  const float2 d = fma2(f2(P.zf2), s, f2(1.0f));
  const float2 hr = mul2(num, make_float2(rsqrt_approx(d.x), rsqrt_approx(d.y)));
  const float2 hs = make_float2(__saturatef(hr.x), __saturatef(hr.y));
  const float2 v = fma2(hs, f2(255.0f), f2(0.5f));
  h0 = static_cast<uint8_t>(__float2uint_rz(v.x));
  h1 = static_cast<uint8_t>(__float2uint_rz(v.y));
}

// Two pixels: gradients (gx, gy) of pixel 0 in .x, pixel 1 in .y.
template <int WANT>
__device__ __forceinline__ void horn_px2(float2 gx, float2 gy, const HornParams& P, float& s0, float& s1, float& a0,
                                         float& a1, uint8_t& h0, uint8_t& h1) {
  const float2 p = mul2(gx, f2(P.inv8cx));
  const float2 q = mul2(gy, f2(P.inv8cy));
  const float2 s = fma2(p, p, mul2(q, q));
  if (WANT & kWantSlope) {
    const float2 v = slope_deg2(s);
    s0 = v.x;
    s1 = v.y;
  }
  if (WANT & kWantAspect) {
    const float2 v = aspect_deg2(p, q);
    a0 = v.x;
    a1 = v.y;
  }
  if (WANT & kWantHs) hillshade_u8_2(p, q, s, P, h0, h1);
}

// The wanted outputs are a compile-time set, so the per-pixel path has no
// branches on which outputs exist.
template <int WANT>
__device__ __forceinline__ void horn_px(float gx, float gy, const HornParams& P, float& so, float& ao, uint8_t& ho) {
  const float p = gx * P.inv8cx;
  const float q = gy * P.inv8cy;
  const float s = fmaf(p, p, q * q);
  if (WANT & kWantSlope) so = slope_deg(s);
  if (WANT & kWantAspect) ao = aspect_deg(p, q);
  if (WANT & kWantHs) ho = hillshade_u8(p, q, s, P);
}

// ---- exact gradients.  Differences of neighbouring FP32 elevations are
// exact when the operands lie within a factor of two of each other
// (Sterbenz), which holds almost everywhere; near 0 m (or where values of
// very different size meet, e.g. nodata) a difference can round, and a
// small gradient formed from large rounded differences loses the aspect's
// accuracy (the reference differences in float64).  Rows where that can
// happen take error-free transformations instead: TwoDiff/TwoSum keep every
// rounding error and the sum is formed to within one final rounding.
__device__ __forceinline__ float2 two_diff(float a, float b) {  // s + e == a - b exactly
  const float s = __fsub_rn(a, b);
  const float z = __fsub_rn(s, a);
  const float e = __fsub_rn(__fsub_rn(a, __fsub_rn(s, z)), __fadd_rn(b, z));
  return make_float2(s, e);
}
__device__ __forceinline__ float2 two_sum(float a, float b) {  // s + e == a + b exactly
  const float s = __fadd_rn(a, b);
  const float z = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, z)), __fsub_rn(b, z));
  return make_float2(s, e);
}
// (x2 - x0) + 2 (y2 - y0) + (z2 - z0), correctly rounded but for a tiny
// fraction of an ulp; non-finite operands fall back to plain arithmetic.
__device__ __forceinline__ float grad_exact(float x0, float x2, float y0, float y2, float z0, float z2) {
  const float2 d1 = two_diff(x2, x0), d2 = two_diff(y2, y0), d3 = two_diff(z2, z0);
  const float2 s12 = two_sum(d1.x, 2.0f * d2.x);
  const float2 s = two_sum(s12.x, d3.x);
  const float err = __fadd_rn(__fadd_rn(s12.y, s.y), __fadd_rn(__fadd_rn(d1.y, 2.0f * d2.y), d3.y));
  const float g = __fadd_rn(s.x, err);
  return fabsf(g) <= 3.402823466e38f ? g : fmaf(2.0f, y2 - y0, (x2 - x0) + (z2 - z0));
}

// Three-input FP32 min / max (sm_100 and later; NaN inputs are ignored as by
// fminf / fmaxf).  The exactness test's range only picks the gradient form,
// so a NaN range simply selects the exact form.
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float max3f(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// Every difference (and the sums) of a row window is exact when all its
// values lie in [m, 2m] for some m > 0, or in [-2m, -m], or are all zero.
__device__ __forceinline__ bool window_exact(float lo, float hi) {
  return (lo > 0.0f && hi <= 2.0f * lo) || (hi < 0.0f && lo >= 2.0f * hi) || (lo == 0.0f && hi == 0.0f);
}

// ------------------------------------------------------------ TMA kernel --
constexpr int kTW = 128;        // output tile width (32 lanes x 4 pixels)
constexpr int kSW = kTW + 8;    // staged width: 4-column halo each side (16 B)

template <int TH>
struct TmaTile {
  static constexpr int SH = TH + 2;
  static constexpr uint32_t kBytes = kSW * SH * 4;
  static constexpr uint32_t kStride = (kBytes + 1023u) & ~1023u;
};

// Shared-memory output tile for TMA stores: slope and aspect TH x 128 f32,
// hillshade TH x 128 u8 (only the wanted ones), 1024-byte aligned.
template <int TH, int WANT>
struct OutTile {
  static constexpr uint32_t kSB = (WANT & 1) ? TH * kTW * 4 : 0;
  static constexpr uint32_t kAB = (WANT & 2) ? TH * kTW * 4 : 0;
  static constexpr uint32_t kHB = (WANT & 4) ? TH * kTW : 0;
  static constexpr uint32_t kS = 0, kA = kSB, kH = kSB + kAB;
  static constexpr uint32_t kBytes = (kSB + kAB + kHB + 1023u) & ~1023u;
};

__device__ __forceinline__ void load6(const float* row, int lane, float v[6]) {
  const float4 m = *reinterpret_cast<const float4*>(row + 4 + 4 * lane);
  v[0] = row[3 + 4 * lane];
  v[1] = m.x;
  v[2] = m.y;
  v[3] = m.z;
  v[4] = m.w;
  v[5] = row[8 + 4 * lane];
}

__device__ __forceinline__ bool is_nd(float v, int kind, float ndv) {
  return kind == VSR_NODATA_VALUE ? (v == ndv) : (kind == VSR_NODATA_NAN ? (v != v) : false);
}

__device__ __forceinline__ uint32_t nd_bits6(const float v[6], int kind, float ndv) {
  uint32_t m = 0;
#pragma unroll
  for (int k = 0; k < 6; ++k) m |= (is_nd(v[k], kind, ndv) ? 1u : 0u) << k;
  return m;
}

// Load one staged row for a lane: 6 values, its 4 horizontal differences
// (x+2 minus x, shared by the three output rows that use the row) and, for
// masked tiles, its 6 nodata bits.
// Also the row's value range for the exactness test; with ``skip_nd``
// nodata values are left out (their windows' outputs are masked).
template <bool MASKED>
__device__ __forceinline__ void stage_row(const float* row, int lane, const HornParams& P, float nd_in, bool skip_nd,
                                          float v[6], float hd[4], uint32_t& m, float& lo, float& hi) {
  load6(row, lane, v);
#pragma unroll
  for (int k = 0; k < 4; ++k) hd[k] = v[k + 2] - v[k];
  m = MASKED ? nd_bits6(v, P.nd_kind, nd_in) : 0u;
  if (MASKED && skip_nd && m) {
    float l[6], h[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const bool nd = (m >> k) & 1u;
      l[k] = nd ? __int_as_float(0x7f800000) : v[k];
      h[k] = nd ? __int_as_float(0xff800000) : v[k];
    }
    lo = fminf(min3f(l[0], l[1], l[2]), min3f(l[3], l[4], l[5]));
    hi = fmaxf(max3f(h[0], h[1], h[2]), max3f(h[3], h[4], h[5]));
  } else {
    lo = fminf(min3f(v[0], v[1], v[2]), min3f(v[3], v[4], v[5]));
    hi = fmaxf(max3f(v[0], v[1], v[2]), max3f(v[3], v[4], v[5]));
  }
}

// One output row (4 pixels of this lane) from the rows above (t) and below
// (b), the three rows' horizontal differences and nodata bits.
// TO_SMEM: the row pointers address a shared-memory output tile (plain
// stores; the streaming global stores below must not see a shared address).
// Gradients of a lane's 4 pixels from the rows above (t), through (mid)
// and below (b) and the rows' horizontal differences: the fast form from
// the (exact) differences, or grad_exact where differences may round.
__device__ __forceinline__ void grad_fast(const float t[6], const float b[6], const float hdt[4], const float hdm[4],
                                          const float hdb[4], float gx[4], float gy[4]) {
  float dv[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) dv[k] = b[k] - t[k];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    gx[k] = fmaf(2.0f, hdm[k], hdt[k] + hdb[k]);
    gy[k] = fmaf(2.0f, dv[k + 1], dv[k] + dv[k + 2]);
  }
}

__device__ __forceinline__ void grad_exact4(const float t[6], const float mid[6], const float b[6], float gx[4],
                                            float gy[4]) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    gx[k] = grad_exact(t[k], t[k + 2], mid[k], mid[k + 2], b[k], b[k + 2]);
    gy[k] = grad_exact(t[k], b[k], t[k + 1], b[k + 1], t[k + 2], b[k + 2]);
  }
}

template <int WANT, bool MASKED, bool EDGE, bool VEC = true, bool TO_SMEM = false>
__device__ __forceinline__ void horn_out_row(const float gx[4], const float gy[4], uint32_t mt, uint32_t mm,
                                             uint32_t mb, const HornParams& P, const MaskRule& rule, int64_t y,
                                             int64_t xs, float* __restrict__ srow, float* __restrict__ arow,
                                             uint8_t* __restrict__ hrow) {
  if (EDGE && (y >= P.height || xs >= P.width)) return;
  float so[4], ao[4];
  uint8_t ho[4];
#pragma unroll
  for (int k = 0; k < 4; k += 2)
    horn_px2<WANT>(make_float2(gx[k], gx[k + 1]), make_float2(gy[k], gy[k + 1]), P, so[k], so[k + 1], ao[k],
                   ao[k + 1], ho[k], ho[k + 1]);
  if (MASKED) {
    const uint32_t hdil = (mt | (mt >> 1) | (mt >> 2)) | (mm | (mm >> 1) | (mm >> 2)) | (mb | (mb >> 1) | (mb >> 2));
    const uint32_t sabits = rule.sa_any ? (rule.sa_center ? (mm >> 1) : hdil) : 0u;
    const uint32_t hsbits = rule.hs_any ? hdil : 0u;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const bool sa_nd = (sabits >> k) & 1u;
      so[k] = sa_nd ? P.nd_out_f : so[k];
      ao[k] = sa_nd ? P.nd_out_f : ao[k];
      ho[k] = ((hsbits >> k) & 1u) ? uint8_t(0) : ho[k];
    }
  }
  const bool full = VEC && (!EDGE || xs + 3 < P.width);
  if (TO_SMEM) {
    if (WANT & kWantSlope) *reinterpret_cast<float4*>(srow) = make_float4(so[0], so[1], so[2], so[3]);
    if (WANT & kWantAspect) *reinterpret_cast<float4*>(arow) = make_float4(ao[0], ao[1], ao[2], ao[3]);
    if (WANT & kWantHs)
      *reinterpret_cast<unsigned int*>(hrow) =
          uint32_t(ho[0]) | (uint32_t(ho[1]) << 8) | (uint32_t(ho[2]) << 16) | (uint32_t(ho[3]) << 24);
  } else if (full) {
    if (WANT & kWantSlope) __stcs(reinterpret_cast<float4*>(srow), make_float4(so[0], so[1], so[2], so[3]));
    if (WANT & kWantAspect) __stcs(reinterpret_cast<float4*>(arow), make_float4(ao[0], ao[1], ao[2], ao[3]));
    if (WANT & kWantHs)
      __stcs(reinterpret_cast<unsigned int*>(hrow), uint32_t(ho[0]) | (uint32_t(ho[1]) << 8) |
                                                         (uint32_t(ho[2]) << 16) | (uint32_t(ho[3]) << 24));
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (xs + k < P.width) {
        if (WANT & kWantSlope) srow[k] = so[k];
        if (WANT & kWantAspect) arow[k] = ao[k];
        if (WANT & kWantHs) hrow[k] = ho[k];
      }
    }
  }
}

// RB output rows of one warp: rows r0 .. r0+RB-1 of the tile (staged rows
// r0 .. r0+RB+1), lane columns xs .. xs+3.  Two output rows per iteration
// (rolled on purpose: a fully unrolled loop overflowed the instruction cache).
// ``srow``/``arow``/``hrow`` point at this lane's first output pixel (global
// memory, or a shared-memory staging tile for TMA stores); ``sp``/``hp``
// are their row pitches in elements.
template <int RB, int WANT, bool MASKED, bool EDGE, bool VEC = true, bool TO_SMEM = false>
__device__ __forceinline__ void horn_rows(const float* S, int lane, int r0, int64_t y0, int64_t xs,
                                          const HornParams& P, const MaskRule& rule, float nd_in,
                                          float* __restrict__ srow, float* __restrict__ arow,
                                          uint8_t* __restrict__ hrow, int64_t sp, int64_t hp) {
  static_assert(RB % 2 == 0, "two output rows per iteration");
  float v0[6], v1[6], hd0[4], hd1[4];
  uint32_t m0, m1;
  float lo0, hi0, lo1, hi1;
  // nodata values may be left out of the exactness test when every output
  // whose window holds one is masked (3x3 dilation; not the centre-only rule)
  const bool skip_nd = !rule.sa_center;
  stage_row<MASKED>(S + (r0 + 0) * kSW, lane, P, nd_in, skip_nd, v0, hd0, m0, lo0, hi0);
  stage_row<MASKED>(S + (r0 + 1) * kSW, lane, P, nd_in, skip_nd, v1, hd1, m1, lo1, hi1);
  const int64_t y = y0 + r0;
#pragma unroll 1
  for (int j = 0; j < RB; j += 2) {
    float v2[6], v3[6], hd2[4], hd3[4];
    uint32_t m2, m3;
    float lo2, hi2, lo3, hi3;
    stage_row<MASKED>(S + (r0 + j + 2) * kSW, lane, P, nd_in, skip_nd, v2, hd2, m2, lo2, hi2);
    stage_row<MASKED>(S + (r0 + j + 3) * kSW, lane, P, nd_in, skip_nd, v3, hd3, m3, lo3, hi3);
    // both output rows of the pair take the exact form if any lane's window may round
    const float lo = fminf(min3f(lo0, lo1, lo2), lo3), hi = fmaxf(max3f(hi0, hi1, hi2), hi3);
    float* srow1 = (WANT & kWantSlope) ? srow + sp : nullptr;
    float* arow1 = (WANT & kWantAspect) ? arow + sp : nullptr;
    uint8_t* hrow1 = (WANT & kWantHs) ? hrow + hp : nullptr;
    float gxa[4], gya[4], gxb[4], gyb[4];
    if (__all_sync(0xffffffffu, window_exact(lo, hi))) {
      grad_fast(v0, v2, hd0, hd1, hd2, gxa, gya);
      grad_fast(v1, v3, hd1, hd2, hd3, gxb, gyb);
    } else {
      grad_exact4(v0, v1, v2, gxa, gya);
      grad_exact4(v1, v2, v3, gxb, gyb);
    }
    horn_out_row<WANT, MASKED, EDGE, VEC, TO_SMEM>(gxa, gya, m0, m1, m2, P, rule, y + j, xs, srow, arow, hrow);
    horn_out_row<WANT, MASKED, EDGE, VEC, TO_SMEM>(gxb, gyb, m1, m2, m3, P, rule, y + j + 1, xs, srow1, arow1, hrow1);
    if (WANT & kWantSlope) srow = srow1 + sp;
    if (WANT & kWantAspect) arow = arow1 + sp;
    if (WANT & kWantHs) hrow = hrow1 + hp;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      v0[k] = v2[k];
      v1[k] = v3[k];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      hd0[k] = hd2[k];
      hd1[k] = hd3[k];
    }
    m0 = m2;
    m1 = m3;
    lo0 = lo2;
    hi0 = hi2;
    lo1 = lo3;
    hi1 = hi3;
  }
}

// This lane's first output pixel of rows starting at y in global memory.
struct RowPtrs {
  float* s;
  float* a;
  uint8_t* h;
};
__device__ __forceinline__ RowPtrs global_rows(float* slope, float* aspect, uint8_t* hs, const HornParams& P,
                                               int64_t y, int64_t xs) {
  return {slope ? slope + y * P.out_pitch + xs : nullptr, aspect ? aspect + y * P.out_pitch + xs : nullptr,
          hs ? hs + y * P.hs_pitch + xs : nullptr};
}

// OB = 0: each lane stores its results straight to global memory.  OB >= 1:
// results go to OB shared-memory output tiles that one thread writes back
// with TMA tensor stores (bulk groups; a tile is rewritten only after its
// store has finished reading it).  The copy engine keeps far more writes in
// flight than the CTA's threads can, and the kernel's traffic is two thirds
// writes.
template <int TH, int STAGES, int THREADS, int WANT, int OB, int MINB = 768 / THREADS>
__global__ void __launch_bounds__(THREADS, MINB) horn_f32_tma(const __grid_constant__ CUtensorMap tmap,
                                                        const __grid_constant__ CUtensorMap smap,
                                                        const __grid_constant__ CUtensorMap amap,
                                                        const __grid_constant__ CUtensorMap hmap,
                                                        const HornParams P, const float nd_in,
                                                        float* __restrict__ slope,
                                                        float* __restrict__ aspect,
                                                        uint8_t* __restrict__ hs,
                                                        uint32_t* err_word) {
  using Tile = TmaTile<TH>;
  using Out = OutTile<TH, WANT>;
  constexpr int WARPS = THREADS / 32;
  constexpr int RB = TH / WARPS;  // output rows per warp
  static_assert(RB * WARPS == TH, "TH must be a multiple of the warp count");
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[STAGES];
  float* stages = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* out_base = reinterpret_cast<unsigned char*>(stages) + STAGES * Tile::kStride;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t W = P.width, H = P.height;
  const int64_t tiles_x = (W + kTW - 1) / kTW;
  const int64_t total = tiles_x * ((H + TH - 1) / TH);
  const MaskRule rule = mask_rule(P);

  auto issue = [&](int64_t t, int s) {
    const int64_t ty = t / tiles_x, tx = t - ty * tiles_x;
    mbar_arrive_expect_tx(&bars[s], Tile::kBytes);
    tma_load_2d(reinterpret_cast<unsigned char*>(stages) + s * Tile::kStride, &tmap,
                static_cast<int>(tx * kTW - 4), static_cast<int>(ty * TH - 1), &bars[s]);
  };

  if (tid == 0) {
    prefetch_tensormap(&tmap);
    for (int s = 0; s < STAGES; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      const int64_t t = blockIdx.x + static_cast<int64_t>(s) * gridDim.x;
      if (t < total) issue(t, s);
    }
  }

  int64_t it = 0;
  for (int64_t t = blockIdx.x; t < total; t += gridDim.x, ++it) {
    const int s = static_cast<int>(it % STAGES);
    const uint32_t parity = static_cast<uint32_t>((it / STAGES) & 1);
    const bool ok = mbar_wait_bounded(&bars[s], parity, err_word, kDevErrTmaTimeout);
    // output tile it % OB is rewritten below: its previous store must have read it
    if (OB > 0 && tid == 0) bulk_wait_read<OB - 1>();
    if (__syncthreads_or(!ok)) {
      if (OB > 0 && tid == 0) bulk_wait_read<0>();
      // Give the other copies in flight a bounded chance to land before the
      // CTA's shared memory is released, then leave.
      if (tid == 0) {
        for (int k = 1; k < STAGES; ++k) {
          const int64_t it2 = it + k;
          if (blockIdx.x + it2 * gridDim.x < total)
            mbar_wait_bounded(&bars[it2 % STAGES], static_cast<uint32_t>((it2 / STAGES) & 1), err_word,
                              kDevErrTmaTimeout);
        }
      }
      __syncthreads();
      return;
    }
    float* S = stages + s * (Tile::kStride / 4);
    const int64_t ty = t / tiles_x, tx = t - ty * tiles_x;
    const int64_t x0 = tx * kTW, y0 = ty * TH;

    // Edge replication in shared memory (TMA fills out-of-range with zeros).
    const bool left = x0 == 0, right = x0 + kTW >= W, top = y0 == 0, bottom = y0 + TH >= H;
    if (left || right) {
      const int rc = static_cast<int>(W - x0) + 4;  // staged column of x = W
      for (int r = tid; r < Tile::SH; r += THREADS) {
        if (left) S[r * kSW + 3] = S[r * kSW + 4];
        if (right) S[r * kSW + rc] = S[r * kSW + rc - 1];
      }
    }
    if (top || bottom) {
      __syncthreads();
      const int rr = static_cast<int>(H - y0) + 1;  // staged row of y = H
      for (int c = tid; c < kSW; c += THREADS) {
        if (top) S[c] = S[kSW + c];
        if (bottom) S[rr * kSW + c] = S[(rr - 1) * kSW + c];
      }
    }
    // Does the staged tile hold any nodata at all?  Clean tiles skip every
    // mask operation.
    bool any_nd = false;
    if (P.nd_kind != VSR_NODATA_NONE) {
      __syncthreads();
      const float4* S4 = reinterpret_cast<const float4*>(S);
      for (int i = tid; i < Tile::SH * kSW / 4; i += THREADS) {
        const float4 v = S4[i];
        any_nd |= is_nd(v.x, P.nd_kind, nd_in) | is_nd(v.y, P.nd_kind, nd_in) |
                  is_nd(v.z, P.nd_kind, nd_in) | is_nd(v.w, P.nd_kind, nd_in);
      }
    }
    const bool masked = __syncthreads_or(any_nd);

    const int64_t xs = x0 + 4 * lane;
    const int r0 = warp * RB;
    if (OB > 0) {
      // whole tile into shared memory (pixels past the raster edge are
      // computed from the replicated halo and clipped by the tensor store)
      unsigned char* ob = out_base + static_cast<uint32_t>(it % (OB > 0 ? OB : 1)) * Out::kBytes;
      float* so = reinterpret_cast<float*>(ob + Out::kS) + r0 * kTW + 4 * lane;
      float* ao = reinterpret_cast<float*>(ob + Out::kA) + r0 * kTW + 4 * lane;
      uint8_t* ho = ob + Out::kH + r0 * kTW + 4 * lane;
      if (masked) horn_rows<RB, WANT, true, false, true, true>(S, lane, r0, y0, xs, P, rule, nd_in, so, ao, ho, kTW, kTW);
      else horn_rows<RB, WANT, false, false, true, true>(S, lane, r0, y0, xs, P, rule, nd_in, so, ao, ho, kTW, kTW);
      fence_proxy_async_smem();  // generic-proxy tile writes -> visible to the tensor store
    } else {
      const bool edge = x0 + kTW > W || y0 + TH > H;
      const RowPtrs g = global_rows(slope, aspect, hs, P, y0 + r0, xs);
      if (masked) {
        if (edge) horn_rows<RB, WANT, true, true>(S, lane, r0, y0, xs, P, rule, nd_in, g.s, g.a, g.h, P.out_pitch, P.hs_pitch);
        else horn_rows<RB, WANT, true, false>(S, lane, r0, y0, xs, P, rule, nd_in, g.s, g.a, g.h, P.out_pitch, P.hs_pitch);
      } else {
        if (edge) horn_rows<RB, WANT, false, true>(S, lane, r0, y0, xs, P, rule, nd_in, g.s, g.a, g.h, P.out_pitch, P.hs_pitch);
        else horn_rows<RB, WANT, false, false>(S, lane, r0, y0, xs, P, rule, nd_in, g.s, g.a, g.h, P.out_pitch, P.hs_pitch);
      }
    }

    __syncthreads();  // every read of stage s (and every write of the output tile) is done
    if (OB > 0 && tid == 0) {
      const unsigned char* ob = out_base + static_cast<uint32_t>(it % (OB > 0 ? OB : 1)) * Out::kBytes;
      if (WANT & kWantSlope) tma_store_2d(&smap, static_cast<int>(x0), static_cast<int>(y0), ob + Out::kS);
      if (WANT & kWantAspect) tma_store_2d(&amap, static_cast<int>(x0), static_cast<int>(y0), ob + Out::kA);
      if (WANT & kWantHs) tma_store_2d(&hmap, static_cast<int>(x0), static_cast<int>(y0), ob + Out::kH);
      bulk_commit();
    }
    if (tid == 0) {
      const int64_t nt = t + static_cast<int64_t>(STAGES) * gridDim.x;
      if (nt < total) {
        fence_proxy_async_smem();  // order the generic-proxy edge patches before the TMA refill
        issue(nt, s);
      }
    }
  }
  if (OB > 0 && tid == 0) bulk_wait_read<0>();  // the last stores must read the tiles before the CTA exits
}

// -------------------------------------------------------- generic kernel --
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
  dim3 grid(static_cast<unsigned>((P.width + 31) / 32), static_cast<unsigned>((P.height + 7) / 8));
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

template <int TH, int STAGES, int THREADS, int WANT, int OB, int MINB = 768 / THREADS>
int launch_tma(const void* src, const HornParams& P, float nd_in, float* slope, float* aspect,
               uint8_t* hs, cudaStream_t st) {
  using Tile = TmaTile<TH>;
  using Out = OutTile<TH, WANT>;
  if (OB > 0 && hs && (!aligned(hs, 16) || P.hs_pitch % 16 != 0))  // tensor-store rows need 16-byte strides
    return launch_tma<TH, STAGES, THREADS, WANT, 0, MINB>(src, P, nd_in, slope, aspect, hs, st);
  CUtensorMap map, smap, amap, hmap;
  int rc = encode_tensor_map_2d(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, src, P.width, P.height,
                                P.in_pitch, kSW, Tile::SH);
  if (rc) return rc;
  smap = amap = hmap = map;  // unused output maps are never read
  if (OB > 0) {
    if (slope && (rc = encode_tensor_map_2d(&smap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, slope, P.width, P.height,
                                            P.out_pitch, kTW, TH)))
      return rc;
    if (aspect && (rc = encode_tensor_map_2d(&amap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, aspect, P.width, P.height,
                                             P.out_pitch, kTW, TH)))
      return rc;
    if (hs && (rc = encode_tensor_map_2d(&hmap, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, hs, P.width, P.height, P.hs_pitch,
                                         kTW, TH)))
      return rc;
  }
  uint32_t* err = device_error_word();
  if (!err) return VSR_ERR_CUDA;
  const size_t smem = STAGES * Tile::kStride + OB * Out::kBytes + 1024;
  auto kern = horn_f32_tma<TH, STAGES, THREADS, WANT, OB, MINB>;
  VSR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  int per_sm = 0;
  VSR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, THREADS, smem));
  if (per_sm < 1) return fail(VSR_ERR_CUDA, "horn_f32_tma cannot be resident (smem %zu)", smem);
  const int64_t tiles = ((P.width + kTW - 1) / kTW) * ((P.height + TH - 1) / TH);
  const int64_t grid = std::min<int64_t>(tiles, static_cast<int64_t>(sm_count()) * per_sm);
  kern<<<static_cast<unsigned>(grid), THREADS, smem, st>>>(map, smap, amap, hmap, P, nd_in, slope, aspect, hs, err);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}

// Launch configurations of the TMA kernel the autotuner chooses between:
// (output rows per tile, pipeline stages, threads per CTA, shared-memory
// output tiles for TMA stores; 0 = direct stores).
struct HornConfig {
  int th, stages, threads, ob, minb;  // minb: CTAs per SM the register budget is sized for
};
constexpr HornConfig kHornConfigs[] = {{64, 2, 128, 0, 4}, {32, 2, 128, 0, 4}, {32, 2, 128, 0, 5},
                                       {32, 2, 128, 0, 6}, {64, 2, 256, 0, 3}, {32, 3, 128, 0, 4},
                                       {32, 2, 256, 2, 3}, {16, 2, 256, 2, 3}};
constexpr int kNumHornConfigs = sizeof(kHornConfigs) / sizeof(kHornConfigs[0]);

template <int WANT>
int launch_tma_want(int cfg, const void* src, const HornParams& P, float nd_in, float* slope, float* aspect,
                    uint8_t* hs, cudaStream_t st) {
  switch (cfg) {
    case 1: return launch_tma<32, 2, 128, WANT, 0, 4>(src, P, nd_in, slope, aspect, hs, st);
    case 2: return launch_tma<32, 2, 128, WANT, 0, 5>(src, P, nd_in, slope, aspect, hs, st);
    case 3: return launch_tma<32, 2, 128, WANT, 0, 6>(src, P, nd_in, slope, aspect, hs, st);
    case 4: return launch_tma<64, 2, 256, WANT, 0, 3>(src, P, nd_in, slope, aspect, hs, st);
    case 5: return launch_tma<32, 3, 128, WANT, 0, 4>(src, P, nd_in, slope, aspect, hs, st);
    case 6: return launch_tma<32, 2, 256, WANT, 2, 3>(src, P, nd_in, slope, aspect, hs, st);
    case 7: return launch_tma<16, 2, 256, WANT, 2, 3>(src, P, nd_in, slope, aspect, hs, st);
    default: return launch_tma<64, 2, 128, WANT, 0, 4>(src, P, nd_in, slope, aspect, hs, st);
  }
}

int launch_tma_config(int cfg, const void* src, const HornParams& P, float nd_in, float* slope,
                      float* aspect, uint8_t* hs, cudaStream_t st) {
  const int want = (slope ? kWantSlope : 0) | (aspect ? kWantAspect : 0) | (hs ? kWantHs : 0);
  switch (want) {
    case 1: return launch_tma_want<1>(cfg, src, P, nd_in, slope, aspect, hs, st);
    case 2: return launch_tma_want<2>(cfg, src, P, nd_in, slope, aspect, hs, st);
    case 3: return launch_tma_want<3>(cfg, src, P, nd_in, slope, aspect, hs, st);
    case 4: return launch_tma_want<4>(cfg, src, P, nd_in, slope, aspect, hs, st);
    case 5: return launch_tma_want<5>(cfg, src, P, nd_in, slope, aspect, hs, st);
    case 6: return launch_tma_want<6>(cfg, src, P, nd_in, slope, aspect, hs, st);
    default: return launch_tma_want<7>(cfg, src, P, nd_in, slope, aspect, hs, st);
  }
}

}  // namespace

int horn_config_count() { return kNumHornConfigs; }

}  // namespace vsr

extern "C" int vsr_horn_fused(const void* dem, int dtype, int64_t height, int64_t width, int64_t pitch,
                              double cell_x, double cell_y, double nodata, int nodata_kind,
                              uint32_t flags, void* slope, void* aspect, int out_dtype,
                              int64_t out_pitch, uint8_t* hillshade, int64_t hs_pitch,
                              double z_factor, double zenith_rad, double azimuth_rad, void* stream) {
  using namespace vsr;
  if (height < 0 || width < 0) return fail(VSR_ERR_INVALID_ARG, "negative raster size");
  if (height == 0 || width == 0) return VSR_OK;
  if (!slope && !aspect && !hillshade) return VSR_OK;
  if (!dem) return fail(VSR_ERR_INVALID_ARG, "dem is NULL");
  if (dtype_size(dtype) == 0) return fail(VSR_ERR_INVALID_ARG, "unsupported dtype %d", dtype);
  if (pitch < width) return fail(VSR_ERR_INVALID_ARG, "pitch %lld < width %lld", (long long)pitch, (long long)width);
  if ((slope || aspect) && out_dtype != VSR_F32 && out_dtype != VSR_F64)
    return fail(VSR_ERR_INVALID_ARG, "slope/aspect out_dtype must be VSR_F32 or VSR_F64");
  if ((slope || aspect) && out_pitch < width) return fail(VSR_ERR_INVALID_ARG, "out_pitch < width");
  if (hillshade && hs_pitch < width) return fail(VSR_ERR_INVALID_ARG, "hs_pitch < width");
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
                      width < (int64_t(1) << 31) && height < (int64_t(1) << 31);
  if (tma_ok)
    return launch_tma_config(tuning_get(VSR_OP_HORN), dem, P, static_cast<float>(ndv),
                             static_cast<float*>(slope), static_cast<float*>(aspect), hillshade, st);
  if ((slope || aspect) && out_dtype == VSR_F64)
    return dispatch_generic<double>(dtype, dem, P, ndv, slope, aspect, hillshade, st);
  return dispatch_generic<float>(dtype, dem, P, ndv, slope, aspect, hillshade, st);
}

// ===================================================================== batch ==
// One persistent, work-queue-scheduled launch over many DEM tiles of uneven
// sizes, each with its own cell size and nodata: slope + aspect (Horn) and a
// KG x KG nodata-aware Gaussian, all from one staged block.  Replaces the
// reference's per-tile / per-band Python loops (dispatch.py:417-506), which
// issue separate launches per raster and per operation.
//
// Work item = (tile, 128 x TH output block).  A CTA claims items with an
// atomic counter (no waits: an exhausted queue simply ends the CTA), finds
// the tile by binary search over the per-tile prefix sums, stages
// (TH + 2*HY) x 136 input values with coalesced loads and clamped
// coordinates (any pitch or alignment; edge replication for Horn), runs the
// Horn rows on them, then the separable Gaussian: a row pass into shared
// memory (numerator and weight sum, validity from coordinates and nodata so
// out-of-bounds taps are skipped), then the column pass.
namespace vsr {
namespace {

struct BatchTileDev {
  const float* src;
  int64_t H, W, pitch;
  float* slope;
  float* aspect;
  float* smooth;
  int64_t out_pitch;
  double cell_x, cell_y, nodata;
  int32_t nd_kind;
  uint32_t flags;
  int64_t first_item;  // prefix sum of items over earlier tiles
  int64_t items_x;     // blocks across this tile
  int32_t vec;         // outputs 16-byte aligned with pitch % 4 == 0
  float inv8cx, inv8cy;  // 1 / (8 cell), formed in FP64 on the device at plan time
  int32_t pad_;
};

struct BatchHeader {  // at the start of the plan
  unsigned long long counter;
  int64_t total_items;
  int32_t n_tiles, kg, th, threads;
  float g[16];          // Gaussian taps (float32 of the float64 weights)
  float gsum;           // sum of g
  float pad_[3];
};

constexpr int kBatchMaxKG = 9;

template <int TH, int THREADS, int KG>
struct BatchSmem {
  static constexpr int HY = KG / 2 > 0 ? KG / 2 : 1;  // staged halo rows (>= 1 for Horn)
  static constexpr int SR = TH + 2 * HY;              // staged rows
  static constexpr int kFloats = 2 * SR * kSW + 2 * SR * kTW;  // two staging buffers, row-pass sums
};


constexpr int kBatchSmemTiles = 2048;  // tiles whose prefix sums are searched in shared memory

template <int TH, int THREADS, int KG>
__global__ void __launch_bounds__(THREADS) batch_terrain_kernel(BatchHeader* __restrict__ hdr,
                                                                const BatchTileDev* __restrict__ tiles,
                                                                uint32_t* err_word) {
  using L = BatchSmem<TH, THREADS, KG>;
  // The plan's item counts were formed with its own block height and its taps
  // with its own Gaussian width: a launch of any other shape would leave rows
  // unwritten or apply the wrong taps, so it reports and does nothing.
  if (hdr->th != TH || (hdr->kg > 1 ? hdr->kg : 1) != KG) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(err_word, kDevErrPlan);
    return;
  }
  constexpr int WARPS = THREADS / 32;
  constexpr int RB = TH / WARPS;
  constexpr int HY = L::HY, SR = L::SR;
  static_assert(RB * WARPS == TH && RB % 2 == 0, "rows per warp");
  extern __shared__ __align__(16) float bsm[];
  float* Sbuf = bsm;                  // 2 x SR x kSW staged values (double buffered)
  float* Rn = Sbuf + 2 * SR * kSW;    // SR x kTW row-pass numerator
  float* Rd = Rn + SR * kTW;          // SR x kTW row-pass weight sum
  __shared__ int64_t sh_first[kBatchSmemTiles];
  __shared__ int64_t sh_item[2];
  __shared__ int sh_tile[2];
  __shared__ HornParams sh_P[2];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t total = hdr->total_items;
  const int n_tiles = hdr->n_tiles;
  const bool smem_search = n_tiles <= kBatchSmemTiles;
  if (smem_search)
    for (int i = tid; i < n_tiles; i += THREADS) sh_first[i] = tiles[i].first_item;
  float gw[KG > 0 ? KG : 1];
#pragma unroll
  for (int t = 0; t < KG; ++t) gw[t] = hdr->g[t];
  const float gs2 = hdr->gsum * hdr->gsum;
  __syncthreads();

  // Items are claimed from the atomic counter one ahead of the one being
  // staged, and staged (cp.async into the other buffer) one ahead of the one
  // being computed, so claim and copy latencies overlap the current item.
  int64_t claimed = 0;  // (thread 0) the next unassigned claim
  auto assign = [&](int b, int64_t item) {  // thread 0: item -> buffer b's tile and params
    sh_item[b] = item;
    if (item >= total) return;
    int lo = 0, hi = n_tiles - 1;  // last tile with first_item <= item
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      const int64_t f = smem_search ? sh_first[mid] : tiles[mid].first_item;
      if (f <= item) lo = mid;
      else hi = mid - 1;
    }
    sh_tile[b] = lo;
    const BatchTileDev& T = tiles[lo];
    HornParams P{};
    P.height = T.H;
    P.width = T.W;
    P.in_pitch = T.pitch;
    P.out_pitch = T.out_pitch;
    P.hs_pitch = T.out_pitch;
    P.inv8cx = T.inv8cx;
    P.inv8cy = T.inv8cy;
    P.nd_out_f = static_cast<float>(T.nodata);
    P.nd_out_d = T.nodata;
    P.flags = T.flags;
    P.nd_kind = T.nd_kind;
    sh_P[b] = P;
  };
  // Stage rows y0-HY .. y0+TH+HY-1, columns x0-4 .. x0+131 (clamped into the
  // tile: edge replication), one warp per row, lanes along the row.
  auto stage = [&](int b) {
    const int64_t item = sh_item[b];
    if (item >= total) return;
    const HornParams& P = sh_P[b];
    const BatchTileDev& T = tiles[sh_tile[b]];
    const int64_t local = item - (smem_search ? sh_first[sh_tile[b]] : T.first_item);
    const int64_t items_x = (P.width + kTW - 1) / kTW;
    const int64_t by = local / items_x, bx = local - by * items_x;
    const int64_t x0 = bx * kTW, y0 = by * TH;
    float* S = Sbuf + b * SR * kSW;
    for (int r = warp; r < SR; r += WARPS) {
      const int64_t gy = min(max(y0 - HY + r, int64_t(0)), P.height - 1);
      const float* rowp = T.src + gy * P.in_pitch;
#pragma unroll
      for (int c = lane; c < kSW; c += 32) {
        const int64_t gx = min(max(x0 - 4 + c, int64_t(0)), P.width - 1);
        cp_async4(S + r * kSW + c, rowp + gx);
      }
    }
  };
  if (tid == 0) {
    assign(0, static_cast<int64_t>(atomicAdd(&hdr->counter, 1ull)));
    claimed = static_cast<int64_t>(atomicAdd(&hdr->counter, 1ull));
  }
  __syncthreads();
  stage(0);
  cp_async_commit();

  for (int it = 0;; ++it) {
    const int b = it & 1;
    if (sh_item[b] >= total) break;  // uniform: written before the last barrier
    if (tid == 0) {
      assign(b ^ 1, claimed);
      if (claimed < total) claimed = static_cast<int64_t>(atomicAdd(&hdr->counter, 1ull));
    }
    __syncthreads();  // buffer b ^ 1's item is known (and its previous reads are done)
    stage(b ^ 1);
    cp_async_commit();
    cp_async_wait<1>();  // this item's copies (all but the group just committed)
    __syncthreads();
    const int64_t item = sh_item[b];
    const BatchTileDev& T = tiles[sh_tile[b]];
    const HornParams P = sh_P[b];
    const float nd_in = static_cast<float>(P.nd_out_d);
    const int64_t local = item - (smem_search ? sh_first[sh_tile[b]] : T.first_item);
    const int64_t items_x = (P.width + kTW - 1) / kTW;
    const int64_t by = local / items_x, bx = local - by * items_x;
    const int64_t x0 = bx * kTW, y0 = by * TH;
    const int64_t H = P.height, W = P.width;
    const float* S = Sbuf + b * SR * kSW;

    // Does the staged block hold nodata?  Clean blocks skip the mask logic.
    bool any_nd = false;
    if (P.nd_kind != VSR_NODATA_NONE)
      for (int i = tid; i < SR * kSW; i += THREADS) any_nd |= is_nd(S[i], P.nd_kind, nd_in);
    const bool masked = __syncthreads_or(any_nd);
    const bool edge = x0 + kTW > W || y0 + TH > H;
    const MaskRule rule = mask_rule(P);

    // Horn slope + aspect.
    if (T.slope || T.aspect) {
      const int64_t xs = x0 + 4 * lane;
      const float* Sh = S + (HY - 1) * kSW;
      const RowPtrs g = global_rows(T.slope, T.aspect, nullptr, P, y0 + warp * RB, xs);
      // both outputs are requested together in the batch plan
      if (T.vec) {
        if (masked) {
          if (edge) horn_rows<RB, 3, true, true, true>(Sh, lane, warp * RB, y0, xs, P, rule, nd_in, g.s, g.a, g.h, P.out_pitch, P.hs_pitch);
          else horn_rows<RB, 3, true, false, true>(Sh, lane, warp * RB, y0, xs, P, rule, nd_in, g.s, g.a, g.h, P.out_pitch, P.hs_pitch);
        } else {
          if (edge) horn_rows<RB, 3, false, true, true>(Sh, lane, warp * RB, y0, xs, P, rule, nd_in, g.s, g.a, g.h, P.out_pitch, P.hs_pitch);
          else horn_rows<RB, 3, false, false, true>(Sh, lane, warp * RB, y0, xs, P, rule, nd_in, g.s, g.a, g.h, P.out_pitch, P.hs_pitch);
        }
      } else {
        if (masked) horn_rows<RB, 3, true, true, false>(Sh, lane, warp * RB, y0, xs, P, rule, nd_in, g.s, g.a, g.h, P.out_pitch, P.hs_pitch);
        else horn_rows<RB, 3, false, true, false>(Sh, lane, warp * RB, y0, xs, P, rule, nd_in, g.s, g.a, g.h, P.out_pitch, P.hs_pitch);
      }
    }

    // Gaussian KG x KG (normalised, nodata-aware, out-of-bounds taps skipped).
    if (T.smooth) {
      constexpr int R = KG / 2;
      const bool exact_den = masked || x0 - R < 0 || y0 - R < 0 || x0 + kTW + R > W || y0 + TH + R > H;
      // row pass: staged rows (HY-R) .. (HY+TH+R-1), 4 columns per lane
      for (int r = warp + (HY - R); r < HY + TH + R; r += WARPS) {
        const int64_t gy = y0 - HY + r;
        const bool row_in = gy >= 0 && gy < H;
        const int c0 = 4 * lane;
        float z[4 + KG - 1], vd[4 + KG - 1];
#pragma unroll
        for (int j = 0; j < 4 + KG - 1; ++j) {
          const int c = c0 + 4 - R + j;  // staged column
          const float v = S[r * kSW + c];
          const int64_t gx = x0 - 4 + c;
          const bool ok = row_in && gx >= 0 && gx < W && !is_nd(v, P.nd_kind, nd_in);
          z[j] = v * (ok ? 1.0f : 0.0f);  // NaN * 0 stays NaN, as in the reference
          vd[j] = ok ? 1.0f : 0.0f;
        }
        float an[4] = {}, ad[4] = {};
#pragma unroll
        for (int t = 0; t < KG; ++t) {
          const float w = gw[t];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            an[u] = fmaf(w, z[u + t], an[u]);
            ad[u] = fmaf(w, vd[u + t], ad[u]);
          }
        }
        *reinterpret_cast<float4*>(Rn + r * kTW + c0) = make_float4(an[0], an[1], an[2], an[3]);
        *reinterpret_cast<float4*>(Rd + r * kTW + c0) = make_float4(ad[0], ad[1], ad[2], ad[3]);
      }
      __syncthreads();
      // column pass: one column per thread, TH*kTW/THREADS consecutive rows
      constexpr int GROUPS = THREADS / kTW;
      constexpr int RY = TH / GROUPS;
      const int c = tid % kTW;
      const int q0 = (tid / kTW) * RY;
      const int64_t x = x0 + c;
#pragma unroll 1
      for (int q = q0; q < q0 + RY; ++q) {
        const int64_t y = y0 + q;
        if (y >= H || x >= W) continue;
        float num = 0.0f, den = 0.0f;
#pragma unroll
        for (int t = 0; t < KG; ++t) {
          const int r = q + HY - R + t;
          const float w = gw[t];
          num = fmaf(w, Rn[r * kTW + c], num);
          den = fmaf(w, Rd[r * kTW + c], den);
        }
        if (!exact_den) den = gs2;
        const float cv = S[(q + HY) * kSW + c + 4];
        const bool centre_ok = !is_nd(cv, P.nd_kind, nd_in);
        T.smooth[y * T.out_pitch + x] = (centre_ok && den > 0.0f) ? num / den : P.nd_out_f;
      }
    }
    __syncthreads();  // row-pass sums are reused by the next item; buffer b is refilled after the next barrier
  }
  cp_async_wait<0>();  // no copy may land after the CTA leaves
}

// Launch configurations the autotuner chooses between: (rows per block,
// threads per CTA); the Gaussian width is a template parameter too.
struct BatchConfig {
  int th, threads;
};
constexpr BatchConfig kBatchConfigs[] = {{32, 256}, {64, 256}, {16, 128}, {32, 128}};
constexpr int kNumBatchConfigs = sizeof(kBatchConfigs) / sizeof(kBatchConfigs[0]);

template <int TH, int THREADS, int KG>
int launch_batch_t(BatchHeader* hdr, const BatchTileDev* tiles, cudaStream_t st) {
  using L = BatchSmem<TH, THREADS, KG>;
  uint32_t* err = device_error_word();
  if (!err) return VSR_ERR_CUDA;
  const size_t smem = static_cast<size_t>(L::kFloats) * 4;
  auto kern = batch_terrain_kernel<TH, THREADS, KG>;
  VSR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  int per_sm = 0;
  VSR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, THREADS, smem));
  if (per_sm < 1) return fail(VSR_ERR_CUDA, "batch kernel cannot be resident");
  kern<<<static_cast<unsigned>(sm_count() * per_sm), THREADS, smem, st>>>(hdr, tiles, err);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}

template <int KG>
int launch_batch_kg(int cfg, BatchHeader* hdr, const BatchTileDev* tiles, cudaStream_t st) {
  switch (cfg) {
    case 1: return launch_batch_t<64, 256, KG>(hdr, tiles, st);
    case 2: return launch_batch_t<16, 128, KG>(hdr, tiles, st);
    case 3: return launch_batch_t<32, 128, KG>(hdr, tiles, st);
    default: return launch_batch_t<32, 256, KG>(hdr, tiles, st);
  }
}

// Per-tile 1 / (8 cell) in FP64 on the device (the cell sizes come from each
// tile's affine transform).
__global__ void prep_batch_cells(BatchTileDev* tiles, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  tiles[i].inv8cx = static_cast<float>(1.0 / (8.0 * tiles[i].cell_x));
  tiles[i].inv8cy = static_cast<float>(1.0 / (8.0 * tiles[i].cell_y));
}

__global__ void prep_batch_gauss(BatchHeader* hdr, int kg, double sigma) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int i = 0; i < kg; ++i) {
    const double a = (i - kg / 2) / sigma;
    const double g = exp(-0.5 * a * a);
    hdr->g[i] = static_cast<float>(g);
    s += static_cast<double>(static_cast<float>(g));
  }
  hdr->gsum = static_cast<float>(s);
}

// Launch shape of every plan built in this process, keyed by the plan's
// device address: vsr_batch_run launches the configuration the plan was
// built for, whatever the tuning table holds by then.
struct PlanShape {
  int cfg, kg;
};
std::mutex g_plan_mutex;
std::unordered_map<const void*, PlanShape> g_plans;

}  // namespace

int batch_config_count() { return kNumBatchConfigs; }

}  // namespace vsr

extern "C" size_t vsr_batch_plan_size(int n_tiles) {
  if (n_tiles <= 0) return 0;
  return ((sizeof(vsr::BatchHeader) + 255) & ~size_t(255)) + static_cast<size_t>(n_tiles) * sizeof(vsr::BatchTileDev);
}

extern "C" int vsr_batch_plan(const vsr_batch_tile* tiles_host, int n_tiles, double sigma, int gauss_k, void* plan,
                              size_t plan_bytes, int64_t* total_items, void* stream) {
  using namespace vsr;
  if (n_tiles <= 0 || !tiles_host) return fail(VSR_ERR_INVALID_ARG, "need at least one tile");
  if (gauss_k != 0 && (gauss_k < 1 || gauss_k > kBatchMaxKG || gauss_k % 2 == 0))
    return fail(VSR_ERR_UNSUPPORTED, "batch Gaussian size must be odd and <= %d", kBatchMaxKG);
  if (gauss_k != 0 && !(sigma > 0.0)) return fail(VSR_ERR_INVALID_ARG, "sigma must be positive, got %g", sigma);
  const size_t need = vsr_batch_plan_size(n_tiles);
  if (!plan || plan_bytes < need || !aligned(plan, 256))
    return fail(VSR_ERR_WORKSPACE, "plan must be 256-byte aligned and >= %zu bytes", need);
  const int cfg = tuning_get(VSR_OP_BATCH);
  const int th = kBatchConfigs[cfg].th;
  std::vector<BatchTileDev> dev(n_tiles);
  int64_t items = 0;
  for (int i = 0; i < n_tiles; ++i) {
    const vsr_batch_tile& t = tiles_host[i];
    if (t.height <= 0 || t.width <= 0 || !t.src) return fail(VSR_ERR_INVALID_ARG, "tile %d is empty or NULL", i);
    if (t.pitch < t.width || t.out_pitch < t.width) return fail(VSR_ERR_INVALID_ARG, "tile %d: pitch < width", i);
    if (!(t.cell_x > 0.0) || !(t.cell_y > 0.0)) return fail(VSR_ERR_INVALID_ARG, "tile %d: cell sizes must be positive", i);
    if ((t.slope == nullptr) != (t.aspect == nullptr))
      return fail(VSR_ERR_INVALID_ARG, "tile %d: slope and aspect are produced together", i);
    if (!aligned(t.src, 4) || (t.slope && !aligned(t.slope, 4)) || (t.aspect && !aligned(t.aspect, 4)) ||
        (t.smooth && !aligned(t.smooth, 4)))
      return fail(VSR_ERR_INVALID_ARG, "tile %d: buffers must be 4-byte aligned", i);
    if (t.smooth && gauss_k == 0) return fail(VSR_ERR_INVALID_ARG, "tile %d wants a Gaussian but gauss_k is 0", i);
    BatchTileDev& d = dev[i];
    d.src = t.src;
    d.H = t.height;
    d.W = t.width;
    d.pitch = t.pitch;
    d.slope = t.slope;
    d.aspect = t.aspect;
    d.smooth = t.smooth;
    d.out_pitch = t.out_pitch;
    d.cell_x = t.cell_x;
    d.cell_y = t.cell_y;
    d.nodata = t.nodata;
    double ev = 0.0;
    d.nd_kind = resolve_nodata(VSR_F32, t.nodata, t.nodata_kind, &ev);
    d.flags = t.flags;
    d.vec = (!t.slope || (aligned(t.slope, 16) && aligned(t.aspect, 16))) && t.out_pitch % 4 == 0;
    d.inv8cx = d.inv8cy = 0.0f;  // set on the device by prep_batch_cells
    d.pad_ = 0;
    d.items_x = (t.width + kTW - 1) / kTW;
    d.first_item = items;
    items += d.items_x * ((t.height + th - 1) / th);
  }
  BatchHeader h{};
  h.counter = 0;
  h.total_items = items;
  h.n_tiles = n_tiles;
  h.kg = gauss_k;
  h.th = th;
  h.threads = kBatchConfigs[cfg].threads;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* base = static_cast<char*>(plan);
  const size_t off = (sizeof(BatchHeader) + 255) & ~size_t(255);
  VSR_CUDA_TRY(cudaMemcpyAsync(base, &h, sizeof(h), cudaMemcpyHostToDevice, st));
  VSR_CUDA_TRY(cudaMemcpyAsync(base + off, dev.data(), dev.size() * sizeof(BatchTileDev), cudaMemcpyHostToDevice, st));
  prep_batch_cells<<<(n_tiles + 127) / 128, 128, 0, st>>>(reinterpret_cast<BatchTileDev*>(base + off), n_tiles);
  VSR_CUDA_TRY(cudaGetLastError());
  if (gauss_k) {
    prep_batch_gauss<<<1, 32, 0, st>>>(reinterpret_cast<BatchHeader*>(base), gauss_k, sigma);
    VSR_CUDA_TRY(cudaGetLastError());
  }
  VSR_CUDA_TRY(cudaStreamSynchronize(st));  // the host descriptors are staged from pageable memory
  {
    std::lock_guard<std::mutex> lk(g_plan_mutex);
    g_plans[plan] = PlanShape{cfg, gauss_k};
  }
  if (total_items) *total_items = items;
  return VSR_OK;
}

extern "C" int vsr_batch_run(void* plan, int gauss_k, void* stream) {
  using namespace vsr;
  if (!plan || !aligned(plan, 256)) return fail(VSR_ERR_INVALID_ARG, "plan must be a 256-byte aligned device pointer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  BatchHeader* hdr = static_cast<BatchHeader*>(plan);
  const BatchTileDev* tiles = reinterpret_cast<const BatchTileDev*>(static_cast<char*>(plan) + ((sizeof(BatchHeader) + 255) & ~size_t(255)));
  PlanShape shape{};
  {
    std::lock_guard<std::mutex> lk(g_plan_mutex);
    const auto it = g_plans.find(plan);
    if (it == g_plans.end())
      return fail(VSR_ERR_INVALID_ARG, "plan %p was not built by vsr_batch_plan in this process", plan);
    shape = it->second;
  }
  if (gauss_k != shape.kg)
    return fail(VSR_ERR_INVALID_ARG, "gauss_k %d does not match the plan's %d", gauss_k, shape.kg);
  VSR_CUDA_TRY(cudaMemsetAsync(&hdr->counter, 0, sizeof(hdr->counter), st));
  const int cfg = shape.cfg;
  switch (gauss_k) {
    case 0:
    case 1: return launch_batch_kg<1>(cfg, hdr, tiles, st);
    case 3: return launch_batch_kg<3>(cfg, hdr, tiles, st);
    case 5: return launch_batch_kg<5>(cfg, hdr, tiles, st);
    case 7: return launch_batch_kg<7>(cfg, hdr, tiles, st);
    case 9: return launch_batch_kg<9>(cfg, hdr, tiles, st);
    default: return fail(VSR_ERR_UNSUPPORTED, "batch Gaussian size must be odd and <= %d", kBatchMaxKG);
  }
}
