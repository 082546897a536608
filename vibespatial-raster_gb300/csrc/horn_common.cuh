// Horn 3x3 terrain arithmetic shared by the fused TMA kernel (horn_tma.cuh),
// the generic kernel (horn.cu) and the batched kernel (batch.cu).
//
// Replaces the arithmetic of the reference's ``slope_aspect`` and
// ``hillshade`` NVRTC kernels (kernels/focal.py:173-283, 303-467).
//
// FP32 on CUDA cores:
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
// The angle arithmetic folds octants with sign-bit copies (copysign is one
// bitwise instruction) rather than compare-and-select chains: the fused
// kernel's integer/logic pipe was its busiest, and these folds move the work
// to the FMA pipe, where pixel pairs share packed f32x2 instructions.
#pragma once

#include "vsr_internal.cuh"

namespace vsr {
namespace horn {

struct HornParams {
  int64_t height, width;
  int64_t in_pitch, out_pitch, hs_pitch;
  int bands;  // band-first stack: band b at b * *_band_stride elements
  int64_t in_band_stride, out_band_stride, hs_band_stride;
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

constexpr int kWantSlope = 1, kWantAspect = 2, kWantHs = 4;

// ------------------------------------------------------------ primitives --
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

// min / max that return NaN when either operand is NaN (fminf/fmaxf would
// return the other operand and hide it).
__device__ __forceinline__ float fmin_nan(float a, float b) {
  float r;
  asm("min.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float fmax_nan(float a, float b) {
  float r;
  asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}

// Three-input FP32 min / max (sm_100 and later; NaN inputs are ignored as by
// fminf / fmaxf).
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

// Packed FP32 pairs (fma/mul/add .f32x2: two IEEE single-precision results
// per instruction, rounded exactly as the scalar forms).
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 copysign2(float2 mag, float2 sgn) {
  return make_float2(copysignf(mag.x, sgn.x), copysignf(mag.y, sgn.y));
}

// ------------------------------------------------------ angle arithmetic --
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

// Slope in degrees from s = p^2 + q^2.  With rs = 1/sqrt(s) and r = s rs,
// t = min(r, 1/r) = min(s rs, rs) and a = atan(t); the result is a for
// s <= 1 and 90 - a above: 45 - (45 - a) or 45 + (45 - a), the sign taken
// from s - 1.  s = 0 gives exactly 0, s = inf gives 90, NaN propagates.
__device__ __forceinline__ float slope_deg(float s) {
  const float rs = rsqrt_approx(s + 1e-30f);
  const float t = fminf(s * rs, rs);
  const float a = atan_poly_deg(t);
  return 45.0f + copysignf(45.0f - a, s - 1.0f);
}

__device__ __forceinline__ float2 slope_deg2(float2 s) {
  const float2 sp = add2(s, f2(1e-30f));
  const float2 rs = make_float2(rsqrt_approx(sp.x), rsqrt_approx(sp.y));
  const float2 r = mul2(s, rs);
  const float2 t = make_float2(fminf(r.x, rs.x), fminf(r.y, rs.y));
  const float2 a = atan_poly_deg2(t);
  const float2 d = fma2(a, f2(-1.0f), f2(45.0f));
  return add2(f2(45.0f), copysign2(d, add2(s, f2(-1.0f))));
}

// Aspect in compass degrees, (90 - theta) mod 360 with theta = atan2(-q, p)
// in degrees, signed zeros as atan2 has them (flat gives exactly 90, the
// axes exactly 0, 90, 180, 270):
//   a0 = atan(min/max of |p|, |q|)                 in [0, 45]
//   a1 = 45 - copysign(45 - a0, |p| - |q|)         angle from the x axis, [0, 90]
//   a2 = 90 - copysign(90 - a1, p)                 [0, 180]
//   theta = copysign(a2, -q)
//   aspect = (270 - theta) - copysign(180, 90 - theta)
// min / max propagate NaN, so a NaN gradient gives a NaN aspect.
__device__ __forceinline__ float aspect_deg(float p, float q) {
  const float ap = fabsf(p), aq = fabsf(q);
  const float mn = fmin_nan(ap, aq), mx = fmax_nan(ap, aq);
  const float a0 = atan_poly_deg(mn * rcp_approx(mx + 1e-30f));
  const float a1 = 45.0f - copysignf(45.0f - a0, ap - aq);
  const float a2 = 90.0f - copysignf(90.0f - a1, p);
  const float th = copysignf(a2, -q);
  return (270.0f - th) - copysignf(180.0f, 90.0f - th);
}

__device__ __forceinline__ float2 aspect_deg2(float2 p, float2 q) {
  const float ap0 = fabsf(p.x), aq0 = fabsf(q.x), ap1 = fabsf(p.y), aq1 = fabsf(q.y);
  const float2 mn = make_float2(fmin_nan(ap0, aq0), fmin_nan(ap1, aq1));
  const float2 mx = add2(make_float2(fmax_nan(ap0, aq0), fmax_nan(ap1, aq1)), f2(1e-30f));
  const float2 a0 = atan_poly_deg2(mul2(mn, make_float2(rcp_approx(mx.x), rcp_approx(mx.y))));
  const float2 dpq = make_float2(ap0 - aq0, ap1 - aq1);
  const float2 a1 = fma2(copysign2(fma2(a0, f2(-1.0f), f2(45.0f)), dpq), f2(-1.0f), f2(45.0f));
  const float2 a2 = fma2(copysign2(fma2(a1, f2(-1.0f), f2(90.0f)), p), f2(-1.0f), f2(90.0f));
  const float2 th = make_float2(copysignf(a2.x, -q.x), copysignf(a2.y, -q.y));
  const float2 e = fma2(th, f2(-1.0f), f2(270.0f));
  const float2 g = fma2(th, f2(-1.0f), f2(90.0f));
  return fma2(copysign2(f2(180.0f), g), f2(-1.0f), e);
}

// Hillshade byte from the unscaled gradient (p, q) and s = p^2 + q^2:
// (cos zen + sin zen (cos az p' - sin az q')) / sqrt(1 + p'^2 + q'^2) with
// p' = zf p, q' = zf q, saturated to [0, 1] (NaN -> 0); the byte is the
// truncation of hs*255 + 0.5, read from the low bits of its sum with 2^23
// rounded toward zero (no float-to-integer conversion).
__device__ __forceinline__ uint32_t hs_byte_bits(float num, float r) {
  const float hs = __saturatef(num * r);
  return __float_as_uint(__fadd_rz(fmaf(hs, 255.0f, 0.5f), 8388608.0f));
}

__device__ __forceinline__ uint8_t hillshade_u8(float p, float q, float s, const HornParams& P) {
  const float num = fmaf(P.hs_a, p, fmaf(-P.hs_b, q, P.cos_z));
  return static_cast<uint8_t>(hs_byte_bits(num, rsqrt_approx(fmaf(P.zf2, s, 1.0f))) & 0xffu);
}

// Two pixels' hillshade bytes, each in the low byte of a word.
__device__ __forceinline__ void hillshade_bits2(float2 p, float2 q, float2 s, const HornParams& P, uint32_t& h0,
                                                uint32_t& h1) {
  const float2 num = fma2(f2(P.hs_a), p, fma2(f2(-P.hs_b), q, f2(P.cos_z)));
  const float2 d = fma2(f2(P.zf2), s, f2(1.0f));
  h0 = hs_byte_bits(num.x, rsqrt_approx(d.x));
  h1 = hs_byte_bits(num.y, rsqrt_approx(d.y));
}

// ------------------------------------------------------ exact gradients --
// Differences of neighbouring FP32 elevations are exact when the operands
// lie within a factor of two of each other (Sterbenz), which holds almost
// everywhere; near 0 m (or where values of very different size meet, e.g.
// nodata) a difference can round, and a small gradient formed from large
// rounded differences loses the aspect's accuracy (the reference differences
// in float64).  Rows where that can happen take error-free transformations
// instead: TwoDiff/TwoSum keep every rounding error and the sum is formed to
// within one final rounding.
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

// Every difference (and the sums) of a row window is exact when all its
// values lie in [m, 2m] for some m > 0, or in [-2m, -m], or are all zero.
__device__ __forceinline__ bool window_exact(float lo, float hi) {
  return (lo > 0.0f && hi <= 2.0f * lo) || (hi < 0.0f && lo >= 2.0f * hi) || (lo == 0.0f && hi == 0.0f);
}

// --------------------------------------------------- staged-row kernels --
constexpr int kTW = 128;      // output tile width (32 lanes x 4 pixels)
constexpr int kSW = kTW + 8;  // staged width: 4-column halo each side (16 B)

// One staged row for a lane: its 6 values (columns 4 lane + 3 .. 4 lane + 8
// of the staged row: the lane's 4 pixels and one neighbour each side), the 4
// horizontal differences (x+2 minus x, shared by the three output rows that
// use the row) and the value range (NaN ignored) for the exactness test.
struct Row {
  float v[6], hd[4];
  float lo, hi;
};

__device__ __forceinline__ void stage_row(const float* row, int lane, Row& r) {
  const float4 m = *reinterpret_cast<const float4*>(row + 4 + 4 * lane);
  r.v[0] = row[3 + 4 * lane];
  r.v[1] = m.x;
  r.v[2] = m.y;
  r.v[3] = m.z;
  r.v[4] = m.w;
  r.v[5] = row[8 + 4 * lane];
#pragma unroll
  for (int k = 0; k < 4; ++k) r.hd[k] = r.v[k + 2] - r.v[k];
  r.lo = fminf(min3f(r.v[0], r.v[1], r.v[2]), min3f(r.v[3], r.v[4], r.v[5]));
  r.hi = fmaxf(max3f(r.v[0], r.v[1], r.v[2]), max3f(r.v[3], r.v[4], r.v[5]));
}

// Could the row hold nodata?  A value nodata can only be present if it lies
// within the row's range; a NaN anywhere makes a difference NaN (inf - inf
// also does: a harmless false alarm).
template <int NDK>
__device__ __forceinline__ bool row_may_hold_nodata(const Row& r, float ndv) {
  if (NDK == VSR_NODATA_VALUE) return ndv >= r.lo && ndv <= r.hi;
  if (NDK == VSR_NODATA_NAN) {
    const float s = (r.hd[0] + r.hd[1]) + (r.hd[2] + r.hd[3]);
    return s != s;
  }
  return false;
}

template <int NDK>
__device__ __forceinline__ bool is_nd(float v, float ndv) {
  return NDK == VSR_NODATA_VALUE ? (v == ndv) : (NDK == VSR_NODATA_NAN ? (v != v) : false);
}

// Nodata bits of a row's 6 values; with ``skip`` its range is narrowed to the
// valid values (outputs whose windows hold nodata are masked anyway).
template <int NDK>
__device__ __forceinline__ uint32_t row_nodata(Row& r, float ndv, bool skip) {
  uint32_t m = 0;
#pragma unroll
  for (int k = 0; k < 6; ++k) m |= (is_nd<NDK>(r.v[k], ndv) ? 1u : 0u) << k;
  if (skip && m) {
    float l[6], h[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const bool nd = (m >> k) & 1u;
      l[k] = nd ? __int_as_float(0x7f800000) : r.v[k];
      h[k] = nd ? __int_as_float(0xff800000) : r.v[k];
    }
    r.lo = fminf(min3f(l[0], l[1], l[2]), min3f(l[3], l[4], l[5]));
    r.hi = fmaxf(max3f(h[0], h[1], h[2]), max3f(h[3], h[4], h[5]));
  }
  return m;
}

// Gradients of a lane's 4 pixels from the rows above (t), through (m) and
// below (b): the fast form from the (exact) differences, or grad_exact where
// differences may round.
__device__ __forceinline__ void grad_fast(const Row& t, const Row& m, const Row& b, float gx[4], float gy[4]) {
  float dv[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) dv[k] = b.v[k] - t.v[k];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    gx[k] = fmaf(2.0f, m.hd[k], t.hd[k] + b.hd[k]);
    gy[k] = fmaf(2.0f, dv[k + 1], dv[k] + dv[k + 2]);
  }
}

__device__ __forceinline__ void grad_exact4(const Row& t, const Row& m, const Row& b, float gx[4], float gy[4]) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    gx[k] = grad_exact(t.v[k], t.v[k + 2], m.v[k], m.v[k + 2], b.v[k], b.v[k + 2]);
    gy[k] = grad_exact(t.v[k], b.v[k], t.v[k + 1], b.v[k + 1], t.v[k + 2], b.v[k + 2]);
  }
}

// One output row (4 pixels of this lane) from its gradients; ``masked``
// (warp-uniform) applies the nodata bits of the three window rows.
template <int WANT, bool EDGE, bool VEC>
__device__ __forceinline__ void horn_out_row(const float gx[4], const float gy[4], bool masked, uint32_t mt,
                                             uint32_t mm, uint32_t mb, const HornParams& P, const MaskRule& rule,
                                             int64_t y, int64_t xs, float* __restrict__ srow,
                                             float* __restrict__ arow, uint8_t* __restrict__ hrow) {
  if (EDGE && (y >= P.height || xs >= P.width)) return;
  float so[4], ao[4];
  uint32_t hb[4];
#pragma unroll
  for (int k = 0; k < 4; k += 2) {
    const float2 p = mul2(make_float2(gx[k], gx[k + 1]), f2(P.inv8cx));
    const float2 q = mul2(make_float2(gy[k], gy[k + 1]), f2(P.inv8cy));
    const float2 s = fma2(p, p, mul2(q, q));
    if (WANT & kWantSlope) {
      const float2 v = slope_deg2(s);
      so[k] = v.x;
      so[k + 1] = v.y;
    }
    if (WANT & kWantAspect) {
      const float2 v = aspect_deg2(p, q);
      ao[k] = v.x;
      ao[k + 1] = v.y;
    }
    if (WANT & kWantHs) hillshade_bits2(p, q, s, P, hb[k], hb[k + 1]);
  }
  if (masked) {
    const uint32_t hdil = (mt | (mt >> 1) | (mt >> 2)) | (mm | (mm >> 1) | (mm >> 2)) | (mb | (mb >> 1) | (mb >> 2));
    const uint32_t sabits = rule.sa_any ? (rule.sa_center ? (mm >> 1) : hdil) : 0u;
    const uint32_t hsbits = rule.hs_any ? hdil : 0u;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const bool sa_nd = (sabits >> k) & 1u;
      so[k] = sa_nd ? P.nd_out_f : so[k];
      ao[k] = sa_nd ? P.nd_out_f : ao[k];
      hb[k] = ((hsbits >> k) & 1u) ? 0u : hb[k];
    }
  }
  const bool full = VEC && (!EDGE || xs + 3 < P.width);
  if (full) {
    if (WANT & kWantSlope) __stcs(reinterpret_cast<float4*>(srow), make_float4(so[0], so[1], so[2], so[3]));
    if (WANT & kWantAspect) __stcs(reinterpret_cast<float4*>(arow), make_float4(ao[0], ao[1], ao[2], ao[3]));
    if (WANT & kWantHs)
      __stcs(reinterpret_cast<unsigned int*>(hrow), __byte_perm(__byte_perm(hb[0], hb[1], 0x0040),
                                                                __byte_perm(hb[2], hb[3], 0x0040), 0x5410));
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (xs + k < P.width) {
        if (WANT & kWantSlope) srow[k] = so[k];
        if (WANT & kWantAspect) arow[k] = ao[k];
        if (WANT & kWantHs) hrow[k] = static_cast<uint8_t>(hb[k] & 0xffu);
      }
    }
  }
}

// RB output rows of one warp: rows r0 .. r0+RB-1 of the tile (staged rows
// r0 .. r0+RB+1), lane columns xs .. xs+3.  Two output rows per iteration
// (rolled on purpose: a fully unrolled loop overflowed the instruction
// cache).  Nodata is looked for per row pair: the mask logic runs only when a
// lane of the warp may see nodata in the pair's four rows.  ``srow`` /
// ``arow`` / ``hrow`` point at this lane's first output pixel; ``sp`` /
// ``hp`` are their row pitches in elements.
template <int RB, int WANT, int NDK, bool EDGE, bool VEC>
__device__ __forceinline__ void horn_rows(const float* S, int lane, int r0, int64_t y0, int64_t xs,
                                          const HornParams& P, const MaskRule& rule, float nd_in,
                                          float* __restrict__ srow, float* __restrict__ arow,
                                          uint8_t* __restrict__ hrow, int64_t sp, int64_t hp) {
  static_assert(RB % 2 == 0, "two output rows per iteration");
  // nodata values may be left out of the exactness test when every output
  // whose window holds one is masked (3x3 dilation; not the centre-only rule)
  const bool skip_nd = !rule.sa_center;
  Row r0v, r1v;
  stage_row(S + (r0 + 0) * kSW, lane, r0v);
  stage_row(S + (r0 + 1) * kSW, lane, r1v);
  bool f0 = row_may_hold_nodata<NDK>(r0v, nd_in), f1 = row_may_hold_nodata<NDK>(r1v, nd_in);
  const int64_t y = y0 + r0;
#pragma unroll 1
  for (int j = 0; j < RB; j += 2) {
    Row r2v, r3v;
    stage_row(S + (r0 + j + 2) * kSW, lane, r2v);
    stage_row(S + (r0 + j + 3) * kSW, lane, r3v);
    const bool f2 = row_may_hold_nodata<NDK>(r2v, nd_in), f3 = row_may_hold_nodata<NDK>(r3v, nd_in);
    const bool masked = NDK != VSR_NODATA_NONE && __any_sync(0xffffffffu, f0 | f1 | f2 | f3);
    uint32_t m0 = 0, m1 = 0, m2 = 0, m3 = 0;
    Row a = r0v, b = r1v, c = r2v, d = r3v;  // ranges narrowed to valid values when masked
    if (masked) {
      m0 = row_nodata<NDK>(a, nd_in, skip_nd);
      m1 = row_nodata<NDK>(b, nd_in, skip_nd);
      m2 = row_nodata<NDK>(c, nd_in, skip_nd);
      m3 = row_nodata<NDK>(d, nd_in, skip_nd);
    }
    // both output rows of the pair take the exact form if any lane's window may round
    const float lo = fminf(min3f(a.lo, b.lo, c.lo), d.lo), hi = fmaxf(max3f(a.hi, b.hi, c.hi), d.hi);
    float* srow1 = (WANT & kWantSlope) ? srow + sp : nullptr;
    float* arow1 = (WANT & kWantAspect) ? arow + sp : nullptr;
    uint8_t* hrow1 = (WANT & kWantHs) ? hrow + hp : nullptr;
    float gxa[4], gya[4], gxb[4], gyb[4];
    if (__all_sync(0xffffffffu, window_exact(lo, hi))) {
      grad_fast(r0v, r1v, r2v, gxa, gya);
      grad_fast(r1v, r2v, r3v, gxb, gyb);
    } else {
      grad_exact4(r0v, r1v, r2v, gxa, gya);
      grad_exact4(r1v, r2v, r3v, gxb, gyb);
    }
    horn_out_row<WANT, EDGE, VEC>(gxa, gya, masked, m0, m1, m2, P, rule, y + j, xs, srow, arow, hrow);
    horn_out_row<WANT, EDGE, VEC>(gxb, gyb, masked, m1, m2, m3, P, rule, y + j + 1, xs, srow1, arow1, hrow1);
    if (WANT & kWantSlope) srow = srow1 + sp;
    if (WANT & kWantAspect) arow = arow1 + sp;
    if (WANT & kWantHs) hrow = hrow1 + hp;
    r0v = r2v;
    r1v = r3v;
    f0 = f2;
    f1 = f3;
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

}  // namespace horn
}  // namespace vsr
