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

// ------------------------------------------------------------ TMA kernel --
constexpr int kTW = 128;        // output tile width (32 lanes x 4 pixels)
constexpr int kSW = kTW + 8;    // staged width: 4-column halo each side (16 B)

template <int TH>
struct TmaTile {
  static constexpr int SH = TH + 2;
  static constexpr uint32_t kBytes = kSW * SH * 4;
  static constexpr uint32_t kStride = (kBytes + 1023u) & ~1023u;
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

// RB output rows of one warp: rows r0 .. r0+RB-1 of the tile (staged rows
// r0 .. r0+RB+1), lane columns xs .. xs+3.  Horizontal differences of a staged
// row are formed once and reused by the three output rows that need them.
template <int RB, bool MASKED>
__device__ __forceinline__ void horn_rows(const float* S, int lane, int r0, int64_t y0, int64_t xs,
                                          const HornParams& P, const MaskRule& rule, float nd_in,
                                          float* __restrict__ slope, float* __restrict__ aspect,
                                          uint8_t* __restrict__ hs) {
  const int64_t W = P.width, H = P.height;
  const bool want_s = slope != nullptr, want_a = aspect != nullptr, want_h = hs != nullptr;
  float top[6], mid[6], bot[6];
  float hdt[4], hdm[4], hdb[4];
  load6(S + (r0 + 0) * kSW, lane, top);
  load6(S + (r0 + 1) * kSW, lane, mid);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    hdt[k] = top[k + 2] - top[k];
    hdm[k] = mid[k + 2] - mid[k];
  }
  uint32_t mt = 0, mm = 0;
  if (MASKED) {
    mt = nd_bits6(top, P.nd_kind, nd_in);
    mm = nd_bits6(mid, P.nd_kind, nd_in);
  }
  // Rolled on purpose: a fully unrolled row loop overflows the instruction
  // cache (ncu: "no instruction" stalls dominated).
#pragma unroll 1
  for (int j = 0; j < RB; ++j) {
    load6(S + (r0 + j + 2) * kSW, lane, bot);
    float dv[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) dv[k] = bot[k] - top[k];
#pragma unroll
    for (int k = 0; k < 4; ++k) hdb[k] = bot[k + 2] - bot[k];
    uint32_t mb = 0;
    if (MASKED) mb = nd_bits6(bot, P.nd_kind, nd_in);
    const int64_t y = y0 + r0 + j;
    if (y < H && xs < W) {
      uint32_t hdil = 0, ctr = 0;
      if (MASKED) {
        hdil = (mt | (mt >> 1) | (mt >> 2)) | (mm | (mm >> 1) | (mm >> 2)) | (mb | (mb >> 1) | (mb >> 2));
        ctr = mm >> 1;
      }
      float so[4], ao[4];
      uint8_t ho[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float gx = fmaf(2.0f, hdm[k], hdt[k] + hdb[k]);
        const float gy = fmaf(2.0f, dv[k + 1], dv[k] + dv[k + 2]);
        const PixelOut o = horn_pixel(gx, gy, P, want_s, want_a, want_h);
        so[k] = o.slope;
        ao[k] = o.aspect;
        ho[k] = o.hs;
        if (MASKED) {
          const bool sa_nd = rule.sa_any && (((rule.sa_center ? ctr : hdil) >> k) & 1u);
          const bool hs_nd = rule.hs_any && ((hdil >> k) & 1u);
          so[k] = sa_nd ? P.nd_out_f : so[k];
          ao[k] = sa_nd ? P.nd_out_f : ao[k];
          ho[k] = hs_nd ? uint8_t(0) : ho[k];
        }
      }
      const bool full = xs + 3 < W;
      if (want_s) {
        float* dst = slope + y * P.out_pitch + xs;
        if (full) __stcs(reinterpret_cast<float4*>(dst), make_float4(so[0], so[1], so[2], so[3]));
        else for (int k = 0; k < 4; ++k) if (xs + k < W) __stcs(dst + k, so[k]);
      }
      if (want_a) {
        float* dst = aspect + y * P.out_pitch + xs;
        if (full) __stcs(reinterpret_cast<float4*>(dst), make_float4(ao[0], ao[1], ao[2], ao[3]));
        else for (int k = 0; k < 4; ++k) if (xs + k < W) __stcs(dst + k, ao[k]);
      }
      if (want_h) {
        uint8_t* dst = hs + y * P.hs_pitch + xs;
        if (full) {
          const uint32_t packed = uint32_t(ho[0]) | (uint32_t(ho[1]) << 8) | (uint32_t(ho[2]) << 16) |
                                  (uint32_t(ho[3]) << 24);
          __stcs(reinterpret_cast<unsigned int*>(dst), packed);
        } else {
          for (int k = 0; k < 4; ++k) if (xs + k < W) dst[k] = ho[k];
        }
      }
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      top[k] = mid[k];
      mid[k] = bot[k];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      hdt[k] = hdm[k];
      hdm[k] = hdb[k];
    }
    mt = mm;
    mm = mb;
  }
}

template <int TH, int STAGES, int THREADS>
__global__ void __launch_bounds__(THREADS) horn_f32_tma(const __grid_constant__ CUtensorMap tmap,
                                                        const HornParams P, const float nd_in,
                                                        float* __restrict__ slope,
                                                        float* __restrict__ aspect,
                                                        uint8_t* __restrict__ hs,
                                                        uint32_t* err_word) {
  using Tile = TmaTile<TH>;
  constexpr int WARPS = THREADS / 32;
  constexpr int RB = TH / WARPS;  // output rows per warp
  static_assert(RB * WARPS == TH, "TH must be a multiple of the warp count");
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[STAGES];
  float* stages = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));

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
    if (__syncthreads_or(!ok)) {
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
    if (masked)
      horn_rows<RB, true>(S, lane, warp * RB, y0, xs, P, rule, nd_in, slope, aspect, hs);
    else
      horn_rows<RB, false>(S, lane, warp * RB, y0, xs, P, rule, nd_in, slope, aspect, hs);

    __syncthreads();  // every read of stage s is done
    if (tid == 0) {
      const int64_t nt = t + static_cast<int64_t>(STAGES) * gridDim.x;
      if (nt < total) {
        fence_proxy_async_smem();  // order the generic-proxy edge patches before the TMA refill
        issue(nt, s);
      }
    }
  }
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
  const float gx = static_cast<float>((v[0][2] - v[0][0]) + D(2) * (v[1][2] - v[1][0]) + (v[2][2] - v[2][0]));
  const float gy = static_cast<float>((v[2][0] - v[0][0]) + D(2) * (v[2][1] - v[0][1]) + (v[2][2] - v[0][2]));
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

template <int TH, int STAGES, int THREADS>
int launch_tma(const void* src, const HornParams& P, float nd_in, float* slope, float* aspect,
               uint8_t* hs, cudaStream_t st) {
  using Tile = TmaTile<TH>;
  CUtensorMap map;
  int rc = encode_tensor_map_2d(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, src, P.width, P.height,
                                P.in_pitch, kSW, Tile::SH);
  if (rc) return rc;
  uint32_t* err = device_error_word();
  if (!err) return VSR_ERR_CUDA;
  const size_t smem = STAGES * Tile::kStride + 1024;
  auto kern = horn_f32_tma<TH, STAGES, THREADS>;
  VSR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  int per_sm = 0;
  VSR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, THREADS, smem));
  if (per_sm < 1) return fail(VSR_ERR_CUDA, "horn_f32_tma cannot be resident (smem %zu)", smem);
  const int64_t tiles = ((P.width + kTW - 1) / kTW) * ((P.height + TH - 1) / TH);
  const int64_t grid = std::min<int64_t>(tiles, static_cast<int64_t>(sm_count()) * per_sm);
  kern<<<static_cast<unsigned>(grid), THREADS, smem, st>>>(map, P, nd_in, slope, aspect, hs, err);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}

// Launch configurations of the TMA kernel the autotuner chooses between:
// (output rows per tile, pipeline stages, threads per CTA).
struct HornConfig {
  int th, stages, threads;
};
constexpr HornConfig kHornConfigs[] = {{32, 3, 256}, {64, 2, 256}, {16, 4, 128}, {32, 2, 128}, {64, 3, 256}};
constexpr int kNumHornConfigs = sizeof(kHornConfigs) / sizeof(kHornConfigs[0]);

int launch_tma_config(int cfg, const void* src, const HornParams& P, float nd_in, float* slope,
                      float* aspect, uint8_t* hs, cudaStream_t st) {
  switch (cfg) {
    case 1: return launch_tma<64, 2, 256>(src, P, nd_in, slope, aspect, hs, st);
    case 2: return launch_tma<16, 4, 128>(src, P, nd_in, slope, aspect, hs, st);
    case 3: return launch_tma<32, 2, 128>(src, P, nd_in, slope, aspect, hs, st);
    case 4: return launch_tma<64, 3, 256>(src, P, nd_in, slope, aspect, hs, st);
    default: return launch_tma<32, 3, 256>(src, P, nd_in, slope, aspect, hs, st);
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
