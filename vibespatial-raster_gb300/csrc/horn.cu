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
  float zf;
  float cos_z, sin_z, cos_az, sin_az;
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

// Degree-valued arctangent: t * P(t^2) on t in [0, 1], P a degree-8 minimax
// polynomial fitted by csrc/fit_atan.py (max error 3.3e-7 deg in float64,
// 5.3e-6 deg evaluated in float32).  Reduction by octant keeps the axes
// exact: atan2_deg(+-y, 0) = +-90, atan2_deg(0, -x) = 180.
__device__ __forceinline__ float atan_poly_deg(float t) {
  const float u = t * t;
  float p = 0.14075983191003316f;
  p = fmaf(p, u, -0.82513653006899812f);
  p = fmaf(p, u, 2.2792953508350795f);
  p = fmaf(p, u, -4.1452671300469577f);
  p = fmaf(p, u, 6.0154525769063225f);
  p = fmaf(p, u, -8.1137865295205867f);
  p = fmaf(p, u, 11.451081054241243f);
  p = fmaf(p, u, -19.09817129772475f);
  p = fmaf(p, u, 57.29577300327405f);
  return t * p;
}

// atan2(y, x) in degrees, (-180, 180]; NaN in -> NaN out.
__device__ __forceinline__ float atan2_deg(float y, float x) {
  const float ay = fabsf(y), ax = fabsf(x);
  const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
  const float t = mx > 0.0f ? __fdividef(mn, mx) : 0.0f;
  float a = atan_poly_deg(t);
  if (ay > ax) a = 90.0f - a;
  if (signbit(x)) a = 180.0f - a;
  a = copysignf(a, y);
  const float nan_probe = x + y;
  return nan_probe != nan_probe ? nan_probe : a;
}

// atan(sqrt(s)) in degrees for s = p^2 + q^2 >= 0 (NaN propagates).
__device__ __forceinline__ float slope_deg_from_sq(float s) {
  const float r = s > 0.0f ? s * rsqrtf(s) : s;
  const bool big = r > 1.0f;
  const float t = big ? __frcp_rn(r) : r;
  const float a = atan_poly_deg(t);
  return big ? 90.0f - a : a;
}

// gx, gy: raw Horn sums (before the 1/(8 cell) scale).
__device__ __forceinline__ PixelOut horn_pixel(float gx, float gy, const HornParams& P, bool want_s,
                                               bool want_a, bool want_h) {
  PixelOut o;
  const float p = gx * P.inv8cx;
  const float q = gy * P.inv8cy;
  if (want_s) o.slope = slope_deg_from_sq(p * p + q * q);
  if (want_a) {
    const float t = 90.0f - atan2_deg(-q, p);
    o.aspect = t < 0.0f ? t + 360.0f : t;
  }
  if (want_h) {
    const float ph = p * P.zf, qh = q * P.zf;
    const float num = P.cos_z + P.sin_z * (P.cos_az * ph - P.sin_az * qh);
    float hs = num * rsqrtf(1.0f + ph * ph + qh * qh);
    hs = fminf(fmaxf(hs, 0.0f), 1.0f);  // NaN -> 0
    o.hs = static_cast<uint8_t>(__float2uint_rz(hs * 255.0f + 0.5f));
  }
  return o;
}

// ------------------------------------------------------------ TMA kernel --
constexpr int kTW = 128;        // output tile width (32 lanes x 4 pixels)
constexpr int kSW = kTW + 8;    // staged width: 4-column halo each side (16 B)
constexpr int kThreads = 256;

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

__device__ __forceinline__ uint32_t nd_bits6(const float v[6], int kind, float ndv) {
  uint32_t m = 0;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const bool b = (kind == VSR_NODATA_VALUE) ? (v[k] == ndv) : (kind == VSR_NODATA_NAN ? (v[k] != v[k]) : false);
    m |= (b ? 1u : 0u) << k;
  }
  return m;
}

template <int TH, int STAGES>
__global__ void __launch_bounds__(kThreads) horn_f32_tma(const __grid_constant__ CUtensorMap tmap,
                                                         const HornParams P, const float nd_in,
                                                         float* __restrict__ slope,
                                                         float* __restrict__ aspect,
                                                         uint8_t* __restrict__ hs,
                                                         uint32_t* err_word) {
  using Tile = TmaTile<TH>;
  constexpr int RB = TH / (kThreads / 32);  // rows per warp
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[STAGES];
  float* stages = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t W = P.width, H = P.height;
  const int64_t tiles_x = (W + kTW - 1) / kTW;
  const int64_t total = tiles_x * ((H + TH - 1) / TH);
  const MaskRule rule = mask_rule(P);
  const bool want_s = slope != nullptr, want_a = aspect != nullptr, want_h = hs != nullptr;

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
      for (int r = tid; r < Tile::SH; r += kThreads) {
        if (left) S[r * kSW + 3] = S[r * kSW + 4];
        if (right) S[r * kSW + rc] = S[r * kSW + rc - 1];
      }
    }
    if (top || bottom) {
      __syncthreads();
      const int rr = static_cast<int>(H - y0) + 1;  // staged row of y = H
      for (int c = tid; c < kSW; c += kThreads) {
        if (top) S[c] = S[kSW + c];
        if (bottom) S[rr * kSW + c] = S[(rr - 1) * kSW + c];
      }
    }
    __syncthreads();

    // Each warp: RB output rows; each lane: 4 adjacent columns.
    const int64_t xs = x0 + 4 * lane;
    const int r0 = warp * RB;
    float top6[6], mid6[6], bot6[6];
    load6(S + (r0 + 0) * kSW, lane, top6);
    load6(S + (r0 + 1) * kSW, lane, mid6);
    uint32_t mt = nd_bits6(top6, P.nd_kind, nd_in);
    uint32_t mm = nd_bits6(mid6, P.nd_kind, nd_in);
#pragma unroll
    for (int j = 0; j < RB; ++j) {
      load6(S + (r0 + j + 2) * kSW, lane, bot6);
      const uint32_t mb = nd_bits6(bot6, P.nd_kind, nd_in);
      const int64_t y = y0 + r0 + j;
      if (y < H && xs < W) {
        const uint32_t hdil = (mt | (mt >> 1) | (mt >> 2)) | (mm | (mm >> 1) | (mm >> 2)) |
                              (mb | (mb >> 1) | (mb >> 2));
        const uint32_t ctr = mm >> 1;
        float so[4], ao[4];
        uint8_t ho[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float gx = (top6[k + 2] - top6[k]) + 2.0f * (mid6[k + 2] - mid6[k]) + (bot6[k + 2] - bot6[k]);
          const float gy = (bot6[k] - top6[k]) + 2.0f * (bot6[k + 1] - top6[k + 1]) + (bot6[k + 2] - top6[k + 2]);
          PixelOut o = horn_pixel(gx, gy, P, want_s, want_a, want_h);
          const bool sa_nd = rule.sa_any && (((rule.sa_center ? ctr : hdil) >> k) & 1u);
          const bool hs_nd = rule.hs_any && ((hdil >> k) & 1u);
          so[k] = sa_nd ? P.nd_out_f : o.slope;
          ao[k] = sa_nd ? P.nd_out_f : o.aspect;
          ho[k] = hs_nd ? uint8_t(0) : o.hs;
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
        top6[k] = mid6[k];
        mid6[k] = bot6[k];
      }
      mt = mm;
      mm = mb;
    }

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

template <int TH, int STAGES>
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
  auto kern = horn_f32_tma<TH, STAGES>;
  static bool attr_set[64] = {};
  int dev = 0;
  VSR_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 64 && !attr_set[dev]) {
    VSR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    attr_set[dev] = true;
  }
  int per_sm = 0;
  VSR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem));
  if (per_sm < 1) return fail(VSR_ERR_CUDA, "horn_f32_tma cannot be resident (smem %zu)", smem);
  const int64_t tiles = ((P.width + kTW - 1) / kTW) * ((P.height + TH - 1) / TH);
  const int64_t grid = std::min<int64_t>(tiles, static_cast<int64_t>(sm_count()) * per_sm);
  kern<<<static_cast<unsigned>(grid), kThreads, smem, st>>>(map, P, nd_in, slope, aspect, hs, err);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}

}  // namespace
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
  P.cos_z = static_cast<float>(std::cos(zenith_rad));
  P.sin_z = static_cast<float>(std::sin(zenith_rad));
  P.cos_az = static_cast<float>(std::cos(azimuth_rad));
  P.sin_az = static_cast<float>(std::sin(azimuth_rad));
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
    return launch_tma<32, 3>(dem, P, static_cast<float>(ndv), static_cast<float*>(slope),
                             static_cast<float*>(aspect), hillshade, st);
  if ((slope || aspect) && out_dtype == VSR_F64)
    return dispatch_generic<double>(dtype, dem, P, ndv, slope, aspect, hillshade, st);
  return dispatch_generic<float>(dtype, dem, P, ndv, slope, aspect, hillshade, st);
}
