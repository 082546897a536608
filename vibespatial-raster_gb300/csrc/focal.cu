// Focal convolution (plain FP32), Gaussian filter and focal mean.
//
// * conv_direct  -- nodata-aware normalised correlation (kernels/focal.py:
//   36-146 of the reference).  A CTA stages a (32 + kh - 1) x (128 + kw - 1)
//   tile of v*valid and valid into shared memory (v*valid keeps the
//   reference's NaN * 0 = NaN poisoning), then each thread accumulates a
//   4 x 4 register block of outputs with a register window sliding along the
//   row (kernel width bucketed at compile time, the loop guarded by the
//   runtime width), one row partial sum per kernel row (for accuracy) and
//   16-byte broadcast weight loads.  The weight-sum pass runs only on tiles
//   that touch the border or hold nodata; other tiles use the full sum.
// * sep_tile     -- the Gaussian as two 1-D passes inside one CTA: the row
//   pass over the staged tile is held in shared memory and the column pass
//   reads it.  Numerator and weight sum are both separable, so this equals
//   the reference's dense k x k normalised correlation with weights
//   outer(g, g)/sum in real arithmetic, border and nodata handling included.
// * box_mean     -- focal mean as exact separable sums: int32 for <= 16-bit
//   integer rasters, float TwoSum pairs for float32, float64 otherwise;
//   mean = sum / count formed in float64 (reference: Welford in float64,
//   kernels/focal.py:672-769 / scipy generic_filter, algebra.py:3083-3101).
#include <algorithm>
#include <type_traits>
#include <cmath>

#include "vsr_internal.cuh"

namespace vsr {
namespace {

// ------------------------------------------------------------ element IO --
struct NodataSpec {
  int kind;     // resolved VSR_NODATA_*
  float fv;     // value as float (float32 rasters)
  double dv;    // value as double (float64 rasters)
  int64_t iv;   // value as integer (integer rasters)
};

// Load element ``idx`` of a raster of ``dtype``; returns the value as float
// and sets ``valid`` (not nodata).
__device__ __forceinline__ float load_elem(const void* base, int dtype, int64_t idx,
                                           const NodataSpec& nd, bool& valid) {
  switch (dtype) {
    case VSR_F32: {
      const float v = __ldg(static_cast<const float*>(base) + idx);
      valid = !(nd.kind == VSR_NODATA_VALUE ? v == nd.fv : (nd.kind == VSR_NODATA_NAN ? v != v : false));
      return v;
    }
    case VSR_F64: {
      const double v = __ldg(static_cast<const double*>(base) + idx);
      valid = !(nd.kind == VSR_NODATA_VALUE ? v == nd.dv : (nd.kind == VSR_NODATA_NAN ? v != v : false));
      return static_cast<float>(v);
    }
    case VSR_U8: {
      const int v = __ldg(static_cast<const uint8_t*>(base) + idx);
      valid = !(nd.kind == VSR_NODATA_VALUE && v == nd.iv);
      return static_cast<float>(v);
    }
    case VSR_I16: {
      const int v = __ldg(static_cast<const int16_t*>(base) + idx);
      valid = !(nd.kind == VSR_NODATA_VALUE && v == nd.iv);
      return static_cast<float>(v);
    }
    case VSR_U16: {
      const int v = __ldg(static_cast<const uint16_t*>(base) + idx);
      valid = !(nd.kind == VSR_NODATA_VALUE && v == nd.iv);
      return static_cast<float>(v);
    }
    default: {
      const int v = __ldg(static_cast<const int32_t*>(base) + idx);
      valid = !(nd.kind == VSR_NODATA_VALUE && v == nd.iv);
      return static_cast<float>(v);
    }
  }
}

__device__ __forceinline__ int elem_size(int dtype) {
  return dtype == VSR_U8 ? 1 : (dtype == VSR_I16 || dtype == VSR_U16) ? 2 : (dtype == VSR_F64 ? 8 : 4);
}

// Base pointer of band blockIdx.z (band-first stacks, ``stride`` elements apart).
__device__ __forceinline__ const void* band_src(const void* p, int dtype, int64_t stride) {
  return static_cast<const char*>(p) + static_cast<int64_t>(blockIdx.z) * stride * elem_size(dtype);
}
__device__ __forceinline__ void* band_dst(void* p, int out_dtype, int64_t stride) {
  return static_cast<char*>(p) + static_cast<int64_t>(blockIdx.z) * stride * (out_dtype == VSR_F64 ? 8 : 4);
}

__device__ __forceinline__ void store_out(void* dst, int out_dtype, int64_t idx, double v) {
  if (out_dtype == VSR_F64) static_cast<double*>(dst)[idx] = v;
  else static_cast<float*>(dst)[idx] = static_cast<float>(v);
}

NodataSpec make_nodata(int dtype, double nodata, int kind) {
  NodataSpec s{};
  double ev = 0.0;
  s.kind = resolve_nodata(dtype, nodata, kind, &ev);
  s.dv = ev;
  s.fv = static_cast<float>(ev);
  s.iv = static_cast<int64_t>(ev);
  return s;
}

// Bank-spreading position inside a staged row: one pad word per 32 floats,
// so lanes reading 4 columns apart hit distinct banks.
__device__ __forceinline__ int pos(int c) { return c + (c >> 5); }
__host__ __device__ inline int padded_width(int w) { return w + (w >> 5) + 1; }

// ---------------------------------------------------------- weight prep --
// float64 weights -> float32 rows padded to a multiple of 4 (zero fill) and
// the float64 total.  One CTA.
__global__ void prep_weights(const double* __restrict__ w64, int kh, int kw, int kw4,
                             float* __restrict__ w32, float* __restrict__ wsum) {
  __shared__ double part[256];
  double acc = 0.0;
  for (int i = threadIdx.x; i < kh * kw4; i += blockDim.x) {
    const int r = i / kw4, c = i % kw4;
    const double v = c < kw ? w64[r * kw + c] : 0.0;
    w32[i] = static_cast<float>(v);
    acc += v;
  }
  part[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) part[threadIdx.x] += part[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) wsum[0] = static_cast<float>(part[0]);
}

// Gaussian weights in float64 on the device: g_i = exp(-0.5 ((i - k/2)/sigma)^2),
// as float32 g (1-D, padded to a multiple of 4) and, when ``w2`` is given,
// the dense outer(g, g) / sum as float32 rows padded to k4 (the reference's
// weights, algebra.py:2149-2152) plus its float64 total.
__global__ void prep_gaussian(int k, int k4, double sigma, float* __restrict__ g32,
                              float* __restrict__ w2, float* __restrict__ wsum) {
  extern __shared__ double g64[];
  for (int i = threadIdx.x; i < k; i += blockDim.x) {
    const double a = (i - k / 2) / sigma;
    g64[i] = exp(-0.5 * a * a);
  }
  __syncthreads();
  __shared__ double total;
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < k; ++i) s += g64[i];
    total = s * s;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < k4; i += blockDim.x) g32[i] = i < k ? static_cast<float>(g64[i]) : 0.0f;
  if (w2) {
    for (int i = threadIdx.x; i < k * k4; i += blockDim.x) {
      const int r = i / k4, c = i % k4;
      w2[i] = c < k ? static_cast<float>(g64[r] * g64[c] / total) : 0.0f;
    }
    if (threadIdx.x == 0) wsum[0] = 1.0f;
  }
}

// ---------------------------------------------------------- conv_direct --
constexpr int kCRX = 4, kCRY = 4;            // outputs per thread (x, y)
constexpr int kCTW = 32 * kCRX, kCTH = 8 * kCRY;  // 128 x 32 tile, 256 threads

struct ConvArgs {
  const void* src;
  int dtype;
  int64_t H, W, pitch;
  NodataSpec nd;
  const float* w32;   // kh x kw4
  const float* wsum;  // total weight (float)
  int kh, kw, kw4;
  double nd_out;
  void* dst;
  int out_dtype;
  int64_t out_pitch;
  int64_t band_stride, out_band_stride;  // elements between bands (grid z)
};

inline size_t conv_smem_bytes(int kh, int kw) {
  const int SH = kCTH + kh - 1, SW = kCTW + kw - 1;
  const int kw4 = (kw + 3) & ~3;
  return static_cast<size_t>(2 * SH * padded_width(SW) + kh * kw4) * 4 + 16;
}

// One pass of register-blocked correlation over plane ``P`` (v*valid or valid).
template <int MAXW>
__device__ __forceinline__ void conv_accumulate(const float* __restrict__ P, int PW,
                                                const float* __restrict__ wt, int kh, int kw, int kw4,
                                                int r0, int c0, float acc[kCRY][kCRX]) {
  for (int iy = 0; iy < kCRY + kh - 1; ++iy) {
    float V[kCRX + MAXW - 1];
    const float* row = P + (r0 + iy) * PW;
#pragma unroll
    for (int j = 0; j < kCRX + MAXW - 1; ++j)
      V[j] = (j < kCRX + kw - 1) ? row[pos(c0 + j)] : 0.0f;
#pragma unroll
    for (int ry = 0; ry < kCRY; ++ry) {
      const int ky = iy - ry;
      if (ky < 0 || ky >= kh) continue;
      const float* wr = wt + ky * kw4;
      float part[kCRX] = {};
#pragma unroll
      for (int kx = 0; kx < MAXW; kx += 4) {
        if (kx >= kw) break;
        const float4 w4 = *reinterpret_cast<const float4*>(wr + kx);
        const float wv[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          // never multiply a zero pad weight: a NaN outside this output's
          // window must not leak in through 0 * NaN
          if (kx + u < kw) {
#pragma unroll
            for (int rx = 0; rx < kCRX; ++rx) part[rx] = fmaf(wv[u], V[rx + kx + u], part[rx]);
          }
        }
      }
#pragma unroll
      for (int rx = 0; rx < kCRX; ++rx) acc[ry][rx] += part[rx];
    }
  }
}

template <int MAXW>
__global__ void __launch_bounds__(256) conv_direct(const ConvArgs a) {
  extern __shared__ __align__(16) float smem[];
  const int SH = kCTH + a.kh - 1, SW = kCTW + a.kw - 1, PW = padded_width(SW);
  float* vz = smem;
  float* vd = vz + SH * PW;
  float* wt = vd + SH * PW;  // 16-byte aligned: SH*PW*2 floats precede it
  // keep wt 16-byte aligned
  wt = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(wt) + 15) & ~uintptr_t(15));
  const int tid = threadIdx.y * 32 + threadIdx.x;
  const int64_t x0 = static_cast<int64_t>(blockIdx.x) * kCTW;
  const int64_t y0 = static_cast<int64_t>(blockIdx.y) * kCTH;
  const int px = a.kw / 2, py = a.kh / 2;
  const void* src = band_src(a.src, a.dtype, a.band_stride);
  void* dst = band_dst(a.dst, a.out_dtype, a.out_band_stride);

  for (int i = tid; i < a.kh * a.kw4; i += 256) wt[i] = a.w32[i];
  bool any_gap = false;
  for (int i = tid; i < SH * SW; i += 256) {
    const int r = i / SW, c = i - r * SW;
    const int64_t gy = y0 + r - py, gx = x0 + c - px;
    float v = 0.0f, d = 0.0f;
    if (gy >= 0 && gy < a.H && gx >= 0 && gx < a.W) {
      bool ok;
      const float x = load_elem(src, a.dtype, gy * a.pitch + gx, a.nd, ok);
      v = x * (ok ? 1.0f : 0.0f);  // NaN * 0 stays NaN, as in the reference
      d = ok ? 1.0f : 0.0f;
      any_gap |= !ok;
    } else {
      any_gap = true;
    }
    vz[r * PW + pos(c)] = v;
    vd[r * PW + pos(c)] = d;
  }
  const bool need_den = __syncthreads_or(any_gap);

  const int r0 = threadIdx.y * kCRY, c0 = threadIdx.x * kCRX;
  float num[kCRY][kCRX] = {};
  conv_accumulate<MAXW>(vz, PW, wt, a.kh, a.kw, a.kw4, r0, c0, num);
  float den[kCRY][kCRX];
  if (need_den) {
#pragma unroll
    for (int ry = 0; ry < kCRY; ++ry)
#pragma unroll
      for (int rx = 0; rx < kCRX; ++rx) den[ry][rx] = 0.0f;
    conv_accumulate<MAXW>(vd, PW, wt, a.kh, a.kw, a.kw4, r0, c0, den);
  } else {
    const float ws = *a.wsum;
#pragma unroll
    for (int ry = 0; ry < kCRY; ++ry)
#pragma unroll
      for (int rx = 0; rx < kCRX; ++rx) den[ry][rx] = ws;
  }
#pragma unroll
  for (int ry = 0; ry < kCRY; ++ry) {
    const int64_t y = y0 + r0 + ry;
    if (y >= a.H) break;
#pragma unroll
    for (int rx = 0; rx < kCRX; ++rx) {
      const int64_t x = x0 + c0 + rx;
      if (x >= a.W) break;
      const bool centre_ok = vd[(r0 + ry + py) * PW + pos(c0 + rx + px)] != 0.0f;
      const float dn = den[ry][rx];
      const double out = (centre_ok && dn > 0.0f) ? static_cast<double>(num[ry][rx] / dn) : a.nd_out;
      store_out(dst, a.out_dtype, y * a.out_pitch + x, out);
    }
  }
}

template <int MAXW>
int launch_conv_direct(const ConvArgs& a, cudaStream_t st, int bands = 1) {
  const size_t smem = conv_smem_bytes(a.kh, a.kw);
  auto kern = conv_direct<MAXW>;
  VSR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  dim3 grid(static_cast<unsigned>((a.W + kCTW - 1) / kCTW), static_cast<unsigned>((a.H + kCTH - 1) / kCTH), bands);
  if (grid.y > 65535u) return fail(VSR_ERR_UNSUPPORTED, "raster too tall for the direct convolution grid");
  kern<<<grid, dim3(32, 8), smem, st>>>(a);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}

int run_conv_direct(const ConvArgs& a, cudaStream_t st, int bands = 1) {
  if (a.kw <= 4) return launch_conv_direct<4>(a, st, bands);
  if (a.kw <= 8) return launch_conv_direct<8>(a, st, bands);
  if (a.kw <= 16) return launch_conv_direct<16>(a, st, bands);
  if (a.kw <= 32) return launch_conv_direct<32>(a, st, bands);
  if (a.kw <= 48) return launch_conv_direct<48>(a, st, bands);
  if (a.kw <= 64) return launch_conv_direct<64>(a, st, bands);
  return launch_conv_direct<80>(a, st, bands);
}

constexpr int kMaxDirectK = 80;

// ------------------------------------------------------------- sep_tile --
// Separable Gaussian for k <= 33 within a 128 x 32 output tile.
constexpr int kSTW = 128, kSTH = 32;

struct SepArgs {
  const void* src;
  int dtype;
  int64_t H, W, pitch;
  NodataSpec nd;
  const float* g32;  // k4 floats
  int k;
  double nd_out;
  void* dst;
  int out_dtype;
  int64_t out_pitch;
  int64_t band_stride, out_band_stride;
};

inline size_t sep_smem_bytes(int k) {
  const int SH = kSTH + k - 1, SW = kSTW + k - 1;
  // staged v*valid and valid, row-pass numerator and denominator, weights
  return static_cast<size_t>(((2 * SH * padded_width(SW) + 3) & ~3) + 2 * SH * kSTW + ((k + 3) & ~3)) * 4 + 16;
}

template <int MAXK>
__global__ void __launch_bounds__(256) sep_tile(const SepArgs a) {
  extern __shared__ __align__(16) float smem[];
  const int k = a.k, r = k / 2;
  const int SH = kSTH + k - 1, SW = kSTW + k - 1, PW = padded_width(SW);
  float* vz = smem;
  float* vd = vz + SH * PW;
  float* rn = vz + ((2 * SH * PW + 3) & ~3);  // SH x kSTW row-pass numerator (16-byte aligned)
  float* rd = rn + SH * kSTW;
  float* g = rd + SH * kSTW;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t x0 = static_cast<int64_t>(blockIdx.x) * kSTW;
  const int64_t y0 = static_cast<int64_t>(blockIdx.y) * kSTH;
  const void* src = band_src(a.src, a.dtype, a.band_stride);
  void* dst = band_dst(a.dst, a.out_dtype, a.out_band_stride);

  for (int i = tid; i < k; i += 256) g[i] = a.g32[i];
  for (int i = tid; i < SH * SW; i += 256) {
    const int rr = i / SW, c = i - rr * SW;
    const int64_t gy = y0 + rr - r, gx = x0 + c - r;
    float v = 0.0f, d = 0.0f;
    if (gy >= 0 && gy < a.H && gx >= 0 && gx < a.W) {
      bool ok;
      const float x = load_elem(src, a.dtype, gy * a.pitch + gx, a.nd, ok);
      v = x * (ok ? 1.0f : 0.0f);
      d = ok ? 1.0f : 0.0f;
    }
    vz[rr * PW + pos(c)] = v;
    vd[rr * PW + pos(c)] = d;
  }
  __syncthreads();

  // Row pass: each lane 4 adjacent columns of one staged row.
  for (int rr = warp; rr < SH; rr += 8) {
    const int c0 = 4 * lane;
#pragma unroll
    for (int plane = 0; plane < 2; ++plane) {
      const float* row = (plane == 0 ? vz : vd) + rr * PW;
      float V[4 + MAXK - 1];
#pragma unroll
      for (int j = 0; j < 4 + MAXK - 1; ++j) V[j] = (j < 4 + k - 1) ? row[pos(c0 + j)] : 0.0f;
      float acc[4] = {};
#pragma unroll
      for (int t = 0; t < MAXK; ++t) {
        if (t >= k) break;
        const float w = g[t];
#pragma unroll
        for (int u = 0; u < 4; ++u) acc[u] = fmaf(w, V[u + t], acc[u]);
      }
      float* o = (plane == 0 ? rn : rd) + rr * kSTW + c0;
      *reinterpret_cast<float4*>(o) = make_float4(acc[0], acc[1], acc[2], acc[3]);
    }
  }
  __syncthreads();

  // Column pass: each thread one column, 16 consecutive output rows.
  constexpr int RY = kSTH / 2;
  const int c = tid & (kSTW - 1);
  const int q0 = (tid >> 7) * RY;
  float num[RY] = {}, den[RY] = {};
#pragma unroll
  for (int plane = 0; plane < 2; ++plane) {
    const float* P = plane == 0 ? rn : rd;
    float* acc = plane == 0 ? num : den;
    for (int i = 0; i < RY + k - 1; ++i) {
      const float v = P[(q0 + i) * kSTW + c];
#pragma unroll
      for (int ry = 0; ry < RY; ++ry) {
        const int t = i - ry;
        if (t >= 0 && t < k) acc[ry] = fmaf(g[t], v, acc[ry]);
      }
    }
  }
  const int64_t x = x0 + c;
  if (x < a.W) {
#pragma unroll
    for (int ry = 0; ry < RY; ++ry) {
      const int64_t y = y0 + q0 + ry;
      if (y >= a.H) break;
      const bool centre_ok = vd[(q0 + ry + r) * PW + pos(c + r)] != 0.0f;
      const double out = (centre_ok && den[ry] > 0.0f) ? static_cast<double>(num[ry] / den[ry]) : a.nd_out;
      store_out(dst, a.out_dtype, y * a.out_pitch + x, out);
    }
  }
}

template <int MAXK>
int launch_sep(const SepArgs& a, cudaStream_t st, int bands = 1) {
  const size_t smem = sep_smem_bytes(a.k);
  auto kern = sep_tile<MAXK>;
  VSR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  dim3 grid(static_cast<unsigned>((a.W + kSTW - 1) / kSTW), static_cast<unsigned>((a.H + kSTH - 1) / kSTH), bands);
  if (grid.y > 65535u) return fail(VSR_ERR_UNSUPPORTED, "raster too tall for the separable Gaussian grid");
  kern<<<grid, 256, smem, st>>>(a);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}

constexpr int kMaxSepK = 33;

// ------------------------------------------------------------ sep_strip --
// Separable Gaussian for large k (> 33, e.g. sigma 8 -> 65 x 65): a CTA walks
// a 128-column strip down a 512-row segment.  Every input row is reduced
// along x once (row pass) into a ring of the last k + 15 row results; every
// 16 new rows the column pass combines k ring rows into 16 output rows.
// Numerator (v * valid) and weight sum (valid) travel together as float2
// pairs through Blackwell's packed FP32 FMA (fma.rn.f32x2), so both sums cost
// one instruction per tap.  Each lane makes 8 adjacent outputs per pass from
// a register window of 15 values advanced 8 taps at a time, the tap weight a
// shared-memory broadcast.  Work per output pixel: 2k packed FMAs.
constexpr int kSTW2 = 128;  // strip width
constexpr int kSBR = 16;    // rows per step
constexpr int kSSEG = 512;  // rows per CTA segment

__host__ __device__ inline int strip_pos(int i) { return i + (i >> 3); }  // conflict-free 8-wide lane strides
__host__ __device__ inline int strip_pw(int k) { return strip_pos(kSTW2 + k + 7) + 1; }
// Ring rows: output rows are produced in groups of 16 aligned to the segment
// start; a group's k window rows plus the 15 rows staged past them must fit,
// and with a multiple of 16 every window starts on a multiple of 8 slots,
// so the ring wraps only between 8-row blocks.
__host__ __device__ inline int strip_nr(int k) { return ((k - 1 + 15) & ~15) + kSBR; }
// Position of column c in a ring row: column pairs XOR-swizzled inside each
// group of 8 pairs, so the row pass's 16-byte stores (lane l: pairs 4l .. 4l+3)
// spread over all banks while a warp's 32 consecutive columns in the column
// pass still cover one contiguous 256-byte span.
__device__ __forceinline__ int ring_pos(int c) { return c ^ (((c >> 4) & 7) << 1); }

inline size_t strip_smem_bytes(int k) {
  const int NR = strip_nr(k);
  const int k8 = (k + 7) & ~7;
  return (static_cast<size_t>(NR) * kSTW2 + static_cast<size_t>(kSBR) * strip_pw(k) + k8) * sizeof(float2) +
         static_cast<size_t>(NR) * 8 * 4 + 16;  // + validity bits of 256 staged columns per ring row
}

// acc[u] += sum_{t < k} g2[t] * fetch(u + t) for u = 0..7: 8 outputs from a
// 15-value register window advanced 8 taps at a time.  KB > 0: k lies in
// (8 (KB - 1), 8 KB] and the blocks are unrolled (the window shift becomes
// register renaming, only the last block's taps are tested against k);
// KB == 0: run-time k, full blocks unguarded, then the remainder.  Taps past
// k are never multiplied: their window values may be NaN.
template <int KB, class Fetch>
__device__ __forceinline__ void taps8(const float2* __restrict__ g2, int k, Fetch fetch, float2 acc[8]) {
  float2 win[15];
#pragma unroll
  for (int j = 0; j < 7; ++j) win[j] = fetch(j);
  if (KB > 0) {
#pragma unroll
    for (int b = 0; b < KB; ++b) {
#pragma unroll
      for (int j = 0; j < 8; ++j) win[7 + j] = fetch(8 * b + 7 + j);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        if (b < KB - 1 || 8 * b + j < k) {
          const float2 w = g2[8 * b + j];
#pragma unroll
          for (int u = 0; u < 8; ++u) acc[u] = __ffma2_rn(w, win[u + j], acc[u]);
        }
      }
#pragma unroll
      for (int j = 0; j < 7; ++j) win[j] = win[8 + j];
    }
  } else {
    int t = 0;
    for (; t + 8 <= k; t += 8) {
#pragma unroll
      for (int j = 0; j < 8; ++j) win[7 + j] = fetch(t + 7 + j);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float2 w = g2[t + j];
#pragma unroll
        for (int u = 0; u < 8; ++u) acc[u] = __ffma2_rn(w, win[u + j], acc[u]);
      }
#pragma unroll
      for (int j = 0; j < 7; ++j) win[j] = win[8 + j];
    }
    if (t < k) {
#pragma unroll
      for (int j = 0; j < 8; ++j) win[7 + j] = fetch(t + 7 + j);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        if (t + j < k) {
          const float2 w = g2[t + j];
#pragma unroll
          for (int u = 0; u < 8; ++u) acc[u] = __ffma2_rn(w, win[u + j], acc[u]);
        }
      }
    }
  }
}

// One staged tap: (v * valid, valid); out-of-raster taps are (0, 0).  DT is
// the raster's dtype when known at compile time (0: dispatch at run time).
template <int DT>
__device__ __forceinline__ float2 strip_tap(const void* src, int dtype, int64_t idx, const NodataSpec& nd) {
  bool ok;
  float x;
  if (DT == VSR_U16) {
    const int v = __ldg(static_cast<const uint16_t*>(src) + idx);
    ok = !(nd.kind == VSR_NODATA_VALUE && v == nd.iv);
    x = static_cast<float>(v);
  } else if (DT == VSR_F32) {
    x = __ldg(static_cast<const float*>(src) + idx);
    ok = !(nd.kind == VSR_NODATA_VALUE ? x == nd.fv : (nd.kind == VSR_NODATA_NAN ? x != x : false));
  } else {
    x = load_elem(src, dtype, idx, nd, ok);
  }
  return make_float2(x * (ok ? 1.0f : 0.0f), ok ? 1.0f : 0.0f);  // NaN * 0 stays NaN (reference poisoning)
}

template <int DT, int KB>
__global__ void __launch_bounds__(256, 2) sep_strip(const SepArgs a) {
  extern __shared__ __align__(16) float2 ssm2[];
  const int k = a.k, r = k / 2;
  const int NR = strip_nr(k);
  const int PW = strip_pw(k);
  const int k8 = (k + 7) & ~7;
  float2* ring = ssm2;                  // NR x 128 (num, den) row-pass results
  float2* stg = ring + NR * kSTW2;      // kSBR x PW staged (v * valid, valid)
  float2* g2 = stg + kSBR * PW;         // k8 weight pairs (w, w), zero padded
  uint32_t* vbits = reinterpret_cast<uint32_t*>(g2 + k8);  // NR x 8 words: staged-column validity bits
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t x0 = static_cast<int64_t>(blockIdx.x) * kSTW2;
  const int64_t ys = static_cast<int64_t>(blockIdx.y) * kSSEG;
  const int64_t ye = min(ys + kSSEG, a.H);
  const void* src = band_src(a.src, a.dtype, a.band_stride);
  void* dst = band_dst(a.dst, a.out_dtype, a.out_band_stride);
  for (int i = tid; i < k8; i += 256) {
    const float w = i < k ? a.g32[i] : 0.0f;
    g2[i] = make_float2(w, w);
  }
  const int SW = kSTW2 + k - 1;  // staged columns x0 - r .. x0 + 127 + r
  // Input rows ys - r .. ye + r - 1 pass through the ring; row gy lives in
  // slot (gy - (ys - r)) % NR.
  const int64_t first = ys - r;
  const int64_t last = ye + r;  // exclusive
  int64_t next_out = ys;
  // staging: thread tid takes column tid (SW <= 128 + 79 < 256 threads) of
  // each of the kSBR rows.  The next step's taps are loaded into registers
  // during this step's passes and kept raw (uint16 / float; other dtypes
  // converted at load), so nothing waits on the loads until the values are
  // stored to shared memory at the start of the next step.
  using Raw = std::conditional_t<DT == VSR_U16, uint32_t, std::conditional_t<DT == VSR_F32, float, float2>>;
  Raw pre[kSBR];
  uint32_t pin = 0;  // bit q: tap q of the staged step lies in the raster
  const int c_st = tid;
  auto load_step = [&](int64_t rb) {
    pin = 0;
    const int64_t gx = x0 + c_st - r;
    const bool col_in = c_st < SW && gx >= 0 && gx < a.W;
#pragma unroll
    for (int q = 0; q < kSBR; ++q) {
      const int64_t gy = rb + q;
      const bool in = col_in && gy < last && gy >= 0 && gy < a.H;
      const int64_t idx = gy * a.pitch + gx;
      if constexpr (DT == VSR_U16) pre[q] = in ? static_cast<uint32_t>(__ldg(static_cast<const uint16_t*>(src) + idx)) : 0u;
      else if constexpr (DT == VSR_F32) pre[q] = in ? __ldg(static_cast<const float*>(src) + idx) : 0.0f;
      else pre[q] = in ? strip_tap<DT>(src, a.dtype, idx, a.nd) : make_float2(0.0f, 0.0f);
      pin |= (in ? 1u : 0u) << q;
    }
  };
  // staged tap q as (v * valid, valid); NaN * 0 stays NaN (reference poisoning)
  auto tap_of = [&](int q) -> float2 {
    const bool in = (pin >> q) & 1u;
    if constexpr (DT == VSR_U16) {
      const bool ok = in && !(a.nd.kind == VSR_NODATA_VALUE && static_cast<int>(pre[q]) == a.nd.iv);
      return make_float2(ok ? static_cast<float>(pre[q]) : 0.0f, ok ? 1.0f : 0.0f);
    } else if constexpr (DT == VSR_F32) {
      const float x = pre[q];
      const bool ok = in && !(a.nd.kind == VSR_NODATA_VALUE ? x == a.nd.fv : (a.nd.kind == VSR_NODATA_NAN ? x != x : false));
      return make_float2(x * (ok ? 1.0f : 0.0f), ok ? 1.0f : 0.0f);
    } else {
      return pre[q];
    }
  };
  load_step(first);
  __syncthreads();  // weights
  int slot_rb = 0;  // ring slot of row rb: (rb - first) % NR, kept incrementally
  for (int64_t rb = first; rb < last; rb += kSBR, slot_rb = (slot_rb + kSBR) % NR) {
    // No barrier needed here: the staging rows were last read by the previous
    // row pass (before its column pass); the barrier below keeps this step's
    // row pass from overwriting ring rows the previous column pass reads.
#pragma unroll
    for (int q = 0; q < kSBR; ++q) {
      const float2 t = tap_of(q);
      if (c_st < SW) stg[q * PW + strip_pos(c_st)] = t;
      // validity of staged column c_st (the column pass reads its centres' bits)
      const uint32_t bits = __ballot_sync(0xffffffffu, c_st < SW && t.y != 0.0f);
      if (lane == 0) {
        const int sq = slot_rb + q;
        vbits[(sq >= NR ? sq - NR : sq) * 8 + (c_st >> 5)] = bits;
      }
    }
    __syncthreads();
    if (rb + kSBR < last) load_step(rb + kSBR);
    // row pass: half-warp h takes staged row 2 warp + h, 8 columns per lane
    {
      const int q = 2 * warp + (lane >> 4);
      const int64_t gy = rb + q;
      if (gy < last) {
        const int slot = slot_rb + q >= NR ? slot_rb + q - NR : slot_rb + q;
        const int c0 = 8 * (lane & 15);
        // staged column c0 + i sits at strip_pos(c0 + i) = 9 (c0 / 8) + i + i / 8
        const float2* row = stg + q * PW + 9 * (lane & 15);
        float2 acc[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) acc[u] = make_float2(0.0f, 0.0f);
        taps8<KB>(g2, k, [&](int i) { return row[i + (i >> 3)]; }, acc);  // reads stay inside the padded row
        float2* dst_ring = ring + slot * kSTW2;
#pragma unroll
        for (int u = 0; u < 8; u += 2)
          *reinterpret_cast<float4*>(dst_ring + ring_pos(c0 + u)) =
              make_float4(acc[u].x, acc[u].y, acc[u + 1].x, acc[u + 1].y);
      }
    }
    __syncthreads();
    // column pass: output rows in groups of 16 aligned to the segment start;
    // a group runs once the last row of its last window (y - r + k - 1) is
    // in the ring (one group per step, two at most at the segment end):
    // 2 sets of 128 threads, 8 rows each
    while (next_out < ye) {
      const int64_t ready_to = min(next_out + kSBR, ye);
      if (ready_to - 1 - r + k - 1 >= rb + kSBR) break;
      const int c = tid & (kSTW2 - 1);
      const int grp = tid >> 7;
      const int64_t x = x0 + c;
      const int64_t yb = next_out + 8 * grp;
      if (yb < ready_to) {
        float2 acc[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) acc[u] = make_float2(0.0f, 0.0f);
        // slot of row yb - r: yb - ys is a multiple of 8 and NR of 16, so
        // sl0 is a multiple of 8 and the window wraps (once at most) only
        // between 8-row blocks: one slot test per block, the block's rows at
        // fixed offsets.  Slots past the window hold other rows: read,
        // never multiplied
        const int sl0 = static_cast<int>(yb - r - first) % NR;
        const float2* col = ring + ring_pos(c);
        taps8<KB>(g2, k, [&](int i) {
          const int sb = sl0 + (i & ~7);
          return col[((sb >= NR ? sb - NR : sb) + (i & 7)) * kSTW2];
        }, acc);
        if (x < a.W) {
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int64_t y = yb + u;
            if (y >= ready_to) break;
            // centre validity: its staged weight was 1 (in the raster and not nodata);
            // row y = yb + u sits r + u slots after row yb - r
            int sc = sl0 + r + u;
            sc = sc >= NR ? sc - NR : sc;
            const bool centre_ok = (vbits[sc * 8 + ((c + r) >> 5)] >> ((c + r) & 31)) & 1u;
            const float num = acc[u].x, den = acc[u].y;
            const bool ok = centre_ok && den > 0.0f;
            if (a.out_dtype == VSR_F64) static_cast<double*>(dst)[y * a.out_pitch + x] = ok ? static_cast<double>(num / den) : a.nd_out;
            else static_cast<float*>(dst)[y * a.out_pitch + x] = ok ? num / den : static_cast<float>(a.nd_out);
          }
        }
      }
      next_out = ready_to;
    }
  }
}

int launch_strip(const SepArgs& a, cudaStream_t st, int bands) {
  const size_t smem = strip_smem_bytes(a.k);
  if (smem > 227 * 1024) return fail(VSR_ERR_UNSUPPORTED, "Gaussian kernel %d too large for the strip kernel", a.k);
  // the taps of k in 65..72 (sigma 8 at 4 sigma) are unrolled; other k run-time
  const bool k9 = a.k > 64 && a.k <= 72;
  auto kern = a.dtype == VSR_U16 ? (k9 ? sep_strip<VSR_U16, 9> : sep_strip<VSR_U16, 0>)
              : a.dtype == VSR_F32 ? (k9 ? sep_strip<VSR_F32, 9> : sep_strip<VSR_F32, 0>)
                                   : (k9 ? sep_strip<0, 9> : sep_strip<0, 0>);
  VSR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  dim3 grid(static_cast<unsigned>((a.W + kSTW2 - 1) / kSTW2), static_cast<unsigned>((a.H + kSSEG - 1) / kSSEG), bands);
  if (grid.y > 65535u) return fail(VSR_ERR_UNSUPPORTED, "raster too tall for the Gaussian grid");
  kern<<<grid, 256, smem, st>>>(a);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}

// ------------------------------------------------------------- box_mean --
// Accumulators of the general kernel: float TwoSum pairs (float32 rasters),
// float64 (everything else; 8/16-bit rasters reach it only for windows too
// large for the exact integer kernels).
struct AccF2 {
  float s, c;
  __device__ void zero() { s = 0.0f; c = 0.0f; }
  __device__ void add_term(float v) {
    // TwoSum (Knuth): s + v = t + e exactly
    const float t = s + v;
    const float bp = t - s;
    const float e = (s - (t - bp)) + (v - bp);
    s = t;
    c += e;
  }
  __device__ void add(float v) { add_term(v); }
  __device__ void add(const AccF2& o) { add_term(o.s); c += o.c; }
  __device__ double value() const { return static_cast<double>(s) + static_cast<double>(c); }
};
struct AccD {
  double s;
  __device__ void zero() { s = 0.0; }
  __device__ void add(double v) { s += v; }
  __device__ void add(const AccD& o) { s += o.s; }
  __device__ double value() const { return s; }
};

constexpr int kBTW = 128, kBTH = 32;

struct BoxArgs {
  const void* src;
  int dtype;
  int64_t H, W, pitch;
  NodataSpec nd;
  int ry, rx;
  double nd_out;
  void* dst;
  int out_dtype;
  int64_t out_pitch;
  int64_t band_stride, out_band_stride;
};

template <class Acc>
inline size_t box_smem_bytes(int ry, int rx) {
  const int SH = kBTH + 2 * ry, SW = kBTW + 2 * rx;
  // staged value (as Acc input) + valid byte; row sums (Acc) + row counts (int)
  return static_cast<size_t>(SH) * SW * (sizeof(double) + 1) + static_cast<size_t>(SH) * kBTW * (sizeof(Acc) + 4) + 64;
}

// Element value for the accumulator: exact for every supported dtype.
template <class Acc>
__device__ __forceinline__ double box_load(const void* base, int dtype, int64_t idx, const NodataSpec& nd,
                                           bool& valid) {
  if (dtype == VSR_F64) {
    const double v = __ldg(static_cast<const double*>(base) + idx);
    valid = !(nd.kind == VSR_NODATA_VALUE ? v == nd.dv : false) && v == v;
    return v;
  }
  if (dtype == VSR_I32) {
    const int32_t v = __ldg(static_cast<const int32_t*>(base) + idx);
    valid = !(nd.kind == VSR_NODATA_VALUE && v == nd.iv);
    return static_cast<double>(v);
  }
  const float v = load_elem(base, dtype, idx, nd, valid);
  valid = valid && (v == v);  // NaN never counts (reference CPU mean excludes it)
  return static_cast<double>(v);
}

template <class Acc>
__global__ void __launch_bounds__(256) box_mean(const BoxArgs a) {
  extern __shared__ __align__(16) unsigned char braw[];
  const int SH = kBTH + 2 * a.ry, SW = kBTW + 2 * a.rx;
  double* sv = reinterpret_cast<double*>(braw);                 // SH x SW values
  Acc* rs = reinterpret_cast<Acc*>(sv + SH * SW);               // SH x kBTW row sums
  int32_t* rc = reinterpret_cast<int32_t*>(rs + SH * kBTW);     // SH x kBTW row counts
  uint8_t* sd = reinterpret_cast<uint8_t*>(rc + SH * kBTW);     // SH x SW valid
  const int tid = threadIdx.x;
  const int64_t x0 = static_cast<int64_t>(blockIdx.x) * kBTW;
  const int64_t y0 = static_cast<int64_t>(blockIdx.y) * kBTH;
  const void* src = band_src(a.src, a.dtype, a.band_stride);
  void* dst = band_dst(a.dst, a.out_dtype, a.out_band_stride);

  for (int i = tid; i < SH * SW; i += 256) {
    const int rr = i / SW, c = i - rr * SW;
    const int64_t gy = y0 + rr - a.ry, gx = x0 + c - a.rx;
    double v = 0.0;
    bool ok = false;
    if (gy >= 0 && gy < a.H && gx >= 0 && gx < a.W) v = box_load<Acc>(src, a.dtype, gy * a.pitch + gx, a.nd, ok);
    sv[i] = ok ? v : 0.0;
    sd[i] = ok ? 1 : 0;
  }
  __syncthreads();
  const int wx = 2 * a.rx + 1, wy = 2 * a.ry + 1;
  for (int i = tid; i < SH * kBTW; i += 256) {
    const int rr = i / kBTW, c = i - rr * kBTW;
    Acc s;
    s.zero();
    int n = 0;
    const double* row = sv + rr * SW + c;
    const uint8_t* drow = sd + rr * SW + c;
    for (int t = 0; t < wx; ++t) {
      s.add(static_cast<decltype(Acc::s)>(row[t]));
      n += drow[t];
    }
    rs[i] = s;
    rc[i] = n;
  }
  __syncthreads();
  for (int i = tid; i < kBTH * kBTW; i += 256) {
    const int q = i / kBTW, c = i - q * kBTW;
    const int64_t y = y0 + q, x = x0 + c;
    if (y >= a.H || x >= a.W) continue;
    Acc s;
    s.zero();
    int n = 0;
    for (int t = 0; t < wy; ++t) {
      s.add(rs[(q + t) * kBTW + c]);
      n += rc[(q + t) * kBTW + c];
    }
    // The reference masks only nodata centres (algebra.py:3099-3100); a NaN
    // centre that is not the nodata value still gets its window mean.
    bool centre_ok = true;
    if (a.nd.kind != VSR_NODATA_NONE) (void)load_elem(src, a.dtype, y * a.pitch + x, a.nd, centre_ok);
    const bool centre_nodata = !centre_ok;
    const double out = (centre_nodata || n == 0) ? a.nd_out : s.value() / static_cast<double>(n);
    store_out(dst, a.out_dtype, y * a.out_pitch + x, out);
  }
}

template <class Acc>
int launch_box(const BoxArgs& a, cudaStream_t st, int bands = 1) {
  const size_t smem = box_smem_bytes<Acc>(a.ry, a.rx);
  if (smem > 227 * 1024) return fail(VSR_ERR_UNSUPPORTED, "focal mean radius (%d, %d) too large", a.ry, a.rx);
  auto kern = box_mean<Acc>;
  VSR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  dim3 grid(static_cast<unsigned>((a.W + kBTW - 1) / kBTW), static_cast<unsigned>((a.H + kBTH - 1) / kBTH), bands);
  if (grid.y > 65535u) return fail(VSR_ERR_UNSUPPORTED, "raster too tall for the focal mean grid");
  kern<<<grid, 256, smem, st>>>(a);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}

// -------------------------------------------------------- box_mean_fast --
// Focal mean for <= 16-bit integer (exact int32 sums) and float32 (TwoSum
// float pairs) rasters.  A 128 x 32 output tile is staged as values (0 where
// invalid) plus a byte count plane; the row pass slides a (2rx+1)-wide
// window along runs of 16 columns (add the entering value, subtract the
// leaving one: exact for integers, compensated for floats), the column pass
// slides a (2ry+1)-tall window down 16-row runs.  mean = sum / count.
constexpr int kFTW = 128, kFTH = 32, kFRun = 16;

template <bool FLOAT>
struct FastSum;
template <>
struct FastSum<false> {
  int32_t s;
  __device__ void zero() { s = 0; }
  // integer rasters are staged as int32 bit patterns in the value plane
  __device__ void add(float v) { s += __float_as_int(v); }
  __device__ void sub(float v) { s -= __float_as_int(v); }
  __device__ void add(const FastSum& o) { s += o.s; }
  __device__ void sub(const FastSum& o) { s -= o.s; }
  __device__ double value() const { return static_cast<double>(s); }
};
template <>
struct FastSum<true> {
  float s, c;
  __device__ void zero() { s = 0.0f; c = 0.0f; }
  __device__ void two_sum(float v) {
    const float t = s + v;
    const float bp = t - s;
    c += (s - (t - bp)) + (v - bp);
    s = t;
  }
  __device__ void add(float v) { two_sum(v); }
  __device__ void sub(float v) { two_sum(-v); }
  __device__ void add(const FastSum& o) { two_sum(o.s); c += o.c; }
  __device__ void sub(const FastSum& o) { two_sum(-o.s); c -= o.c; }
  __device__ double value() const { return static_cast<double>(s) + static_cast<double>(c); }
};

constexpr int kFRS = kFTW + 1;  // odd row stride of the row-sum planes (no bank conflicts)
constexpr int kMaxFastWindow = 1023;  // windows up to 1023 taps use the fast kernel

template <bool FLOAT>
inline size_t box_fast_smem(int ry, int rx) {
  const int SH = kFTH + 2 * ry, SWp = (kFTW + 2 * rx) | 1;
  return static_cast<size_t>(SH) * SWp * 5 + static_cast<size_t>(SH) * kFRS * (sizeof(FastSum<FLOAT>) + 4) + 64;
}

template <bool FLOAT>
__global__ void __launch_bounds__(256) box_mean_fast(const BoxArgs a) {
  using Sum = FastSum<FLOAT>;
  extern __shared__ __align__(16) unsigned char fraw[];
  const int SH = kFTH + 2 * a.ry, SW = kFTW + 2 * a.rx, SWp = SW | 1;  // odd stride: rows in distinct banks
  const int wx = 2 * a.rx + 1, wy = 2 * a.ry + 1;
  Sum* rs = reinterpret_cast<Sum*>(fraw);                      // SH x kFRS row sums (8-byte aligned first)
  float* sv = reinterpret_cast<float*>(rs + SH * kFRS);        // SH x SWp values (0 where invalid)
  int32_t* rc = reinterpret_cast<int32_t*>(sv + SH * SWp);     // SH x kFRS row counts
  uint8_t* sd = reinterpret_cast<uint8_t*>(rc + SH * kFRS);    // SH x SWp valid
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t x0 = static_cast<int64_t>(blockIdx.x) * kFTW;
  const int64_t y0 = static_cast<int64_t>(blockIdx.y) * kFTH;
  const void* src = band_src(a.src, a.dtype, a.band_stride);
  void* dst = band_dst(a.dst, a.out_dtype, a.out_band_stride);
  // 1/n for every possible count (float32 outputs)
  __shared__ float inv_n[kMaxFastWindow + 1];
  for (int i = tid; i <= wx * wy && i <= kMaxFastWindow; i += 256) inv_n[i] = i ? 1.0f / static_cast<float>(i) : 0.0f;

  for (int rr = warp; rr < SH; rr += 8) {
    const int64_t gy = y0 + rr - a.ry;
    const bool row_in = gy >= 0 && gy < a.H;
    for (int c = lane; c < SW; c += 32) {
      const int64_t gx = x0 + c - a.rx;
      float v = 0.0f;
      bool ok = false;
      if (row_in && gx >= 0 && gx < a.W) {
        v = load_elem(src, a.dtype, gy * a.pitch + gx, a.nd, ok);
        ok = ok && (v == v);  // NaN never counts (the CPU reference excludes it)
      }
      // float rasters: the value; integer rasters: its int32 bit pattern
      sv[rr * SWp + c] = FLOAT ? (ok ? v : 0.0f) : __int_as_float(ok ? static_cast<int32_t>(v) : 0);
      sd[rr * SWp + c] = ok ? 1 : 0;
    }
  }
  __syncthreads();
  // row pass: units (row, 16-column run); consecutive lanes take consecutive rows
  const int runs_x = kFTW / kFRun;
  for (int u = tid; u < SH * runs_x; u += 256) {
    const int rr = u % SH, c0 = (u / SH) * kFRun;
    const float* row = sv + rr * SWp + c0;
    const uint8_t* drow = sd + rr * SWp + c0;
    Sum sum;
    sum.zero();
    int n = 0;
    for (int t = 0; t < wx; ++t) {
      sum.add(row[t]);
      n += drow[t];
    }
    rs[rr * kFRS + c0] = sum;
    rc[rr * kFRS + c0] = n;
    for (int j = 1; j < kFRun; ++j) {
      sum.add(row[j + wx - 1]);
      sum.sub(row[j - 1]);
      n += static_cast<int>(drow[j + wx - 1]) - static_cast<int>(drow[j - 1]);
      rs[rr * kFRS + c0 + j] = sum;
      rc[rr * kFRS + c0 + j] = n;
    }
  }
  __syncthreads();
  // column pass: one column, a run of 16 rows per thread
  const int c = tid & (kFTW - 1);
  const int64_t x = x0 + c;
  for (int q0 = (tid >> 7) * kFRun; q0 < kFTH; q0 += 2 * kFRun) {
    Sum sum;
    sum.zero();
    int n = 0;
    for (int t = 0; t < wy; ++t) {
      sum.add(rs[(q0 + t) * kFRS + c]);
      n += rc[(q0 + t) * kFRS + c];
    }
    for (int j = 0; j < kFRun; ++j) {
      if (j > 0) {
        sum.add(rs[(q0 + j + wy - 1) * kFRS + c]);
        sum.sub(rs[(q0 + j - 1) * kFRS + c]);
        n += rc[(q0 + j + wy - 1) * kFRS + c] - rc[(q0 + j - 1) * kFRS + c];
      }
      const int64_t y = y0 + q0 + j;
      if (y >= a.H || x >= a.W) continue;
      // nodata centre: the reference masks only nodata (not NaN) centres
      bool centre_ok = true;
      if (a.nd.kind != VSR_NODATA_NONE && !sd[(q0 + j + a.ry) * SWp + c + a.rx]) {
        bool ok;
        (void)load_elem(src, a.dtype, y * a.pitch + x, a.nd, ok);
        centre_ok = ok;
      }
      double out;
      if (!centre_ok || n == 0) {
        out = a.nd_out;
      } else if (a.out_dtype == VSR_F64) {
        out = sum.value() / static_cast<double>(n);
      } else {
        // float32 output: one multiply by the count's reciprocal (<= 1 ulp)
        out = FLOAT ? static_cast<double>(static_cast<float>(sum.value()) * inv_n[n])
                    : static_cast<double>(static_cast<float>(sum.s) * inv_n[n]);
      }
      store_out(dst, a.out_dtype, y * a.out_pitch + x, out);
    }
  }
}

template <bool FLOAT>
int launch_box_fast(const BoxArgs& a, cudaStream_t st, int bands) {
  const size_t smem = box_fast_smem<FLOAT>(a.ry, a.rx);
  if (smem > 227 * 1024) return fail(VSR_ERR_UNSUPPORTED, "focal mean radius (%d, %d) too large", a.ry, a.rx);
  auto kern = box_mean_fast<FLOAT>;
  VSR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  dim3 grid(static_cast<unsigned>((a.W + kFTW - 1) / kFTW), static_cast<unsigned>((a.H + kFTH - 1) / kFTH), bands);
  if (grid.y > 65535u) return fail(VSR_ERR_UNSUPPORTED, "raster too tall for the focal mean grid");
  kern<<<grid, 256, smem, st>>>(a);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}

// ------------------------------------------------------- box_slide_int --
// Focal mean of 8/16-bit integer rasters with a square (2R+1)^2 window,
// R <= 7, rows of any alignment (box_warp_int, below, takes R <= 4 with rows
// aligned to 4 elements, e.g. the 12 x 10980^2 uint16 stack's 7 x 7 mean).
//
// Each tap is packed into one 32-bit word, value (offset to be
// non-negative) in the low bits and a count bit above them:
//   p = valid ? (v + off) | 1 << S : 0,
// so one integer add sums value and count together and every sum is exact.
// A block owns 128 columns (one per thread) and a strip of 256 rows.  Input
// rows stream through a two-slot shared-memory ring (16 rows a slot, loaded
// into registers one slot ahead); each thread forms the horizontal window
// sum of its column per input row and slides the vertical window with a
// register shift register (add the entering row, subtract the leaving one).
// mean = (sum - off count) / count, one correctly rounded division.
template <int R>
struct SlidePack {
  static constexpr int kTaps = (2 * R + 1) * (2 * R + 1);
  // value-sum bits: the smallest S with taps * 65535 < 2^S
  static constexpr int kShift = kTaps * 65535ll < (1ll << 22) ? 22 : (kTaps * 65535ll < (1ll << 23) ? 23 : 24);
  static_assert(kTaps * 65535ll < (1ll << kShift), "value sum overflows the low field");
  static_assert(kTaps < (1 << (32 - kShift)), "count overflows the high field");
};

constexpr int kSlTW = 128;               // output columns per block
constexpr int kSlHalo = 8;               // staged columns each side (R <= 7, even for pair loads)
constexpr int kSlSW = kSlTW + 2 * kSlHalo;  // 144 staged elements per row
constexpr int kSlCH = 16;                // rows per ring slot
constexpr int kSlStrip = 256;            // output rows per block
constexpr int kSlWords = kSlCH * kSlSW / 2;  // element pairs per slot
constexpr int kSlPer = (kSlWords + kSlTW - 1) / kSlTW;  // pairs per thread per slot

template <int R, typename T, bool PAIR>
__global__ void __launch_bounds__(kSlTW) box_slide_int(const BoxArgs a) {
  using Pk = SlidePack<R>;
  constexpr int OFF = std::is_signed<T>::value ? 32768 : 0;
  constexpr uint32_t kOne = 1u << Pk::kShift, kLow = kOne - 1u;
  __shared__ uint32_t ring[2][kSlCH][kSlSW];
  const int c = threadIdx.x;
  const int64_t x0 = static_cast<int64_t>(blockIdx.x) * kSlTW;
  const int64_t ys = static_cast<int64_t>(blockIdx.y) * kSlStrip;
  const T* src = static_cast<const T*>(band_src(a.src, a.dtype, a.band_stride));
  void* dst = band_dst(a.dst, a.out_dtype, a.out_band_stride);
  const int64_t nout = a.H - ys < kSlStrip ? a.H - ys : static_cast<int64_t>(kSlStrip);
  const int nin = static_cast<int>(nout) + 2 * R;  // input rows ys - R .. ys + nout + R - 1
  const int nchunks = (nin + kSlCH - 1) / kSlCH;
  const bool has_nd = a.nd.kind == VSR_NODATA_VALUE;
  const int64_t ndv = a.nd.iv;

  auto pack = [&](uint32_t e, bool inb) -> uint32_t {
    const T v = static_cast<T>(e);
    const bool ok = inb && !(has_nd && static_cast<int64_t>(v) == ndv);
    return ok ? ((static_cast<uint32_t>(static_cast<int>(v) + OFF)) | kOne) : 0u;
  };
  // Element pairs of a slot: pair w -> staged row w / (kSlSW / 2), columns
  // 2 (w % (kSlSW / 2)) and +1.  A thread's pairs sit at the same columns
  // in every chunk: their offsets and column bounds are fixed up front.
  // Loads go to raw registers one chunk ahead; packing happens at the store
  // (a load's value is not needed until then).
  int64_t coff[kSlPer];
  int prow[kSlPer];
  uint32_t colin = 0u;  // 2 bits per pair: element in [0, W)
#pragma unroll
  for (int i = 0; i < kSlPer; ++i) {
    const int w = c + kSlTW * i;
    prow[i] = w < kSlWords ? w / (kSlSW / 2) : -1;
    const int wc = w - (w / (kSlSW / 2)) * (kSlSW / 2);
    const int64_t gx = x0 - kSlHalo + 2 * wc;
    coff[i] = gx;
    colin |= (static_cast<uint32_t>(gx >= 0 && gx < a.W) | (static_cast<uint32_t>(gx + 1 >= 0 && gx + 1 < a.W) << 1))
             << (2 * i);
  }
  uint32_t raw[kSlPer];
  uint32_t inb = 0u;  // 2 bits per pair: element loaded (inside the raster)
  auto load_chunk = [&](int k) {
    inb = 0u;
    const int64_t gy0 = ys - R + static_cast<int64_t>(k) * kSlCH;
#pragma unroll
    for (int i = 0; i < kSlPer; ++i) {
      raw[i] = 0u;
      if (prow[i] < 0) continue;
      const int64_t gy = gy0 + prow[i];
      if (gy < 0 || gy >= a.H) continue;
      const uint32_t cb = (colin >> (2 * i)) & 3u;
      const T* rp = src + gy * a.pitch + coff[i];
      if (PAIR && cb == 3u) {
        raw[i] = __ldg(reinterpret_cast<const uint32_t*>(rp));
      } else {
        const uint32_t e0 = (cb & 1u) ? static_cast<uint32_t>(static_cast<std::make_unsigned_t<T>>(__ldg(rp))) : 0u;
        const uint32_t e1 = (cb & 2u) ? static_cast<uint32_t>(static_cast<std::make_unsigned_t<T>>(__ldg(rp + 1))) : 0u;
        raw[i] = e0 | (e1 << 16);
      }
      inb |= cb << (2 * i);
    }
  };
  auto store_chunk = [&](int slot) {
#pragma unroll
    for (int i = 0; i < kSlPer; ++i) {
      if (prow[i] < 0) continue;
      const int wc = (c + kSlTW * i) - prow[i] * (kSlSW / 2);
      const uint32_t b = (inb >> (2 * i)) & 3u;
      *reinterpret_cast<uint2*>(&ring[slot][prow[i]][2 * wc]) =
          make_uint2(pack(raw[i] & 0xFFFFu, b & 1u), pack(raw[i] >> 16, (b >> 1) & 1u));
    }
  };

  __shared__ float inv_n[Pk::kTaps + 1];  // correctly rounded 1/n for the float32 quotient
  for (int i = c; i <= Pk::kTaps; i += kSlTW) inv_n[i] = i ? __frcp_rn(static_cast<float>(i)) : 0.0f;
  load_chunk(0);
  store_chunk(0);
  __syncthreads();
  if (nchunks > 1) load_chunk(1);
  uint32_t h[2 * R + 1];
#pragma unroll
  for (int j = 0; j <= 2 * R; ++j) h[j] = 0u;
  uint32_t V = 0u;
  const int64_t x = x0 + c;
  const bool col_in = x < a.W;
  const bool f64 = a.out_dtype == VSR_F64;
  // input row i (strip index); its output row is i - 2R (centre row i - R)
  auto row_step = [&](int slot, int r, int i) {
    const uint32_t* row = &ring[slot][r][c + kSlHalo - R];
    uint32_t hn = 0u;
#pragma unroll
    for (int t = 0; t <= 2 * R; ++t) hn += row[t];
    V += hn - h[0];
#pragma unroll
    for (int j = 0; j < 2 * R; ++j) h[j] = h[j + 1];
    h[2 * R] = hn;
    const int jc = i - R;
    const uint32_t pc = ring[(jc >> 4) & 1][jc & (kSlCH - 1)][c + kSlHalo];
    const int cnt = static_cast<int>(V >> Pk::kShift);
    const int sum = static_cast<int>(V & kLow) - OFF * cnt;
    if (i >= 2 * R && col_in) {
      const int64_t o = (ys + (i - 2 * R)) * a.out_pitch + x;
      const bool nd = pc == 0u || cnt == 0;
      if (f64) {
        static_cast<double*>(dst)[o] = nd ? a.nd_out : static_cast<double>(sum) / static_cast<double>(cnt);
      } else {
        // RN(sum / cnt): quotient with the exact reciprocal, one FMA correction
        // (Markstein); sum and cnt are exact in float32
        const float fs = static_cast<float>(sum), fn = static_cast<float>(cnt), rn = inv_n[cnt];
        const float q0 = fs * rn;
        const float q = fmaf(fmaf(-q0, fn, fs), rn, q0);
        static_cast<float*>(dst)[o] = nd ? static_cast<float>(a.nd_out) : q;
      }
    }
  };
  for (int k = 0; k < nchunks; ++k) {
    const int slot = k & 1;
    if ((k + 1) * kSlCH <= nin) {
#pragma unroll
      for (int r = 0; r < kSlCH; ++r) row_step(slot, r, k * kSlCH + r);
    } else {
      for (int r = 0; k * kSlCH + r < nin; ++r) row_step(slot, r, k * kSlCH + r);
    }
    __syncthreads();  // every read of this chunk and of the last rows of the previous one is done
    if (k + 1 < nchunks) {
      store_chunk((k + 1) & 1);
      __syncthreads();
      if (k + 2 < nchunks) load_chunk(k + 2);
    }
  }
}

// ------------------------------------------------------- box_warp_int --
// The same focal mean (8/16-bit integers, square (2R+1)^2 window) for
// R <= 4 when rows are aligned to 4 elements, held in registers.
//
// One warp owns a 128-column strip, 4 columns per lane; lanes 0 and 31 only
// supply their columns to their neighbours, so a warp writes the 120 columns
// of lanes 1-30 and consecutive warps overlap by 8 columns.  Per input row
// each lane loads its 4 elements (one vector load, prefetched 2R+1 rows
// ahead), packs them as value | count words (the packing of box_slide_int),
// takes R words from each neighbour by shuffles and forms its 4 horizontal
// window sums by sliding; the vertical window slides over a register ring of
// the last 2R+1 horizontal sums, with the row loop unrolled by 2R+1 so that
// every ring index is a compile-time constant.  The float32 quotient is the
// same correctly rounded division as box_slide_int's.
constexpr int kBwLanes = 30;            // output lanes per warp
constexpr int kBwCols = 4 * kBwLanes;   // output columns per warp
constexpr int kBwWarps = 4;             // warps per block, side by side
constexpr int kBwStrip = 256;           // output rows per warp

template <typename T>
struct Vec4Of {  // 4 elements in one load
  using type = uint2;
};
template <>
struct Vec4Of<uint8_t> {
  using type = uint32_t;
};

template <int R, typename T, bool VOUT, bool F64>
__global__ void __launch_bounds__(32 * kBwWarps) box_warp_int(const BoxArgs a) {
  static_assert(R >= 1 && R <= 4, "the neighbour exchange covers radii up to 4");
  using Pk = SlidePack<R>;
  using V4 = typename Vec4Of<T>::type;
  constexpr int P = 2 * R + 1;
  constexpr bool kByte = sizeof(T) == 1;
  constexpr int OFF = std::is_signed<T>::value ? 32768 : 0;
  constexpr uint32_t kOne = 1u << Pk::kShift, kLow = kOne - 1u;
  static_assert(Pk::kShift >= 16 && Pk::kShift <= 23, "the count bit sits in byte 2; value sums stay below 2^23");
  // int16 values + 32768 = their bits with bit 15 flipped
  constexpr uint32_t kFlip = OFF ? 0x80008000u : 0u;
  __shared__ float2 tab[Pk::kTaps + 1];  // (RN(1/n), -n)
  for (int i = threadIdx.x; i <= Pk::kTaps; i += blockDim.x)
    tab[i] = make_float2(i ? __frcp_rn(static_cast<float>(i)) : 0.0f, -static_cast<float>(i));
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t xw = (static_cast<int64_t>(blockIdx.x) * kBwWarps + (threadIdx.x >> 5)) * kBwCols;
  if (xw >= a.W) return;  // the whole warp: no block-wide barrier follows
  const int64_t xs = xw - 4 + 4 * lane;  // this lane's first column (a multiple of 4)
  const int64_t ys = static_cast<int64_t>(blockIdx.y) * kBwStrip;
  const T* src = static_cast<const T*>(band_src(a.src, a.dtype, a.band_stride));
  void* dst = band_dst(a.dst, a.out_dtype, a.out_band_stride);
  const int nout = static_cast<int>(a.H - ys < kBwStrip ? a.H - ys : kBwStrip);
  const int nin = nout + 2 * R;  // input rows ys - R .. ys + nout + R - 1
  const bool has_nd = a.nd.kind == VSR_NODATA_VALUE;
  // the nodata value's bit pattern in every element slot of a word
  const uint32_t ndp = static_cast<uint32_t>(a.nd.iv) & (kByte ? 0xFFu : 0xFFFFu);
  const uint32_t nd_word = kByte ? ndp * 0x01010101u : ndp * 0x00010001u;
  // elements of the group inside [0, W), as byte (8-bit) or half-word masks
  // of the two words; one vector load per group inside the raster, element
  // loads for the group that straddles column W
  uint32_t cmx = 0u, cmy = 0u;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const uint32_t in = (xs + e >= 0 && xs + e < a.W) ? 1u : 0u;
    if (kByte) cmx |= (in * 0xFFu) << (8 * e);
    else if (e < 2) cmx |= (in * 0xFFFFu) << (16 * e);
    else cmy |= (in * 0xFFFFu) << (16 * (e - 2));
  }
  const bool ld = xs >= 0 && xs < a.W, whole = xs >= 0 && xs + 4 <= a.W;
  const bool out_lane = lane >= 1 && lane <= kBwLanes;

  // input row i is raster row ys - R + i; its pointer steps by the pitch
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
        if constexpr (kByte) v = e[0] | (e[1] << 8) | (e[2] << 16) | (e[3] << 24);
        else v = make_uint2(e[0] | (e[1] << 16), e[2] | (e[3] << 16));
      }
    }
    return v;
  };
  V4 pre[P];
#pragma unroll
  for (int u = 0; u < P; ++u) pre[u] = load(u, rp + u * a.pitch);
  const T* lp = rp + P * a.pitch;  // the row P ahead
  uint32_t hs[P][4];  // horizontal sums of the last P rows (ring slot = row % P)
  uint32_t vm[P];     // their validity, one byte per element (0xFF valid)
#pragma unroll
  for (int u = 0; u < P; ++u) {
    vm[u] = 0u;
#pragma unroll
    for (int c = 0; c < 4; ++c) hs[u][c] = 0u;
  }
  uint32_t V[4] = {0u, 0u, 0u, 0u};
  const float ndf = static_cast<float>(a.nd_out);
  int64_t orow = ys * a.out_pitch + xs;  // output row i - 2R
  // correctly rounded sum / count for two columns: q0 = fs / n by the
  // reciprocal, one FMA residual correction (exact integers in float32)
  auto quot2 = [&](uint32_t va, uint32_t vb) -> float2 {
    const float2 ta = tab[va >> Pk::kShift], tb = tab[vb >> Pk::kShift];
    float2 fs = __fadd2_rn(make_float2(__uint_as_float(0x4B000000u | (va & kLow)), __uint_as_float(0x4B000000u | (vb & kLow))),
                           make_float2(-8388608.0f, -8388608.0f));
    const float2 rn = make_float2(ta.x, tb.x), nn = make_float2(ta.y, tb.y);
    if (OFF) fs = __ffma2_rn(make_float2(static_cast<float>(OFF), static_cast<float>(OFF)), nn, fs);
    const float2 q0 = __fmul2_rn(fs, rn);
    return __ffma2_rn(__ffma2_rn(q0, nn, fs), rn, q0);
  };
  for (int g0 = 0; g0 < nin; g0 += P) {
#pragma unroll
    for (int u = 0; u < P; ++u) {
      const int i = g0 + u;
      if (i >= nin) break;
      const V4 raw = pre[u];
      pre[u] = load(i + P, lp);
      lp += a.pitch;
      const uint32_t rowm = static_cast<uint64_t>(ys - R + i) < static_cast<uint64_t>(a.H) ? 0xFFFFFFFFu : 0u;
      // packed words: the element (plus the offset) in bits 0-15, the count
      // bit above, or 0 where invalid -- byte permutes of the raw words
      uint32_t w[12];  // left neighbour's 4 words, this lane's, the right neighbour's
      uint32_t m;      // validity, one byte per element
      if constexpr (kByte) {
        const uint32_t x = raw;
        uint32_t k = cmx & rowm;
        if (has_nd) k &= ~__vcmpeq4(x, nd_word);
        m = k;
        w[4] = __byte_perm(x, kOne, 0x7640) & __byte_perm(k, 0u, 0x0000);
        w[5] = __byte_perm(x, kOne, 0x7641) & __byte_perm(k, 0u, 0x1111);
        w[6] = __byte_perm(x, kOne, 0x7642) & __byte_perm(k, 0u, 0x2222);
        w[7] = __byte_perm(x, kOne, 0x7643) & __byte_perm(k, 0u, 0x3333);
      } else {
        const uint32_t x = raw.x, y = raw.y;  // (v0 | v1 << 16), (v2 | v3 << 16)
        uint32_t kx = cmx & rowm, ky = cmy & rowm;
        if (has_nd) {
          kx &= ~__vcmpeq2(x, nd_word);
          ky &= ~__vcmpeq2(y, nd_word);
        }
        m = __byte_perm(kx, ky, 0x6420);
        w[4] = __byte_perm(x ^ kFlip, kOne, 0x7610) & __byte_perm(kx, 0u, 0x1010);
        w[5] = __byte_perm(x ^ kFlip, kOne, 0x7632) & __byte_perm(kx, 0u, 0x3232);
        w[6] = __byte_perm(y ^ kFlip, kOne, 0x7610) & __byte_perm(ky, 0u, 0x1010);
        w[7] = __byte_perm(y ^ kFlip, kOne, 0x7632) & __byte_perm(ky, 0u, 0x3232);
      }
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        w[e] = __shfl_up_sync(0xffffffffu, w[4 + e], 1);
        w[8 + e] = __shfl_down_sync(0xffffffffu, w[4 + e], 1);
      }
      uint32_t h = 0u;
#pragma unroll
      for (int j = 4 - R; j <= 4 + R; ++j) h += w[j];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        if (c > 0) h += w[4 + c + R] - w[3 + c - R];
        V[c] += h - hs[u][c];
        hs[u][c] = h;
      }
      vm[u] = m;
      if (i >= 2 * R) {
        if (out_lane) {
          const uint32_t cm = vm[(u + P - R) % P];  // the centre row i - R
          if constexpr (F64) {
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              const int cnt = static_cast<int>(V[c] >> Pk::kShift);
              const int sum = static_cast<int>(V[c] & kLow) - OFF * cnt;
              if (xs + c < a.W)
                static_cast<double*>(dst)[orow + c] =
                    ((cm >> (8 * c)) & 1u) ? static_cast<double>(sum) / static_cast<double>(cnt) : a.nd_out;
            }
          } else {
            const float2 q01 = quot2(V[0], V[1]), q23 = quot2(V[2], V[3]);
            const float q[4] = {(cm & 1u) ? q01.x : ndf, ((cm >> 8) & 1u) ? q01.y : ndf,
                                ((cm >> 16) & 1u) ? q23.x : ndf, ((cm >> 24) & 1u) ? q23.y : ndf};
            float* op = static_cast<float*>(dst) + orow;
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

template <int R, typename T>
int launch_warp_t(const BoxArgs& a, cudaStream_t st, int bands) {
  dim3 grid(static_cast<unsigned>((a.W + kBwWarps * kBwCols - 1) / (kBwWarps * kBwCols)),
            static_cast<unsigned>((a.H + kBwStrip - 1) / kBwStrip), bands);
  if (grid.y > 65535u) return fail(VSR_ERR_UNSUPPORTED, "raster too tall for the focal mean grid");
  const bool vout = a.out_dtype == VSR_F32 && aligned(a.dst, 16) && a.out_pitch % 4 == 0 &&
                    (bands == 1 || a.out_band_stride % 4 == 0);
  if (a.out_dtype == VSR_F64) box_warp_int<R, T, false, true><<<grid, 32 * kBwWarps, 0, st>>>(a);
  else if (vout) box_warp_int<R, T, true, false><<<grid, 32 * kBwWarps, 0, st>>>(a);
  else box_warp_int<R, T, false, false><<<grid, 32 * kBwWarps, 0, st>>>(a);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}

template <int R, typename T>
int launch_slide_t(const BoxArgs& a, cudaStream_t st, int bands) {
  if constexpr (R <= 4) {  // rows aligned to 4 elements: the register-resident form
    if (aligned(a.src, 4 * sizeof(T)) && a.pitch % 4 == 0 && (bands == 1 || a.band_stride % 4 == 0))
      return launch_warp_t<R, T>(a, st, bands);
  }
  const bool pair = sizeof(T) == 2 && aligned(a.src, 4) && a.pitch % 2 == 0 && a.band_stride % 2 == 0;
  dim3 grid(static_cast<unsigned>((a.W + kSlTW - 1) / kSlTW), static_cast<unsigned>((a.H + kSlStrip - 1) / kSlStrip),
            bands);
  if (grid.y > 65535u) return fail(VSR_ERR_UNSUPPORTED, "raster too tall for the focal mean grid");
  if (pair) box_slide_int<R, T, true><<<grid, kSlTW, 0, st>>>(a);
  else box_slide_int<R, T, false><<<grid, kSlTW, 0, st>>>(a);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}

template <int R>
int launch_slide_r(const BoxArgs& a, cudaStream_t st, int bands) {
  switch (a.dtype) {
    case VSR_U8: return launch_slide_t<R, uint8_t>(a, st, bands);
    case VSR_I16: return launch_slide_t<R, int16_t>(a, st, bands);
    default: return launch_slide_t<R, uint16_t>(a, st, bands);
  }
}

// Square windows of radius 1..7 on 8/16-bit integer rasters; 0 otherwise.
int launch_slide(const BoxArgs& a, cudaStream_t st, int bands) {
  if (a.ry != a.rx) return -1;
  switch (a.ry) {
    case 1: return launch_slide_r<1>(a, st, bands);
    case 2: return launch_slide_r<2>(a, st, bands);
    case 3: return launch_slide_r<3>(a, st, bands);
    case 4: return launch_slide_r<4>(a, st, bands);
    case 5: return launch_slide_r<5>(a, st, bands);
    case 6: return launch_slide_r<6>(a, st, bands);
    case 7: return launch_slide_r<7>(a, st, bands);
    default: return -1;
  }
}

// ------------------------------------------------------- shared checks --
int check_raster(const void* src, int dtype, int64_t H, int64_t W, int64_t pitch, const void* dst,
                 int out_dtype, int64_t out_pitch) {
  if (H < 0 || W < 0) return fail(VSR_ERR_INVALID_ARG, "negative raster size");
  if (H == 0 || W == 0) return VSR_OK;
  if (!src || !dst) return fail(VSR_ERR_INVALID_ARG, "src/dst must not be NULL");
  if (dtype_size(dtype) == 0) return fail(VSR_ERR_INVALID_ARG, "unsupported dtype %d", dtype);
  if (out_dtype != VSR_F32 && out_dtype != VSR_F64) return fail(VSR_ERR_INVALID_ARG, "out_dtype must be VSR_F32 or VSR_F64");
  if (pitch < W || out_pitch < W) return fail(VSR_ERR_INVALID_ARG, "pitch smaller than width");
  if (!aligned(src, dtype_size(dtype)) || !aligned(dst, out_dtype == VSR_F64 ? 8 : 4))
    return fail(VSR_ERR_INVALID_ARG, "src/dst not aligned to their element size");
  return VSR_OK;
}

}  // namespace

// Workspace layout for the plain FP32 convolution:
//   [0, 8 kh kw)                  float64 weights (copied from the host)
//   [256-aligned) kh x kw4 float  float32 weight rows
//   [+256-aligned) 1 float        total weight
size_t conv_ws_plain(int kh, int kw) {
  const size_t a = (static_cast<size_t>(kh) * kw * 8 + 255) & ~size_t(255);
  const size_t b = (static_cast<size_t>(kh) * ((kw + 3) & ~3) * 4 + 255) & ~size_t(255);
  return a + b + 256;
}

}  // namespace vsr

using namespace vsr;

namespace vsr {
size_t conv_tc_workspace(int kh, int kw);  // conv_tc.cu
int conv_tc_supported(int kh, int kw);
int run_conv_tc(const void* src, int dtype, int bands, int64_t band_stride, int64_t H, int64_t W, int64_t pitch,
                const double* weights_host, int kh, int kw, double nodata, int nodata_kind, void* dst, int out_dtype,
                int64_t out_band_stride, int64_t out_pitch, void* workspace, size_t ws_bytes, cudaStream_t st);
int gauss_tc_supported(int dtype, int k);  // gauss_tc.cu
size_t gauss_tc_workspace(int64_t H, int64_t W, int dtype, int k);
size_t gauss_tc_workspace_bands(int64_t H, int64_t W, int dtype, int k, int bands);
int run_gauss_tc(const void* src, int dtype, int bands, int64_t band_stride, int64_t H, int64_t W, int64_t pitch,
                 double sigma, int k, double nodata, int nodata_kind, void* dst, int out_dtype,
                 int64_t out_band_stride, int64_t out_pitch, void* workspace, size_t ws_bytes, cudaStream_t st);
}  // namespace vsr

extern "C" size_t vsr_convolve_workspace_size(int kh, int kw, int precision) {
  if (kh <= 0 || kw <= 0) return 0;
  size_t n = conv_ws_plain(kh, kw);
  if (precision != VSR_PREC_FP32 && conv_tc_supported(kh, kw)) n = std::max(n, conv_tc_workspace(kh, kw));
  return n;
}

extern "C" int vsr_convolve_bands(const void* src, int dtype, int bands, int64_t band_stride, int64_t height,
                                  int64_t width, int64_t pitch, const double* weights_host, int kh, int kw,
                                  double nodata, int nodata_kind, void* dst, int out_dtype, int64_t out_band_stride,
                                  int64_t out_pitch, int precision, void* workspace, size_t workspace_bytes,
                                  void* stream) {
  if (bands < 1 || bands > 65535) return fail(VSR_ERR_INVALID_ARG, "bands must be in [1, 65535]");
  int rc = check_raster(src, dtype, height, width, pitch, dst, out_dtype, out_pitch);
  if (rc || height == 0 || width == 0) return rc;
  if (bands > 1 && (band_stride < pitch * height || out_band_stride < out_pitch * height))
    return fail(VSR_ERR_INVALID_ARG, "band strides smaller than one band");
  if (!weights_host) return fail(VSR_ERR_INVALID_ARG, "weights_host is NULL");
  if (kh <= 0 || kw <= 0) return fail(VSR_ERR_INVALID_ARG, "kernel must be at least 1 x 1");
  if (precision < VSR_PREC_AUTO || precision > VSR_PREC_SPLIT) return fail(VSR_ERR_INVALID_ARG, "bad precision %d", precision);
  if (kh > kMaxDirectK || kw > kMaxDirectK)
    return fail(VSR_ERR_UNSUPPORTED, "kernel %dx%d larger than the supported %dx%d", kh, kw, kMaxDirectK, kMaxDirectK);
  // Tensor-core path: float32 rasters and kernels that fit its shared-memory
  // plan.  AUTO takes it for k >= 15 on both axes when the kernel is well
  // conditioned: split weights carry 16 mantissa bits, and a weight sum
  // that nearly cancels (sum |w| > 4 |sum w|) would amplify that rounding.
  const bool tc_ok = dtype == VSR_F32 && conv_tc_supported(kh, kw) && aligned(src, 4);
  if (precision == VSR_PREC_SPLIT && !tc_ok)
    return fail(VSR_ERR_UNSUPPORTED, "split-precision convolution needs a float32 raster and a kernel of at most 41x41");
  bool well_conditioned = false;
  if (precision == VSR_PREC_AUTO && tc_ok && kh >= 15 && kw >= 15) {
    double s = 0.0, sa = 0.0;
    for (int i = 0; i < kh * kw; ++i) {
      s += weights_host[i];
      sa += std::fabs(weights_host[i]);
    }
    well_conditioned = sa <= 4.0 * std::fabs(s);
  }
  if (precision == VSR_PREC_SPLIT || well_conditioned)
    return run_conv_tc(src, dtype, bands, band_stride, height, width, pitch, weights_host, kh, kw, nodata,
                       nodata_kind, dst, out_dtype, out_band_stride, out_pitch, workspace, workspace_bytes,
                       static_cast<cudaStream_t>(stream));
  const size_t need = conv_ws_plain(kh, kw);
  if (!workspace || workspace_bytes < need || !aligned(workspace, 256))
    return fail(VSR_ERR_WORKSPACE, "workspace must be 256-byte aligned and >= %zu bytes", need);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* ws = static_cast<char*>(workspace);
  double* w64 = reinterpret_cast<double*>(ws);
  float* w32 = reinterpret_cast<float*>(ws + ((static_cast<size_t>(kh) * kw * 8 + 255) & ~size_t(255)));
  float* wsum = reinterpret_cast<float*>(ws + need - 256);
  const int kw4 = (kw + 3) & ~3;
  VSR_CUDA_TRY(cudaMemcpyAsync(w64, weights_host, static_cast<size_t>(kh) * kw * 8, cudaMemcpyHostToDevice, st));
  prep_weights<<<1, 256, 0, st>>>(w64, kh, kw, kw4, w32, wsum);
  VSR_CUDA_TRY(cudaGetLastError());
  ConvArgs a{src, dtype, height, width, pitch, make_nodata(dtype, nodata, nodata_kind), w32, wsum, kh, kw, kw4,
             nodata, dst, out_dtype, out_pitch, bands > 1 ? band_stride : 0, bands > 1 ? out_band_stride : 0};
  return run_conv_direct(a, st, bands);
}

extern "C" int vsr_convolve(const void* src, int dtype, int64_t height, int64_t width, int64_t pitch,
                            const double* weights_host, int kh, int kw, double nodata, int nodata_kind,
                            void* dst, int out_dtype, int64_t out_pitch, int precision, void* workspace,
                            size_t workspace_bytes, void* stream) {
  return vsr_convolve_bands(src, dtype, 1, 0, height, width, pitch, weights_host, kh, kw, nodata, nodata_kind, dst,
                            out_dtype, 0, out_pitch, precision, workspace, workspace_bytes, stream);
}

// Gaussian workspace: g (k4 floats) | dense weights (k x k4 floats) | total.
static size_t gauss_ws(int k) {
  const int k4 = (k + 3) & ~3;
  const size_t a = (static_cast<size_t>(k4) * 4 + 255) & ~size_t(255);
  const size_t b = (static_cast<size_t>(k) * k4 * 4 + 255) & ~size_t(255);
  return a + b + 256;
}

static int gaussian_size(double sigma, int kernel_size) {
  int k = kernel_size > 0 ? kernel_size : static_cast<int>(2.0 * std::ceil(3.0 * sigma) + 1.0);
  if (k % 2 == 0) k += 1;
  return k;
}

extern "C" size_t vsr_gaussian_workspace_size(int kernel_size, int precision) {
  (void)precision;
  if (kernel_size <= 0) return 0;
  const int k = kernel_size % 2 == 0 ? kernel_size + 1 : kernel_size;
  return gauss_ws(k);
}

// VSR_PREC_AUTO takes the split-precision line passes where the separable FP32
// kernels would use the strip kernel (k > 33) on an 8/16-bit integer raster
// (exact BF16 hi/lo values) and the caller's workspace holds their planes.
static bool gauss_tc_auto(int dtype, int64_t height, int64_t width, int k, const void* workspace, size_t bytes) {
  return k > kMaxSepK && gauss_tc_supported(dtype, k) && workspace && aligned(workspace, 256) &&
         bytes >= gauss_tc_workspace(height, width, dtype, k);
}

extern "C" size_t vsr_gaussian_workspace_bytes(int64_t height, int64_t width, int dtype, double sigma,
                                               int kernel_size, int precision) {
  if (!(sigma > 0.0) || height < 0 || width < 0) return 0;
  const int k = gaussian_size(sigma, kernel_size);
  const bool tc = gauss_tc_supported(dtype, k) &&
                  (precision == VSR_PREC_SPLIT || (precision == VSR_PREC_AUTO && k > kMaxSepK));
  return tc ? std::max(gauss_ws(k), gauss_tc_workspace(height, width, dtype, k)) : gauss_ws(k);
}

extern "C" size_t vsr_gaussian_bands_workspace_bytes(int bands, int64_t height, int64_t width, int dtype,
                                                     double sigma, int kernel_size, int precision) {
  if (!(sigma > 0.0) || height < 0 || width < 0 || bands < 1) return 0;
  const int k = gaussian_size(sigma, kernel_size);
  const bool tc = gauss_tc_supported(dtype, k) &&
                  (precision == VSR_PREC_SPLIT || (precision == VSR_PREC_AUTO && k > kMaxSepK));
  return tc ? std::max(gauss_ws(k), gauss_tc_workspace_bands(height, width, dtype, k, bands)) : gauss_ws(k);
}

static int gaussian_impl(const void* src, int dtype, int bands, int64_t band_stride, int64_t height, int64_t width,
                         int64_t pitch, double sigma, int kernel_size, double nodata, int nodata_kind, void* dst,
                         int out_dtype, int64_t out_band_stride, int64_t out_pitch, int precision, void* workspace,
                         size_t workspace_bytes, void* stream) {
  if (!(sigma > 0.0)) return fail(VSR_ERR_INVALID_ARG, "sigma must be positive, got %g", sigma);
  if (bands < 1) return fail(VSR_ERR_INVALID_ARG, "bands must be >= 1");
  int rc = check_raster(src, dtype, height, width, pitch, dst, out_dtype, out_pitch);
  if (rc || height == 0 || width == 0) return rc;
  if (precision < VSR_PREC_AUTO || precision > VSR_PREC_SPLIT) return fail(VSR_ERR_INVALID_ARG, "bad precision %d", precision);
  const int k = gaussian_size(sigma, kernel_size);
  if (k > kMaxDirectK) return fail(VSR_ERR_UNSUPPORTED, "Gaussian kernel %d larger than %d", k, kMaxDirectK);
  if (precision == VSR_PREC_SPLIT || gauss_tc_auto(dtype, height, width, k, workspace, workspace_bytes))
    return run_gauss_tc(src, dtype, bands, band_stride, height, width, pitch, sigma, k, nodata, nodata_kind, dst,
                        out_dtype, out_band_stride, out_pitch, workspace, workspace_bytes,
                        static_cast<cudaStream_t>(stream));
  const size_t need = gauss_ws(k);
  if (!workspace || workspace_bytes < need || !aligned(workspace, 256))
    return fail(VSR_ERR_WORKSPACE, "workspace must be 256-byte aligned and >= %zu bytes", need);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int k4 = (k + 3) & ~3;
  char* ws = static_cast<char*>(workspace);
  float* g32 = reinterpret_cast<float*>(ws);
  prep_gaussian<<<1, 256, k * sizeof(double), st>>>(k, k4, sigma, g32, nullptr, nullptr);
  VSR_CUDA_TRY(cudaGetLastError());
  const NodataSpec nd = make_nodata(dtype, nodata, nodata_kind);
  SepArgs a{src, dtype, height, width, pitch, nd, g32, k, nodata, dst, out_dtype, out_pitch, band_stride,
            out_band_stride};
  if (k <= 8) return launch_sep<8>(a, st, bands);
  if (k <= 16) return launch_sep<16>(a, st, bands);
  if (k <= 33) return launch_sep<33>(a, st, bands);
  return launch_strip(a, st, bands);
}

extern "C" int vsr_gaussian(const void* src, int dtype, int64_t height, int64_t width, int64_t pitch, double sigma,
                            int kernel_size, double nodata, int nodata_kind, void* dst, int out_dtype,
                            int64_t out_pitch, int precision, void* workspace, size_t workspace_bytes,
                            void* stream) {
  return gaussian_impl(src, dtype, 1, 0, height, width, pitch, sigma, kernel_size, nodata, nodata_kind, dst,
                       out_dtype, 0, out_pitch, precision, workspace, workspace_bytes, stream);
}

extern "C" int vsr_gaussian_bands(const void* src, int dtype, int bands, int64_t band_stride, int64_t height,
                                  int64_t width, int64_t pitch, double sigma, int kernel_size, double nodata,
                                  int nodata_kind, void* dst, int out_dtype, int64_t out_band_stride,
                                  int64_t out_pitch, int precision, void* workspace, size_t workspace_bytes,
                                  void* stream) {
  return gaussian_impl(src, dtype, bands, band_stride, height, width, pitch, sigma, kernel_size, nodata, nodata_kind,
                       dst, out_dtype, out_band_stride, out_pitch, precision, workspace, workspace_bytes, stream);
}

static int focal_mean_impl(const void* src, int dtype, int bands, int64_t band_stride, int64_t height,
                           int64_t width, int64_t pitch, int radius_y, int radius_x, double nodata, int nodata_kind,
                           void* dst, int out_dtype, int64_t out_band_stride, int64_t out_pitch, void* stream) {
  if (bands < 1) return fail(VSR_ERR_INVALID_ARG, "bands must be >= 1");
  int rc = check_raster(src, dtype, height, width, pitch, dst, out_dtype, out_pitch);
  if (rc || height == 0 || width == 0) return rc;
  if (radius_y < 0 || radius_x < 0) return fail(VSR_ERR_INVALID_ARG, "radius must be non-negative");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  BoxArgs a{src, dtype, height, width, pitch, make_nodata(dtype, nodata, nodata_kind), radius_y, radius_x,
            nodata, dst, out_dtype, out_pitch, band_stride, out_band_stride};
  switch (dtype) {
    case VSR_U8:
    case VSR_I16:
    case VSR_U16: {
      const int rc2 = launch_slide(a, st, bands);  // square windows up to 15 x 15
      if (rc2 >= 0) return rc2;
      // int32 sums stay exact for windows of <= 1023 16-bit values
      if ((2 * radius_y + 1) * (2 * radius_x + 1) <= kMaxFastWindow) return launch_box_fast<false>(a, st, bands);
    }
      return launch_box<AccD>(a, st, bands);
    case VSR_F32:
      if ((2 * radius_y + 1) * (2 * radius_x + 1) <= kMaxFastWindow) return launch_box_fast<true>(a, st, bands);
      return launch_box<AccF2>(a, st, bands);
    default: return launch_box<AccD>(a, st, bands);
  }
}

namespace vsr {
int focal_mean_bands_impl(const void* src, int dtype, int bands, int64_t band_stride, int64_t height, int64_t width,
                          int64_t pitch, int radius_y, int radius_x, double nodata, int nodata_kind, void* dst,
                          int out_dtype, int64_t out_band_stride, int64_t out_pitch, void* stream) {
  return focal_mean_impl(src, dtype, bands, band_stride, height, width, pitch, radius_y, radius_x, nodata,
                         nodata_kind, dst, out_dtype, out_band_stride, out_pitch, stream);
}
}  // namespace vsr

extern "C" int vsr_focal_mean(const void* src, int dtype, int64_t height, int64_t width, int64_t pitch,
                              int radius_y, int radius_x, double nodata, int nodata_kind, void* dst, int out_dtype,
                              int64_t out_pitch, void* stream) {
  return focal_mean_impl(src, dtype, 1, 0, height, width, pitch, radius_y, radius_x, nodata, nodata_kind, dst,
                         out_dtype, 0, out_pitch, stream);
}

extern "C" int vsr_focal_mean_bands(const void* src, int dtype, int bands, int64_t band_stride, int64_t height,
                                    int64_t width, int64_t pitch, int radius_y, int radius_x, double nodata,
                                    int nodata_kind, void* dst, int out_dtype, int64_t out_band_stride,
                                    int64_t out_pitch, void* stream) {
  return focal_mean_impl(src, dtype, bands, band_stride, height, width, pitch, radius_y, radius_x, nodata,
                         nodata_kind, dst, out_dtype, out_band_stride, out_pitch, stream);
}
