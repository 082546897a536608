// Split-BF16 tcgen05 implicit GEMM for large normalised focal convolutions.
//
// Formulation (one output tile = 128 image rows x N image columns):
//   out[y0+m, x0+n] = sum_ky sum_k' X[m+ky][k'] * w[ky][k'-n]
// where X is the tile's input window (128+kh-1 rows x N+kw-1 columns).  For
// each kernel row ky this is a GEMM  C[m][n] += A_ky[m][k'] B_ky[k'][n]  with
// A_ky = X shifted down ky rows and B_ky the Toeplitz band of weight row ky.
//
// Operand layouts (canonical K-major, no swizzle: 8-row x 16-byte core
// matrices, LBO = stride between core matrices along K, SBO = along M/N):
//  * A is stored with its K index reversed (k = Kp-1-k') and rows 16 bytes
//    apart, so A_ky is the same descriptor advanced by ky*16 bytes -- no copy
//    per kernel row.
//  * B (also K-reversed) satisfies B[n+8][k-8] = B[n][k]; with SBO = LBO =
//    128 bytes every (n-group, k-chunk) pair maps to core matrix n/8 + k/8,
//    so a kernel row's Toeplitz band needs only (Kp/8 + N/8 - 1) core
//    matrices of shared memory.
// Precision: values are centred on the tile's centre pixel (mu) and split
// z = z_hi + z_lo, w = w_hi + w_lo (BF16); num = z_hi w_hi + z_hi w_lo +
// z_lo w_hi accumulates in FP32 in tensor memory.  The weight sum comes from
// the same split weights (a 0/1 validity operand times w_hi and w_lo), so the
// quotient is a consistently weighted average; out = num/den + mu.
// NaN taps (the reference's NaN * 0 poisoning) and +-inf are excluded from
// the GEMM and their window footprint is marked NaN from per-row bitmasks.
//
// Pipeline per persistent CTA (128 threads, one CTA per SM):
//   TMA 2-D load of the tile window -> all threads convert to BF16 hi/lo and
//   validity in the MMA layout -> the next tile's TMA is issued -> thread 0
//   issues the tcgen05.mma chains and commits to an mbarrier; the epilogue of
//   the previous tile (tcgen05.ld of its accumulators, FP32 sums, stores)
//   runs while the tensor core works on this one (two A-operand buffers when
//   they fit, two TMEM buffers).
// Every wait is bounded (an error code in the device word on expiry; the
// CTA then frees its tensor memory and leaves).
#include <cuda_bf16.h>

#include "vsr_internal.cuh"

namespace vsr {

size_t conv_tc_workspace(int kh, int kw);
int conv_tc_supported(int kh, int kw);
int run_conv_tc(const void* src, int dtype, int64_t H, int64_t W, int64_t pitch, const double* weights_host,
                int kh, int kw, double nodata, int nodata_kind, void* dst, int out_dtype, int64_t out_pitch,
                void* workspace, size_t ws_bytes, cudaStream_t st);

namespace {

constexpr int kM = 128;     // output rows per tile (TMEM lanes)
constexpr int kTN = 16;     // output columns per tile (MMA N)
constexpr int kThreadsTC = 256;
constexpr int kMaxTCK = 41;

struct TcGeom {
  int kh, kw;
  int R;       // staged rows = kM + kh - 1
  int KW;      // useful window width = kTN + kw - 1
  int Kp;      // GEMM K (KW rounded up to 16)
  int KC;      // Kp / 8 core-matrix columns
  int KS;      // Kp / 16 MMA k-steps
  int NB;      // core matrices per Toeplitz band = KC + kTN/8 - 1
  int BW;      // TMA box width (floats), 16-byte multiple covering KW + 3
};

__host__ __device__ inline TcGeom make_geom(int kh, int kw) {
  TcGeom g;
  g.kh = kh;
  g.kw = kw;
  g.R = kM + kh - 1;
  g.KW = kTN + kw - 1;
  g.Kp = (g.KW + 15) & ~15;
  g.KC = g.Kp / 8;
  g.KS = g.Kp / 16;
  g.NB = g.KC + kTN / 8 - 1;
  g.BW = (g.KW + 3 + 3) & ~3;
  return g;
}

struct TcSmem {  // byte offsets inside the 1024-aligned dynamic shared memory
  uint32_t a_hi, a_lo, a_valid, a_stride, bw, stage, ctr, nanrow, total;
};

// nbuf A-operand buffers (2: the next tile is converted while the tensor core
// works on the current one; 1 when two do not fit).
__host__ __device__ inline TcSmem make_smem(const TcGeom& g, int nbuf) {
  TcSmem s;
  const uint32_t a_bytes = (static_cast<uint32_t>(g.KC) * g.R * 16 + 127) & ~127u;
  s.a_stride = a_bytes;  // between buffers of one operand
  s.a_hi = 0;
  s.a_lo = s.a_hi + nbuf * a_bytes;
  s.a_valid = s.a_lo + nbuf * a_bytes;
  s.bw = s.a_valid + nbuf * a_bytes;
  const uint32_t b_bytes = static_cast<uint32_t>(g.kh) * 2 * g.NB * 128;
  s.stage = (s.bw + b_bytes + 1023) & ~1023u;
  const uint32_t stage_bytes = static_cast<uint32_t>(g.R) * g.BW * 4;
  s.ctr = (s.stage + stage_bytes + 127) & ~127u;
  s.nanrow = (s.ctr + 2 * kM * kTN + 127) & ~127u;
  s.total = s.nanrow + 2 * static_cast<uint32_t>(g.R) * 8;
  return s;
}

// --- tcgen05 / descriptor helpers (PTX ISA: tcgen05 family, sm_100a+) ---
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  // start address, leading byte offset, stride byte offset (all >> 4),
  // descriptor version 1 (bits 46-47), no swizzle (bits 61-63 = 0).
  return (static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4)) |
         (static_cast<uint64_t>((lbo & 0x3FFFFu) >> 4) << 16) |
         (static_cast<uint64_t>((sbo & 0x3FFFFu) >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major,
// M = 128, N = kTN.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(kTN >> 3) << 17) |
                            (static_cast<uint32_t>(kM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 8 consecutive f32 columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float v[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// 16 consecutive f32 columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

struct TcNodata {
  int kind;
  float fv;
};

struct TcArgs {
  int64_t H, W;
  TcNodata nd;
  double nd_out;
  void* dst;
  int out_dtype;
  int64_t out_pitch;
  const uint4* bw_img;  // kh x 2 x NB core matrices (bf16) from the prep kernel
  const float* wsum;    // sum of (w_hi + w_lo) over all taps
  int kh, kw;
  int nbuf;             // A-operand buffers (1 or 2)
};

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
  const __nv_bfloat16 ha = __float2bfloat16_rn(a), hb = __float2bfloat16_rn(b);
  return static_cast<uint32_t>(__bfloat16_as_ushort(ha)) | (static_cast<uint32_t>(__bfloat16_as_ushort(hb)) << 16);
}

// Accumulators per TMEM buffer (192 columns): hi*hi groups at [0, 64), the
// correction terms at [64, 80), weight-sum groups at [96, 160).  Each group
// takes at most ~64 MMAs: tensor-core accumulation error grows with the
// number of MMAs chained into one accumulator.
__host__ __device__ inline int tc_groups(int kh, int ks) {
  const int g = (kh * ks + 63) / 64;
  return g < 1 ? 1 : (g > 4 ? 4 : g);
}

__global__ void __launch_bounds__(kThreadsTC, 1) conv_tc_kernel(const __grid_constant__ CUtensorMap tmap,
                                                                 const TcArgs a, uint32_t* err_word) {
  extern __shared__ unsigned char tc_raw[];
  __shared__ __align__(8) uint64_t tma_bar, mma_bar[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int64_t info_x0[2], info_y0[2];
  __shared__ float info_mu[2];
  __shared__ int info_inv[2], info_nan[2];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(tc_raw) + 1023) & ~uintptr_t(1023));
  const TcGeom g = make_geom(a.kh, a.kw);
  const TcSmem L = make_smem(g, a.nbuf);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t tiles_x = (a.W + kTN - 1) / kTN;
  const int64_t total = tiles_x * ((a.H + kM - 1) / kM);
  const uint32_t s_base = smem_u32(sm);
  float* stage = reinterpret_cast<float*>(sm + L.stage);
  const int G = tc_groups(a.kh, g.KS);
  const uint32_t cols_per_buf = 192;  // hh groups | corr | den groups

  // Weight Toeplitz images -> shared memory (once per CTA).
  {
    uint4* dstw = reinterpret_cast<uint4*>(sm + L.bw);
    const int n16 = a.kh * 2 * g.NB * 8;
    for (int i = tid; i < n16; i += kThreadsTC) dstw[i] = a.bw_img[i];
  }
  __shared__ float s_wsum;
  if (tid == 0) s_wsum = *a.wsum;
  if (warp == 0) tmem_alloc(&tmem_slot, 512);
  if (tid == 0) {
    prefetch_tensormap(&tmap);
    mbar_init(&tma_bar, 1);
    mbar_init(&mma_bar[0], 1);
    mbar_init(&mma_bar[1], 1);
    fence_mbar_init();
  }
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t stage_bytes = static_cast<uint32_t>(g.R) * g.BW * 4;
  const uint32_t lbo_a = static_cast<uint32_t>(g.R) * 16;

  auto window_x = [&](int64_t t, int64_t& gx0, int64_t& xs) {
    const int64_t tx = t % tiles_x;
    gx0 = tx * kTN - a.kw / 2;
    xs = gx0 >= 0 ? (gx0 & ~int64_t(3)) : -((-gx0 + 3) & ~int64_t(3));
  };
  auto issue = [&](int64_t t) {
    int64_t gx0, xs;
    window_x(t, gx0, xs);
    mbar_arrive_expect_tx(&tma_bar, stage_bytes);
    tma_load_2d(stage, &tmap, static_cast<int>(xs), static_cast<int>((t / tiles_x) * kM - a.kh / 2), &tma_bar);
  };

  // Epilogue of the tile whose accumulators sit in TMEM buffer tb.
  auto epilogue = [&](int tb) {
    const int64_t x0 = info_x0[tb], y0 = info_y0[tb];
    const float mu = info_mu[tb];
    const int quarter = warp & 3, half = warp >> 2;  // lanes 32q.., columns 8h..
    const int m = quarter * 32 + lane;
    const uint32_t base = tmem + tb * cols_per_buf + (static_cast<uint32_t>(quarter * 32) << 16) + half * 8;
    float num[8], part[8], den[8];
    tmem_ld8(base, num);
    for (int gi = 1; gi < G; ++gi) {
      tmem_ld8(base + gi * kTN, part);
#pragma unroll
      for (int n = 0; n < 8; ++n) num[n] += part[n];
    }
    tmem_ld8(base + 64, part);  // correction terms
#pragma unroll
    for (int n = 0; n < 8; ++n) num[n] += part[n];
    if (info_inv[tb]) {
      tmem_ld8(base + 96, den);
      for (int gi = 1; gi < G; ++gi) {
        tmem_ld8(base + 96 + gi * kTN, part);
#pragma unroll
        for (int n = 0; n < 8; ++n) den[n] += part[n];
      }
    } else {
#pragma unroll
      for (int n = 0; n < 8; ++n) den[n] = s_wsum;
    }
    const uint8_t* ctr = sm + L.ctr + tb * (kM * kTN);
    const unsigned long long* nanrow = reinterpret_cast<const unsigned long long*>(sm + L.nanrow) + tb * g.R;
    unsigned long long nanfoot = 0ull;
    if (info_nan[tb])
      for (int j = 0; j < a.kh; ++j) nanfoot |= nanrow[m + j];
    const int64_t y = y0 + m;
    if (y < a.H) {
#pragma unroll
      for (int n8 = 0; n8 < 8; ++n8) {
        const int n = half * 8 + n8;
        const int64_t x = x0 + n;
        if (x >= a.W) break;
        double out;
        if (!ctr[m * kTN + n] || !(den[n8] > 0.0f)) out = a.nd_out;
        else if ((nanfoot >> n) & 1ull) out = __int_as_float(0x7fc00000);
        else out = static_cast<double>(num[n8] / den[n8] + mu);
        if (a.out_dtype == VSR_F64) static_cast<double*>(a.dst)[y * a.out_pitch + x] = out;
        else static_cast<float*>(a.dst)[y * a.out_pitch + x] = static_cast<float>(out);
      }
    }
  };

  if (tid == 0 && static_cast<int64_t>(blockIdx.x) < total) issue(blockIdx.x);

  uint32_t tma_phase = 0;
  uint32_t mma_phase[2] = {0u, 0u};
  bool failed = false;
  int it = 0;
  bool prev_pending = false;  // an MMA batch whose epilogue has not run yet
  for (int64_t t = blockIdx.x; t < total; t += gridDim.x, ++it) {
    const int b = it % a.nbuf, tb = it & 1;
    if (a.nbuf == 1 && prev_pending) {
      // single A buffer: the previous tile's MMAs must finish before it is rewritten
      const bool done = mbar_wait_bounded(&mma_bar[tb ^ 1], mma_phase[tb ^ 1], err_word, kDevErrMmaTimeout);
      if (__syncthreads_or(!done)) { failed = true; break; }
    }
    const bool ok = mbar_wait_bounded(&tma_bar, tma_phase, err_word, kDevErrTmaTimeout);
    tma_phase ^= 1;
    if (__syncthreads_or(!ok)) { failed = true; break; }
    const int64_t ty = t / tiles_x;
    int64_t gx0, xs;
    window_x(t, gx0, xs);
    const int64_t x0 = (t % tiles_x) * kTN, y0 = ty * kM;
    const int off = static_cast<int>(gx0 - xs);
    const int64_t gy0 = y0 - a.kh / 2;
    float mu = 0.0f;
    {
      const int rc = g.R / 2, kc = g.KW / 2;
      const int64_t yy = gy0 + rc, xx = gx0 + kc;
      const float v = stage[rc * g.BW + off + kc];
      const bool valid = yy >= 0 && yy < a.H && xx >= 0 && xx < a.W &&
                         !(a.nd.kind == VSR_NODATA_VALUE ? v == a.nd.fv : (a.nd.kind == VSR_NODATA_NAN ? v != v : false));
      if (valid && isfinite(v)) mu = v;
    }
    unsigned long long* nanrow = reinterpret_cast<unsigned long long*>(sm + L.nanrow) + tb * g.R;
    uint8_t* ctr = sm + L.ctr + tb * (kM * kTN);
    for (int i = tid; i < g.R; i += kThreadsTC) nanrow[i] = 0ull;
    __syncthreads();

    const uint32_t abuf = b * L.a_stride;
    bool any_invalid = false, any_nan = false;
    const int items = g.KC * g.R;
    for (int itm = tid; itm < items; itm += kThreadsTC) {
      const int kc = itm / g.R, rho = itm - kc * g.R;
      const int64_t yy = gy0 + rho;
      const bool row_in = yy >= 0 && yy < a.H;
      float hi[8], lo[8], vd[8];
      unsigned long long nanbits = 0ull;
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const int kp = g.Kp - 1 - (8 * kc + e);
        float z = 0.0f, valid = 0.0f;
        if (kp < g.KW) {
          const int64_t xx = gx0 + kp;
          const float v = stage[rho * g.BW + off + kp];
          const bool inb = row_in && xx >= 0 && xx < a.W;
          const bool okv = inb && !(a.nd.kind == VSR_NODATA_VALUE ? v == a.nd.fv
                                                                  : (a.nd.kind == VSR_NODATA_NAN ? v != v : false));
          // reference product v * w * valid: NaN (and inf * 0) poison the window
          if (inb && !isfinite(v * (okv ? 1.0f : 0.0f))) nanbits |= 1ull << kp;
          if (okv && isfinite(v)) {
            z = v - mu;
            valid = 1.0f;
          }
          any_invalid |= !okv;
          const int m = rho - a.kh / 2, n = kp - a.kw / 2;
          if (m >= 0 && m < kM && n >= 0 && n < kTN) ctr[m * kTN + n] = okv ? 1 : 0;
        }
        const float h = __bfloat162float(__float2bfloat16_rn(z));
        hi[e] = h;
        lo[e] = z - h;
        vd[e] = valid;
      }
      if (nanbits) {
        any_nan = true;
        atomicOr(&nanrow[rho], nanbits);
      }
      const uint32_t o = abuf + static_cast<uint32_t>(kc) * g.R * 16 + rho * 16;
      *reinterpret_cast<uint4*>(sm + L.a_hi + o) =
          make_uint4(pack_bf16x2(hi[0], hi[1]), pack_bf16x2(hi[2], hi[3]), pack_bf16x2(hi[4], hi[5]), pack_bf16x2(hi[6], hi[7]));
      *reinterpret_cast<uint4*>(sm + L.a_lo + o) =
          make_uint4(pack_bf16x2(lo[0], lo[1]), pack_bf16x2(lo[2], lo[3]), pack_bf16x2(lo[4], lo[5]), pack_bf16x2(lo[6], lo[7]));
      *reinterpret_cast<uint4*>(sm + L.a_valid + o) =
          make_uint4(pack_bf16x2(vd[0], vd[1]), pack_bf16x2(vd[2], vd[3]), pack_bf16x2(vd[4], vd[5]), pack_bf16x2(vd[6], vd[7]));
    }
    fence_proxy_async_smem();
    const bool has_invalid = __syncthreads_or(any_invalid);
    const bool has_nan = __syncthreads_or(any_nan);
    if (tid == 0) {
      info_x0[tb] = x0;
      info_y0[tb] = y0;
      info_mu[tb] = mu;
      info_inv[tb] = has_invalid;
      info_nan[tb] = has_nan;
      // the staging buffer is consumed: prefetch the next tile's window
      const int64_t nt = t + gridDim.x;
      if (nt < total) issue(nt);
      tc_fence_after();
      // descriptors advance by plain adds on the 16-byte start-address field
      const uint64_t d_ahi = smem_desc(s_base + L.a_hi + abuf, lbo_a, 128);
      const uint64_t d_alo = smem_desc(s_base + L.a_lo + abuf, lbo_a, 128);
      const uint64_t d_av = smem_desc(s_base + L.a_valid + abuf, lbo_a, 128);
      const uint64_t d_b = smem_desc(s_base + L.bw, 128, 128);
      const uint64_t a_ks = 2 * lbo_a >> 4, b_band = static_cast<uint64_t>(g.NB) * 8;
      const uint32_t t_acc = tmem + tb * cols_per_buf;
      const uint32_t t_corr = t_acc + 64, t_den = t_acc + 96;
      for (int ky = 0; ky < a.kh; ++ky) {
        const int grp = (ky * G) / a.kh;
        const bool grp_first = ky == 0 || ((ky - 1) * G) / a.kh != grp;
        const uint64_t bh0 = d_b + static_cast<uint64_t>(2 * ky) * b_band;
        const uint64_t bl0 = bh0 + b_band;
        for (int ks = 0; ks < g.KS; ++ks) {
          const uint64_t ao = static_cast<uint64_t>(ky) + ks * a_ks;
          const uint64_t bo = static_cast<uint64_t>(ks) * 16;  // 2 core matrices of 128 B
          mma_bf16(t_acc + grp * kTN, d_ahi + ao, bh0 + bo, !(grp_first && ks == 0));
          mma_bf16(t_corr, d_ahi + ao, bl0 + bo, (ky | ks) != 0);
          mma_bf16(t_corr, d_alo + ao, bh0 + bo, 1);
          if (has_invalid) {
            mma_bf16(t_den + grp * kTN, d_av + ao, bh0 + bo, !(grp_first && ks == 0));
            mma_bf16(t_den + grp * kTN, d_av + ao, bl0 + bo, 1);
          }
        }
      }
      mma_commit(&mma_bar[tb]);
    }
    // horizontal NaN footprint of this tile (read by its epilogue later)
    if (has_nan) {
      for (int rho = tid; rho < g.R; rho += kThreadsTC) {
        const unsigned long long mrow = nanrow[rho];
        unsigned long long h = 0ull;
        for (int j = 0; j < a.kw; ++j) h |= mrow >> j;  // bit n: a NaN in columns [n, n+kw)
        nanrow[rho] = h;
      }
    }
    // epilogue of the previous tile while the tensor core works on this one
    if (prev_pending) {
      if (a.nbuf == 2) {
        const bool done = mbar_wait_bounded(&mma_bar[tb ^ 1], mma_phase[tb ^ 1], err_word, kDevErrMmaTimeout);
        if (__syncthreads_or(!done)) { failed = true; break; }
      }
      mma_phase[tb ^ 1] ^= 1;
      tc_fence_after();
      epilogue(tb ^ 1);
    }
    prev_pending = true;
    tc_fence_before();
    __syncthreads();
  }
  if (!failed && prev_pending) {
    const int tb = (it - 1) & 1;
    const bool done = mbar_wait_bounded(&mma_bar[tb], mma_phase[tb], err_word, kDevErrMmaTimeout);
    if (!__syncthreads_or(!done)) {
      tc_fence_after();
      epilogue(tb);
    } else {
      failed = true;
    }
  }
  if (failed && tid == 0) {
    // A copy may still be in flight into the staging buffer: give it a
    // bounded chance to land before shared memory is released.
    mbar_wait_bounded(&tma_bar, tma_phase, err_word, kDevErrTmaTimeout);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

// Toeplitz band images: for ky, split s in {hi, lo}, core matrix c, row r,
// element e -> w[ky][Kp-1-8c-e-r] (0 outside [0, kw)), split as
// w = bf16(w) + bf16(w - bf16(w)); also the total of (w_hi + w_lo).
__global__ void prep_tc_weights(const double* __restrict__ w64, int kh, int kw, int Kp, int NB,
                                uint16_t* __restrict__ img, float* __restrict__ wsum) {
  const int per_row = NB * 64;
  const int total = kh * per_row;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int ky = i / per_row, rem = i - ky * per_row;
    const int c = rem / 64, r = (rem / 8) & 7, e = rem & 7;
    const int kx = Kp - 1 - 8 * c - e - r;
    const double w = (kx >= 0 && kx < kw) ? w64[ky * kw + kx] : 0.0;
    const __nv_bfloat16 hi = __float2bfloat16_rn(static_cast<float>(w));
    const __nv_bfloat16 lo = __float2bfloat16_rn(static_cast<float>(w - static_cast<double>(__bfloat162float(hi))));
    img[((ky * 2 + 0) * NB + c) * 64 + r * 8 + e] = __bfloat16_as_ushort(hi);
    img[((ky * 2 + 1) * NB + c) * 64 + r * 8 + e] = __bfloat16_as_ushort(lo);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < kh * kw; ++i) {
      const __nv_bfloat16 hi = __float2bfloat16_rn(static_cast<float>(w64[i]));
      const double h = __bfloat162float(hi);
      const double l = __bfloat162float(__float2bfloat16_rn(static_cast<float>(w64[i] - h)));
      s += h + l;
    }
    wsum[0] = static_cast<float>(s);
  }
}

}  // namespace

static int tc_nbuf(int kh, int kw) {
  const TcGeom g = make_geom(kh, kw);
  return make_smem(g, 2).total + 1024 <= 227 * 1024 ? 2 : 1;
}

int conv_tc_supported(int kh, int kw) {
  if (kh < 1 || kw < 1 || kh > kMaxTCK || kw > kMaxTCK) return 0;
  const TcGeom g = make_geom(kh, kw);
  return make_smem(g, 1).total + 1024 <= 227 * 1024 && g.KW <= 64 && g.BW <= 256 && g.R <= 256;
}

// Workspace: float64 weights | Toeplitz images | total.
size_t conv_tc_workspace(int kh, int kw) {
  const TcGeom g = make_geom(kh, kw);
  const size_t a = (static_cast<size_t>(kh) * kw * 8 + 255) & ~size_t(255);
  const size_t b = (static_cast<size_t>(kh) * 2 * g.NB * 128 + 255) & ~size_t(255);
  return a + b + 256;
}

int run_conv_tc(const void* src, int dtype, int64_t H, int64_t W, int64_t pitch, const double* weights_host, int kh,
                int kw, double nodata, int nodata_kind, void* dst, int out_dtype, int64_t out_pitch, void* workspace,
                size_t ws_bytes, cudaStream_t st) {
  if (dtype != VSR_F32) return fail(VSR_ERR_UNSUPPORTED, "split-BF16 convolution reads float32 rasters");
  if (!conv_tc_supported(kh, kw))
    return fail(VSR_ERR_UNSUPPORTED, "split-BF16 convolution supports kernels up to %dx%d", kMaxTCK, kMaxTCK);
  if (!aligned(src, 16) || (pitch % 4) != 0)
    return fail(VSR_ERR_UNSUPPORTED, "split-BF16 convolution needs 16-byte aligned rows");
  const size_t need = conv_tc_workspace(kh, kw);
  if (!workspace || ws_bytes < need || !aligned(workspace, 256))
    return fail(VSR_ERR_WORKSPACE, "workspace must be 256-byte aligned and >= %zu bytes", need);
  const TcGeom g = make_geom(kh, kw);
  const int nbuf = tc_nbuf(kh, kw);
  const TcSmem L = make_smem(g, nbuf);
  char* ws = static_cast<char*>(workspace);
  double* w64 = reinterpret_cast<double*>(ws);
  const size_t off_img = (static_cast<size_t>(kh) * kw * 8 + 255) & ~size_t(255);
  uint16_t* img = reinterpret_cast<uint16_t*>(ws + off_img);
  float* wsum = reinterpret_cast<float*>(ws + need - 256);
  VSR_CUDA_TRY(cudaMemcpyAsync(w64, weights_host, static_cast<size_t>(kh) * kw * 8, cudaMemcpyHostToDevice, st));
  prep_tc_weights<<<16, 256, 0, st>>>(w64, kh, kw, g.Kp, g.NB, img, wsum);
  VSR_CUDA_TRY(cudaGetLastError());

  CUtensorMap map;
  int rc = encode_tensor_map_2d(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, src, W, H, pitch, g.BW, g.R);
  if (rc) return rc;
  uint32_t* err = device_error_word();
  if (!err) return VSR_ERR_CUDA;
  double ndv = 0.0;
  const int kind = resolve_nodata(VSR_F32, nodata, nodata_kind, &ndv);
  TcArgs a{H, W, {kind, static_cast<float>(ndv)}, nodata, dst, out_dtype, out_pitch,
           reinterpret_cast<const uint4*>(img), wsum, kh, kw, nbuf};
  // At least 116 KB of shared memory keeps one CTA per SM.
  const size_t smem = std::max<size_t>(L.total + 1024, 116 * 1024);
  VSR_CUDA_TRY(cudaFuncSetAttribute(conv_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  const int64_t tiles = ((W + kTN - 1) / kTN) * ((H + kM - 1) / kM);
  const int64_t grid = std::min<int64_t>(tiles, sm_count());
  conv_tc_kernel<<<static_cast<unsigned>(grid), kThreadsTC, smem, st>>>(map, a, err);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}

}  // namespace vsr
