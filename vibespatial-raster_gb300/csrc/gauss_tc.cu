// Separable split-precision Gaussian on the tcgen05 tensor cores: two line passes.
//
// The reference's k x k Gaussian weights outer(g, g) / sum (algebra.py:2120-2152,
// applied as the normalised convolution of kernels/focal.py:101-145) factor
// into a pass along the rows and one along the columns.  Each is a 1-D
// normalised convolution of "lines",
//   num(l, p) = sum_j g[j] a_num(l, p - r + j),  den(l, p) = sum_j g[j] a_den(l, p - r + j),
// computed as a GEMM against the Toeplitz band of g, T[k][n] = g[k - n], in
// the K-reversed layouts of the 2-D kernel (conv_tc.cu): 16-byte rows of 8
// K-elements, window positions reversed along K, and the band stored once
// per anti-diagonal (core matrix c holds g[Kp - 1 - s - 8c - e - rr], read
// with leading and stride byte offsets of 128 B).  Weights are split into
// F16 hi/lo parts (22 significant bits; x 2^12 so the 4-sigma tails stay
// normal), FP32 accumulation.
//
// Pass 1 (lines = raster rows y, positions = raster columns x) reads the
// 8/16-bit integer raster.  Its tile is 128 positions x 64 lines and the
// operands are swapped against pass 2: A = the Toeplitz band (M = 128
// positions, hi and lo), B = the raster window (N = lines, K = 64 + 128
// positions), so the accumulator holds the row sums already transposed:
// TMEM lane = raster column, column = raster row.  Each value v is split
// exactly into bytes, v = 256 h + l (h signed for int16), and the B rows are
// F16 integers built with byte permutes and one packed F16 add each (the
// byte under the exponent of 1024, then 1024 subtracted):
//   plane 1 (N = 128): h of the 64 lines, then their validity (0 or 1),
//   plane 2 (N = 64):  l of the 64 lines,
// four MMAs per K step (hi and lo band against each plane) into one
// accumulator of 192 columns.  The epilogue forms the row sums
//   P_num = sum g v/2 = (256 D_h + D_l) 2^-13,   P_den = 2^8 sum g valid = D_v 2^-4
// (the weight scale removed), splits them into F16 hi/lo and stores, per
// raster column, 16-byte rows of 8 raster rows straight into pass 2's A
// layout: per 64-column block, 2 KB chunks of 8 positions (numerator rows of
// the block's columns, then weight-sum rows, positions reversed inside a
// row), chunks in descending position order, so a pass-2 tile's window is
// one contiguous run per plane.  A warp's 32 lanes write 32 consecutive
// rows: 512 contiguous bytes per store.
//
// Pass 2 (lines = raster columns, positions = raster rows) copies each
// 64-line x 64-position tile's window of the two chunk planes into shared
// memory with cp.async.bulk (no conversion); the MMA's M = 128 rows stack
// the tile's numerator operand over its weight-sum operand, three MMAs per
// K step (hi*hi into one accumulator, the corrections hi*lo + lo*hi into
// another), and the epilogue writes out[y][x] = 2^9 num / den where the
// centre pixel is valid and den > 0, else the nodata value.
//
// Windows start at p0 - ra, ra = r rounded up to 8 (aligned chunks and
// loads); the band is shifted by s = ra - r to match.
//
// Roles per persistent CTA (one per SM): warp 0 issues the MMAs; pass 1:
// warps 1-8 load each tile's raster window a tile ahead into registers,
// convert it into a B buffer and run the epilogue two tiles behind the
// conversion (tile j-1's MMAs overlap tile j's conversion); pass 2: warp 1
// bulk-copies the A windows in, warps 2-17 copy the centre pixels and run the
// epilogue (16 warps: 4 per TMEM lane quarter).  Operand buffers and TMEM accumulators are double-buffered and
// handed over through mbarriers; every wait is bounded (on expiry an error
// bit is recorded, a shared abort flag ends the other roles' waits, and the
// MMA issuer and the copy producer wait for their operations in flight
// before the CTA frees tensor memory).
#include "tc_common.cuh"

namespace vsr {

int gauss_tc_supported(int dtype, int k);
size_t gauss_tc_workspace(int64_t H, int64_t W, int dtype, int k);
size_t gauss_tc_workspace_bands(int64_t H, int64_t W, int dtype, int k, int bands);
int run_gauss_tc(const void* src, int dtype, int bands, int64_t band_stride, int64_t H, int64_t W, int64_t pitch,
                 double sigma, int k, double nodata, int nodata_kind, void* dst, int out_dtype,
                 int64_t out_band_stride, int64_t out_pitch, void* workspace, size_t ws_bytes, cudaStream_t st);

namespace {

using namespace tc;

// ---- pass 2 (columns) geometry
constexpr int kGL = kMmaM / 2;        // lines per tile
constexpr int kGN = kMmaN;            // positions per tile (MMA N)
constexpr int kGWarps = 16;           // centre-copy / epilogue warps (warps 2..17)
constexpr int kGConv = 32 * kGWarps;  // their threads
constexpr int kGThreads = 64 + kGConv;
constexpr int kGPosPart = kGN / (kGWarps / 4);  // positions per epilogue warp (4 warps per TMEM lane quarter)
constexpr int kGRowStep = kGConv / kGL;         // output rows between a thread's quotients
constexpr uint32_t kGChunk = kMmaM * 16;  // pass-2 A: one 8-position core-matrix column of 128 rows (2 KB)
constexpr int kGMaxK = 79;
constexpr int kGXPitch = kGN + 1;     // pass-2 exchange rows (floats; odd: conflict-free)
constexpr float kGScaleV = 0.5f;       // the row sums carry v/2
constexpr double kGScaleW = 4096.0;    // weights
constexpr float kGScaleD = 256.0f;     // the row pass's weight sums
// Pass-2 centre buffers: tile t's are copied at the start of iteration t and
// read in its epilogue (iteration t + 2) up to the barrier opening iteration
// t + 3's epilogue, so a buffer is rewritten four tiles later at the earliest.
constexpr int kGCenBufs = 4;

// ---- pass 1 (rows) geometry
constexpr int kRM = kMmaM;          // positions (raster columns) per tile: the MMA's M
constexpr int kRL = 64;             // lines (raster rows) per tile
constexpr int kRN1 = 2 * kRL;       // N of plane 1: high bytes, then validity
constexpr int kRN2 = kRL;           // N of plane 2: low bytes
constexpr int kRRp1 = kRN1 + 1;     // 16-byte rows between plane 1's core-matrix columns (odd: spreads the banks)
constexpr int kRRp2 = kRN2 + 1;
constexpr int kRWarps = 8;          // converter / epilogue warps (warps 1..8)
constexpr int kRConv = 32 * kRWarps;
constexpr int kRThreads = 32 + kRConv;
constexpr uint32_t kRAccStride = 256;  // TMEM columns between the two accumulator buffers (192 used)
constexpr uint32_t kRTmemCols = 512;
constexpr uint32_t kF16OneX2 = 0x3c003c00u;  // (1.0, 1.0) in F16
constexpr uint32_t kF16Exp1024X2 = 0x64646464u;  // bytes 0x64: F16 0x64bb = 1024 + bb
// kind::f16 instruction descriptors (D = F32, A = B = F16, K-major) for M = 128, N = 128 / 64
constexpr uint32_t kIdescN128 = (1u << 4) | ((128u >> 3) << 17) | ((static_cast<uint32_t>(kMmaM) >> 4) << 24);
constexpr uint32_t kIdescN64 = kIdescF16;
static_assert(kMmaN == 64, "kIdescF16 is the N = 64 form");

struct GaussGeom {
  int k, r;
  int ra;    // window lead: r rounded up to 8
  int s;     // band shift ra - r
  int KW;    // window positions per tile: positions + k - 1 + s
  int Kp;    // GEMM K: KW rounded up to 16
  int KC;    // Kp / 8 core-matrix columns
  int KS;    // Kp / 16 k-steps
  int NB;    // core matrices of the Toeplitz band: KC + (positions per tile)/8 - 1
  int ngrp;  // 4-position groups: pass 2, covering KW; pass 1, covering Kp
};

// pass 1: tile of kRM positions; pass 2: kGN positions
__host__ __device__ inline GaussGeom gauss_geom(int k, int pass = 2) {
  const int npos = pass == 1 ? kRM : kGN;
  GaussGeom g;
  g.k = k;
  g.r = k / 2;
  g.ra = (g.r + 7) & ~7;
  g.s = g.ra - g.r;
  g.KW = npos + k - 1 + g.s;
  g.Kp = (g.KW + 15) & ~15;
  g.KC = g.Kp / 8;
  g.KS = g.Kp / 16;
  g.NB = g.KC + npos / 8 - 1;
  g.ngrp = pass == 1 ? g.Kp / 4 : (g.KW + 3) / 4;
  return g;
}

// Pass-2 chunk planes: per 64-line block, np chunks of 2 KB.
__host__ __device__ inline int64_t gauss_np(int64_t H, const GaussGeom& g) {
  return ((H + kGN - 1) / kGN * kGN - kGN + g.Kp) / 8;
}

struct GaussPlan {  // pass 2: shared-memory byte offsets from the 1024-aligned base
  uint32_t a_bytes;  // one operand plane
  uint32_t lbo;      // its core-matrix column stride
  uint32_t band;     // hi band, then lo band (NB x 128 B each); buffer b: hi plane at 2 b a_bytes, lo after it
  uint32_t xch;      // 128 x kGXPitch floats (numerator rows over weight-sum rows)
  uint32_t raw;      // kGCenBufs buffers x 64 rows x 128 B of centre pixels
  uint32_t total;
};

__host__ __device__ inline GaussPlan gauss_plan(const GaussGeom& g) {
  GaussPlan p;
  p.lbo = kGChunk;
  p.a_bytes = (static_cast<uint32_t>(g.KC) * p.lbo + 127) & ~127u;
  p.band = 4 * p.a_bytes;
  p.xch = p.band + 2 * static_cast<uint32_t>(g.NB) * 128;
  p.raw = p.xch + static_cast<uint32_t>(kMmaM) * kGXPitch * 4;
  p.total = p.raw + static_cast<uint32_t>(kGCenBufs) * kGL * 128;
  return p;
}

struct RowPlan {  // pass 1: shared-memory byte offsets from the 1024-aligned base
  uint32_t lbo1, lbo2;        // core-matrix column strides of planes 1 and 2
  uint32_t p1_bytes, p2_bytes;  // one buffer of each plane
  uint32_t p1, p2;            // buffer 0 of each (buffer b at + b x bytes)
  uint32_t band;              // hi band, then lo band (NB x 128 B each)
  uint32_t total;
};

__host__ __device__ inline RowPlan row_plan(const GaussGeom& g) {
  RowPlan p;
  p.lbo1 = kRRp1 * 16;
  p.lbo2 = kRRp2 * 16;
  p.p1_bytes = (static_cast<uint32_t>(g.KC) * p.lbo1 + 127) & ~127u;
  p.p2_bytes = (static_cast<uint32_t>(g.KC) * p.lbo2 + 127) & ~127u;
  p.p1 = 0;
  p.p2 = 2 * p.p1_bytes;
  p.band = p.p2 + 2 * p.p2_bytes;
  p.total = p.band + 2 * static_cast<uint32_t>(g.NB) * 128;
  return p;
}

struct GaussArgs {
  const void* src;       // pass 1: the raster band
  int64_t lines, len;    // tile space: lines x positions
  int64_t pitch;         // pass 1: raster row pitch
  unsigned char* chi;    // chunk planes: pass 1 writes, pass 2 copies in
  unsigned char* clo;
  int64_t np;            // chunks per 64-line block
  const void* raster;    // pass 2: the raster band (centre validity)
  int64_t r_pitch;
  int nd_kind;           // the raster's resolved VSR_NODATA_*
  int64_t nd_iv;
  void* dst;             // pass 2 output
  int out_dtype;
  int64_t out_pitch;
  double nd_out;
  const uint16_t* band;  // this pass's Toeplitz band image: hi band then lo band
  int k;
  int bands;             // band-first stack, tiles band-major
  int64_t src_bstride;   // elements between raster bands (pass 1 src, pass 2 raster)
  size_t plane_bstride;  // bytes between the chunk planes of consecutive bands
  int64_t out_bstride;   // elements between output bands (pass 2)
};

// Named barrier 1 over the NT converter / epilogue threads; g_any also ORs a predicate.
template <int NT>
__device__ __forceinline__ void g_sync() {
  asm volatile("bar.sync 1, %0;" ::"n"(NT) : "memory");
}

template <int NT>
__device__ __forceinline__ bool g_any(bool p) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred q, o;\n\t"
      "setp.ne.u32 q, %1, 0;\n\t"
      "bar.red.or.pred o, 1, %2, q;\n\t"
      "selp.u32 %0, 1, 0, o;\n\t}"
      : "=r"(r)
      : "r"(static_cast<uint32_t>(p)), "n"(NT)
      : "memory");
  return r != 0;
}

__device__ __forceinline__ void mma_f16_n(uint32_t d_tmem, uint32_t a_lo, uint32_t b_lo, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t.reg .b64 da, db;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "mov.b64 da, {%1, %5};\n\t"
      "mov.b64 db, {%2, %5};\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], da, db, %3, p;\n\t}"
      ::"r"(d_tmem), "r"(a_lo), "r"(b_lo), "r"(idesc), "r"(accumulate), "r"(kDescHi));
}

__device__ __forceinline__ uint32_t hadd2_bits(uint32_t a, uint32_t b) {
  uint32_t r;
  asm("add.rn.f16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}

// 8 values as one 16-byte row of F16 hi parts and one of lo parts, element
// order reversed (element 0 holds v[7]); the residuals in packed f32x2
// (rounded as the scalar subtraction).
__device__ __forceinline__ void split_row8(const float v[8], uint4& hi, uint4& lo) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const float2 ab = make_float2(v[7 - 2 * q], v[6 - 2 * q]);
    const __half2 hv = __floats2half2_rn(ab.x, ab.y);
    const float2 r = __ffma2_rn(__half22float2(hv), make_float2(-1.0f, -1.0f), ab);
    const __half2 lv = __floats2half2_rn(r.x, r.y);
    h[q] = f16x2_bits(hv);
    l[q] = f16x2_bits(lv);
  }
  hi = make_uint4(h[0], h[1], h[2], h[3]);
  lo = make_uint4(l[0], l[1], l[2], l[3]);
}

// Persistent tile walk without divisions in the loop: tile t = (band bd,
// line block lb, position block pb), band-major; a CTA starts at blockIdx.x
// and steps by gridDim.x, the step split once into whole bands, line blocks
// and position blocks (32-bit: the host caps a launch at 2^31 tiles).
struct TileWalk {
  uint32_t npb, nlb;                  // position blocks per line block, line blocks per band
  uint32_t step_b, step_l, step_p;    // gridDim.x as bands, line blocks, position blocks
  uint32_t bd, lb, pb;                // the current tile
  __device__ void init(uint32_t npb_, uint32_t nlb_) {
    npb = npb_;
    nlb = nlb_;
    const uint32_t per_band = npb * nlb, step = gridDim.x, t = blockIdx.x;
    step_b = step / per_band;
    step_l = (step - step_b * per_band) / npb;
    step_p = step - step_b * per_band - step_l * npb;
    bd = t / per_band;
    lb = (t - bd * per_band) / npb;
    pb = t - bd * per_band - lb * npb;
  }
  __device__ void next() {
    pb += step_p;
    lb += step_l;
    if (pb >= npb) {
      pb -= npb;
      ++lb;
    }
    bd += step_b;
    if (lb >= nlb) {
      lb -= nlb;
      ++bd;
    }
  }
};

// ======================================================================
// Pass 1: rows.  DT: the raster's dtype (VSR_U8, VSR_I16, VSR_U16).
// ======================================================================
template <int DT>
__global__ void __launch_bounds__(kRThreads, 1) gauss_row_kernel(const GaussArgs a, uint32_t* err_word) {
  extern __shared__ unsigned char g_raw[];
  __shared__ __align__(8) uint64_t b_full[2], acc_full[2], acc_empty[2], drain_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(g_raw) + 1023) & ~uintptr_t(1023));
  const GaussGeom g = gauss_geom(a.k, 1);
  const RowPlan L = row_plan(g);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t npb = static_cast<uint32_t>((a.len + kRM - 1) / kRM);  // position blocks per line block
  const uint32_t nlb = static_cast<uint32_t>((a.lines + kRL - 1) / kRL);
  const int64_t total = static_cast<int64_t>(npb) * nlb * a.bands;
  const int64_t nx = (a.len + kGL - 1) / kGL;  // 64-column blocks of the chunk planes
  const uint32_t s_base = smem_u32(sm);

  // ---- set-up: the Toeplitz bands, the barriers, tensor memory (two
  // accumulator buffers of 192 columns: high bytes | validity | low bytes)
  for (int i = tid; i < g.NB * 16; i += kRThreads)  // 2 bands x NB x 128 B in 16-byte pieces
    reinterpret_cast<uint4*>(sm + L.band)[i] = __ldg(reinterpret_cast<const uint4*>(a.band) + i);
  if (tid == 0) {
    abort_flag = 0;
    for (int i = 0; i < 2; ++i) {
      mbar_init(&b_full[i], kRConv);
      mbar_init(&acc_full[i], 1);
      mbar_init(&acc_empty[i], kRConv);
    }
    mbar_init(&drain_bar, 1);
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(&tmem_slot, kRTmemCols);
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == 0) {
    // ========================================================= MMA issuer
    if (lane == 0) {
      const uint32_t ah0 = desc_lo(s_base + L.band, 128);
      const uint32_t al0 = desc_lo(s_base + L.band + static_cast<uint32_t>(g.NB) * 128, 128);
      const uint32_t k1 = (2 * L.lbo1) >> 4, k2 = (2 * L.lbo2) >> 4;  // one k-step: two core-matrix columns
      int j = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < total; t += gridDim.x, ++j) {
        const int b = j & 1;
        ok = wait_or_abort(&b_full[b], (j >> 1) & 1, &abort_flag, err_word, kDevErrMmaTimeout);
        if (ok && j >= 2) ok = wait_or_abort(&acc_empty[b], ((j >> 1) - 1) & 1, &abort_flag, err_word, kDevErrMmaTimeout);
        if (!ok) break;
        tc_fence_after();
        uint32_t ah = ah0, al = al0;
        uint32_t b1 = desc_lo(s_base + L.p1 + b * L.p1_bytes, L.lbo1);
        uint32_t b2 = desc_lo(s_base + L.p2 + b * L.p2_bytes, L.lbo2);
        const uint32_t d1 = tmem + b * kRAccStride, d2 = d1 + kRN1;
#pragma unroll 1
        for (int ks = 0; ks < g.KS; ++ks) {
          mma_f16_n(d1, ah, b1, kIdescN128, ks != 0);
          mma_f16_n(d1, al, b1, kIdescN128, 1u);
          mma_f16_n(d2, ah, b2, kIdescN64, ks != 0);
          mma_f16_n(d2, al, b2, kIdescN64, 1u);
          ah += 16;  // two 128-byte core matrices of the band
          al += 16;
          b1 += k1;
          b2 += k2;
        }
        mma_commit(&acc_full[b]);
      }
      if (!ok) {
        // MMAs already issued must finish before tensor memory is released
        mma_commit(&drain_bar);
        mbar_wait_bounded(&drain_bar, 0, err_word, kDevErrMmaTimeout);
      }
    }
  } else {
    // ========================================================= converters + epilogue
    const int ct = tid - 32;            // worker thread 0..255
    const int quarter = warp & 3;       // the TMEM lane quarter this warp may read
    const int lhalf = (warp - 1) >> 2;  // epilogue: lines 32 lhalf .. +31
    constexpr int kEsz = DT == VSR_U8 ? 1 : 2;
    const bool nd_val = a.nd_kind == VSR_NODATA_VALUE;
    // the nodata value's bit pattern in every element slot of a word
    const uint32_t ndp = static_cast<uint32_t>(a.nd_iv) & (kEsz == 1 ? 0xFFu : 0xFFFFu);
    const uint32_t nd_word = kEsz == 1 ? ndp * 0x01010101u : ndp * 0x00010001u;
    const int cw = ct >> 5;  // worker warp: lines cw + 8 q of a tile
    const char* srcb = static_cast<const char*>(a.src);
    const int64_t rstep = static_cast<int64_t>(kRWarps) * a.pitch * kEsz;  // bytes between a warp's lines
    // This thread's window groups: grp = lane + 32 h (h = 0, 1; grp < ngrp),
    // positions 4 grp .. 4 grp + 3 of the window (raster columns p0 - ra +
    // 4 grp ..), on lines cw + 8 q (q = 0..7); one 4- or 8-byte load each
    // (element loads for a group that straddles column W), held in
    // registers a tile ahead.  Their K-reversed B offsets (element klo =
    // Kp - 4 - 4 grp holds position 4 grp + 3) are fixed per thread.
    bool gon[2];
    uint32_t o1[2], o2[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int grp = lane + 32 * h;
      gon[h] = grp < g.ngrp;
      const int klo = g.Kp - 4 - 4 * grp;
      const uint32_t c8 = static_cast<uint32_t>(klo >> 3), e8 = static_cast<uint32_t>(klo & 7) * 2;
      o1[h] = c8 * L.lbo1 + e8 + cw * 16;
      o2[h] = c8 * L.lbo2 + e8 + cw * 16;
    }
    constexpr int kLinesPerWarp = kRL / kRWarps;
    uint2 raw[kLinesPerWarp][2];
    auto load_tile = [&](uint32_t bd, int64_t l0, int64_t p0) {
      const char* base = srcb + (static_cast<int64_t>(bd) * a.src_bstride + (l0 + cw) * a.pitch + p0 - g.ra) * kEsz;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int64_t xb = p0 - g.ra + 4 * (lane + 32 * h);
        const bool in = gon[h] && xb >= 0 && xb < a.len, whole = xb + 4 <= a.len;
        const char* gp = base + 4 * (lane + 32 * h) * kEsz;
#pragma unroll
        for (int q = 0; q < kLinesPerWarp; ++q, gp += rstep) {
          uint2 v = make_uint2(0u, 0u);
          if (in && l0 + cw + kRWarps * q < a.lines) {
            if (whole) {
              if (kEsz == 1) v.x = __ldg(reinterpret_cast<const uint32_t*>(gp));
              else v = __ldg(reinterpret_cast<const uint2*>(gp));
            } else {
              uint32_t e[4] = {0u, 0u, 0u, 0u};
              for (int c = 0; c < 4 && xb + c < a.len; ++c)
                e[c] = kEsz == 1 ? __ldg(reinterpret_cast<const uint8_t*>(gp) + c)
                                 : __ldg(reinterpret_cast<const uint16_t*>(gp) + c);
              if (kEsz == 1) v.x = e[0] | (e[1] << 8) | (e[2] << 16) | (e[3] << 24);
              else v = make_uint2(e[0] | (e[1] << 16), e[2] | (e[3] << 16));
            }
          }
          raw[q][h] = v;
        }
      }
    };
    // ... converted into B buffer b: the 8-byte segment of a group is (v3,
    // v2 | v1, v0); plane 1 row `line` = high bytes, row 64 + line =
    // validity, plane 2 row `line` = low bytes.  Invalid (nodata, outside
    // the raster) -> 0.
    auto convert_tile = [&](int b, int64_t l0, int64_t p0) {
      unsigned char* p1 = sm + L.p1 + b * L.p1_bytes;
      unsigned char* p2 = sm + L.p2 + b * L.p2_bytes;
      const bool interior = p0 - g.ra >= 0 && p0 - g.ra + g.Kp <= a.len;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (!gon[h]) continue;
        const int64_t xb = p0 - g.ra + 4 * (lane + 32 * h);
        // keep masks per 16-bit slot: word 0 = (v3, v2), word 1 = (v1, v0)
        uint32_t cm0 = 0xFFFFFFFFu, cm1 = 0xFFFFFFFFu;
        if (!interior) {
          const auto in = [&](int e) { return xb + e >= 0 && xb + e < a.len; };
          cm0 = (in(3) ? 0x0000FFFFu : 0u) | (in(2) ? 0xFFFF0000u : 0u);
          cm1 = (in(1) ? 0x0000FFFFu : 0u) | (in(0) ? 0xFFFF0000u : 0u);
        }
        const int64_t left = a.lines - l0 - cw;  // this warp's lines inside the raster: q * 8 < left
#pragma unroll
        for (int q = 0; q < kLinesPerWarp; ++q) {
          uint32_t keep0 = cm0, keep1 = cm1;
          if (kRWarps * q >= left) keep0 = keep1 = 0u;
          uint32_t h0, h1, l0w, l1w;
          if (kEsz == 1) {
            const uint32_t x = raw[q][h].x;  // bytes v0 .. v3
            if (nd_val) {
              const uint32_t eq = __vcmpeq4(x, nd_word);
              keep0 &= ~__byte_perm(eq, 0u, 0x2233);
              keep1 &= ~__byte_perm(eq, 0u, 0x0011);
            }
            h0 = 0u;
            h1 = 0u;
            l0w = hadd2_bits(__byte_perm(x, kF16Exp1024X2, 0x4243), 0xE400E400u);
            l1w = hadd2_bits(__byte_perm(x, kF16Exp1024X2, 0x4041), 0xE400E400u);
          } else {
            const uint32_t x = raw[q][h].x, y2 = raw[q][h].y;  // (v0 | v1 << 16), (v2 | v3 << 16)
            if (nd_val) {
              keep0 &= ~__vcmpeq2(__byte_perm(y2, 0u, 0x1032), nd_word);
              keep1 &= ~__vcmpeq2(__byte_perm(x, 0u, 0x1032), nd_word);
            }
            // int16: the high byte is signed; flip bit 15 so the byte is h + 128
            constexpr uint32_t flip = DT == VSR_I16 ? 0x80008000u : 0u;
            constexpr uint32_t hoff = DT == VSR_I16 ? 0xE480E480u : 0xE400E400u;  // -1152 or -1024
            h0 = hadd2_bits(__byte_perm(y2 ^ flip, kF16Exp1024X2, 0x4143), hoff);
            h1 = hadd2_bits(__byte_perm(x ^ flip, kF16Exp1024X2, 0x4143), hoff);
            l0w = hadd2_bits(__byte_perm(y2, kF16Exp1024X2, 0x4042), 0xE400E400u);
            l1w = hadd2_bits(__byte_perm(x, kF16Exp1024X2, 0x4042), 0xE400E400u);
          }
          unsigned char* q1 = p1 + o1[h] + q * (kRWarps * 16);
          *reinterpret_cast<uint2*>(q1) = make_uint2(h0 & keep0, h1 & keep1);
          *reinterpret_cast<uint2*>(q1 + kRL * 16) = make_uint2(kF16OneX2 & keep0, kF16OneX2 & keep1);
          *reinterpret_cast<uint2*>(p2 + o2[h] + q * (kRWarps * 16)) = make_uint2(l0w & keep0, l1w & keep1);
        }
      }
    };

    // Tile jj's row sums for this thread's raster column x = p0 + 32 quarter
    // + lane and raster rows l0 + 32 lhalf .. +31, stored as chunk rows.
    auto epilogue = [&](int jj, int64_t bd, int64_t l0, int64_t p0) -> bool {
      const int b = jj & 1;
      bool got = true;
      if (ct == 0) got = wait_or_abort(&acc_full[b], (jj >> 1) & 1, &abort_flag, err_word, kDevErrMmaTimeout);
      if (g_any<kRConv>(!got)) return false;
      tc_fence_after();
      const uint32_t lane_base = tmem + b * kRAccStride + (static_cast<uint32_t>(quarter * 32) << 16) + lhalf * 32;
      const int64_t x = p0 + quarter * 32 + lane;
      const int64_t lb = x / kGL;
      const bool xin = x < a.len, store = lb < nx;  // columns past the planes' last block: nothing to store
      const int64_t h8 = (a.lines + 7) & ~int64_t(7);
      const int64_t P0 = (l0 + g.ra) / 8 + lhalf * 4;  // padded chunk of this thread's first row
      const size_t off0 = store ? bd * a.plane_bstride +
                                      (static_cast<size_t>(lb) * a.np + static_cast<size_t>(a.np - 1 - P0)) * kGChunk +
                                      static_cast<size_t>(x & (kGL - 1)) * 16
                                : 0;
      // two halves of 16 rows: high bytes, validity and low bytes of each
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        uint32_t rh[16], rv[16], rl[16];
        tmem_ld16_issue(lane_base + 16 * hh, rh);
        tmem_ld16_issue(lane_base + kRL + 16 * hh, rv);
        tmem_ld16_issue(lane_base + kRN1 + 16 * hh, rl);
        tmem_wait_ld16(rh);
        tmem_wait_ld16(rv);
        tmem_wait_ld16(rl);
        if (hh == 1) {
          tc_fence_before();
          mbar_arrive(&acc_empty[b]);  // the accumulators may be reused
        }
#pragma unroll
        for (int c2 = 0; c2 < 2; ++c2) {  // 8 rows a chunk
          const int c = 2 * hh + c2;
          const int64_t y0 = l0 + lhalf * 32 + 8 * c;
          if (!store || y0 >= h8) continue;
          float num[8], den[8];
#pragma unroll
          for (int e = 0; e < 8; e += 2) {  // packed pairs: (256 D_h + D_l) 2^-13, D_v 2^-4
            const int n = 8 * c2 + e;
            const float2 nl = __fmul2_rn(make_float2(__uint_as_float(rl[n]), __uint_as_float(rl[n + 1])),
                                         make_float2(0.0001220703125f, 0.0001220703125f));
            const float2 nn = __ffma2_rn(make_float2(__uint_as_float(rh[n]), __uint_as_float(rh[n + 1])),
                                         make_float2(0.03125f, 0.03125f), nl);
            const float2 dd = __fmul2_rn(make_float2(__uint_as_float(rv[n]), __uint_as_float(rv[n + 1])),
                                         make_float2(0.0625f, 0.0625f));
            num[e] = nn.x;
            num[e + 1] = nn.y;
            den[e] = dd.x;
            den[e + 1] = dd.y;
          }
          if (!xin || y0 + 8 > a.lines) {  // rows past the raster, or a column past it: zeros
            const int nrow = xin ? static_cast<int>(a.lines - y0) : 0;
#pragma unroll
            for (int e = 0; e < 8; ++e)
              if (e >= nrow) num[e] = den[e] = 0.0f;
          }
          uint4 nh, nl, dh, dl;
          split_row8(num, nh, nl);
          split_row8(den, dh, dl);
          const size_t o = off0 - static_cast<size_t>(c) * kGChunk;  // chunks stored in descending order
          *reinterpret_cast<uint4*>(a.chi + o) = nh;
          *reinterpret_cast<uint4*>(a.clo + o) = nl;
          *reinterpret_cast<uint4*>(a.chi + o + kGL * 16) = dh;
          *reinterpret_cast<uint4*>(a.clo + o + kGL * 16) = dl;
        }
      }
      return true;
    };

    // Per tile j: tile j-2's epilogue (its MMAs finished while tile j-1's
    // were issued), then tile j's window (loaded an iteration ago) is
    // converted into B buffer j & 1 -- last read by tile j-2's MMAs, complete
    // once its accumulators were -- and tile j+1's window is loaded.
    TileWalk w;
    w.init(npb, nlb);
    int j = 0;
    bool ok = true;
    int64_t b1 = 0, l1 = 0, p1 = 0, b2 = 0, l2 = 0, p2 = 0;  // band / first line / position of tiles j-1, j-2
    if (w.bd < static_cast<uint32_t>(a.bands)) load_tile(w.bd, static_cast<int64_t>(w.lb) * kRL, static_cast<int64_t>(w.pb) * kRM);
    for (; w.bd < static_cast<uint32_t>(a.bands); ++j) {
      const int64_t bd = w.bd, l0 = static_cast<int64_t>(w.lb) * kRL, p0 = static_cast<int64_t>(w.pb) * kRM;
      if (j >= 2 && !epilogue(j - 2, b2, l2, p2)) {
        ok = false;
        break;
      }
      convert_tile(j & 1, l0, p0);
      fence_proxy_async_smem();  // generic-proxy operand writes -> visible to the tensor core
      mbar_arrive(&b_full[j & 1]);
      w.next();
      if (w.bd < static_cast<uint32_t>(a.bands))
        load_tile(w.bd, static_cast<int64_t>(w.lb) * kRL, static_cast<int64_t>(w.pb) * kRM);
      b2 = b1;
      l2 = l1;
      p2 = p1;
      b1 = bd;
      l1 = l0;
      p1 = p0;
    }
    if (ok && j >= 2) ok = epilogue(j - 2, b2, l2, p2);
    if (ok && j >= 1) epilogue(j - 1, b1, l1, p1);
  }
  __syncwarp();
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    tc_fence_after();
    tmem_dealloc(tmem, kRTmemCols);
  }
}

// ======================================================================
// Pass 2: columns.  DT: the raster's dtype (centre validity).
// ======================================================================
template <int DT>
__global__ void __launch_bounds__(kGThreads, 1) gauss_col_kernel(const GaussArgs a, uint32_t* err_word) {
  extern __shared__ unsigned char g_raw[];
  __shared__ __align__(8) uint64_t a_full[2], a_empty[2], acc_full[2], acc_empty[2], drain_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(g_raw) + 1023) & ~uintptr_t(1023));
  const GaussGeom g = gauss_geom(a.k, 2);
  const GaussPlan L = gauss_plan(g);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t npb = static_cast<uint32_t>((a.len + kGN - 1) / kGN);
  const uint32_t nlb = static_cast<uint32_t>((a.lines + kGL - 1) / kGL);
  const int64_t total = static_cast<int64_t>(npb) * nlb * a.bands;
  const uint32_t s_base = smem_u32(sm);

  // ---- set-up: load the Toeplitz bands, initialise the barriers, allocate
  // tensor memory (two buffers of hi*hi | correction accumulators, 64
  // columns each)
  for (int i = tid; i < g.NB * 16; i += kGThreads)  // 2 bands x NB x 128 B in 16-byte pieces
    reinterpret_cast<uint4*>(sm + L.band)[i] = __ldg(reinterpret_cast<const uint4*>(a.band) + i);
  if (tid == 0) {
    abort_flag = 0;
    for (int i = 0; i < 2; ++i) {
      mbar_init(&a_full[i], 1);
      mbar_init(&a_empty[i], 1);
      mbar_init(&acc_full[i], 1);
      mbar_init(&acc_empty[i], kGConv);
    }
    mbar_init(&drain_bar, 1);
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(&tmem_slot, 256);
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == 0) {
    // ========================================================= MMA issuer
    if (lane == 0) {
      const uint32_t a_ks = (2 * L.lbo) >> 4;  // one k-step = two core matrices along K
      const uint32_t bh0 = desc_lo(s_base + L.band, 128);
      const uint32_t bl0 = desc_lo(s_base + L.band + static_cast<uint32_t>(g.NB) * 128, 128);
      int j = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < total; t += gridDim.x, ++j) {
        const int b = j & 1;
        ok = wait_or_abort(&a_full[b], (j >> 1) & 1, &abort_flag, err_word, kDevErrMmaTimeout);
        if (ok && j >= 2) ok = wait_or_abort(&acc_empty[b], ((j >> 1) - 1) & 1, &abort_flag, err_word, kDevErrMmaTimeout);
        if (!ok) break;
        tc_fence_after();
        uint32_t ah = desc_lo(s_base + 2 * b * L.a_bytes, L.lbo);
        uint32_t al = desc_lo(s_base + (2 * b + 1) * L.a_bytes, L.lbo);
        uint32_t bh = bh0, bl = bl0;
        const uint32_t t_hh = tmem + b * 2 * kGN, t_cr = t_hh + kGN;
#pragma unroll 1
        for (int ks = 0; ks < g.KS; ++ks) {
          mma_f16(t_hh, ah, bh, ks != 0);
          mma_f16(t_cr, ah, bl, ks != 0);
          mma_f16(t_cr, al, bh, 1u);
          ah += a_ks;
          al += a_ks;
          bh += 16;
          bl += 16;
        }
        mma_commit(&a_empty[b]);
        mma_commit(&acc_full[b]);
      }
      if (!ok) {
        // MMAs already issued must finish before tensor memory is released
        mma_commit(&drain_bar);
        mbar_wait_bounded(&drain_bar, 0, err_word, kDevErrMmaTimeout);
      }
    }
  } else if (warp == 1) {
    // ========================================================= window copies
    if (lane == 0) {
      const uint32_t bytes = static_cast<uint32_t>(g.KC) * kGChunk;
      TileWalk w;
      w.init(npb, nlb);
      int j = 0;
      bool ok = true;
      for (; w.bd < static_cast<uint32_t>(a.bands); w.next(), ++j) {
        const int b = j & 1;
        if (j >= 2) {
          ok = wait_or_abort(&a_empty[b], ((j >> 1) - 1) & 1, &abort_flag, err_word, kDevErrTmaTimeout);
          if (!ok) break;
        }
        // chunks p0/8 .. p0/8 + KC - 1 of line block lb, stored in descending order
        const size_t off = w.bd * a.plane_bstride +
                           (static_cast<size_t>(w.lb) * a.np + (a.np - g.KC - static_cast<int64_t>(w.pb) * (kGN / 8))) * kGChunk;
        mbar_arrive_expect_tx(&a_full[b], 2 * bytes);
        bulk_g2s(sm + 2 * b * L.a_bytes, a.chi + off, bytes, &a_full[b]);
        bulk_g2s(sm + (2 * b + 1) * L.a_bytes, a.clo + off, bytes, &a_full[b]);
      }
      if (!ok) {
        // the copies in flight must land before shared memory is released
        for (int jj = (j >= 2 ? j - 2 : 0); jj < j; ++jj)
          mbar_wait_bounded(&a_full[jj & 1], (jj >> 1) & 1, err_word, kDevErrTmaTimeout);
      }
    }
  } else {
    // ========================================================= centre copies + epilogue
    const int ct = tid - 64;           // thread 0..255
    const int quarter = warp & 3;      // the TMEM lane quarter this warp may read
    const int part = (warp - 2) >> 2;  // epilogue: positions kGPosPart part .. + kGPosPart - 1
    const bool nd_val = a.nd_kind == VSR_NODATA_VALUE;
    constexpr int kEsz = DT == VSR_U8 ? 1 : 2;  // raster element bytes

    // a tile's centre pixels (raster rows p0 .. p0+63, columns l0 .. l0+63)
    // copied with cp.async into centre buffer cb: 64 rows x 128 bytes,
    // 8-byte pieces spread over the threads (zero-filled outside the
    // raster); read after the copier's wait and a barrier.
    constexpr int kCenPieces = kGL * kEsz / 8;  // 8-byte pieces per row
    auto copy_centres = [&](int cb, int64_t bd, int64_t l0, int64_t p0) {
#pragma unroll
      for (int k2 = ct; k2 < kGN * kCenPieces; k2 += kGConv) {
        const int row = k2 / kCenPieces, pc = k2 - row * kCenPieces;
        const int64_t y = p0 + row, xb = l0 + pc * (8 / kEsz);
        const int64_t nin = a.lines - xb > 8 / kEsz ? 8 / kEsz : (a.lines - xb > 0 ? a.lines - xb : 0);
        const bool in = y < a.len && nin > 0;
        const void* gp =
            in ? static_cast<const void*>(static_cast<const char*>(a.raster) + (bd * a.src_bstride + y * a.r_pitch + xb) * kEsz)
               : a.raster;
        cp_async_zfill<8>(sm + L.raw + (static_cast<uint32_t>(cb) * kGN + row) * 128 + pc * 8, gp,
                          in ? static_cast<uint32_t>(nin * kEsz) : 0u);
      }
    };
    const int i2 = ct & (kGL - 1);
    auto centre = [&](int cb, int row, int col) -> int {
      const unsigned char* rp = sm + L.raw + (static_cast<uint32_t>(cb) * kGN + row) * 128;
      if (DT == VSR_U8) return rp[col];
      if (DT == VSR_I16) return reinterpret_cast<const int16_t*>(rp)[col];
      return reinterpret_cast<const uint16_t*>(rp)[col];
    };

    // Tile jj's sums: hi*hi + corrections per TMEM lane (row m: the
    // numerator of line m, or the weight sum of line m - 64) and this
    // warp's 32 positions; cb: its centre buffer.
    auto epilogue = [&](int jj, int64_t bd, int64_t l0, int64_t p0, int cb) -> bool {
      const int b = jj & 1;
      const int64_t x2 = l0 + i2;
      // one thread waits for the accumulators; the barrier-reduction orders
      // the others after it -- and after their reads of the previous tile's
      // exchange -- and shares a failed wait
      bool got = true;
      if (ct == 0) got = wait_or_abort(&acc_full[b], (jj >> 1) & 1, &abort_flag, err_word, kDevErrMmaTimeout);
      if (g_any<kGConv>(!got)) return false;
      tc_fence_after();
      const int m = quarter * 32 + lane;
      const uint32_t lane_base = tmem + b * 2 * kGN + (static_cast<uint32_t>(quarter * 32) << 16) + part * kGPosPart;
      float* xs = reinterpret_cast<float*>(sm + L.xch);
#pragma unroll
      for (int h16 = 0; h16 < kGPosPart / 16; ++h16) {
        uint32_t ra_[16], rb_[16];
        tmem_ld16_issue(lane_base + 16 * h16, ra_);
        tmem_ld16_issue(lane_base + kGN + 16 * h16, rb_);
        tmem_wait_ld16(ra_);
        tmem_wait_ld16(rb_);
#pragma unroll
        for (int n = 0; n < 16; n += 2) {
          const float2 sum = __fadd2_rn(make_float2(__uint_as_float(ra_[n]), __uint_as_float(ra_[n + 1])),
                                        make_float2(__uint_as_float(rb_[n]), __uint_as_float(rb_[n + 1])));
          xs[m * kGXPitch + part * kGPosPart + 16 * h16 + n] = sum.x;
          xs[m * kGXPitch + part * kGPosPart + 16 * h16 + n + 1] = sum.y;
        }
      }
      tc_fence_before();
      mbar_arrive(&acc_empty[b]);  // the accumulators may be reused
      cp_async_wait<2>();          // this thread's centre copies of this tile have landed
      g_sync<kGConv>();
      // output: thread ct takes line i2 (raster column x2) and positions
      // (rows) ct / 64 + kGRowStep q; a warp's lanes are 32 consecutive x
      // quotient: __fdividef (within 2 ulp; den <= 2^20 here, far below
      // its 2^126 limit), exact power-of-two rescale
      if (x2 < a.lines) {
        const int64_t y0 = p0 + (ct >> 6);
        const int64_t nrem = (a.len - y0 + kGRowStep - 1) / kGRowStep;  // rows y0 + kGRowStep q inside the raster
        const int nq = nrem < kGN / kGRowStep ? static_cast<int>(nrem) : kGN / kGRowStep;
        if (a.out_dtype == VSR_F64) {
          double* op = static_cast<double*>(a.dst) + bd * a.out_bstride + y0 * a.out_pitch + x2;
#pragma unroll
          for (int q = 0; q < kGN / kGRowStep; ++q, op += kGRowStep * a.out_pitch) {
            if (q >= nq) break;
            const int p = (ct >> 6) + kGRowStep * q;
            const float num = xs[i2 * kGXPitch + p], den = xs[(kGL + i2) * kGXPitch + p];
            const bool ok = !(nd_val && centre(cb, p, i2) == a.nd_iv) && den > 0.0f;
            *op = ok ? static_cast<double>(__fdividef(num, den) * (kGScaleD / kGScaleV)) : a.nd_out;
          }
        } else {
          float* op = static_cast<float*>(a.dst) + bd * a.out_bstride + y0 * a.out_pitch + x2;
          const float ndf = static_cast<float>(a.nd_out);
#pragma unroll
          for (int q = 0; q < kGN / kGRowStep; ++q, op += kGRowStep * a.out_pitch) {
            if (q >= nq) break;
            const int p = (ct >> 6) + kGRowStep * q;
            const float num = xs[i2 * kGXPitch + p], den = xs[(kGL + i2) * kGXPitch + p];
            const bool ok = !(nd_val && centre(cb, p, i2) == a.nd_iv) && den > 0.0f;
            *op = ok ? __fdividef(num, den) * (kGScaleD / kGScaleV) : ndf;
          }
        }
      }
      return true;
    };

    // Per tile j: tile j's centre copies are issued, then tile j-2's
    // epilogue runs.  One cp.async group per iteration.
    TileWalk w;
    w.init(npb, nlb);
    int j = 0;
    bool ok = true;
    int64_t b1 = 0, l1 = 0, p1 = 0, b2 = 0, l2 = 0, p2 = 0;  // band / first line / position of tiles j-1, j-2
    for (; w.bd < static_cast<uint32_t>(a.bands); w.next(), ++j) {
      const int64_t bd = w.bd, l0 = static_cast<int64_t>(w.lb) * kGL, p0 = static_cast<int64_t>(w.pb) * kGN;
      copy_centres(j % kGCenBufs, bd, l0, p0);
      cp_async_commit();
      if (j >= 2 && !epilogue(j - 2, b2, l2, p2, (j - 2) % kGCenBufs)) {
        ok = false;
        break;
      }
      b2 = b1;
      l2 = l1;
      p2 = p1;
      b1 = bd;
      l1 = l0;
      p1 = p0;
    }
    // the last two epilogues; one empty cp.async group per call keeps the
    // wait count (at most 2 newer groups) right
    if (ok && j >= 2) {
      cp_async_commit();
      ok = epilogue(j - 2, b2, l2, p2, (j - 2) % kGCenBufs);
    }
    if (ok && j >= 1) {
      cp_async_commit();
      epilogue(j - 1, b1, l1, p1, (j - 1) % kGCenBufs);
    }
    cp_async_wait<0>();
  }
  __syncwarp();
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    tc_fence_after();
    tmem_dealloc(tmem, 256);
  }
}

// Toeplitz band of the normalised 1-D Gaussian g_i = exp(-0.5 ((i - k/2) /
// sigma)^2) / sum (float64) times 2^12, shifted by s positions (windows
// start ra = r + s before the output), split g = f16(g) + f16(g - f16(g)):
// core matrix c, row rr, element e -> g[Kp-1-8c-e-rr-s] (0 outside [0, k));
// the hi band's NB core matrices, then the lo band's.
__global__ void prep_gauss_band(int k, double sigma, int Kp, int NB, int s, uint16_t* __restrict__ img) {
  __shared__ double g64[kGMaxK];
  __shared__ double tot;
  for (int i = threadIdx.x; i < k; i += blockDim.x) {
    const double t = (i - k / 2) / sigma;
    g64[i] = exp(-0.5 * t * t);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double acc = 0.0;
    for (int i = 0; i < k; ++i) acc += g64[i];
    tot = acc;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < NB * 64; i += blockDim.x) {
    const int c = i / 64, rr = (i / 8) & 7, e = i & 7;
    const int kx = Kp - 1 - 8 * c - e - rr - s;
    const double w = (kx >= 0 && kx < k) ? g64[kx] / tot * kGScaleW : 0.0;
    const __half hi = __float2half_rn(static_cast<float>(w));
    const __half lo = __float2half_rn(static_cast<float>(w - static_cast<double>(__half2float(hi))));
    img[i] = __half_as_ushort(hi);
    img[NB * 64 + i] = __half_as_ushort(lo);
  }
}

template <int DT>
int launch_gauss_tc(const GaussArgs& p1, const GaussArgs& p2, uint32_t* err, cudaStream_t st) {
  auto k1 = gauss_row_kernel<DT>;
  auto k2 = gauss_col_kernel<DT>;
  const size_t s1 = row_plan(gauss_geom(p1.k, 1)).total + 1024, s2 = gauss_plan(gauss_geom(p2.k, 2)).total + 1024;
  VSR_CUDA_TRY(cudaFuncSetAttribute(k1, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(s1)));
  VSR_CUDA_TRY(cudaFuncSetAttribute(k2, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(s2)));
  const int64_t t1 = ((p1.lines + kRL - 1) / kRL) * ((p1.len + kRM - 1) / kRM) * p1.bands;
  const int64_t t2 = ((p2.lines + kGL - 1) / kGL) * ((p2.len + kGN - 1) / kGN) * p2.bands;
  if (t1 >= (int64_t(1) << 31) || t2 >= (int64_t(1) << 31))
    return fail(VSR_ERR_UNSUPPORTED, "tensor-core Gaussian: more than 2^31 tiles in one launch");
  k1<<<static_cast<unsigned>(std::min<int64_t>(t1, sm_count())), kRThreads, s1, st>>>(p1, err);
  VSR_CUDA_TRY(cudaGetLastError());
  k2<<<static_cast<unsigned>(std::min<int64_t>(t2, sm_count())), kGThreads, s2, st>>>(p2, err);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}

size_t chunk_plane_bytes(int64_t H, int64_t W, const GaussGeom& g) {
  return static_cast<size_t>((W + kGL - 1) / kGL) * gauss_np(H, g) * kGChunk;
}

}  // namespace

int gauss_tc_supported(int dtype, int k) {
  return (dtype == VSR_U8 || dtype == VSR_I16 || dtype == VSR_U16) && k >= 1 && k <= kGMaxK;
}

namespace {
// The kernels copy raster rows in 4- and 8-byte pieces: the band's base and
// rows must be 8-byte aligned, else the band is first copied to an aligned
// pitch in the workspace.
bool gauss_tc_aligned(const void* band, int64_t pitch, int64_t esz) {
  return aligned(band, 8) && (pitch * esz) % 8 == 0;
}
int64_t gauss_aligned_pitch(int64_t W, int64_t esz) { return (W * esz + 7) / 8 * 8 / esz; }
}  // namespace

// Workspace: pass-2 band image | pass-1 band image | an aligned copy of one raster band (used when the
// caller's rows are not 8-byte aligned) | hi chunk planes of a group of
// bands | lo chunk planes of the group.  A workspace with room for the
// planes of every band runs the whole stack in one launch per pass; a
// smaller one runs the bands in groups (down to one band per launch pair).
size_t gauss_tc_workspace_bands(int64_t H, int64_t W, int dtype, int k, int bands) {
  const GaussGeom g = gauss_geom(k), g1 = gauss_geom(k, 1);
  const int64_t esz = dtype == VSR_U8 ? 1 : 2;
  const size_t band = ((static_cast<size_t>(2) * g.NB * 128 + 255) & ~size_t(255)) +
                      ((static_cast<size_t>(2) * g1.NB * 128 + 255) & ~size_t(255));
  const size_t copy = (static_cast<size_t>(H) * gauss_aligned_pitch(W, esz) * esz + 255) & ~size_t(255);
  return band + copy + 2 * static_cast<size_t>(bands) * chunk_plane_bytes(H, W, g);
}

size_t gauss_tc_workspace(int64_t H, int64_t W, int dtype, int k) { return gauss_tc_workspace_bands(H, W, dtype, k, 1); }

int run_gauss_tc(const void* src, int dtype, int bands, int64_t band_stride, int64_t H, int64_t W, int64_t pitch,
                 double sigma, int k, double nodata, int nodata_kind, void* dst, int out_dtype,
                 int64_t out_band_stride, int64_t out_pitch, void* workspace, size_t ws_bytes, cudaStream_t st) {
  if (!gauss_tc_supported(dtype, k))
    return fail(VSR_ERR_UNSUPPORTED, "split-precision tensor-core Gaussian reads 8/16-bit integer rasters with kernels up to %d", kGMaxK);
  const size_t need = gauss_tc_workspace(H, W, dtype, k);
  if (!workspace || ws_bytes < need || !aligned(workspace, 256))
    return fail(VSR_ERR_WORKSPACE, "workspace must be 256-byte aligned and >= %zu bytes", need);
  const GaussGeom g = gauss_geom(k), g1 = gauss_geom(k, 1);
  const int64_t np = gauss_np(H, g);
  const int64_t nx = (W + kGL - 1) / kGL;
  const size_t esz = dtype == VSR_U8 ? 1 : 2;
  const size_t osz = out_dtype == VSR_F64 ? 8 : 4;
  const int64_t apitch = gauss_aligned_pitch(W, static_cast<int64_t>(esz));
  char* ws = static_cast<char*>(workspace);
  uint16_t* band = reinterpret_cast<uint16_t*>(ws);
  const size_t off_band1 = (static_cast<size_t>(2) * g.NB * 128 + 255) & ~size_t(255);
  uint16_t* band1 = reinterpret_cast<uint16_t*>(ws + off_band1);
  const size_t off_copy = off_band1 + ((static_cast<size_t>(2) * g1.NB * 128 + 255) & ~size_t(255));
  const size_t off_planes = off_copy + ((static_cast<size_t>(H) * apitch * esz + 255) & ~size_t(255));
  void* acopy = ws + off_copy;
  const size_t plane = chunk_plane_bytes(H, W, g);
  // bands per launch pair: as many as the workspace holds planes for, when
  // every band's rows are 8-byte aligned; else one band at a time (each
  // copied to an aligned pitch when its own rows are not)
  const bool all_aligned = gauss_tc_aligned(src, pitch, static_cast<int64_t>(esz)) &&
                           (bands == 1 || (band_stride * static_cast<int64_t>(esz)) % 8 == 0);
  const int64_t fit = static_cast<int64_t>((ws_bytes - off_planes) / (2 * plane));
  const int group = all_aligned ? static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(bands, fit))) : 1;
  unsigned char* chi = reinterpret_cast<unsigned char*>(ws + off_planes);
  unsigned char* clo = chi + static_cast<size_t>(group) * plane;
  double ndv = 0.0;
  const int kind = resolve_nodata(dtype, nodata, nodata_kind, &ndv);
  uint32_t* err = device_error_word();
  if (!err) return VSR_ERR_CUDA;
  prep_gauss_band<<<1, 256, 0, st>>>(k, sigma, g.Kp, g.NB, g.s, band);
  VSR_CUDA_TRY(cudaGetLastError());
  prep_gauss_band<<<1, 256, 0, st>>>(k, sigma, g1.Kp, g1.NB, g1.s, band1);
  VSR_CUDA_TRY(cudaGetLastError());
  // zero chunks: the padded positions before row 0 (the last ra/8 chunks of
  // each line block) and from round8(H) on (the first chunks); pass 1
  // writes every other chunk's rows of lines < W.  The group's planes are
  // consecutive line blocks of np chunks each.
  const int64_t lead = g.ra / 8, tail = np - (g.ra + ((H + 7) & ~int64_t(7))) / 8;
  for (unsigned char* pl : {chi, clo}) {
    VSR_CUDA_TRY(cudaMemset2DAsync(pl + (np - lead) * kGChunk, np * kGChunk, 0, lead * kGChunk, nx * group, st));
    if (tail > 0) VSR_CUDA_TRY(cudaMemset2DAsync(pl, np * kGChunk, 0, tail * kGChunk, nx * group, st));
  }
  for (int b0 = 0; b0 < bands; b0 += group) {
    const int nb = std::min(group, bands - b0);
    const void* bsrc = static_cast<const char*>(src) + static_cast<size_t>(b0) * band_stride * esz;
    void* bdst = static_cast<char*>(dst) + static_cast<size_t>(b0) * out_band_stride * osz;
    int64_t bp = pitch;
    if (!gauss_tc_aligned(bsrc, pitch, static_cast<int64_t>(esz))) {  // group == 1 here
      VSR_CUDA_TRY(cudaMemcpy2DAsync(acopy, apitch * esz, bsrc, pitch * esz, W * esz, H, cudaMemcpyDeviceToDevice, st));
      bsrc = acopy;
      bp = apitch;
    }
    const int64_t sb = nb > 1 ? band_stride : 0, ob = nb > 1 ? out_band_stride : 0;
    GaussArgs p1{bsrc, H, W, bp, chi, clo, np, nullptr, 0, kind, static_cast<int64_t>(ndv),
                 nullptr, out_dtype, out_pitch, nodata, band1, k, nb, sb, plane, 0};
    GaussArgs p2{nullptr, W, H, 0, chi, clo, np, bsrc, bp, kind, static_cast<int64_t>(ndv),
                 bdst, out_dtype, out_pitch, nodata, band, k, nb, sb, plane, ob};
    int rc = dtype == VSR_U8 ? launch_gauss_tc<VSR_U8>(p1, p2, err, st)
             : dtype == VSR_I16 ? launch_gauss_tc<VSR_I16>(p1, p2, err, st)
                                : launch_gauss_tc<VSR_U16>(p1, p2, err, st);
    if (rc) return rc;
  }
  return VSR_OK;
}

}  // namespace vsr
