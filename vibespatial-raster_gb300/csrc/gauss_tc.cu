// Separable split-precision Gaussian on the tcgen05 tensor cores: two line passes.
//
// The reference's k x k Gaussian weights outer(g, g) / sum (algebra.py:2120-2152,
// applied as the normalised convolution of kernels/focal.py:101-145) factor
// into a pass along the rows and one along the columns.  Each is a 1-D
// normalised convolution of "lines",
//   num(l, p) = sum_j g[j] a_num(l, p - r + j),  den(l, p) = sum_j g[j] a_den(l, p - r + j),
// computed as a GEMM against the Toeplitz band of g:
//   D[m][n] = sum_k A[m][k] B[k][n],  A = the tile's line windows, B[k][n] = g[k - n],
// with the K-reversed operand layouts of the 2-D kernel (conv_tc.cu) for one
// kernel row: A rows 16 bytes apart (SBO = 128 B; core-matrix columns
// 129 x 16 B apart in pass 1, 2 KB apart in pass 2), the band with
// SBO = LBO = 128 B.
//
// Tile: 64 lines x 64 positions.  The MMA's M = 128 rows stack the tile's
// numerator operand (rows 0-63) over its weight-sum operand (rows 64-127),
// so one k-step is three MMAs for both sums: hi*hi into one accumulator and
// the corrections hi*lo + lo*hi into another; the two are added in FP32
// registers.
//
// Operands are split into FP16 hi/lo pairs, a = a_hi + a_lo, g = g_hi + g_lo
// (kind::f16 with F16 inputs, FP32 accumulation).  An F16 pair carries 22
// significant bits, a BF16 pair only 16: pass 2's inputs are float32 sums,
// and with BF16 pairs their split residuals (up to 2^-16 relative) left
// ~5e-6 relative error in the output; with F16 pairs the residuals and the
// dropped lo*lo products are ~2^-22.  Power-of-two scales keep every operand
// in F16's normal range and cancel exactly in the quotient: values x 1/2
// (|v| <= 32768), weights x 2^12 (the 4-sigma tails stay normal), the row
// pass's weight sums x 2^8.
//  * pass 1 (lines = raster rows, positions = columns) reads an 8/16-bit
//    integer raster: a_num = v/2 * valid, exact as an F16 pair (16 significant
//    bits), and a_den = valid (0/1, exact: its lo rows stay zero), converted
//    by the converter warps into the A layout.  Its epilogue writes the row
//    sums P_num = sum g v/2 and P_den = 2^8 sum g valid already split into
//    F16 hi/lo, transposed (pass-2 line = raster column x, position = row y)
//    and in pass 2's A layout: per 64-line block, 2 KB chunks of 8 positions
//    (numerator rows of the block's lines, then weight-sum rows, 16 bytes
//    each, positions reversed inside a row), chunks in descending position
//    order -- so a pass-2 tile's window is one contiguous run per plane.
//  * pass 2 (lines = columns, positions = rows) copies each tile's window of
//    the two planes into shared memory with cp.async.bulk (no conversion)
//    and writes out[y][x] = 2^9 num / den where the centre pixel is valid and
//    den > 0, else the nodata value.
// Windows start at p0 - ra, ra = r rounded up to 8 (aligned chunks and
// loads); the band is shifted by s = ra - r to match.
//
// Roles per persistent CTA (one per SM): warp 0 issues the MMAs; warp 1
// (pass 2) bulk-copies the A windows in; warps 2-9 (pass 1) copy each tile's
// raster window a tile ahead with cp.async into thread-private staging and
// convert it into an A buffer, and run the epilogue two tiles behind the
// conversion, so tile j-1's MMAs overlap tile j's conversion: tcgen05.ld,
// then pass 1 stages its output chunks in shared memory for cp.async.bulk
// stores and pass 2 exchanges numerator and weight sum through shared memory
// and writes the quotients (its centre pixels copied a tile ahead).  A
// buffers and TMEM accumulators are double-buffered and handed over through
// mbarriers; every wait is bounded (on expiry an error bit is recorded, a
// shared abort flag ends the other roles' waits, and the MMA issuer and the
// copy producer wait for their operations in flight before the CTA frees
// tensor memory).
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

constexpr int kGL = kMmaM / 2;        // lines per tile
constexpr int kGN = kMmaN;            // positions per tile (MMA N)
constexpr int kGWarps = 8;            // converter / epilogue warps (warps 2..9)
constexpr int kGConv = 32 * kGWarps;  // converter threads
constexpr int kGThreads = 64 + kGConv;
constexpr int kGRp = kMmaM | 1;       // pass-1 A: 16-byte rows between core-matrix columns (odd: conflict-free stores)
constexpr uint32_t kGChunk = kMmaM * 16;  // pass-2 A: one 8-position core-matrix column of 128 rows (2 KB)
constexpr uint32_t kGStgChunk = kGChunk + 16;  // pass-1 staging chunk stride (conflict-free 2-byte stores)
constexpr int kGMaxK = 79;
constexpr int kGXPitch = kGN + 1;     // pass-2 exchange rows (floats; odd: conflict-free)
constexpr int kGLinesPerWarp = kGL / kGWarps;
constexpr float kGScaleV = 0.5f;       // pass-1 values
constexpr double kGScaleW = 4096.0;    // weights
constexpr float kGScaleD = 256.0f;     // the row pass's weight sums
constexpr uint32_t kF16One = 0x3c00u;  // 1.0 in F16
// Pass-2 centre buffers: tile t's are copied at the start of iteration t and
// read in its epilogue (iteration t + 2) up to the barrier opening iteration
// t + 3's epilogue, so a buffer is rewritten four tiles later at the earliest.
constexpr int kGCenBufs = 4;

struct GaussGeom {
  int k, r;
  int ra;    // window lead: r rounded up to 8
  int s;     // band shift ra - r
  int KW;    // window positions per tile: kGN + k - 1 + s
  int Kp;    // GEMM K: KW rounded up to 16
  int KC;    // Kp / 8 core-matrix columns
  int KS;    // Kp / 16 k-steps
  int NB;    // core matrices of the Toeplitz band: KC + kGN/8 - 1
  int ngrp;  // 4-position groups covering KW (lane l takes groups l, l + 32, ...)
};

__host__ __device__ inline GaussGeom gauss_geom(int k) {
  GaussGeom g;
  g.k = k;
  g.r = k / 2;
  g.ra = (g.r + 7) & ~7;
  g.s = g.ra - g.r;
  g.KW = kGN + k - 1 + g.s;
  g.Kp = (g.KW + 15) & ~15;
  g.KC = g.Kp / 8;
  g.KS = g.Kp / 16;
  g.NB = g.KC + kGN / 8 - 1;
  g.ngrp = (g.KW + 3) / 4;
  return g;
}

// Pass-2 chunk planes: per 64-line block, np chunks of 2 KB.
__host__ __device__ inline int64_t gauss_np(int64_t H, const GaussGeom& g) {
  return ((H + kGN - 1) / kGN * kGN - kGN + g.Kp) / 8;
}

struct GaussPlan {  // shared-memory byte offsets from the 1024-aligned base
  uint32_t a_bytes;  // one operand plane
  uint32_t lbo;      // its core-matrix column stride
  uint32_t band;     // hi band, then lo band (NB x 128 B each); buffer b: hi plane at 2 b a_bytes, lo after it
  uint32_t xch;      // pass 2: 128 x kGXPitch floats (numerator rows over weight-sum rows);
                     // pass 1: the output staging, hi then lo, 8 chunks of kGStgChunk bytes each
  uint32_t raw;      // pass 1: 2 buffers x 64 rows x ngrp groups x 8 B of raw raster values;
                     // pass 2: kGCenBufs buffers x 64 rows x 128 B of centre pixels
  uint32_t total;
};

__host__ __device__ inline GaussPlan gauss_plan(const GaussGeom& g, int pass) {
  GaussPlan p;
  p.lbo = pass == 1 ? kGRp * 16 : kGChunk;
  p.a_bytes = (static_cast<uint32_t>(g.KC) * p.lbo + 127) & ~127u;
  p.band = 4 * p.a_bytes;
  p.xch = p.band + 2 * static_cast<uint32_t>(g.NB) * 128;
  p.raw = p.xch + (pass == 2 ? static_cast<uint32_t>(kMmaM) * kGXPitch * 4 : 2 * (kGL / 8) * kGStgChunk);
  p.total = p.raw + (pass == 1 ? 2u * kGL * g.ngrp * 8 : static_cast<uint32_t>(kGCenBufs) * kGL * 128);
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
  const uint16_t* band;  // hi band then lo band
  int k;
  int bands;             // band-first stack, tiles band-major
  int64_t src_bstride;   // elements between raster bands (pass 1 src, pass 2 raster)
  size_t plane_bstride;  // bytes between the chunk planes of consecutive bands
  int64_t out_bstride;   // elements between output bands (pass 2)
};

// Named barrier 1 over the converter warps; g_any also ORs a predicate.
__device__ __forceinline__ void g_sync() { asm volatile("bar.sync 1, %0;" ::"n"(kGConv) : "memory"); }

__device__ __forceinline__ bool g_any(bool p) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred q, o;\n\t"
      "setp.ne.u32 q, %1, 0;\n\t"
      "bar.red.or.pred o, 1, %2, q;\n\t"
      "selp.u32 %0, 1, 0, o;\n\t}"
      : "=r"(r)
      : "r"(static_cast<uint32_t>(p)), "n"(kGConv)
      : "memory");
  return r != 0;
}

// Four window values (positions 4 grp .. 4 grp + 3) as the 8-byte segments
// of one K-reversed A row, split z = hi + lo in F16: element klo holds
// position 4 grp + 3.
__device__ __forceinline__ void split4(const float z[4], uint2& hi, uint2& lo) {
  const __half2 h32 = __floats2half2_rn(z[3], z[2]);
  const __half2 h10 = __floats2half2_rn(z[1], z[0]);
  const __half2 l32 = __floats2half2_rn(z[3] - __low2float(h32), z[2] - __high2float(h32));
  const __half2 l10 = __floats2half2_rn(z[1] - __low2float(h10), z[0] - __high2float(h10));
  hi = make_uint2(f16x2_bits(h32), f16x2_bits(h10));
  lo = make_uint2(f16x2_bits(l32), f16x2_bits(l10));
}

// PASS 1 or 2; DT: the raster's dtype (VSR_U8, VSR_I16, VSR_U16).
template <int PASS, int DT>
__global__ void __launch_bounds__(kGThreads, 1) gauss_line_kernel(const GaussArgs a, uint32_t* err_word) {
  extern __shared__ unsigned char g_raw[];
  __shared__ __align__(8) uint64_t a_full[2], a_empty[2], acc_full[2], acc_empty[2], drain_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(g_raw) + 1023) & ~uintptr_t(1023));
  const GaussGeom g = gauss_geom(a.k);
  const GaussPlan L = gauss_plan(g, PASS);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t npb = (a.len + kGN - 1) / kGN;
  const int64_t per_band = npb * ((a.lines + kGL - 1) / kGL);
  const int64_t total = per_band * a.bands;
  const uint32_t s_base = smem_u32(sm);
  // tile t -> band, first line l0 and first position p0 (band-major order)
  auto tile_of = [&](int64_t t, int64_t& bd, int64_t& l0, int64_t& p0) {
    bd = t / per_band;
    const int64_t rem = t - bd * per_band, lb = rem / npb;
    l0 = lb * kGL;
    p0 = (rem - lb * npb) * kGN;
  };

  // ---- set-up: zero the A planes (pass 1: the K padding and the lo rows of
  // the weight-sum operand stay zero for good), load the Toeplitz bands,
  // initialise the barriers, allocate tensor memory (two buffers of hi*hi |
  // correction accumulators, 64 columns each)
  if (PASS == 1)
    for (uint32_t i = tid * 16; i < L.band; i += kGThreads * 16)
      *reinterpret_cast<uint4*>(sm + i) = make_uint4(0u, 0u, 0u, 0u);
  for (int i = tid; i < g.NB * 16; i += kGThreads)  // 2 bands x NB x 128 B in 16-byte pieces
    reinterpret_cast<uint4*>(sm + L.band)[i] = __ldg(reinterpret_cast<const uint4*>(a.band) + i);
  if (tid == 0) {
    abort_flag = 0;
    for (int i = 0; i < 2; ++i) {
      mbar_init(&a_full[i], PASS == 1 ? kGConv : 1);
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
    // ========================================================= pass 2: window copies
    if (PASS == 2 && lane == 0) {
      const uint32_t bytes = static_cast<uint32_t>(g.KC) * kGChunk;
      int j = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < total; t += gridDim.x, ++j) {
        const int b = j & 1;
        if (j >= 2) {
          ok = wait_or_abort(&a_empty[b], ((j >> 1) - 1) & 1, &abort_flag, err_word, kDevErrTmaTimeout);
          if (!ok) break;
        }
        int64_t bd, l0, p0;
        tile_of(t, bd, l0, p0);
        // chunks p0/8 .. p0/8 + KC - 1 of line block l0/64, stored in descending order
        const size_t off = bd * a.plane_bstride + (static_cast<size_t>(l0 / kGL) * a.np + (a.np - g.KC - p0 / 8)) * kGChunk;
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
    // ========================================================= converters + epilogue
    const int ct = tid - 64;           // converter thread 0..255
    const int cw = ct >> 5;            // converter warp 0..7: tile lines cw, cw + 8, ...
    const int quarter = warp & 3;      // the TMEM lane quarter this warp may read
    const int half = (warp - 2) >> 2;  // epilogue: positions 32 half .. +31
    const bool nd_val = a.nd_kind == VSR_NODATA_VALUE;

    constexpr int kEsz = DT == VSR_U8 ? 1 : 2;  // raster element bytes
    // pass 1: this thread's raw window values of a tile -- rows l0 + cw + 8 q,
    // columns p0 - ra + 4 grp .. + 3 (4 elements, one 4- or 8-byte copy;
    // zero-filled outside the raster) -- copied with cp.async into its own
    // staging slots a tile ahead; the thread converts exactly what it copied.
    auto raw_slot = [&](int rb, int q, int grp) {
      return sm + L.raw + ((static_cast<uint32_t>(rb) * kGL + cw + kGWarps * q) * g.ngrp + grp) * 8;
    };
    auto copy_rows = [&](int rb, int64_t bd, int64_t l0, int64_t p0) {
      const int rows = static_cast<int>(a.lines - l0 < kGL ? a.lines - l0 : kGL);  // tile rows inside the raster
      const int64_t rstep = kGWarps * a.pitch * kEsz;
      for (int grp = lane; grp < g.ngrp; grp += 32) {
        const int64_t xb = p0 - g.ra + 4 * grp;
        const int nin = xb < 0 ? 0 : static_cast<int>(a.len - xb > 4 ? 4 : (a.len - xb > 0 ? a.len - xb : 0));
        const char* gp = static_cast<const char*>(a.src) + (bd * a.src_bstride + (l0 + cw) * a.pitch + xb) * kEsz;
#pragma unroll
        for (int q = 0; q < kGLinesPerWarp; ++q, gp += rstep) {
          const bool in = cw + kGWarps * q < rows && nin > 0;
          cp_async_zfill<4 * kEsz>(raw_slot(rb, q, grp), in ? static_cast<const void*>(gp) : a.src,
                                   in ? static_cast<uint32_t>(nin * kEsz) : 0u);
        }
      }
    };
    // ... converted into the K-reversed A rows of buffer b (element klo =
    // Kp - 4 - 4 grp holds position 4 grp + 3): v/2 split into F16 hi/lo,
    // validity 0/1 (inside the raster and not nodata)
    auto convert_rows = [&](int rb, int b, int64_t l0, int64_t p0) {
      unsigned char* ahi = sm + 2 * b * L.a_bytes;
      unsigned char* alo = ahi + L.a_bytes;
      const int rows = static_cast<int>(a.lines - l0 < kGL ? a.lines - l0 : kGL);
      for (int grp = lane; grp < g.ngrp; grp += 32) {
        const int klo = g.Kp - 4 - 4 * grp;
        const uint32_t go = static_cast<uint32_t>(klo >> 3) * L.lbo + (klo & 7) * 2;
        const int64_t xb = p0 - g.ra + 4 * grp;
        uint32_t colm = 0;  // columns inside the raster
#pragma unroll
        for (int e = 0; e < 4; ++e) colm |= static_cast<uint32_t>(xb + e >= 0 && xb + e < a.len) << e;
#pragma unroll
        for (int q = 0; q < kGLinesPerWarp; ++q) {
          const int i = cw + kGWarps * q;
          if (i >= rows) continue;  // rows of lines past the raster are never stored
          int v[4];
          if (DT == VSR_U8) {
            const uint32_t w = *reinterpret_cast<const uint32_t*>(raw_slot(rb, q, grp));
#pragma unroll
            for (int e = 0; e < 4; ++e) v[e] = (w >> (8 * e)) & 0xFFu;
          } else {
            const uint2 w = *reinterpret_cast<const uint2*>(raw_slot(rb, q, grp));
            v[0] = w.x & 0xFFFFu;
            v[1] = w.x >> 16;
            v[2] = w.y & 0xFFFFu;
            v[3] = w.y >> 16;
            if (DT == VSR_I16) {
#pragma unroll
              for (int e = 0; e < 4; ++e) v[e] = static_cast<int16_t>(v[e]);
            }
          }
          float z[4];
          uint32_t okm = 0;
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const bool ok = ((colm >> e) & 1u) && !(nd_val && v[e] == a.nd_iv);
            z[e] = ok ? kGScaleV * static_cast<float>(v[e]) : 0.0f;
            okm |= static_cast<uint32_t>(ok) << e;
          }
          uint2 hi, lo;
          split4(z, hi, lo);
          *reinterpret_cast<uint2*>(ahi + go + i * 16) = hi;
          *reinterpret_cast<uint2*>(alo + go + i * 16) = lo;
          *reinterpret_cast<uint2*>(ahi + go + (kGL + i) * 16) =
              make_uint2(((okm & 8u) ? kF16One : 0u) | ((okm & 4u) ? kF16One << 16 : 0u),
                         ((okm & 2u) ? kF16One : 0u) | ((okm & 1u) ? kF16One << 16 : 0u));
        }
      }
    };

    // pass 2: a tile's centre pixels (raster rows p0 .. p0+63, columns
    // l0 .. l0+63) copied with cp.async into centre buffer cb: 64 rows x 128
    // bytes, 8-byte pieces spread over the threads (zero-filled outside the
    // raster); read after the copier's wait and a converter barrier.
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
    // warp's 32 positions; cb: its centre buffer (pass 2).
    auto epilogue = [&](int jj, int64_t bd, int64_t l0, int64_t p0, int cb) -> bool {
      const int b = jj & 1;
      const int64_t x2 = l0 + i2;
      // one thread waits for the accumulators (and, pass 1, for the previous
      // tile's output copies to have read the staging); the barrier-reduction
      // orders the others after it -- and after their reads of the previous
      // tile's exchange / staging -- and shares a failed wait
      bool got = true;
      if (PASS == 1 && ct < 16) bulk_wait_read<0>();  // this thread's chunk copy has read the staging
      if (ct == 0) got = wait_or_abort(&acc_full[b], (jj >> 1) & 1, &abort_flag, err_word, kDevErrMmaTimeout);
      if (g_any(!got)) return false;
      tc_fence_after();
      const int m = quarter * 32 + lane;
      const uint32_t lane_base = tmem + b * 2 * kGN + (static_cast<uint32_t>(quarter * 32) << 16) + half * 32;
      // this warp's 32 positions in two halves of 16: hi*hi + corrections
      auto sums16 = [&](int h16, float v[16]) {
        uint32_t ra_[16], rb_[16];
        tmem_ld16_issue(lane_base + 16 * h16, ra_);
        tmem_ld16_issue(lane_base + kGN + 16 * h16, rb_);
        tmem_wait_ld16(ra_);
        tmem_wait_ld16(rb_);
#pragma unroll
        for (int n = 0; n < 16; n += 2) {
          const float2 sum = __fadd2_rn(make_float2(__uint_as_float(ra_[n]), __uint_as_float(ra_[n + 1])),
                                        make_float2(__uint_as_float(rb_[n]), __uint_as_float(rb_[n + 1])));
          v[n] = sum.x;
          v[n + 1] = sum.y;
        }
      };
      if (PASS == 1) {
        // P_num = sum g v/2, P_den = 2^8 sum g valid (the weight scale
        // removed), split into F16 hi/lo in pass 2's A layout: the tile's
        // rows y = l0 .. l0+63 are the 8 chunks of padded positions
        // l0 + ra .. + 63 of line block p0/64, contiguous (descending) in
        // the planes.  They are staged in shared memory (row x mod 64 of the
        // numerator or weight-sum half, element 7 - yp % 8), then written by
        // one thread with bulk copies.  Rows y in [H, round8(H)) share the
        // last chunk: zeros there; lines x >= W: zeros.
        const int iy = m & (kGL - 1);
        const int64_t y = l0 + iy;
        unsigned char* stg = sm + L.xch;
        // chunk cl = 7 - iy / 8 of the tile (descending), element 7 - iy % 8
        const uint32_t o = (7 - iy / 8) * kGStgChunk + (m < kGL ? 0u : kGChunk / 2) + (7 - (iy & 7)) * 2;
        unsigned short* hrow = reinterpret_cast<unsigned short*>(stg + o);
        unsigned short* lrow = reinterpret_cast<unsigned short*>(stg + 8 * kGStgChunk + o);
        const float sc = m < kGL ? static_cast<float>(1.0 / kGScaleW) : static_cast<float>(kGScaleD / kGScaleW);
        const bool keep = y < a.lines;
        const int cols = static_cast<int>(a.len - p0 < kGN ? a.len - p0 : kGN);  // lines x inside the raster
#pragma unroll
        for (int h16 = 0; h16 < 2; ++h16) {
          float v[16];
          sums16(h16, v);
#pragma unroll
          for (int n = 0; n < 16; n += 2) {  // two lines (rows mx, mx + 1 of the chunk) at a time
            const int mx = half * 32 + 16 * h16 + n;
            const float2 z = __fmul2_rn(make_float2((keep && mx < cols) ? v[n] : 0.0f,
                                                    (keep && mx + 1 < cols) ? v[n + 1] : 0.0f),
                                        make_float2(sc, sc));
            const __half2 hv = __floats2half2_rn(z.x, z.y);
            const float2 rest = __fadd2_rn(z, make_float2(-__low2float(hv), -__high2float(hv)));
            const __half2 lv = __floats2half2_rn(rest.x, rest.y);
            hrow[mx * 8] = __half_as_ushort(__low2half(hv));
            hrow[mx * 8 + 8] = __half_as_ushort(__high2half(hv));
            lrow[mx * 8] = __half_as_ushort(__low2half(lv));
            lrow[mx * 8 + 8] = __half_as_ushort(__high2half(lv));
          }
        }
        tc_fence_before();
        mbar_arrive(&acc_empty[b]);  // the accumulators may be reused
        fence_proxy_async_smem();    // generic-proxy staging writes -> visible to the bulk copies
        g_sync();
        if (ct < 16) {
          // thread ct copies chunk cl = ct % 8 of plane ct / 8 (hi, lo): it holds
          // padded positions of chunk P = (l0 + ra)/8 + 7 - cl, stored at
          // np - 1 - P of line block p0/64; chunks past round8(H) are skipped
          const int cl = ct & 7;
          const int64_t P0 = (l0 + g.ra) / 8;
          if (l0 + 8 * (7 - cl) < ((a.lines + 7) & ~int64_t(7))) {
            unsigned char* gb = (ct < 8 ? a.chi : a.clo) + bd * a.plane_bstride +
                                (static_cast<size_t>(p0 / kGN) * a.np + (a.np - 1 - P0 - 7 + cl)) * kGChunk;
            bulk_s2g(gb, stg + ((ct >> 3) * 8 + cl) * kGStgChunk, kGChunk);
          }
          bulk_commit();
        }
      } else {
        float* xs = reinterpret_cast<float*>(sm + L.xch);
#pragma unroll
        for (int h16 = 0; h16 < 2; ++h16) {
          float v[16];
          sums16(h16, v);
#pragma unroll
          for (int n = 0; n < 16; ++n) xs[m * kGXPitch + half * 32 + 16 * h16 + n] = v[n];
        }
        tc_fence_before();
        mbar_arrive(&acc_empty[b]);  // the accumulators may be reused
        cp_async_wait<2>();          // this thread's centre copies of this tile have landed
        g_sync();
        // output: thread ct takes line i2 (raster column x2) and positions
        // (rows) ct / 64 + 4 q; a warp's lanes are 32 consecutive x
        // quotient: __fdividef (within 2 ulp; den <= 2^20 here, far below
        // its 2^126 limit), exact power-of-two rescale
        if (x2 < a.lines) {
          const int64_t y0 = p0 + (ct >> 6);
          const int64_t nrem = (a.len - y0 + 3) / 4;  // rows y0 + 4 q inside the raster
          const int nq = nrem < kGN / 4 ? static_cast<int>(nrem) : kGN / 4;
          if (a.out_dtype == VSR_F64) {
            double* op = static_cast<double*>(a.dst) + bd * a.out_bstride + y0 * a.out_pitch + x2;
#pragma unroll
            for (int q = 0; q < kGN / 4; ++q, op += 4 * a.out_pitch) {
              if (q >= nq) break;
              const int p = (ct >> 6) + 4 * q;
              const float num = xs[i2 * kGXPitch + p], den = xs[(kGL + i2) * kGXPitch + p];
              const bool ok = !(nd_val && centre(cb, p, i2) == a.nd_iv) && den > 0.0f;
              *op = ok ? static_cast<double>(__fdividef(num, den) * (kGScaleD / kGScaleV)) : a.nd_out;
            }
          } else {
            float* op = static_cast<float*>(a.dst) + bd * a.out_bstride + y0 * a.out_pitch + x2;
            const float ndf = static_cast<float>(a.nd_out);
#pragma unroll
            for (int q = 0; q < kGN / 4; ++q, op += 4 * a.out_pitch) {
              if (q >= nq) break;
              const int p = (ct >> 6) + 4 * q;
              const float num = xs[i2 * kGXPitch + p], den = xs[(kGL + i2) * kGXPitch + p];
              const bool ok = !(nd_val && centre(cb, p, i2) == a.nd_iv) && den > 0.0f;
              *op = ok ? __fdividef(num, den) * (kGScaleD / kGScaleV) : ndf;
            }
          }
        }
      }
      return true;
    };

    // Per tile j: (pass 1) tile j+1's raw copies are issued, tile j-2's
    // epilogue runs (its MMAs finished while tile j-1's were issued; tile
    // j-1's run meanwhile), then tile j's raw values (copied an iteration
    // ago) are converted into its A buffer.  Two A buffers and two
    // accumulator buffers: MMA j needs A(j) and the epilogue of j-2, both
    // released in iteration j.  (pass 2) tile j's centre copies are issued,
    // then tile j-2's epilogue runs.  One cp.async group per iteration.
    int j = 0;
    bool ok = true;
    int64_t b1 = 0, l1 = 0, p1 = 0, b2 = 0, l2 = 0, p2 = 0;  // band / first line / position of tiles j-1, j-2
    if (PASS == 1 && blockIdx.x < total) {
      int64_t bd, l0, p0;
      tile_of(blockIdx.x, bd, l0, p0);
      copy_rows(0, bd, l0, p0);
      cp_async_commit();
    }
    for (int64_t t = blockIdx.x; t < total; t += gridDim.x, ++j) {
      int64_t bd, l0, p0;
      tile_of(t, bd, l0, p0);
      if (PASS == 1) {
        const int64_t tn = t + gridDim.x;
        if (tn < total) {
          int64_t bn, ln, pn;
          tile_of(tn, bn, ln, pn);
          copy_rows((j + 1) & 1, bn, ln, pn);
        }
      } else {
        copy_centres(j % kGCenBufs, bd, l0, p0);
      }
      cp_async_commit();
      if (j >= 2 && !epilogue(j - 2, b2, l2, p2, (j - 2) % kGCenBufs)) {
        ok = false;
        break;
      }
      if (PASS == 1) {
        // A buffer j&1 was last read by tile j-2's MMAs, complete once its
        // accumulators were (the epilogue above waited for them)
        const int b = j & 1;
        cp_async_wait<1>();  // tile j's raw copies have landed (tile j+1's may be in flight)
        convert_rows(j & 1, b, l0, p0);
        fence_proxy_async_smem();  // generic-proxy operand writes -> visible to the tensor core
        mbar_arrive(&a_full[b]);
      }
      b2 = b1;
      l2 = l1;
      p2 = p1;
      b1 = bd;
      l1 = l0;
      p1 = p0;
    }
    // the last two epilogues; one empty cp.async group per call keeps the
    // pass-2 wait count (at most 2 newer groups) right
    if (ok && j >= 2) {
      cp_async_commit();
      ok = epilogue(j - 2, b2, l2, p2, (j - 2) % kGCenBufs);
    }
    if (ok && j >= 1) {
      cp_async_commit();
      epilogue(j - 1, b1, l1, p1, (j - 1) % kGCenBufs);
    }
    cp_async_wait<0>();
    if (PASS == 1 && ct < 16) bulk_wait_all();  // the output copies are done before the CTA ends
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
  const GaussGeom g = gauss_geom(p1.k);
  auto k1 = gauss_line_kernel<1, DT>;
  auto k2 = gauss_line_kernel<2, DT>;
  const size_t s1 = gauss_plan(g, 1).total + 1024, s2 = gauss_plan(g, 2).total + 1024;
  VSR_CUDA_TRY(cudaFuncSetAttribute(k1, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(s1)));
  VSR_CUDA_TRY(cudaFuncSetAttribute(k2, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(s2)));
  const int64_t t1 = ((p1.lines + kGL - 1) / kGL) * ((p1.len + kGN - 1) / kGN) * p1.bands;
  const int64_t t2 = ((p2.lines + kGL - 1) / kGL) * ((p2.len + kGN - 1) / kGN) * p2.bands;
  k1<<<static_cast<unsigned>(std::min<int64_t>(t1, sm_count())), kGThreads, s1, st>>>(p1, err);
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

// Workspace: band image | an aligned copy of one raster band (used when the
// caller's rows are not 8-byte aligned) | hi chunk planes of a group of
// bands | lo chunk planes of the group.  A workspace with room for the
// planes of every band runs the whole stack in one launch per pass; a
// smaller one runs the bands in groups (down to one band per launch pair).
size_t gauss_tc_workspace_bands(int64_t H, int64_t W, int dtype, int k, int bands) {
  const GaussGeom g = gauss_geom(k);
  const int64_t esz = dtype == VSR_U8 ? 1 : 2;
  const size_t band = (static_cast<size_t>(2) * g.NB * 128 + 255) & ~size_t(255);
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
  const GaussGeom g = gauss_geom(k);
  const int64_t np = gauss_np(H, g);
  const int64_t nx = (W + kGL - 1) / kGL;
  const size_t esz = dtype == VSR_U8 ? 1 : 2;
  const size_t osz = out_dtype == VSR_F64 ? 8 : 4;
  const int64_t apitch = gauss_aligned_pitch(W, static_cast<int64_t>(esz));
  char* ws = static_cast<char*>(workspace);
  uint16_t* band = reinterpret_cast<uint16_t*>(ws);
  const size_t off_copy = (static_cast<size_t>(2) * g.NB * 128 + 255) & ~size_t(255);
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
                 nullptr, out_dtype, out_pitch, nodata, band, k, nb, sb, plane, 0};
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
