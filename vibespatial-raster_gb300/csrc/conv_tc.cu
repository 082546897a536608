// Split-BF16 tcgen05 implicit GEMM for large normalised focal convolutions.
//
// Formulation (one output tile = 128 image rows x 64 image columns):
//   out[y0+m, x0+n] = sum_ky sum_k' X[m+ky][k'] * w[ky][k'-n]
// where X is the tile's input window (128+kh-1 rows x 64+kw-1 columns).  For
// each kernel row ky this is a GEMM  C[m][n] += A_ky[m][k'] B_ky[k'][n]  with
// A_ky = X shifted down ky rows and B_ky the Toeplitz band of weight row ky.
//
// Operand layouts (canonical K-major, no swizzle: 8-row x 16-byte core
// matrices, LBO = stride between core matrices along K, SBO = along M/N):
//  * A is stored with its K index reversed (k = Kp-1-k') and rows 16 bytes
//    apart, so A_ky is the same descriptor advanced by ky*16 bytes.
//  * B (also K-reversed) satisfies B[n+8][k-8] = B[n][k]; with SBO = LBO =
//    128 bytes every (n-group, k-chunk) pair maps to core matrix n/8 + k/8,
//    so one kernel row's Toeplitz band is Kp/8 + 64/8 - 1 core matrices.
// Tile width: a tcgen05.mma with M = 128 costs a fixed ~51 cycles up to
// N = 64 and runs at the full rate only from N = 128 (measured on GB300 with
// a one-thread loop of dependent MMAs); with the Toeplitz padding (N + kw - 1
// taps of K per N outputs) N = 64 and N = 128 cost the same per output and
// N = 64 needs half the shared memory.
//
// Precision: values are centred on the tile's centre pixel (mu), scaled by
// a power of two zs (from the raster's largest finite value, so that
// |z| < 2^15) and split z = z_hi + z_lo with z_hi BF16 and z_lo F16; the
// weights, scaled by a power of two ws (largest |w| near 2^13), are split
// w = w_hi + w_lo (BF16) and also kept as w16 = F16(w_hi + w_lo).  Three
// products per tap: z_hi*w_hi and z_hi*w_lo (BF16 MMAs) and z_lo*w16 (an F16
// MMA; each MMA's two operands share a type).  The F16 low part carries 11
// more bits of z than a BF16 one would, and pairing it with a full-precision
// weight leaves out only z_lo * (w - w16), about 2^-20 of a product, where a
// BF16 pair leaves out z_lo * w_lo, about 2^-18.  The hi*hi chain
// accumulates in FP32 tensor memory in groups of kernel rows (the
// accumulation error grows with the number of MMAs chained into one
// accumulator), the two correction products in one more accumulator; the
// groups are added in FP32 registers and the sum is scaled back by 1/zs.
// The accumulators' rounding grows with their magnitude, so each window
// row r is also centred on its own mean o_r (when every in-raster tap of the
// row is valid and finite; else o_r = 0): the A operand holds z - o_r, and
// -o_r at the row's columns outside the raster, so that every output row m
// gets back the same sum_ky o[m+ky] * rowsum_ky(w), formed in the epilogue
// with compensated FP32 arithmetic (error-free products and sums) from the
// row sums of the split weights.  A smooth raster then leaves only its
// local noise in the accumulators.  The weight sum uses the same split weights, so the
// quotient is a consistently weighted mean: on tiles whose window holds no
// nodata it comes from a summed-area table of w_hi + w_lo (borders only
// clip the window), otherwise from a 0/1 validity operand times w_hi and
// w_lo.  out = num/den + mu.  NaN taps (the reference's NaN * valid
// poisoning) and +-inf are kept out of the GEMM; per-row bitmasks give
// their window footprints: NaN, or the infinite sum the reference forms.
//
// Persistent CTA, one per SM, 6 warps with fixed roles:
//   warp 0      issues the tcgen05.mma chains of each tile
//   warp 1      streams the Toeplitz bands, one kernel row per stage, into a
//               shared-memory ring with cp.async.bulk
//   warps 2..5  convert the next tile's window to BF16 hi/lo (+ validity) in
//               the MMA layout straight from global memory, then run the
//               previous tile's epilogue (tcgen05.ld, FP32 sums, stores)
// The roles hand over through mbarriers: full/empty pairs for the A buffers
// (two when they fit), the TMEM accumulator buffers (two when they fit) and
// the band ring.  Every wait is bounded: on expiry the waiter records an
// error code and raises a shared abort flag that ends the other roles'
// waits; the MMA issuer and the band producer then wait (bounded) for their
// own operations in flight before the CTA frees its tensor memory.
#include "tc_common.cuh"

namespace vsr {

size_t conv_tc_workspace(int kh, int kw);
int conv_tc_supported(int kh, int kw);
int run_conv_tc(const void* src, int dtype, int bands, int64_t band_stride, int64_t H, int64_t W, int64_t pitch,
                const double* weights_host, int kh, int kw, double nodata, int nodata_kind, void* dst, int out_dtype,
                int64_t out_band_stride, int64_t out_pitch, void* workspace, size_t ws_bytes, cudaStream_t st);

namespace {

using namespace tc;

constexpr int kM = kMmaM;          // output rows per tile (TMEM lanes, MMA M)
constexpr int kTN = kMmaN;         // output columns per tile (MMA N)
constexpr int kConvWarps = 8;      // warps 2..9
constexpr int kConvThreads = 32 * kConvWarps;
constexpr int kThreadsTC = 64 + kConvThreads;
constexpr int kMaxTCK = 41;
constexpr int kMaxStages = 8;      // Toeplitz band ring depth (at most)
constexpr int kRowsPerStage = 2;   // kernel rows per ring stage (one wait and one release per stage)
constexpr int kConvRows = 6;       // window rows a converter warp loads per batch

struct TcGeom {
  int kh, kw;
  int R;   // window rows = kM + kh - 1
  int Rp;  // A operand: 16-byte rows between core-matrix columns (odd: conflict-free 8-byte stores)
  int KW;  // window columns = kTN + kw - 1
  int Kp;  // GEMM K per kernel row (KW rounded up to 16)
  int KC;  // Kp / 8 core-matrix columns
  int KS;  // Kp / 16 MMA k-steps
  int NB;  // core matrices per Toeplitz band = KC + kTN/8 - 1
  int G;   // hi*hi (and weight-sum) accumulator groups
};

__host__ __device__ inline TcGeom make_geom(int kh, int kw) {
  TcGeom g;
  g.kh = kh;
  g.kw = kw;
  g.R = kM + kh - 1;
  g.Rp = g.R | 1;
  g.KW = kTN + kw - 1;
  g.Kp = (g.KW + 15) & ~15;
  g.KC = g.Kp / 8;
  g.KS = g.Kp / 16;
  g.NB = g.KC + kTN / 8 - 1;
  // MMAs per output that touch non-zero weights: kh rows x the k-steps a
  // kw-wide band overlaps; at most ~64 of them per accumulator.
  const int chain = kh * ((kw + 15) / 16 + 1);
  g.G = chain <= 64 ? 1 : (chain <= 128 ? 2 : 3);
  return g;
}

struct TcPlan {  // shared-memory byte offsets (1024-aligned base) and pipeline shape
  uint32_t a_bytes;             // one operand buffer
  uint32_t a_hi, a_lo, a_vd;    // nbuf buffers each
  uint32_t ring;                // nst stages of kRowsPerStage x (hi, lo, f16 band)
  uint32_t row_bytes, stage_bytes;
  uint32_t sat;                 // (kh+1) x (kw+1) doubles
  uint32_t ctr;                 // 2 x kM u64 centre-validity bits
  uint32_t nanrow;              // 2 x R unsigned __int128 NaN footprints
  uint32_t infrow;              // 2 x R unsigned __int128 +-inf footprints
  uint32_t okrow;               // 2 x R unsigned __int128 validity masks (nodata rules)
  uint32_t orow;                // 2 x R float row offsets (see the precision note)
  uint32_t rstab;               // kh float2 (hi, lo) row sums of the split weights
  uint32_t total;
  int nbuf;                     // A buffers (1 or 2)
  int nst;                      // ring stages
  int cols;                     // TMEM columns per accumulator buffer
  int tbuf;                     // TMEM accumulator buffers (1 or 2)
};

__host__ __device__ inline TcPlan make_plan(const TcGeom& g, bool has_nd, int nbuf, int nst) {
  TcPlan p;
  p.nbuf = nbuf;
  p.nst = nst;
  p.a_bytes = (static_cast<uint32_t>(g.KC) * g.Rp * 16 + 127) & ~127u;
  p.a_hi = 0;
  p.a_lo = p.a_hi + nbuf * p.a_bytes;
  p.a_vd = p.a_lo + nbuf * p.a_bytes;
  p.ring = p.a_vd + (has_nd ? nbuf * p.a_bytes : 0u);
  p.row_bytes = 3u * g.NB * 128;
  p.stage_bytes = kRowsPerStage * p.row_bytes;
  p.sat = p.ring + nst * p.stage_bytes;
  p.ctr = (p.sat + static_cast<uint32_t>(g.kh + 1) * (g.kw + 1) * 8 + 127) & ~127u;
  p.nanrow = p.ctr + 2 * kM * 8;
  p.infrow = p.nanrow + 2 * static_cast<uint32_t>(g.R) * 16;
  p.okrow = p.infrow + 2 * static_cast<uint32_t>(g.R) * 16;
  p.orow = p.okrow + (has_nd ? 2 * static_cast<uint32_t>(g.R) * 16 : 0u);
  p.rstab = p.orow + ((2 * static_cast<uint32_t>(g.R) * 4 + 15) & ~15u);
  p.total = p.rstab + static_cast<uint32_t>(g.kh) * 8;
  p.cols = (g.G + 1 + (has_nd ? g.G : 0)) * kTN;  // hh groups | corrections | weight-sum groups
  p.tbuf = 2 * p.cols <= 512 ? 2 : 1;
  return p;
}

// Named barrier 1 over the converter warps; conv_any also ORs a predicate.
__device__ __forceinline__ void conv_sync() { asm volatile("bar.sync 1, %0;" ::"n"(kConvThreads) : "memory"); }

__device__ __forceinline__ bool conv_any(bool p) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred q, o;\n\t"
      "setp.ne.u32 q, %1, 0;\n\t"
      "bar.red.or.pred o, 1, %2, q;\n\t"
      "selp.u32 %0, 1, 0, o;\n\t}"
      : "=r"(r)
      : "r"(static_cast<uint32_t>(p)), "n"(kConvThreads)
      : "memory");
  return r != 0;
}

// Bit l of b[q] flags window column 4l + q (lane l holds columns 4l..4l+3);
// returns word w of the column-major mask (columns 32w..32w+31).
__device__ __forceinline__ uint32_t interleave4(const uint32_t b[4], int w) {
  uint32_t out = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    uint32_t x = (b[q] >> (8 * w)) & 0xFFu;  // lanes 8w..8w+7
    x = (x | (x << 12)) & 0x000F000Fu;
    x = (x | (x << 6)) & 0x03030303u;
    x = (x | (x << 3)) & 0x11111111u;  // bit i -> bit 4i
    out |= x << q;
  }
  return out;
}

struct TcArgs {
  const float* src;
  int64_t H, W, pitch;
  int nd_kind;
  float nd_f;
  double nd_out;
  void* dst;
  int out_dtype;
  int64_t out_pitch;
  int vec_out;                  // float32 output with 16-byte aligned rows
  const unsigned char* bw_img;  // per kernel row: hi, lo (BF16) and w16 (F16) bands, NB core matrices each
  const double* sat;            // (kh+1) x (kw+1) prefix sums of w_hi + w_lo (scaled by ws)
  const uint32_t* vmax_bits;    // largest finite |value| of the raster (float bits), sets zs
  const double* w64;            // the kernel as given (windows holding +-inf)
  int kh, kw;
  int nbuf, nst;
  int bands;                    // band-first stack: tiles are band-major
  int64_t band_stride, out_band_stride;
};

__device__ __forceinline__ int64_t clamp64(int64_t v, int64_t lo, int64_t hi) {
  return v < lo ? lo : (v > hi ? hi : v);
}


// Output of a window that holds +-inf values (and no NaN): the reference
// sums v * w, so each valid infinite tap adds +-inf (NaN for a zero weight)
// and the sum is +-inf, or NaN when both signs meet.  Scans the window; such
// windows are rare.
__device__ __noinline__ float inf_window(const float* __restrict__ src, int64_t H, int64_t W, int64_t pitch,
                                         const double* __restrict__ w64, int kh, int kw, int nd_kind, float nd_f,
                                         int64_t y, int64_t x) {
  bool pos = false, neg = false, nan = false;
  for (int ky = 0; ky < kh; ++ky) {
    const int64_t yy = y + ky - kh / 2;
    if (yy < 0 || yy >= H) continue;
    for (int kx = 0; kx < kw; ++kx) {
      const int64_t xx = x + kx - kw / 2;
      if (xx < 0 || xx >= W) continue;
      const float v = __ldg(src + yy * pitch + xx);
      if (!isinf(v) || (nd_kind == VSR_NODATA_VALUE && v == nd_f)) continue;
      const double t = static_cast<double>(v) * w64[ky * kw + kx];
      pos |= t > 0.0;
      neg |= t < 0.0;
      nan |= t != t;
    }
  }
  if (nan || (pos && neg)) return __int_as_float(0x7fc00000);
  return pos ? __int_as_float(0x7f800000) : __int_as_float(0xff800000);
}

// ND: the raster's nodata rule (0 none, 1 a value, 2 NaN).
template <int ND>
__global__ void __launch_bounds__(kThreadsTC, 1) conv_tc_kernel(const TcArgs a, uint32_t* err_word) {
  extern __shared__ unsigned char tc_raw[];
  __shared__ __align__(8) uint64_t a_full[2], a_empty[2], acc_full[2], acc_empty[2], b_full[kMaxStages],
      b_empty[kMaxStages], drain_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;
  __shared__ int64_t info_x0[2], info_y0[2], info_band[2];
  __shared__ float info_mu[2];
  __shared__ int info_nan[2], info_inf[2], info_nd[2];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(tc_raw) + 1023) & ~uintptr_t(1023));
  const TcGeom g = make_geom(a.kh, a.kw);
  const TcPlan L = make_plan(g, ND != 0, a.nbuf, a.nst);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // value scale zs = 2^(14 - E) for a largest |value| below 2^E: |v - mu| < 2^15
  int zexp = 0;
  {
    const float vmax = __uint_as_float(*a.vmax_bits);
    if (vmax > 0.0f && isfinite(vmax)) {
      int e = 0;
      frexpf(vmax, &e);
      zexp = max(-120, min(120, 14 - e));
    }
  }
  const float zs = ldexpf(1.0f, zexp), unscale = ldexpf(1.0f, -zexp);
  const int64_t tiles_x = (a.W + kTN - 1) / kTN;
  const int64_t per_band = tiles_x * ((a.H + kM - 1) / kM);
  const int64_t total = per_band * a.bands;
  const uint32_t s_base = smem_u32(sm);
  double* sat = reinterpret_cast<double*>(sm + L.sat);

  // ---- set-up: zero the A buffers (K-padding columns stay zero for good),
  // copy the summed-area table, initialise barriers, allocate tensor memory
  for (uint32_t i = tid * 16; i < L.ring; i += kThreadsTC * 16)
    *reinterpret_cast<uint4*>(sm + i) = make_uint4(0u, 0u, 0u, 0u);
  for (int i = tid; i < (a.kh + 1) * (a.kw + 1); i += kThreadsTC) sat[i] = a.sat[i];
  {
    float2* rs = reinterpret_cast<float2*>(sm + L.rstab);
    const int S1 = a.kw + 1;
    for (int ky = tid; ky < a.kh; ky += kThreadsTC) {
      const double r = (a.sat[(ky + 1) * S1 + a.kw] - a.sat[ky * S1 + a.kw]);
      const float hi = static_cast<float>(r);
      rs[ky] = make_float2(hi, static_cast<float>(r - static_cast<double>(hi)));
    }
  }
  if (tid == 0) {
    abort_flag = 0;
    for (int i = 0; i < 2; ++i) {
      mbar_init(&a_full[i], kConvThreads);
      mbar_init(&a_empty[i], 1);
      mbar_init(&acc_full[i], 1);
      mbar_init(&acc_empty[i], kConvThreads);
    }
    for (int s = 0; s < L.nst; ++s) {
      mbar_init(&b_full[s], 1);
      mbar_init(&b_empty[s], 1);
    }
    mbar_init(&drain_bar, 1);
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(&tmem_slot, 512);
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == 0) {
    // ========================================================= MMA issuer
    if (lane == 0) {
      const uint32_t lbo_a = static_cast<uint32_t>(g.Rp) * 16;
      const uint32_t a_ks = (2 * lbo_a) >> 4;  // one k-step = two core matrices along K
      const uint32_t w_ring = desc_lo(s_base + L.ring, 128), stage_w = L.stage_bytes >> 4, row_w = L.row_bytes >> 4;
      // first kernel rows of accumulator groups 1 and 2 (kh when absent):
      // row ky belongs to group floor(ky G / kh)
      const int gb1 = g.G > 1 ? (a.kh + g.G - 1) / g.G : a.kh;
      const int gb2 = g.G > 2 ? (2 * a.kh + g.G - 1) / g.G : a.kh;
      uint32_t u = 0;                          // band-ring uses
      int j = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < total; t += gridDim.x, ++j) {
        const int b = j % a.nbuf, tb = j % L.tbuf, slot = j & 1;
        ok = wait_or_abort(&a_full[b], (j / a.nbuf) & 1, &abort_flag, err_word, kDevErrMmaTimeout);
        if (ok && j >= L.tbuf)
          ok = wait_or_abort(&acc_empty[tb], ((j / L.tbuf) - 1) & 1, &abort_flag, err_word, kDevErrMmaTimeout);
        if (!ok) break;
        tc_fence_after();
        const bool den_mma = info_nd[slot] != 0;
        const uint32_t w_ahi = desc_lo(s_base + L.a_hi + b * L.a_bytes, lbo_a);
        const uint32_t w_alo = desc_lo(s_base + L.a_lo + b * L.a_bytes, lbo_a);
        const uint32_t w_avd = desc_lo(s_base + L.a_vd + b * L.a_bytes, lbo_a);
        const uint32_t t_acc = tmem + tb * L.cols;
        const uint32_t t_corr = t_acc + g.G * kTN, t_den = t_acc + (g.G + 1) * kTN;
        // Per ring stage one wait and one release; per kernel row a few
        // integer ops, then the MMAs (the thread's overhead between rows is
        // time the tensor pipe may run dry).  The band-full wait needs no
        // tcgen05 fence: the copy completes on the mbarrier itself.
        for (int ky0 = 0; ky0 < a.kh; ky0 += kRowsPerStage, ++u) {
          const uint32_t s = u % L.nst;
          ok = wait_or_abort(&b_full[s], (u / L.nst) & 1, &abort_flag, err_word, kDevErrMmaTimeout);
          if (!ok) break;
          const int ky1 = min(a.kh, ky0 + kRowsPerStage);
          for (int ky = ky0; ky < ky1; ++ky) {
            const int grp = (ky >= gb1) + (ky >= gb2);
            const uint32_t f = (ky == 0 || ky == gb1 || ky == gb2) ? 0u : 1u;  // first row of its group
            const uint32_t tg = t_acc + grp * kTN, td = t_den + grp * kTN;
            // A_ky = the window advanced ky rows (16 bytes each); one k-step =
            // two core matrices along K on both operands
            uint32_t ah = w_ahi + ky, al = w_alo + ky, av = w_avd + ky;
            uint32_t bh = w_ring + s * stage_w + (ky - ky0) * row_w, bl = bh + g.NB * 8, bf = bh + 2 * g.NB * 8;
            mma_bf16(tg, ah, bh, f);
            mma_bf16(t_corr, ah, bl, ky != 0);
            mma_f16(t_corr, al, bf, 1u);
            if (den_mma) {
              mma_bf16(td, av, bh, f);
              mma_bf16(td, av, bl, 1u);
#pragma unroll 1
              for (int ks = 1; ks < g.KS; ++ks) {
                ah += a_ks;
                al += a_ks;
                av += a_ks;
                bh += 16;
                bl += 16;
                bf += 16;
                mma_bf16(tg, ah, bh, 1u);
                mma_bf16(t_corr, ah, bl, 1u);
                mma_f16(t_corr, al, bf, 1u);
                mma_bf16(td, av, bh, 1u);
                mma_bf16(td, av, bl, 1u);
              }
            } else {
#pragma unroll 2
              for (int ks = 1; ks < g.KS; ++ks) {
                ah += a_ks;
                al += a_ks;
                bh += 16;
                bl += 16;
                bf += 16;
                mma_bf16(tg, ah, bh, 1u);
                mma_bf16(t_corr, ah, bl, 1u);
                mma_f16(t_corr, al, bf, 1u);
              }
            }
          }
          mma_commit(&b_empty[s]);  // the stage is free once these MMAs have read it
        }
        if (!ok) break;
        mma_commit(&a_empty[b]);
        mma_commit(&acc_full[tb]);
      }
      if (!ok) {
        // MMAs already issued must finish before tensor memory is released
        mma_commit(&drain_bar);
        mbar_wait_bounded(&drain_bar, 0, err_word, kDevErrMmaTimeout);
      }
    }
  } else if (warp == 1) {
    // ========================================================= band producer
    if (lane == 0) {
      uint32_t u = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < total && ok; t += gridDim.x) {
        for (int ky0 = 0; ky0 < a.kh; ky0 += kRowsPerStage, ++u) {
          const uint32_t s = u % L.nst;
          if (u >= static_cast<uint32_t>(L.nst)) {
            ok = wait_or_abort(&b_empty[s], ((u / L.nst) - 1) & 1, &abort_flag, err_word, kDevErrTmaTimeout);
            if (!ok) break;
          }
          // a tile's rows ky0 .. ky0+1 (fewer at the end) are contiguous in the image
          const uint32_t bytes = static_cast<uint32_t>(min(kRowsPerStage, a.kh - ky0)) * L.row_bytes;
          mbar_arrive_expect_tx(&b_full[s], bytes);
          bulk_g2s(sm + L.ring + s * L.stage_bytes, a.bw_img + static_cast<size_t>(ky0) * L.row_bytes, bytes,
                   &b_full[s]);
        }
      }
      if (!ok) {
        // every stage's newest copy must land before shared memory is released
        const uint32_t nst = static_cast<uint32_t>(L.nst);
        for (uint32_t k = (u > nst ? u - nst : 0u); k < u; ++k)
          mbar_wait_bounded(&b_full[k % nst], (k / nst) & 1, err_word, kDevErrTmaTimeout);
      }
    }
  } else {
    // ========================================================= converters + epilogue
    const int cw = warp - 2;            // converter warp 0..7
    const int ct = tid - 64;            // converter thread
    const int quarter = warp & 3;       // the TMEM lane quarter this warp may read
    const int chalf = cw >> 2;          // epilogue: output columns 32*chalf .. +31
    const int m = quarter * 32 + lane;  // epilogue: output row in the tile
    const int kh2 = a.kh / 2, kw2 = a.kw / 2;
    const int S1 = a.kw + 1;
    const float wtot = static_cast<float>(sat[a.kh * S1 + a.kw]);
    const float inv_wtot = __frcp_rn(wtot) * unscale;
    // this lane's window columns 4*lane .. 4*lane+3; in the K-reversed A
    // layout they are elements klo+3 .. klo of one core-matrix row, so each
    // operand takes one 8-byte store per window row
    const int kp0 = 4 * lane;
    const bool lane_cols = kp0 < g.KW;
    const int klo = g.Kp - 4 - kp0;
    const uint32_t o_lane = lane_cols ? static_cast<uint32_t>(klo >> 3) * g.Rp * 16 + (klo & 7) * 2 : 0u;
    bool ok = true;

    auto epilogue = [&](int jj) {
      const int tb = jj % L.tbuf, slot = jj & 1;
      const bool got = wait_or_abort(&acc_full[tb], (jj / L.tbuf) & 1, &abort_flag, err_word, kDevErrMmaTimeout);
      if (conv_any(!got)) {
        ok = false;
        return;
      }
      tc_fence_after();
      const int64_t x0 = info_x0[slot], y0 = info_y0[slot], band = info_band[slot];
      const float* bsrc = a.src + band * a.band_stride;
      const float mu = info_mu[slot];
      const bool den_mma = info_nd[slot] != 0;
      const int64_t y = y0 + m;
      // centre validity of this row's 64 outputs
      uint64_t cbits;
      if (ND == 0) {
        const int64_t nx = a.W - x0;
        cbits = y >= a.H ? 0ull : (nx >= 64 ? ~0ull : ((1ull << nx) - 1ull));
      } else {
        const unsigned __int128 okm = reinterpret_cast<const unsigned __int128*>(sm + L.okrow)[slot * g.R + m + kh2];
        cbits = static_cast<uint64_t>(okm >> kw2);
      }
      unsigned __int128 foot = 0, ifoot = 0;
      if (info_nan[slot]) {
        const unsigned __int128* nr = reinterpret_cast<const unsigned __int128*>(sm + L.nanrow) + slot * g.R;
        for (int r2 = 0; r2 < a.kh; ++r2) foot |= nr[m + r2];
      }
      if (info_inf[slot]) {
        const unsigned __int128* ir = reinterpret_cast<const unsigned __int128*>(sm + L.infrow) + slot * g.R;
        for (int r2 = 0; r2 < a.kh; ++r2) ifoot |= ir[m + r2];
      }
      const uint32_t lane_base = tmem + tb * L.cols + (static_cast<uint32_t>(quarter * 32) << 16);
      // the output row's window rows clipped to the raster (summed-area table rows);
      // float64: a clipped window's sum is a difference of larger prefix sums
      const int ky_lo = static_cast<int>(clamp64(kh2 - y, 0, a.kh));
      const int ky_hi = static_cast<int>(clamp64(a.H - y + kh2, ky_lo, a.kh));
      const double* s_lo = sat + ky_lo * S1;
      const double* s_hi = sat + ky_hi * S1;
      const bool interior = ky_lo == 0 && ky_hi == a.kh && x0 - kw2 >= 0 && x0 + kTN - 1 + (a.kw - 1 - kw2) < a.W;
      // the row offsets' share of this output row: sum_ky o[m+ky] rowsum_ky,
      // as a compensated (hi, lo) pair
      float c_hi = 0.0f, c_lo = 0.0f;
      {
        const float* orow = reinterpret_cast<const float*>(sm + L.orow) + slot * g.R + m;
        const float2* rs = reinterpret_cast<const float2*>(sm + L.rstab);
        for (int ky = 0; ky < a.kh; ++ky) {
          const float o = orow[ky];
          const float2 w = rs[ky];
          const float p = o * w.x;
          const float pe = fmaf(o, w.x, -p) + o * w.y;  // the product's rounding error + the lo part
          const float t = c_hi + p;
          const float bp = t - c_hi;
          c_lo += ((c_hi - (t - bp)) + (p - bp)) + pe;
          c_hi = t;
        }
      }
#pragma unroll 1
      for (int sc = 0; sc < 2; ++sc) {
        const int c0 = chalf * 32 + sc * 16;  // first of this pass's 16 output columns
        float num[16], den[16], part[16];
        tmem_ld16(lane_base + c0, num);
        for (int gi = 1; gi < g.G; ++gi) {
          tmem_ld16(lane_base + gi * kTN + c0, part);
#pragma unroll
          for (int n = 0; n < 16; ++n) num[n] += part[n];
        }
        tmem_ld16(lane_base + g.G * kTN + c0, part);  // correction products
#pragma unroll
        for (int n = 0; n < 16; ++n) num[n] += part[n];
        if (ND != 0 && den_mma) {
          tmem_ld16(lane_base + (g.G + 1) * kTN + c0, den);
          for (int gi = 1; gi < g.G; ++gi) {
            tmem_ld16(lane_base + (g.G + 1 + gi) * kTN + c0, part);
#pragma unroll
            for (int n = 0; n < 16; ++n) den[n] += part[n];
          }
        } else if (interior) {
#pragma unroll
          for (int n = 0; n < 16; ++n) den[n] = wtot;
        } else {
#pragma unroll
          for (int n = 0; n < 16; ++n) {
            const int64_t x = x0 + c0 + n;
            const int kx_lo = static_cast<int>(clamp64(kw2 - x, 0, a.kw));
            const int kx_hi = static_cast<int>(clamp64(a.W - x + kw2, kx_lo, a.kw));
            den[n] = static_cast<float>((s_hi[kx_hi] - s_lo[kx_hi]) - (s_hi[kx_lo] - s_lo[kx_lo]));
          }
        }
        if (y < a.H) {
          const int64_t xb = x0 + c0;
          const uint32_t cb = static_cast<uint32_t>(cbits >> c0) & 0xFFFFu;
          const uint32_t fb = static_cast<uint32_t>(static_cast<uint64_t>(foot >> c0)) & 0xFFFFu;
          const uint32_t ib = static_cast<uint32_t>(static_cast<uint64_t>(ifoot >> c0)) & 0xFFFFu & ~fb;
          uint32_t ndm = 0;  // outputs that take the nodata value
#pragma unroll
          for (int n = 0; n < 16; ++n) {
            const bool nd = !((cb >> n) & 1u) || !(den[n] > 0.0f);
            ndm |= static_cast<uint32_t>(nd) << n;
            const float inv = (ND == 0 || !den_mma) && interior ? inv_wtot : __frcp_rn(den[n]) * unscale;
            num[n] = ((fb >> n) & 1u) ? __int_as_float(0x7fc00000) : fmaf((num[n] + c_hi) + c_lo, inv, mu);
          }
          for (uint32_t r = ib & ~ndm; r; r &= r - 1) {  // windows holding +-inf (rare)
            const int n = __ffs(r) - 1;
            if (xb + n < a.W) {
              const float v = inf_window(bsrc, a.H, a.W, a.pitch, a.w64, a.kh, a.kw, a.nd_kind, a.nd_f, y, xb + n);
#pragma unroll
              for (int q = 0; q < 16; ++q)
                if (q == n) num[q] = v;
            }
          }
          if (a.out_dtype == VSR_F64) {
            double* row = static_cast<double*>(a.dst) + band * a.out_band_stride + y * a.out_pitch + xb;
#pragma unroll
            for (int n = 0; n < 16; ++n)
              if (xb + n < a.W) row[n] = ((ndm >> n) & 1u) ? a.nd_out : static_cast<double>(num[n]);
          } else {
            const float ndf = static_cast<float>(a.nd_out);
#pragma unroll
            for (int n = 0; n < 16; ++n) num[n] = ((ndm >> n) & 1u) ? ndf : num[n];
            float* row = static_cast<float*>(a.dst) + band * a.out_band_stride + y * a.out_pitch + xb;
            if (a.vec_out && xb + 16 <= a.W) {
#pragma unroll
              for (int q = 0; q < 4; ++q)
                reinterpret_cast<float4*>(row)[q] = make_float4(num[4 * q], num[4 * q + 1], num[4 * q + 2], num[4 * q + 3]);
            } else {
#pragma unroll
              for (int n = 0; n < 16; ++n)
                if (xb + n < a.W) row[n] = num[n];
            }
          }
        }
      }
      tc_fence_before();
      mbar_arrive(&acc_empty[tb]);
    };

    int j = 0;
    for (int64_t t = blockIdx.x; t < total; t += gridDim.x, ++j) {
      const int b = j % a.nbuf, slot = j & 1;
      if (j >= a.nbuf) {
        const bool got = wait_or_abort(&a_empty[b], ((j / a.nbuf) - 1) & 1, &abort_flag, err_word, kDevErrMmaTimeout);
        if (conv_any(!got)) {
          ok = false;
          break;
        }
      }
      const int64_t band = t / per_band, rem = t - band * per_band;
      const int64_t ty = rem / tiles_x;
      const int64_t x0 = (rem - ty * tiles_x) * kTN, y0 = ty * kM;
      const float* bsrc = a.src + band * a.band_stride;
      const int64_t gx0 = x0 - kw2, gy0 = y0 - kh2;
      float mu = 0.0f;
      {
        // the window's centre pixel, moved inside the raster on edge tiles
        // (a centre far from the tile's values would cost accumulator bits)
        const int64_t yy = clamp64(gy0 + g.R / 2, 0, a.H - 1), xx = clamp64(gx0 + g.KW / 2, 0, a.W - 1);
        const float v = __ldg(bsrc + yy * a.pitch + xx);
        const bool nd = ND == 1 ? v == a.nd_f : (ND == 2 ? v != v : false);
        if (!nd && isfinite(v)) mu = v;
      }
      uint32_t colv = 0;  // this lane's columns inside the window and the raster
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int64_t xx = gx0 + kp0 + q;
        colv |= static_cast<uint32_t>(kp0 + q < g.KW && xx >= 0 && xx < a.W) << q;
      }
      uint32_t* nanw = reinterpret_cast<uint32_t*>(sm + L.nanrow) + slot * g.R * 4;
      uint32_t* infw = reinterpret_cast<uint32_t*>(sm + L.infrow) + slot * g.R * 4;
      uint32_t* okw = reinterpret_cast<uint32_t*>(sm + L.okrow) + slot * g.R * 4;
      float* orow = reinterpret_cast<float*>(sm + L.orow) + slot * g.R;
      // window columns inside the raster (the same for every row of the tile)
      int ncols = __popc(colv);
#pragma unroll
      for (int o = 16; o; o >>= 1) ncols += __shfl_xor_sync(0xffffffffu, ncols, o);
      const float inv_ncols = 1.0f / static_cast<float>(ncols > 0 ? ncols : 1);
      unsigned char* ahi = sm + L.a_hi + b * L.a_bytes + o_lane;
      unsigned char* alo = sm + L.a_lo + b * L.a_bytes + o_lane;
      unsigned char* avd = sm + L.a_vd + b * L.a_bytes + o_lane;
      bool any_nan = false, any_inf = false, any_nd = false;
      // one warp per window row, 4 columns per lane; kConvRows rows are
      // loaded before any is converted, so the loads' latencies overlap
      for (int r0 = cw; r0 < g.R; r0 += kConvWarps * kConvRows) {
        float vb[kConvRows][4];
#pragma unroll
        for (int r = 0; r < kConvRows; ++r) {
          const int rho = r0 + kConvWarps * r;
          const int64_t yy = gy0 + rho;
          const uint32_t in = (rho < g.R && yy >= 0 && yy < a.H) ? colv : 0u;
          const int64_t base = (in ? yy : 0) * a.pitch + gx0 + kp0;
#pragma unroll
          for (int q = 0; q < 4; ++q) vb[r][q] = ((in >> q) & 1u) ? __ldg(bsrc + base + q) : 0.0f;
        }
#pragma unroll
        for (int r = 0; r < kConvRows; ++r) {
          const int rho = r0 + kConvWarps * r;
          if (rho >= g.R) break;
          const int64_t yy = gy0 + rho;
          const uint32_t in = (yy >= 0 && yy < a.H) ? colv : 0u;
          float z[4];
          uint32_t okm = 0, badm = 0;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const float v = vb[r][q];
            const bool inb = (in >> q) & 1u;
            const bool okv = inb && (ND == 1 ? v != a.nd_f : (ND == 2 ? v == v : true));
            const bool fin = fabsf(v) <= 3.402823466e38f;  // false for NaN and +-inf
            z[q] = (okv && fin) ? (v - mu) * zs : 0.0f;
            okm |= static_cast<uint32_t>(okv) << q;
            badm |= static_cast<uint32_t>(inb && !fin) << q;
          }
          if (ND != 0) any_nd |= okm != in;
          // row offset: the mean of a row whose in-raster taps are all valid
          // and finite (else 0); columns outside the raster carry -o
          float o = 0.0f;
          const bool row_clean = __all_sync(0xffffffffu, okm == in && badm == 0u);  // every lane votes
          if (yy >= 0 && yy < a.H && row_clean) {  // warp-uniform: one warp per window row
            float sum = (z[0] + z[1]) + (z[2] + z[3]);
#pragma unroll
            for (int sh = 16; sh; sh >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, sh);
            o = sum * inv_ncols;
#pragma unroll
            for (int q = 0; q < 4; ++q)
              z[q] = ((in >> q) & 1u) ? z[q] - o : (kp0 + q < g.KW ? -o : 0.0f);
          }
          if (lane == 0) orow[rho] = o;
          if (lane_cols) {
            const __nv_bfloat162 h32 = __floats2bfloat162_rn(z[3], z[2]);
            const __nv_bfloat162 h10 = __floats2bfloat162_rn(z[1], z[0]);
            const __half2 l32 = __floats2half2_rn(z[3] - __low2float(h32), z[2] - __high2float(h32));
            const __half2 l10 = __floats2half2_rn(z[1] - __low2float(h10), z[0] - __high2float(h10));
            *reinterpret_cast<uint2*>(ahi + rho * 16) = make_uint2(bf16x2_bits(h32), bf16x2_bits(h10));
            *reinterpret_cast<uint2*>(alo + rho * 16) = make_uint2(f16x2_bits(l32), f16x2_bits(l10));
            if (ND != 0)
              *reinterpret_cast<uint2*>(avd + rho * 16) =
                  make_uint2(((okm & 8u) ? 0x3f80u : 0u) | ((okm & 4u) ? 0x3f800000u : 0u),
                             ((okm & 2u) ? 0x3f80u : 0u) | ((okm & 1u) ? 0x3f800000u : 0u));
          }
          uint32_t bq[4];
          if (__any_sync(0xffffffffu, badm != 0)) {
            // NaN taps poison the window (reference product v * w * valid,
            // NaN * 0 included); valid +-inf taps make it infinite (inf_window)
            uint32_t pm = 0, im = 0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const float v = vb[r][q];
              const float vm = v * (((okm >> q) & 1u) ? 1.0f : 0.0f);
              pm |= static_cast<uint32_t>(((in >> q) & 1u) && vm != vm) << q;
              im |= static_cast<uint32_t>(((okm >> q) & 1u) && isinf(v)) << q;
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) bq[q] = __ballot_sync(0xffffffffu, (pm >> q) & 1u);
            const uint32_t wn = interleave4(bq, lane & 3);
#pragma unroll
            for (int q = 0; q < 4; ++q) bq[q] = __ballot_sync(0xffffffffu, (im >> q) & 1u);
            const uint32_t wi = interleave4(bq, lane & 3);
            if (lane < 4) {
              nanw[rho * 4 + lane] = wn;
              infw[rho * 4 + lane] = wi;
            }
            any_nan |= pm != 0;
            any_inf |= im != 0;
          } else if (lane < 4) {
            nanw[rho * 4 + lane] = 0u;
            infw[rho * 4 + lane] = 0u;
          }
          if (ND != 0) {
#pragma unroll
            for (int q = 0; q < 4; ++q) bq[q] = __ballot_sync(0xffffffffu, (okm >> q) & 1u);
            const uint32_t wo = interleave4(bq, lane & 3);
            if (lane < 4) okw[rho * 4 + lane] = wo;
          }
        }
      }
      fence_proxy_async_smem();  // generic-proxy operand writes -> visible to the tensor core
      const bool tile_nan = conv_any(any_nan);
      const bool tile_inf = conv_any(any_inf);
      const bool tile_nd = ND != 0 && conv_any(any_nd);
      if (ct == 0) {
        info_x0[slot] = x0;
        info_y0[slot] = y0;
        info_band[slot] = band;
        info_mu[slot] = mu;
        info_nan[slot] = tile_nan;
        info_inf[slot] = tile_inf;
        info_nd[slot] = tile_nd;
      }
      mbar_arrive(&a_full[b]);
      // horizontal footprints (bit n: such a tap in window columns [n, n+kw))
      if (tile_nan || tile_inf) {
        unsigned __int128* nanrow = reinterpret_cast<unsigned __int128*>(sm + L.nanrow) + slot * g.R;
        unsigned __int128* infrow = reinterpret_cast<unsigned __int128*>(sm + L.infrow) + slot * g.R;
        for (int rho = ct; rho < g.R; rho += kConvThreads) {
          const unsigned __int128 mrow = nanrow[rho], irow = infrow[rho];
          unsigned __int128 h = 0, hi = 0;
          for (int q = 0; q < a.kw; ++q) {
            h |= mrow >> q;
            hi |= irow >> q;
          }
          nanrow[rho] = h;
          infrow[rho] = hi;
        }
      }
      if (j >= 1) {
        epilogue(j - 1);
        if (!ok) break;
      }
      conv_sync();  // this iteration's reads of the older slot end before the next tile rewrites it
    }
    if (ok && j >= 1) epilogue(j - 1);
  }
  __syncwarp();
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

// Toeplitz band images: for kernel row ky, band s, core matrix c, row r,
// element e -> w'[ky][Kp-1-8c-e-r] (0 outside [0, kw)) with w' = w * ws:
// s = 0: BF16(w'), s = 1: BF16(w' - hi), s = 2: F16(hi + lo); laid out
// [ky][s][c][r][e] so a kernel row's three bands are one contiguous copy.
__global__ void prep_tc_weights(const double* __restrict__ w64, int kh, int kw, int Kp, int NB, double ws,
                                uint16_t* __restrict__ img) {
  const int per_row = NB * 64;
  const int total = kh * per_row;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int ky = i / per_row, rem = i - ky * per_row;
    const int c = rem / 64, r = (rem / 8) & 7, e = rem & 7;
    const int kx = Kp - 1 - 8 * c - e - r;
    const double w = (kx >= 0 && kx < kw) ? w64[ky * kw + kx] * ws : 0.0;
    const __nv_bfloat16 hi = __float2bfloat16_rn(static_cast<float>(w));
    const double h = static_cast<double>(__bfloat162float(hi));
    const __nv_bfloat16 lo = __float2bfloat16_rn(static_cast<float>(w - h));
    const __half w16 = __float2half_rn(static_cast<float>(h + static_cast<double>(__bfloat162float(lo))));
    img[((ky * 3 + 0) * NB + c) * 64 + r * 8 + e] = __bfloat16_as_ushort(hi);
    img[((ky * 3 + 1) * NB + c) * 64 + r * 8 + e] = __bfloat16_as_ushort(lo);
    img[((ky * 3 + 2) * NB + c) * 64 + r * 8 + e] = __half_as_ushort(w16);
  }
}

// Summed-area table of the split scaled weights w_hi + w_lo in float64:
// sat[i][j] = sum of w' over rows < i and columns < j.  One block: split
// weights to shared memory, row prefix sums (a thread per row), then
// column sums (a thread per column).
__global__ void prep_tc_sat(const double* __restrict__ w64, int kh, int kw, double wscale, double* __restrict__ sat) {
  __shared__ double ws[kMaxTCK * kMaxTCK];
  const int tid = threadIdx.x;
  for (int i = tid; i < kh * kw; i += blockDim.x) {
    const double w = w64[i] * wscale;
    const double h = __bfloat162float(__float2bfloat16_rn(static_cast<float>(w)));
    ws[i] = h + static_cast<double>(__bfloat162float(__float2bfloat16_rn(static_cast<float>(w - h))));
  }
  __syncthreads();
  if (tid < kh) {
    double acc = 0.0;
    for (int c = 0; c < kw; ++c) {
      acc += ws[tid * kw + c];
      ws[tid * kw + c] = acc;
    }
  }
  __syncthreads();
  if (tid <= kw) {
    double acc = 0.0;
    sat[tid] = 0.0;
    for (int i = 1; i <= kh; ++i) {
      if (tid > 0) acc += ws[(i - 1) * kw + tid - 1];
      sat[i * (kw + 1) + tid] = acc;
    }
  }
}

// Largest |v| over the finite, non-nodata values of every band, as float
// bits (non-negative floats order like their bit patterns), ORed into
// *out by atomicMax.  Rows are spread over the grid; 16-byte loads when the
// rows allow.
__global__ void __launch_bounds__(256) raster_absmax(const float* __restrict__ src, int64_t H, int64_t W,
                                                     int64_t pitch, int bands, int64_t band_stride, int nd_kind,
                                                     float nd_f, int vec, uint32_t* __restrict__ out) {
  float m = 0.0f;
  auto take = [&](float v) {
    const bool ok = isfinite(v) && !(nd_kind == VSR_NODATA_VALUE && v == nd_f);
    m = ok ? fmaxf(m, fabsf(v)) : m;
  };
  const int64_t rows = static_cast<int64_t>(bands) * H;
  for (int64_t rr = blockIdx.x; rr < rows; rr += gridDim.x) {
    const int64_t b = rr / H, y = rr - b * H;
    const float* row = src + b * band_stride + y * pitch;
    int64_t x0 = 0;
    if (vec) {
      const int64_t n4 = W / 4;
      for (int64_t i = threadIdx.x; i < n4; i += blockDim.x) {
        const float4 q = __ldg(reinterpret_cast<const float4*>(row) + i);
        take(q.x);
        take(q.y);
        take(q.z);
        take(q.w);
      }
      x0 = n4 * 4;
    }
    for (int64_t x = x0 + threadIdx.x; x < W; x += blockDim.x) take(__ldg(row + x));
  }
  for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.0f) atomicMax(out, __float_as_uint(m));
}

}  // namespace

constexpr uint32_t kSmemLimit = 227 * 1024 - 1024;  // less the 1024-byte alignment slack

// Two A buffers (conversion overlaps the MMAs) with at least three ring
// stages when they fit, else one A buffer; then as many stages as fit.
static void tc_shape(int kh, int kw, bool has_nd, int* nbuf, int* nst) {
  const TcGeom g = make_geom(kh, kw);
  for (int nb = 2; nb >= 1; --nb)
    for (int st = kMaxStages; st >= (nb == 2 ? 3 : 2); --st)
      if (make_plan(g, has_nd, nb, st).total <= kSmemLimit) {
        *nbuf = nb;
        *nst = st;
        return;
      }
  *nbuf = 0;
  *nst = 0;
}

int conv_tc_supported(int kh, int kw) {
  if (kh < 1 || kw < 1 || kh > kMaxTCK || kw > kMaxTCK) return 0;
  const TcGeom g = make_geom(kh, kw);
  const TcPlan p = make_plan(g, true, 1, 2);
  return p.total <= kSmemLimit && g.KW <= 128 && p.cols <= 512;
}

// Workspace: float64 weights | Toeplitz band images | summed-area table |
// the largest |value| word (256 bytes).
size_t conv_tc_workspace(int kh, int kw) {
  const TcGeom g = make_geom(kh, kw);
  const size_t a = (static_cast<size_t>(kh) * kw * 8 + 255) & ~size_t(255);
  const size_t b = (static_cast<size_t>(kh) * 3 * g.NB * 128 + 255) & ~size_t(255);
  const size_t c = (static_cast<size_t>(kh + 1) * (kw + 1) * 8 + 255) & ~size_t(255);
  return a + b + c + 256;
}

int run_conv_tc(const void* src, int dtype, int bands, int64_t band_stride, int64_t H, int64_t W, int64_t pitch,
                const double* weights_host, int kh, int kw, double nodata, int nodata_kind, void* dst, int out_dtype,
                int64_t out_band_stride, int64_t out_pitch, void* workspace, size_t ws_bytes, cudaStream_t st) {
  if (dtype != VSR_F32) return fail(VSR_ERR_UNSUPPORTED, "split-precision convolution reads float32 rasters");
  if (!conv_tc_supported(kh, kw))
    return fail(VSR_ERR_UNSUPPORTED, "split-precision convolution supports kernels up to %dx%d", kMaxTCK, kMaxTCK);
  const size_t need = conv_tc_workspace(kh, kw);
  if (!workspace || ws_bytes < need || !aligned(workspace, 256))
    return fail(VSR_ERR_WORKSPACE, "workspace must be 256-byte aligned and >= %zu bytes", need);
  const TcGeom g = make_geom(kh, kw);
  double ndv = 0.0;
  const int kind = resolve_nodata(VSR_F32, nodata, nodata_kind, &ndv);
  const bool has_nd = kind != VSR_NODATA_NONE;
  int nbuf = 0, nst = 0;
  tc_shape(kh, kw, has_nd, &nbuf, &nst);
  if (!nbuf) return fail(VSR_ERR_UNSUPPORTED, "split-precision convolution: %dx%d kernel does not fit shared memory", kh, kw);
  const TcPlan L = make_plan(g, has_nd, nbuf, nst);
  char* ws = static_cast<char*>(workspace);
  double* w64 = reinterpret_cast<double*>(ws);
  const size_t off_img = (static_cast<size_t>(kh) * kw * 8 + 255) & ~size_t(255);
  const size_t off_sat = off_img + ((static_cast<size_t>(kh) * 3 * g.NB * 128 + 255) & ~size_t(255));
  const size_t off_vmax = off_sat + ((static_cast<size_t>(kh + 1) * (kw + 1) * 8 + 255) & ~size_t(255));
  uint16_t* img = reinterpret_cast<uint16_t*>(ws + off_img);
  double* sat = reinterpret_cast<double*>(ws + off_sat);
  uint32_t* vmax = reinterpret_cast<uint32_t*>(ws + off_vmax);
  // weight scale: a power of two bringing the largest |w| to [2^12, 2^13)
  double wmax = 0.0;
  for (int i = 0; i < kh * kw; ++i)
    if (std::isfinite(weights_host[i])) wmax = std::max(wmax, std::fabs(weights_host[i]));
  int we = 0;
  if (wmax > 0.0) std::frexp(wmax, &we);
  const double wscale = wmax > 0.0 ? std::ldexp(1.0, std::max(-900, std::min(900, 13 - we))) : 1.0;
  VSR_CUDA_TRY(cudaMemcpyAsync(w64, weights_host, static_cast<size_t>(kh) * kw * 8, cudaMemcpyHostToDevice, st));
  prep_tc_weights<<<16, 256, 0, st>>>(w64, kh, kw, g.Kp, g.NB, wscale, img);
  VSR_CUDA_TRY(cudaGetLastError());
  prep_tc_sat<<<1, 64, 0, st>>>(w64, kh, kw, wscale, sat);
  VSR_CUDA_TRY(cudaGetLastError());
  VSR_CUDA_TRY(cudaMemsetAsync(vmax, 0, sizeof(uint32_t), st));
  {
    const bool vec = aligned(src, 16) && pitch % 4 == 0 && (bands == 1 || band_stride % 4 == 0);
    const int64_t rows = static_cast<int64_t>(bands) * H;
    const int blocks = static_cast<int>(std::min<int64_t>(rows, static_cast<int64_t>(sm_count()) * 8));
    raster_absmax<<<blocks, 256, 0, st>>>(static_cast<const float*>(src), H, W, pitch, bands,
                                          bands > 1 ? band_stride : 0, kind, static_cast<float>(ndv), vec ? 1 : 0,
                                          vmax);
    VSR_CUDA_TRY(cudaGetLastError());
  }
  uint32_t* err = device_error_word();
  if (!err) return VSR_ERR_CUDA;
  const bool vec_out =
      out_dtype == VSR_F32 && aligned(dst, 16) && out_pitch % 4 == 0 && (bands == 1 || out_band_stride % 4 == 0);
  TcArgs a{static_cast<const float*>(src), H, W, pitch, kind, static_cast<float>(ndv), nodata, dst, out_dtype,
           out_pitch, vec_out ? 1 : 0, reinterpret_cast<const unsigned char*>(img), sat, vmax, w64, kh, kw, nbuf, nst,
           bands, bands > 1 ? band_stride : 0, bands > 1 ? out_band_stride : 0};
  // At least 116 KB of shared memory keeps one CTA (and its 512 TMEM columns) per SM.
  const size_t smem = std::max<size_t>(L.total + 1024, 116 * 1024);
  auto kern = kind == VSR_NODATA_NONE ? conv_tc_kernel<0> : (kind == VSR_NODATA_VALUE ? conv_tc_kernel<1> : conv_tc_kernel<2>);
  VSR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  const int64_t tiles = ((W + kTN - 1) / kTN) * ((H + kM - 1) / kM) * bands;
  const int64_t grid = std::min<int64_t>(tiles, sm_count());
  kern<<<static_cast<unsigned>(grid), kThreadsTC, smem, st>>>(a, err);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}

}  // namespace vsr
