// The batched-tiles kernel (batch_terrain_kernel) and its launch, templated
// on the Gaussian width KG; batch.cu holds the host side (plan, run), and
// batch_k1_3.cu / batch_k5.cu / batch_k7_9.cu instantiate the launches per
// Gaussian width so that they compile in parallel.
#pragma once

#include "horn_common.cuh"

// One persistent, work-queue-scheduled launch over many DEM tiles of uneven
// sizes, each with its own cell size and nodata: slope + aspect (Horn) and a
// KG x KG nodata-aware Gaussian, all from one staged block.  Replaces the
// reference's per-tile / per-band Python loops (dispatch.py:417-506), which
// issue separate launches per raster and per operation.
//
// Work item = (tile, 128 x TH output block).  A CTA claims items with an
// atomic counter (no waits: an exhausted queue simply ends the CTA), finds
// the tile by binary search over the per-tile prefix sums, stages
// (TH + 2*HY) x 136 input values one item ahead with cp.async -- 16- or
// 8-byte copies for the column groups inside a tile whose rows allow them,
// clamped 4-byte copies elsewhere (any pitch or alignment; edge replication
// for Horn) -- runs the Horn rows on them, then the separable Gaussian
// (batch_gauss: each warp for its own output rows, (numerator, weight sum)
// pairs from packed f32x2 FMAs, validity from coordinates and nodata so that
// out-of-bounds taps are skipped, a rolling window of row sums in registers).
namespace vsr {
namespace bk {


using namespace horn;

__device__ __forceinline__ bool is_nd_rt(float v, int kind, float ndv) {
  return kind == VSR_NODATA_VALUE ? (v == ndv) : (kind == VSR_NODATA_NAN ? (v != v) : false);
}

// Horn rows of one batch item for the tile's nodata kind (warp-uniform).
template <int RB, bool EDGE, bool VEC>
__device__ __forceinline__ void batch_horn_rows(const float* S, int lane, int r0, int64_t y0, int64_t xs,
                                                const HornParams& P, const MaskRule& rule, float nd_in, float* srow,
                                                float* arow, int64_t sp) {
  if (P.nd_kind == VSR_NODATA_VALUE)
    horn_rows<RB, 3, VSR_NODATA_VALUE, EDGE, VEC>(S, lane, r0, y0, xs, P, rule, nd_in, srow, arow, nullptr, sp, sp);
  else if (P.nd_kind == VSR_NODATA_NAN)
    horn_rows<RB, 3, VSR_NODATA_NAN, EDGE, VEC>(S, lane, r0, y0, xs, P, rule, nd_in, srow, arow, nullptr, sp, sp);
  else
    horn_rows<RB, 3, VSR_NODATA_NONE, EDGE, VEC>(S, lane, r0, y0, xs, P, rule, nd_in, srow, arow, nullptr, sp, sp);
}

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
  int32_t stage;       // staging copy width: 16 (source 16-byte aligned, pitch % 4 == 0), 8 (8-byte, even pitch) or 4
  int32_t vec_smooth;  // Gaussian output 16-byte aligned with pitch % 4 == 0
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
  static constexpr int kFloats = 2 * SR * kSW;        // two staging buffers
};


template <int NDK>
__device__ __forceinline__ bool is_nd_k(float v, float ndv) {
  if constexpr (NDK == VSR_NODATA_VALUE) return v == ndv;
  else if constexpr (NDK == VSR_NODATA_NAN) return v != v;
  else return false;
}

// The KG x KG Gaussian of one staged item, by each warp for its own RB
// output rows and its lanes' 4 columns: a horizontal pass per staged row
// forms (v * valid, valid) pairs with packed FMAs (NaN * 0 stays NaN, as in
// the reference), a rolling window of the last KG such row sums in
// registers gives the vertical pass.  No shared memory beyond the staged
// block and no barrier: the RB + KG - 1 horizontal passes per RB rows cost
// less than the occupancy a row-sum buffer would take.
template <int TH, int THREADS, int KG, int NDK, bool VEC>
__device__ __forceinline__ void batch_gauss(const float* __restrict__ S, const float (&gw)[KG], int lane, int warp,
                                            int64_t x0, int64_t y0, int64_t H, int64_t W, float nd_in,
                                            float nd_out, const BatchTileDev& T) {
  using L = BatchSmem<TH, THREADS, KG>;
  constexpr int WARPS = THREADS / 32;
  constexpr int RB = TH / WARPS;
  constexpr int HY = L::HY;
  constexpr int R = KG / 2;
  const int c0 = 4 * lane;
  const int q0 = warp * RB;  // first output row of this warp
  // window columns of this lane inside the tile (bit j: column x0 + c0 - R + j)
  uint32_t colbits = 0;
#pragma unroll
  for (int j = 0; j < 4 + KG - 1; ++j) {
    const int64_t gx = x0 + c0 - R + j;
    colbits |= static_cast<uint32_t>(gx >= 0 && gx < W) << j;
  }
  // staged rows inside the tile: [first_in, rows_in)
  const int64_t hin = H - y0 + HY;
  const int rows_in = static_cast<int>(hin < L::SR ? hin : int64_t(L::SR));
  const int first_in = y0 >= HY ? 0 : static_cast<int>(HY - y0);
  const int nrows = static_cast<int>(H - y0 < TH ? H - y0 : int64_t(TH));  // output rows inside the tile
  const int64_t xs = x0 + c0;
  const int ncols = static_cast<int>(W - xs < 4 ? (W - xs > 0 ? W - xs : 0) : 4);
  float2 win[KG][4];
#pragma unroll
  for (int i = 0; i < RB + KG - 1; ++i) {
    const int r = q0 + i + HY - R;  // staged row of this horizontal pass
    const uint32_t bits = (r >= first_in && r < rows_in) ? colbits : 0u;
    const float* sp = S + r * kSW + c0 + 4 - R;
    float2 zv[4 + KG - 1];
#pragma unroll
    for (int j = 0; j < 4 + KG - 1; ++j) {
      const float v = sp[j];
      const bool ok = ((bits >> j) & 1u) && !is_nd_k<NDK>(v, nd_in);
      const float o = ok ? 1.0f : 0.0f;
      zv[j] = make_float2(v * o, o);
    }
#pragma unroll
    for (int t = 0; t < KG - 1; ++t)
#pragma unroll
      for (int u = 0; u < 4; ++u) win[t][u] = win[t + 1][u];
#pragma unroll
    for (int u = 0; u < 4; ++u) win[KG - 1][u] = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int t = 0; t < KG; ++t) {
      const float2 w2 = make_float2(gw[t], gw[t]);
#pragma unroll
      for (int u = 0; u < 4; ++u) win[KG - 1][u] = fma2(w2, zv[u + t], win[KG - 1][u]);
    }
    if (i >= KG - 1) {
      const int q = q0 + i - (KG - 1);  // output row
      if (q < nrows && ncols > 0) {
        float o4[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
          for (int t = 0; t < KG; ++t) acc = fma2(make_float2(gw[t], gw[t]), win[t][u], acc);
          const bool centre_ok = !is_nd_k<NDK>(S[(q + HY) * kSW + c0 + 4 + u], nd_in);
          o4[u] = (centre_ok && acc.y > 0.0f) ? __fdividef(acc.x, acc.y) : nd_out;
        }
        float* out = T.smooth + (y0 + q) * T.out_pitch + xs;
        if (VEC && ncols == 4) {
          __stcs(reinterpret_cast<float4*>(out), make_float4(o4[0], o4[1], o4[2], o4[3]));
        } else {
#pragma unroll
          for (int u = 0; u < 4; ++u)
            if (u < ncols) out[u] = o4[u];
        }
      }
    }
  }
}

constexpr int kBatchSmemTiles = 1024;  // tiles whose prefix sums are searched in shared memory

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
  float* Sbuf = bsm;  // 2 x SR x kSW staged values (double buffered)
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
    // 4-column groups (16 B) or pairs (8 B) entirely inside the tile take one
    // copy; the rest (the tile's left and right edges) are clamped per element
    const int64_t W = P.width;
    for (int r = warp; r < SR; r += WARPS) {
      const int64_t gy = min(max(y0 - HY + r, int64_t(0)), P.height - 1);
      const float* rowp = T.src + gy * P.in_pitch;
      float* srow = S + r * kSW;
      if (T.stage == 16) {
        for (int gq = lane; gq < kSW / 4; gq += 32) {
          const int64_t gx0 = x0 - 4 + 4 * gq;
          if (gx0 >= 0 && gx0 + 3 < W) {
            cp_async16(srow + 4 * gq, rowp + gx0);
          } else {
#pragma unroll
            for (int e = 0; e < 4; ++e) cp_async4(srow + 4 * gq + e, rowp + min(max(gx0 + e, int64_t(0)), W - 1));
          }
        }
      } else if (T.stage == 8) {
        for (int gq = lane; gq < kSW / 2; gq += 32) {
          const int64_t gx0 = x0 - 4 + 2 * gq;
          if (gx0 >= 0 && gx0 + 1 < W) {
            cp_async8(srow + 2 * gq, rowp + gx0);
          } else {
            cp_async4(srow + 2 * gq, rowp + min(max(gx0, int64_t(0)), W - 1));
            cp_async4(srow + 2 * gq + 1, rowp + min(max(gx0 + 1, int64_t(0)), W - 1));
          }
        }
      } else {
        const bool inside = x0 - 4 >= 0 && x0 + kSW - 4 <= W;
#pragma unroll
        for (int c = lane; c < kSW; c += 32) {
          const int64_t gx = inside ? x0 - 4 + c : min(max(x0 - 4 + c, int64_t(0)), W - 1);
          cp_async4(srow + c, rowp + gx);
        }
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

    const bool edge = x0 + kTW > W || y0 + TH > H;
    const MaskRule rule = mask_rule(P);

    // Horn slope + aspect.
    if (T.slope || T.aspect) {
      const int64_t xs = x0 + 4 * lane;
      const float* Sh = S + (HY - 1) * kSW;
      const RowPtrs g = global_rows(T.slope, T.aspect, nullptr, P, y0 + warp * RB, xs);
      // both outputs are requested together in the batch plan
      if (T.vec) {
        if (edge) batch_horn_rows<RB, true, true>(Sh, lane, warp * RB, y0, xs, P, rule, nd_in, g.s, g.a, P.out_pitch);
        else batch_horn_rows<RB, false, true>(Sh, lane, warp * RB, y0, xs, P, rule, nd_in, g.s, g.a, P.out_pitch);
      } else {
        batch_horn_rows<RB, true, false>(Sh, lane, warp * RB, y0, xs, P, rule, nd_in, g.s, g.a, P.out_pitch);
      }
    }

    // Gaussian KG x KG (normalised, nodata-aware, out-of-bounds taps skipped).
    if (T.smooth) {
      const bool vec = T.vec_smooth != 0;
      if (P.nd_kind == VSR_NODATA_VALUE) {
        if (vec) batch_gauss<TH, THREADS, KG, VSR_NODATA_VALUE, true>(S, gw, lane, warp, x0, y0, H, W, nd_in, P.nd_out_f, T);
        else batch_gauss<TH, THREADS, KG, VSR_NODATA_VALUE, false>(S, gw, lane, warp, x0, y0, H, W, nd_in, P.nd_out_f, T);
      } else if (P.nd_kind == VSR_NODATA_NAN) {
        if (vec) batch_gauss<TH, THREADS, KG, VSR_NODATA_NAN, true>(S, gw, lane, warp, x0, y0, H, W, nd_in, P.nd_out_f, T);
        else batch_gauss<TH, THREADS, KG, VSR_NODATA_NAN, false>(S, gw, lane, warp, x0, y0, H, W, nd_in, P.nd_out_f, T);
      } else {
        if (vec) batch_gauss<TH, THREADS, KG, VSR_NODATA_NONE, true>(S, gw, lane, warp, x0, y0, H, W, nd_in, P.nd_out_f, T);
        else batch_gauss<TH, THREADS, KG, VSR_NODATA_NONE, false>(S, gw, lane, warp, x0, y0, H, W, nd_in, P.nd_out_f, T);
      }
    }
    __syncthreads();  // every read of buffer b and of its item slots is done before they are reassigned
  }
  cp_async_wait<0>();  // no copy may land after the CTA leaves
}

// Launch configurations the autotuner chooses between: (rows per block,
// threads per CTA); the Gaussian width is a template parameter too.
struct BatchConfig {
  int th, threads;
};
constexpr BatchConfig kBatchConfigs[] = {{32, 128}, {48, 128}, {64, 256}, {16, 128}};
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
    case 1: return launch_batch_t<48, 128, KG>(hdr, tiles, st);
    case 2: return launch_batch_t<64, 256, KG>(hdr, tiles, st);
    case 3: return launch_batch_t<16, 128, KG>(hdr, tiles, st);
    default: return launch_batch_t<32, 128, KG>(hdr, tiles, st);
  }
}

}  // namespace bk
}  // namespace vsr
