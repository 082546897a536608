// The fused Horn kernel for float32 rasters with 16-byte aligned rows
// (horn_f32_tma) and its launch, templated on the wanted outputs; each
// translation unit that includes this header instantiates some output sets
// (horn_tma_all.cu: slope + aspect + hillshade; horn_tma_sub.cu: the others),
// so the instantiations compile in parallel.
//
// Persistent CTAs walk the 128 x TH output tiles of every band (band-major);
// each tile plus a 4-column / 1-row halo is staged into shared memory by a
// 3-D TMA load (x, y, band; multi-stage mbarrier pipeline), edge replication
// is patched in shared memory on border tiles, each lane computes 4 adjacent pixels per row from a rolling 3-row
// register window (horn_rows) and writes 128-bit slope/aspect and 32-bit
// hillshade streaming stores.
#pragma once

#include "horn_common.cuh"

namespace vsr {
namespace horn {

template <int TH>
struct TmaTile {
  static constexpr int SH = TH + 2;
  static constexpr uint32_t kBytes = kSW * SH * 4;
  static constexpr uint32_t kStride = (kBytes + 1023u) & ~1023u;
};

template <int TH, int STAGES, int THREADS, int WANT, int NDK, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) horn_f32_tma(const __grid_constant__ CUtensorMap tmap,
                                                              const HornParams P, const float nd_in,
                                                              float* __restrict__ slope,
                                                              float* __restrict__ aspect,
                                                              uint8_t* __restrict__ hs, uint32_t* err_word) {
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
  const int64_t per_band = tiles_x * ((H + TH - 1) / TH);
  const int64_t total = per_band * P.bands;
  const MaskRule rule = mask_rule(P);

  auto issue = [&](int64_t t, int s) {
    const int64_t b = t / per_band, r = t - b * per_band;
    const int64_t ty = r / tiles_x, tx = r - ty * tiles_x;
    mbar_arrive_expect_tx(&bars[s], Tile::kBytes);
    tma_load_3d(reinterpret_cast<unsigned char*>(stages) + s * Tile::kStride, &tmap, static_cast<int>(tx * kTW - 4),
                static_cast<int>(ty * TH - 1), static_cast<int>(b), &bars[s]);
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
    const int64_t b = t / per_band, rem = t - b * per_band;
    const int64_t ty = rem / tiles_x, tx = rem - ty * tiles_x;
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
    if (left || right || top || bottom) __syncthreads();

    const int64_t xs = x0 + 4 * lane;
    const int r0 = warp * RB;
    const bool edge = x0 + kTW > W || y0 + TH > H;
    const RowPtrs g = global_rows(slope ? slope + b * P.out_band_stride : nullptr,
                                  aspect ? aspect + b * P.out_band_stride : nullptr,
                                  hs ? hs + b * P.hs_band_stride : nullptr, P, y0 + r0, xs);
    if (edge) horn_rows<RB, WANT, NDK, true, true>(S, lane, r0, y0, xs, P, rule, nd_in, g.s, g.a, g.h, P.out_pitch, P.hs_pitch);
    else horn_rows<RB, WANT, NDK, false, true>(S, lane, r0, y0, xs, P, rule, nd_in, g.s, g.a, g.h, P.out_pitch, P.hs_pitch);

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

template <int TH, int STAGES, int THREADS, int WANT, int NDK, int MINB>
int launch_tma_t(const CUtensorMap& map, const HornParams& P, float nd_in, float* slope, float* aspect,
                 uint8_t* hs, uint32_t* err, cudaStream_t st) {
  using Tile = TmaTile<TH>;
  const size_t smem = STAGES * Tile::kStride + 1024;
  auto kern = horn_f32_tma<TH, STAGES, THREADS, WANT, NDK, MINB>;
  VSR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  int per_sm = 0;
  VSR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, THREADS, smem));
  if (per_sm < 1) return fail(VSR_ERR_CUDA, "horn_f32_tma cannot be resident (smem %zu)", smem);
  const int64_t tiles = ((P.width + kTW - 1) / kTW) * ((P.height + TH - 1) / TH) * P.bands;
  const int64_t grid = std::min<int64_t>(tiles, static_cast<int64_t>(sm_count()) * per_sm);
  kern<<<static_cast<unsigned>(grid), THREADS, smem, st>>>(map, P, nd_in, slope, aspect, hs, err);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}

template <int TH, int STAGES, int THREADS, int WANT, int MINB>
int launch_tma_kind(const CUtensorMap& map, const HornParams& P, float nd_in, float* slope, float* aspect,
                    uint8_t* hs, uint32_t* err, cudaStream_t st) {
  switch (P.nd_kind) {
    case VSR_NODATA_VALUE:
      return launch_tma_t<TH, STAGES, THREADS, WANT, VSR_NODATA_VALUE, MINB>(map, P, nd_in, slope, aspect, hs, err, st);
    case VSR_NODATA_NAN:
      return launch_tma_t<TH, STAGES, THREADS, WANT, VSR_NODATA_NAN, MINB>(map, P, nd_in, slope, aspect, hs, err, st);
    default:
      return launch_tma_t<TH, STAGES, THREADS, WANT, VSR_NODATA_NONE, MINB>(map, P, nd_in, slope, aspect, hs, err, st);
  }
}

// Launch configurations of the TMA kernel the autotuner chooses between
// (kHornConfigs in horn.cu): output rows per tile, pipeline stages, threads
// per CTA, CTAs per SM the register budget is sized for.  The tuner times
// the full output set; the partial sets (one or two outputs: less work per
// pixel, so the memory-bound shape) are compiled for the 64-row shape only.
template <int WANT>
int launch_tma_want(int cfg, const CUtensorMap& map, const HornParams& P, float nd_in, float* slope, float* aspect,
                    uint8_t* hs, uint32_t* err, cudaStream_t st) {
  if constexpr (WANT == 7) {
    switch (cfg) {
      case 1: return launch_tma_kind<48, 2, 128, WANT, 4>(map, P, nd_in, slope, aspect, hs, err, st);
      case 2: return launch_tma_kind<32, 2, 128, WANT, 4>(map, P, nd_in, slope, aspect, hs, err, st);
      case 3: return launch_tma_kind<32, 2, 128, WANT, 5>(map, P, nd_in, slope, aspect, hs, err, st);
      case 4: return launch_tma_kind<64, 2, 256, WANT, 2>(map, P, nd_in, slope, aspect, hs, err, st);
      default: return launch_tma_kind<64, 2, 128, WANT, 4>(map, P, nd_in, slope, aspect, hs, err, st);
    }
  }
  (void)cfg;
  return launch_tma_kind<64, 2, 128, WANT, 4>(map, P, nd_in, slope, aspect, hs, err, st);
}

}  // namespace horn
}  // namespace vsr
