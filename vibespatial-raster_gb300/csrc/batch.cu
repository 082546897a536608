// One persistent, work-queue-scheduled launch over many DEM tiles of uneven
// sizes (vsr_batch_plan / vsr_batch_run).
#include <mutex>
#include <unordered_map>
#include <vector>

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
// (TH + 2*HY) x 136 input values one item ahead with cp.async -- 16-byte
// copies for the 4-column groups inside a 16-byte aligned tile, clamped
// 4-byte copies elsewhere (any pitch or alignment; edge replication for
// Horn) -- runs the Horn rows on them, then the separable Gaussian: a row
// pass into shared memory that forms (numerator, weight sum) pairs with
// packed f32x2 FMAs (validity from coordinates and nodata, so out-of-bounds
// taps are skipped), then a column pass down each column with a rolling
// window of KG row sums in registers.
namespace vsr {
namespace {

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
  int32_t vec_in;      // source 16-byte aligned with pitch % 4 == 0 (16-byte staging copies)
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
  static constexpr int RG = TH + 2 * (KG / 2);        // row-pass rows of the Gaussian
  static constexpr int kFloats = 2 * SR * kSW + 2 * RG * kTW;  // staging x 2, row-pass pairs
};


constexpr int kBatchSmemTiles = 2048;  // tiles whose prefix sums are searched in shared memory

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
  float* Sbuf = bsm;                                         // 2 x SR x kSW staged values (double buffered)
  float2* Rg = reinterpret_cast<float2*>(Sbuf + 2 * SR * kSW);  // RG x kTW (numerator, weight sum) row sums
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
    if (T.vec_in) {
      for (int r = warp; r < SR; r += WARPS) {
        const int64_t gy = min(max(y0 - HY + r, int64_t(0)), P.height - 1);
        const float* rowp = T.src + gy * P.in_pitch;
        for (int gq = lane; gq < kSW / 4; gq += 32) {
          const int64_t gx0 = x0 - 4 + 4 * gq;
          float* d = S + r * kSW + 4 * gq;
          if (gx0 >= 0 && gx0 + 3 < P.width) {
            cp_async16(d, rowp + gx0);
          } else {
#pragma unroll
            for (int e = 0; e < 4; ++e) cp_async4(d + e, rowp + min(max(gx0 + e, int64_t(0)), P.width - 1));
          }
        }
      }
    } else {
      for (int r = warp; r < SR; r += WARPS) {
        const int64_t gy = min(max(y0 - HY + r, int64_t(0)), P.height - 1);
        const float* rowp = T.src + gy * P.in_pitch;
#pragma unroll
        for (int c = lane; c < kSW; c += 32) {
          const int64_t gx = min(max(x0 - 4 + c, int64_t(0)), P.width - 1);
          cp_async4(S + r * kSW + c, rowp + gx);
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
      constexpr int R = KG / 2;
      // row pass: row-sum row rr = staged row rr + HY - R; 4 columns per lane,
      // (v * valid, valid) pairs summed with packed FMAs (NaN * 0 stays NaN,
      // as in the reference)
      const int c0 = 4 * lane;
      for (int rr = warp; rr < L::RG; rr += WARPS) {
        const int r = rr + HY - R;
        const int64_t gy = y0 - HY + r;
        const bool row_in = gy >= 0 && gy < H;
        const float* sp = S + r * kSW + c0 + 4 - R;
        float2 zv[4 + KG - 1];
#pragma unroll
        for (int j = 0; j < 4 + KG - 1; ++j) {
          const float v = sp[j];
          const int64_t gx = x0 + c0 - R + j;
          const bool ok = row_in && gx >= 0 && gx < W && !is_nd_rt(v, P.nd_kind, nd_in);
          const float o = ok ? 1.0f : 0.0f;
          zv[j] = make_float2(v * o, o);
        }
        float2 acc[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) acc[u] = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int t = 0; t < KG; ++t) {
          const float2 w2 = make_float2(gw[t], gw[t]);
#pragma unroll
          for (int u = 0; u < 4; ++u) acc[u] = fma2(w2, zv[u + t], acc[u]);
        }
        float4* dst = reinterpret_cast<float4*>(Rg + rr * kTW + c0);
        dst[0] = make_float4(acc[0].x, acc[0].y, acc[1].x, acc[1].y);
        dst[1] = make_float4(acc[2].x, acc[2].y, acc[3].x, acc[3].y);
      }
      __syncthreads();
      // column pass: column c, RY consecutive output rows, the KG row sums of
      // the current window held in registers
      constexpr int GROUPS = THREADS / kTW;
      constexpr int RY = TH / GROUPS;
      const int c = tid % kTW;
      const int q0 = (tid / kTW) * RY;
      const int64_t x = x0 + c;
      float2 win[KG];
#pragma unroll
      for (int t = 0; t < KG - 1; ++t) win[t] = Rg[(q0 + t) * kTW + c];
#pragma unroll
      for (int i = 0; i < RY; ++i) {
        win[KG - 1] = Rg[(q0 + i + KG - 1) * kTW + c];
        float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int t = 0; t < KG; ++t) acc = fma2(make_float2(gw[t], gw[t]), win[t], acc);
#pragma unroll
        for (int t = 0; t < KG - 1; ++t) win[t] = win[t + 1];
        const int q = q0 + i;
        const int64_t y = y0 + q;
        if (y < H && x < W) {
          const float cv = S[(q + HY) * kSW + c + 4];
          const bool centre_ok = !is_nd_rt(cv, P.nd_kind, nd_in);
          T.smooth[y * T.out_pitch + x] = (centre_ok && acc.y > 0.0f) ? acc.x / acc.y : P.nd_out_f;
        }
      }
    }
    __syncthreads();  // row-pass sums are reused by the next item; buffer b is refilled after the next barrier
  }
  cp_async_wait<0>();  // no copy may land after the CTA leaves
}

// Launch configurations the autotuner chooses between: (rows per block,
// threads per CTA); the Gaussian width is a template parameter too.
struct BatchConfig {
  int th, threads;
};
constexpr BatchConfig kBatchConfigs[] = {{32, 256}, {64, 256}, {16, 128}, {32, 128}};
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
    case 1: return launch_batch_t<64, 256, KG>(hdr, tiles, st);
    case 2: return launch_batch_t<16, 128, KG>(hdr, tiles, st);
    case 3: return launch_batch_t<32, 128, KG>(hdr, tiles, st);
    default: return launch_batch_t<32, 256, KG>(hdr, tiles, st);
  }
}

// Per-tile 1 / (8 cell) in FP64 on the device (the cell sizes come from each
// tile's affine transform).
__global__ void prep_batch_cells(BatchTileDev* tiles, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  tiles[i].inv8cx = static_cast<float>(1.0 / (8.0 * tiles[i].cell_x));
  tiles[i].inv8cy = static_cast<float>(1.0 / (8.0 * tiles[i].cell_y));
}

__global__ void prep_batch_gauss(BatchHeader* hdr, int kg, double sigma) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int i = 0; i < kg; ++i) {
    const double a = (i - kg / 2) / sigma;
    const double g = exp(-0.5 * a * a);
    hdr->g[i] = static_cast<float>(g);
    s += static_cast<double>(static_cast<float>(g));
  }
  hdr->gsum = static_cast<float>(s);
}

// Launch shape of every plan built in this process, keyed by the plan's
// device address: vsr_batch_run launches the configuration the plan was
// built for, whatever the tuning table holds by then.
struct PlanShape {
  int cfg, kg;
};
std::mutex g_plan_mutex;
std::unordered_map<const void*, PlanShape> g_plans;

}  // namespace

int batch_config_count() { return kNumBatchConfigs; }

}  // namespace vsr

extern "C" size_t vsr_batch_plan_size(int n_tiles) {
  if (n_tiles <= 0) return 0;
  return ((sizeof(vsr::BatchHeader) + 255) & ~size_t(255)) + static_cast<size_t>(n_tiles) * sizeof(vsr::BatchTileDev);
}

extern "C" int vsr_batch_plan(const vsr_batch_tile* tiles_host, int n_tiles, double sigma, int gauss_k, void* plan,
                              size_t plan_bytes, int64_t* total_items, void* stream) {
  using namespace vsr;
  if (n_tiles <= 0 || !tiles_host) return fail(VSR_ERR_INVALID_ARG, "need at least one tile");
  if (gauss_k != 0 && (gauss_k < 1 || gauss_k > kBatchMaxKG || gauss_k % 2 == 0))
    return fail(VSR_ERR_UNSUPPORTED, "batch Gaussian size must be odd and <= %d", kBatchMaxKG);
  if (gauss_k != 0 && !(sigma > 0.0)) return fail(VSR_ERR_INVALID_ARG, "sigma must be positive, got %g", sigma);
  const size_t need = vsr_batch_plan_size(n_tiles);
  if (!plan || plan_bytes < need || !aligned(plan, 256))
    return fail(VSR_ERR_WORKSPACE, "plan must be 256-byte aligned and >= %zu bytes", need);
  const int cfg = tuning_get(VSR_OP_BATCH);
  const int th = kBatchConfigs[cfg].th;
  std::vector<BatchTileDev> dev(n_tiles);
  int64_t items = 0;
  for (int i = 0; i < n_tiles; ++i) {
    const vsr_batch_tile& t = tiles_host[i];
    if (t.height <= 0 || t.width <= 0 || !t.src) return fail(VSR_ERR_INVALID_ARG, "tile %d is empty or NULL", i);
    if (t.pitch < t.width || t.out_pitch < t.width) return fail(VSR_ERR_INVALID_ARG, "tile %d: pitch < width", i);
    if (!(t.cell_x > 0.0) || !(t.cell_y > 0.0)) return fail(VSR_ERR_INVALID_ARG, "tile %d: cell sizes must be positive", i);
    if ((t.slope == nullptr) != (t.aspect == nullptr))
      return fail(VSR_ERR_INVALID_ARG, "tile %d: slope and aspect are produced together", i);
    if (!aligned(t.src, 4) || (t.slope && !aligned(t.slope, 4)) || (t.aspect && !aligned(t.aspect, 4)) ||
        (t.smooth && !aligned(t.smooth, 4)))
      return fail(VSR_ERR_INVALID_ARG, "tile %d: buffers must be 4-byte aligned", i);
    if (t.smooth && gauss_k == 0) return fail(VSR_ERR_INVALID_ARG, "tile %d wants a Gaussian but gauss_k is 0", i);
    BatchTileDev& d = dev[i];
    d.src = t.src;
    d.H = t.height;
    d.W = t.width;
    d.pitch = t.pitch;
    d.slope = t.slope;
    d.aspect = t.aspect;
    d.smooth = t.smooth;
    d.out_pitch = t.out_pitch;
    d.cell_x = t.cell_x;
    d.cell_y = t.cell_y;
    d.nodata = t.nodata;
    double ev = 0.0;
    d.nd_kind = resolve_nodata(VSR_F32, t.nodata, t.nodata_kind, &ev);
    d.flags = t.flags;
    d.vec = (!t.slope || (aligned(t.slope, 16) && aligned(t.aspect, 16))) && t.out_pitch % 4 == 0;
    d.inv8cx = d.inv8cy = 0.0f;  // set on the device by prep_batch_cells
    d.vec_in = aligned(t.src, 16) && t.pitch % 4 == 0;
    d.items_x = (t.width + kTW - 1) / kTW;
    d.first_item = items;
    items += d.items_x * ((t.height + th - 1) / th);
  }
  BatchHeader h{};
  h.counter = 0;
  h.total_items = items;
  h.n_tiles = n_tiles;
  h.kg = gauss_k;
  h.th = th;
  h.threads = kBatchConfigs[cfg].threads;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* base = static_cast<char*>(plan);
  const size_t off = (sizeof(BatchHeader) + 255) & ~size_t(255);
  VSR_CUDA_TRY(cudaMemcpyAsync(base, &h, sizeof(h), cudaMemcpyHostToDevice, st));
  VSR_CUDA_TRY(cudaMemcpyAsync(base + off, dev.data(), dev.size() * sizeof(BatchTileDev), cudaMemcpyHostToDevice, st));
  prep_batch_cells<<<(n_tiles + 127) / 128, 128, 0, st>>>(reinterpret_cast<BatchTileDev*>(base + off), n_tiles);
  VSR_CUDA_TRY(cudaGetLastError());
  if (gauss_k) {
    prep_batch_gauss<<<1, 32, 0, st>>>(reinterpret_cast<BatchHeader*>(base), gauss_k, sigma);
    VSR_CUDA_TRY(cudaGetLastError());
  }
  VSR_CUDA_TRY(cudaStreamSynchronize(st));  // the host descriptors are staged from pageable memory
  {
    std::lock_guard<std::mutex> lk(g_plan_mutex);
    g_plans[plan] = PlanShape{cfg, gauss_k};
  }
  if (total_items) *total_items = items;
  return VSR_OK;
}

extern "C" int vsr_batch_run(void* plan, int gauss_k, void* stream) {
  using namespace vsr;
  if (!plan || !aligned(plan, 256)) return fail(VSR_ERR_INVALID_ARG, "plan must be a 256-byte aligned device pointer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  BatchHeader* hdr = static_cast<BatchHeader*>(plan);
  const BatchTileDev* tiles = reinterpret_cast<const BatchTileDev*>(static_cast<char*>(plan) + ((sizeof(BatchHeader) + 255) & ~size_t(255)));
  PlanShape shape{};
  {
    std::lock_guard<std::mutex> lk(g_plan_mutex);
    const auto it = g_plans.find(plan);
    if (it == g_plans.end())
      return fail(VSR_ERR_INVALID_ARG, "plan %p was not built by vsr_batch_plan in this process", plan);
    shape = it->second;
  }
  if (gauss_k != shape.kg)
    return fail(VSR_ERR_INVALID_ARG, "gauss_k %d does not match the plan's %d", gauss_k, shape.kg);
  VSR_CUDA_TRY(cudaMemsetAsync(&hdr->counter, 0, sizeof(hdr->counter), st));
  const int cfg = shape.cfg;
  switch (gauss_k) {
    case 0:
    case 1: return launch_batch_kg<1>(cfg, hdr, tiles, st);
    case 3: return launch_batch_kg<3>(cfg, hdr, tiles, st);
    case 5: return launch_batch_kg<5>(cfg, hdr, tiles, st);
    case 7: return launch_batch_kg<7>(cfg, hdr, tiles, st);
    case 9: return launch_batch_kg<9>(cfg, hdr, tiles, st);
    default: return fail(VSR_ERR_UNSUPPORTED, "batch Gaussian size must be odd and <= %d", kBatchMaxKG);
  }
}
