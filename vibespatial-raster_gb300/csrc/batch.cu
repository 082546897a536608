// One persistent, work-queue-scheduled launch over many DEM tiles of uneven
// sizes (vsr_batch_plan / vsr_batch_run).
#include <mutex>
#include <unordered_map>
#include <vector>

#include "batch_kernel.cuh"

namespace vsr {
namespace bk {
// instantiated in batch_k1_3.cu, batch_k5.cu, batch_k7_9.cu
extern template int launch_batch_kg<1>(int, BatchHeader*, const BatchTileDev*, cudaStream_t);
extern template int launch_batch_kg<3>(int, BatchHeader*, const BatchTileDev*, cudaStream_t);
extern template int launch_batch_kg<5>(int, BatchHeader*, const BatchTileDev*, cudaStream_t);
extern template int launch_batch_kg<7>(int, BatchHeader*, const BatchTileDev*, cudaStream_t);
extern template int launch_batch_kg<9>(int, BatchHeader*, const BatchTileDev*, cudaStream_t);
}  // namespace bk

namespace {

using namespace bk;

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

int batch_config_count() { return bk::kNumBatchConfigs; }

}  // namespace vsr

extern "C" size_t vsr_batch_plan_size(int n_tiles) {
  if (n_tiles <= 0) return 0;
  return ((sizeof(vsr::bk::BatchHeader) + 255) & ~size_t(255)) +
         static_cast<size_t>(n_tiles) * sizeof(vsr::bk::BatchTileDev);
}

extern "C" int vsr_batch_plan(const vsr_batch_tile* tiles_host, int n_tiles, double sigma, int gauss_k, void* plan,
                              size_t plan_bytes, int64_t* total_items, void* stream) {
  using namespace vsr;
  using namespace vsr::bk;
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
    d.stage = (aligned(t.src, 16) && t.pitch % 4 == 0) ? 16 : ((aligned(t.src, 8) && t.pitch % 2 == 0) ? 8 : 4);
    d.vec_smooth = t.smooth && aligned(t.smooth, 16) && t.out_pitch % 4 == 0;
    d.pad_ = 0;
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
  using namespace vsr::bk;
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
