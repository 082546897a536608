// Library-level entry points: version, per-thread error messages, device
// info, the device-side error word and tensor-map encoding.
#include <cstdarg>
#include <cstring>
#include <atomic>
#include <mutex>

#include "vsr_internal.cuh"

namespace vsr {

static thread_local char t_last_error[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(t_last_error, sizeof(t_last_error), fmt, ap);
  va_end(ap);
}

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(t_last_error, sizeof(t_last_error), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  set_error("%s failed: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
  return VSR_ERR_CUDA;
}

// One word per device that loads the library; kernels OR DeviceError codes
// into it.
static __device__ uint32_t g_device_error_word;

static constexpr int kMaxDevices = 64;
static std::mutex g_dev_mutex;
static uint32_t* g_err_ptr[kMaxDevices];
static int g_sm_count[kMaxDevices];

uint32_t* device_error_word() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    set_error("cudaGetDevice failed or device index out of range");
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_dev_mutex);
  if (!g_err_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_device_error_word);
    if (e != cudaSuccess) {
      cuda_fail(e, "cudaGetSymbolAddress(device error word)");
      return nullptr;
    }
    g_err_ptr[dev] = static_cast<uint32_t*>(p);
  }
  return g_err_ptr[dev];
}

int sm_count() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 0;
  std::lock_guard<std::mutex> lk(g_dev_mutex);
  if (!g_sm_count[dev]) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    g_sm_count[dev] = n;
  }
  return g_sm_count[dev];
}

int resolve_nodata(int dtype, double nodata, int kind, double* as_elem) {
  *as_elem = 0.0;
  if (kind == VSR_NODATA_NONE) return VSR_NODATA_NONE;
  if (kind == VSR_NODATA_NAN || std::isnan(nodata)) {
    // NaN cannot occur in integer rasters; the mask is then all False.
    return (dtype == VSR_F32 || dtype == VSR_F64) ? VSR_NODATA_NAN : VSR_NODATA_NONE;
  }
  double v = nodata;
  switch (dtype) {
    case VSR_F32: {
      float f = static_cast<float>(v);
      if (static_cast<double>(f) != v) return VSR_NODATA_NONE;
      break;
    }
    case VSR_F64: break;
    case VSR_U8:
      if (v != std::floor(v) || v < 0 || v > 255) return VSR_NODATA_NONE;
      break;
    case VSR_I16:
      if (v != std::floor(v) || v < -32768 || v > 32767) return VSR_NODATA_NONE;
      break;
    case VSR_U16:
      if (v != std::floor(v) || v < 0 || v > 65535) return VSR_NODATA_NONE;
      break;
    case VSR_I32:
      if (v != std::floor(v) || v < -2147483648.0 || v > 2147483647.0) return VSR_NODATA_NONE;
      break;
    default: return VSR_NODATA_NONE;
  }
  *as_elem = v;
  return VSR_NODATA_VALUE;
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

int encode_tensor_map_2d(CUtensorMap* map, CUtensorMapDataType type, size_t elem_bytes,
                         const void* base, uint64_t width, uint64_t height, uint64_t pitch_elems,
                         uint32_t box_w, uint32_t box_h) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return fail(VSR_ERR_CUDA, "cuTensorMapEncodeTiled entry point unavailable");
  cuuint64_t dims[2] = {width, height};
  cuuint64_t strides[1] = {pitch_elems * elem_bytes};
  cuuint32_t box[2] = {box_w, box_h};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, type, 2, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return fail(VSR_ERR_CUDA, "cuTensorMapEncodeTiled failed (CUresult %d)", static_cast<int>(r));
  return VSR_OK;
}

int encode_tensor_map_3d(CUtensorMap* map, CUtensorMapDataType type, size_t elem_bytes, const void* base,
                         uint64_t width, uint64_t height, uint64_t depth, uint64_t pitch_elems, uint64_t plane_elems,
                         uint32_t box_w, uint32_t box_h) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return fail(VSR_ERR_CUDA, "cuTensorMapEncodeTiled entry point unavailable");
  cuuint64_t dims[3] = {width, height, depth};
  cuuint64_t strides[2] = {pitch_elems * elem_bytes, plane_elems * elem_bytes};
  cuuint32_t box[3] = {box_w, box_h, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(map, type, 3, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return fail(VSR_ERR_CUDA, "cuTensorMapEncodeTiled (3-D) failed (CUresult %d)", static_cast<int>(r));
  return VSR_OK;
}

// Selected launch configuration per tunable operation (process-wide).
static std::atomic<int> g_tuning[VSR_OP_COUNT];

int tuning_get(int op) { return (op >= 0 && op < VSR_OP_COUNT) ? g_tuning[op].load() : 0; }

}  // namespace vsr

extern "C" {

int vsr_version(void) { return 100; /* 0.1.0 */ }

const char* vsr_last_error(void) { return vsr::t_last_error; }

int vsr_device_info(int* sm_count, int* cc_major, int* cc_minor) {
  int dev = 0;
  VSR_CUDA_TRY(cudaGetDevice(&dev));
  if (sm_count) VSR_CUDA_TRY(cudaDeviceGetAttribute(sm_count, cudaDevAttrMultiProcessorCount, dev));
  if (cc_major) VSR_CUDA_TRY(cudaDeviceGetAttribute(cc_major, cudaDevAttrComputeCapabilityMajor, dev));
  if (cc_minor) VSR_CUDA_TRY(cudaDeviceGetAttribute(cc_minor, cudaDevAttrComputeCapabilityMinor, dev));
  return VSR_OK;
}

int vsr_tuning_count(int op) {
  switch (op) {
    case VSR_OP_HORN: return vsr::horn_config_count();
    case VSR_OP_BATCH: return vsr::batch_config_count();
    default: return 0;
  }
}

int vsr_tuning_set(int op, int config) {
  const int n = vsr_tuning_count(op);
  if (n == 0) return vsr::fail(VSR_ERR_INVALID_ARG, "operation %d has no tunable configurations", op);
  if (config < 0 || config >= n) return vsr::fail(VSR_ERR_INVALID_ARG, "config %d out of range [0, %d)", config, n);
  vsr::g_tuning[op].store(config);
  return VSR_OK;
}

int vsr_tuning_get(int op) { return vsr::tuning_get(op); }

int vsr_poll_device_error(void* stream, uint32_t* code) {
  if (!code) return vsr::fail(VSR_ERR_INVALID_ARG, "code must not be NULL");
  uint32_t* w = vsr::device_error_word();
  if (!w) return VSR_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  VSR_CUDA_TRY(cudaStreamSynchronize(s));
  uint32_t v = 0;
  VSR_CUDA_TRY(cudaMemcpy(&v, w, sizeof(v), cudaMemcpyDeviceToHost));
  if (v) VSR_CUDA_TRY(cudaMemset(w, 0, sizeof(v)));
  *code = v;
  return VSR_OK;
}

}  // extern "C"
