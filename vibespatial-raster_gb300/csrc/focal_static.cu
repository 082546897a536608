// vsr_convolve_noalloc: the normalised focal convolution for callers that
// cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc, and cannot hand us a
// workspace either: a serving process whose device memory budget was fixed
// when it started, or a host that reaches this library through a plugin
// boundary (ctypes / cgo / JNI) with no access to the process's device
// allocator.  For them this entry point takes only the inputs and the output;
// its scratch (the staged float64 weights, the float32 or split-precision
// operand images built from them, and the tensor-core path's largest-value
// word) lives in a file-scope __device__ array sized for the largest
// supported kernel of either precision.  Every GPU that loads the library
// holds that array (kNoAllocScratchBytes, 350.5 KiB) until the process exits.
//
// Host code cannot use the array's name as a device address, so on the first
// call on each device (with that device current) the address is resolved
// with cudaGetSymbolAddress and cached; make that first call before any
// stream capture.  All calls share the one array and it keeps the last
// call's contents: each call rewrites every byte it reads, and the one word
// that must start at zero (the tensor-core path's largest |value|) is
// cleared by a cudaMemsetAsync on the caller's stream.  Calls whose kernels
// overlap on the GPU -- e.g. on two streams at once -- race on it.
#include <mutex>

#include "vsr_internal.cuh"

namespace vsr {

namespace {

constexpr int kNoAllocMaxK = 80;
// The larger of the two workspaces vsr_convolve can ask for:
//  * FP32 path, 80 x 80: 51,200 B float64 weights + 25,600 B float32 rows +
//    256 B for the total = 77,056 B;
//  * tensor-core path, 41 x 41: 13,568 B float64 weights + 330,752 B
//    Toeplitz band images (three bands of 21 core matrices per kernel row) +
//    14,336 B float64 summed-area table + 256 B for the largest-value word
//    = 358,912 B.
constexpr size_t kNoAllocScratchBytes = 358912;

static __device__ __align__(256) unsigned char g_conv_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_scratch_ptr[kMaxDevices];

void* scratch_for_current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    set_error("cudaGetDevice failed or device index out of range");
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_conv_scratch);
    if (e != cudaSuccess) {
      cuda_fail(e, "cudaGetSymbolAddress(convolution scratch)");
      return nullptr;
    }
    g_scratch_ptr[dev] = p;
  }
  return g_scratch_ptr[dev];
}

}  // namespace
}  // namespace vsr

extern "C" int vsr_convolve_noalloc(const void* src, int dtype, int64_t height, int64_t width, int64_t pitch,
                                    const double* weights_host, int kh, int kw, double nodata,
                                    int nodata_kind, void* dst, int out_dtype, int64_t out_pitch,
                                    int precision, void* stream) {
  using namespace vsr;
  if (kh > kNoAllocMaxK || kw > kNoAllocMaxK)
    return fail(VSR_ERR_UNSUPPORTED, "vsr_convolve_noalloc: kernel %dx%d exceeds the %dx%d maximum of its static scratch",
                kh, kw, kNoAllocMaxK, kNoAllocMaxK);
  // Whatever path vsr_convolve takes for this kernel and precision (the FP32
  // kernels, or the tensor-core path that AUTO may pick), its workspace must
  // fit the static array.
  if (kh > 0 && kw > 0 && vsr_convolve_workspace_size(kh, kw, precision) > kNoAllocScratchBytes)
    return fail(VSR_ERR_UNSUPPORTED, "vsr_convolve_noalloc: kernel %dx%d needs more than %zu scratch bytes", kh, kw,
                kNoAllocScratchBytes);
  void* ws = scratch_for_current_device();
  if (!ws) return VSR_ERR_CUDA;
  return vsr_convolve(src, dtype, height, width, pitch, weights_host, kh, kw, nodata, nodata_kind, dst, out_dtype,
                      out_pitch, precision, ws, kNoAllocScratchBytes, stream);
}
