// Instantiates the batched-tiles launch for Gaussian widths 5.
#include "batch_kernel.cuh"

namespace vsr {
namespace bk {
template int launch_batch_kg<5>(int, BatchHeader*, const BatchTileDev*, cudaStream_t);
}  // namespace bk
}  // namespace vsr
