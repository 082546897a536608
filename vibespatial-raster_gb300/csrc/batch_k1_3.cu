// Instantiates the batched-tiles launch for Gaussian widths 1, 3.
#include "batch_kernel.cuh"

namespace vsr {
namespace bk {
template int launch_batch_kg<1>(int, BatchHeader*, const BatchTileDev*, cudaStream_t);
template int launch_batch_kg<3>(int, BatchHeader*, const BatchTileDev*, cudaStream_t);
}  // namespace bk
}  // namespace vsr
