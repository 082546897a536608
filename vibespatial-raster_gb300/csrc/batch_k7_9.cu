// Instantiates the batched-tiles launch for Gaussian widths 7, 9.
#include "batch_kernel.cuh"

namespace vsr {
namespace bk {
template int launch_batch_kg<7>(int, BatchHeader*, const BatchTileDev*, cudaStream_t);
template int launch_batch_kg<9>(int, BatchHeader*, const BatchTileDev*, cudaStream_t);
}  // namespace bk
}  // namespace vsr
