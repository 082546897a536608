// horn_f32_tma instantiated for slope + aspect + hillshade (the fused
// terrain pass), every launch configuration of the tuning table.
#include "horn_tma.cuh"

namespace vsr {
namespace horn {
template int launch_tma_want<7>(int, const CUtensorMap&, const HornParams&, float, float*, float*, uint8_t*,
                                uint32_t*, cudaStream_t);
}  // namespace horn
}  // namespace vsr
