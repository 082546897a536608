// horn_f32_tma instantiated for the partial output sets (slope, aspect or
// hillshade alone, or two of them).
#include "horn_tma.cuh"

namespace vsr {
namespace horn {
#define VSR_HORN_WANT(W)                                                                                    \
  template int launch_tma_want<W>(int, const CUtensorMap&, const HornParams&, float, float*, float*, uint8_t*, \
                                  uint32_t*, cudaStream_t);
VSR_HORN_WANT(1)
VSR_HORN_WANT(2)
VSR_HORN_WANT(3)
VSR_HORN_WANT(4)
VSR_HORN_WANT(5)
VSR_HORN_WANT(6)
#undef VSR_HORN_WANT
}  // namespace horn
}  // namespace vsr
