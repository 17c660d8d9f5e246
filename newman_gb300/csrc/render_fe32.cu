// FP32 mantissa + int exponent (floatexp) perturbation kernel.
#include "engine.hpp"

namespace nmg {

int fe32_blocks_per_sm() { return 1; }

cudaError_t launch_fe32(const DeviceView&, const RenderCtl&, cudaStream_t, int, int) {
  return cudaErrorNotSupported;
}

}  // namespace nmg
