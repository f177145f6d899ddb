// The single-stack outlier kernel for 3-channel stacks with f32 distances (rel thresholds, other weights).
#include "cp_tile.cuh"

namespace cp {

int launch_composite_f32_c3(const StackDev& s, int grid, int smem, void* stream, uint32_t* error) {
  return launch_composite_kind<3, kF32Kind>(s, grid, smem, stream, error);
}

}  // namespace cp
