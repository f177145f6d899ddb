// The single-stack outlier kernel for 3-channel stacks with abs thresholds with 0/1 weights (exact integer distances).
#include "cp_tile.cuh"

namespace cp {

int launch_composite_int_c3(const StackDev& s, int grid, int smem, void* stream, uint32_t* error) {
  return launch_composite_kind<3, kIntKind>(s, grid, smem, stream, error);
}

}  // namespace cp
