// cp_kernels_multi.cu — instantiations of the multi-setting outlier kernel
// (cp_outlier_multi.cuh) per plane-word count, with and without quartiles.
#include "cp_outlier_multi.cuh"

namespace cp {

int px_multi(const MultiArgs& a, bool rel, bool occupancy_only, int grid, int smem, void* stream,
             uint32_t* error) {
#define CP_MULTI_CASE(NW, REL)                                                      \
  if (a.sets[0].nw == NW && rel == REL)                                             \
    return occupancy_only ? multi_occupancy_t<NW, REL>(smem)                        \
                          : multi_launch_t<NW, REL>(a, grid, smem, stream, error);
  CP_MULTI_CASE(1, false)
  CP_MULTI_CASE(1, true)
  CP_MULTI_CASE(2, false)
  CP_MULTI_CASE(2, true)
  CP_MULTI_CASE(4, false)
  CP_MULTI_CASE(4, true)
#undef CP_MULTI_CASE
  return -1;
}

}  // namespace cp
