// One single-stack outlier kernel chosen at compile time (the build compiles this file once
// per variant): CP_CH channels, distance kind CP_KIND (1 integer, 2 f32) and outlier group
// CP_OG (0 any, 1 extreme / first / last, 2 average, 3 forward / backward). Separate
// translation units keep the build parallel.
#include "cp_tile.cuh"

#if !defined(CP_CH) || !defined(CP_KIND) || !defined(CP_OG)
#error "CP_CH, CP_KIND and CP_OG must be defined"
#endif

#define CP_CAT_(a, b, c, d, e, f) a##b##c##d##e##f
#define CP_CAT(a, b, c, d, e, f) CP_CAT_(a, b, c, d, e, f)

namespace cp {

int CP_CAT(launch_composite_c, CP_CH, _k, CP_KIND, _g, CP_OG)(const StackDev& s, int grid,
                                                              int smem, void* stream,
                                                              uint32_t* error) {
  return launch_composite_kind<CP_CH, CP_KIND, CP_OG>(s, grid, smem, stream, error);
}

int CP_CAT(max_ctas_c, CP_CH, _k, CP_KIND, _g, CP_OG)(int threads, int smem) {
  return max_ctas_kind<CP_CH, CP_KIND, CP_OG>(threads, smem);
}

}  // namespace cp
