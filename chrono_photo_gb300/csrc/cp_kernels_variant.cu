// One single-stack outlier kernel chosen at compile time (the build compiles this file once
// per entry of CP_VARIANTS in cp_internal.h): CP_CH channels, distance kind CP_KIND
// (1 integer, 2 paired f32, 3 scalar f32), outlier group CP_OG (0 any, 1 extreme / first /
// last, 2 average, 3 forward / backward) and background CP_BG (0 any, 1 first). Separate
// translation units keep the build parallel.
#include "cp_tile.cuh"

#if !defined(CP_CH) || !defined(CP_KIND) || !defined(CP_OG) || !defined(CP_BG)
#error "CP_CH, CP_KIND, CP_OG and CP_BG must be defined"
#endif

#define CP_CAT_(a, b, c, d, e, f, g, h) a##b##c##d##e##f##g##h
#define CP_CAT(a, b, c, d, e, f, g, h) CP_CAT_(a, b, c, d, e, f, g, h)

namespace cp {

int CP_CAT(launch_composite_c, CP_CH, _k, CP_KIND, _g, CP_OG, _b, CP_BG)(const StackDev& s,
                                                                         int grid, int smem,
                                                                         void* stream,
                                                                         uint32_t* error) {
  return launch_composite_kind<CP_CH, CP_KIND, CP_OG, CP_BG>(s, grid, smem, stream, error);
}

int CP_CAT(max_ctas_c, CP_CH, _k, CP_KIND, _g, CP_OG, _b, CP_BG)(int threads, int smem) {
  return max_ctas_kind<CP_CH, CP_KIND, CP_OG, CP_BG>(threads, smem);
}

}  // namespace cp
