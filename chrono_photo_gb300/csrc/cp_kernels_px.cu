// One pixel-thread outlier kernel family chosen at compile time (the build compiles this file
// once per entry of CP_PX_VARIANTS in cp_internal.h): distance kind CP_KIND (1 integer,
// 2 paired f32), outlier group CP_OG (1 extreme / first / last, 2 average, 3 forward /
// backward) and background CP_BG (0 any, 1 first). Separate translation units keep the build
// parallel.
#include "cp_outlier_px.cuh"

#if !defined(CP_KIND) || !defined(CP_OG) || !defined(CP_BG)
#error "CP_KIND, CP_OG and CP_BG must be defined"
#endif

#define CP_PCAT_(a, b, c, d, e, f) a##b##c##d##e##f
#define CP_PCAT(a, b, c, d, e, f) CP_PCAT_(a, b, c, d, e, f)

namespace cp {

int CP_PCAT(px_launch_k, CP_KIND, _g, CP_OG, _b, CP_BG)(const StackDev& s, int pa, bool db,
                                                       bool occupancy_only, int grid, int smem,
                                                       void* stream, uint32_t* error) {
  return px_dispatch<CP_KIND, CP_OG, CP_BG>(s, pa, db, occupancy_only, grid, smem, stream, error);
}

}  // namespace cp
