// One batched outlier kernel for batches whose stacks all take the same specialised variant
// (the build compiles this file once per entry of CP_BATCH_VARIANTS in cp_internal.h).
#include "cp_tile.cuh"

#if !defined(CP_CH) || !defined(CP_KIND) || !defined(CP_OG) || !defined(CP_BG)
#error "CP_CH, CP_KIND, CP_OG and CP_BG must be defined"
#endif

#define CP_CAT_(a, b, c, d, e, f, g, h) a##b##c##d##e##f##g##h
#define CP_CAT(a, b, c, d, e, f, g, h) CP_CAT_(a, b, c, d, e, f, g, h)

namespace cp {

int CP_CAT(launch_batch_c, CP_CH, _k, CP_KIND, _g, CP_OG, _b, CP_BG)(
    const StackDev* stacks, const int32_t* prefix, int32_t n_stacks, int32_t total,
    int32_t interleave, uint32_t* counter, uint32_t* error, int grid, int smem, void* stream) {
  return launch_batch_kind<CP_CH, CP_KIND, CP_OG, CP_BG>(stacks, prefix, n_stacks, total,
                                                         interleave, counter, error, grid, smem,
                                                         stream);
}

int CP_CAT(batch_max_ctas_c, CP_CH, _k, CP_KIND, _g, CP_OG, _b, CP_BG)(int smem) {
  return batch_max_ctas_kind<CP_CH, CP_KIND, CP_OG, CP_BG>(smem);
}

}  // namespace cp
