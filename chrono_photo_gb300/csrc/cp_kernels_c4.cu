// Instantiates the compositing kernels for 4-channel images and their launchers.
#include "cp_tile.cuh"

namespace cp {

int composite_max_ctas_c4(int threads, int smem) {
  const void* fn = reinterpret_cast<const void*>(&k_composite<4, kAnyKind, kOgAny, kBgAny>);
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, threads, smem) != cudaSuccess)
    return 1;
  return blocks < 1 ? 1 : blocks;
}

// The general kernel (single-stack launches of darker / lighter stacks the streaming kernel
// does not take); outlier stacks launch a specialised kernel (cp_kernels_variant.cu).
int launch_composite_c4(const StackDev& s, int grid, int smem, void* stream, uint32_t* error) {
  return launch_composite_kind<4, kAnyKind, kOgAny, kBgAny>(s, grid, smem, stream, error);
}

int launch_batch_c4(const StackDev* stacks, const int32_t* prefix, int32_t n_stacks,
                     int32_t total, int32_t interleave, uint32_t* counter, uint32_t* error,
                     int grid, int smem, void* stream) {
  return launch_batch_kind<4, kAnyKind, kOgAny, kBgAny>(stacks, prefix, n_stacks, total,
                                                         interleave, counter, error, grid, smem,
                                                         stream);
}

int simple_stream_max_ctas_c4(bool fast) {
  const void* fn = fast ? reinterpret_cast<const void*>(&k_simple_stream<4, true>)
                        : reinterpret_cast<const void*>(&k_simple_stream<4, false>);
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, kStreamThreads, kStreamSmem<4>) !=
      cudaSuccess)
    return 1;
  return blocks < 1 ? 1 : blocks;
}

int simple_stream_chunk_px_c4() { return kStreamChunkPx; }

int launch_simple_stream_c4(const StackDev& s, bool fast, int grid, void* stream, uint32_t* error) {
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (fast)
    k_simple_stream<4, true><<<grid, kStreamThreads, kStreamSmem<4>, st>>>(s, error);
  else
    k_simple_stream<4, false><<<grid, kStreamThreads, kStreamSmem<4>, st>>>(s, error);
  return static_cast<int>(cudaGetLastError());
}

}  // namespace cp
