// cp_shake.cu — camera-shake block search (ShakeAnalyzer::calc_diffs, src/shake.rs:345-385).
//
// For frames f = 1..n-1 and offsets (ox, oy) in [0, 2s]^2:
//   diff[f][oy][ox] = sum over anchors a, window pixels (dy, dx) in [0, 2r]^2, channels c of
//                     (win_a[dy][dx][c] - img_f[cy+oy-s+dy-r][cx+ox-s+dx-r][c])^2
// accumulated in wrapping 32-bit integers (the reference's release profile disables
// overflow checks). Addition modulo 2^32 is associative, so the CTAs may add their partial
// sums in any order and the result is bit-identical to the sequential loop.
//
// One CTA per (frame, anchor, oy): the anchor window (from frame 0) and the (2r+1) image
// rows it slides over are staged in shared memory as 32-bit words; each thread owns one ox
// and sums 4 channel bytes per step with __vabsdiffu4 + __dp4a.

#include <cuda_runtime.h>

#include <cstdint>

#include "cp_internal.h"

namespace cp {
namespace {

// Shared-memory rows are padded to whole words; bytes past the row are zero in both the
// window and the image copy so they contribute nothing.
__global__ void __launch_bounds__(128) k_shake_diffs(const uint8_t* const* __restrict__ frames,
                                                    int32_t width, int32_t channels,
                                                    const int32_t* __restrict__ anchors,
                                                    int32_t r, int32_t s,
                                                    int32_t* __restrict__ diffs) {
  extern __shared__ __align__(16) uint32_t sm[];
  const int f = blockIdx.z + 1;
  const int a = blockIdx.y;
  const int oy = blockIdx.x;
  const int size = 2 * r + 1, ssize = 2 * s + 1;
  const int C = channels;
  const int win_bytes = size * C;                     // one window row
  const int win_words = (win_bytes + 3) / 4 + 1;      // +1: room for the shifted read
  const int img_bytes = (size + 2 * s) * C;           // one search row
  const int img_words = (img_bytes + 3) / 4 + 2;
  uint32_t* win = sm;                                  // [size][win_words]
  uint32_t* img = sm + size * win_words;               // [size][img_words]
  uint8_t* win8 = reinterpret_cast<uint8_t*>(win);
  uint8_t* img8 = reinterpret_cast<uint8_t*>(img);
  const int cx = anchors[2 * a], cy = anchors[2 * a + 1];
  const uint8_t* f0 = frames[0];
  const uint8_t* fi = frames[f];
  // stage: window rows of frame 0 and image rows y = cy + oy - s + dy - r of frame f
  for (int i = threadIdx.x; i < size * win_words * 4; i += blockDim.x) {
    const int dy = i / (win_words * 4), b = i - dy * (win_words * 4);
    uint8_t v = 0;
    if (b < win_bytes) {
      const long long yy = cy + dy - r, xx = cx - r;
      v = f0[(yy * width + xx) * C + b];
    }
    win8[i] = v;
  }
  for (int i = threadIdx.x; i < size * img_words * 4; i += blockDim.x) {
    const int dy = i / (img_words * 4), b = i - dy * (img_words * 4);
    uint8_t v = 0;
    if (b < img_bytes) {
      const long long yy = cy + oy - s + dy - r, xx = cx - s - r;
      v = fi[(yy * width + xx) * C + b];
    }
    img8[i] = v;
  }
  __syncthreads();
  for (int ox = threadIdx.x; ox < ssize; ox += blockDim.x) {
    const int boff = ox * C;  // byte offset of this offset's window in the image row
    const int wq = boff >> 2, sh = (boff & 3) * 8;
    uint32_t acc = 0;
    for (int dy = 0; dy < size; ++dy) {
      const uint32_t* wr = win + dy * win_words;
      const uint32_t* ir = img + dy * img_words + wq;
      uint32_t lo = ir[0];
      for (int j = 0; j < win_words - 1; ++j) {
        const uint32_t hi = ir[j + 1];
        uint32_t iv = __funnelshift_r(lo, hi, sh);
        const uint32_t wv = wr[j];
        // bytes of the image word past the window row must not count: the window word is
        // zero there, so mask the image word to the window's valid bytes
        const int rem = win_bytes - 4 * j;
        if (rem < 4) iv &= (1u << (8 * rem)) - 1u;
        const uint32_t d = __vabsdiffu4(wv, iv);
        acc = __dp4a(d, d, acc);
        lo = hi;
      }
    }
    atomicAdd(reinterpret_cast<unsigned int*>(diffs) + (size_t)(f - 1) * ssize * ssize +
                  oy * ssize + ox,
              acc);
  }
}

}  // namespace

int launch_shake(const uint8_t* const* frames_dev, int32_t n, int32_t width, int32_t height,
                 int32_t channels, const int32_t* anchors_dev, int32_t n_anchors, int32_t r,
                 int32_t s, int32_t* diffs_dev, void* stream) {
  (void)height;
  if (n < 2 || n_anchors < 1) return 0;
  const int size = 2 * r + 1, ssize = 2 * s + 1;
  const int win_words = (size * channels + 3) / 4 + 1;
  const int img_words = ((size + 2 * s) * channels + 3) / 4 + 2;
  const size_t smem = (size_t)size * (win_words + img_words) * 4;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (smem > 227 * 1024) return static_cast<int>(cudaErrorInvalidValue);
  cudaFuncSetAttribute(reinterpret_cast<const void*>(&k_shake_diffs),
                       cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  dim3 grid(ssize, n_anchors, n - 1);
  k_shake_diffs<<<grid, 128, smem, st>>>(frames_dev, width, channels, anchors_dev, r, s,
                                         diffs_dev);
  return static_cast<int>(cudaGetLastError());
}

}  // namespace cp
