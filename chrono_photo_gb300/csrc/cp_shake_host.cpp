// cp_shake_host.cpp — ShakeAnalyzer::analyze (src/shake.rs:190-313) on the device.

#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "../../include/chrono_gpu.h"
#include "cp_host_internal.h"
#include "cp_internal.h"

using namespace cp;

extern "C" int cp_shake_analyze_device(cp_ctx* ctx, const uint8_t* const* frames, int32_t n,
                                       int32_t width, int32_t height, int32_t channels,
                                       const int32_t* anchors, int32_t n_anchors,
                                       int32_t anchor_radius, int32_t search_radius,
                                       int32_t* offsets, int32_t* diffs) {
  if (!ctx || !frames || n < 1 || width < 1 || height < 1 || channels < 1 || channels > 4 ||
      anchor_radius < 0 || search_radius < 0 || n_anchors < 0 || !offsets ||
      (n_anchors > 0 && !anchors))
    return CP_ERR_ARG;
  const int r = anchor_radius, s = search_radius;
  // fill_windows needs the window inside frame 0 (shake.rs:333-336); calc_diffs the whole
  // search range inside each frame (shake.rs:371-374). The reference panics otherwise.
  for (int a = 0; a < n_anchors; ++a) {
    const int cx = anchors[2 * a], cy = anchors[2 * a + 1];
    if (cx - r < 0 || cy - r < 0 || cx + r >= width || cy + r >= height) return CP_ERR_RANGE;
    if (n > 1 && (cx - s - r < 0 || cy - s - r < 0 || cx + s + r >= width || cy + s + r >= height))
      return CP_ERR_RANGE;
  }
  offsets[0] = 0;  // shake.rs:308
  offsets[1] = 0;
  if (n == 1) return CP_OK;
  const int S = 2 * s + 1;
  const uint64_t nd = static_cast<uint64_t>(n - 1) * S * S;
  std::lock_guard<std::mutex> call(ctx->call_mu);
  cudaSetDevice(ctx->device);
  // device scratch: frame table, anchors, sums
  const uint64_t bytes = sizeof(void*) * n + 8ull * (n_anchors + 1) + 4 * nd + 256;
  void* scratch = nullptr;
  int rc = dev_alloc(ctx, bytes, &scratch);
  if (rc) return rc;
  uint8_t* base = static_cast<uint8_t*>(scratch);
  const uint8_t** d_frames = reinterpret_cast<const uint8_t**>(base);
  int32_t* d_anchors = reinterpret_cast<int32_t*>(base + sizeof(void*) * n);
  int32_t* d_diffs = reinterpret_cast<int32_t*>(base + ((sizeof(void*) * n + 8ull * (n_anchors + 1) + 255) / 256) * 256);
  std::vector<int32_t> h(nd);
  cudaStream_t st = ctx->stream;
  cudaError_t e = cudaMemcpyAsync(d_frames, frames, sizeof(void*) * n, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && n_anchors > 0)
    e = cudaMemcpyAsync(d_anchors, anchors, 8ull * n_anchors, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_diffs, 0, 4 * nd, st);
  if (e == cudaSuccess && n_anchors > 0) {
    e = static_cast<cudaError_t>(launch_shake(d_frames, n, width, height, channels, d_anchors,
                                              n_anchors, r, s, d_diffs, st));
    count_launches(ctx, 1);
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), d_diffs, 4 * nd, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  dev_free(ctx, scratch);
  if (e != cudaSuccess) return cuda_status(ctx, e, "shake");
  // first minimum of the i32 sums per frame (Iterator::min_by_key, shake.rs:294-297)
  for (int f = 1; f < n; ++f) {
    const int32_t* dd = h.data() + static_cast<uint64_t>(f - 1) * S * S;
    int best = 0;
    for (int k = 1; k < S * S; ++k)
      if (dd[k] < dd[best]) best = k;
    offsets[2 * f] = best % S - s;
    offsets[2 * f + 1] = best / S - s;
  }
  if (diffs) std::memcpy(diffs, h.data(), 4 * nd);
  return CP_OK;
}
