// cp_host.cpp — C ABI of libchrono_gpu.so: contexts, device memory and host staging entry
// points, and the launch plans of the compositing kernels (single and multi-setting). Option
// preparation is in cp_prepare.cpp, memory accounting in cp_memory.cpp.

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/chrono_gpu.h"
#include "cp_host_internal.h"
#include "cp_internal.h"

using namespace cp;

// ---------------------------------------------------------------------------------------------
// Launch plans
// ---------------------------------------------------------------------------------------------
namespace cp {

int launch_single(cp_ctx* ctx, const StackDev& d, cudaStream_t stream) {
  if (d.mode != CP_MODE_OUTLIER && !d.shifted && !d.has_crop &&
      (reinterpret_cast<uintptr_t>(d.out) & 15) == 0) {
    // darker/lighter on aligned frames: the streaming kernel (no tiles)
    const bool fast = d.unit_w && d.no_fade;
    const int key = 1000 + d.channels * 2 + (fast ? 1 : 0);
    int per_sm = 1;
    {
      std::lock_guard<std::mutex> lk(ctx->mu);
      auto it = ctx->occupancy.find(std::make_pair(key, 0));
      if (it != ctx->occupancy.end()) {
        per_sm = it->second;
      } else {
        switch (d.channels) {
          case 1: per_sm = simple_stream_max_ctas_c1(fast); break;
          case 3: per_sm = simple_stream_max_ctas_c3(fast); break;
          default: per_sm = simple_stream_max_ctas_c4(fast); break;
        }
        ctx->occupancy[std::make_pair(key, 0)] = per_sm;
      }
    }
    const int chunk = simple_stream_chunk_px_c3();  // the same for every channel count
    const int chunks = (d.px_end - d.px_begin + chunk - 1) / chunk;
    const int grid = std::max(1, std::min(chunks, per_sm * ctx->sm_count));
    int rc;
    switch (d.channels) {
      case 1: rc = launch_simple_stream_c1(d, fast, grid, stream, ctx->d_error); break;
      case 3: rc = launch_simple_stream_c3(d, fast, grid, stream, ctx->d_error); break;
      default: rc = launch_simple_stream_c4(d, fast, grid, stream, ctx->d_error); break;
    }
    count_launches(ctx, 1);
    return cuda_status(ctx, static_cast<cudaError_t>(rc), "simple launch");
  }
  if (d.mode == CP_MODE_OUTLIER && d.channels == 3 && !d.shifted && !d.has_crop &&
      (d.fast_int || d.pair_f32) && px_smem_bytes(d.n, false) <= ctx->max_smem) {
    // the pixel-thread kernel (cp_outlier_px.cuh), configured by cp_tune.cpp
    return launch_px(ctx, d, stream);
  }
  const int smem = smem_bytes_for(d.n, d.channels);
  if (smem > ctx->max_smem) {
    ctx_error(ctx, "tile needs %d bytes of shared memory", smem);
    return CP_ERR_ARG;
  }
  int per_sm = 1, rc = 0;
  const bool outlier = d.mode == CP_MODE_OUTLIER;
  int k = 0, g = 0, b = 0;
  if (outlier) outlier_variant(d, &k, &g, &b);
  // occupancy of the kernel this stack launches with, cached per (variant, channels, smem)
  const auto key = std::make_pair(2000 + 64 * d.channels + single_variant(d), smem);
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->occupancy.find(key);
    if (it != ctx->occupancy.end()) {
      per_sm = it->second;
    } else {
      per_sm = 0;
      if (outlier) {
#define CP_VARIANT_OCC(CH, K, G, B)                                      \
  if (d.channels == CH && k == K && g == G && b == B)                  \
    per_sm = max_ctas_c##CH##_k##K##_g##G##_b##B(d.threads, smem);
        CP_VARIANTS(CP_VARIANT_OCC)
#undef CP_VARIANT_OCC
      } else {
        switch (d.channels) {
          case 1: per_sm = composite_max_ctas_c1(d.threads, smem); break;
          case 3: per_sm = composite_max_ctas_c3(d.threads, smem); break;
          default: per_sm = composite_max_ctas_c4(d.threads, smem); break;
        }
      }
      if (per_sm < 1) per_sm = 1;
      ctx->occupancy[key] = per_sm;
    }
  }
  const int grid = std::max(1, std::min(d.tiles, per_sm * ctx->sm_count));
  rc = -1;
  if (outlier) {
#define CP_VARIANT_LAUNCH(CH, K, G, B)                                             \
  if (d.channels == CH && k == K && g == G && b == B)                            \
    rc = launch_composite_c##CH##_k##K##_g##G##_b##B(d, grid, smem, stream, ctx->d_error);
    CP_VARIANTS(CP_VARIANT_LAUNCH)
#undef CP_VARIANT_LAUNCH
    if (rc < 0) {
      ctx_error(ctx, "no kernel for %d channels, variant %d/%d/%d", d.channels, k, g, b);
      return CP_ERR_ARG;
    }
  } else {
    switch (d.channels) {
      case 1: rc = launch_composite_c1(d, grid, smem, stream, ctx->d_error); break;
      case 3: rc = launch_composite_c3(d, grid, smem, stream, ctx->d_error); break;
      default: rc = launch_composite_c4(d, grid, smem, stream, ctx->d_error); break;
    }
  }
  count_launches(ctx, 1);
  return cuda_status(ctx, static_cast<cudaError_t>(rc), "composite launch");
}

namespace {

}  // namespace

// The pixel-thread kernels take the stack (RGB, aligned rows, no crop, integer or paired f32
// distances); the multi-setting kernel takes those same stacks.
bool px_eligible(cp_ctx* ctx, const StackDev& d) {
  return d.mode == CP_MODE_OUTLIER && d.channels == 3 && !d.shifted && !d.has_crop &&
         (d.fast_int || d.pair_f32) && px_smem_bytes(d.n, false) <= ctx->max_smem &&
         (d.nw == 1 || d.nw == 2 || d.nw == 4);
}

namespace {

// Darker / lighter settings the multi-setting kernel folds on its staged rows: RGB, rows
// starting 16-byte aligned, no crop.
bool simple_eligible(const StackDev& d) {
  return d.mode != CP_MODE_OUTLIER && d.channels == 3 && !d.shifted && !d.has_crop;
}

// Settings over the same frames and band.
bool same_stack(const StackDev& a, const StackDev& b) {
  return a.n == b.n && a.px_begin == b.px_begin && a.px_end == b.px_end && a.tiles == b.tiles &&
         std::memcmp(a.frames, b.frames, sizeof(a.frames[0]) * static_cast<size_t>(a.n)) == 0;
}

// Settings whose order statistics are the same: one stack, band and (sub)sample (the
// quartile ranks follow from the sample size; prepare_stack fills them for rel settings).
bool same_stats(const StackDev& a, const StackDev& b) {
  return same_stack(a, b) && a.n_sub == b.n_sub && a.med_k == b.med_k && a.med_pair == b.med_pair &&
         std::memcmp(a.sample_mask, b.sample_mask, sizeof a.sample_mask) == 0;
}

// The fields the distance pass reads (besides the order statistics): equal fields give equal
// outlier flags and extreme.
struct DistKey {
  int32_t thr_abs;
  uint32_t wmask, fast_int, pair_f32, finite_w, neg_w;
  float w[4];
  float thr_sq;
  int32_t thr_int[5];
};
DistKey dist_key(const StackDev& d) {
  DistKey k;
  std::memset(&k, 0, sizeof k);
  k.thr_abs = d.thr_abs;
  k.wmask = d.wmask;
  k.fast_int = d.fast_int;
  k.pair_f32 = d.pair_f32;
  k.finite_w = d.finite_w;
  k.neg_w = d.neg_w;
  std::memcpy(k.w, d.w, sizeof k.w);
  k.thr_sq = d.thr_sq;
  std::memcpy(k.thr_int, d.thr_int, sizeof k.thr_int);
  return k;
}
bool operator<(const DistKey& a, const DistKey& b) { return std::memcmp(&a, &b, sizeof a) < 0; }
bool operator==(const DistKey& a, const DistKey& b) { return std::memcmp(&a, &b, sizeof a) == 0; }

}  // namespace

int launch_multi(cp_ctx* ctx, const std::vector<StackDev>& ds, cudaStream_t stream) {
  // settings the multi-setting kernel takes together: pixel-kernel stacks with the order
  // statistics of the first of them; at least two, or there is nothing to share
  std::vector<size_t> fused, rest, simple;
  for (size_t i = 0; i < ds.size(); ++i) {
    const bool ok = px_eligible(ctx, ds[i]) && (fused.empty() || same_stats(ds[fused[0]], ds[i]));
    (ok ? fused : rest).push_back(i);
  }
  if (fused.empty()) {
    for (size_t i : rest) {
      const int rc = launch_single(ctx, ds[i], stream);
      if (rc) return rc;
    }
    return CP_OK;
  }
  // darker / lighter of the same stack fold the staged rows of the outlier settings' launch
  // (reading the stack again in their own launch costs more than the fold)
  for (auto it = rest.begin(); it != rest.end();) {
    if (simple_eligible(ds[*it]) && same_stack(ds[fused[0]], ds[*it])) {
      simple.push_back(*it);
      it = rest.erase(it);
    } else {
      ++it;
    }
  }
  // equal distance passes next to each other, so that each runs once; the outlier settings
  // first (sets[0] gives the launch its sampling), then darker / lighter
  std::stable_sort(fused.begin(), fused.end(), [&](size_t a, size_t b) {
    return dist_key(ds[a]) < dist_key(ds[b]);
  });
  fused.insert(fused.end(), simple.begin(), simple.end());
  if (fused.size() < 2) {
    rest.insert(rest.end(), fused.begin(), fused.end());
    fused.clear();
  }
  std::unique_ptr<MultiArgs> m(new MultiArgs());
  for (size_t c0 = 0; c0 < fused.size(); c0 += kMultiMax) {
    const size_t cnt = std::min<size_t>(kMultiMax, fused.size() - c0);
    if (cnt == 1) {
      rest.push_back(fused[c0]);
      continue;
    }
    if (ds[fused[c0]].mode != CP_MODE_OUTLIER) {  // a chunk of darker / lighter only
      for (size_t k = 0; k < cnt; ++k) rest.push_back(fused[c0 + k]);
      continue;
    }
    std::memset(m.get(), 0, sizeof(MultiArgs));
    bool rel = false;
    for (size_t k = 0; k < cnt; ++k) {
      const StackDev& d = ds[fused[c0 + k]];
      const bool outlier = d.mode == CP_MODE_OUTLIER;
      m->sets[k] = d;
      m->share_dist[k] = outlier && k > 0 && ds[fused[c0 + k - 1]].mode == CP_MODE_OUTLIER &&
                                 dist_key(d) == dist_key(ds[fused[c0 + k - 1]])
                             ? 1
                             : 0;
      rel = rel || (outlier && !d.thr_abs);
    }
    m->count = static_cast<int32_t>(cnt);
    if (rel) {  // the kernel selects the quartiles with the ranks of sets[0]
      for (size_t k = 0; k < cnt; ++k) {
        const StackDev& d = m->sets[k];
        if (d.mode != CP_MODE_OUTLIER || d.thr_abs) continue;
        StackDev& d0w = m->sets[0];
        d0w.q1_k = d.q1_k;
        d0w.q1_pair = d.q1_pair;
        d0w.q1_frac = d.q1_frac;
        d0w.q3_k = d.q3_k;
        d0w.q3_pair = d.q3_pair;
        d0w.q3_frac = d.q3_frac;
        break;
      }
    }
    const StackDev& d0 = m->sets[0];
    const int smem = px_smem_bytes(d0.n, false);
    int per_sm = 1;
    {
      const auto key = std::make_pair(6000 + d0.nw * 2 + (rel ? 1 : 0), smem);
      std::lock_guard<std::mutex> lk(ctx->mu);
      auto it = ctx->occupancy.find(key);
      if (it != ctx->occupancy.end()) {
        per_sm = it->second;
      } else {
        per_sm = std::max(1, px_multi(*m, rel, true, 0, smem, nullptr, nullptr));
        ctx->occupancy[key] = per_sm;
      }
    }
    const int grid = std::max(1, std::min(d0.tiles, per_sm * ctx->sm_count));
    const int rc = px_multi(*m, rel, false, grid, smem, stream, ctx->d_error);
    if (rc < 0) {
      ctx_error(ctx, "no multi-setting kernel for %d plane words", d0.nw);
      return CP_ERR_ARG;
    }
    const int st = cuda_status(ctx, static_cast<cudaError_t>(rc), "multi-setting launch");
    if (st) return st;
    count_launches(ctx, 1);
    ctx->n_multi += 1;
    ctx->n_multi_settings += cnt;
  }
  std::sort(rest.begin(), rest.end());
  for (size_t i : rest) {
    const int rc = launch_single(ctx, ds[i], stream);
    if (rc) return rc;
  }
  return CP_OK;
}

int check_device_error(cp_ctx* ctx) {
  uint32_t err = 0;
  cudaError_t e = cudaMemcpy(&err, ctx->d_error, sizeof err, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(ctx, e, "error flag read");
  if (err) {
    cudaMemset(ctx->d_error, 0, sizeof err);
    ctx_error(ctx, "a device-side wait timed out (error flags 0x%x)", err);
    return CP_ERR_TIMEOUT;
  }
  return CP_OK;
}

}  // namespace cp

// ---------------------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------------------
extern "C" {

const char* cp_version(void) { return "chrono-gpu 0.1.0 (sm_103a)"; }

int cp_video_windows(int32_t image_count, int32_t in_has_start, int32_t in_start,
                     int32_t in_has_end, int32_t in_end, int32_t in_step, int32_t out_has_start,
                     int32_t out_start, int32_t out_has_end, int32_t out_end, int32_t out_step,
                     int32_t* n_windows, int64_t* n_indices, int64_t* win_start, int32_t* win_len,
                     int32_t* win_indices, int32_t* win_frame) {
  // create_video window arithmetic, src/main.rs:230-286
  if (!n_windows || !n_indices || in_step <= 0 || out_step <= 0) return CP_ERR_ARG;
  int32_t v_lower;
  if (out_has_start)
    v_lower = out_start;
  else if (in_has_start && in_has_end)
    v_lower = -(in_end - in_start) + 1;
  else
    v_lower = 0;
  const int32_t v_upper = out_has_end ? out_end : image_count;
  int32_t count = (v_upper - v_lower) / out_step;
  if (count < 0) count = 0;
  int64_t total = 0;
  for (int32_t k = 0; k < count; ++k) {
    const int32_t frame = k * out_step + v_lower;
    int32_t start = 0;
    if (in_has_start) {
      int32_t s = frame + in_start;
      while (s < 0) s += in_step;
      start = std::max(s % in_step, frame + in_start);
    }
    int32_t end = image_count;
    if (in_has_end) end = std::min(image_count + (frame + in_end) % in_step - in_step, frame + in_end);
    int32_t len = 0;
    for (int32_t f = start; f < end; f += in_step) {
      if (win_indices) win_indices[total + len] = f;
      ++len;
    }
    if (win_start) win_start[k] = total;
    if (win_len) win_len[k] = len;
    if (win_frame) win_frame[k] = frame - v_lower;
    total += len;
  }
  *n_windows = count;
  *n_indices = total;
  return CP_OK;
}

int cp_crop_create(const int32_t* offsets, int32_t n, int32_t width, int32_t height,
                   int32_t* has_crop, int32_t* crops) {
  // Crop::create, src/shake.rs:136-176
  if (!offsets || n < 0 || !has_crop) return CP_ERR_ARG;
  int32_t xmin = 0, ymin = 0, xmax = 0, ymax = 0;
  for (int i = 0; i < n; ++i) {
    xmin = std::min(xmin, offsets[2 * i]);
    ymin = std::min(ymin, offsets[2 * i + 1]);
    xmax = std::max(xmax, offsets[2 * i]);
    ymax = std::max(ymax, offsets[2 * i + 1]);
  }
  if (xmin == 0 && ymin == 0 && xmax == 0 && ymax == 0) {
    *has_crop = 0;
    return CP_OK;
  }
  if (!crops) return CP_ERR_ARG;
  *has_crop = 1;
  const int32_t w = width + xmin - xmax, h = height + ymin - ymax;
  for (int i = 0; i < n; ++i) {
    crops[4 * i] = offsets[2 * i] - xmin;
    crops[4 * i + 1] = offsets[2 * i + 1] - ymin;
    crops[4 * i + 2] = w;
    crops[4 * i + 3] = h;
  }
  return CP_OK;
}

int cp_sample_indices(int32_t n, int32_t count, uint64_t seed, int32_t* out, int32_t* n_out) {
  if (n < 0 || count < 0 || !out || !n_out) return CP_ERR_ARG;
  if (count >= n) {  // src/chrono.rs:153-154
    for (int i = 0; i < n; ++i) out[i] = i;
    *n_out = n;
    return CP_OK;
  }
  // partial Fisher-Yates with a splitmix64 stream, then sorted (src/chrono.rs:156-158)
  std::vector<int32_t> idx(static_cast<size_t>(n));
  for (int i = 0; i < n; ++i) idx[static_cast<size_t>(i)] = i;
  uint64_t x = seed;
  for (int i = 0; i < count; ++i) {
    x += 0x9E3779B97F4A7C15ull;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const int j = i + static_cast<int>(((z >> 32) * static_cast<uint64_t>(n - i)) >> 32);
    std::swap(idx[static_cast<size_t>(i)], idx[static_cast<size_t>(j)]);
  }
  std::sort(idx.begin(), idx.begin() + count);
  for (int i = 0; i < count; ++i) out[i] = idx[static_cast<size_t>(i)];
  *n_out = count;
  return CP_OK;
}

int cp_ctx_create(int32_t device, uint64_t hbm_budget, cp_ctx** out) {
  if (!out) return CP_ERR_ARG;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
    cudaGetLastError();
    return CP_ERR_NODEV;
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return CP_ERR_NODEV;
  if (prop.major != 10 || prop.minor != 3) return CP_ERR_NODEV;  // built for sm_103a only
  if (cudaSetDevice(device) != cudaSuccess) return CP_ERR_NODEV;
  std::unique_ptr<cp_ctx> ctx(new cp_ctx());
  ctx->device = device;
  ctx->budget = hbm_budget;
  ctx->sm_count = prop.multiProcessorCount;
  ctx->gpu_name = prop.name;
  ctx->max_smem = static_cast<int>(prop.sharedMemPerBlockOptin);
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->copy_stream2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->d2h_stream, cudaStreamNonBlocking) != cudaSuccess)
    return CP_ERR_CUDA;
  void* p = nullptr;
  if (dev_alloc(ctx.get(), 256, &p) != CP_OK) return CP_ERR_OOM;
  ctx->d_error = static_cast<uint32_t*>(p);
  ctx->d_warn = reinterpret_cast<unsigned long long*>(static_cast<uint8_t*>(p) + 64);
  if (cudaMemset(p, 0, 256) != cudaSuccess) return CP_ERR_CUDA;
  *out = ctx.release();
  return CP_OK;
}

void cp_ctx_destroy(cp_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  cudaStreamSynchronize(ctx->copy_stream);
  cudaStreamSynchronize(ctx->copy_stream2);
  cudaStreamSynchronize(ctx->d2h_stream);
  release_plans(ctx);
  jpeg_release(ctx);
  std::vector<void*> ptrs;
  for (auto& kv : ctx->allocs) ptrs.push_back(kv.first);
  for (void* q : ptrs) cudaFree(q);
  for (auto& pb : {&ctx->pin_in, &ctx->pin_out, &ctx->pin_blend})
    if (pb->ptr) cudaFreeHost(pb->ptr);
  for (auto& ev : ctx->band_events) cudaEventDestroy(ev);
  cudaStreamDestroy(ctx->stream);
  cudaStreamDestroy(ctx->copy_stream);
  cudaStreamDestroy(ctx->copy_stream2);
  cudaStreamDestroy(ctx->d2h_stream);
  delete ctx;
}

void* cp_ctx_stream(cp_ctx* ctx) { return ctx ? ctx->stream : nullptr; }

int cp_ctx_synchronize(cp_ctx* ctx) {
  if (!ctx) return CP_ERR_ARG;
  cudaSetDevice(ctx->device);
  int rc = cuda_status(ctx, cudaStreamSynchronize(ctx->stream), "synchronize");
  if (rc) return rc;
  return check_device_error(ctx);
}

int cp_ctx_set_wait_limit(cp_ctx* ctx, uint64_t cycles) {
  if (!ctx || cycles > (uint64_t(1) << 62)) return CP_ERR_ARG;
  ctx->wait_cycles = static_cast<int64_t>(cycles);
  return CP_OK;
}

int cp_dev_alloc(cp_ctx* ctx, uint64_t bytes, void** ptr) {
  if (!ctx) return CP_ERR_ARG;
  return dev_alloc(ctx, bytes, ptr);
}
int cp_dev_free(cp_ctx* ctx, void* ptr) {
  if (!ctx) return CP_ERR_ARG;
  return dev_free(ctx, ptr);
}
int cp_host_alloc(cp_ctx* ctx, uint64_t bytes, void** ptr) {
  if (!ctx || !ptr) return CP_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (injected_alloc_failure(ctx)) return CP_ERR_OOM;
  return cuda_status(ctx, cudaHostAlloc(ptr, bytes, cudaHostAllocPortable), "cudaHostAlloc");
}
int cp_host_free(cp_ctx* ctx, void* ptr) {
  if (!ctx) return CP_ERR_ARG;
  return cuda_status(ctx, cudaFreeHost(ptr), "cudaFreeHost");
}
int cp_memcpy_h2d(cp_ctx* ctx, void* dst, const void* src, uint64_t bytes, void* stream) {
  if (!ctx) return CP_ERR_ARG;
  cudaSetDevice(ctx->device);
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  int rc = cuda_status(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st), "h2d");
  if (rc || stream) return rc;
  return cuda_status(ctx, cudaStreamSynchronize(st), "h2d sync");
}
int cp_memcpy_d2h(cp_ctx* ctx, void* dst, const void* src, uint64_t bytes, void* stream) {
  if (!ctx) return CP_ERR_ARG;
  cudaSetDevice(ctx->device);
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  int rc = cuda_status(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st), "d2h");
  if (rc || stream) return rc;
  return cuda_status(ctx, cudaStreamSynchronize(st), "d2h sync");
}

int cp_composite_device(cp_ctx* ctx, const cp_stack* stack, const cp_params* params,
                        uint8_t* out, uint8_t* out_blend, const cp_debug* dbg,
                        uint64_t* warnings, void* stream) {
  if (!ctx || !stack || !params || !out) return CP_ERR_ARG;
  cudaSetDevice(ctx->device);
  std::vector<const uint8_t*> fr(static_cast<size_t>(std::max(stack->n, 0)));
  for (int i = 0; i < stack->n && i < CP_MAX_FRAMES; ++i)
    fr[static_cast<size_t>(i)] = stack->frames ? stack->frames[i] : stack->base + stack->frame_stride * i;
  if (stack->n < 1 || stack->n > CP_MAX_FRAMES) return CP_ERR_ARG;
  std::unique_ptr<StackDev> d(new StackDev());
  int rc = prepare_stack(ctx, stack, params, fr.data(), d.get());
  if (rc) return rc;
  d->out = out;
  d->blend = params->mode == CP_MODE_OUTLIER ? out_blend : nullptr;
  d->warnings = reinterpret_cast<unsigned long long*>(warnings);
  if (dbg && params->mode == CP_MODE_OUTLIER) {
    d->dbg_median = dbg->median;
    d->dbg_q1 = dbg->q1;
    d->dbg_q3 = dbg->q3;
    d->dbg_bits = dbg->outlier_bits;
    d->dbg_chosen = dbg->chosen;
    d->dbg_bg = dbg->background;
    d->dbg_nout = dbg->n_outliers;
  }
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  return launch_single(ctx, *d, st);
}

int cp_ctx_launch_counts(cp_ctx* ctx, uint64_t* launches, uint64_t* multi_launches,
                         uint64_t* multi_settings) {
  if (!ctx) return CP_ERR_ARG;
  if (launches) *launches = ctx->n_launches.load();
  if (multi_launches) *multi_launches = ctx->n_multi.load();
  if (multi_settings) *multi_settings = ctx->n_multi_settings.load();
  return CP_OK;
}

int cp_composite_device_multi(cp_ctx* ctx, const cp_stack* stack, const cp_params* params,
                              int32_t count, uint8_t* const* out, uint8_t* const* out_blend,
                              uint64_t* warnings, void* stream) {
  if (!ctx || !stack || !params || !out || count < 1) return CP_ERR_ARG;
  if (count > CP_MAX_SETTINGS) return CP_ERR_LIMIT;
  if (stack->n < 1 || stack->n > CP_MAX_FRAMES || (!stack->frames && !stack->base))
    return CP_ERR_ARG;
  for (int32_t k = 0; k < count; ++k)
    if (!out[k]) return CP_ERR_ARG;
  cudaSetDevice(ctx->device);
  try {
    std::vector<const uint8_t*> fr(static_cast<size_t>(stack->n));
    for (int i = 0; i < stack->n; ++i)
      fr[static_cast<size_t>(i)] =
          stack->frames ? stack->frames[i] : stack->base + stack->frame_stride * i;
    std::vector<StackDev> ds(static_cast<size_t>(count));
    for (int32_t k = 0; k < count; ++k) {
      StackDev& d = ds[static_cast<size_t>(k)];
      const int rc = prepare_stack(ctx, stack, &params[k], fr.data(), &d);
      if (rc) return rc;
      d.out = out[k];
      d.blend = params[k].mode == CP_MODE_OUTLIER && out_blend ? out_blend[k] : nullptr;
      d.warnings = warnings ? reinterpret_cast<unsigned long long*>(warnings) + k : nullptr;
    }
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    return launch_multi(ctx, ds, st);
  } catch (const std::exception& e) {
    ctx_error(ctx, "cp_composite_device_multi: %s", e.what());
    return CP_ERR_OOM;
  }
}

}  // extern "C"
