// cp_batch.cpp — many stacks in one persistent launch (cp_composite_batch_device).
//
// Replaces the rayon loop of src/main.rs:254-330, which builds one OutlierProcessor per
// chrono-video window and re-reads every frame for each. Here the windows reference frames
// already resident on the device; their (stack, tile) work items are flattened through a
// prefix sum and pulled by persistent CTAs from a device counter. The memset of the counter
// and the kernel are captured once into a CUDA graph per batch plan and replayed while the
// batch is unchanged.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <utility>
#include <vector>

#include "../../include/chrono_gpu.h"
#include "cp_host_internal.h"
#include "cp_internal.h"

namespace cp {


void release_plans(cp_ctx* ctx) {
  for (auto& p : ctx->plans) {
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    if (p->dev) dev_free(ctx, p->dev);
  }
  ctx->plans.clear();
}

// Index in CP_BATCH_VARIANTS of the specialised batched kernel a stack takes, or -1 (the
// general batched kernel).
int batch_variant_key(const StackDev& d) {
  if (d.mode != CP_MODE_OUTLIER || d.channels != 3) return -1;
  int k, g, b;
  outlier_variant(d, &k, &g, &b);
  int idx = 0, key = -1;
#define CP_BATCH_KEY(CH, K, G, B) \
  if (k == K && g == G && b == B) key = idx; \
  ++idx;
  CP_BATCH_VARIANTS(CP_BATCH_KEY)
#undef CP_BATCH_KEY
  return key;
}

// Stacks of one group share a launch: same batched kernel and plane-word count.
int batch_group_key(const StackDev& d) { return (batch_variant_key(d) + 1) * 8 + d.nw; }

// One persistent launch over `n` stacks (descriptors and prefix sums already on the device):
// the specialised batched kernel when every stack takes the same one, else the general one.
int launch_batch_dispatch(cp_ctx* ctx, const std::vector<StackDev>& host, const StackDev* d_stacks,
                          const int32_t* d_prefix, int32_t total, int32_t interleave,
                          uint32_t* d_counter, int max_n, cudaStream_t st, uint32_t* d_err) {
  uint32_t* err = d_err ? d_err : ctx->d_error;
  const int n = static_cast<int>(host.size());
  const int channels = host[0].channels;
  const int smem = smem_bytes_for(max_n, channels);
  int key = batch_variant_key(host[0]);
  for (const StackDev& d : host)
    if (batch_variant_key(d) != key) key = -1;
  int per_sm = 1;
  if (key >= 0) {
    int idx = 0;
#define CP_BATCH_OCC(CH, K, G, B) \
  if (key == idx) per_sm = batch_max_ctas_c##CH##_k##K##_g##G##_b##B(smem); \
  ++idx;
    CP_BATCH_VARIANTS(CP_BATCH_OCC)
#undef CP_BATCH_OCC
  } else {
    switch (channels) {
      case 1: per_sm = composite_max_ctas_c1(cta_threads(1), smem); break;
      case 3: per_sm = composite_max_ctas_c3(cta_threads(3), smem); break;
      default: per_sm = composite_max_ctas_c4(cta_threads(4), smem); break;
    }
  }
  const int grid = std::max(1, std::min(total, per_sm * ctx->sm_count));
  cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return cuda_status(ctx, e, "memset");
  int rc = 0;
  if (key >= 0) {
    int idx = 0;
#define CP_BATCH_LAUNCH(CH, K, G, B)                                                          \
  if (key == idx)                                                                             \
    rc = launch_batch_c##CH##_k##K##_g##G##_b##B(d_stacks, d_prefix, n, total, interleave,   \
                                                 d_counter, err, grid, smem, st);   \
  ++idx;
    CP_BATCH_VARIANTS(CP_BATCH_LAUNCH)
#undef CP_BATCH_LAUNCH
  } else {
    switch (channels) {
      case 1: rc = launch_batch_c1(d_stacks, d_prefix, n, total, interleave, d_counter, err, grid, smem, st); break;
      case 3: rc = launch_batch_c3(d_stacks, d_prefix, n, total, interleave, d_counter, err, grid, smem, st); break;
      default: rc = launch_batch_c4(d_stacks, d_prefix, n, total, interleave, d_counter, err, grid, smem, st); break;
    }
  }
  // a launch captured into a batch plan's graph counts when the graph is replayed
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(st, &cap);
  if (cap == cudaStreamCaptureStatusNone) count_launches(ctx, 1);
  return cuda_status(ctx, static_cast<cudaError_t>(rc), "batch launch");
}

static int batch_launch_raw(cp_ctx* ctx, BatchPlan& plan, int max_n, cudaStream_t st) {
  const int n_stacks = static_cast<int>(plan.host.size());
  StackDev* d_stacks = static_cast<StackDev*>(plan.dev);
  int32_t* d_prefix = reinterpret_cast<int32_t*>(d_stacks + n_stacks);
  uint32_t* d_counter = reinterpret_cast<uint32_t*>(d_prefix + n_stacks + 1);
  return launch_batch_dispatch(ctx, plan.host, d_stacks, d_prefix, plan.total, plan.interleave,
                               d_counter, max_n, st, nullptr);
}

}  // namespace cp

using namespace cp;

// Batch with per-stack warning counters (device pointers, nullable).
static int batch_run(cp_ctx* ctx, const cp_stack* stacks, const cp_params* params,
                     int32_t n_stacks, uint8_t* const* outs, uint8_t* const* out_blends,
                     uint64_t* const* warn_ptrs, void* stream) {
  if (!ctx || !stacks || !params || !outs || n_stacks < 1) return CP_ERR_ARG;
  cudaSetDevice(ctx->device);
  std::vector<StackDev> host(static_cast<size_t>(n_stacks));
  const int channels = stacks[0].channels;
  int max_n = 0;
  std::vector<int32_t> prefix(static_cast<size_t>(n_stacks) + 1, 0);
  std::vector<const uint8_t*> fr;
  for (int i = 0; i < n_stacks; ++i) {
    const cp_stack& s = stacks[i];
    if (s.channels != channels) {
      ctx_error(ctx, "a batch must have one channel count");
      return CP_ERR_ARG;
    }
    if (s.n < 1 || s.n > CP_MAX_FRAMES || !outs[i]) return CP_ERR_ARG;
    fr.assign(static_cast<size_t>(s.n), nullptr);
    for (int f = 0; f < s.n; ++f)
      fr[static_cast<size_t>(f)] = s.frames ? s.frames[f] : s.base + s.frame_stride * f;
    StackDev& d = host[static_cast<size_t>(i)];
    int rc = prepare_stack(ctx, &s, &params[i], fr.data(), &d);
    if (rc) return rc;
    d.out = outs[i];
    d.blend = (out_blends && params[i].mode == CP_MODE_OUTLIER) ? out_blends[i] : nullptr;
    d.warnings = warn_ptrs ? reinterpret_cast<unsigned long long*>(warn_ptrs[i]) : nullptr;
    max_n = std::max(max_n, s.n);
    prefix[static_cast<size_t>(i) + 1] = prefix[static_cast<size_t>(i)] + d.tiles;
  }
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;

  // a stack the pixel-thread kernel takes and whose tiles fill every SM's resident CTAs at
  // least twice runs on that kernel alone: it needs no batch to fill the GPU, and the
  // pixel-thread kernel is faster per stack than the batched tile kernel (on 1080p
  // chrono-video windows 39.1 vs 46.3 ms for 269 windows); the rest are batched
  {
    std::vector<int> rest;
    bool any_alone = false;
    for (int i = 0; i < n_stacks; ++i) {
      const StackDev& d = host[static_cast<size_t>(i)];
      if (px_eligible(ctx, d) && d.tiles >= 2 * kPxAloneCtas * ctx->sm_count) {
        const int rc = launch_single(ctx, d, st);
        if (rc) return rc;
        any_alone = true;
      } else {
        rest.push_back(i);
      }
    }
    if (any_alone) {
      if (rest.empty()) return CP_OK;
      std::vector<cp_stack> gs;
      std::vector<cp_params> gp;
      std::vector<uint8_t*> go, gb;
      std::vector<uint64_t*> gw;
      for (int i : rest) {
        gs.push_back(stacks[i]);
        gp.push_back(params[i]);
        go.push_back(outs[i]);
        gb.push_back(out_blends ? out_blends[i] : nullptr);
        gw.push_back(warn_ptrs ? warn_ptrs[i] : nullptr);
      }
      return batch_run(ctx, gs.data(), gp.data(), static_cast<int32_t>(gs.size()), go.data(),
                       out_blends ? gb.data() : nullptr, warn_ptrs ? gw.data() : nullptr,
                       stream);
    }
  }
  if (smem_bytes_for(max_n, channels) > ctx->max_smem) return CP_ERR_ARG;

  // stacks that take different specialised batched kernels, or need shared memory for a
  // different number of plane words (a launch sizes every CTA for its largest stack: one
  // 128-frame stack among 16-frame ones would halve the residency of all), run as one launch
  // per group, each group a plan of its own
  std::vector<int> keys(static_cast<size_t>(n_stacks));
  bool mixed = false;
  for (int i = 0; i < n_stacks; ++i) {
    const StackDev& d = host[static_cast<size_t>(i)];
    keys[static_cast<size_t>(i)] = batch_group_key(d);
    if (keys[static_cast<size_t>(i)] != keys[0]) mixed = true;
  }
  if (mixed) {
    std::vector<int> distinct(keys);
    std::sort(distinct.begin(), distinct.end());
    distinct.erase(std::unique(distinct.begin(), distinct.end()), distinct.end());
    for (int key : distinct) {
      std::vector<cp_stack> gs;
      std::vector<cp_params> gp;
      std::vector<uint8_t*> go, gb;
      std::vector<uint64_t*> gw;
      for (int i = 0; i < n_stacks; ++i) {
        if (keys[static_cast<size_t>(i)] != key) continue;
        gs.push_back(stacks[i]);
        gp.push_back(params[i]);
        go.push_back(outs[i]);
        gb.push_back(out_blends ? out_blends[i] : nullptr);
        gw.push_back(warn_ptrs ? warn_ptrs[i] : nullptr);
      }
      const int rc = batch_run(ctx, gs.data(), gp.data(), static_cast<int32_t>(gs.size()),
                               go.data(), out_blends ? gb.data() : nullptr,
                               warn_ptrs ? gw.data() : nullptr, stream);
      if (rc) return rc;
    }
    return CP_OK;
  }

  // find a plan with the same descriptors
  BatchPlan* plan = nullptr;
  for (auto& p : ctx->plans) {
    if (p->host.size() == host.size() &&
        std::memcmp(p->host.data(), host.data(), host.size() * sizeof(StackDev)) == 0) {
      plan = p.get();
      break;
    }
  }
  if (!plan) {
    if (ctx->plans.size() >= 8) {  // keep a few plans; drop the oldest
      cudaStreamSynchronize(st);
      auto& old = ctx->plans.front();
      if (old->exec) cudaGraphExecDestroy(old->exec);
      if (old->graph) cudaGraphDestroy(old->graph);
      if (old->dev) dev_free(ctx, old->dev);
      ctx->plans.erase(ctx->plans.begin());
    }
    std::unique_ptr<BatchPlan> np(new BatchPlan());
    np->host = host;
    np->total = prefix.back();
    np->max_n = max_n;
    np->interleave = 1;
    for (const StackDev& d : host)
      if (d.tiles != host[0].tiles || d.width != host[0].width || d.height != host[0].height ||
          d.has_crop != host[0].has_crop)
        np->interleave = 0;
    np->dev_bytes = sizeof(StackDev) * host.size() + sizeof(int32_t) * prefix.size() + 64;
    int rc = dev_alloc(ctx, np->dev_bytes, &np->dev);
    if (rc) return rc;
    uint8_t* base = static_cast<uint8_t*>(np->dev);
    cudaError_t e = cudaMemcpy(base, host.data(), sizeof(StackDev) * host.size(),
                               cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(base + sizeof(StackDev) * host.size(), prefix.data(),
                     sizeof(int32_t) * prefix.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      dev_free(ctx, np->dev);
      return cuda_status(ctx, e, "batch descriptors");
    }
    // capture memset + persistent kernel into a graph
    cudaStream_t cap;
    cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
    e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      rc = batch_launch_raw(ctx, *np, max_n, cap);
      cudaGraph_t g = nullptr;
      cudaError_t e2 = cudaStreamEndCapture(cap, &g);
      if (rc == CP_OK && e2 == cudaSuccess) {
        np->graph = g;
        e = cudaGraphInstantiate(&np->exec, g, 0);
      } else {
        if (g) cudaGraphDestroy(g);
        e = e2 != cudaSuccess ? e2 : cudaErrorUnknown;
      }
    }
    cudaStreamDestroy(cap);
    if (e != cudaSuccess || rc != CP_OK) {
      if (np->graph) cudaGraphDestroy(np->graph);
      dev_free(ctx, np->dev);
      return rc ? rc : cuda_status(ctx, e, "batch graph");
    }
    ctx->plans.push_back(std::move(np));
    plan = ctx->plans.back().get();
  }
  count_launches(ctx, 1);  // the graph holds one kernel (after the counter reset)
  return cuda_status(ctx, cudaGraphLaunch(plan->exec, st), "graph launch");
}

extern "C" int cp_composite_batch_device(cp_ctx* ctx, const cp_stack* stacks,
                                         const cp_params* params, int32_t n_stacks,
                                         uint8_t* const* outs, uint8_t* const* out_blends,
                                         uint64_t* warnings, void* stream) {
  if (n_stacks < 1) return CP_ERR_ARG;
  std::vector<uint64_t*> wp(static_cast<size_t>(n_stacks), nullptr);
  if (warnings)
    for (int i = 0; i < n_stacks; ++i) wp[static_cast<size_t>(i)] = warnings + i;
  return batch_run(ctx, stacks, params, n_stacks, outs, out_blends, warnings ? wp.data() : nullptr,
                   stream);
}

// Windows that slide by one frame over a sequence of resident frames (chrono-video with
// step 1: every window of the steady middle part of create_video, src/main.rs:230-286) run
// the sliding kernel (cp_video.cu) when the options allow it: RGB, outlier mode with an abs
// threshold and 0/1 weights (integer distances), no fade, no --sample, 16-byte aligned
// frames. Each maximal run of at least kMinSlideRun windows of one length 2..64,
// each window the previous one shifted by one frame, is one run; done[k] marks the windows
// handled here, the rest (the growing and shrinking windows at the ends) go to the batched
// kernel.
static constexpr int kMinSlideRun = 3;

static int video_sliding(cp_ctx* ctx, const uint8_t* const* frames, int32_t image_count,
                         int32_t width, int32_t height, int32_t channels, int32_t n_windows,
                         const int64_t* win_start, const int32_t* win_len,
                         const int32_t* win_indices, const cp_params* params,
                         uint8_t* const* outs, uint8_t* const* out_blends, uint64_t* warnings,
                         void* stream, std::vector<char>& done) {
  if (channels != 3 || params->mode != CP_MODE_OUTLIER || !params->thr_abs ||
      params->fade.enabled || (params->sample && params->n_sample > 0))
    return CP_OK;
  for (int i = 0; i < 3; ++i)
    if (!(params->weights[i] == 0.0f || params->weights[i] == 1.0f)) return CP_OK;
  const int og = outlier_group(params->outlier);
  const int bg_first = params->background == CP_BG_FIRST ? 1 : 0;
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  auto aligned = [&](int k) {
    for (int i = 0; i < win_len[k]; ++i)
      if (reinterpret_cast<uintptr_t>(frames[win_indices[win_start[k] + i]]) & 15) return false;
    return true;
  };
  auto slides = [&](int k) {  // window k is window k - 1 shifted by one frame
    const int L = win_len[k];
    if (win_len[k - 1] != L) return false;
    for (int i = 0; i + 1 < L; ++i)
      if (win_indices[win_start[k - 1] + i + 1] != win_indices[win_start[k] + i]) return false;
    return true;
  };
  std::unique_ptr<VideoArgs> args;
  int k = 0;
  while (k < n_windows) {
    const int L = win_len[k];
    if (L < 2 || L > 64 || !aligned(k)) {
      ++k;
      continue;
    }
    int e = k + 1;
    while (e < n_windows && slides(e) && aligned(e)) ++e;
    if (e - k < kMinSlideRun) {
      k = e;
      continue;
    }
    // windows k .. e-1: one run
    if (!args) args = std::make_unique<VideoArgs>();
    VideoArgs* A = args.get();
    std::memset(A, 0, sizeof(VideoArgs));
    std::vector<const uint8_t*> w0(static_cast<size_t>(L));
    for (int i = 0; i < L; ++i) w0[static_cast<size_t>(i)] = frames[win_indices[win_start[k] + i]];
    cp_stack s0;
    std::memset(&s0, 0, sizeof s0);
    s0.n = L;
    s0.width = width;
    s0.height = height;
    s0.channels = channels;
    s0.frames = w0.data();
    int rc = prepare_stack(ctx, &s0, params, w0.data(), &A->S);
    if (rc) return rc;
    if (!A->S.fast_int) return CP_OK;
    const int smem = video_smem_bytes(L);
    if (smem > ctx->max_smem) return CP_OK;
    int per_sm = 1;
    {
      const auto key = std::make_pair(3000 + og * 16 + bg_first * 8 + A->S.nw, smem);
      std::lock_guard<std::mutex> lk(ctx->mu);
      auto it = ctx->occupancy.find(key);
      if (it != ctx->occupancy.end()) {
        per_sm = it->second;
      } else {
        per_sm = video_slide(A, og, bg_first, true, 0, smem, nullptr, nullptr);
        if (per_sm < 1) per_sm = 1;
        ctx->occupancy[key] = per_sm;
      }
    }
    A->npx = width * height;
    A->tiles = (A->npx + 31) / 32;
    const int grid = std::max(1, std::min(A->tiles, per_sm * ctx->sm_count));
    const int per_launch = std::min(kVideoMaxWin, kVideoMaxRows - L + 1);
    for (int k0 = k; k0 < e; k0 += per_launch) {
      const int nw = std::min(per_launch, e - k0);
      A->n_win = nw;
      A->n_rows = nw + L - 1;
      // row j of the launch: frame j of window k0 for j < L, then the last frame of window
      // k0 + j - L + 1
      for (int j = 0; j < A->n_rows; ++j) {
        const int idx = j < L ? win_indices[win_start[k0] + j]
                              : win_indices[win_start[k0 + j - L + 1] + L - 1];
        A->rows[j] = frames[idx];
      }
      for (int w = 0; w < nw; ++w) {
        A->outs[w] = outs[k0 + w];
        A->blends[w] = out_blends ? out_blends[k0 + w] : nullptr;
        if (!A->outs[w]) return CP_ERR_ARG;
      }
      A->warnings = warnings ? reinterpret_cast<unsigned long long*>(warnings + k0) : nullptr;
      rc = video_slide(A, og, bg_first, false, grid, smem, st, ctx->d_error);
      count_launches(ctx, 1);
      if (rc) return cuda_status(ctx, static_cast<cudaError_t>(rc), "sliding-window launch");
    }
    for (int w = k; w < e; ++w) done[static_cast<size_t>(w)] = 1;
    k = e;
  }
  (void)image_count;
  return CP_OK;
}

extern "C" int cp_composite_video_device(cp_ctx* ctx, const uint8_t* const* frames,
                                         int32_t image_count, int32_t width, int32_t height,
                                         int32_t channels, int32_t n_windows,
                                         const int64_t* win_start, const int32_t* win_len,
                                         const int32_t* win_indices, const cp_params* params,
                                         uint8_t* const* outs, uint8_t* const* out_blends,
                                         uint64_t* warnings, void* stream) {
  // One composite per chrono-video window (src/main.rs:254-330) over frames resident on the
  // device; windows without frames are skipped, as the reference skips them (:326-328).
  if (!ctx || !frames || !win_start || !win_len || !win_indices || !params || !outs ||
      n_windows < 0 || image_count < 1)
    return CP_ERR_ARG;
  for (int k = 0; k < n_windows; ++k)
    for (int i = 0; i < win_len[k]; ++i) {
      const int idx = win_indices[win_start[k] + i];
      if (idx < 0 || idx >= image_count || !frames[idx]) return CP_ERR_ARG;
    }
  std::vector<char> done(static_cast<size_t>(n_windows), 0);
  // CP_VIDEO_SLIDING=0 in the environment sends every window to the batched kernel (for
  // comparing the two paths on one workload)
  const char* sliding_env = std::getenv("CP_VIDEO_SLIDING");
  if (!sliding_env || std::strcmp(sliding_env, "0") != 0) {
    const int rc = video_sliding(ctx, frames, image_count, width, height, channels, n_windows,
                                 win_start, win_len, win_indices, params, outs, out_blends,
                                 warnings, stream, done);
    if (rc) return rc;
  }
  std::vector<cp_stack> stacks;
  std::vector<cp_params> ps;
  std::vector<uint8_t*> o, b;
  std::vector<uint64_t*> wp;
  std::vector<std::vector<const uint8_t*>> tables;
  tables.reserve(static_cast<size_t>(n_windows));
  for (int k = 0; k < n_windows; ++k) {
    const int len = win_len[k];
    if (len <= 0 || done[static_cast<size_t>(k)]) continue;
    std::vector<const uint8_t*> t(static_cast<size_t>(len));
    for (int i = 0; i < len; ++i) {
      const int idx = win_indices[win_start[k] + i];
      if (idx < 0 || idx >= image_count) return CP_ERR_ARG;
      t[static_cast<size_t>(i)] = frames[idx];
    }
    tables.push_back(std::move(t));
    cp_stack s;
    std::memset(&s, 0, sizeof s);
    s.n = len;
    s.width = width;
    s.height = height;
    s.channels = channels;
    s.frames = tables.back().data();
    s.frame_offset = win_indices[win_start[k]];  // indices[0] (src/chrono.rs:103)
    stacks.push_back(s);
    ps.push_back(*params);
    o.push_back(outs[k]);
    b.push_back(out_blends ? out_blends[k] : nullptr);
    wp.push_back(warnings ? warnings + k : nullptr);
  }
  if (stacks.empty()) return CP_OK;
  return batch_run(ctx, stacks.data(), ps.data(), static_cast<int32_t>(stacks.size()), o.data(),
                   out_blends ? b.data() : nullptr, warnings ? wp.data() : nullptr, stream);
}
