// cp_stage.cpp — host-memory compositing (cp_composite): the replacement of the
// reference's time-slice pipeline (src/slicer.rs, src/streams.rs, the per-slice loop of
// src/chrono.rs:96-193). Whole frames are copied to the device in row bands on two copy
// streams (one stream of back-to-back host->device copies leaves the link idle between
// copies: 95-135 GB/s on GB300 for 2-32 MB copies, 207 GB/s with two streams); the kernel of
// band b runs while band b+1 is in flight, and each band's result is copied back on a
// fourth stream as soon as its kernel is done. Equally strided frames move as one 2D copy
// per band and stream. cp_composite_multi runs several parameter sets over each band, so the
// frames cross the host link once for all of them.

#include <cuda_runtime.h>

#include <algorithm>
#include <exception>
#include <cstring>
#include <vector>

#include "../../include/chrono_gpu.h"
#include "cp_host_internal.h"
#include "cp_internal.h"

using namespace cp;

namespace {

constexpr uint64_t kFrameAlign = 256;  // device frame pitch: keeps every frame 16-byte aligned

uint64_t round_up(uint64_t v, uint64_t a) { return (v + a - 1) / a * a; }

int ensure_events(cp_ctx* ctx, size_t count) {
  while (ctx->band_events.size() < count) {
    cudaEvent_t e;
    cudaError_t rc = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    if (rc != cudaSuccess) return cuda_status(ctx, rc, "cudaEventCreate");
    ctx->band_events.push_back(e);
  }
  return CP_OK;
}

}  // namespace

// The warning counters of the settings follow the error flags in the context's 256-byte
// flag block (cp_ctx_create).
static_assert(64 + 8 * CP_MAX_SETTINGS <= 256, "warning counters exceed the flag block");

// The host-staged composite of one stack under `count` parameter sets (cp_composite is
// count = 1, the only form that takes diagnostics).
static int composite_staged(cp_ctx* ctx, const cp_stack* stack, const cp_params* params,
                            int count, uint8_t* const* outs, uint8_t* const* blends,
                            const cp_debug* dbg, uint64_t* n_warnings) {
  if (!ctx || !stack || !params || !outs || count < 1) return CP_ERR_ARG;
  if (count > CP_MAX_SETTINGS) return CP_ERR_LIMIT;
  for (int k = 0; k < count; ++k)
    if (!outs[k]) return CP_ERR_ARG;
  if (stack->n < 1 || stack->n > CP_MAX_FRAMES || (!stack->frames && !stack->base))
    return CP_ERR_ARG;
  std::lock_guard<std::mutex> call(ctx->call_mu);
  cudaSetDevice(ctx->device);
  const int n = stack->n, C = stack->channels;
  const bool crop = stack->crop != nullptr;
  const int sw = crop ? stack->src_width : stack->width;
  const int sh = crop ? stack->src_height : stack->height;
  if (sw < 1 || sh < 1 || C < 1 || C > 4) return CP_ERR_ARG;
  const uint64_t frame_bytes = static_cast<uint64_t>(sw) * sh * C;
  const uint64_t pitch = round_up(frame_bytes + 16, kFrameAlign);
  const uint64_t P = static_cast<uint64_t>(stack->width) * stack->height;
  const uint64_t out_bytes = P * C;
  const uint64_t ostride = round_up(out_bytes, 256);  // one setting's output in out_dev
  std::vector<bool> want_blend(static_cast<size_t>(count));
  bool any_blend = false;
  for (int k = 0; k < count; ++k) {
    want_blend[static_cast<size_t>(k)] =
        blends && blends[k] && params[k].mode == CP_MODE_OUTLIER;
    any_blend = any_blend || want_blend[static_cast<size_t>(k)];
  }
  int rc = ensure_buffer(ctx, ctx->frames_dev, pitch * n);
  if (!rc) rc = ensure_buffer(ctx, ctx->out_dev, ostride * count);
  if (!rc && any_blend) rc = ensure_buffer(ctx, ctx->blend_dev, ostride * count);
  if (rc) return rc;

  // device frame table and one descriptor per setting
  uint8_t* fdev = static_cast<uint8_t*>(ctx->frames_dev.ptr);
  std::vector<const uint8_t*> dev_frames(static_cast<size_t>(n));
  for (int i = 0; i < n; ++i) dev_frames[static_cast<size_t>(i)] = fdev + pitch * i;
  std::vector<StackDev> ds(static_cast<size_t>(count));
  for (int k = 0; k < count; ++k) {
    StackDev& d = ds[static_cast<size_t>(k)];
    rc = prepare_stack(ctx, stack, &params[k], dev_frames.data(), &d);
    if (rc) return rc;
    d.out = static_cast<uint8_t*>(ctx->out_dev.ptr) + ostride * k;
    d.blend = want_blend[static_cast<size_t>(k)]
                  ? static_cast<uint8_t*>(ctx->blend_dev.ptr) + ostride * k
                  : nullptr;
    d.warnings = ctx->d_warn + k;  // CP_MAX_SETTINGS counters behind the error flags
  }

  // optional diagnostics: device arrays, copied back at the end
  const int words = (n + 31) / 32;
  struct DbgPart {
    void* host;
    uint64_t bytes;
    uint64_t off;
  };
  std::vector<DbgPart> parts;
  StackDev& d = ds[0];
  if (dbg && count == 1 && params->mode == CP_MODE_OUTLIER) {
    uint64_t off = 0;
    auto add = [&](void* h, uint64_t bytes) {
      if (!h) return;
      parts.push_back({h, bytes, off});
      off += round_up(bytes, 256);
    };
    add(dbg->median, P * C * 4);
    add(dbg->q1, P * C * 4);
    add(dbg->q3, P * C * 4);
    add(dbg->outlier_bits, P * words * 4);
    add(dbg->chosen, P * 4);
    add(dbg->background, P * 4);
    add(dbg->n_outliers, P * 4);
    if (off) {
      rc = ensure_buffer(ctx, ctx->dbg_dev, off);
      if (rc) return rc;
      uint8_t* base = static_cast<uint8_t*>(ctx->dbg_dev.ptr);
      size_t k = 0;
      auto ptr = [&](void* h) -> void* { return h ? base + parts[k++].off : nullptr; };
      d.dbg_median = static_cast<float*>(ptr(dbg->median));
      d.dbg_q1 = static_cast<float*>(ptr(dbg->q1));
      d.dbg_q3 = static_cast<float*>(ptr(dbg->q3));
      d.dbg_bits = static_cast<uint32_t*>(ptr(dbg->outlier_bits));
      d.dbg_chosen = static_cast<int32_t*>(ptr(dbg->chosen));
      d.dbg_bg = static_cast<int32_t*>(ptr(dbg->background));
      d.dbg_nout = static_cast<int32_t*>(ptr(dbg->n_outliers));
    }
  }

  rc = cuda_status(ctx, cudaMemsetAsync(ctx->d_warn, 0, sizeof(unsigned long long) * count,
                                        ctx->stream), "memset");
  if (rc) return rc;

  // bands: flat pixel ranges in whole tiles; cropped stacks move whole frames at once
  // (a band's copy and its multi-setting launch alternate on the link and the SMs; more
  // bands shorten the unhidden first copy and last launch, but a band much below 50 MB of
  // frames makes launches too small to fill the GPU: 8 bands of a 398 MB stack measured
  // 348 k Mpx-frames/s end to end against 338 k with 4, 12 bands no better)
  int bands = 1;
  if (!crop && P >= static_cast<uint64_t>(kTilePx) * ctx->sm_count * 4)
    bands = frame_bytes * static_cast<uint64_t>(n) >= (256ull << 20) ? 8 : 4;
  // per band: two copies landed, then the band's kernels done
  const int ev_band = 3;
  rc = ensure_events(ctx, static_cast<size_t>(ev_band * bands));
  if (rc) return rc;
  const uint64_t tiles_total = (P + kTilePx - 1) / kTilePx;
  auto host_frame = [&](int i) -> const uint8_t* {
    return stack->frames ? stack->frames[i] : stack->base + stack->frame_stride * i;
  };
  for (int b = 0; b < bands; ++b) {
    const uint64_t t0 = tiles_total * b / bands, t1 = tiles_total * (b + 1) / bands;
    const uint64_t px0 = t0 * kTilePx, px1 = std::min<uint64_t>(t1 * kTilePx, P);
    if (px1 <= px0) continue;
    // frames (or their band) host -> device: frames [0, half) on one copy stream, the rest
    // on the other
    cudaStream_t cs[2] = {ctx->copy_stream, ctx->copy_stream2};
    const int half = (n + 1) / 2;
    if (!crop && !stack->frames && stack->frame_stride >= static_cast<int64_t>(frame_bytes)) {
      const uint64_t w = (px1 - px0) * C;
      for (int k = 0; k < 2; ++k) {
        const int i0 = k ? half : 0, cnt = k ? n - half : half;
        if (cnt < 1) continue;
        rc = cuda_status(ctx, cudaMemcpy2DAsync(fdev + pitch * i0 + px0 * C, pitch,
                                                host_frame(i0) + px0 * C,
                                                static_cast<size_t>(stack->frame_stride), w,
                                                static_cast<size_t>(cnt), cudaMemcpyHostToDevice,
                                                cs[k]), "h2d");
        if (rc) return rc;
      }
    } else {
      for (int i = 0; i < n; ++i) {
        const uint8_t* src = host_frame(i);
        cudaStream_t st = cs[i < half ? 0 : 1];
        if (crop) {
          rc = cuda_status(ctx, cudaMemcpyAsync(fdev + pitch * i, src, frame_bytes,
                                                cudaMemcpyHostToDevice, st), "h2d");
        } else {
          rc = cuda_status(ctx, cudaMemcpyAsync(fdev + pitch * i + px0 * C, src + px0 * C,
                                                (px1 - px0) * C, cudaMemcpyHostToDevice, st),
                           "h2d");
        }
        if (rc) return rc;
      }
    }
    cudaEvent_t copied = ctx->band_events[static_cast<size_t>(ev_band * b)];
    cudaEvent_t copied2 = ctx->band_events[static_cast<size_t>(ev_band * b + 1)];
    cudaEventRecord(copied, cs[0]);
    cudaEventRecord(copied2, cs[1]);
    cudaStreamWaitEvent(ctx->stream, copied, 0);
    cudaStreamWaitEvent(ctx->stream, copied2, 0);
    const uint64_t o0 = crop ? 0 : px0 * C, ob = crop ? out_bytes : (px1 - px0) * C;
    // the band under every setting: settings sharing their order statistics in one
    // multi-setting launch (cp_outlier_multi.cuh), then every result back
    std::vector<StackDev> band(ds);
    for (StackDev& db : band) {
      if (!crop) {
        db.px_begin = static_cast<int32_t>(px0);
        db.px_end = static_cast<int32_t>(px1);
        db.tiles = static_cast<int32_t>(t1 - t0);
      }
    }
    rc = launch_multi(ctx, band, ctx->stream);
    if (rc) return rc;
    cudaEvent_t done = ctx->band_events[static_cast<size_t>(ev_band * b + 2)];
    cudaEventRecord(done, ctx->stream);
    cudaStreamWaitEvent(ctx->d2h_stream, done, 0);
    for (int k = 0; k < count; ++k) {
      const StackDev& db = band[static_cast<size_t>(k)];
      rc = cuda_status(ctx, cudaMemcpyAsync(outs[k] + o0, db.out + o0, ob,
                                            cudaMemcpyDeviceToHost, ctx->d2h_stream), "d2h");
      if (!rc && db.blend)
        rc = cuda_status(ctx, cudaMemcpyAsync(blends[k] + o0, db.blend + o0, ob,
                                              cudaMemcpyDeviceToHost, ctx->d2h_stream), "d2h");
      if (rc) return rc;
    }
  }
  uint64_t warn[CP_MAX_SETTINGS] = {};
  cudaEvent_t all = ctx->band_events[0];
  cudaEventRecord(all, ctx->stream);
  cudaStreamWaitEvent(ctx->d2h_stream, all, 0);
  rc = cuda_status(ctx, cudaMemcpyAsync(warn, ctx->d_warn, sizeof(uint64_t) * count,
                                        cudaMemcpyDeviceToHost, ctx->d2h_stream), "d2h");
  if (rc) return rc;
  for (const auto& part : parts) {
    rc = cuda_status(ctx, cudaMemcpyAsync(part.host, static_cast<uint8_t*>(ctx->dbg_dev.ptr) + part.off,
                                          part.bytes, cudaMemcpyDeviceToHost, ctx->d2h_stream),
                     "d2h");
    if (rc) return rc;
  }
  rc = cuda_status(ctx, cudaStreamSynchronize(ctx->d2h_stream), "synchronize");
  if (rc) return rc;
  rc = check_device_error(ctx);
  if (rc) return rc;
  if (n_warnings)
    for (int k = 0; k < count; ++k) n_warnings[k] = warn[k];
  return CP_OK;
}

// composite_staged with no C++ exception crossing the C ABI (host allocations).
static int composite_guarded(cp_ctx* ctx, const cp_stack* stack, const cp_params* params,
                             int count, uint8_t* const* outs, uint8_t* const* blends,
                             const cp_debug* dbg, uint64_t* n_warnings) {
  try {
    return composite_staged(ctx, stack, params, count, outs, blends, dbg, n_warnings);
  } catch (const std::exception& e) {
    ctx_error(ctx, "host staging: %s", e.what());
    return CP_ERR_OOM;
  }
}

extern "C" int cp_composite(cp_ctx* ctx, const cp_stack* stack, const cp_params* params,
                            uint8_t* out, uint8_t* out_blend, const cp_debug* dbg,
                            uint64_t* n_warnings) {
  return composite_guarded(ctx, stack, params, 1, &out, &out_blend, dbg, n_warnings);
}

extern "C" int cp_composite_multi(cp_ctx* ctx, const cp_stack* stack, const cp_params* params,
                                  int32_t count, uint8_t* const* out, uint8_t* const* out_blend,
                                  uint64_t* n_warnings) {
  return composite_guarded(ctx, stack, params, count, out, out_blend, nullptr, n_warnings);
}
