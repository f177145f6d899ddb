// cp_prepare.cpp — option semantics on the host: error text, the fade table, quantile
// positions and prepare_stack, which turns a stack and its options into the kernels' StackDev
// descriptor; the C ABI's status strings, default options, fade table and cp_ctx_last_error.
// Host-only code (no device calls), shared by every entry point and the server.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/chrono_gpu.h"
#include "cp_host_internal.h"
#include "cp_internal.h"

namespace cp {

void ctx_error(cp_ctx* ctx, const char* fmt, ...) {
  if (!ctx) return;
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  std::lock_guard<std::mutex> lk(ctx->err_mu);
  ctx->last_error = buf;
}

int cuda_status(cp_ctx* ctx, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return CP_OK;
  ctx_error(ctx, "%s: %s", what, cudaGetErrorString(e));
  if (e == cudaErrorMemoryAllocation) return CP_ERR_OOM;
  return CP_ERR_CUDA;
}

// Fade::new / Fade::get / fade() (src/options.rs:69-139, src/chrono.rs:496-502).
int fade_lut(const cp_fade* f, int32_t n, int32_t frame_offset, float* out) {
  if (n < 0 || (n > 0 && !out)) return CP_ERR_ARG;
  if (!f || !f->enabled) {
    for (int i = 0; i < n; ++i) out[i] = 1.0f;
    return CP_OK;
  }
  if (f->n_points < 2 || !f->frames || !f->values) return CP_ERR_ARG;
  const int32_t offset = f->frames[0];
  const int32_t last = f->frames[f->n_points - 1];
  if (last < offset) return CP_ERR_ARG;
  const size_t len = static_cast<size_t>(last - offset);
  std::vector<float> values(len + 1, 1.0f);
  size_t idx = 0;
  for (size_t i = 0; i < len + 1; ++i) {
    if (idx + 1 >= static_cast<size_t>(f->n_points)) return CP_ERR_ARG;
    const int32_t f1 = f->frames[idx], f2 = f->frames[idx + 1];
    const float v1 = f->values[idx], v2 = f->values[idx + 1];
    const int32_t frame = static_cast<int32_t>(i) + offset;
    // v1 + (v2 - v1) * (frame - f1) as f32 / (f2 - f1) as f32, left to right
    values[i] = v1 + (v2 - v1) * static_cast<float>(frame - f1) / static_cast<float>(f2 - f1);
    if (frame == f2) idx += 1;
  }
  const int32_t vlen = static_cast<int32_t>(values.size());
  auto get = [&](int32_t frame) -> float {
    int32_t i = frame - offset;
    if (i >= 0 && i < vlen) return values[static_cast<size_t>(i)];
    if (!f->repeat) return i < 0 ? values[0] : values[static_cast<size_t>(vlen - 1)];
    while (i < 0) i += vlen;
    return values[static_cast<size_t>(i % vlen)];
  };
  for (int32_t i = 0; i < n; ++i) out[i] = f->absolute ? get(frame_offset + i) : get(n - i - 1);
  return CP_OK;
}

// quantile() index resolution of src/chrono.rs:567-579 for a sample of `len` values.
static void quantile_spec(int len, float q, int32_t* k, int32_t* pair, float* frac) {
  const float pos = static_cast<float>(len + 1) * q;
  const int p1 = static_cast<int>(pos) - 1;
  const float fr = pos - std::trunc(pos);
  if (fr < 0.001f) {
    *k = p1;
    *pair = 0;
    *frac = 0.0f;
  } else if (fr > 0.999f) {
    *k = p1 + 1;
    *pair = 0;
    *frac = 0.0f;
  } else {
    *k = p1;
    *pair = 1;
    *frac = fr;
  }
}

int prepare_stack(cp_ctx* ctx, const cp_stack* st, const cp_params* p,
                  const uint8_t* const* dev_frames, StackDev* d) {
  if (!st || !p || !d) return CP_ERR_ARG;
  const int n = st->n;
  if (n < 1 || n > CP_MAX_FRAMES) {
    ctx_error(ctx, "stack of %d frames: supported 1..%d", n, CP_MAX_FRAMES);
    return CP_ERR_ARG;
  }
  if (st->width < 1 || st->height < 1 ||
      static_cast<int64_t>(st->width) * st->height > (int64_t(1) << 30)) {
    ctx_error(ctx, "image size %dx%d unsupported", st->width, st->height);
    return CP_ERR_ARG;
  }
  if (st->channels != 1 && st->channels != 3 && st->channels != 4) {
    ctx_error(ctx, "%d channels unsupported (1, 3 or 4)", st->channels);
    return CP_ERR_ARG;
  }
  if (p->mode < CP_MODE_OUTLIER || p->mode > CP_MODE_LIGHTER) return CP_ERR_ARG;
  if (p->mode == CP_MODE_OUTLIER) {
    if (p->outlier < CP_OUTLIER_FIRST || p->outlier > CP_OUTLIER_BACKWARD) return CP_ERR_ARG;
    if (p->background < CP_BG_FIRST || p->background > CP_BG_MEDIAN) return CP_ERR_ARG;
  }
  std::memset(d, 0, sizeof(*d));
  d->n = n;
  d->width = st->width;
  d->height = st->height;
  d->channels = st->channels;
  d->has_crop = st->crop != nullptr;
  d->src_width = d->has_crop ? st->src_width : st->width;
  if (d->has_crop) {
    if (st->src_width < st->width || st->src_height < st->height) return CP_ERR_ARG;
    for (int i = 0; i < n; ++i) {
      const int cx = st->crop[2 * i], cy = st->crop[2 * i + 1];
      if (cx < 0 || cy < 0 || cx + st->width > st->src_width || cy + st->height > st->src_height) {
        ctx_error(ctx, "crop origin (%d,%d) of frame %d outside the source", cx, cy, i);
        return CP_ERR_ARG;
      }
      d->crop[2 * i] = cx;
      d->crop[2 * i + 1] = cy;
    }
  }
  bool shifted = d->has_crop;
  for (int i = 0; i < n; ++i) {
    d->frames[i] = dev_frames[i];
    if (!dev_frames[i]) return CP_ERR_ARG;
    if (reinterpret_cast<uintptr_t>(dev_frames[i]) & 15) shifted = true;
  }
  d->shifted = shifted;
  d->threads = cta_threads(st->channels);
  d->tile_px = kTilePx;
  d->nw = nw_for(n);
  d->px_begin = 0;
  d->px_end = st->width * st->height;
  d->row_begin = 0;
  if (d->has_crop) {
    d->tiles_per_row = (st->width + kTilePx - 1) / kTilePx;
    d->tiles = d->tiles_per_row * st->height;
  } else {
    d->tiles_per_row = 0;
    d->tiles = (d->px_end + kTilePx - 1) / kTilePx;
  }
  // options
  d->mode = p->mode;
  d->outlier = p->outlier;
  d->background = p->background;
  d->thr_abs = p->thr_abs ? 1 : 0;
  bool unit = true, neg = false, finite = true;
  uint32_t wmask = 0;
  for (int c = 0; c < 4; ++c) {
    d->w[c] = p->weights[c];
    if (c < st->channels && p->weights[c] != 0.0f) wmask |= 1u << c;
    if (c < st->channels && !(p->weights[c] == 0.0f || p->weights[c] == 1.0f)) unit = false;
    if (c < st->channels && std::signbit(p->weights[c]) && p->weights[c] != 0.0f) neg = true;
    if (c < st->channels && std::isnan(p->weights[c])) neg = true;
    if (c < st->channels && !(std::fabs(p->weights[c]) < 1e30f)) finite = false;
  }
  d->wmask = wmask;
  d->neg_w = neg ? 1u : 0u;
  d->unit_w = unit ? 1u : 0u;
  d->finite_w = finite ? 1u : 0u;
  d->fast_int = (d->thr_abs && unit) ? 1u : 0u;
  // Threshold::new, src/options.rs:197-213 (f32 arithmetic)
  if (d->thr_abs) {
    d->thr_min = p->thr_min * 255.0f;
    d->thr_max = p->thr_max * 255.0f;
    d->thr_scale = 1.0f / ((p->thr_max - p->thr_min) * 255.0f);
  } else {
    d->thr_min = p->thr_min;
    d->thr_max = p->thr_max;
    d->thr_scale = 1.0f / (p->thr_max - p->thr_min);
  }
  d->thr_sq = d->thr_min * d->thr_min;  // src/chrono.rs:220
  // The paired f32 distance pass computes every term on (median - p) / 2, i.e. each term,
  // sum and threshold scaled by exactly 1/4. Scaling by a power of two commutes with f32
  // rounding while no value leaves the normal range: nonzero weights within [2^-53, 2^39]
  // keep |t| = |w * iqr_inv * diff| (iqr_inv <= 2^16, 1/2 <= |diff| <= 255) and t^2 / 4
  // normal and the three-term sum finite; negative weights (cancelling sums) are excluded.
  bool pair = finite && !neg && std::isfinite(d->thr_sq) &&
              (d->thr_sq == 0.0f || d->thr_sq >= std::ldexp(1.0f, -124));
  for (int c = 0; c < st->channels; ++c) {
    const float a = std::fabs(p->weights[c]);
    if (a != 0.0f && !(a >= std::ldexp(1.0f, -53) && a <= std::ldexp(1.0f, 39))) pair = false;
  }
  d->pair_f32 = pair ? 1u : 0u;
  for (int nh = 0; nh <= 4; ++nh) {
    // smallest integer D' with D' + nh/4 >= thr_sq (exact in double)
    const double need = static_cast<double>(d->thr_sq) - 0.25 * nh;
    double t;
    if (std::isnan(need))
      t = 2147483647.0;
    else
      t = std::ceil(need);
    if (t < 0) t = 0;
    if (t > 2147483647.0) t = 2147483647.0;
    d->thr_int[nh] = static_cast<int32_t>(t);
  }
  // (sub)sample for the order statistics
  int len = n;
  d->sample_mask[0] = d->sample_mask[1] = d->sample_mask[2] = d->sample_mask[3] = 0;
  if (p->sample && p->n_sample > 0 && p->n_sample < n) {
    len = p->n_sample;
    int prev = -1;
    for (int i = 0; i < p->n_sample; ++i) {
      const int s = p->sample[i];
      if (s <= prev || s >= n) {
        ctx_error(ctx, "sample indices must be sorted, distinct and < n");
        return CP_ERR_ARG;
      }
      prev = s;
      d->sample_mask[s >> 5] |= 1u << (s & 31);
    }
  } else {
    for (int i = 0; i < n; ++i) d->sample_mask[i >> 5] |= 1u << (i & 31);
  }
  d->n_sub = len;
  if (p->mode == CP_MODE_OUTLIER && !p->thr_abs && len < 3) {
    ctx_error(ctx, "relative threshold needs at least 3 samples (got %d)", len);
    return CP_ERR_ARG;
  }
  // median(), src/chrono.rs:582-591
  if ((len + 1) % 2 == 0) {
    d->med_k = (len + 1) / 2 - 1;
    d->med_pair = 0;
  } else {
    d->med_k = (len + 1) / 2 - 1;
    d->med_pair = 1;
  }
  if (!p->thr_abs) {
    quantile_spec(len, 0.25f, &d->q1_k, &d->q1_pair, &d->q1_frac);
    quantile_spec(len, 0.75f, &d->q3_k, &d->q3_pair, &d->q3_frac);
  }
  d->seed = p->rng_seed;
  d->wait_cycles = (ctx && ctx->wait_cycles > 0) ? ctx->wait_cycles : kDefaultWaitCycles;
  if (fade_lut(&p->fade, n, st->frame_offset, d->fade) != CP_OK) {
    ctx_error(ctx, "invalid fade specification");
    return CP_ERR_ARG;
  }
  d->no_fade = 1u;
  d->unit_fade = 1u;
  for (int i = 0; i < n; ++i) {
    if (!(d->fade[i] >= 1.0f)) d->no_fade = 0u;
    if (d->fade[i] != 1.0f) d->unit_fade = 0u;
  }
  return CP_OK;
}

}  // namespace cp

extern "C" {

const char* cp_status_str(int status) {
  switch (status) {
    case CP_OK: return "ok";
    case CP_ERR_ARG: return "invalid argument";
    case CP_ERR_OOM: return "out of memory";
    case CP_ERR_TIMEOUT: return "timed out";
    case CP_ERR_CUDA: return "CUDA error";
    case CP_ERR_BUDGET: return "HBM budget exceeded";
    case CP_ERR_RANGE: return "coordinate out of range";
    case CP_ERR_STATE: return "invalid state";
    case CP_ERR_NODEV: return "no sm_103 device";
    case CP_ERR_LIMIT: return "request above the fixed limit of the allocation-free entry point";
    case CP_ERR_CANCELLED: return "job cancelled";
    case CP_ERR_IO: return "image file missing, unreadable or unsupported";
    default: return "unknown status";
  }
}

void cp_params_default(cp_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->mode = CP_MODE_OUTLIER;
  p->thr_abs = 1;
  p->thr_min = 0.05f;
  p->thr_max = 0.2f;
  p->outlier = CP_OUTLIER_EXTREME;
  p->background = CP_BG_RANDOM;
  for (float& w : p->weights) w = 1.0f;
  p->fade.enabled = 0;
  p->rng_seed = 0x5EEDull;
}

int cp_fade_lut(const cp_fade* fade, int32_t n, int32_t frame_offset, float* out) {
  return cp::fade_lut(fade, n, frame_offset, out);
}

int cp_ctx_last_error(cp_ctx* ctx, char* buf, size_t len) {
  if (!ctx || !buf || len == 0) return CP_ERR_ARG;
  std::lock_guard<std::mutex> lk(ctx->err_mu);
  std::snprintf(buf, len, "%s", ctx->last_error.c_str());
  return CP_OK;
}

}  // extern "C"
