// chrono_oracle.cpp — CPU restatement of chrono-photo 0.6.5's compositing hot path.
//
// TEST INFRASTRUCTURE ONLY. This file is the parity oracle: only the test suite, the smoke
// check and the CPU-baseline leg of the benchmark load it, as the checker or as the timed
// CPU reference. The product library never links or calls it.
//
// The reference is Rust and cannot be built here, so every function below restates the
// reference's arithmetic in the same f32 operation order (compiled with
// -ffp-contract=off: no fused multiply-add, as rustc emits none). Rust semantics that C++
// does not share are written out: `f32::round` is round-half-away (roundf), `f32 as u8`
// saturates (NaN -> 0), integer overflow in the release profile wraps (Cargo.toml:7-13).
// Parity pins: the reference's only known-answer test on this path, quartiles_test
// (src/chrono.rs:598-604), plus hand-derived known answers in tests/golden/.
//
// The two places where the reference uses an unseeded ThreadRng (--background random,
// --sample) take a seeded counter-based generator here and in the CUDA library; their
// parity with the Rust binary is distributional only.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "../include/chrono_gpu.h"

namespace {

// Rust `f32 as u8`: saturating, NaN -> 0.
inline uint8_t sat_u8(float v) {
  if (!(v > 0.0f)) return 0;  // NaN, negatives, zero
  if (v >= 255.0f) return 255;
  return (uint8_t)v;  // truncation toward zero, as `as` does
}
// Rust `f32::round`: half away from zero.
inline float rround(float v) { return std::round(v); }
// Rust `f32::signum`: +-1 by the sign bit, NaN for NaN.
inline float rsignum(float w) { return std::isnan(w) ? w : (std::signbit(w) ? -1.0f : 1.0f); }

// Counter-based draw replacing ThreadRng::gen_range(0, n): splitmix64 of the seed and the
// (pixel, draw) counter, scaled by a 32x32 multiply-high. Shared with the CUDA library.
inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
inline uint32_t gen_range(uint64_t seed, uint64_t pixel, uint32_t n) {
  uint64_t h = splitmix64(seed ^ splitmix64(pixel));
  return (uint32_t)(((h >> 32) * (uint64_t)n) >> 32);
}

// Threshold, src/options.rs:189-244.
struct Threshold {
  bool absolute;
  float min, max, scale;
  Threshold(bool abs, float mn, float mx) : absolute(abs) {
    if (abs) {  // options.rs:198-204: bounds scaled by 255, scale from the raw bounds
      min = mn * 255.0f;
      max = mx * 255.0f;
      scale = 1.0f / ((mx - mn) * 255.0f);
    } else {  // options.rs:206-211
      min = mn;
      max = mx;
      scale = 1.0f / (mx - mn);
    }
  }
  // options.rs:223-231
  float blend_value(float dist) const {
    if (dist <= min) return 0.0f;
    if (dist >= max) return 1.0f;
    return (dist - min) * scale;
  }
};

// Fade, src/options.rs:60-139.
struct Fade {
  bool is_none = true, repeat = false, absolute = true;
  int32_t offset = 0;
  std::vector<float> values;
  static bool build(const cp_fade* f, Fade* out) {
    Fade r;
    if (!f || !f->enabled) {  // Fade::none(), options.rs:97-105
      *out = r;
      return true;
    }
    if (f->n_points < 2 || !f->frames || !f->values) return false;  // options.rs:73 expect
    r.is_none = false;
    r.repeat = f->repeat != 0;
    r.absolute = f->absolute != 0;
    r.offset = f->frames[0];  // options.rs:70
    int32_t last = f->frames[f->n_points - 1];
    if (last < r.offset) return false;
    size_t len = (size_t)(last - r.offset);  // options.rs:71-75
    r.values.assign(len + 1, 1.0f);
    size_t idx = 0;
    for (size_t i = 0; i < len + 1; ++i) {  // options.rs:78-86
      if (idx + 1 >= (size_t)f->n_points) return false;
      int32_t f1 = f->frames[idx], f2 = f->frames[idx + 1];
      float v1 = f->values[idx], v2 = f->values[idx + 1];
      int32_t frame = (int32_t)i + r.offset;
      r.values[i] = v1 + (v2 - v1) * (float)(frame - f1) / (float)(f2 - f1);
      if (frame == f2) idx += 1;
    }
    *out = r;
    return true;
  }
  // options.rs:113-139
  float get(int32_t frame) const {
    if (is_none) return 1.0f;
    int32_t i = frame - offset;
    int32_t len = (int32_t)values.size();
    if (i >= 0 && i < len) return values[(size_t)i];
    if (!repeat) return i < 0 ? values[0] : values[(size_t)len - 1];
    while (i < 0) i += len;
    i = i % len;
    return values[(size_t)i];
  }
  // fade(), src/chrono.rs:496-502 and src/simple.rs:170-176
  float at(int32_t frame, int32_t total, int32_t offs) const {
    return absolute ? get(offs + frame) : get(total - frame - 1);
  }
};

// color.rs:4-16
inline void blend_into_u8(uint8_t* a, const uint8_t* b, int c, float blend) {
  c = std::min(c, 4);
  if (blend <= 0.0f) {
  } else if (blend >= 1.0f) {
    for (int i = 0; i < c; ++i) a[i] = b[i];
  } else {
    for (int i = 0; i < c; ++i) {
      float aa = (float)a[i];
      a[i] = sat_u8(rround(aa + ((float)b[i] - aa) * blend));
    }
  }
}
// color.rs:32-44
inline void blend_into_f32_u8(float* a, const uint8_t* b, int c, float blend) {
  if (blend <= 0.0f) {
  } else if (blend >= 1.0f) {
    for (int i = 0; i < c; ++i) a[i] = (float)b[i];
  } else {
    for (int i = 0; i < c; ++i) {
      float aa = a[i];
      a[i] = aa + ((float)b[i] - aa) * blend;
    }
  }
}

// chrono.rs:567-579. Requires len >= 3 (the reference underflows p1 and panics below that).
inline float quantile(const uint8_t* d, size_t len, float q) {
  float pos = (float)(len + 1) * q;
  size_t p1 = (size_t)pos - 1;
  float frac = pos - std::trunc(pos);
  if (frac < 0.001f) return (float)d[p1];
  if (frac > 0.999f) return (float)d[p1 + 1];
  return (1.0f - frac) * (float)d[p1] + frac * (float)d[p1 + 1];
}
// chrono.rs:581-591
inline float median(const uint8_t* d, size_t len) {
  if ((len + 1) % 2 == 0) return (float)d[(len + 1) / 2 - 1];
  size_t idx = (len + 1) / 2;
  return 0.5f * ((float)d[idx - 1] + (float)d[idx]);
}

struct PixelOut {
  float median[4], q1[4], q3[4];
  int32_t chosen, background, n_outliers;
  bool warning;
  uint8_t blend;
};

// Per-stack state of OutlierProcessor (chrono.rs:32-42, ThreadData :23-28).
struct Outlier {
  Threshold thr;
  int32_t background, outlier;
  float weights[4];
  const float* fade_lut;  // fade(i, samples, frame_offset) for every sample i
  std::vector<int32_t> sample_indices;
  uint64_t seed;
  // ThreadData
  std::vector<std::pair<size_t, float>> outlier_indices;
  std::vector<size_t> non_outlier_indices;
  std::vector<uint8_t> values;

  // first_excluded, chrono.rs:504-530
  std::pair<size_t, bool> first_excluded(size_t samples, size_t num_outliers) const {
    if (num_outliers == samples) return {0, true};
    size_t excl = 0;
    for (size_t i = 0; i < samples; ++i) {
      if (excl < num_outliers && i == outlier_indices[excl].first)
        excl += 1;
      else
        return {i, false};
    }
    return {0, true};  // unreachable: num_outliers < samples
  }
  // sample_excluded, chrono.rs:531-555 (swap-based candidate list, seeded draw)
  std::pair<size_t, bool> sample_excluded(size_t samples, size_t num_outliers, uint64_t pixel) {
    if (num_outliers == samples) return {gen_range(seed, pixel, (uint32_t)samples), true};
    for (size_t i = 0; i < non_outlier_indices.size(); ++i) non_outlier_indices[i] = i;
    size_t candidates = samples;
    for (size_t j = 0; j < num_outliers; ++j) {
      std::swap(non_outlier_indices[outlier_indices[j].first], non_outlier_indices[candidates - 1]);
      candidates -= 1;
    }
    size_t idx = gen_range(seed, pixel, (uint32_t)candidates);
    return {non_outlier_indices[idx], false};
  }

  // calc_pixel, chrono.rs:208-494. `px(i)` is the C-byte sample of frame i.
  template <typename PX>
  void calc_pixel(PX px, size_t samples, int channels, uint8_t* pixel, uint64_t pixel_id,
                  PixelOut* o) {
    const size_t sub_samples = sample_indices.size();
    const float threshold_sq = thr.min * thr.min;  // :220
    float med[4] = {0, 0, 0, 0}, iqr_inv[4] = {0, 0, 0, 0};
    for (int c = 0; c < 4; ++c) o->q1[c] = o->q3[c] = 0.0f;

    // :227-235 gather of the (sub)sample for weighted channels
    for (size_t s = 0; s < sub_samples; ++s) {
      const uint8_t* p = px(sample_indices[s]);
      for (int ch = 0; ch < channels; ++ch)
        if (weights[ch] != 0.0f) values[(size_t)ch * sub_samples + s] = p[ch];
    }
    // :238-255 medians and inverse IQR
    for (int i = 0; i < channels; ++i) {
      if (weights[i] != 0.0f) {
        uint8_t* sl = &values[(size_t)i * sub_samples];
        std::sort(sl, sl + sub_samples);
        if (thr.absolute) {
          med[i] = median(sl, sub_samples);
        } else {
          float q1 = quantile(sl, sub_samples, 0.25f);
          float md = median(sl, sub_samples);
          float q3 = quantile(sl, sub_samples, 0.75f);
          med[i] = md;
          o->q1[i] = q1;
          o->q3[i] = q3;
          iqr_inv[i] = q3 - q1;
          if (iqr_inv[i] == 0.0f) iqr_inv[i] = 1.0f;
          iqr_inv[i] = 1.0f / iqr_inv[i];
        }
      }
    }

    // :257-288 distance to the median over ALL samples; outliers in ascending order
    size_t num_outliers = 0;
    float max_dist_sq = 0.0f;
    size_t max_index = 0;
    for (size_t s = 0; s < samples; ++s) {
      const uint8_t* p = px(s);
      float dist_sq = 0.0f;
      for (int i = 0; i < channels; ++i) {
        float w = weights[i];
        if (w != 0.0f) {
          float diff = med[i] - (float)p[i];
          float term;
          if (diff == 0.0f) {
            term = 0.0f;
          } else if (thr.absolute) {
            float t = w * diff;
            term = rsignum(w) * (t * t);
          } else {
            float t = w * iqr_inv[i] * diff;
            term = rsignum(w) * (t * t);
          }
          dist_sq += term;
        }
      }
      if (dist_sq >= threshold_sq) {
        outlier_indices[num_outliers] = {s, dist_sq};
        num_outliers += 1;
        if (dist_sq > max_dist_sq) {
          max_dist_sq = dist_sq;
          max_index = s;
        }
      }
    }

    const bool has_outliers = num_outliers > 0;
    bool has_warning = false;
    o->background = -1;

    // :293-375 background
    if (background == CP_BG_AVERAGE) {
      float mean[4] = {0, 0, 0, 0};
      for (size_t s = 0; s < samples; ++s) {
        const uint8_t* p = px(s);
        for (int i = 0; i < channels; ++i) mean[i] += (float)p[i];
      }
      for (int i = 0; i < 4; ++i) mean[i] /= (float)samples;
      if (has_outliers) {
        if (num_outliers == 1) {
          const uint8_t* sample = px(outlier_indices[0].first);
          for (int ch = 0; ch < channels; ++ch)
            pixel[ch] = sat_u8(rround(mean[ch] * ((float)samples / (float)(samples - 1)) -
                                      (float)sample[ch] / (float)samples));
        } else {
          float outlier_sum[4] = {0, 0, 0, 0};
          for (size_t j = 0; j < num_outliers; ++j) {
            const uint8_t* p = px(outlier_indices[j].first);
            for (int ch = 0; ch < channels; ++ch) outlier_sum[ch] += (float)p[ch];
          }
          size_t num_non_outliers = samples - num_outliers;
          for (int ch = 0; ch < channels; ++ch)
            pixel[ch] = sat_u8(rround(mean[ch] * ((float)samples / (float)num_non_outliers) -
                                      outlier_sum[ch] / (float)samples));
        }
      } else {
        for (int ch = 0; ch < channels; ++ch) pixel[ch] = sat_u8(rround(mean[ch]));
      }
    } else if (background == CP_BG_MEDIAN) {
      for (int ch = 0; ch < channels; ++ch) pixel[ch] = sat_u8(rround(med[ch]));
    } else {  // First | Random
      std::pair<size_t, bool> sel;
      if (background == CP_BG_FIRST)
        sel = has_outliers ? first_excluded(samples, num_outliers) : std::make_pair((size_t)0, false);
      else
        sel = has_outliers ? sample_excluded(samples, num_outliers, pixel_id)
                           : std::make_pair((size_t)gen_range(seed, pixel_id, (uint32_t)samples), false);
      const uint8_t* sample = px(sel.first);
      for (int ch = 0; ch < channels; ++ch) pixel[ch] = sample[ch];
      if (sel.second) has_warning = true;
      o->background = (int32_t)sel.first;
    }

    for (int c = 0; c < 4; ++c) o->median[c] = med[c];
    o->n_outliers = (int32_t)num_outliers;
    o->warning = has_warning;
    o->chosen = -1;

    // :377-493 outlier pick and blend
    if (!has_outliers) {
      o->blend = 0;
      return;
    }
    if (num_outliers == 1) {
      size_t si = outlier_indices[0].first;
      float dsq = outlier_indices[0].second;
      float blend = fade_lut[si] * thr.blend_value(std::sqrt(dsq));
      blend_into_u8(pixel, px(si), channels, blend);
      o->blend = sat_u8(rround(blend * 255.0f));
      o->chosen = (int32_t)si;
      return;
    }
    if (outlier == CP_OUTLIER_FORWARD || outlier == CP_OUTLIER_BACKWARD) {
      float pix_new[4] = {0, 0, 0, 0};
      float blend_inv = 1.0f;
      for (int ch = 0; ch < channels; ++ch) pix_new[ch] = (float)pixel[ch];
      for (size_t jj = 0; jj < num_outliers; ++jj) {
        size_t j = outlier == CP_OUTLIER_FORWARD ? jj : num_outliers - 1 - jj;
        size_t si = outlier_indices[j].first;
        float blend = fade_lut[si] * thr.blend_value(std::sqrt(outlier_indices[j].second));
        blend_into_f32_u8(pix_new, px(si), channels, blend);
        blend_inv *= 1.0f - blend;
      }
      for (int ch = 0; ch < channels; ++ch) pixel[ch] = sat_u8(rround(pix_new[ch]));
      o->blend = sat_u8(rround((1.0f - blend_inv) * 255.0f));
      o->chosen = -2;
      return;
    }
    uint8_t temp_sample[4] = {0, 0, 0, 0};
    size_t si;
    const uint8_t* sample;
    float dist;
    if (outlier == CP_OUTLIER_AVERAGE) {
      // :439-453 computes the mean over all samples and then zeroes it: no effect.
      float mean[4] = {0, 0, 0, 0};
      float mean_dist = 0.0f;
      for (size_t j = 0; j < num_outliers; ++j) {
        const uint8_t* p = px(outlier_indices[j].first);
        for (int ch = 0; ch < channels; ++ch) mean[ch] += (float)p[ch];
        mean_dist += std::sqrt(outlier_indices[j].second);
      }
      for (int ch = 0; ch < channels; ++ch)
        temp_sample[ch] = sat_u8(rround(mean[ch] / (float)num_outliers));
      si = 0;
      sample = temp_sample;
      dist = mean_dist / (float)num_outliers;
    } else {
      float dsq;
      if (outlier == CP_OUTLIER_FIRST) {
        si = outlier_indices[0].first;
        dsq = outlier_indices[0].second;
      } else if (outlier == CP_OUTLIER_LAST) {
        si = outlier_indices[num_outliers - 1].first;
        dsq = outlier_indices[num_outliers - 1].second;
      } else {  // Extreme
        si = max_index;
        dsq = max_dist_sq;
      }
      sample = px(si);
      dist = std::sqrt(dsq);
    }
    float blend = fade_lut[si] * thr.blend_value(dist);
    blend_into_u8(pixel, sample, channels, blend);
    o->blend = sat_u8(rround(blend * 255.0f));
    o->chosen = (int32_t)si;
  }
};

bool valid_params(const cp_stack* s, const cp_params* p) {
  if (!s || !p) return false;
  if (s->n < 1 || s->n > CP_MAX_FRAMES || s->width < 1 || s->height < 1) return false;
  if (s->channels < 1 || s->channels > 4) return false;
  if (!s->frames && !s->base) return false;
  if (s->crop && (s->src_width < s->width || s->src_height < s->height)) return false;
  return true;
}

struct StackView {
  const cp_stack* s;
  int32_t sw;  // source row width in pixels
  const uint8_t* frame(int i) const {
    return s->frames ? s->frames[i] : s->base + (int64_t)i * s->frame_stride;
  }
  const uint8_t* at(int i, int x, int y) const {
    int cx = 0, cy = 0;
    if (s->crop) {
      cx = s->crop[2 * i];
      cy = s->crop[2 * i + 1];
    }
    return frame(i) + ((int64_t)(y + cy) * sw + (x + cx)) * s->channels;
  }
};

int outlier_rows(const cp_stack* st, const cp_params* p, const float* lut, int y0, int y1,
                 uint8_t* out, uint8_t* blend_out, const cp_debug* dbg, uint64_t* warnings) {
  const int C = st->channels, N = st->n, W = st->width;
  Outlier proc{Threshold(p->thr_abs != 0, p->thr_min, p->thr_max), p->background, p->outlier,
               {p->weights[0], p->weights[1], p->weights[2], p->weights[3]}, lut, {}, p->rng_seed,
               {}, {}, {}};
  if (p->sample && p->n_sample > 0 && p->n_sample < N) {
    proc.sample_indices.assign(p->sample, p->sample + p->n_sample);
  } else {
    proc.sample_indices.resize((size_t)N);
    for (int i = 0; i < N; ++i) proc.sample_indices[(size_t)i] = i;
  }
  proc.outlier_indices.assign((size_t)N, {0, 0.0f});
  proc.non_outlier_indices.assign((size_t)N, 0);
  proc.values.assign(proc.sample_indices.size() * (size_t)C, 0);
  StackView v{st, st->crop ? st->src_width : st->width};
  const int words = (N + 31) / 32;
  uint64_t warn = 0;
  uint8_t pixel[4];
  PixelOut o;
  for (int y = y0; y < y1; ++y) {
    for (int x = 0; x < W; ++x) {
      const uint64_t pid = (uint64_t)y * (uint64_t)W + (uint64_t)x;
      auto px = [&](size_t i) { return v.at((int)i, x, y); };
      proc.calc_pixel(px, (size_t)N, C, pixel, pid, &o);
      if (o.warning) warn += 1;
      // chrono.rs:183-191: composite and blend mask (255 in channels >= 3)
      for (int ch = 0; ch < C; ++ch) {
        out[pid * C + ch] = pixel[ch];
        if (blend_out) blend_out[pid * C + ch] = ch < 3 ? o.blend : 255;
      }
      if (dbg) {
        for (int ch = 0; ch < C; ++ch) {
          if (dbg->median) dbg->median[pid * C + ch] = o.median[ch];
          if (dbg->q1) dbg->q1[pid * C + ch] = o.q1[ch];
          if (dbg->q3) dbg->q3[pid * C + ch] = o.q3[ch];
        }
        if (dbg->outlier_bits) {
          uint32_t* bits = dbg->outlier_bits + pid * words;
          for (int wd = 0; wd < words; ++wd) bits[wd] = 0;
          for (int j = 0; j < o.n_outliers; ++j) {
            size_t si = proc.outlier_indices[(size_t)j].first;
            bits[si / 32] |= 1u << (si % 32);
          }
        }
        if (dbg->chosen) dbg->chosen[pid] = o.chosen;
        if (dbg->background) dbg->background[pid] = o.background;
        if (dbg->n_outliers) dbg->n_outliers[pid] = o.n_outliers;
      }
    }
  }
  *warnings += warn;
  return CP_OK;
}

// SimpleProcessor fold, src/simple.rs:96-133, over rows [y0, y1).
int simple_rows(const cp_stack* st, const cp_params* p, const float* lut, int y0, int y1,
                uint8_t* out) {
  const int C = st->channels, N = st->n, W = st->width;
  const bool darker = p->mode == CP_MODE_DARKER;
  StackView v{st, st->crop ? st->src_width : st->width};
  std::vector<float> extreme((size_t)W);
  for (int y = y0; y < y1; ++y) {
    uint8_t* row = out + (size_t)y * W * C;
    std::memset(row, 0, (size_t)W * C);  // simple.rs:71-74
    std::fill(extreme.begin(), extreme.end(), darker ? 3.40282347e+38f : -3.40282347e+38f);
    for (int i = 0; i < N; ++i) {
      for (int x = 0; x < W; ++x) {
        const uint8_t* in_pix = v.at(i, x, y);
        uint8_t* out_pix = row + (size_t)x * C;
        float value = 0.0f;
        for (int ch = 0; ch < C; ++ch) value += (float)in_pix[ch] * p->weights[ch];
        bool is_extreme = darker ? (value < extreme[x]) : (value > extreme[x]);
        if (is_extreme) {
          extreme[x] = value;
          float fade = lut[i];
          if (fade > 0.0f) {
            if (fade >= 1.0f) {
              for (int ch = 0; ch < C; ++ch) out_pix[ch] = in_pix[ch];
            } else {
              blend_into_u8(out_pix, in_pix, C, fade);
            }
          }
        }
      }
    }
  }
  return CP_OK;
}

}  // namespace

extern "C" {

// ---- scalar pieces, for known-answer tests ----------------------------------------------
// quartiles() on an already sorted slice, chrono.rs:559-565.
int or_quartiles(const uint8_t* sorted, int32_t len, float* q1, float* med, float* q3) {
  if (!sorted || len < 3) return CP_ERR_ARG;
  *q1 = quantile(sorted, (size_t)len, 0.25f);
  *med = median(sorted, (size_t)len);
  *q3 = quantile(sorted, (size_t)len, 0.75f);
  return CP_OK;
}
float or_median(const uint8_t* sorted, int32_t len) { return median(sorted, (size_t)len); }
float or_blend_value(int32_t abs, float mn, float mx, float dist) {
  return Threshold(abs != 0, mn, mx).blend_value(dist);
}
void or_threshold(int32_t abs, float mn, float mx, float* out3) {
  Threshold t(abs != 0, mn, mx);
  out3[0] = t.min;
  out3[1] = t.max;
  out3[2] = t.scale;
}
void or_blend_into_u8(uint8_t* a, const uint8_t* b, int32_t c, float blend) {
  blend_into_u8(a, b, c, blend);
}
uint32_t or_gen_range(uint64_t seed, uint64_t pixel, uint32_t n) { return gen_range(seed, pixel, n); }

int or_fade_lut(const cp_fade* f, int32_t n, int32_t frame_offset, float* out) {
  Fade fd;
  if (!Fade::build(f, &fd) || n < 0) return CP_ERR_ARG;
  for (int32_t i = 0; i < n; ++i) out[i] = fd.at(i, n, frame_offset);
  return CP_OK;
}

// ---- whole stacks ------------------------------------------------------------------------
// OutlierProcessor::process / SimpleProcessor::process for one output frame. Host memory.
// threads > 1 splits the rows over std::threads (the reference's own pixel loop is
// sequential, chrono.rs:169; its parallelism is over video windows, main.rs:254-261).
int or_composite(const cp_stack* st, const cp_params* p, uint8_t* out, uint8_t* blend_out,
                 const cp_debug* dbg, uint64_t* n_warnings, int32_t threads) {
  if (!valid_params(st, p) || !out) return CP_ERR_ARG;
  const int N = st->n;
  if (p->mode == CP_MODE_OUTLIER && !p->thr_abs) {
    int eff = (p->sample && p->n_sample > 0 && p->n_sample < N) ? p->n_sample : N;
    if (eff < 3) return CP_ERR_ARG;  // quantile() underflows below 3 samples
  }
  std::vector<float> lut((size_t)N);
  if (or_fade_lut(&p->fade, N, st->frame_offset, lut.data()) != CP_OK) return CP_ERR_ARG;
  const int H = st->height;
  if (threads < 1) threads = 1;
  if (threads > H) threads = H;
  std::vector<uint64_t> warn((size_t)threads, 0);
  auto work = [&](int t) {
    int y0 = (int)((int64_t)H * t / threads), y1 = (int)((int64_t)H * (t + 1) / threads);
    if (p->mode == CP_MODE_OUTLIER)
      outlier_rows(st, p, lut.data(), y0, y1, out, blend_out, dbg, &warn[(size_t)t]);
    else
      simple_rows(st, p, lut.data(), y0, y1, out);
  };
  if (threads == 1) {
    work(0);
  } else {
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) pool.emplace_back(work, t);
    for (auto& th : pool) th.join();
  }
  uint64_t total = 0;
  for (auto w : warn) total += w;
  if (n_warnings) *n_warnings = total;
  return CP_OK;
}

// ---- camera shake ------------------------------------------------------------------------
// ShakeAnalyzer::analyze, src/shake.rs:190-313, with fill_windows (:315-343) and calc_diffs
// (:345-385). Frames are full images (width x height x channels). Squared differences
// accumulate in wrapping i32 (release profile). diffs (nullable) receives the per-frame
// (2s+1)^2 sums for frames 1..n-1. Out-of-range coordinates (a panic in the reference)
// return CP_ERR_RANGE.
int or_shake_analyze(const uint8_t* const* frames, int32_t n, int32_t w, int32_t h, int32_t c,
                     const int32_t* anchors, int32_t n_anchors, int32_t r, int32_t s,
                     int32_t* offsets, int32_t* diffs, int32_t threads) {
  if (!frames || n < 1 || w < 1 || h < 1 || c < 1 || r < 0 || s < 0 || !offsets) return CP_ERR_ARG;
  const int32_t size = 2 * r + 1, ssize = 2 * s + 1;
  const int64_t win_len = (int64_t)size * size * c;
  // fill_windows: every window pixel must be inside frame 0 (layout.index(...).expect)
  std::vector<uint8_t> wins((size_t)(n_anchors * win_len));
  for (int a = 0; a < n_anchors; ++a) {
    int32_t cx = anchors[2 * a], cy = anchors[2 * a + 1];
    for (int dy = 0; dy < size; ++dy) {
      int32_t yy = cy + dy - r;
      for (int dx = 0; dx < size; ++dx) {
        int32_t xx = cx + dx - r;
        if (xx < 0 || yy < 0 || xx >= w || yy >= h) return CP_ERR_RANGE;
        for (int ch = 0; ch < c; ++ch)
          wins[(size_t)(a * win_len + ((int64_t)dy * size + dx) * c + ch)] =
              frames[0][((int64_t)yy * w + xx) * c + ch];
      }
    }
  }
  // calc_diffs range check, once: the search touches cx-s-r .. cx+s+r
  for (int a = 0; a < n_anchors; ++a) {
    int32_t cx = anchors[2 * a], cy = anchors[2 * a + 1];
    if (n > 1 && (cx - s - r < 0 || cy - s - r < 0 || cx + s + r >= w || cy + s + r >= h))
      return CP_ERR_RANGE;
  }
  offsets[0] = 0;
  offsets[1] = 0;
  if (threads < 1) threads = 1;
  auto frame_work = [&](int f, std::vector<uint32_t>& diff) {
    std::fill(diff.begin(), diff.end(), 0u);
    const uint8_t* img = frames[f];
    for (int a = 0; a < n_anchors; ++a) {
      int32_t cx = anchors[2 * a], cy = anchors[2 * a + 1];
      const uint8_t* win = &wins[(size_t)(a * win_len)];
      for (int oy = 0; oy < ssize; ++oy)
        for (int ox = 0; ox < ssize; ++ox) {
          uint32_t acc = diff[(size_t)(oy * ssize + ox)];
          for (int dy = 0; dy < size; ++dy) {
            int32_t yy = cy + (oy - s) + dy - r;
            for (int dx = 0; dx < size; ++dx) {
              int32_t xx = cx + (ox - s) + dx - r;
              const uint8_t* ip = img + ((int64_t)yy * w + xx) * c;
              const uint8_t* wp = win + ((int64_t)dy * size + dx) * c;
              for (int ch = 0; ch < c; ++ch) {
                int32_t d = (int32_t)wp[ch] - (int32_t)ip[ch];
                acc += (uint32_t)(d * d);  // wrapping i32 add
              }
            }
          }
          diff[(size_t)(oy * ssize + ox)] = acc;
        }
    }
    // min_by_key: first minimum of the i32 values (shake.rs:294-297)
    size_t best = 0;
    for (size_t k = 1; k < diff.size(); ++k)
      if ((int32_t)diff[k] < (int32_t)diff[best]) best = k;
    offsets[2 * f] = (int32_t)(best % (size_t)ssize) - s;
    offsets[2 * f + 1] = (int32_t)(best / (size_t)ssize) - s;
    if (diffs)
      for (size_t k = 0; k < diff.size(); ++k)
        diffs[(size_t)(f - 1) * diff.size() + k] = (int32_t)diff[k];
  };
  auto worker = [&](int t) {
    std::vector<uint32_t> diff((size_t)ssize * ssize);
    for (int f = 1 + t; f < n; f += threads) frame_work(f, diff);
  };
  if (threads == 1) {
    worker(0);
  } else {
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) pool.emplace_back(worker, t);
    for (auto& th : pool) th.join();
  }
  return CP_OK;
}

// Crop::create, src/shake.rs:136-176.
int or_crop_create(const int32_t* offsets, int32_t n, int32_t width, int32_t height,
                   int32_t* has_crop, int32_t* crops) {
  int32_t xmin = 0, ymin = 0, xmax = 0, ymax = 0;
  for (int i = 0; i < n; ++i) {
    int32_t x = offsets[2 * i], y = offsets[2 * i + 1];
    if (x < xmin) xmin = x;
    if (y < ymin) ymin = y;
    if (x > xmax) xmax = x;
    if (y > ymax) ymax = y;
  }
  if (xmin == 0 && ymin == 0 && xmax == 0 && ymax == 0) {
    *has_crop = 0;
    return CP_OK;
  }
  *has_crop = 1;
  int32_t w = width + xmin - xmax, h = height + ymin - ymax;
  for (int i = 0; i < n; ++i) {
    crops[4 * i] = -xmin + offsets[2 * i];
    crops[4 * i + 1] = -ymin + offsets[2 * i + 1];
    crops[4 * i + 2] = w;
    crops[4 * i + 3] = h;
  }
  return CP_OK;
}

// Window enumeration of create_video, src/main.rs:230-286 (the same arithmetic is in
// create_video_simple, :351-403). Ranges follow FrameRange (src/flist.rs:11-45).
int or_video_windows(int32_t image_count, int32_t in_has_start, int32_t in_start,
                     int32_t in_has_end, int32_t in_end, int32_t in_step, int32_t out_has_start,
                     int32_t out_start, int32_t out_has_end, int32_t out_end, int32_t out_step,
                     int32_t* n_windows, int64_t* n_indices, int64_t* win_start, int32_t* win_len,
                     int32_t* win_indices, int32_t* win_frame) {
  if (in_step <= 0 || out_step <= 0) return CP_ERR_ARG;  // division by zero panics
  int32_t v_lower;
  if (out_has_start)
    v_lower = out_start;
  else if (in_has_start && in_has_end)
    v_lower = -(in_end - in_start) + 1;
  else
    v_lower = 0;
  int32_t v_upper = out_has_end ? out_end : image_count;
  int32_t count = (v_upper - v_lower) / out_step;
  if (count < 0) count = 0;
  int64_t total = 0;
  for (int32_t k = 0; k < count; ++k) {
    int32_t frame = k * out_step + v_lower;
    int32_t start = 0;
    if (in_has_start) {
      int32_t st = frame + in_start;
      while (st < 0) st += in_step;
      start = std::max(st % in_step, frame + in_start);
    }
    int32_t end = image_count;
    if (in_has_end) end = std::min(image_count + (frame + in_end) % in_step - in_step, frame + in_end);
    int32_t len = 0;
    for (int32_t f = start; f < end; f += in_step) {
      if (win_indices) win_indices[total + len] = f;
      len += 1;
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

}  // extern "C"
