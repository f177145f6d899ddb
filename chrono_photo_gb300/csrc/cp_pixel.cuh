// cp_pixel.cuh — the per-pixel half of outlier compositing with one thread per pixel: the
// pixel's statistics from its channels' order statistics, the distance pass over its samples
// (src/chrono.rs:257-288) and the epilogue (background, outlier pick and blend, blend mask,
// src/chrono.rs:290-493). Shared by the pixel-thread single-stack kernel (cp_outlier_px.cuh)
// and the sliding-window kernel (cp_video.cu). `load(i)` returns sample i of the pixel as a
// word with its channel bytes in bytes 0..C-1; the bytes above may hold anything (the
// distance arithmetic masks them, the epilogue masks its loads).
//
// The arithmetic is the tile kernel's (cp_tile.cuh), in the reference's f32 operation order
// with explicit _rn intrinsics.

#pragma once
#include "cp_tile.cuh"

namespace cp {
namespace {

template <int C>
struct PxStat {
  uint32_t klo, khi;  // floor / ceil of the medians, channel bytes (integer distances)
  int nh;             // channels with a half-integer median
  float med[C];       // median() per channel, 0 for weight-0 channels (src/chrono.rs:238-255)
  float medo[C];      // med + 2^22 (exact)
  float wi[C];        // w * iqr_inv (rel thresholds) or w (abs)
};

// lo3 / hi3: d[k] and d[k+1] (or d[k] again without a pair) of the median per channel byte;
// wq: w * iqr_inv per channel for rel thresholds (ignored for abs).
template <int C>
DEVI PxStat<C> px_stat(const StackDev& S, uint32_t lo3, uint32_t hi3, const float (&wq)[C]) {
  PxStat<C> r;
  r.klo = r.khi = 0u;
  r.nh = 0;
#pragma unroll
  for (int ch = 0; ch < C; ++ch) {
    const uint32_t lo = (lo3 >> (8 * ch)) & 0xFFu, hi = (hi3 >> (8 * ch)) & 0xFFu;
    const bool wt = (S.wmask >> ch) & 1u;
    r.med[ch] = !wt ? 0.0f
                    : (S.med_pair ? __fmul_rn(0.5f, __fadd_rn(static_cast<float>(lo),
                                                              static_cast<float>(hi)))
                                  : static_cast<float>(lo));
    r.medo[ch] = __fadd_rn(r.med[ch], 4194304.0f);
    r.wi[ch] = S.thr_abs ? S.w[ch] : wq[ch];
    const uint32_t s2 = lo + hi;
    const uint32_t fl = S.med_pair ? (s2 >> 1) : lo, ce = S.med_pair ? ((s2 + 1) >> 1) : lo;
    if (wt) {
      r.klo |= fl << (8 * ch);
      r.khi |= ce << (8 * ch);
      r.nh += static_cast<int>(ce - fl);
    }
  }
  return r;
}

// Bit planes of one pixel's samples: P[ch][r][blk] bit i = bit r of channel byte ch of sample
// 32*blk + i (8x8 bit transposes of 8 samples, then a 4x4 byte transpose of 4 groups).
// Every sample 0..32*NW-1 is loaded: the stage rows past the stack's n are zero (the sample
// mask keeps them out of the selections), so the loads need no bound test.
template <int C, int NW, typename Load>
DEVI void pixel_planes(Load load, uint32_t (&P)[C][8][NW]) {
  if constexpr (C == 3) {
    // RGB: the 12 channel bytes of 4 groups' words r are first packed into 3 words (byte
    // lanes (g0c0 g0c1 g0c2 g1c0), (g1c1 g1c2 g2c0 g2c1), (g2c2 g3c0 g3c1 g3c2)), so 3 bit
    // transposes do the work of 4 with no lane spent on the unused fourth byte
#pragma unroll
    for (int blk = 0; blk < NW; ++blk) {
      uint32_t x[3][8];
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const uint32_t a0 = load(blk * 32 + r), a1 = load(blk * 32 + 8 + r);
        const uint32_t a2 = load(blk * 32 + 16 + r), a3 = load(blk * 32 + 24 + r);
        x[0][r] = __byte_perm(a0, a1, 0x4210);
        x[1][r] = __byte_perm(a1, a2, 0x5421);
        x[2][r] = __byte_perm(a2, a3, 0x6542);
      }
      transpose8(x[0]);
      transpose8(x[1]);
      transpose8(x[2]);
#pragma unroll
      for (int r = 0; r < 8; ++r) {  // plane word: groups 0..3 of the channel in bytes 0..3
        P[0][r][blk] = __byte_perm(__byte_perm(x[0][r], x[1][r], 0x0630), x[2][r], 0x5210);
        P[1 % C][r][blk] = __byte_perm(__byte_perm(x[0][r], x[1][r], 0x0741), x[2][r], 0x6210);
        P[2 % C][r][blk] = __byte_perm(__byte_perm(x[0][r], x[1][r], 0x0052), x[2][r], 0x7410);
      }
    }
    return;
  }
#pragma unroll
  for (int blk = 0; blk < NW; ++blk) {
    uint32_t a[4][8];
#pragma unroll
    for (int g = 0; g < 4; ++g) {
#pragma unroll
      for (int r = 0; r < 8; ++r) a[g][r] = load(blk * 32 + g * 8 + r);
      transpose8(a[g]);
    }
#pragma unroll
    for (int r = 0; r < 8; ++r) {  // 4x4 byte transpose: group g -> byte g
      const uint32_t t0 = __byte_perm(a[0][r], a[1][r], 0x5140);
      const uint32_t t1 = __byte_perm(a[0][r], a[1][r], 0x7362);
      const uint32_t t2 = __byte_perm(a[2][r], a[3][r], 0x5140);
      const uint32_t t3 = __byte_perm(a[2][r], a[3][r], 0x7362);
      if (C > 0) P[0][r][blk] = __byte_perm(t0, t2, 0x5410);
      if (C > 1) P[1 % C][r][blk] = __byte_perm(t0, t2, 0x7632);
      if (C > 2) P[2 % C][r][blk] = __byte_perm(t1, t3, 0x5410);
      if (C > 3) P[3 % C][r][blk] = __byte_perm(t1, t3, 0x7632);
    }
  }
}

// The median pair and, with QUART, the quartile pairs of one pixel through ONE copy of the
// selection code: a runtime loop over the needed ranks (med_k, med_k + 1 if paired, q1_k,
// q1_k + 1, q3_k, q3_k + 1 if paired) instead of one inlined selection per rank (six for rel
// thresholds, each some 300 instructions: their code footprint stalled instruction fetch).
// Results are packed per rank (channel byte ch at bits 8ch) and kept in named registers
// through uniform selects, so no array is indexed at run time.
// quart: the quartiles are wanted (QUART compiles them in).
template <int C, int NW, bool QUART>
DEVI void pixel_ranks(const StackDev& S, const uint32_t (&P)[C][8][NW],
                      const uint32_t (&smask)[NW], bool quart, uint32_t& lo3, uint32_t& hi3,
                      uint32_t& q1a, uint32_t& q1b, uint32_t& q3a, uint32_t& q3b) {
  lo3 = hi3 = q1a = q1b = q3a = q3b = 0u;
  const int nrank = QUART && quart ? 6 : 2;
#pragma unroll 1
  for (int j = 0; j < nrank; ++j) {
    const bool need = j == 0 || (j == 1 && S.med_pair) || j == 2 || (j == 3 && S.q1_pair) ||
                      j == 4 || (j == 5 && S.q3_pair);
    if (!need) continue;
    const int k = j < 2 ? S.med_k + j : (j < 4 ? S.q1_k + j - 2 : S.q3_k + j - 4);
    uint32_t v[C];
    select_rank<NW, C>(P, smask, k, v);
    uint32_t packed = 0u;
#pragma unroll
    for (int ch = 0; ch < C; ++ch) packed |= v[ch] << (8 * ch);
    lo3 = j == 0 ? packed : lo3;
    hi3 = j == 1 ? packed : hi3;
    q1a = j == 2 ? packed : q1a;
    q1b = j == 3 ? packed : q1b;
    q3a = j == 4 ? packed : q3a;
    q3b = j == 5 ? packed : q3b;
  }
  if (!S.med_pair) hi3 = lo3;
}

// 1 / iqr per channel from the packed quartile order statistics (src/chrono.rs:246-252, iqr 0
// counts as 1); q1v / q3v the quartiles.
template <int C>
DEVI void quartiles_from_ranks(const StackDev& S, uint32_t q1a, uint32_t q1b, uint32_t q3a,
                               uint32_t q3b, float (&q1v)[C], float (&q3v)[C],
                               float (&iqr_inv)[C]) {
#pragma unroll
  for (int ch = 0; ch < C; ++ch) {
    const uint32_t a1 = (q1a >> (8 * ch)) & 0xFFu, b1 = (q1b >> (8 * ch)) & 0xFFu;
    const uint32_t a3 = (q3a >> (8 * ch)) & 0xFFu, b3 = (q3b >> (8 * ch)) & 0xFFu;
    const float q1 = quantile_value(a1, S.q1_pair ? b1 : a1, S.q1_pair != 0, S.q1_frac);
    const float q3 = quantile_value(a3, S.q3_pair ? b3 : a3, S.q3_pair != 0, S.q3_frac);
    float iqr = __fsub_rn(q3, q1);
    if (iqr == 0.0f) iqr = 1.0f;
    iqr_inv[ch] = __fdiv_rn(1.0f, iqr);
    q1v[ch] = q1;
    q3v[ch] = q3;
  }
}

// Order statistics of one pixel from its own samples: bit planes, radix selections of the
// median pair and, for rel thresholds, the quartiles (src/chrono.rs:220-255). lo3 / hi3 as
// for px_stat; wq = w * iqr_inv; q1v / q3v the quartiles (debug outputs).
template <int C, int NW, int KIND, typename Load>
DEVI void pixel_order_stats(const StackDev& S, Load load, uint32_t& lo3, uint32_t& hi3,
                            float (&wq)[C], float (&q1v)[C], float (&q3v)[C]) {
  uint32_t P[C][8][NW];
  pixel_planes<C, NW>(load, P);
  uint32_t smask[NW];
#pragma unroll
  for (int w = 0; w < NW; ++w) smask[w] = S.sample_mask[w];
  const bool quart = KIND != kIntKind && !S.thr_abs;
  uint32_t q1a, q1b, q3a, q3b;
  pixel_ranks<C, NW, KIND != kIntKind>(S, P, smask, quart, lo3, hi3, q1a, q1b, q3a, q3b);
#pragma unroll
  for (int ch = 0; ch < C; ++ch) {
    wq[ch] = 0.0f;
    q1v[ch] = 0.0f;
    q3v[ch] = 0.0f;
  }
  if (quart) {  // quartiles and w * iqr_inv, src/chrono.rs:246-252
    float iqr_inv[C], q1[C], q3[C];
    quartiles_from_ranks<C>(S, q1a, q1b, q3a, q3b, q1, q3, iqr_inv);
#pragma unroll
    for (int ch = 0; ch < C; ++ch) {
      wq[ch] = __fmul_rn(S.w[ch], iqr_inv[ch]);
      const bool wt = (S.wmask >> ch) & 1u;
      q1v[ch] = wt ? q1[ch] : 0.0f;
      q3v[ch] = wt ? q3[ch] : 0.0f;
    }
  }
}

// Largest-distance bookkeeping is compiled in for the outlier groups that pick `extreme`.
template <int OG>
constexpr bool kKeepMax = OG == kOgAny || OG == kOgSingle;

// Distance pass over samples 0..n-1 (src/chrono.rs:257-288): outlier flags pb (bit i of word
// i/32), and for `extreme` the largest distance, earliest sample first: integer kind as the
// key (D' << 8) + 255 - i, f32 kinds as (dmax, imax).
// CH: samples per straight-line chunk of the integer pass (8 keeps the code small for the
// kernels that walk many code paths per tile; the sliding-window kernel takes whole words).
template <int C, int NW, int KIND, int OG, typename Load, int CH = 8>
DEVI void px_distance(const StackDev& S, int n, const PxStat<C>& st, uint32_t wbytes, Load load,
                      uint32_t (&pb)[NW], int32_t& key, float& dmax, int& imax) {
  key = st.nh > 0 ? -1 : 255;
  dmax = 0.0f;
  imax = 0;
#pragma unroll
  for (int w = 0; w < NW; ++w) pb[w] = 0u;
  // Each 32-sample word runs in straight-line chunks of 8 samples (immediate shared-memory
  // offsets, no per-sample bound test), then a loop over the samples left. The word loop is
  // not unrolled (one copy of the chunk): its flag word reaches pb[w] through uniform selects.
  if (KIND == kIntKind || ((KIND == kAnyKind || KIND == kPxKind) && S.fast_int)) {
    const int32_t thr1 = S.thr_int[st.nh] - 1;
    // thr1 - d = (thr1 - klo.khi) + v.klo + v.khi - v.v, accumulated by the dp4a chain
    const uint32_t base = static_cast<uint32_t>(thr1) - __dp4a(st.klo, st.khi, 0u);
    // flags enter at bit 0 and move up (a funnel shift takes the sign of thr - 1 - d: set
    // iff d >= thr); one bit reversal per word puts sample i at bit i
    uint32_t ob;
    // extreme: the smallest (thr - 1 - d) * 256 + i is the largest d, earliest sample first
    // (i < 256); every D' >= 0 (no integer lies strictly between the floor and ceiling of a
    // median), so over n >= 1 samples this gives the key's maximum. With any outlier,
    // thr <= 3 * 255^2 and |thr - 1 - d| < 2^19, so the product is exact; with none (a
    // threshold beyond every distance) it may wrap, and only its index bits, a valid sample,
    // are read
    int32_t tmin = 0x7FFFFFFF;
    auto sample = [&](int i) {
      const uint32_t v = load(i) & wbytes;
      const uint32_t t = __dp4a(v, st.khi, __dp4a(v, st.klo, base)) - __dp4a(v, v, 0u);
      ob = __funnelshift_l(t, ob, 1);
      if (kKeepMax<OG>) tmin = min(tmin, static_cast<int32_t>((t << 8) + static_cast<uint32_t>(i)));
    };
#pragma unroll 1
    for (int blk = 0; blk < NW; ++blk) {
      const int i0 = blk * 32, iend = min(n, i0 + 32);
      ob = 0u;
      int i = i0;
#pragma unroll 1
      for (; i + CH <= iend; i += CH) {
#pragma unroll
        for (int j = 0; j < CH; ++j) sample(i + j);
      }
#pragma unroll 1
      for (; i < iend; ++i) sample(i);
      const uint32_t word = iend > i0 ? __brev(ob) >> (32 - (iend - i0)) : 0u;
#pragma unroll
      for (int w = 0; w < NW; ++w) pb[w] = w == blk ? word : pb[w];
    }
    if (kKeepMax<OG>) key = ((thr1 - (tmin >> 8)) << 8) + 255 - (tmin & 255);
  } else if (KIND == kF32Kind || KIND == kPxKind || (KIND == kAnyKind && S.pair_f32)) {
    // two samples per instruction in float2 lanes, every term on (median - p) / 2: the
    // sample -(2^14 + p/2) is one byte permute of the pixel byte into -2^14's mantissa, the
    // median 2^14 + median/2 is exact, so terms, sums and the threshold are the reference's
    // values times exactly 1/4 (ranges checked on the host). Products are summed with scalar
    // adds: a paired add after a paired multiply was contracted into a fused multiply-add.
    float2 mq[C], wq2[C];
#pragma unroll
    for (int ch = 0; ch < C; ++ch) {
      const float m = __fadd_rn(__fmul_rn(__fsub_rn(st.medo[ch], 4194304.0f), 0.5f), 16384.0f);
      mq[ch] = make_float2(m, m);
      wq2[ch] = make_float2(st.wi[ch], st.wi[ch]);
    }
    const float thr4 = __fmul_rn(S.thr_sq, 0.25f);
    // every channel of two samples; a weight-0 channel adds +0 (w * iqr_inv = 0 and the
    // median term finite), which leaves the non-negative sum unchanged
    auto pair_dist = [&](uint32_t p0, uint32_t p1) -> float2 {
      float2 dq = make_float2(0.0f, 0.0f);
#pragma unroll
      for (int ch = 0; ch < C; ++ch) {
        const uint32_t sel = 0x7604u | (static_cast<uint32_t>(ch) << 4);
        const float2 nv = make_float2(__uint_as_float(__byte_perm(p0, 0xC6800000u, sel)),
                                      __uint_as_float(__byte_perm(p1, 0xC6800000u, sel)));
        const float2 tt = mul2_rn(wq2[ch], add2_rn(mq[ch], nv));
        const float2 sq = mul2_rn(tt, tt);
        dq.x = __fadd_rn(dq.x, sq.x);
        dq.y = __fadd_rn(dq.y, sq.y);
      }
      return dq;
    };
    // the sign of dq - thr4 is 0 exactly when dq >= thr4 (equal: +0; both finite and
    // non-negative): sign bits of the non-outliers enter at bit 0 and move up
    uint32_t nb;
    // extreme: the largest distance of all samples, earliest first. With an outlier it is an
    // outlier's (the largest is >= every outlier's >= thr4); without one it is not used.
    auto one = [&](float dq, int i) {
      nb = __funnelshift_l(__float_as_uint(__fsub_rn(dq, thr4)), nb, 1);
      if (kKeepMax<OG>) {
        const bool up = dq > dmax;
        dmax = up ? dq : dmax;
        imax = up ? i : imax;
      }
    };
#pragma unroll 1
    for (int blk = 0; blk < NW; ++blk) {
      const int i0 = blk * 32, iend = min(n, i0 + 32);
      nb = 0u;
      int i = i0;
#pragma unroll 1
      for (; i + 8 <= iend; i += 8) {
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
          const float2 dq = pair_dist(load(i + j), load(i + j + 1));
          one(dq.x, i + j);
          one(dq.y, i + j + 1);
        }
      }
#pragma unroll 1
      for (; i < iend; ++i) {
        const uint32_t p = load(i);
        one(pair_dist(p, p).x, i);
      }
      const uint32_t word = iend > i0 ? __brev(~nb) >> (32 - (iend - i0)) : 0u;
#pragma unroll
      for (int w = 0; w < NW; ++w) pb[w] = w == blk ? word : pb[w];
    }
    dmax = __fmul_rn(dmax, 4.0f);  // scaled back exactly
  } else {
#pragma unroll
    for (int blk = 0; blk < NW; ++blk) {
      uint32_t ob = 0u;
      const int iend = min(n, blk * 32 + 32);
      for (int i = blk * 32; i < iend; ++i) {
        const uint32_t px = load(i);
        const float d = S.finite_w ? dist_f32<C, true>(S, st.medo, st.wi, px)
                                   : dist_f32<C, false>(S, st.medo, st.wi, px);
        const bool o = d >= S.thr_sq;
        ob |= o ? (1u << (i & 31)) : 0u;
        if (kKeepMax<OG>) {
          const bool up = o && d > dmax;
          dmax = up ? d : dmax;
          imax = up ? i : imax;
        }
      }
      pb[blk] = ob;
    }
  }
}

// SimpleProcessor's fold for one pixel (src/simple.rs:96-133), over samples 0..n-1: running
// extreme of sum_c p_c * w_c (f32, c ascending, strict compare: the earliest sample wins
// ties); on a new extreme the sample is blended into the running output (starting at 0) with
// its fade. With 0/1 weights and every fade factor >= 1 the sums are exact integers (dp4a)
// and a new extreme copies the sample.
template <int C, typename Load>
DEVI uint32_t px_simple(const StackDev& S, int n, Load load) {
  const bool darker = S.mode == CP_MODE_DARKER;
  uint32_t outw = 0u;
  if (S.unit_w && S.no_fade) {
    uint32_t ones = 0u;
#pragma unroll
    for (int ch = 0; ch < C; ++ch)
      if ((S.wmask >> ch) & 1u) ones |= 1u << (8 * ch);
    // key v * 128 + i (darker: smallest) or v * 128 + 127 - i (lighter: largest) of the
    // channel sum v <= 1020 and sample i < 128: the extreme, earliest sample first; the
    // winning sample is loaded once at the end
    int idx;
    if (darker) {
      int32_t key = 0x7FFFFFFF;
      for (int i = 0; i < n; ++i)
        key = min(key, static_cast<int32_t>(__dp4a(load(i), ones, 0u)) * 128 + i);
      idx = key & 127;
    } else {
      int32_t key = -1;
      for (int i = 0; i < n; ++i)
        key = max(key, static_cast<int32_t>(__dp4a(load(i), ones, 0u)) * 128 + 127 - i);
      idx = 127 - (key & 127);
    }
    return load(idx) & (0xFFFFFFFFu >> (32 - 8 * C));
  }
  float ext = darker ? FLT_MAX : -FLT_MAX;
  for (int i = 0; i < n; ++i) {
    const uint32_t px = load(i) & (0xFFFFFFFFu >> (32 - 8 * C));
    float value = 0.0f;
#pragma unroll
    for (int ch = 0; ch < C; ++ch)
      value = __fadd_rn(value, __fmul_rn(u8f((px >> (8 * ch)) & 0xFFu), S.w[ch]));
    const bool up = darker ? (value < ext) : (value > ext);
    ext = up ? value : ext;
    const float fade = S.fade[i];
    if (up && fade > 0.0f) outw = fade >= 1.0f ? px : blend_into_u8<C>(outw, px, fade);
  }
  return outw;
}

// Darker and lighter of the same weights, both in the integer form (0/1 weights, every fade
// factor >= 1), in one pass: each sample is loaded and summed once for both extremes.
template <int C, typename Load>
DEVI void px_simple_pair(const StackDev& S, int n, Load load, uint32_t& dark, uint32_t& light) {
  uint32_t ones = 0u;
#pragma unroll
  for (int ch = 0; ch < C; ++ch)
    if ((S.wmask >> ch) & 1u) ones |= 1u << (8 * ch);
  // keys as in px_simple: the smallest v * 128 + i is the darkest sample and the largest
  // v * 128 + 127 - i the lightest, earliest first (dp4a with `ones` ignores bytes >= C)
  int32_t kd = 0x7FFFFFFF, kl = -1;
  for (int i = 0; i < n; ++i) {
    const int32_t v = static_cast<int32_t>(__dp4a(load(i), ones, 0u));
    kd = min(kd, v * 128 + i);
    kl = max(kl, v * 128 + 127 - i);
  }
  dark = load(kd & 127) & (0xFFFFFFFFu >> (32 - 8 * C));
  light = load(127 - (kl & 127)) & (0xFFFFFFFFu >> (32 - 8 * C));
}

struct PxOut {
  uint32_t pix;   // composite, channel bytes
  uint32_t mask;  // blend mask value of channels 0..2
  int chosen;     // debug: sample blended in (-1 none, -2 several), or 0 for an averaged pick
  int bg_idx;     // debug: background sample (first / random), else -1
  int nout;
  bool warning;   // every sample an outlier under a first / random background
};

// The epilogue of one pixel (src/chrono.rs:290-493). sums: the channel sums over all n
// samples for the average background (computed here when null).
template <int C, int NW, int KIND, int OG, int BG, typename Load>
DEVI PxOut px_epilogue(const StackDev& S, int n, const PxStat<C>& st, uint32_t wbytes,
                       const uint32_t (&pb)[NW], int32_t key, float dmax_f, int imax_f,
                       int pix_idx, const uint32_t* sums, Load load_raw) {
  PxOut r;
  auto load = [&](int i) -> uint32_t { return load_raw(i) & (0xFFFFFFFFu >> (32 - 8 * C)); };
  const bool fast = KIND == kIntKind || ((KIND == kAnyKind || KIND == kPxKind) && S.fast_int);
  // fade factor of sample i; without a fade every factor is 1 (and x * 1 = x exactly), so
  // the per-lane lookups (a different sample in each lane) are skipped
  auto fade_at = [&](int i) -> float {
    float f = 1.0f;
    if (!S.unit_fade) f = S.fade[i];
    return f;
  };
  auto dsq_px = [&](uint32_t px) -> float {  // dist_sq of a sample, recomputed
    if (fast)
      return static_cast<float>(dist_int(px, wbytes, st.klo, st.khi)) +
             0.25f * static_cast<float>(st.nh);
    // paired-f32 stacks have finite, non-negative weights (host-checked)
    if constexpr (KIND == kF32Kind || KIND == kPxKind)
      return dist_f32<C, true, false>(S, st.medo, st.wi, px);
    return S.finite_w ? dist_f32<C, true>(S, st.medo, st.wi, px)
                      : dist_f32<C, false>(S, st.medo, st.wi, px);
  };
  int nout = 0;
#pragma unroll
  for (int w = 0; w < NW; ++w) nout += __popc(pb[w]);
  const int bgm = BG == kBgFirst ? CP_BG_FIRST : S.background;
  bool warning = false;
  int bg_idx = -1;
  uint32_t pix = 0;
  // background, src/chrono.rs:293-375
  if (bgm == CP_BG_FIRST || bgm == CP_BG_RANDOM) {
    if (bgm == CP_BG_FIRST) {
      if (nout == 0) {
        bg_idx = 0;
      } else if (nout == n) {
        bg_idx = 0;
        warning = true;
      } else {
        uint32_t inv[NW];
#pragma unroll
        for (int w = 0; w < NW; ++w) inv[w] = ~pb[w];
        bg_idx = first_set<NW>(inv);  // first_excluded, src/chrono.rs:504-530
      }
    } else {
      const uint64_t pid = static_cast<uint64_t>(pix_idx);
      if (nout == 0 || nout == n) {
        bg_idx = static_cast<int>(gen_range(S.seed, pid, static_cast<uint32_t>(n)));
        warning = nout == n;
      } else {
        // sample_excluded, src/chrono.rs:531-555: the j-th outlier (ascending) was swapped
        // with position n-1-j; trace the drawn position back through the swaps.
        int pos = static_cast<int>(gen_range(S.seed, pid, static_cast<uint32_t>(n - nout)));
        int j = nout - 1;
#pragma unroll
        for (int w = NW - 1; w >= 0; --w) {
          uint32_t m = pb[w];
          while (m) {
            const int bpos = 31 - __clz(m);
            m &= ~(1u << bpos);
            const int a = 32 * w + bpos, b = n - 1 - j;
            if (pos == a)
              pos = b;
            else if (pos == b)
              pos = a;
            --j;
          }
        }
        bg_idx = pos;
      }
    }
    pix = load(bg_idx);
  } else if (bgm == CP_BG_AVERAGE) {
    uint32_t sum[C];
    if (sums) {
#pragma unroll
      for (int ch = 0; ch < C; ++ch) sum[ch] = sums[ch];
    } else {
#pragma unroll
      for (int ch = 0; ch < C; ++ch) sum[ch] = 0u;
      for (int i = 0; i < n; ++i) {
        const uint32_t px = load(i);
#pragma unroll
        for (int ch = 0; ch < C; ++ch) sum[ch] += (px >> (8 * ch)) & 0xFFu;
      }
    }
    const float nf = static_cast<float>(n);
    if (nout == 0) {
#pragma unroll
      for (int ch = 0; ch < C; ++ch)
        pix |= sat_u8(rround(__fdiv_rn(static_cast<float>(sum[ch]), nf))) << (8 * ch);
    } else {
      uint32_t osum[C];
#pragma unroll
      for (int ch = 0; ch < C; ++ch) osum[ch] = 0u;
#pragma unroll
      for (int w = 0; w < NW; ++w) {
        uint32_t m = pb[w];
        while (m) {
          const int bpos = __ffs(m) - 1;
          m &= m - 1;
          const uint32_t px = load(32 * w + bpos);
#pragma unroll
          for (int ch = 0; ch < C; ++ch) osum[ch] += (px >> (8 * ch)) & 0xFFu;
        }
      }
      // src/chrono.rs:307-333 (the reference's own formula, incl. k = n -> inf)
      const float ratio = __fdiv_rn(nf, static_cast<float>(n - nout));
#pragma unroll
      for (int ch = 0; ch < C; ++ch) {
        const float mean = __fdiv_rn(static_cast<float>(sum[ch]), nf);
        const float v = __fsub_rn(__fmul_rn(mean, ratio),
                                  __fdiv_rn(static_cast<float>(osum[ch]), nf));
        pix |= sat_u8(rround(v)) << (8 * ch);
      }
    }
  } else {  // median (outliers included), src/chrono.rs:340-345
#pragma unroll
    for (int ch = 0; ch < C; ++ch) pix |= sat_u8(rround(st.med[ch])) << (8 * ch);
  }

  // outlier pick and blend, src/chrono.rs:377-493
  float blend = 0.0f;
  int chosen = -1;
  uint32_t mask = 0;
  const bool single_group = og_is<OG>(S, kOgSingle);
  const bool blend_group = og_is<OG>(S, kOgBlend);
  const bool extreme = single_group && S.outlier == CP_OUTLIER_EXTREME;
  // the average group takes every outlier count through the averaging branch: with one
  // outlier its sums are that sample's bytes and its distance (divided by 1, exact), and the
  // fade is taken at that sample, as the single-sample branch does; one branch instead of
  // two for warps that mix single- and multi-outlier pixels
  const bool avg_group = og_is<OG>(S, kOgAverage);
  const bool multi = !single_group && (nout > 1 || avg_group);
  if (!multi) {
    int si;
    float dsq = 0.0f;
    if (extreme) {
      if (fast) {
        si = key < 0 ? 0 : 255 - (key & 255);
        const int32_t dm = key < 0 ? -1 : (key >> 8);
        dsq = dm < 0 ? 0.0f : static_cast<float>(dm) + 0.25f * static_cast<float>(st.nh);
      } else {
        si = imax_f;
        dsq = dmax_f;
      }
    } else {
      // the multi-outlier groups come here with at most one outlier: first == last
      si = (single_group && S.outlier == CP_OUTLIER_LAST) ? last_set<NW>(pb) : first_set<NW>(pb);
      si = si < 0 ? 0 : si;
    }
    const uint32_t sample = load(si);
    if (!extreme) dsq = dsq_px(sample);
    blend = nout == 0 ? 0.0f : __fmul_rn(fade_at(si), blend_value(S, __fsqrt_rn(dsq)));
    pix = blend_into_u8<C>(pix, sample, blend);
    mask = sat_u8(rround(__fmul_rn(blend, 255.0f)));
    chosen = nout == 0 ? -1 : si;
  } else if (blend_group) {
    float pf[C];
#pragma unroll
    for (int ch = 0; ch < C; ++ch) pf[ch] = static_cast<float>((pix >> (8 * ch)) & 0xFFu);
    float binv = 1.0f;
    auto blend_one = [&](int f) {
      const uint32_t sv = load(f);
      const float bk = __fmul_rn(fade_at(f), blend_value(S, __fsqrt_rn(dsq_px(sv))));
      // blend_into_f32_u8, src/color.rs:32-44
      if (bk <= 0.0f) {
      } else if (bk >= 1.0f) {
#pragma unroll
        for (int ch = 0; ch < C; ++ch) pf[ch] = static_cast<float>((sv >> (8 * ch)) & 0xFFu);
      } else {
#pragma unroll
        for (int ch = 0; ch < C; ++ch) {
          const float x = static_cast<float>((sv >> (8 * ch)) & 0xFFu);
          pf[ch] = __fadd_rn(pf[ch], __fmul_rn(__fsub_rn(x, pf[ch]), bk));
        }
      }
      binv = __fmul_rn(binv, __fsub_rn(1.0f, bk));
    };
    // outliers in ascending (forward) or descending (backward) sample order
    if constexpr (OG == kOgAny) {
      // the generic epilogue (multi-setting kernel): one loop with one copy of blend_one,
      // each turn taking the lowest (highest) remaining flag; a smaller instruction footprint
      // for a kernel that walks every setting kind per tile
      const bool fwd = S.outlier == CP_OUTLIER_FORWARD;
      uint32_t m[NW];
#pragma unroll
      for (int w = 0; w < NW; ++w) m[w] = pb[w];
#pragma unroll 1
      for (int t = 0; t < nout; ++t) {
        int f = 0;
        if (fwd) {
#pragma unroll
          for (int w = NW - 1; w >= 0; --w)
            if (m[w]) f = 32 * w + __ffs(m[w]) - 1;
        } else {
#pragma unroll
          for (int w = 0; w < NW; ++w)
            if (m[w]) f = 32 * w + 31 - __clz(m[w]);
        }
#pragma unroll
        for (int w = 0; w < NW; ++w)
          if (w == (f >> 5)) m[w] &= ~(1u << (f & 31));
        blend_one(f);
      }
    } else if (S.outlier == CP_OUTLIER_FORWARD) {
#pragma unroll
      for (int w = 0; w < NW; ++w) {
        uint32_t m = pb[w];
        while (m) {
          const int f = 32 * w + __ffs(m) - 1;
          m &= m - 1;
          blend_one(f);
        }
      }
    } else {
#pragma unroll
      for (int w = NW - 1; w >= 0; --w) {
        uint32_t m = pb[w];
        while (m) {
          const int bpos = 31 - __clz(m);
          m &= ~(1u << bpos);
          blend_one(32 * w + bpos);
        }
      }
    }
    pix = 0;
#pragma unroll
    for (int ch = 0; ch < C; ++ch) pix |= sat_u8(rround(pf[ch])) << (8 * ch);
    mask = sat_u8(rround(__fmul_rn(__fsub_rn(1.0f, binv), 255.0f)));
    chosen = -2;
  } else {  // average of the outliers, src/chrono.rs:429-468 (one or none: :377-428)
    // channel sums in 16-bit lanes (n * 255 < 2^16): even bytes, odd bytes
    const int si = first_set<NW>(pb);  // the outlier, when there is one
    uint32_t se = 0u, so = 0u;
    float mdist = 0.0f;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      uint32_t m = pb[w];
      while (m) {
        const int f = 32 * w + __ffs(m) - 1;
        m &= m - 1;
        const uint32_t px = load(f);
        se += px & 0x00FF00FFu;
        so += (px >> 8) & 0x00FF00FFu;
        mdist = __fadd_rn(mdist, __fsqrt_rn(dsq_px(px)));
      }
    }
    const float kf = static_cast<float>(nout);
    uint32_t sample = 0;
#pragma unroll
    for (int ch = 0; ch < C; ++ch) {
      const uint32_t os = ((ch & 1) ? so : se) >> (16 * (ch >> 1)) & 0xFFFFu;
      sample |= sat_u8(rround(__fdiv_rn(static_cast<float>(os), kf))) << (8 * ch);
    }
    // the fade of an averaged outlier is taken at sample 0 (src/chrono.rs:467), that of a
    // single one at its own sample; no outlier: no blend (the sums divided by 0 are unused)
    const float bk =
        __fmul_rn(fade_at(nout == 1 ? si : 0), blend_value(S, __fdiv_rn(mdist, kf)));
    blend = nout == 0 ? 0.0f : bk;
    pix = blend_into_u8<C>(pix, sample, blend);
    mask = sat_u8(rround(__fmul_rn(blend, 255.0f)));
    chosen = nout == 0 ? -1 : (nout == 1 ? si : 0);
  }
  r.pix = pix;
  r.mask = mask;
  r.chosen = chosen;
  r.bg_idx = bg_idx;
  r.nout = nout;
  r.warning = warning;
  return r;
}

}  // namespace
}  // namespace cp
