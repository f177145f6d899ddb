// cp_tile.cuh — frame-stack compositing kernels for sm_103a (included once per channel
// count by cp_kernels_c*.cu, which instantiate the kernels and their launchers).
//
// One CTA processes tiles of `tile_px` consecutive output pixels (4 per thread) across all
// n frames of a stack:
//   1. Warp 0 stages the tile with one cp.async.bulk (TMA engine) per frame row into shared
//      memory, frame-major, completing on an mbarrier (bounded wait).
//   2. Each thread owns `C` 32-bit words per frame row (4 pixels x C channels). For every
//      word it transposes 8 frames x 4 bytes with three delta swaps (8x8 bit transposes)
//      and a 4x4 byte transpose, giving 8 bit planes of up to 32*NW frames per channel
//      byte (frame i = bit i).
//   3. Order statistics (median, quartiles) come from a radix select on the planes: 8 steps
//      of popcounts on candidate masks; the next order statistic is the minimum above.
//   4. Distance pass over all frames: with an abs threshold and 0/1 weights the doubled
//      distance is exact integer arithmetic, 4*(p-m)^2 = 4*|p-floor m|*|p-ceil m| + [m
//      half-integer], one dp4a of two vabsdiff4 per pixel and frame; otherwise the f32
//      terms of src/chrono.rs:261-288 in the reference's operation order.
//   5. Per-pixel epilogue restating src/chrono.rs:290-493: background, outlier pick and
//      linear blend, the blend mask (src/chrono.rs:183-191) and optional diagnostics.
// darker/lighter (src/simple.rs:96-133) use the same staging with a streaming fold.
//
// Every f32 operation that must round like the Rust reference is an explicit _rn
// intrinsic, and the library is compiled with -fmad=false: no contraction anywhere.

#pragma once
#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>

#include "cp_internal.h"

namespace cp {
namespace {

#define DEVI __device__ __forceinline__

constexpr int kSmemHeader = 256;            // mbarrier + per-frame byte shifts
constexpr long long kWaitCycles = 1ll << 32; // ~2 s at 2 GHz before a wait gives up

// ---- PTX wrappers ------------------------------------------------------------------------
DEVI uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
DEVI void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
DEVI void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
DEVI void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
DEVI void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
DEVI bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// One bulk copy global -> shared (16-byte aligned addresses, size a multiple of 16).
DEVI void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// Bounded wait on an mbarrier phase: false after ~2 s (the caller records an error).
DEVI bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > kWaitCycles) return false;
  }
  return true;
}

// ---- Rust scalar semantics ------------------------------------------------------------------
// `f32 as u8`: saturating, NaN -> 0.
DEVI uint32_t sat_u8(float v) {
  if (!(v > 0.0f)) return 0u;
  if (v >= 255.0f) return 255u;
  return static_cast<uint32_t>(__float2int_rz(v));
}
// `f32::round`: half away from zero (CUDA roundf has the same definition).
DEVI float rround(float v) { return roundf(v); }
DEVI float u8f(uint32_t b) { return __uint_as_float(0x4B000000u | b) - 8388608.0f; }
DEVI float rsignum(float w) { return isnan(w) ? w : (signbit(w) ? -1.0f : 1.0f); }

// Threshold::blend_value, src/options.rs:223-231.
DEVI float blend_value(const StackDev& S, float dist) {
  if (dist <= S.thr_min) return 0.0f;
  if (dist >= S.thr_max) return 1.0f;
  return __fmul_rn(__fsub_rn(dist, S.thr_min), S.thr_scale);
}

// Counter-based replacement of ThreadRng::gen_range(0, n) (same definition as the oracle).
DEVI uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
DEVI uint32_t gen_range(uint64_t seed, uint64_t pixel, uint32_t n) {
  const uint64_t h = splitmix64(seed ^ splitmix64(pixel));
  return static_cast<uint32_t>(((h >> 32) * static_cast<uint64_t>(n)) >> 32);
}

// ---- tiles ------------------------------------------------------------------------------------
struct TileGeo {
  int out_px0;  // first output pixel (flat index)
  int npx;      // valid pixels in the tile
  int y, x0;    // row and first column (row-segment tiles)
};
DEVI TileGeo tile_geo(const StackDev& S, int t) {
  TileGeo g;
  if (S.tiles_per_row > 0) {
    const int row = t / S.tiles_per_row;
    g.y = S.row_begin + row;
    g.x0 = (t - row * S.tiles_per_row) * S.tile_px;
    g.npx = min(S.tile_px, S.width - g.x0);
    g.out_px0 = g.y * S.width + g.x0;
  } else {
    g.out_px0 = S.px_begin + t * S.tile_px;
    g.npx = min(S.tile_px, S.px_end - g.out_px0);
    g.y = 0;
    g.x0 = 0;
  }
  return g;
}

__host__ __device__ __forceinline__ int row_pitch(int tile_px, int C) { return tile_px * C + 32; }

// Warp 0 stages the n frame rows of a tile into `buf` (row f at f * pitch). A source that is
// not 16-byte aligned (cropped stacks, unaligned frames) is copied from the aligned address
// below it and the offset is recorded in shifts[f]. Must be called by all 32 lanes of warp 0.
template <int C>
DEVI void issue_tile(const StackDev& S, const TileGeo& g, uint8_t* buf, int pitch,
                     uint8_t* shifts, uint64_t* bar) {
  const int lane = threadIdx.x & 31;
  const int row_bytes = g.npx * C;
  uint32_t total = 0;
  for (int f = lane; f < S.n; f += 32) {
    long long off;
    if (S.has_crop) {
      const int cx = S.crop[2 * f], cy = S.crop[2 * f + 1];
      off = ((long long)(g.y + cy) * S.src_width + g.x0 + cx) * C;
    } else {
      off = (long long)g.out_px0 * C;
    }
    const uintptr_t src = reinterpret_cast<uintptr_t>(S.frames[f]) + off;
    const uintptr_t a0 = src & ~uintptr_t(15);
    const uintptr_t a1 = (src + row_bytes + 15) & ~uintptr_t(15);
    total += static_cast<uint32_t>(a1 - a0);
    shifts[f] = static_cast<uint8_t>(src - a0);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) total += __shfl_xor_sync(0xffffffffu, total, o);
  if (lane == 0) mbar_expect_tx(bar, total);
  __syncwarp();
  for (int f = lane; f < S.n; f += 32) {
    long long off;
    if (S.has_crop) {
      const int cx = S.crop[2 * f], cy = S.crop[2 * f + 1];
      off = ((long long)(g.y + cy) * S.src_width + g.x0 + cx) * C;
    } else {
      off = (long long)g.out_px0 * C;
    }
    const uintptr_t src = reinterpret_cast<uintptr_t>(S.frames[f]) + off;
    const uintptr_t a0 = src & ~uintptr_t(15);
    const uintptr_t a1 = (src + row_bytes + 15) & ~uintptr_t(15);
    bulk_g2s(buf + (size_t)f * pitch, reinterpret_cast<const void*>(a0),
             static_cast<uint32_t>(a1 - a0), bar);
  }
}

// Word `word` (0..C-1) of this thread's 4-pixel column in frame row f.
struct RowReader {
  const uint8_t* buf;
  const uint8_t* shifts;
  int pitch;
  int col;  // byte offset of this thread's column: 4 * C * thread
  bool shifted;  // rows may start off a 16-byte boundary: per-frame byte shift
  DEVI uint32_t word(int f, int w) const {
    const uint8_t* row = buf + (size_t)f * pitch;
    if (!shifted) return *reinterpret_cast<const uint32_t*>(row + col + 4 * w);
    const int off = shifts[f] + col + 4 * w;
    const uint32_t* r = reinterpret_cast<const uint32_t*>(row + (off & ~3));
    return __funnelshift_r(r[0], r[1], (off & 3) * 8);
  }
};

// Pixel p (0..3) of a thread's column as a word with its C channel bytes in bytes 0..C-1.
template <int C>
DEVI uint32_t pixel_word(const uint32_t (&w)[C], int p) {
  if constexpr (C == 1) {
    return (w[0] >> (8 * p)) & 0xFFu;
  } else if constexpr (C == 2) {
    return ((p < 2 ? w[0] : w[1]) >> (16 * (p & 1))) & 0xFFFFu;
  } else if constexpr (C == 3) {
    if (p == 0) return w[0] & 0x00FFFFFFu;
    if (p == 1) return __funnelshift_r(w[0], w[1], 24) & 0x00FFFFFFu;
    if (p == 2) return __funnelshift_r(w[1], w[2], 16) & 0x00FFFFFFu;
    return w[2] >> 8;
  } else {
    return w[p];
  }
}
// Pixel p (runtime 0..3) of frame f, loading only the words it spans.
template <int C>
DEVI uint32_t load_pixel(const RowReader& rd, int f, int p) {
  if constexpr (C == 1) {
    return (rd.word(f, 0) >> (8 * p)) & 0xFFu;
  } else if constexpr (C == 2) {
    return (rd.word(f, p >> 1) >> (16 * (p & 1))) & 0xFFFFu;
  } else if constexpr (C == 3) {
    if (p == 0) return rd.word(f, 0) & 0x00FFFFFFu;
    if (p == 1) return __funnelshift_r(rd.word(f, 0), rd.word(f, 1), 24) & 0x00FFFFFFu;
    if (p == 2) return __funnelshift_r(rd.word(f, 1), rd.word(f, 2), 16) & 0x00FFFFFFu;
    return rd.word(f, 2) >> 8;
  } else {
    return rd.word(f, p);
  }
}

// ---- bit planes -----------------------------------------------------------------------------
// 8x8 bit transpose of each byte column of 8 words: afterwards a[r] byte k bit i = bit r of
// byte k of input word i.
DEVI void transpose8(uint32_t (&a)[8]) {
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const uint32_t t = ((a[i] >> 4) ^ a[i + 4]) & 0x0F0F0F0Fu;
    a[i + 4] ^= t;
    a[i] ^= t << 4;
  }
#pragma unroll
  for (int i = 0; i < 8; i += 4) {
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const uint32_t t = ((a[i + j] >> 2) ^ a[i + j + 2]) & 0x33333333u;
      a[i + j + 2] ^= t;
      a[i + j] ^= t << 2;
    }
  }
#pragma unroll
  for (int i = 0; i < 8; i += 2) {
    const uint32_t t = ((a[i] >> 1) ^ a[i + 1]) & 0x55555555u;
    a[i + 1] ^= t;
    a[i] ^= t << 1;
  }
}

// Planes of byte positions KP0..KP0+BP-1 of word `w` over all frames: P[k][r][blk] bit i =
// bit r of the byte of frame 32*blk + i.
// One 32-frame block of planes: q[k][r] bit i = bit r of byte k of frame 32*blk + i.
DEVI void planes_block(uint32_t (&q)[4][8], const RowReader& rd, int w, int blk, int n) {
  uint32_t a[4][8];
#pragma unroll
  for (int g = 0; g < 4; ++g) {
    const int f0 = blk * 32 + g * 8;
    if (f0 + 8 <= n) {
#pragma unroll
      for (int r = 0; r < 8; ++r) a[g][r] = rd.word(f0 + r, w);
      transpose8(a[g]);
    } else if (f0 < n) {
#pragma unroll
      for (int r = 0; r < 8; ++r) a[g][r] = (f0 + r < n) ? rd.word(f0 + r, w) : 0u;
      transpose8(a[g]);
    } else {
#pragma unroll
      for (int r = 0; r < 8; ++r) a[g][r] = 0u;
    }
  }
#pragma unroll
  for (int r = 0; r < 8; ++r) {  // 4x4 byte transpose: group g -> byte g
    const uint32_t t0 = __byte_perm(a[0][r], a[1][r], 0x5140);
    const uint32_t t1 = __byte_perm(a[0][r], a[1][r], 0x7362);
    const uint32_t t2 = __byte_perm(a[2][r], a[3][r], 0x5140);
    const uint32_t t3 = __byte_perm(a[2][r], a[3][r], 0x7362);
    q[0][r] = __byte_perm(t0, t2, 0x5410);
    q[1][r] = __byte_perm(t0, t2, 0x7632);
    q[2][r] = __byte_perm(t1, t3, 0x5410);
    q[3][r] = __byte_perm(t1, t3, 0x7632);
  }
}

// Planes of byte positions KP0..KP0+BP-1 of word `w` over all frames: P[k][r][blk] bit i =
// bit r of the byte of frame 32*blk + i. Up to 64 frames the block loop is unrolled; above,
// a rolled loop shifts each block in from the top.
template <int C, int NW, int BP, int KP0>
DEVI void build_planes(uint32_t (&P)[BP][8][NW], const RowReader& rd, int w, int n) {
  if constexpr (NW <= 2) {
#pragma unroll
    for (int blk = 0; blk < NW; ++blk) {
      uint32_t q[4][8];
      planes_block(q, rd, w, blk, n);
#pragma unroll
      for (int k = 0; k < BP; ++k)
#pragma unroll
        for (int r = 0; r < 8; ++r) P[k][r][blk] = q[KP0 + k][r];
    }
  } else {
#pragma unroll 1
    for (int blk = 0; blk < NW; ++blk) {
      uint32_t q[4][8];
      planes_block(q, rd, w, blk, n);
#pragma unroll
      for (int k = 0; k < BP; ++k)
#pragma unroll
        for (int r = 0; r < 8; ++r) {
#pragma unroll
          for (int i = 0; i + 1 < NW; ++i) P[k][r][i] = P[k][r][i + 1];
          P[k][r][NW - 1] = q[KP0 + k][r];
        }
    }
  }
}

// k-th smallest (lo) and, when `pair`, (k+1)-th smallest (hi) of the frames in `S` given
// their bit planes. Radix select over the 8 bits; hi is lo when the run of lo continues,
// else the minimum of the values above lo.
template <int NW>
DEVI void select_pair(const uint32_t (&P)[8][NW], const uint32_t (&S)[NW], int k, bool pair,
                      uint32_t& lo, uint32_t& hi) {
  uint32_t c[NW];
#pragma unroll
  for (int w = 0; w < NW; ++w) c[w] = S[w];
  int kk = k;
  uint32_t res = 0;
#pragma unroll
  for (int b = 7; b >= 0; --b) {
    uint32_t z[NW];
    int cz = 0;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      z[w] = c[w] & ~P[b][w];
      cz += __popc(z[w]);
    }
    const bool one = kk >= cz;
    kk = one ? kk - cz : kk;
#pragma unroll
    for (int w = 0; w < NW; ++w) c[w] = one ? (c[w] & P[b][w]) : z[w];
    res |= static_cast<uint32_t>(one) << b;
  }
  lo = res;
  hi = res;
  if (!pair) return;
  int ceq = 0;
#pragma unroll
  for (int w = 0; w < NW; ++w) ceq += __popc(c[w]);
  const bool need = kk + 1 >= ceq;
  if (!__any_sync(0xffffffffu, need)) return;
  uint32_t gt[NW], eq[NW];
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    gt[w] = 0u;
    eq[w] = S[w];
  }
#pragma unroll
  for (int b = 7; b >= 0; --b) {
    const uint32_t rb = 0u - ((res >> b) & 1u);
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      gt[w] |= eq[w] & P[b][w] & ~rb;
      eq[w] &= ~(P[b][w] ^ rb);
    }
  }
  uint32_t m = 0;
#pragma unroll
  for (int b = 7; b >= 0; --b) {
    uint32_t z[NW];
    uint32_t any = 0;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      z[w] = gt[w] & ~P[b][w];
      any |= z[w];
    }
    const bool one = any == 0u;
#pragma unroll
    for (int w = 0; w < NW; ++w) gt[w] = one ? (gt[w] & P[b][w]) : z[w];
    m |= static_cast<uint32_t>(one) << b;
  }
  if (need) hi = m;
}

// quantile() of src/chrono.rs:567-579 from its two order statistics: (1-frac)*d[p1] +
// frac*d[p1+1], or d[k] when the host resolved frac < 0.001 / > 0.999 to a single index.
DEVI float quantile_value(uint32_t lo, uint32_t hi, bool pair, float frac) {
  if (!pair) return static_cast<float>(lo);
  return __fadd_rn(__fmul_rn(__fsub_rn(1.0f, frac), static_cast<float>(lo)),
                   __fmul_rn(frac, static_cast<float>(hi)));
}

// ---- per-pixel statistics -----------------------------------------------------------------
template <int C>
struct PixelStats {
  // f32 path: median and per-channel factor w*iqr_inv (rel) or w (abs)
  float med[4][C];
  float wi[4][C];
  float q1[4][C];
  float q3[4][C];
  // integer path: floor/ceil of the median per channel byte, nh = half-integer medians
  uint32_t klo[4], khi[4];
  int nh[4];
};

// Fill the statistics of the 4 pixels of this thread's column for one word of channel
// bytes. POS = byte index (0..4C-1) of the first position handled.
template <int C, int NW, int BP, int KP0>
DEVI void stats_for_word(const StackDev& S, const RowReader& rd, int w, PixelStats<C>& st,
                         const uint32_t (&smask)[NW]) {
  uint32_t P[BP][8][NW];
  build_planes<C, NW, BP, KP0>(P, rd, w, S.n);
#pragma unroll
  for (int k = 0; k < BP; ++k) {
    const int q = w * 4 + KP0 + k;  // byte within the 4C-byte column
    const int p = q / C, ch = q % C;
    if (!((S.wmask >> ch) & 1u)) continue;  // weight 0: median stays 0 (chrono.rs:230, :239)
    uint32_t lo, hi;
    select_pair<NW>(P[k], smask, S.med_k, S.med_pair != 0, lo, hi);
    const float med = S.med_pair ? __fmul_rn(0.5f, __fadd_rn(static_cast<float>(lo),
                                                             static_cast<float>(hi)))
                                 : static_cast<float>(lo);
    st.med[p][ch] = med;
    const uint32_t s2 = lo + hi;  // 2 * median when paired
    const uint32_t fl = S.med_pair ? (s2 >> 1) : lo;
    const uint32_t ce = S.med_pair ? ((s2 + 1) >> 1) : lo;
    st.klo[p] |= fl << (8 * ch);
    st.khi[p] |= ce << (8 * ch);
    st.nh[p] += static_cast<int>(ce - fl);
    if (!S.thr_abs) {
      uint32_t a, b;
      select_pair<NW>(P[k], smask, S.q1_k, S.q1_pair != 0, a, b);
      const float q1 = quantile_value(a, b, S.q1_pair != 0, S.q1_frac);
      select_pair<NW>(P[k], smask, S.q3_k, S.q3_pair != 0, a, b);
      const float q3 = quantile_value(a, b, S.q3_pair != 0, S.q3_frac);
      st.q1[p][ch] = q1;
      st.q3[p][ch] = q3;
      float iqr = __fsub_rn(q3, q1);  // src/chrono.rs:248-252
      if (iqr == 0.0f) iqr = 1.0f;
      const float inv = __fdiv_rn(1.0f, iqr);
      st.wi[p][ch] = __fmul_rn(S.w[ch], inv);
    } else {
      st.wi[p][ch] = S.w[ch];
    }
  }
}

// f32 squared distance of one pixel word to the median, src/chrono.rs:261-279.
template <int C>
DEVI float dist_f32(const StackDev& S, const float (&med)[C], const float (&wi)[C], uint32_t px) {
  float d = 0.0f;
#pragma unroll
  for (int ch = 0; ch < C; ++ch) {
    if ((S.wmask >> ch) & 1u) {
      const float v = u8f((px >> (8 * ch)) & 0xFFu);
      const float diff = __fsub_rn(med[ch], v);
      const float t = __fmul_rn(wi[ch], diff);
      float term = __fmul_rn(t, t);
      if (S.neg_w) term = __fmul_rn(rsignum(S.w[ch]), term);
      d = __fadd_rn(d, diff == 0.0f ? 0.0f : term);
    }
  }
  return d;
}
// Exact integer form for abs thresholds and 0/1 weights: D' with dist_sq = D' + nh/4.
DEVI uint32_t dist_int(uint32_t px, uint32_t wbytes, uint32_t klo, uint32_t khi) {
  const uint32_t v = px & wbytes;
  return __dp4a(__vabsdiffu4(v, klo), __vabsdiffu4(v, khi), 0u);
}

// blend_into_u8, src/color.rs:4-16, on a pixel word.
template <int C>
DEVI uint32_t blend_into_u8(uint32_t a, uint32_t b, float blend) {
  if (blend <= 0.0f) return a;
  if (blend >= 1.0f) return b;
  uint32_t r = 0;
#pragma unroll
  for (int ch = 0; ch < C; ++ch) {
    const float aa = static_cast<float>((a >> (8 * ch)) & 0xFFu);
    const float bb = static_cast<float>((b >> (8 * ch)) & 0xFFu);
    r |= sat_u8(rround(__fadd_rn(aa, __fmul_rn(__fsub_rn(bb, aa), blend)))) << (8 * ch);
  }
  return r;
}

template <int NW>
DEVI int popc_n(const uint32_t (&b)[NW]) {
  int c = 0;
#pragma unroll
  for (int w = 0; w < NW; ++w) c += __popc(b[w]);
  return c;
}
template <int NW>
DEVI int first_set(const uint32_t (&b)[NW]) {
#pragma unroll
  for (int w = 0; w < NW; ++w)
    if (b[w]) return 32 * w + __ffs(b[w]) - 1;
  return -1;
}
template <int NW>
DEVI int last_set(const uint32_t (&b)[NW]) {
#pragma unroll
  for (int w = NW - 1; w >= 0; --w)
    if (b[w]) return 32 * w + 31 - __clz(b[w]);
  return -1;
}

// Per-pixel state handed from the distance pass to the epilogue.
template <int C, int NW>
struct PixState {
  uint32_t bits[NW];  // outlier flags, frame i = bit i%32 of word i/32
  int32_t imax, dmax_i;
  float dmax_f;
  uint32_t klo, khi;
  int32_t nh;
  float med[C], wi[C], q1[C], q3[C];
};

// Background, outlier pick and blend of one pixel, src/chrono.rs:290-493, and its
// diagnostics. Kept out of line and called in a rolled loop to bound code size.
template <int C, int NW>
__device__ __noinline__ void pixel_epilogue(const StackDev& S, const RowReader& rd, int p,
                                            int pix_idx, bool valid, bool fast,
                                            uint32_t wbytes, const PixState<C, NW>& ps,
                                            uint32_t& out_pix, uint32_t& out_mask,
                                            uint32_t& warn_count) {
  const int n = S.n;
  auto dsq_of = [&](int f) -> float {  // dist_sq of frame f, recomputed
    const uint32_t px = load_pixel<C>(rd, f, p);
    if (fast)
      return static_cast<float>(dist_int(px, wbytes, ps.klo, ps.khi)) +
             0.25f * static_cast<float>(ps.nh);
    return dist_f32<C>(S, ps.med, ps.wi, px);
  };
  const int nout = popc_n<NW>(ps.bits);
  bool warning = false;
  int bg_idx = -1;
  uint32_t pix = 0;
  // background
  if (S.background == CP_BG_FIRST || S.background == CP_BG_RANDOM) {
    if (S.background == CP_BG_FIRST) {
      if (nout == 0) {
        bg_idx = 0;
      } else if (nout == n) {
        bg_idx = 0;
        warning = true;
      } else {
        uint32_t inv[NW];
#pragma unroll
        for (int w = 0; w < NW; ++w) inv[w] = ~ps.bits[w];
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
          uint32_t m = ps.bits[w];
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
    pix = load_pixel<C>(rd, bg_idx, p);
  } else if (S.background == CP_BG_AVERAGE) {
    uint32_t sum[C];
#pragma unroll
    for (int ch = 0; ch < C; ++ch) sum[ch] = 0u;
    for (int f = 0; f < n; ++f) {
      const uint32_t px = load_pixel<C>(rd, f, p);
#pragma unroll
      for (int ch = 0; ch < C; ++ch) sum[ch] += (px >> (8 * ch)) & 0xFFu;
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
        uint32_t m = ps.bits[w];
        while (m) {
          const int bpos = __ffs(m) - 1;
          m &= m - 1;
          const uint32_t px = load_pixel<C>(rd, 32 * w + bpos, p);
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
    for (int ch = 0; ch < C; ++ch) pix |= sat_u8(rround(ps.med[ch])) << (8 * ch);
  }

  // outlier pick and blend
  float blend = 0.0f;
  int chosen = -1;
  uint32_t mask = 0;
  if (nout == 1) {
    const int si = first_set<NW>(ps.bits);
    const float dsq = dsq_of(si);
    blend = __fmul_rn(S.fade[si], blend_value(S, __fsqrt_rn(dsq)));
    pix = blend_into_u8<C>(pix, load_pixel<C>(rd, si, p), blend);
    mask = sat_u8(rround(__fmul_rn(blend, 255.0f)));
    chosen = si;
  } else if (nout > 1) {
    if (S.outlier == CP_OUTLIER_FORWARD || S.outlier == CP_OUTLIER_BACKWARD) {
      float pf[C];
#pragma unroll
      for (int ch = 0; ch < C; ++ch) pf[ch] = static_cast<float>((pix >> (8 * ch)) & 0xFFu);
      float binv = 1.0f;
      const bool fwd = S.outlier == CP_OUTLIER_FORWARD;
      // outliers in ascending (forward) or descending (backward) frame order
      auto blend_one = [&](int f) {
        const float b = __fmul_rn(S.fade[f], blend_value(S, __fsqrt_rn(dsq_of(f))));
        const uint32_t s = load_pixel<C>(rd, f, p);
        // blend_into_f32_u8, src/color.rs:32-44
        if (b <= 0.0f) {
        } else if (b >= 1.0f) {
#pragma unroll
          for (int ch = 0; ch < C; ++ch) pf[ch] = static_cast<float>((s >> (8 * ch)) & 0xFFu);
        } else {
#pragma unroll
          for (int ch = 0; ch < C; ++ch) {
            const float sv = static_cast<float>((s >> (8 * ch)) & 0xFFu);
            pf[ch] = __fadd_rn(pf[ch], __fmul_rn(__fsub_rn(sv, pf[ch]), b));
          }
        }
        binv = __fmul_rn(binv, __fsub_rn(1.0f, b));
      };
      if (fwd) {
#pragma unroll
        for (int w = 0; w < NW; ++w) {
          uint32_t m = ps.bits[w];
          while (m) {
            const int f = 32 * w + __ffs(m) - 1;
            m &= m - 1;
            blend_one(f);
          }
        }
      } else {
#pragma unroll
        for (int w = NW - 1; w >= 0; --w) {
          uint32_t m = ps.bits[w];
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
    } else {
      int si;
      float dist;
      uint32_t sample;
      if (S.outlier == CP_OUTLIER_AVERAGE) {
        uint32_t osum[C];
#pragma unroll
        for (int ch = 0; ch < C; ++ch) osum[ch] = 0u;
        float mdist = 0.0f;
#pragma unroll
        for (int w = 0; w < NW; ++w) {
          uint32_t m = ps.bits[w];
          while (m) {
            const int f = 32 * w + __ffs(m) - 1;
            m &= m - 1;
            const uint32_t px = load_pixel<C>(rd, f, p);
#pragma unroll
            for (int ch = 0; ch < C; ++ch) osum[ch] += (px >> (8 * ch)) & 0xFFu;
            mdist = __fadd_rn(mdist, __fsqrt_rn(dsq_of(f)));
          }
        }
        const float kf = static_cast<float>(nout);
        sample = 0;
#pragma unroll
        for (int ch = 0; ch < C; ++ch)
          sample |= sat_u8(rround(__fdiv_rn(static_cast<float>(osum[ch]), kf))) << (8 * ch);
        si = 0;  // src/chrono.rs:467: the fade of an averaged outlier is taken at frame 0
        dist = __fdiv_rn(mdist, kf);
      } else {
        float dsq;
        if (S.outlier == CP_OUTLIER_FIRST) {
          si = first_set<NW>(ps.bits);
          dsq = dsq_of(si);
        } else if (S.outlier == CP_OUTLIER_LAST) {
          si = last_set<NW>(ps.bits);
          dsq = dsq_of(si);
        } else {  // extreme
          si = ps.imax;
          dsq = fast ? static_cast<float>(ps.dmax_i < 0 ? 0 : ps.dmax_i) +
                           (ps.dmax_i < 0 ? 0.0f : 0.25f * static_cast<float>(ps.nh))
                     : ps.dmax_f;
        }
        sample = load_pixel<C>(rd, si, p);
        dist = __fsqrt_rn(dsq);
      }
      blend = __fmul_rn(S.fade[si], blend_value(S, dist));
      pix = blend_into_u8<C>(pix, sample, blend);
      mask = sat_u8(rround(__fmul_rn(blend, 255.0f)));
      chosen = si;
    }
  }
  out_pix = pix;
  out_mask = mask;
  if (valid && warning) warn_count += 1;
  if (valid) {
    if (S.dbg_median || S.dbg_q1 || S.dbg_q3) {
#pragma unroll
      for (int ch = 0; ch < C; ++ch) {
        const size_t o = static_cast<size_t>(pix_idx) * C + ch;
        if (S.dbg_median) S.dbg_median[o] = ps.med[ch];
        if (S.dbg_q1) S.dbg_q1[o] = ps.q1[ch];
        if (S.dbg_q3) S.dbg_q3[o] = ps.q3[ch];
      }
    }
    if (S.dbg_bits) {
      const int words = (n + 31) / 32;
#pragma unroll
      for (int w = 0; w < NW; ++w)
        if (w < words) S.dbg_bits[static_cast<size_t>(pix_idx) * words + w] = ps.bits[w];
    }
    if (S.dbg_chosen) S.dbg_chosen[pix_idx] = chosen;
    if (S.dbg_bg) S.dbg_bg[pix_idx] = bg_idx;
    if (S.dbg_nout) S.dbg_nout[pix_idx] = nout;
  }
}

// ---- the outlier tile -----------------------------------------------------------------------
template <int C, int NW>
__device__ __noinline__ void outlier_tile(const StackDev& S, const TileGeo& g,
                                          const RowReader& rd, uint32_t& warn_count) {
  constexpr int BP = NW <= 2 ? 4 : 2;
  const int n = S.n;
  PixelStats<C> st;
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    st.klo[p] = st.khi[p] = 0u;
    st.nh[p] = 0;
#pragma unroll
    for (int ch = 0; ch < C; ++ch) st.med[p][ch] = st.wi[p][ch] = st.q1[p][ch] = st.q3[p][ch] = 0.0f;
  }
  uint32_t smask[NW];
#pragma unroll
  for (int w = 0; w < NW; ++w) smask[w] = S.sample_mask[w];

  // (2)+(3) planes and order statistics, word by word
#pragma unroll
  for (int w = 0; w < C; ++w) {
    if constexpr (BP == 4) {
      stats_for_word<C, NW, 4, 0>(S, rd, w, st, smask);
    } else {
      stats_for_word<C, NW, 2, 0>(S, rd, w, st, smask);
      stats_for_word<C, NW, 2, 2>(S, rd, w, st, smask);
    }
  }

  // (4) distance pass over all frames (src/chrono.rs:261-288)
  const bool fast = S.fast_int != 0;
  uint32_t wbytes = 0;
#pragma unroll
  for (int ch = 0; ch < C; ++ch)
    if ((S.wmask >> ch) & 1u) wbytes |= 0xFFu << (8 * ch);
  uint32_t bits[4][NW];
  int imax[4];
  int32_t dmax_i[4];
  float dmax_f[4];
  int32_t thr_i[4];
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    imax[p] = 0;
    dmax_i[p] = st.nh[p] > 0 ? -1 : 0;  // dist_sq > 0.0 <=> 4D' + nh > 0
    dmax_f[p] = 0.0f;
    thr_i[p] = S.thr_int[st.nh[p]];
#pragma unroll
    for (int w = 0; w < NW; ++w) bits[p][w] = 0u;
  }
#pragma unroll
  for (int blk = 0; blk < NW; ++blk) {
    const int f0 = blk * 32;
    const int fend = min(n, f0 + 32);
    uint32_t ob[4] = {0u, 0u, 0u, 0u};
    if (fast) {
      for (int f = f0; f < fend; ++f) {
        uint32_t wv[C];
#pragma unroll
        for (int i = 0; i < C; ++i) wv[i] = rd.word(f, i);
#pragma unroll
        for (int p = 0; p < 4; ++p) {
          const int32_t d =
              static_cast<int32_t>(dist_int(pixel_word<C>(wv, p), wbytes, st.klo[p], st.khi[p]));
          const bool o = d >= thr_i[p];
          ob[p] |= static_cast<uint32_t>(o) << (f - f0);
          if (o && d > dmax_i[p]) {
            dmax_i[p] = d;
            imax[p] = f;
          }
        }
      }
    } else {
      for (int f = f0; f < fend; ++f) {
        uint32_t wv[C];
#pragma unroll
        for (int i = 0; i < C; ++i) wv[i] = rd.word(f, i);
#pragma unroll
        for (int p = 0; p < 4; ++p) {
          const float d = dist_f32<C>(S, st.med[p], st.wi[p], pixel_word<C>(wv, p));
          const bool o = d >= S.thr_sq;
          ob[p] |= static_cast<uint32_t>(o) << (f - f0);
          if (o && d > dmax_f[p]) {
            dmax_f[p] = d;
            imax[p] = f;
          }
        }
      }
    }
#pragma unroll
    for (int p = 0; p < 4; ++p) bits[p][blk] = ob[p];
  }

  // (5) per-pixel epilogue
  PixState<C, NW> ps[4];
#pragma unroll
  for (int p = 0; p < 4; ++p) {
#pragma unroll
    for (int w = 0; w < NW; ++w) ps[p].bits[w] = bits[p][w];
    ps[p].imax = imax[p];
    ps[p].dmax_i = dmax_i[p];
    ps[p].dmax_f = dmax_f[p];
    ps[p].klo = st.klo[p];
    ps[p].khi = st.khi[p];
    ps[p].nh = st.nh[p];
#pragma unroll
    for (int ch = 0; ch < C; ++ch) {
      ps[p].med[ch] = st.med[p][ch];
      ps[p].wi[ch] = st.wi[p][ch];
      ps[p].q1[ch] = st.q1[p][ch];
      ps[p].q3[ch] = st.q3[p][ch];
    }
  }
  uint32_t outw[4], maskb[4];
#pragma unroll 1
  for (int p = 0; p < 4; ++p) {
    const int pix_idx = g.out_px0 + 4 * static_cast<int>(threadIdx.x) + p;
    const bool valid = 4 * static_cast<int>(threadIdx.x) + p < g.npx;
    pixel_epilogue<C, NW>(S, rd, p, pix_idx, valid, fast, wbytes, ps[p], outw[p], maskb[p],
                          warn_count);
  }

  // output: composite and blend mask (255 in channels >= 3), src/chrono.rs:183-191
  const int first = 4 * threadIdx.x;
  if (first >= g.npx) return;
  const size_t obyte = static_cast<size_t>(g.out_px0 + first) * C;
  uint32_t bm[4];
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    uint32_t v = 0;
#pragma unroll
    for (int ch = 0; ch < C; ++ch) v |= (ch < 3 ? maskb[p] : 255u) << (8 * ch);
    bm[p] = v;
  }
  const bool aligned = ((reinterpret_cast<uintptr_t>(S.out + obyte) |
                        (S.blend ? reinterpret_cast<uintptr_t>(S.blend + obyte) : 0)) & 3) == 0;
  if (first + 4 <= g.npx && aligned) {
    // 4 pixels = C words
    uint32_t ow[C], mw[C];
#pragma unroll
    for (int i = 0; i < C; ++i) ow[i] = mw[i] = 0u;
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
      for (int ch = 0; ch < C; ++ch) {
        const int q = p * C + ch;
        ow[q / 4] |= ((outw[p] >> (8 * ch)) & 0xFFu) << (8 * (q % 4));
        mw[q / 4] |= ((bm[p] >> (8 * ch)) & 0xFFu) << (8 * (q % 4));
      }
    uint32_t* o32 = reinterpret_cast<uint32_t*>(S.out + obyte);
#pragma unroll
    for (int i = 0; i < C; ++i) o32[i] = ow[i];
    if (S.blend) {
      uint32_t* b32 = reinterpret_cast<uint32_t*>(S.blend + obyte);
#pragma unroll
      for (int i = 0; i < C; ++i) b32[i] = mw[i];
    }
  } else {
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      if (first + p >= g.npx) break;
#pragma unroll
      for (int ch = 0; ch < C; ++ch) {
        S.out[obyte + p * C + ch] = static_cast<uint8_t>(outw[p] >> (8 * ch));
        if (S.blend) S.blend[obyte + p * C + ch] = static_cast<uint8_t>(bm[p] >> (8 * ch));
      }
    }
  }
}

// ---- darker / lighter tile ----------------------------------------------------------------
// SimpleProcessor fold, src/simple.rs:96-133: running extreme of sum_c p_c * w_c (f32, c
// ascending, strict compare: the earliest frame wins ties); on a new extreme the frame's
// pixel is blended into the running output (starting at 0) with the fade.
template <int C>
__device__ __noinline__ void simple_tile(const StackDev& S, const TileGeo& g,
                                         const RowReader& rd) {
  const bool darker = S.mode == CP_MODE_DARKER;
  float ext[4];
  uint32_t outw[4];
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    ext[p] = darker ? FLT_MAX : -FLT_MAX;
    outw[p] = 0u;
  }
  for (int f = 0; f < S.n; ++f) {
    uint32_t wv[C];
#pragma unroll
    for (int i = 0; i < C; ++i) wv[i] = rd.word(f, i);
    const float fade = S.fade[f];
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      const uint32_t px = pixel_word<C>(wv, p);
      float value = 0.0f;
#pragma unroll
      for (int ch = 0; ch < C; ++ch)
        value = __fadd_rn(value, __fmul_rn(u8f((px >> (8 * ch)) & 0xFFu), S.w[ch]));
      const bool is_ext = darker ? (value < ext[p]) : (value > ext[p]);
      if (is_ext) {
        ext[p] = value;
        if (fade > 0.0f) outw[p] = fade >= 1.0f ? px : blend_into_u8<C>(outw[p], px, fade);
      }
    }
  }
  const int first = 4 * threadIdx.x;
  if (first >= g.npx) return;
  const size_t obyte = static_cast<size_t>(g.out_px0 + first) * C;
  if (first + 4 <= g.npx && (reinterpret_cast<uintptr_t>(S.out + obyte) & 3) == 0) {
    uint32_t ow[C];
#pragma unroll
    for (int i = 0; i < C; ++i) ow[i] = 0u;
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
      for (int ch = 0; ch < C; ++ch) {
        const int q = p * C + ch;
        ow[q / 4] |= ((outw[p] >> (8 * ch)) & 0xFFu) << (8 * (q % 4));
      }
    uint32_t* o32 = reinterpret_cast<uint32_t*>(S.out + obyte);
#pragma unroll
    for (int i = 0; i < C; ++i) o32[i] = ow[i];
  } else {
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      if (first + p >= g.npx) break;
#pragma unroll
      for (int ch = 0; ch < C; ++ch)
        S.out[obyte + p * C + ch] = static_cast<uint8_t>(outw[p] >> (8 * ch));
    }
  }
}

template <int C>
DEVI void process_tile(const StackDev& S, const TileGeo& g, const RowReader& rd,
                       uint32_t& warn) {
  if (S.mode != CP_MODE_OUTLIER) {
    simple_tile<C>(S, g, rd);
  } else if (S.nw == 1) {
    outlier_tile<C, 1>(S, g, rd, warn);
  } else if (S.nw == 2) {
    outlier_tile<C, 2>(S, g, rd, warn);
  } else {
    outlier_tile<C, 4>(S, g, rd, warn);
  }
}

DEVI void flush_warnings(unsigned long long* dst, uint32_t w) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
  if ((threadIdx.x & 31) == 0 && w && dst) atomicAdd(dst, static_cast<unsigned long long>(w));
}

struct SmemLayout {
  uint64_t* bar;
  uint8_t* shifts;
  uint8_t* buf;
};
DEVI SmemLayout smem_layout(uint8_t* smem) {
  SmemLayout l;
  l.bar = reinterpret_cast<uint64_t*>(smem);
  l.shifts = smem + 16;
  l.buf = smem + kSmemHeader;
  return l;
}

// One stack, persistent CTAs striding over its tiles.
template <int C>
__global__ void __launch_bounds__(kThreads) k_composite(const __grid_constant__ StackDev S, uint32_t* error) {
  extern __shared__ __align__(128) uint8_t smem[];
  const SmemLayout L = smem_layout(smem);
  if (threadIdx.x == 0) {
    mbar_init(L.bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  const int pitch = row_pitch(S.tile_px, C);
  const RowReader rd{L.buf, L.shifts, pitch, 4 * C * static_cast<int>(threadIdx.x), S.shifted != 0};
  uint32_t phase = 0, warn = 0;
  for (int t = blockIdx.x; t < S.tiles; t += gridDim.x) {
    const TileGeo g = tile_geo(S, t);
    if (threadIdx.x < 32) {
      fence_proxy_async();
      issue_tile<C>(S, g, L.buf, pitch, L.shifts, L.bar);
    }
    __syncthreads();
    if (!mbar_wait(L.bar, phase)) {
      if (error) atomicOr(error, 1u);
      return;
    }
    phase ^= 1u;
    process_tile<C>(S, g, rd, warn);
    __syncthreads();
  }
  flush_warnings(S.warnings, warn);
}

// Many stacks: persistent CTAs pull (stack, tile) items from a device counter.
template <int C>
__global__ void __launch_bounds__(kThreads) k_composite_batch(const StackDev* __restrict__ stacks,
                                                        const int32_t* __restrict__ prefix,
                                                        int32_t n_stacks, int32_t total,
                                                        uint32_t* counter, uint32_t* error) {
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ int item_s, stack_s;
  const SmemLayout L = smem_layout(smem);
  if (threadIdx.x == 0) {
    mbar_init(L.bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  uint32_t phase = 0;
  for (;;) {
    if (threadIdx.x == 0) {
      const int it = static_cast<int>(atomicAdd(counter, 1u));
      int lo = 0, hi = n_stacks;  // largest s with prefix[s] <= it
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (prefix[mid] <= it) lo = mid; else hi = mid;
      }
      item_s = it;
      stack_s = lo;
    }
    __syncthreads();
    const int it = item_s, s = stack_s;
    if (it >= total) break;
    const StackDev& S = stacks[s];
    const int pitch = row_pitch(S.tile_px, C);
    const TileGeo g = tile_geo(S, it - prefix[s]);
    if (threadIdx.x < 32) {
      fence_proxy_async();
      issue_tile<C>(S, g, L.buf, pitch, L.shifts, L.bar);
    }
    __syncthreads();
    if (!mbar_wait(L.bar, phase)) {
      if (error) atomicOr(error, 1u);
      return;
    }
    phase ^= 1u;
    const RowReader rd{L.buf, L.shifts, pitch, 4 * C * static_cast<int>(threadIdx.x), S.shifted != 0};
    uint32_t warn = 0;
    if (static_cast<int>(threadIdx.x) < S.threads) process_tile<C>(S, g, rd, warn);
    flush_warnings(S.warnings, warn);
    __syncthreads();
  }
}

}  // namespace
}  // namespace cp
