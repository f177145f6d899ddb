// cp_tile.cuh — frame-stack compositing kernels for sm_103a (included by cp_kernels_c*.cu,
// which instantiate the general kernels and their launchers, and by cp_kernels_variant.cu /
// cp_kernels_batch_variant.cu, compiled once per specialised kernel).
//
// A tile is 128 consecutive output pixels: 32 columns of 4 pixels, i.e. C 32-bit words per
// column and frame row. A CTA of C warps processes tiles across all n frames of a stack:
//   1. Warp 0 stages the tile with one cp.async.bulk (TMA engine) per frame row into shared
//      memory, frame-major, completing on an mbarrier (bounded wait).
//   2. Warp w takes word w of every column (lane = column) and transposes 8 frames x 4
//      bytes with three delta swaps (8x8 bit transposes) and a 4x4 byte transpose, giving
//      8 bit planes of up to 32*NW frames per channel byte (frame i = bit i).
//   3. Order statistics (median, quartiles) come from a radix select on the planes: 8 steps
//      of popcounts on candidate masks; a pair d[k], d[k+1] takes two passes.
//   4. Distance pass, warp w over the frames f = w (mod C), 4 pixels per lane: with an abs
//      threshold and 0/1 weights the doubled distance is exact integer arithmetic (three
//      dp4a per pixel and frame); otherwise the f32 terms of src/chrono.rs:261-288 in the
//      reference's operation order (two pixels per instruction where the ranges allow).
//   5. Per-pixel epilogue restating src/chrono.rs:290-493: background, outlier pick and
//      linear blend, the blend mask (src/chrono.rs:183-191) and optional diagnostics.
// Results cross warps through a shared-memory exchange area (Aux). darker/lighter
// (src/simple.rs:96-133) stream through a TMA stage ring (k_simple_stream), or use the tile
// staging for cropped / unaligned stacks (simple_tile).
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

constexpr long long kWaitCycles = kDefaultWaitCycles;  // ~2 s at 2 GHz before a wait gives up

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
// Bounded wait on an mbarrier phase: false once `limit` SM clock cycles have passed (the
// caller records an error); a limit of 1 or less gives up without testing the phase.
DEVI bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit = kWaitCycles) {
  if (limit <= 1) return false;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > limit) return false;
  }
  return true;
}

// Paired f32 add / multiply, round to nearest, as PTX with an explicit rounding mode; each
// lane rounds like __fadd_rn / __fmul_rn. A paired product must not feed a paired sum: the
// compiler contracted both __fadd2_rn(d, __fmul2_rn(t, t)) and add.rn.f32x2 after
// mul.rn.f32x2 into a fused multiply-add even with -fmad=false (one ulp off, which breaks
// ties between equal distances); products are therefore summed with scalar __fadd_rn.
DEVI unsigned long long f2_bits(float2 v) {
  return static_cast<unsigned long long>(__float_as_uint(v.x)) |
         (static_cast<unsigned long long>(__float_as_uint(v.y)) << 32);
}
DEVI float2 bits_f2(unsigned long long b) {
  return make_float2(__uint_as_float(static_cast<uint32_t>(b)),
                     __uint_as_float(static_cast<uint32_t>(b >> 32)));
}
DEVI float2 add2_rn(float2 a, float2 b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return bits_f2(r);
}
DEVI float2 mul2_rn(float2 a, float2 b) {
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return bits_f2(r);
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

// Shared-memory row pitch of a tile: 4 pixels per thread, plus room for the byte shift of
// rows copied from below an unaligned source.
template <int C>
constexpr int kPitch = kTilePx * C + 32;

// Resident CTAs per SM the register allocation is sized for: 6 x 96 threads at <= 112
// registers for RGB; RGBA (4 warps) is limited to 4 by shared memory at 64 frames anyway;
// grayscale (1 warp) at 16.
template <int C>
constexpr int kMinCtas = C == 3 ? 6 : (C == 4 ? 4 : 16);

// Warp 0 stages the n frame rows of a tile into `buf` (row f at f * pitch) from the frame
// bases cached in shared memory. A source that is not 16-byte aligned (cropped stacks,
// unaligned frames) is copied from the aligned address below it and the offset is recorded
// in shifts[f]. Must be called by all 32 lanes of warp 0.
template <int C>
DEVI void issue_tile(const StackDev& S, const TileGeo& g, uint8_t* buf, uint8_t* shifts,
                     const uintptr_t* fbase, uint64_t* bar) {
  constexpr int pitch = kPitch<C>;
  const int lane = threadIdx.x & 31;
  const uint32_t row_bytes = static_cast<uint32_t>(g.npx * C);
  if (!S.shifted) {  // every row starts 16-byte aligned: one size for all
    const uint32_t sz = (row_bytes + 15u) & ~15u;
    const uintptr_t off = static_cast<uintptr_t>(g.out_px0) * C;
    if (lane == 0) mbar_expect_tx(bar, sz * static_cast<uint32_t>(S.n));
    __syncwarp();
    for (int f = lane; f < S.n; f += 32)
      bulk_g2s(buf + (size_t)f * pitch, reinterpret_cast<const void*>(fbase[f] + off), sz, bar);
    return;
  }
  uint32_t total = 0;
  for (int f = lane; f < S.n; f += 32) {
    long long off;
    if (S.has_crop) {
      const int cx = S.crop[2 * f], cy = S.crop[2 * f + 1];
      off = ((long long)(g.y + cy) * S.src_width + g.x0 + cx) * C;
    } else {
      off = (long long)g.out_px0 * C;
    }
    const uintptr_t src = fbase[f] + off;
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
    const uintptr_t src = fbase[f] + off;
    const uintptr_t a0 = src & ~uintptr_t(15);
    const uintptr_t a1 = (src + row_bytes + 15) & ~uintptr_t(15);
    bulk_g2s(buf + (size_t)f * pitch, reinterpret_cast<const void*>(a0),
             static_cast<uint32_t>(a1 - a0), bar);
  }
}

// ---- shared-memory rows ------------------------------------------------------------------------
// Word w (0..C-1) of this thread's 4-pixel column in frame row f. SHIFTED rows start
// shifts[f] bytes into their shared-memory row (sources below a 16-byte boundary).
template <int C, bool SHIFTED>
struct Rows {
  const uint8_t* col;  // shared-memory data + 4 * C * thread
  const uint8_t* shifts;
  DEVI uint32_t word(int f, int w) const {
    const uint8_t* row = col + f * kPitch<C>;
    if constexpr (!SHIFTED) {
      return *reinterpret_cast<const uint32_t*>(row + 4 * w);
    } else {
      const int off = shifts[f] + 4 * w;
      const uint32_t* r = reinterpret_cast<const uint32_t*>(row + (off & ~3));
      return __funnelshift_r(r[0], r[1], (off & 3) * 8);
    }
  }
  DEVI void frame(int f, uint32_t (&wv)[C]) const {
#pragma unroll
    for (int i = 0; i < C; ++i) wv[i] = word(f, i);
  }
};

// Pixel p (0..3) of a thread's column as a word with its C channel bytes in bytes 0..C-1.
template <int C>
DEVI uint32_t pixel_word(const uint32_t (&w)[C], int p) {
  if constexpr (C == 1) {
    return (w[0] >> (8 * p)) & 0xFFu;
  } else if constexpr (C == 3) {
    if (p == 0) return w[0] & 0x00FFFFFFu;
    if (p == 1) return __funnelshift_r(w[0], w[1], 24) & 0x00FFFFFFu;
    if (p == 2) return __funnelshift_r(w[1], w[2], 16) & 0x00FFFFFFu;
    return w[2] >> 8;
  } else {
    return w[p];
  }
}
// Same with a runtime pixel index, loading only the words the pixel spans.
template <int C, bool SH>
DEVI uint32_t load_pixel(const Rows<C, SH>& rd, int f, int p) {
  if constexpr (C == 1) {
    return (rd.word(f, 0) >> (8 * p)) & 0xFFu;
  } else if constexpr (C == 3) {
    // bytes 3p .. 3p+2 of the column: word 3p/4 shifted right by (3p mod 4) bytes, topped up
    // from the next word (no branch on p)
    const int q = 3 * p, w0 = q >> 2;
    return __funnelshift_r(rd.word(f, w0), rd.word(f, min(w0 + 1, 2)), 8 * (q & 3)) &
           0x00FFFFFFu;
  } else {
    return rd.word(f, p);
  }
}

// Element p of a 4-array held in registers, selected without local memory.
template <typename T>
DEVI T pick4(const T (&a)[4], int p) {
  T v = a[0];
  v = p == 1 ? a[1] : v;
  v = p == 2 ? a[2] : v;
  v = p == 3 ? a[3] : v;
  return v;
}

// ---- bit planes ------------------------------------------------------------------------------
// 8x8 bit transpose of each byte column of 8 words: afterwards a[r] byte k bit i = bit r of
// byte k of input word i.
DEVI void transpose8(uint32_t (&a)[8]) {
  // swap the off-diagonal blocks of each 8x8 bit matrix at scales 4, 2, 1: the bits of b
  // under M move up by s into a, the bits of a above M move down into b
  auto swap = [](uint32_t& x, uint32_t& y, int sh, uint32_t m) {
    const uint32_t nx = (x & ~(m << sh)) | ((y << sh) & (m << sh));
    const uint32_t ny = (y & ~m) | ((x >> sh) & m);
    x = nx;
    y = ny;
  };
#pragma unroll
  for (int i = 0; i < 4; ++i) swap(a[i], a[i + 4], 4, 0x0F0F0F0Fu);
#pragma unroll
  for (int i = 0; i < 8; i += 4) {
    swap(a[i], a[i + 2], 2, 0x33333333u);
    swap(a[i + 1], a[i + 3], 2, 0x33333333u);
  }
#pragma unroll
  for (int i = 0; i < 8; i += 2) swap(a[i], a[i + 1], 1, 0x55555555u);
}

// One 32-frame block of planes of word w: q[k][r] bit i = bit r of byte k of frame 32*blk+i.
template <int C, bool SH>
DEVI void planes_block(uint32_t (&q)[4][8], const Rows<C, SH>& rd, int w, int blk, int n) {
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

// Planes of the BP byte positions kp0.. of word w over all frames: P[k][r][blk] bit i = bit
// r of the byte of frame 32*blk + i. kp0 is 0 when BP == 4, 0 or 2 when BP == 2.
template <int C, int NW, int BP, bool SH>
DEVI void build_planes(uint32_t (&P)[BP][8][NW], const Rows<C, SH>& rd, int w, int kp0, int n) {
#pragma unroll
  for (int blk = 0; blk < NW; ++blk) {
    uint32_t q[4][8];
    planes_block<C, SH>(q, rd, w, blk, n);
#pragma unroll
    for (int k = 0; k < BP; ++k)
#pragma unroll
      for (int r = 0; r < 8; ++r) P[k][r][blk] = (BP == 4 || kp0 == 0) ? q[k][r] : q[k + BP][r];
  }
}

// Order statistic d[k] for BP byte positions at once (independent chains the scheduler
// interleaves): one radix pass over the 8 bit planes, each step counting the candidates with
// a 0 bit (POPC) and keeping the half that holds rank k. A pair d[k], d[k+1] is two passes:
// measured cheaper than tracking the sibling branch of rank k+1 and walking it afterwards.
template <int NW, int BP>
DEVI void select_rank(const uint32_t (&P)[BP][8][NW], const uint32_t (&S)[NW], int k,
                      uint32_t (&v)[BP]) {
  // Per step: d = kk - (candidates with a 0 bit); its sign mask M (-1: rank kk lies among
  // them) selects the half by one LOP3 per word (c & (P ^ M)) and keeps kk or d; the value
  // bits accumulate as u = 2u + M (u = -(bits of the zero halves)), so v = 255 + u.
  uint32_t c[BP][NW];
  int kk[BP], u[BP];
#pragma unroll
  for (int j = 0; j < BP; ++j) {
#pragma unroll
    for (int w = 0; w < NW; ++w) c[j][w] = S[w];
    kk[j] = k;
    u[j] = 0;
  }
#pragma unroll
  for (int b = 7; b >= 0; --b) {
#pragma unroll
    for (int j = 0; j < BP; ++j) {
      int d = kk[j];
#pragma unroll
      for (int w = 0; w < NW; ++w) d -= __popc(c[j][w] & ~P[j][b][w]);
      const int m = d >> 31;
#pragma unroll
      for (int w = 0; w < NW; ++w) c[j][w] &= P[j][b][w] ^ static_cast<uint32_t>(m);
      kk[j] = (kk[j] & m) | (d & ~m);
      u[j] = 2 * u[j] + m;
    }
  }
#pragma unroll
  for (int j = 0; j < BP; ++j) v[j] = static_cast<uint32_t>(255 + u[j]);
}

// quantile() of src/chrono.rs:567-579 from its order statistics: (1-frac)*d[p1] +
// frac*d[p1+1], or d[k] alone when the host resolved frac < 0.001 / > 0.999 to one index.
DEVI float quantile_value(uint32_t lo, uint32_t hi, bool pair, float frac) {
  if (!pair) return static_cast<float>(lo);
  return __fadd_rn(__fmul_rn(__fsub_rn(1.0f, frac), static_cast<float>(lo)),
                   __fmul_rn(frac, static_cast<float>(hi)));
}

// ---- per-pixel arithmetic ------------------------------------------------------------------
// f32 squared distance of one pixel word to the median, src/chrono.rs:261-279, in the
// reference's operation order. `medo` is median + 2^22: with the sample byte placed in the
// mantissa of 2^22 (ulp 0.5) both are exact and their difference is exactly median - p.
// The `diff == 0 -> 0` case needs no select when every w * iqr_inv is finite (FINITE), since
// then t = wi * 0 = 0 and t * t = 0.
// NEGW: some weight may be negative (the paired kind excludes them).
template <int C, bool FINITE, bool NEGW = true>
DEVI float dist_f32(const StackDev& S, const float (&medo)[C], const float (&wi)[C], uint32_t px) {
  float d = 0.0f;
#pragma unroll
  for (int ch = 0; ch < C; ++ch) {
    if ((S.wmask >> ch) & 1u) {
      const float v = __uint_as_float(0x4A800000u + (((px >> (8 * ch)) & 0xFFu) << 1));
      const float diff = __fsub_rn(medo[ch], v);
      const float t = __fmul_rn(wi[ch], diff);
      float term = __fmul_rn(t, t);
      if (NEGW && S.neg_w) term = __fmul_rn(rsignum(S.w[ch]), term);
      if constexpr (!FINITE) term = diff == 0.0f ? 0.0f : term;
      d = __fadd_rn(d, term);
    }
  }
  return d;
}
// Exact integer form for abs thresholds and 0/1 weights: D' with dist_sq = D' + nh/4.
// Each channel term |p - lo| * |p - hi| = (p - lo) * (p - hi) (hi - lo is 0 or 1 and p is an
// integer, so the product is never negative) = p*p - p*lo - p*hi + lo*hi: three dp4a.
DEVI uint32_t dist_int(uint32_t px, uint32_t wbytes, uint32_t klo, uint32_t khi) {
  const uint32_t v = px & wbytes;
  return __dp4a(v, v, __dp4a(klo, khi, 0u)) - __dp4a(v, khi, __dp4a(v, klo, 0u));
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


// ---- tile exchange area ------------------------------------------------------------------
// A tile is 32 columns x 4 pixels, served by C warps: warp w builds the planes and order
// statistics of word w of every column, all warps run the distance pass over the frames of
// their residue class (f = w mod C), and the epilogue is split by pixel. Results move between
// warps through this shared-memory area behind the staged rows.

// Per-pixel statistics of column t from the words' order statistics (positions q = p*C + ch).
template <int C>
struct PixStats {
  uint32_t klo, khi;  // floor / ceil of the medians, channel bytes (integer path)
  int nh;             // channels with a half-integer median
  float med[C], medo[C], wi[C];
};
template <int C, int NW>
DEVI PixStats<C> pixel_stats(const StackDev& S, const Aux<C, NW>& A, int t, int p) {
  PixStats<C> r;
  r.klo = r.khi = 0u;
  r.nh = 0;
  const bool rel = !S.thr_abs;
#pragma unroll
  for (int ch = 0; ch < C; ++ch) {
    const int q = p * C + ch;
    const uint32_t lo = (A.lo[q >> 2][t] >> (8 * (q & 3))) & 0xFFu;
    const uint32_t hi = (A.hi[q >> 2][t] >> (8 * (q & 3))) & 0xFFu;
    const bool wt = (S.wmask >> ch) & 1u;
    // median(), src/chrono.rs:582-591; weight-0 channels keep 0 (chrono.rs:222, :239)
    r.med[ch] = !wt ? 0.0f
                    : (S.med_pair ? __fmul_rn(0.5f, __fadd_rn(static_cast<float>(lo),
                                                              static_cast<float>(hi)))
                                  : static_cast<float>(lo));
    r.medo[ch] = __fadd_rn(r.med[ch], 4194304.0f);  // exact: med is a multiple of 1/2
    r.wi[ch] = rel ? A.wi[q >> 2][q & 3][t] : S.w[ch];
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

// Stores the tile's staged output rows (C words per column) with coalesced 32-bit stores;
// a partial or misaligned tile stores its valid bytes one by one.
template <int C>
DEVI void store_rows(uint8_t* out, const TileGeo& g, const uint32_t (&rows)[C][32]) {
  const uint8_t* src = reinterpret_cast<const uint8_t*>(rows);
  uint8_t* dst = out + static_cast<size_t>(g.out_px0) * C;
  const int nbytes = g.npx * C;
  const bool full = nbytes == kTilePx * C && (reinterpret_cast<uintptr_t>(dst) & 3) == 0;
  for (int i = threadIdx.x; i < 32 * C; i += 32 * C) {
    // word i of the row: column i / C, word i % C
    const uint32_t v = rows[i % C][i / C];
    if (full) {
      reinterpret_cast<uint32_t*>(dst)[i] = v;
    } else {
#pragma unroll
      for (int b = 0; b < 4; ++b)
        if (4 * i + b < nbytes) dst[4 * i + b] = static_cast<uint8_t>(v >> (8 * b));
    }
  }
  (void)src;
}

// ---- the outlier tile -----------------------------------------------------------------------
// Kernel kinds: kAnyKind handles every stack (batches mix them); a single-stack launch takes
// the kind of its distance arithmetic, so each kernel holds only the code it runs (smaller
// instruction footprint, register allocation of its own).
// Kinds: kIntKind (abs, 0/1 weights: integer distances), kF32Kind (paired f32 distances),
// kF32GenKind (scalar f32 distances), kPxKind (integer or paired f32 by the stack's flags,
// never scalar: the settings of a multi-setting launch). Likewise the outlier group (OG)
// fixes the epilogue:
// kOgSingle (extreme / first / last: one sample), kOgAverage, kOgBlend (forward / backward),
// or kOgAny; and BG the background: kBgFirst or kBgAny.
enum : int { kAnyKind = 0, kIntKind = 1, kF32Kind = 2, kF32GenKind = 3, kPxKind = 4 };
enum : int { kOgAny = 0, kOgSingle = 1, kOgAverage = 2, kOgBlend = 3 };
enum : int { kBgAny = 0, kBgFirst = 1 };
template <int KIND>
DEVI bool fast_path(const StackDev& S) {
  return KIND == kIntKind ? true : (KIND == kAnyKind ? S.fast_int != 0 : false);
}
template <int KIND>
DEVI bool pair_path(const StackDev& S) {
  return KIND == kF32Kind ? true : (KIND == kAnyKind ? S.pair_f32 != 0 : false);
}
template <int OG>
DEVI bool og_is(const StackDev& S, int og) {
  if (OG != kOgAny) return OG == og;
  const int m = S.outlier;
  if (og == kOgAverage) return m == CP_OUTLIER_AVERAGE;
  if (og == kOgBlend) return m == CP_OUTLIER_FORWARD || m == CP_OUTLIER_BACKWARD;
  return m == CP_OUTLIER_EXTREME || m == CP_OUTLIER_FIRST || m == CP_OUTLIER_LAST;
}

// (2)+(3) of a tile: bit planes of word wp of column t and the order statistics of its 4
// byte positions: plo / phi = d[k], d[k+1] of the median per byte (d[k] twice without a pair),
// and for rel thresholds wq[k] = w * iqr_inv (src/chrono.rs:220-255) and the debug quartiles.
template <int C, int NW, bool SH, int KIND, int BPR = (NW <= 2 ? 4 : 2)>
DEVI void word_order_stats(const StackDev& S, const TileGeo& g, const Rows<C, SH>& rd, int wp,
                           int t, uint32_t& plo_out, uint32_t& phi_out, float (&wq_out)[4]) {
  constexpr int BP = BPR;  // byte positions per plane build (register budget)
  const int n = S.n;
  uint32_t smask[NW];
#pragma unroll
  for (int w = 0; w < NW; ++w) smask[w] = S.sample_mask[w];
  const bool rel = KIND == kIntKind ? false : !S.thr_abs;  // the integer path is abs only
    uint32_t plo = 0u, phi = 0u;
    float wq[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int kp0 = 0; kp0 < 4; kp0 += BP) {
      uint32_t P[BP][8][NW];
      build_planes<C, NW, BP, SH>(P, rd, wp, kp0, n);
      // d[k] (and d[k+1] of a pair) of the median, and for rel thresholds of Q1 and Q3,
      // through one copy of the selection code per path: loops rather than inlined
      // selections (measured faster; the instruction cache is the tighter resource). The
      // loop shapes differ per kernel kind because each measured best for its kind.
      uint32_t a1[BP], b1[BP], a3[BP], b3[BP];
      if constexpr (KIND == kIntKind) {  // abs thresholds only
        uint32_t mlo[BP], mhi[BP];
#pragma unroll 1
        for (int r = 0; r < 2; ++r) {
          if (r == 1 && !S.med_pair) continue;
          uint32_t v[BP];
          select_rank<NW, BP>(P, smask, S.med_k + r, v);
#pragma unroll
          for (int k = 0; k < BP; ++k) {
            mlo[k] = r == 0 ? v[k] : mlo[k];
            mhi[k] = v[k];  // the successor, or the value itself without a pair
          }
        }
#pragma unroll
        for (int k = 0; k < BP; ++k) {
          plo |= mlo[k] << (8 * (kp0 + k));
          phi |= mhi[k] << (8 * (kp0 + k));
        }
      } else {
        if (!rel) {
          uint32_t lo[BP], hi[BP];
#pragma unroll 1
          for (int r = 0; r < (S.med_pair ? 2 : 1); ++r) {
            uint32_t v[BP];
            select_rank<NW, BP>(P, smask, S.med_k + r, v);
#pragma unroll
            for (int k = 0; k < BP; ++k) {
              lo[k] = r == 0 ? v[k] : lo[k];
              hi[k] = v[k];
            }
          }
#pragma unroll
          for (int k = 0; k < BP; ++k) {
            plo |= lo[k] << (8 * (kp0 + k));
            phi |= hi[k] << (8 * (kp0 + k));
          }
        }
        uint32_t mlo[BP], mhi[BP];
#pragma unroll 1
        for (int r = 0; r < (rel ? 6 : 0); ++r) {
          const int rk = r >> 1;  // 0 median, 1 Q1, 2 Q3; odd r: the successor d[k+1]
          const int kr = rk == 0 ? S.med_k : (rk == 1 ? S.q1_k : S.q3_k);
          const int pr = rk == 0 ? S.med_pair : (rk == 1 ? S.q1_pair : S.q3_pair);
          if ((r & 1) && !pr) continue;
          uint32_t v[BP];
          select_rank<NW, BP>(P, smask, kr + (r & 1), v);
#pragma unroll
          for (int k = 0; k < BP; ++k) {
            if (!(r & 1)) {
              mlo[k] = rk == 0 ? v[k] : mlo[k];
              a1[k] = rk == 1 ? v[k] : a1[k];
              a3[k] = rk == 2 ? v[k] : a3[k];
            }
            // the successor, or the value itself when the rank has no pair
            mhi[k] = rk == 0 ? v[k] : mhi[k];
            b1[k] = rk == 1 ? v[k] : b1[k];
            b3[k] = rk == 2 ? v[k] : b3[k];
          }
        }
        if (rel) {
#pragma unroll
          for (int k = 0; k < BP; ++k) {
            plo |= mlo[k] << (8 * (kp0 + k));
            phi |= mhi[k] << (8 * (kp0 + k));
          }
        }
      }
      if (rel) {  // quartiles and w * iqr_inv, src/chrono.rs:246-252
#pragma unroll
        for (int k = 0; k < BP; ++k) {
          const float q1 = quantile_value(a1[k], b1[k], S.q1_pair != 0, S.q1_frac);
          const float q3 = quantile_value(a3[k], b3[k], S.q3_pair != 0, S.q3_frac);
          float iqr = __fsub_rn(q3, q1);
          if (iqr == 0.0f) iqr = 1.0f;
          const int q = 4 * wp + kp0 + k, ch = q % C;
          wq[kp0 + k] = __fmul_rn(S.w[ch], __fdiv_rn(1.0f, iqr));
          const int px = 4 * t + q / C;
          if ((S.dbg_q1 || S.dbg_q3) && px < g.npx) {
            const size_t o = static_cast<size_t>(g.out_px0 + px) * C + ch;
            const bool wt = (S.wmask >> ch) & 1u;
            if (S.dbg_q1) S.dbg_q1[o] = wt ? q1 : 0.0f;
            if (S.dbg_q3) S.dbg_q3[o] = wt ? q3 : 0.0f;
          }
        }
      }
    }
    plo_out = plo;
    phi_out = phi;
#pragma unroll
    for (int k = 0; k < 4; ++k) wq_out[k] = wq[k];
}

template <int C, int NW, bool SH, int KIND, int OG, int BG>
DEVI void outlier_tile(const StackDev& S, const TileGeo& g, const Rows<C, SH>& rd,
                       Aux<C, NW>& A, uint32_t& warn_count) {
  const int n = S.n;
  const int wp = static_cast<int>(threadIdx.x) >> 5;  // warp: word, frame class, pixels
  const int t = static_cast<int>(threadIdx.x) & 31;   // column

  // (2)+(3) planes and order statistics of word wp, BP positions per round
  {
    uint32_t plo = 0u, phi = 0u;
    float wq[4];
    word_order_stats<C, NW, SH, KIND>(S, g, rd, wp, t, plo, phi, wq);
    A.lo[wp][t] = plo;
    A.hi[wp][t] = phi;
#pragma unroll
    for (int k = 0; k < 4; ++k) A.wi[wp][k][t] = wq[k];
  }
  __syncthreads();

  // per-pixel statistics of this column
  const bool fast = fast_path<KIND>(S);
  uint32_t wbytes = 0;
#pragma unroll
  for (int ch = 0; ch < C; ++ch)
    if ((S.wmask >> ch) & 1u) wbytes |= 0xFFu << (8 * ch);
  uint32_t klo[4], khi[4];
  int nh[4];
  float medo[4][C], wi[4][C];
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const PixStats<C> ps = pixel_stats<C, NW>(S, A, t, p);
    klo[p] = ps.klo;
    khi[p] = ps.khi;
    nh[p] = ps.nh;
#pragma unroll
    for (int ch = 0; ch < C; ++ch) {
      medo[p][ch] = ps.medo[ch];
      wi[p][ch] = ps.wi[ch];
    }
  }
  if (S.dbg_median && wp == 0) {
#pragma unroll
    for (int p = 0; p < 4; ++p)
      if (4 * t + p < g.npx) {
        const PixStats<C> ps = pixel_stats<C, NW>(S, A, t, p);
#pragma unroll
        for (int ch = 0; ch < C; ++ch)
          S.dbg_median[static_cast<size_t>(g.out_px0 + 4 * t + p) * C + ch] = ps.med[ch];
      }
  }

  // (4) distance pass (src/chrono.rs:261-288) over the frames f = wp (mod C)
  {
    uint32_t bits[4][NW];
    int32_t kmax[4], thr_i[4], imax[4];
    float dmax_f[4];
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      // max key (D' << 8) + 255 - f; the reference starts from dist_sq 0.0 at frame 0 and
      // takes strictly larger values: with nh > 0 every frame beats that start (-1)
      kmax[p] = nh[p] > 0 ? -1 : 255;
      thr_i[p] = S.thr_int[nh[p]];
      dmax_f[p] = 0.0f;
      imax[p] = 0;
#pragma unroll
      for (int w = 0; w < NW; ++w) bits[p][w] = 0u;
    }
#pragma unroll
    for (int blk = 0; blk < NW; ++blk) {
      const int f0 = blk * 32;
      const int fend = min(n, f0 + 32);
      int fs = f0 + ((wp - f0 % C) % C + C) % C;  // first frame of class wp in the block
      uint32_t ob[4] = {0u, 0u, 0u, 0u};
      if (fast) {
#pragma unroll 2
        for (int f = fs; f < fend; f += C) {
          uint32_t wv[C];
          rd.frame(f, wv);
          const uint32_t m = 1u << (f - f0);
          const int32_t fk = 255 - f;
#pragma unroll
          for (int p = 0; p < 4; ++p) {
            const int32_t d =
                static_cast<int32_t>(dist_int(pixel_word<C>(wv, p), wbytes, klo[p], khi[p]));
            ob[p] |= d >= thr_i[p] ? m : 0u;
            // the largest distance, earliest frame first: the argmax over all frames is an
            // outlier whenever any frame is one (src/chrono.rs:283-286)
            kmax[p] = max(kmax[p], (d << 8) + fk);
          }
        }
      } else if (pair_path<KIND>(S)) {
        // pixels (0, 1) and (2, 3) in float2 lanes, every term on (median - p) / 2: the
        // sample -(2^14 + p/2) is one byte permute of the pixel byte into -2^14's mantissa,
        // the median 2^14 + median/2 is exact, and their sum is exactly (median - p) / 2.
        // Terms, sums and the threshold are the reference's values times exactly 1/4.
        float2 mq[2][C], wq[2][C];
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
          for (int ch = 0; ch < C; ++ch) {
            const float m0 = __fsub_rn(medo[2 * h][ch], 4194304.0f);
            const float m1 = __fsub_rn(medo[2 * h + 1][ch], 4194304.0f);
            mq[h][ch] = make_float2(__fadd_rn(__fmul_rn(m0, 0.5f), 16384.0f),
                                    __fadd_rn(__fmul_rn(m1, 0.5f), 16384.0f));
            wq[h][ch] = make_float2(wi[2 * h][ch], wi[2 * h + 1][ch]);
          }
        const float thr4 = __fmul_rn(S.thr_sq, 0.25f);
        for (int f = fs; f < fend; f += C) {
          uint32_t wv[C];
          rd.frame(f, wv);
          const uint32_t m = 1u << (f - f0);
          float2 dq[2] = {make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f)};
#pragma unroll
          for (int ch = 0; ch < C; ++ch) {
            if (!((S.wmask >> ch) & 1u)) continue;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const int q0 = 2 * h * C + ch, q1 = q0 + C;  // byte of pixel 2h / 2h+1
              const float2 nv = make_float2(
                  __uint_as_float(__byte_perm(wv[q0 >> 2], 0xC6800000u, 0x7604u | ((q0 & 3) << 4))),
                  __uint_as_float(__byte_perm(wv[q1 >> 2], 0xC6800000u, 0x7604u | ((q1 & 3) << 4))));
              const float2 tt = mul2_rn(wq[h][ch], add2_rn(mq[h][ch], nv));
              const float2 sq = mul2_rn(tt, tt);
              dq[h].x = __fadd_rn(dq[h].x, sq.x);
              dq[h].y = __fadd_rn(dq[h].y, sq.y);
            }
          }
          const float dd[4] = {dq[0].x, dq[0].y, dq[1].x, dq[1].y};
#pragma unroll
          for (int p = 0; p < 4; ++p) {
            const bool o = dd[p] >= thr4;
            ob[p] |= o ? m : 0u;
            const bool up = o && dd[p] > dmax_f[p];
            dmax_f[p] = up ? dd[p] : dmax_f[p];
            imax[p] = up ? f : imax[p];
          }
        }
      } else if (S.finite_w) {
        for (int f = fs; f < fend; f += C) {
          uint32_t wv[C];
          rd.frame(f, wv);
          const uint32_t m = 1u << (f - f0);
#pragma unroll
          for (int p = 0; p < 4; ++p) {
            const float d = dist_f32<C, true>(S, medo[p], wi[p], pixel_word<C>(wv, p));
            const bool o = d >= S.thr_sq;
            ob[p] |= o ? m : 0u;
            const bool up = o && d > dmax_f[p];
            dmax_f[p] = up ? d : dmax_f[p];
            imax[p] = up ? f : imax[p];
          }
        }
      } else {
        for (int f = fs; f < fend; f += C) {
          uint32_t wv[C];
          rd.frame(f, wv);
          const uint32_t m = 1u << (f - f0);
#pragma unroll
          for (int p = 0; p < 4; ++p) {
            const float d = dist_f32<C, false>(S, medo[p], wi[p], pixel_word<C>(wv, p));
            const bool o = d >= S.thr_sq;
            ob[p] |= o ? m : 0u;
            const bool up = o && d > dmax_f[p];
            dmax_f[p] = up ? d : dmax_f[p];
            imax[p] = up ? f : imax[p];
          }
        }
      }
#pragma unroll
      for (int p = 0; p < 4; ++p) bits[p][blk] = ob[p];
    }
#pragma unroll
    for (int p = 0; p < 4; ++p) {
#pragma unroll
      for (int w = 0; w < NW; ++w) A.bits[wp][p][w][t] = bits[p][w];
      // only `extreme` reads the largest distance: other outlier groups leave it (and, the
      // compiler seeing it dead, its computation in the distance pass) out
      if (OG == kOgAny || OG == kOgSingle) {
        // the paired pass kept distances / 4: scale back exactly
        A.best[wp][p][t] =
            fast ? kmax[p]
                 : __float_as_int(pair_path<KIND>(S) ? __fmul_rn(dmax_f[p], 4.0f) : dmax_f[p]);
        A.imf[wp][p][t] = imax[p];
      }
    }
  }
  __syncthreads();

  // (5) per-pixel epilogue, src/chrono.rs:290-493: warp wp takes pixels wp, wp + C, ...
#pragma unroll 1
  for (int p = wp; p < 4; p += C) {
    const int pix_idx = g.out_px0 + 4 * t + p;
    const bool valid = 4 * t + p < g.npx;
    // combine the frame classes: flags OR, integer key max, f32 (distance, earliest frame)
    uint32_t pb[NW];
    constexpr bool kMaxKept = OG == kOgAny || OG == kOgSingle;  // see the distance pass
    int32_t key = kMaxKept ? A.best[0][p][t] : -1;
    float pdmax_f = kMaxKept ? __int_as_float(A.best[0][p][t]) : 0.0f;
    int pimf = kMaxKept ? A.imf[0][p][t] : 0;
#pragma unroll
    for (int w = 0; w < NW; ++w) pb[w] = A.bits[0][p][w][t];
#pragma unroll
    for (int c = 1; c < C; ++c) {
#pragma unroll
      for (int w = 0; w < NW; ++w) pb[w] |= A.bits[c][p][w][t];
      if (kMaxKept) {
        key = max(key, A.best[c][p][t]);
        const float d = __int_as_float(A.best[c][p][t]);
        const int fi = A.imf[c][p][t];
        const bool better = d > pdmax_f || (d == pdmax_f && fi < pimf);
        pdmax_f = better ? d : pdmax_f;
        pimf = better ? fi : pimf;
      }
    }
    const PixStats<C> ps = pixel_stats<C, NW>(S, A, t, p);
    const uint32_t pklo = ps.klo, pkhi = ps.khi;
    const int pnh = ps.nh;
    float pmed[C], pmedo[C], pwi[C];
#pragma unroll
    for (int ch = 0; ch < C; ++ch) {
      pmed[ch] = ps.med[ch];
      pmedo[ch] = ps.medo[ch];
      pwi[ch] = ps.wi[ch];
    }
    const int pimax = fast ? (key < 0 ? 0 : 255 - (key & 255)) : pimf;
    const int32_t pdmax_i = key < 0 ? -1 : (key >> 8);
    auto dsq_px = [&](uint32_t px) -> float {  // dist_sq of a sample, recomputed
      if (fast)
        return static_cast<float>(dist_int(px, wbytes, pklo, pkhi)) +
               0.25f * static_cast<float>(pnh);
      // the paired kind runs only for finite, non-negative weights
      if constexpr (KIND == kF32Kind) return dist_f32<C, true, false>(S, pmedo, pwi, px);
      return dist_f32<C, false>(S, pmedo, pwi, px);
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
      pix = load_pixel<C, SH>(rd, bg_idx, p);
    } else if (bgm == CP_BG_AVERAGE) {
      uint32_t sum[C];
#pragma unroll
      for (int ch = 0; ch < C; ++ch) sum[ch] = 0u;
      for (int f = 0; f < n; ++f) {
        const uint32_t px = load_pixel<C, SH>(rd, f, p);
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
          uint32_t m = pb[w];
          while (m) {
            const int bpos = __ffs(m) - 1;
            m &= m - 1;
            const uint32_t px = load_pixel<C, SH>(rd, 32 * w + bpos, p);
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
      for (int ch = 0; ch < C; ++ch) pix |= sat_u8(rround(pmed[ch])) << (8 * ch);
    }

    // outlier pick and blend, src/chrono.rs:377-493. One outlier (any mode) and first / last /
    // extreme pick a single sample: one branch-free path for every lane, where no outlier
    // gives blend 0 (the background unchanged, mask 0). Average / forward / backward with
    // several outliers loop over them.
    float blend = 0.0f;
    int chosen = -1;
    uint32_t mask = 0;
    const bool single_group = og_is<OG>(S, kOgSingle);
    const bool blend_group = og_is<OG>(S, kOgBlend);
    const bool extreme = single_group && S.outlier == CP_OUTLIER_EXTREME;
    const bool multi = nout > 1 && !single_group;
    if (!multi) {
      int si;
      float dsq;
      if (extreme) {
        si = pimax;
        if (fast) {
          const int32_t dm = pdmax_i;
          dsq = dm < 0 ? 0.0f : static_cast<float>(dm) + 0.25f * static_cast<float>(pnh);
        } else {
          dsq = pdmax_f;
        }
      } else {
        // the multi-outlier groups come here with at most one outlier: first == last
        si = (single_group && S.outlier == CP_OUTLIER_LAST) ? last_set<NW>(pb) : first_set<NW>(pb);
        si = si < 0 ? 0 : si;
      }
      const uint32_t sample = load_pixel<C, SH>(rd, si, p);
      if (!extreme) dsq = dsq_px(sample);
      blend = nout == 0 ? 0.0f : __fmul_rn(S.fade[si], blend_value(S, __fsqrt_rn(dsq)));
      pix = blend_into_u8<C>(pix, sample, blend);
      mask = sat_u8(rround(__fmul_rn(blend, 255.0f)));
      chosen = nout == 0 ? -1 : si;
    } else {
      if (blend_group) {
        float pf[C];
#pragma unroll
        for (int ch = 0; ch < C; ++ch) pf[ch] = static_cast<float>((pix >> (8 * ch)) & 0xFFu);
        float binv = 1.0f;
        auto blend_one = [&](int f) {
          const uint32_t sv = load_pixel<C, SH>(rd, f, p);
          const float bk = __fmul_rn(S.fade[f], blend_value(S, __fsqrt_rn(dsq_px(sv))));
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
        // outliers in ascending (forward) or descending (backward) frame order
        if (S.outlier == CP_OUTLIER_FORWARD) {
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
      } else {  // average, src/chrono.rs:429-468
        int si;
        float dist;
        uint32_t sample;
        {
          // channel sums in 16-bit lanes (n * 255 < 2^16): even bytes, odd bytes
          uint32_t se = 0u, so = 0u;
          float mdist = 0.0f;
#pragma unroll
          for (int w = 0; w < NW; ++w) {
            uint32_t m = pb[w];
            while (m) {
              const int f = 32 * w + __ffs(m) - 1;
              m &= m - 1;
              const uint32_t px = load_pixel<C, SH>(rd, f, p);
              se += px & 0x00FF00FFu;
              so += (px >> 8) & 0x00FF00FFu;
              mdist = __fadd_rn(mdist, __fsqrt_rn(dsq_px(px)));
            }
          }
          const float kf = static_cast<float>(nout);
          sample = 0;
#pragma unroll
          for (int ch = 0; ch < C; ++ch) {
            const uint32_t os = ((ch & 1) ? so : se) >> (16 * (ch >> 1)) & 0xFFFFu;
            sample |= sat_u8(rround(__fdiv_rn(static_cast<float>(os), kf))) << (8 * ch);
          }
          si = 0;  // src/chrono.rs:467: the fade of an averaged outlier is taken at frame 0
          dist = __fdiv_rn(mdist, kf);
        }
        blend = __fmul_rn(S.fade[si], blend_value(S, dist));
        pix = blend_into_u8<C>(pix, sample, blend);
        mask = sat_u8(rround(__fmul_rn(blend, 255.0f)));
        chosen = si;
      }
    }
    // stage the pixel's composite and mask bytes (255 in channels >= 3, chrono.rs:183-191)
    uint8_t* ob = reinterpret_cast<uint8_t*>(A.out);
    uint8_t* bb = reinterpret_cast<uint8_t*>(A.blend);
#pragma unroll
    for (int ch = 0; ch < C; ++ch) {
      const int q = p * C + ch;  // byte q of column t = word q/4 byte q%4
      const int off = 4 * (32 * (q >> 2) + t) + (q & 3);
      ob[off] = static_cast<uint8_t>(pix >> (8 * ch));
      bb[off] = static_cast<uint8_t>(ch < 3 ? mask : 255u);
    }
    if (valid) {
      if (warning) warn_count += 1;
      if (S.dbg_bits) {
        const int words = (n + 31) / 32;
#pragma unroll
        for (int w = 0; w < NW; ++w)
          if (w < words) S.dbg_bits[static_cast<size_t>(pix_idx) * words + w] = pb[w];
      }
      if (S.dbg_chosen) S.dbg_chosen[pix_idx] = chosen;
      if (S.dbg_bg) S.dbg_bg[pix_idx] = bg_idx;
      if (S.dbg_nout) S.dbg_nout[pix_idx] = nout;
    }
  }
  __syncthreads();
  store_rows<C>(S.out, g, A.out);
  if (S.blend) store_rows<C>(S.blend, g, A.blend);
}

// ---- darker / lighter tile ----------------------------------------------------------------
// SimpleProcessor fold, src/simple.rs:96-133, for stacks the streaming kernel does not take
// (cropped or unaligned frames): running extreme of sum_c p_c * w_c (f32, c ascending, strict
// compare: the earliest frame wins ties); on a new extreme the frame's pixel is blended into
// the running output (starting at 0) with the frame's fade. Warp wp takes pixels wp, wp+C, ...
template <int C, int NW, bool SH>
DEVI void simple_tile(const StackDev& S, const TileGeo& g, const Rows<C, SH>& rd, Aux<C, NW>& A) {
  const bool darker = S.mode == CP_MODE_DARKER;
  const int wp = static_cast<int>(threadIdx.x) >> 5;
  const int t = static_cast<int>(threadIdx.x) & 31;
#pragma unroll 1
  for (int p = wp; p < 4; p += C) {
    float ext = darker ? FLT_MAX : -FLT_MAX;
    uint32_t outw = 0u;
    for (int f = 0; f < S.n; ++f) {
      const uint32_t px = load_pixel<C, SH>(rd, f, p);
      float value = 0.0f;
#pragma unroll
      for (int ch = 0; ch < C; ++ch)
        value = __fadd_rn(value, __fmul_rn(u8f((px >> (8 * ch)) & 0xFFu), S.w[ch]));
      const bool up = darker ? (value < ext) : (value > ext);
      ext = up ? value : ext;
      const float fade = S.fade[f];
      if (up && fade > 0.0f) outw = fade >= 1.0f ? px : blend_into_u8<C>(outw, px, fade);
    }
    uint8_t* ob = reinterpret_cast<uint8_t*>(A.out);
#pragma unroll
    for (int ch = 0; ch < C; ++ch) {
      const int q = p * C + ch;
      ob[4 * (32 * (q >> 2) + t) + (q & 3)] = static_cast<uint8_t>(outw >> (8 * ch));
    }
  }
  __syncthreads();
  store_rows<C>(S.out, g, A.out);
}

// Kinds other than kAnyKind only run outlier stacks.
template <int C, bool SH, int KIND, int OG, int BG>
DEVI void process_tile(const StackDev& S, const TileGeo& g, const Rows<C, SH>& rd,
                       uint8_t* aux, uint32_t& warn) {
  if (S.nw == 1) {
    Aux<C, 1>& A = *reinterpret_cast<Aux<C, 1>*>(aux);
    if (KIND == kAnyKind && S.mode != CP_MODE_OUTLIER) simple_tile<C, 1, SH>(S, g, rd, A);
    else outlier_tile<C, 1, SH, KIND, OG, BG>(S, g, rd, A, warn);
  } else if (S.nw == 2) {
    Aux<C, 2>& A = *reinterpret_cast<Aux<C, 2>*>(aux);
    if (KIND == kAnyKind && S.mode != CP_MODE_OUTLIER) simple_tile<C, 2, SH>(S, g, rd, A);
    else outlier_tile<C, 2, SH, KIND, OG, BG>(S, g, rd, A, warn);
  } else {
    Aux<C, 4>& A = *reinterpret_cast<Aux<C, 4>*>(aux);
    if (KIND == kAnyKind && S.mode != CP_MODE_OUTLIER) simple_tile<C, 4, SH>(S, g, rd, A);
    else outlier_tile<C, 4, SH, KIND, OG, BG>(S, g, rd, A, warn);
  }
}

DEVI void flush_warnings(unsigned long long* dst, uint32_t w) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
  if ((threadIdx.x & 31) == 0 && w && dst) atomicAdd(dst, static_cast<unsigned long long>(w));
}

struct SmemLayout {
  uint64_t* bar;
  uint8_t* shifts;    // [CP_MAX_FRAMES]
  uintptr_t* fbase;   // [CP_MAX_FRAMES] frame base pointers of the current stack
  uint8_t* buf;
};
DEVI SmemLayout smem_layout(uint8_t* smem) {
  SmemLayout l;
  l.bar = reinterpret_cast<uint64_t*>(smem);
  l.shifts = smem + 16;
  l.fbase = reinterpret_cast<uintptr_t*>(smem + 256);
  l.buf = smem + kSmemHeader;
  return l;
}
// Warp 0 copies the stack's frame pointers into shared memory (once per stack).
DEVI void load_fbase(const StackDev& S, const SmemLayout& L) {
  if (threadIdx.x < 32)
    for (int f = threadIdx.x; f < S.n; f += 32)
      L.fbase[f] = reinterpret_cast<uintptr_t>(S.frames[f]);
}

// Stage a tile, wait for it (bounded) and process it. Returns false after a timed-out wait.
// The exchange area sits behind the n staged rows.
template <int C, int KIND, int OG, int BG>
DEVI bool run_tile(const StackDev& S, const TileGeo& g, const SmemLayout& L, uint32_t& phase,
                   uint32_t* error, uint32_t& warn) {
  if (threadIdx.x < 32) {
    fence_proxy_async();
    issue_tile<C>(S, g, L.buf, L.shifts, L.fbase, L.bar);
  }
  __syncthreads();
  // bounded wait; the CTA leaves together if any thread's wait gave up, once the copies in
  // flight into its shared memory have landed
  const bool ok = mbar_wait(L.bar, phase, S.wait_cycles);
  if (__syncthreads_or(ok ? 0 : 1)) {
    if (!ok) mbar_wait(L.bar, phase);
    if (error && threadIdx.x == 0) atomicOr(error, 1u);
    return false;
  }
  phase ^= 1u;
  const uint8_t* col = L.buf + 4 * C * (threadIdx.x & 31);
  uint8_t* aux = L.buf + static_cast<size_t>(S.n) * kPitch<C>;
  if (S.shifted) {
    const Rows<C, true> rd{col, L.shifts};
    process_tile<C, true, KIND, OG, BG>(S, g, rd, aux, warn);
  } else {
    const Rows<C, false> rd{col, L.shifts};
    process_tile<C, false, KIND, OG, BG>(S, g, rd, aux, warn);
  }
  __syncthreads();
  return true;
}

// One stack, persistent CTAs (C warps each) striding over its tiles.
template <int C, int KIND, int OG, int BG>
__global__ void __launch_bounds__(32 * C, kMinCtas<C>) k_composite(const __grid_constant__ StackDev S,
                                                      uint32_t* error) {
  extern __shared__ __align__(128) uint8_t smem[];
  const SmemLayout L = smem_layout(smem);
  if (threadIdx.x == 0) {
    mbar_init(L.bar, 1);
    fence_mbar_init();
  }
  load_fbase(S, L);
  __syncthreads();
  uint32_t phase = 0, warn = 0;
  for (int t = blockIdx.x; t < S.tiles; t += gridDim.x)
    if (!run_tile<C, KIND, OG, BG>(S, tile_geo(S, t), L, phase, error, warn)) return;
  flush_warnings(S.warnings, warn);
}

template <int C, int KIND, int OG, int BG>
int max_ctas_kind(int threads, int smem) {
  const void* fn = reinterpret_cast<const void*>(&k_composite<C, KIND, OG, BG>);
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, threads, smem) != cudaSuccess)
    return 1;
  return blocks < 1 ? 1 : blocks;
}

template <int C, int KIND, int OG, int BG>
int launch_composite_kind(const StackDev& s, int grid, int smem, void* stream, uint32_t* error) {
  const void* fn = reinterpret_cast<const void*>(&k_composite<C, KIND, OG, BG>);
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  k_composite<C, KIND, OG, BG><<<grid, s.threads, smem, static_cast<cudaStream_t>(stream)>>>(s, error);
  return static_cast<int>(cudaGetLastError());
}

// Many stacks: persistent CTAs pull (stack, tile) items from a device counter.
constexpr int kBatchPrefixSmem = 65;  // batches of up to 64 stacks search their prefix sums in
                                      // shared memory (bigger ones in global memory) A batch whose
// stacks all take one specialised variant (chrono-video windows share their settings) runs
// that variant; mixed batches the general kernel.
template <int C, int KIND, int OG, int BG>
__global__ void __launch_bounds__(32 * C, kMinCtas<C>) k_composite_batch(const StackDev* __restrict__ stacks,
                                                            const int32_t* __restrict__ prefix,
                                                            int32_t n_stacks, int32_t total,
                                                            int32_t interleave,
                                                            uint32_t* counter, uint32_t* error) {
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ int item_s, stack_s;
  __shared__ int32_t prefix_s[kBatchPrefixSmem];  // the tile prefix sums of small batches
  const SmemLayout L = smem_layout(smem);
  const bool small = n_stacks < kBatchPrefixSmem;
  if (small && !interleave)
    for (int i = threadIdx.x; i <= n_stacks; i += blockDim.x) prefix_s[i] = prefix[i];
  // work item `it` -> (stack_s, item_s); thread 0
  auto decode = [&](int it) {
    if (interleave) {
      // stacks of one geometry (chrono-video windows): tile-major order, so consecutive
      // items read the same rows of mostly the same frames while they are in L2
      stack_s = it % n_stacks;
      item_s = it / n_stacks;
    } else {
      const int32_t* pf = small ? prefix_s : prefix;
      int lo = 0, hi = n_stacks;  // largest s with prefix[s] <= it
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (pf[mid] <= it) lo = mid; else hi = mid;
      }
      stack_s = lo;
      item_s = it - pf[lo];
    }
    if (it >= total) item_s = -1;
  };
  if (threadIdx.x == 0) {
    mbar_init(L.bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) decode(static_cast<int>(atomicAdd(counter, 1u)));
  __syncthreads();
  uint32_t phase = 0;
  int cached = -1;  // stack whose frame bases are in shared memory
  int tile = item_s, s = stack_s;
  while (tile >= 0) {
    // the next item is drawn now and decoded after this tile: the atomic's latency hides
    // behind the tile's work
    int next_it = 0;
    if (threadIdx.x == 0) next_it = static_cast<int>(atomicAdd(counter, 1u));
    const StackDev& S = stacks[s];
    if (s != cached) {
      load_fbase(S, L);
      cached = s;
      __syncthreads();
    }
    uint32_t warn = 0;
    if (!run_tile<C, KIND, OG, BG>(S, tile_geo(S, tile), L, phase, error, warn)) return;
    flush_warnings(S.warnings, warn);
    // run_tile ended with a barrier: every thread has read item_s / stack_s
    if (threadIdx.x == 0) decode(next_it);
    __syncthreads();
    tile = item_s;
    s = stack_s;
  }
}

template <int C, int KIND, int OG, int BG>
int batch_max_ctas_kind(int smem) {
  const void* fn = reinterpret_cast<const void*>(&k_composite_batch<C, KIND, OG, BG>);
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, 32 * C, smem) != cudaSuccess)
    return 1;
  return blocks < 1 ? 1 : blocks;
}

template <int C, int KIND, int OG, int BG>
int launch_batch_kind(const StackDev* stacks, const int32_t* prefix, int32_t n_stacks,
                      int32_t total, int32_t interleave, uint32_t* counter, uint32_t* error,
                      int grid, int smem, void* stream) {
  const void* fn = reinterpret_cast<const void*>(&k_composite_batch<C, KIND, OG, BG>);
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  k_composite_batch<C, KIND, OG, BG><<<grid, 32 * C, smem, static_cast<cudaStream_t>(stream)>>>(
      stacks, prefix, n_stacks, total, interleave, counter, error);
  return static_cast<int>(cudaGetLastError());
}

// darker/lighter streaming over an aligned, uncropped stack: a CTA of 128 threads owns chunks
// of 2048 pixels (16 per thread) and pulls the chunk's row of every frame through a ring of
// kStreamStages shared-memory stages with one cp.async.bulk each (TMA engine; thread 0 issues
// stage s again as soon as all threads have folded it), so several frame rows per CTA are in
// flight at all times. Each thread folds its 16 pixels frame by frame in order. FAST: weights
// 0/1 and every fade >= 1, where the f32 sum of src/simple.rs:103-106 is an exact integer and
// a new extreme copies the pixel.
constexpr int kStreamThreads = 128;
constexpr int kStreamPx = 16;  // pixels per thread
constexpr int kStreamStages = 4;
constexpr int kStreamChunkPx = kStreamThreads * kStreamPx;
template <int C>
constexpr int kStreamStageBytes = kStreamChunkPx * C;

template <int C, bool FAST>
__global__ void __launch_bounds__(kStreamThreads, 8)
    k_simple_stream(const __grid_constant__ StackDev S, uint32_t* error) {
  constexpr int NWD = 4 * C;  // 32-bit words per thread per frame
  extern __shared__ __align__(128) uint8_t smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  uint8_t* stage = smem + 128;
  const bool darker = S.mode == CP_MODE_DARKER;
  const int n = S.n;
  const int P = S.px_end - S.px_begin;
  const int chunks = (P + kStreamChunkPx - 1) / kStreamChunkPx;
  const int mine = static_cast<int>(blockIdx.x) < chunks
                       ? (chunks - 1 - static_cast<int>(blockIdx.x)) / static_cast<int>(gridDim.x) + 1
                       : 0;
  const int items = mine * n;  // (chunk, frame) in chunk-major order
  if (items == 0) return;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int st = 0; st < kStreamStages; ++st) mbar_init(&full[st], 1);
    fence_mbar_init();
  }
  __syncthreads();
  auto chunk_px0 = [&](int i) {
    return S.px_begin + (static_cast<int>(blockIdx.x) + (i / n) * static_cast<int>(gridDim.x)) *
                            kStreamChunkPx;
  };
  auto issue = [&](int i) {  // thread 0: item i into stage i % kStreamStages
    const int px0 = chunk_px0(i);
    const int npx = min(kStreamChunkPx, S.px_end - px0);
    const uint32_t bytes = (static_cast<uint32_t>(npx * C) + 15u) & ~15u;
    uint64_t* bar = &full[i % kStreamStages];
    mbar_expect_tx(bar, bytes);
    bulk_g2s(stage + (i % kStreamStages) * kStreamStageBytes<C>,
             S.frames[i % n] + static_cast<size_t>(px0) * C, bytes, bar);
  };
  if (threadIdx.x == 0)
    for (int i = 0; i < min(kStreamStages, items); ++i) issue(i);
  uint32_t wbytes = 0;
#pragma unroll
  for (int ch = 0; ch < C; ++ch)
    if ((S.wmask >> ch) & 1u) wbytes |= 0xFFu << (8 * ch);
  int32_t exti[kStreamPx];
  float extf[kStreamPx];
  uint32_t outw[kStreamPx];
  for (int i = 0; i < items; ++i) {
    const int f = i % n, st = i % kStreamStages;
    if (f == 0) {
#pragma unroll
      for (int p = 0; p < kStreamPx; ++p) {
        exti[p] = darker ? 0x7FFFFFFF : -1;
        extf[p] = darker ? FLT_MAX : -FLT_MAX;
        outw[p] = 0u;
      }
    }
    const bool ok = mbar_wait(&full[st], static_cast<uint32_t>(i / kStreamStages) & 1u,
                              S.wait_cycles);
    if (__syncthreads_or(ok ? 0 : 1)) {
      if (error && threadIdx.x == 0) atomicOr(error, 1u);
      // every stage's copy in flight completes (bounded) before the CTA leaves
      for (int j = i; j < min(i + kStreamStages, items); ++j)
        mbar_wait(&full[j % kStreamStages], static_cast<uint32_t>(j / kStreamStages) & 1u);
      return;
    }
    uint32_t wv[NWD];
    const uint4* src = reinterpret_cast<const uint4*>(stage + st * kStreamStageBytes<C> +
                                                      threadIdx.x * (kStreamPx * C));
#pragma unroll
    for (int q = 0; q < C; ++q) {
      const uint4 v = src[q];
      wv[4 * q] = v.x;
      wv[4 * q + 1] = v.y;
      wv[4 * q + 2] = v.z;
      wv[4 * q + 3] = v.w;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      uint32_t sub[C];
#pragma unroll
      for (int k = 0; k < C; ++k) sub[k] = wv[q * C + k];
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        const int pp = q * 4 + p;
        const uint32_t px = pixel_word<C>(sub, p);
        if constexpr (FAST) {
          const int32_t v = static_cast<int32_t>(__dp4a(px & wbytes, 0x01010101u, 0u));
          const bool up = darker ? v < exti[pp] : v > exti[pp];
          exti[pp] = up ? v : exti[pp];
          outw[pp] = up ? px : outw[pp];
        } else {
          float value = 0.0f;
#pragma unroll
          for (int ch = 0; ch < C; ++ch)
            value = __fadd_rn(value, __fmul_rn(u8f((px >> (8 * ch)) & 0xFFu), S.w[ch]));
          const bool up = darker ? (value < extf[pp]) : (value > extf[pp]);
          extf[pp] = up ? value : extf[pp];
          const float fade = S.fade[f];
          if (up && fade > 0.0f)
            outw[pp] = fade >= 1.0f ? px : blend_into_u8<C>(outw[pp], px, fade);
        }
      }
    }
    if (f == n - 1) {  // the chunk's 16 pixels of this thread: C 16-byte words
      const int px = chunk_px0(i) + static_cast<int>(threadIdx.x) * kStreamPx;
      uint32_t ow[NWD];
#pragma unroll
      for (int k = 0; k < NWD; ++k) ow[k] = 0u;
#pragma unroll
      for (int pp = 0; pp < kStreamPx; ++pp)
#pragma unroll
        for (int ch = 0; ch < C; ++ch) {
          const int bb = pp * C + ch;
          ow[bb / 4] |= ((outw[pp] >> (8 * ch)) & 0xFFu) << (8 * (bb % 4));
        }
      uint8_t* dst = S.out + static_cast<size_t>(px) * C;
      if (px + kStreamPx <= S.px_end) {
#pragma unroll
        for (int q = 0; q < C; ++q)
          reinterpret_cast<uint4*>(dst)[q] =
              make_uint4(ow[4 * q], ow[4 * q + 1], ow[4 * q + 2], ow[4 * q + 3]);
      } else if (px < S.px_end) {
        const int valid = S.px_end - px;
#pragma unroll
        for (int pp = 0; pp < kStreamPx; ++pp)
          if (pp < valid) {
#pragma unroll
            for (int ch = 0; ch < C; ++ch) dst[pp * C + ch] = static_cast<uint8_t>(outw[pp] >> (8 * ch));
          }
      }
    }
    __syncthreads();  // stage st folded by every thread
    if (threadIdx.x == 0 && i + kStreamStages < items) {
      fence_proxy_async();
      issue(i + kStreamStages);
    }
  }
}
template <int C>
constexpr int kStreamSmem = 128 + kStreamStages * kStreamStageBytes<C>;

}  // namespace
}  // namespace cp
