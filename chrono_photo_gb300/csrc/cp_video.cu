// cp_video.cu — chrono-video windows that slide by one frame, with work shared between
// overlapping windows.
//
// create_video (src/main.rs:214-331) composites one window of frames per output frame; with
// `--video-in` step 1 consecutive windows [f, f+L) and [f+1, f+L+1) share L-1 frames. The
// reference (and the batched kernel) recompute each window from scratch: decode, sort and
// select every pixel's L samples again. Here one warp owns a tile of 32 consecutive pixels
// (one pixel per lane) and walks it through every window of the call:
//   - the tile's frame rows stream through a ring of L + kVideoPF shared-memory rows
//     (16-byte cp.async copies issued kVideoPF windows ahead), each frame read from HBM once
//     per tile instead of once per window;
//   - each lane keeps a 256-bin count histogram per channel of its pixel's current window in
//     shared memory and the order statistics d[k] (and d[k+1] of an even-length window) as
//     (value, count below) pointers; sliding the window removes one sample and adds one, and
//     each pointer walks to its new value over the histogram (one or two bins for a slowly
//     changing background) instead of a fresh selection over L samples;
//   - the distance pass, outlier flags and the per-pixel epilogue (background, outlier pick,
//     blend, blend mask) run per window with the integer arithmetic of the plain kernel.
// Every result equals what the single-stack kernel gives the same window: the order
// statistics are exact (a histogram of the window's samples), and the rest is the same code
// path (src/chrono.rs:208-494).

#include <cuda_runtime.h>

#include "../../include/chrono_gpu.h"
#include "cp_internal.h"
#include "cp_tile.cuh"

namespace cp {
namespace {

constexpr int kVC = 3;                      // channels of the sliding kernel (RGB)
constexpr int kVideoPF = 4;                 // frame rows in flight ahead of the window
constexpr int kVideoRowPitch = 112;         // 96 bytes of a 32-pixel RGB row + read slack
constexpr int kVideoHistBytes = kVC * 64 * 32 * 4;  // [channel][bin / 4][lane] words

DEVI void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src)
               : "memory");
}
DEVI void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
DEVI void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// The lane's RGB pixel of a staged 32-pixel row (bytes 3*lane .. 3*lane+2).
DEVI uint32_t row_pixel(const uint8_t* row, int lane) {
  const int b = 3 * lane;
  const uint32_t* w = reinterpret_cast<const uint32_t*>(row) + (b >> 2);
  return __funnelshift_r(w[0], w[1], 8 * (b & 3)) & 0x00FFFFFFu;
}

// Histogram bin v of channel c of this lane (bank = lane: conflict-free).
DEVI uint32_t* hist_word(uint32_t* hist, int lane, int c, uint32_t v) {
  return hist + ((c * 64 + static_cast<int>(v >> 2)) * 32 + lane);
}
DEVI int hist_count(uint32_t* hist, int lane, int c, int v) {
  return static_cast<int>((*hist_word(hist, lane, c, static_cast<uint32_t>(v)) >> (8 * (v & 3))) &
                          0xFFu);
}
// inc = 1 adds the sample, inc = 0xFFFFFFFF removes it (the bin holds it, so no borrow).
DEVI void hist_update(uint32_t* hist, int lane, int c, uint32_t v, uint32_t inc) {
  uint32_t* p = hist_word(hist, lane, c, v);
  *p += inc << (8 * (v & 3));
}

// Moves the pointer (value m, samples below m = b) to the order statistic of rank kk:
// b <= kk < b + count(m). Bounded: a histogram holding kk + 1 or more samples stops it inside
// [0, 255]; anything else sets `bad`.
DEVI void walk(uint32_t* hist, int lane, int c, int kk, int& m, int& b, bool& bad) {
  int guard = 0;
  while (b > kk && m > 0 && guard < 256) {
    --m;
    b -= hist_count(hist, lane, c, m);
    ++guard;
  }
  int h = hist_count(hist, lane, c, m);
  while (b + h <= kk && m < 255 && guard < 512) {
    b += h;
    ++m;
    h = hist_count(hist, lane, c, m);
    ++guard;
  }
  if (b > kk || b + h <= kk) bad = true;
}

template <int OG, int BG, int NW>
__global__ void __launch_bounds__(32, 8) k_video_slide(const __grid_constant__ VideoArgs A,
                                                        uint32_t* error) {
  constexpr int C = kVC;
  extern __shared__ __align__(128) uint8_t smem[];
  const StackDev& S = A.S;
  const int n = S.n;
  const int R = n + kVideoPF;
  const int lane = static_cast<int>(threadIdx.x);
  uint32_t* hist = reinterpret_cast<uint32_t*>(smem);
  uint8_t* ring = smem + kVideoHistBytes;
  uint8_t* stage = ring + R * kVideoRowPitch;
  const int kl = S.med_k;                    // d[k] (and d[k+1] of a pair)
  const int kh = S.med_k + (S.med_pair ? 1 : 0);
  uint32_t wbytes = 0;
#pragma unroll
  for (int ch = 0; ch < C; ++ch)
    if ((S.wmask >> ch) & 1u) wbytes |= 0xFFu << (8 * ch);
  bool bad = false;

  for (int tile = blockIdx.x; tile < A.tiles; tile += gridDim.x) {
    const int px0 = tile * 32;
    const int npx = min(32, A.npx - px0);
    const int nbytes = npx * C;
    const size_t src_off = static_cast<size_t>(px0) * C;
    // prologue: frame rows 0 .. R-1 into ring slots 0 .. R-1, one copy group per row
    __syncwarp();
    for (int r = 0; r < R; ++r) {
      if (r < A.n_rows && lane * 16 < nbytes)
        cp_async16(ring + r * kVideoRowPitch + lane * 16, A.rows[r] + src_off + lane * 16);
      cp_async_commit();
    }
    for (int j = 0; j < C * 64; ++j) hist[j * 32 + lane] = 0u;
    cp_async_wait<0>();
    __syncwarp();
    // the first window: histogram, running sums, and the pointers started at frame 0's value
    int ml[C], bl[C], mh[C], bh[C];
    uint32_t sum[C];
    {
      const uint32_t p0 = row_pixel(ring, lane);
#pragma unroll
      for (int ch = 0; ch < C; ++ch) {
        ml[ch] = static_cast<int>((p0 >> (8 * ch)) & 0xFFu);
        bl[ch] = 0;
        sum[ch] = 0u;
      }
      for (int i = 0; i < n; ++i) {
        const uint32_t px = row_pixel(ring + i * kVideoRowPitch, lane);
#pragma unroll
        for (int ch = 0; ch < C; ++ch) {
          const uint32_t v = (px >> (8 * ch)) & 0xFFu;
          hist_update(hist, lane, ch, v, 1u);
          bl[ch] += static_cast<int>(v) < ml[ch] ? 1 : 0;
          sum[ch] += v;
        }
      }
#pragma unroll
      for (int ch = 0; ch < C; ++ch) {
        mh[ch] = ml[ch];
        bh[ch] = bl[ch];
        walk(hist, lane, ch, kl, ml[ch], bl[ch], bad);
        walk(hist, lane, ch, kh, mh[ch], bh[ch], bad);
      }
    }
    for (int k = 0; k < A.n_win; ++k) {
      const int head = k % R;  // ring slot of the window's first frame
      if (k > 0) {
        // slide: drop row k-1 (slot of the previous head), add row k+n-1
        const int old = head == 0 ? R - 1 : head - 1;
        const uint32_t xo = row_pixel(ring + old * kVideoRowPitch, lane);
        __syncwarp();  // every lane has read the slot before it is refilled
        const int nr = k - 1 + R;
        if (nr < A.n_rows && lane * 16 < nbytes)
          cp_async16(ring + old * kVideoRowPitch + lane * 16, A.rows[nr] + src_off + lane * 16);
        cp_async_commit();
        cp_async_wait<kVideoPF>();
        __syncwarp();
        int in_slot = head + n - 1;
        if (in_slot >= R) in_slot -= R;
        const uint32_t xi = row_pixel(ring + in_slot * kVideoRowPitch, lane);
#pragma unroll
        for (int ch = 0; ch < C; ++ch) {
          const int vo = static_cast<int>((xo >> (8 * ch)) & 0xFFu);
          const int vi = static_cast<int>((xi >> (8 * ch)) & 0xFFu);
          hist_update(hist, lane, ch, static_cast<uint32_t>(vo), 0xFFFFFFFFu);
          hist_update(hist, lane, ch, static_cast<uint32_t>(vi), 1u);
          bl[ch] += (vi < ml[ch] ? 1 : 0) - (vo < ml[ch] ? 1 : 0);
          bh[ch] += (vi < mh[ch] ? 1 : 0) - (vo < mh[ch] ? 1 : 0);
          sum[ch] += static_cast<uint32_t>(vi) - static_cast<uint32_t>(vo);
          walk(hist, lane, ch, kl, ml[ch], bl[ch], bad);
          walk(hist, lane, ch, kh, mh[ch], bh[ch], bad);
        }
      }
      // per-pixel statistics (pixel_stats of the tile kernel): floor / ceil of the medians
      uint32_t klo = 0u, khi = 0u;
      int nh = 0;
      float med[C];
#pragma unroll
      for (int ch = 0; ch < C; ++ch) {
        const bool wt = (S.wmask >> ch) & 1u;
        const uint32_t lo = static_cast<uint32_t>(ml[ch]), hi = static_cast<uint32_t>(mh[ch]);
        med[ch] = !wt ? 0.0f
                      : (S.med_pair ? __fmul_rn(0.5f, __fadd_rn(static_cast<float>(lo),
                                                                static_cast<float>(hi)))
                                    : static_cast<float>(lo));
        const uint32_t s2 = lo + hi;
        const uint32_t fl = S.med_pair ? (s2 >> 1) : lo, ce = S.med_pair ? ((s2 + 1) >> 1) : lo;
        if (wt) {
          klo |= fl << (8 * ch);
          khi |= ce << (8 * ch);
          nh += static_cast<int>(ce - fl);
        }
      }
      // distance pass over the window, earliest sample first (src/chrono.rs:257-288)
      const int32_t thr = S.thr_int[nh];
      uint32_t pb[NW];
      int32_t key = nh > 0 ? -1 : 255;
#pragma unroll
      for (int blk = 0; blk < NW; ++blk) {
        uint32_t ob = 0u;
        const int iend = min(n, blk * 32 + 32);
        int slot = head + blk * 32;
        if (slot >= R) slot -= R;
        for (int i = blk * 32; i < iend; ++i) {
          const uint32_t px = row_pixel(ring + slot * kVideoRowPitch, lane);
          slot = slot + 1 == R ? 0 : slot + 1;
          const int32_t d = static_cast<int32_t>(dist_int(px, wbytes, klo, khi));
          ob |= d >= thr ? (1u << (i & 31)) : 0u;
          if (OG == kOgSingle) key = max(key, (d << 8) + 255 - i);
        }
        pb[blk] = ob;
      }
      auto sample = [&](int i) -> uint32_t {
        int s = head + i;
        if (s >= R) s -= R;
        return row_pixel(ring + s * kVideoRowPitch, lane);
      };
      auto dsq_px = [&](uint32_t px) -> float {
        return static_cast<float>(dist_int(px, wbytes, klo, khi)) + 0.25f * static_cast<float>(nh);
      };
      int nout = 0;
#pragma unroll
      for (int w = 0; w < NW; ++w) nout += __popc(pb[w]);
      const int pix_idx = px0 + lane;
      const int bgm = BG == kBgFirst ? CP_BG_FIRST : S.background;
      bool warning = false;
      uint32_t pix = 0;
      // background, src/chrono.rs:293-375
      if (bgm == CP_BG_FIRST || bgm == CP_BG_RANDOM) {
        int bg_idx;
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
            // sample_excluded, src/chrono.rs:531-555 (see the tile kernel)
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
        pix = sample(bg_idx);
      } else if (bgm == CP_BG_AVERAGE) {
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
              const uint32_t px = sample(32 * w + bpos);
#pragma unroll
              for (int ch = 0; ch < C; ++ch) osum[ch] += (px >> (8 * ch)) & 0xFFu;
            }
          }
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
        for (int ch = 0; ch < C; ++ch) pix |= sat_u8(rround(med[ch])) << (8 * ch);
      }
      // outlier pick and blend, src/chrono.rs:377-493
      float blend = 0.0f;
      uint32_t mask = 0;
      const bool single_group = og_is<OG>(S, kOgSingle);
      const bool blend_group = og_is<OG>(S, kOgBlend);
      const bool extreme = single_group && S.outlier == CP_OUTLIER_EXTREME;
      const bool multi = nout > 1 && !single_group;
      if (!multi) {
        int si;
        float dsq = 0.0f;
        if (extreme) {
          si = key < 0 ? 0 : 255 - (key & 255);
          const int32_t dm = key < 0 ? -1 : (key >> 8);
          dsq = dm < 0 ? 0.0f : static_cast<float>(dm) + 0.25f * static_cast<float>(nh);
        } else {
          si = (single_group && S.outlier == CP_OUTLIER_LAST) ? last_set<NW>(pb)
                                                              : first_set<NW>(pb);
          si = si < 0 ? 0 : si;
        }
        const uint32_t smp = sample(si);
        if (!extreme) dsq = dsq_px(smp);
        blend = nout == 0 ? 0.0f : __fmul_rn(S.fade[si], blend_value(S, __fsqrt_rn(dsq)));
        pix = blend_into_u8<C>(pix, smp, blend);
        mask = sat_u8(rround(__fmul_rn(blend, 255.0f)));
      } else if (blend_group) {
        float pf[C];
#pragma unroll
        for (int ch = 0; ch < C; ++ch) pf[ch] = static_cast<float>((pix >> (8 * ch)) & 0xFFu);
        float binv = 1.0f;
        auto blend_one = [&](int f) {
          const uint32_t sv = sample(f);
          const float bk = __fmul_rn(S.fade[f], blend_value(S, __fsqrt_rn(dsq_px(sv))));
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
      } else {  // average of several outliers, src/chrono.rs:429-468
        uint32_t se = 0u, so = 0u;
        float mdist = 0.0f;
#pragma unroll
        for (int w = 0; w < NW; ++w) {
          uint32_t m = pb[w];
          while (m) {
            const int f = 32 * w + __ffs(m) - 1;
            m &= m - 1;
            const uint32_t px = sample(f);
            se += px & 0x00FF00FFu;
            so += (px >> 8) & 0x00FF00FFu;
            mdist = __fadd_rn(mdist, __fsqrt_rn(dsq_px(px)));
          }
        }
        const float kf = static_cast<float>(nout);
        uint32_t smp = 0;
#pragma unroll
        for (int ch = 0; ch < C; ++ch) {
          const uint32_t os = ((ch & 1) ? so : se) >> (16 * (ch >> 1)) & 0xFFFFu;
          smp |= sat_u8(rround(__fdiv_rn(static_cast<float>(os), kf))) << (8 * ch);
        }
        // the fade of an averaged outlier is taken at sample 0 (src/chrono.rs:467)
        blend = __fmul_rn(S.fade[0], blend_value(S, __fdiv_rn(mdist, kf)));
        pix = blend_into_u8<C>(pix, smp, blend);
        mask = sat_u8(rround(__fmul_rn(blend, 255.0f)));
      }
      // stage the composite and mask bytes, then store the rows coalesced
      __syncwarp();
#pragma unroll
      for (int ch = 0; ch < C; ++ch) {
        stage[3 * lane + ch] = static_cast<uint8_t>(pix >> (8 * ch));
        stage[kVideoRowPitch + 3 * lane + ch] = static_cast<uint8_t>(mask);
      }
      __syncwarp();
      uint8_t* out = A.outs[k] + src_off;
      uint8_t* bl_out = A.blends[k] ? A.blends[k] + src_off : nullptr;
      const bool full = nbytes == 32 * C && (reinterpret_cast<uintptr_t>(out) & 3) == 0 &&
                        (!bl_out || (reinterpret_cast<uintptr_t>(bl_out) & 3) == 0);
      if (full) {
        if (lane < 8 * C) {
          reinterpret_cast<uint32_t*>(out)[lane] = reinterpret_cast<const uint32_t*>(stage)[lane];
          if (bl_out)
            reinterpret_cast<uint32_t*>(bl_out)[lane] =
                reinterpret_cast<const uint32_t*>(stage + kVideoRowPitch)[lane];
        }
      } else {
        for (int b = lane; b < nbytes; b += 32) {
          out[b] = stage[b];
          if (bl_out) bl_out[b] = stage[kVideoRowPitch + b];
        }
      }
      if (A.warnings) {
        const uint32_t wm = __ballot_sync(0xFFFFFFFFu, warning && lane < npx);
        if (lane == 0 && wm) atomicAdd(A.warnings + k, static_cast<unsigned long long>(__popc(wm)));
      }
    }
    cp_async_wait<0>();  // no copy of this tile is in flight when the ring is reused
    __syncwarp();
  }
  if (bad && error) atomicOr(error, 2u);
}

}  // namespace

int video_smem_bytes(int n) {
  return kVideoHistBytes + (n + kVideoPF) * kVideoRowPitch + 2 * kVideoRowPitch;
}

template <int OG, int BG, int NW>
static int video_launch_t(const VideoArgs& a, int grid, int smem, void* stream, uint32_t* error) {
  const void* fn = reinterpret_cast<const void*>(&k_video_slide<OG, BG, NW>);
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  k_video_slide<OG, BG, NW><<<grid, 32, smem, static_cast<cudaStream_t>(stream)>>>(a, error);
  return static_cast<int>(cudaGetLastError());
}
template <int OG, int BG, int NW>
static int video_occupancy_t(int smem) {
  const void* fn = reinterpret_cast<const void*>(&k_video_slide<OG, BG, NW>);
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, 32, smem) != cudaSuccess)
    return 1;
  return blocks < 1 ? 1 : blocks;
}

template <int OG, int BG>
static int video_dispatch_nw(const VideoArgs& a, int nw, bool occupancy_only, int grid, int smem,
                             void* stream, uint32_t* error) {
  switch (nw) {
    case 1: return occupancy_only ? video_occupancy_t<OG, BG, 1>(smem)
                                  : video_launch_t<OG, BG, 1>(a, grid, smem, stream, error);
    case 2: return occupancy_only ? video_occupancy_t<OG, BG, 2>(smem)
                                  : video_launch_t<OG, BG, 2>(a, grid, smem, stream, error);
    default: return occupancy_only ? video_occupancy_t<OG, BG, 4>(smem)
                                   : video_launch_t<OG, BG, 4>(a, grid, smem, stream, error);
  }
}

// One launch of the sliding kernel (occupancy_only: CTAs per SM instead). The outlier group
// and background pick the specialised kernel as for the single-stack kernels.
int video_slide(const void* args, int og, int bg_first, bool occupancy_only, int grid, int smem,
                void* stream, uint32_t* error) {
  const VideoArgs& a = *static_cast<const VideoArgs*>(args);
  const int nw = a.S.nw;
  if (bg_first) {
    if (og == 1) return video_dispatch_nw<kOgSingle, kBgFirst>(a, nw, occupancy_only, grid, smem, stream, error);
    if (og == 2) return video_dispatch_nw<kOgAverage, kBgFirst>(a, nw, occupancy_only, grid, smem, stream, error);
    return video_dispatch_nw<kOgBlend, kBgFirst>(a, nw, occupancy_only, grid, smem, stream, error);
  }
  if (og == 1) return video_dispatch_nw<kOgSingle, kBgAny>(a, nw, occupancy_only, grid, smem, stream, error);
  if (og == 2) return video_dispatch_nw<kOgAverage, kBgAny>(a, nw, occupancy_only, grid, smem, stream, error);
  return video_dispatch_nw<kOgBlend, kBgAny>(a, nw, occupancy_only, grid, smem, stream, error);
}

size_t video_args_bytes() { return sizeof(VideoArgs); }

}  // namespace cp
