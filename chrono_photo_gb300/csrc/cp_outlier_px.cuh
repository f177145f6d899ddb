// cp_outlier_px.cuh — the single-stack outlier kernel with one thread per pixel after the
// order statistics (RGB stacks whose frame rows start 16-byte aligned, no crop).
//
// A tile is 128 consecutive pixels: 32 columns of 4 pixels, 3 words per column and frame.
// A CTA has 4 warps:
//   - warp 3 stages the tile with one cp.async.bulk per frame row (TMA engine) into shared
//     memory, completing on an mbarrier (optionally double buffered: the CTA's next tile is
//     staged while the current one is processed);
//   - phase A, warps 0..2: bit planes and radix selections of word w of every column (the tile
//     kernel's word_order_stats); d[k], d[k+1] (and w * iqr_inv for rel thresholds) go to a
//     small shared-memory exchange area;
//   - one CTA barrier; phases B and C, warp p: pixel p of every column, one thread per pixel,
//     the distance pass over all samples and the epilogue (cp_pixel.cuh), with no further
//     exchange between warps and no per-pixel imbalance (four pixels, four warps);
//   - one CTA barrier; the tile's composite and mask rows are stored coalesced.
// The tile kernel (cp_tile.cuh) splits the distance pass by frame class across its 3 warps
// and the epilogue by pixel over 3 warps (4 pixels per column), with two more barriers and
// an exchange of flags per frame class; this kernel replaces it for the stacks above.

#pragma once
#include "cp_internal.h"
#include "cp_pixel.cuh"

namespace cp {
namespace {

// CTAs per SM the register allocation is made for. Per-pixel phase A (PA 2) fits 72
// registers without spills at two plane words, so 7 CTAs (the shared-memory limit of a
// 64-frame tile) are resident; the word-column layout needs 96 (5 CTAs).
template <int NW, bool DB, int PA>
constexpr int kPxMinCtas = NW == 1 ? 6 : (NW == 2 ? (DB ? 4 : (PA == 2 ? 7 : 5)) : 2);

// PA: how phase A runs. 0: warps 0..2, word per lane, 4 byte positions per selection round;
// 1: the same with 2 byte positions per round (fewer registers); 2: every warp builds the
// planes of its own pixel's samples (no exchange, no idle warp, a quarter of each transpose
// unused).
template <int KIND, int OG, int BG, int NW, bool DB, int PA = 0>
__global__ void __launch_bounds__(kPxThreads, (kPxMinCtas<NW, DB, PA>))
    k_outlier_px(const __grid_constant__ StackDev S, uint32_t* error) {
  constexpr int C = 3;
  extern __shared__ __align__(128) uint8_t smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);  // one per stage buffer
  uintptr_t* fbase = reinterpret_cast<uintptr_t*>(smem + 256);
  uint8_t* stage0 = smem + kSmemHeader;
  const int n = S.n;
  const int stage_bytes = 32 * NW * kPitch<C>;  // rows padded to whole words (px_stage_rows)
  PxAux& A = *reinterpret_cast<PxAux*>(stage0 + (DB ? 2 : 1) * stage_bytes);
  const int warp = static_cast<int>(threadIdx.x) >> 5;
  const int lane = static_cast<int>(threadIdx.x) & 31;
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
  }
  for (int f = threadIdx.x; f < n; f += kPxThreads)
    fbase[f] = reinterpret_cast<uintptr_t>(S.frames[f]);
  // the padding rows n..32*NW-1 stay zero: the copies write rows 0..n-1 only
  for (int b = 0; b < (DB ? 2 : 1); ++b) {
    uint32_t* z = reinterpret_cast<uint32_t*>(stage0 + b * stage_bytes + n * kPitch<C>);
    for (int i = threadIdx.x; i < (32 * NW - n) * (kPitch<C> / 4); i += kPxThreads) z[i] = 0u;
  }
  if (threadIdx.x < 32) {
    A.lo[3][lane] = 0u;
    A.hi[3][lane] = 0u;
  }
  __syncthreads();
  uint32_t wbytes = 0;
#pragma unroll
  for (int ch = 0; ch < C; ++ch)
    if ((S.wmask >> ch) & 1u) wbytes |= 0xFFu << (8 * ch);
  uint32_t phase0 = 0, phase1 = 0, warn = 0;
  const int stride = static_cast<int>(gridDim.x);
  int tile = static_cast<int>(blockIdx.x);
  if (DB && tile < S.tiles && warp == 3) {
    fence_proxy_async();
    issue_tile<C>(S, tile_geo(S, tile), stage0, nullptr, fbase, &bars[0]);
  }
  for (int it = 0; tile < S.tiles; tile += stride, ++it) {
    const int b = DB ? (it & 1) : 0;
    uint8_t* buf = stage0 + b * stage_bytes;
    const TileGeo g = tile_geo(S, tile);
    bool next_issued = false;
    if (warp == 3) {
      if (!DB) {
        fence_proxy_async();
        issue_tile<C>(S, g, buf, nullptr, fbase, &bars[0]);
      } else if (tile + stride < S.tiles) {
        fence_proxy_async();
        issue_tile<C>(S, tile_geo(S, tile + stride), stage0 + (b ^ 1) * stage_bytes, nullptr,
                      fbase, &bars[b ^ 1]);
        next_issued = true;
      }
    }
    uint32_t& ph = b ? phase1 : phase0;
    // bounded wait; every thread of the CTA leaves together if any wait gave up, once the
    // copies in flight into its shared memory have landed
    const bool ok = mbar_wait(&bars[b], ph, S.wait_cycles);
    if (__syncthreads_or(ok ? 0 : 1)) {
      if (!ok) mbar_wait(&bars[b], ph);
      if (error && threadIdx.x == 0) atomicOr(error, 1u);
      if (DB && next_issued) mbar_wait(&bars[b ^ 1], b ? phase0 : phase1);
      return;
    }
    ph ^= 1u;
    // phase A: order statistics of word `warp` of every column
    if (PA != 2) {
      if (warp < 3) {
        const Rows<C, false> rd{buf + 4 * C * lane, nullptr};
        uint32_t plo, phi;
        float wq[4];
        word_order_stats<C, NW, false, KIND, (PA == 1 ? 2 : (NW <= 2 ? 4 : 2))>(
            S, g, rd, warp, lane, plo, phi, wq);
        A.lo[warp][lane] = plo;
        A.hi[warp][lane] = phi;
        if (!S.thr_abs) {
#pragma unroll
          for (int k = 0; k < 4; ++k) A.wq[4 * warp + k][lane] = wq[k];
        }
      }
      __syncthreads();
    }
    // phases B and C: pixel `warp` of column `lane`
    {
      const int p = warp;
      const int pin = 4 * lane + p;
      const int pix_idx = g.out_px0 + pin;
      const int q0 = 3 * p, wa = q0 >> 2, sh = 8 * (q0 & 3);
      // sample i of this pixel: bytes 12 * lane + 3 * p of row i (byte 3 unspecified)
      const uint32_t* col = reinterpret_cast<const uint32_t*>(buf) + 3 * lane + wa;
      auto load = [&](int i) -> uint32_t {
        const uint32_t* r = col + i * (kPitch<C> / 4);
        return __funnelshift_r(r[0], r[1], sh);
      };
      uint32_t lo3, hi3;
      float wq3[C];
      if (PA == 2) {
        float q1v[C], q3v[C];
        pixel_order_stats<C, NW, KIND>(S, load, lo3, hi3, wq3, q1v, q3v);
        if (pin < g.npx && (S.dbg_q1 || S.dbg_q3)) {
#pragma unroll
          for (int ch = 0; ch < C; ++ch) {
            const size_t o = static_cast<size_t>(pix_idx) * C + ch;
            if (S.dbg_q1) S.dbg_q1[o] = q1v[ch];
            if (S.dbg_q3) S.dbg_q3[o] = q3v[ch];
          }
        }
      } else {
        lo3 = __funnelshift_r(A.lo[wa][lane], A.lo[wa + 1][lane], sh) & 0x00FFFFFFu;
        hi3 = __funnelshift_r(A.hi[wa][lane], A.hi[wa + 1][lane], sh) & 0x00FFFFFFu;
#pragma unroll
        for (int ch = 0; ch < C; ++ch) wq3[ch] = S.thr_abs ? 0.0f : A.wq[q0 + ch][lane];
      }
      const PxStat<C> st = px_stat<C>(S, lo3, hi3, wq3);
      uint32_t pb[NW];
      int32_t key;
      float dmax;
      int imax;
      px_distance<C, NW, KIND, OG>(S, n, st, wbytes, load, pb, key, dmax, imax);
      const PxOut r = px_epilogue<C, NW, KIND, OG, BG>(S, n, st, wbytes, pb, key, dmax, imax,
                                                       pix_idx, nullptr, load);
      uint8_t* ob = reinterpret_cast<uint8_t*>(A.out);
      uint8_t* bb = reinterpret_cast<uint8_t*>(A.blend);
#pragma unroll
      for (int ch = 0; ch < C; ++ch) {
        const int q = q0 + ch;
        const int off = 4 * (32 * (q >> 2) + lane) + (q & 3);
        ob[off] = static_cast<uint8_t>(r.pix >> (8 * ch));
        bb[off] = static_cast<uint8_t>(r.mask);
      }
      if (pin < g.npx) {
        if (r.warning) warn += 1;
        if (S.dbg_median) {
#pragma unroll
          for (int ch = 0; ch < C; ++ch)
            S.dbg_median[static_cast<size_t>(pix_idx) * C + ch] = st.med[ch];
        }
        if (S.dbg_bits) {
          const int words = (n + 31) / 32;
#pragma unroll
          for (int w = 0; w < NW; ++w)
            if (w < words) S.dbg_bits[static_cast<size_t>(pix_idx) * words + w] = pb[w];
        }
        if (S.dbg_chosen) S.dbg_chosen[pix_idx] = r.chosen;
        if (S.dbg_bg) S.dbg_bg[pix_idx] = r.bg_idx;
        if (S.dbg_nout) S.dbg_nout[pix_idx] = r.nout;
      }
    }
    __syncthreads();
    store_rows<C>(S.out, g, A.out);
    if (S.blend) store_rows<C>(S.blend, g, A.blend);
  }
  flush_warnings(S.warnings, warn);
}

// Static phase-A choice (what the autotuner starts from): per-pixel planes for every kind.
// Measured on the 64 x 1080p stack with 7 CTAs per SM against the word-column layout's 5:
// abs average 0.278 vs 0.288 ms, rel average 0.451 vs 0.496 ms (whose six selections per
// channel spill in the word-column layout).
template <int KIND>
constexpr int kPxPhaseA = 2;

template <int KIND, int OG, int BG, int NW, bool DB, int PA>
int px_launch_t(const StackDev& s, int grid, int smem, void* stream, uint32_t* error) {
  const void* fn = reinterpret_cast<const void*>(&k_outlier_px<KIND, OG, BG, NW, DB, PA>);
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  k_outlier_px<KIND, OG, BG, NW, DB, PA>
      <<<grid, kPxThreads, smem, static_cast<cudaStream_t>(stream)>>>(s, error);
  return static_cast<int>(cudaGetLastError());
}
template <int KIND, int OG, int BG, int NW, bool DB, int PA>
int px_occupancy_t(int smem) {
  const void* fn = reinterpret_cast<const void*>(&k_outlier_px<KIND, OG, BG, NW, DB, PA>);
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, kPxThreads, smem) != cudaSuccess)
    return 1;
  return blocks < 1 ? 1 : blocks;
}

// Launch (occupancy_only: CTAs per SM instead) of the variant for s.nw, phase-A mode pa
// (0 word-column, 2 per-pixel; -1 the static choice of the kind) and staging buffers db.
template <int KIND, int OG, int BG>
int px_dispatch(const StackDev& s, int pa, bool db, bool occupancy_only, int grid, int smem,
                void* stream, uint32_t* error) {
  if (pa < 0) pa = kPxPhaseA<KIND>;
#define CP_PX_CASE(NW, DBV, PAV)                                                          \
  if (s.nw == NW && db == DBV && pa == PAV)                                               \
    return occupancy_only                                                                 \
               ? px_occupancy_t<KIND, OG, BG, NW, DBV, PAV>(smem)                         \
               : px_launch_t<KIND, OG, BG, NW, DBV, PAV>(s, grid, smem, stream, error);
  CP_PX_CASE(1, false, 0)
  CP_PX_CASE(1, false, 2)
  CP_PX_CASE(1, true, 0)
  CP_PX_CASE(1, true, 2)
  CP_PX_CASE(2, false, 0)
  CP_PX_CASE(2, false, 2)
  CP_PX_CASE(2, true, 0)
  CP_PX_CASE(2, true, 2)
  CP_PX_CASE(4, false, 0)
  CP_PX_CASE(4, false, 2)
#undef CP_PX_CASE
  return -1;
}

}  // namespace
}  // namespace cp
