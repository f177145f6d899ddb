// cp_outlier_multi.cuh — several outlier settings of one RGB stack in one pass.
//
// A caller that composites one stack under several settings (cp_composite_multi,
// cp_composite_device_multi: a threshold or outlier-mode sweep, or the six composites of one
// step of the benchmark) would otherwise run the whole pixel-thread kernel per setting:
// stage every frame row, build the bit planes and select the medians again, although those
// depend only on the stack and its (sub)sample. This kernel stages a tile once, builds the
// planes and the median pair (and the quartiles when a setting has a rel threshold) once
// per pixel, then runs each setting's distance pass and epilogue (cp_pixel.cuh) on the
// staged rows; a setting with the distance kind, threshold and weights of the one before
// reuses its outlier flags and extreme. Darker / lighter settings of the same stack fold the
// same staged rows (px_simple) instead of reading the stack again in their own launch. Each
// setting's outputs are what the single-setting kernels give it: the arithmetic per setting
// is the same code.
//
// A CTA has 4 warps, 128 pixels per tile as in k_outlier_px (warp 3 stages, warp p owns
// pixel p of every column); results are staged per setting in one of two shared-memory rows
// and stored coalesced after one barrier per setting.

#pragma once
#include "cp_internal.h"
#include "cp_pixel.cuh"

namespace cp {
namespace {

struct MultiAux {
  uint32_t out[2][3][32], blend[2][3][32];
};
static_assert(sizeof(MultiAux) <= sizeof(PxAux), "the multi kernel reuses px_smem_bytes");

template <int NW>
constexpr int kMultiMinCtas = NW == 4 ? 2 : 7;

template <int NW, bool REL>
__global__ void __launch_bounds__(kPxThreads, kMultiMinCtas<NW>)
    k_outlier_multi(const __grid_constant__ MultiArgs M, uint32_t* error) {
  constexpr int C = 3;
  const StackDev& S = M.sets[0];
  extern __shared__ __align__(128) uint8_t smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  uintptr_t* fbase = reinterpret_cast<uintptr_t*>(smem + 256);
  uint8_t* buf = smem + kSmemHeader;
  const int n = S.n;
  MultiAux& A = *reinterpret_cast<MultiAux*>(buf + 32 * NW * kPitch<C>);  // padded rows
  const int warp = static_cast<int>(threadIdx.x) >> 5;
  const int lane = static_cast<int>(threadIdx.x) & 31;
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  for (int f = threadIdx.x; f < n; f += kPxThreads)
    fbase[f] = reinterpret_cast<uintptr_t>(S.frames[f]);
  // the padding rows n..32*NW-1 stay zero: the copies write rows 0..n-1 only
  for (int i = threadIdx.x; i < (32 * NW - n) * (kPitch<C> / 4); i += kPxThreads)
    reinterpret_cast<uint32_t*>(buf + n * kPitch<C>)[i] = 0u;
  __syncthreads();
  uint32_t phase = 0;
  const int stride = static_cast<int>(gridDim.x);
  for (int tile = static_cast<int>(blockIdx.x); tile < S.tiles; tile += stride) {
    const TileGeo g = tile_geo(S, tile);
    if (warp == 3) {
      fence_proxy_async();
      issue_tile<C>(S, g, buf, nullptr, fbase, bar);
    }
    // bounded wait; the CTA leaves together if any wait gave up, once the copies in flight
    // into its shared memory have landed
    const bool ok = mbar_wait(bar, phase, S.wait_cycles);
    if (__syncthreads_or(ok ? 0 : 1)) {
      if (!ok) mbar_wait(bar, phase);
      if (error && threadIdx.x == 0) atomicOr(error, 1u);
      return;
    }
    phase ^= 1u;
    const int p = warp;
    const int pin = 4 * lane + p;
    const int pix_idx = g.out_px0 + pin;
    const int q0 = 3 * p, wa = q0 >> 2, sh = 8 * (q0 & 3);
    const uint32_t* col = reinterpret_cast<const uint32_t*>(buf) + 3 * lane + wa;
    auto load = [&](int i) -> uint32_t {
      const uint32_t* r = col + i * (kPitch<C> / 4);
      return __funnelshift_r(r[0], r[1], sh);
    };
    // order statistics of the pixel, shared by every setting
    uint32_t lo3, hi3;
    float iqr_inv[C];
    {
      uint32_t P[C][8][NW];
      pixel_planes<C, NW>(load, P);
      uint32_t smask[NW];
#pragma unroll
      for (int w = 0; w < NW; ++w) smask[w] = S.sample_mask[w];
      uint32_t q1a, q1b, q3a, q3b;
      pixel_ranks<C, NW, REL>(S, P, smask, REL, lo3, hi3, q1a, q1b, q3a, q3b);
      if (REL) {
        float q1[C], q3[C];
        quartiles_from_ranks<C>(S, q1a, q1b, q3a, q3b, q1, q3, iqr_inv);
      } else {
#pragma unroll
        for (int ch = 0; ch < C; ++ch) iqr_inv[ch] = 1.0f;
      }
    }
    uint32_t pb[NW];
#pragma unroll
    for (int w = 0; w < NW; ++w) pb[w] = 0u;
    int32_t key = -1;
    float dmax = 0.0f;
    int imax = 0;
    uint32_t carried = 0u;  // the second result of a darker / lighter pair
    bool have_carried = false;
    for (int s = 0; s < M.count; ++s) {
      const StackDev& T = M.sets[s];
      PxOut r;
      if (T.mode != CP_MODE_OUTLIER) {  // darker / lighter on the same staged rows
        r.mask = 0u;
        r.warning = false;
        if (have_carried) {
          r.pix = carried;
          have_carried = false;
        } else if (s + 1 < M.count && M.sets[s + 1].mode != CP_MODE_OUTLIER &&
                   M.sets[s + 1].mode != T.mode && T.unit_w && T.no_fade &&
                   M.sets[s + 1].unit_w && M.sets[s + 1].no_fade &&
                   M.sets[s + 1].wmask == T.wmask) {
          uint32_t dark, light;
          px_simple_pair<C>(T, n, load, dark, light);
          const bool d = T.mode == CP_MODE_DARKER;
          r.pix = d ? dark : light;
          carried = d ? light : dark;
          have_carried = true;
        } else {
          r.pix = px_simple<C>(T, n, load);
        }
      } else {
        uint32_t wbytes = 0;
#pragma unroll
        for (int ch = 0; ch < C; ++ch)
          if ((T.wmask >> ch) & 1u) wbytes |= 0xFFu << (8 * ch);
        float wq[C];
#pragma unroll
        for (int ch = 0; ch < C; ++ch)
          wq[ch] = T.thr_abs ? 0.0f : __fmul_rn(T.w[ch], iqr_inv[ch]);
        const PxStat<C> st = px_stat<C>(T, lo3, hi3, wq);
        if (!M.share_dist[s])
          px_distance<C, NW, kPxKind, kOgAny>(T, n, st, wbytes, load, pb, key, dmax, imax);
        r = px_epilogue<C, NW, kPxKind, kOgAny, kBgAny>(T, n, st, wbytes, pb, key, dmax, imax,
                                                         pix_idx, nullptr, load);
      }
      const int b = s & 1;
      uint8_t* ob = reinterpret_cast<uint8_t*>(A.out[b]);
      uint8_t* bb = reinterpret_cast<uint8_t*>(A.blend[b]);
#pragma unroll
      for (int ch = 0; ch < C; ++ch) {
        const int q = q0 + ch;
        const int off = 4 * (32 * (q >> 2) + lane) + (q & 3);
        ob[off] = static_cast<uint8_t>(r.pix >> (8 * ch));
        bb[off] = static_cast<uint8_t>(r.mask);
      }
      const uint32_t wm = __ballot_sync(0xFFFFFFFFu, r.warning && pin < g.npx);
      if (lane == 0 && wm && T.warnings)
        atomicAdd(T.warnings, static_cast<unsigned long long>(__popc(wm)));
      // the setting's rows are complete; the other row buffer was last read before this
      // barrier, so the next setting may write it while these rows are stored
      __syncthreads();
      store_rows<C>(T.out, g, A.out[b]);
      if (T.blend) store_rows<C>(T.blend, g, A.blend[b]);
    }
  }
}

template <int NW, bool REL>
int multi_launch_t(const MultiArgs& a, int grid, int smem, void* stream, uint32_t* error) {
  const void* fn = reinterpret_cast<const void*>(&k_outlier_multi<NW, REL>);
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  k_outlier_multi<NW, REL><<<grid, kPxThreads, smem, static_cast<cudaStream_t>(stream)>>>(a, error);
  return static_cast<int>(cudaGetLastError());
}
template <int NW, bool REL>
int multi_occupancy_t(int smem) {
  const void* fn = reinterpret_cast<const void*>(&k_outlier_multi<NW, REL>);
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, kPxThreads, smem) != cudaSuccess)
    return 1;
  return blocks < 1 ? 1 : blocks;
}

}  // namespace
}  // namespace cp
