// cp_video.cu — chrono-video windows that slide by one frame, with work shared between
// overlapping windows.
//
// create_video (src/main.rs:214-331) composites one window of frames per output frame; with
// `--video-in` step 1, consecutive windows [f, f+L) and [f+1, f+L+1) share L-1 frames. The
// reference (and the batched kernel) recompute each window from scratch: read every frame
// of the window, build the order statistics of every pixel's L samples. Here one warp owns a
// tile of 32 consecutive pixels (one pixel per lane) and walks it through every window of the
// call:
//   - the tile's frame rows stream through a small ring of shared-memory rows (16-byte
//     cp.async copies issued kVideoPF frames ahead), each frame read from HBM once per tile
//     instead of once per window; each lane keeps its pixel's L samples in a shared-memory
//     ring of words, every frame stored twice (slots s and s + L), so that the window is L
//     consecutive slots and sample i one load at a fixed offset from the window's first;
//   - each lane keeps the bit planes of its pixel's window in registers (8 planes per
//     channel, window position i at bit 32*NW - L + i); sliding the window shifts every
//     plane down by one and inserts the entering frame's bits at the top (two funnel shifts
//     per plane word) instead of re-transposing L frames;
//   - the medians come from the same radix selection as the tile kernel (select_rank), with
//     the window's bits as the candidate set; the distance pass, outlier flags and epilogue
//     (background, outlier pick, blend, blend mask) are the pixel-thread code of cp_pixel.cuh.
// Every result equals what the single-stack kernel gives the same window.

#include <cuda_runtime.h>

#include "../../include/chrono_gpu.h"
#include "cp_internal.h"
#include "cp_pixel.cuh"

namespace cp {
namespace {

constexpr int kVC = 3;                // channels of the sliding kernel (RGB)
constexpr int kVideoPF = 4;           // frame rows in flight ahead of the one consumed
constexpr int kVideoRowPitch = 112;   // 96 bytes of a 32-pixel RGB row + read slack

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

// Slides the window planes by one frame: every plane word moves down by one bit and the
// entering sample's bit enters at the top (bit 32*NW - 1).
template <int NW>
DEVI void planes_push(uint32_t (&P)[kVC][8][NW], uint32_t px) {
#pragma unroll
  for (int ch = 0; ch < kVC; ++ch)
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const uint32_t in = px >> (8 * ch + b);  // bit 0: the entering bit
#pragma unroll
      for (int w = 0; w < NW; ++w)
        P[ch][b][w] = __funnelshift_r(P[ch][b][w], w + 1 < NW ? P[ch][b][w + 1] : in, 1);
    }
}

template <int OG, int BG, int NW>
__global__ void __launch_bounds__(32, 16) k_video_slide(const __grid_constant__ VideoArgs A) {
  constexpr int C = kVC;
  extern __shared__ __align__(128) uint8_t smem[];
  const StackDev& S = A.S;
  const int n = S.n;
  const int lane = static_cast<int>(threadIdx.x);
  uint32_t* ring = reinterpret_cast<uint32_t*>(smem);             // [2n][32] pixel words
  uint8_t* rows = smem + 2 * n * 32 * 4;                          // [kVideoPF][row pitch]
  uint8_t* stage = rows + kVideoPF * kVideoRowPitch;              // [2][row pitch] outputs
  uint32_t wbytes = 0;
#pragma unroll
  for (int ch = 0; ch < C; ++ch)
    if ((S.wmask >> ch) & 1u) wbytes |= 0xFFu << (8 * ch);
  // the window's bits: positions 0..n-1 at bits 32*NW - n .. 32*NW - 1
  uint32_t smask[NW];
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    const int lo_bit = 32 * NW - n - 32 * w;  // first window bit inside word w
    smask[w] = lo_bit <= 0 ? 0xFFFFFFFFu : (lo_bit >= 32 ? 0u : (0xFFFFFFFFu << lo_bit));
  }

  for (int tile = blockIdx.x; tile < A.tiles; tile += gridDim.x) {
    const int px0 = tile * 32;
    const int npx = min(32, A.npx - px0);
    const int nbytes = npx * C;
    const size_t src_off = static_cast<size_t>(px0) * C;
    // row j of the launch goes to staging slot j % kVideoPF, one copy group per row
    auto issue = [&](int j) {
      if (j < A.n_rows && lane * 16 < nbytes)
        cp_async16(rows + (j % kVideoPF) * kVideoRowPitch + lane * 16,
                   A.rows[j] + src_off + lane * 16);
      cp_async_commit();
    };
    // the lane's sample of row j; issues row j + kVideoPF into the freed slot
    auto consume = [&](int j) -> uint32_t {
      cp_async_wait<kVideoPF - 1>();
      __syncwarp();
      const uint32_t x = row_pixel(rows + (j % kVideoPF) * kVideoRowPitch, lane);
      __syncwarp();  // every lane has read the slot before it is refilled
      issue(j + kVideoPF);
      return x;
    };
    __syncwarp();
    for (int j = 0; j < kVideoPF; ++j) issue(j);
    uint32_t P[C][8][NW];
#pragma unroll
    for (int ch = 0; ch < C; ++ch)
#pragma unroll
      for (int b = 0; b < 8; ++b)
#pragma unroll
        for (int w = 0; w < NW; ++w) P[ch][b][w] = 0u;
    uint32_t sum[C] = {0u, 0u, 0u};
    for (int j = 0; j < n; ++j) {  // the first window
      const uint32_t x = consume(j);
      ring[j * 32 + lane] = x;
      ring[(j + n) * 32 + lane] = x;
      planes_push<NW>(P, x);
#pragma unroll
      for (int ch = 0; ch < C; ++ch) sum[ch] += (x >> (8 * ch)) & 0xFFu;
    }
    for (int k = 0; k < A.n_win; ++k) {
      const int head = k % n;  // ring slot of window position 0
      if (k > 0) {
        const uint32_t xi = consume(k + n - 1);
        const int slot = head == 0 ? n - 1 : head - 1;  // the leaving sample's slot
        const uint32_t xo = ring[slot * 32 + lane];
        ring[slot * 32 + lane] = xi;
        ring[(slot + n) * 32 + lane] = xi;
        planes_push<NW>(P, xi);
#pragma unroll
        for (int ch = 0; ch < C; ++ch)
          sum[ch] += ((xi >> (8 * ch)) & 0xFFu) - ((xo >> (8 * ch)) & 0xFFu);
      }
      // medians d[k] (and d[k+1] of a pair) of the window, all channels at once
      uint32_t lo[C], hi[C];
      select_rank<NW, C>(P, smask, S.med_k, lo);
      if (S.med_pair) {
        select_rank<NW, C>(P, smask, S.med_k + 1, hi);
      } else {
#pragma unroll
        for (int ch = 0; ch < C; ++ch) hi[ch] = lo[ch];
      }
      uint32_t lo3 = 0u, hi3 = 0u;
#pragma unroll
      for (int ch = 0; ch < C; ++ch) {
        lo3 |= lo[ch] << (8 * ch);
        hi3 |= hi[ch] << (8 * ch);
      }
      const float wq0[C] = {0.0f, 0.0f, 0.0f};
      const PxStat<C> st = px_stat<C>(S, lo3, hi3, wq0);
      // window position i is slot head + i (< 2n): no wrap
      const uint32_t* win = ring + head * 32 + lane;
      auto load = [&](int i) -> uint32_t { return win[i * 32]; };
      uint32_t pb[NW];
      int32_t key;
      float dmax;
      int imax;
      px_distance<C, NW, kIntKind, OG, decltype(load), 32>(S, n, st, wbytes, load, pb, key, dmax,
                                                         imax);
      const PxOut r = px_epilogue<C, NW, kIntKind, OG, BG>(S, n, st, wbytes, pb, key, dmax,
                                                           imax, px0 + lane, sum, load);
      // stage the composite and mask bytes, then store the rows coalesced
      __syncwarp();
#pragma unroll
      for (int ch = 0; ch < C; ++ch) {
        stage[3 * lane + ch] = static_cast<uint8_t>(r.pix >> (8 * ch));
        stage[kVideoRowPitch + 3 * lane + ch] = static_cast<uint8_t>(r.mask);
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
        const uint32_t wm = __ballot_sync(0xFFFFFFFFu, r.warning && lane < npx);
        if (lane == 0 && wm) atomicAdd(A.warnings + k, static_cast<unsigned long long>(__popc(wm)));
      }
    }
    cp_async_wait<0>();  // no copy of this tile is in flight when the rows are reused
    __syncwarp();
  }
}

}  // namespace

int video_smem_bytes(int n) { return 2 * n * 32 * 4 + (kVideoPF + 2) * kVideoRowPitch; }

template <int OG, int BG, int NW>
static int video_launch_t(const VideoArgs& a, int grid, int smem, void* stream) {
  const void* fn = reinterpret_cast<const void*>(&k_video_slide<OG, BG, NW>);
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  k_video_slide<OG, BG, NW><<<grid, 32, smem, static_cast<cudaStream_t>(stream)>>>(a);
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
  (void)error;  // the sliding kernel has no bounded waits: cp.async groups always complete
  if (nw == 1)
    return occupancy_only ? video_occupancy_t<OG, BG, 1>(smem)
                          : video_launch_t<OG, BG, 1>(a, grid, smem, stream);
  return occupancy_only ? video_occupancy_t<OG, BG, 2>(smem)
                        : video_launch_t<OG, BG, 2>(a, grid, smem, stream);
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
