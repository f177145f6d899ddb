// cp_internal.h — types shared by the host layer (cp_host.cpp) and the CUDA kernels.
#pragma once
#include <cstdint>

#include "../../include/chrono_gpu.h"

namespace cp {

constexpr int kTilePx = 128;      // pixels per tile: 32 columns, served by `channels` warps
constexpr long long kDefaultWaitCycles = 1ll << 32;  // ~2 s: the default bounded-wait limit
inline int cta_threads(int channels) { return 32 * channels; }

// Shared-memory exchange area of a compositing tile, behind its staged frame rows: warp w
// builds the order statistics of word w of every column, every warp the distance pass over
// its frame class, the epilogue is split by pixel; results cross warps here.
// The column index is innermost everywhere, so a warp's accesses hit 32 distinct banks.
template <int C, int NW>
struct Aux {
  uint32_t lo[C][32], hi[C][32];  // word w of column t: order statistics d[k], d[k+1]
  float wi[C][4][32];             // rel threshold: w * iqr_inv per position of word w
  uint32_t bits[C][4][NW][32];    // per frame class, pixel, flag word, column
  int32_t best[C][4][32];         // integer path: max (D' << 8) + 255 - f; f32 path: max distance
  int32_t imf[C][4][32];          // f32 path: frame of that maximum
  uint32_t out[C][32], blend[C][32];  // the tile's output rows, C words per column
};
inline int aux_bytes(int channels, int nw) {
  switch (channels * 8 + nw) {
    case 8 + 1: return sizeof(Aux<1, 1>);
    case 8 + 2: return sizeof(Aux<1, 2>);
    case 8 + 4: return sizeof(Aux<1, 4>);
    case 24 + 1: return sizeof(Aux<3, 1>);
    case 24 + 2: return sizeof(Aux<3, 2>);
    case 24 + 4: return sizeof(Aux<3, 4>);
    case 32 + 1: return sizeof(Aux<4, 1>);
    case 32 + 2: return sizeof(Aux<4, 2>);
    default: return sizeof(Aux<4, 4>);
  }
}
inline int nw_for(int n) { return n <= 32 ? 1 : (n <= 64 ? 2 : 4); }

// Device-side descriptor of one stack and its options, prepared on the host from cp_stack
// and cp_params. A single-stack launch passes it by value (kernel parameter space, so the
// per-frame tables need no device allocation); a batch keeps an array in device memory.
struct StackDev {
  // geometry
  int32_t n, width, height, channels;
  int32_t src_width;      // row pitch (pixels) of the source frames
  int32_t tiles;          // work items of this stack
  int32_t tiles_per_row;  // > 0: tiles are row segments (cropped stacks); 0: flat pixel ranges
  int32_t tile_px;        // pixels per tile
  int32_t px_begin;       // flat tiles: first output pixel covered (row bands)
  int32_t px_end;         //             one past the last
  int32_t row_begin;      // row tiles: first output row covered
  int32_t nw;             // 32-frame words per bit plane: 1, 2 or 4
  int32_t threads;        // CTA size the stack was planned for
  int32_t has_crop;
  int32_t shifted;        // some frame row may start off a 16-byte boundary
  // outputs
  uint8_t* out;
  uint8_t* blend;
  unsigned long long* warnings;
  float* dbg_median;
  float* dbg_q1;
  float* dbg_q3;
  uint32_t* dbg_bits;
  int32_t* dbg_chosen;
  int32_t* dbg_bg;
  int32_t* dbg_nout;
  // options
  int32_t mode, outlier, background, thr_abs;
  float w[4];
  uint32_t wmask;      // bit c: weights[c] != 0
  uint32_t fast_int;   // abs threshold and every weight 0 or 1: exact integer distances
  uint32_t neg_w;      // some weight negative
  uint32_t unit_w;     // every weight 0 or 1
  uint32_t finite_w;   // every weight finite with |w| < 1e30: w * iqr_inv stays finite
  uint32_t pair_f32;   // f32 distances may run halved, two pixels per instruction (see host)
  uint32_t no_fade;    // every fade factor >= 1 (darker/lighter copy the pixel)
  float thr_min, thr_max, thr_scale, thr_sq;
  int32_t thr_int[5];  // smallest integer D' with D' + nh/4 >= thr_sq, per nh = 0..4
  // order statistics of the (sub)sample (quantile/median, src/chrono.rs:567-591)
  int32_t n_sub;
  int32_t med_k, med_pair;
  int32_t q1_k, q1_pair;
  float q1_frac;
  int32_t q3_k, q3_pair;
  float q3_frac;
  uint32_t sample_mask[4];  // frames in the (sub)sample, bit i of word i/32
  uint64_t seed;
  int64_t wait_cycles;  // SM clock cycles before a bounded wait gives up
  uint32_t unit_fade;   // every fade factor is exactly 1 (the epilogue skips its fade lookups)
  uint32_t pad0;        // keeps the descriptor a multiple of 16 bytes (copied in 16-byte words)
  // per-frame tables
  const uint8_t* frames[CP_MAX_FRAMES];
  int32_t crop[2 * CP_MAX_FRAMES];
  float fade[CP_MAX_FRAMES];  // fade(i, n, frame_offset)
};

inline int row_pitch_host(int channels) { return kTilePx * channels + 32; }
// Shared-memory header of a compositing CTA: mbarrier, per-row byte shifts, and the cached
// frame base pointers of the stack being processed.
constexpr int kSmemHeader = 256 + 8 * CP_MAX_FRAMES;
// header + n staged rows + the exchange area
inline int smem_bytes_for(int n, int channels) {
  return kSmemHeader + n * row_pitch_host(channels) + aux_bytes(channels, nw_for(n));
}

// Per-channel-count kernel entry points (cp_kernels_c*.cu). Return cudaError_t values.
#define CP_DECLARE_CH(CH)                                                                 \
  int composite_max_ctas_c##CH(int threads, int smem); /* the general (any-stack) kernel */\
  int launch_composite_c##CH(const StackDev& s, int grid, int smem, void* stream,         \
                             uint32_t* error);                                            \
  int launch_batch_c##CH(const StackDev* stacks, const int32_t* prefix, int32_t n_stacks, \
                         int32_t total, int32_t interleave, uint32_t* counter,            \
                         uint32_t* error, int grid, int smem, void* stream);              \
  int simple_stream_max_ctas_c##CH(bool fast);                                            \
  int simple_stream_chunk_px_c##CH();                                                     \
  int launch_simple_stream_c##CH(const StackDev& s, bool fast, int grid, void* stream,    \
                                 uint32_t* error);
CP_DECLARE_CH(1)
CP_DECLARE_CH(3)
CP_DECLARE_CH(4)
#undef CP_DECLARE_CH

// Single-stack outlier kernels specialised at compile time (cp_kernels_variant.cu, one
// translation unit each): (channels, distance kind k: 1 integer / 2 paired f32 / 3 scalar
// f32, outlier group g: 0 any / 1 extreme, first, last / 2 average / 3 forward, backward,
// background b: 0 any / 1 first). RGB has one kernel per (k, g, b) for k = 1, 2; the other
// cases one per kind. build.py compiles the same list.
#define CP_VARIANTS(X)                                                                       \
  X(3, 1, 1, 1) X(3, 1, 2, 1) X(3, 1, 3, 1) X(3, 1, 1, 0) X(3, 1, 2, 0) X(3, 1, 3, 0)       \
  X(3, 2, 1, 1) X(3, 2, 2, 1) X(3, 2, 3, 1) X(3, 2, 1, 0) X(3, 2, 2, 0) X(3, 2, 3, 0)       \
  X(3, 3, 0, 0) X(1, 1, 0, 0) X(1, 2, 0, 0) X(1, 3, 0, 0) X(4, 1, 0, 0) X(4, 2, 0, 0)       \
  X(4, 3, 0, 0)
#define CP_DECLARE_VARIANT(CH, K, G, B)                                                      \
  int launch_composite_c##CH##_k##K##_g##G##_b##B(const StackDev& s, int grid, int smem,    \
                                                  void* stream, uint32_t* error);           \
  int max_ctas_c##CH##_k##K##_g##G##_b##B(int threads, int smem);
CP_VARIANTS(CP_DECLARE_VARIANT)
#undef CP_DECLARE_VARIANT
// Batched kernels for uniform RGB batches with background first (cp_kernels_batch_variant.cu).
#define CP_BATCH_VARIANTS(X)                                                                 \
  X(3, 1, 1, 1) X(3, 1, 2, 1) X(3, 1, 3, 1) X(3, 2, 1, 1) X(3, 2, 2, 1) X(3, 2, 3, 1)
#define CP_DECLARE_BATCH_VARIANT(CH, K, G, B)                                                \
  int launch_batch_c##CH##_k##K##_g##G##_b##B(const StackDev* stacks, const int32_t* prefix,\
                                              int32_t n_stacks, int32_t total,              \
                                              int32_t interleave, uint32_t* counter,        \
                                              uint32_t* error, int grid, int smem,          \
                                              void* stream);                                \
  int batch_max_ctas_c##CH##_k##K##_g##G##_b##B(int smem);
CP_BATCH_VARIANTS(CP_DECLARE_BATCH_VARIANT)
#undef CP_DECLARE_BATCH_VARIANT
// Outlier group of a stack's outlier mode.
inline int outlier_group(int outlier) {
  return outlier == CP_OUTLIER_AVERAGE ? 2
         : (outlier == CP_OUTLIER_FORWARD || outlier == CP_OUTLIER_BACKWARD) ? 3 : 1;
}
// The specialised kernel (k, g, b) an outlier stack launches with.
inline void outlier_variant(const StackDev& s, int* k, int* g, int* b) {
  *k = s.fast_int ? 1 : (s.pair_f32 ? 2 : 3);
  const bool split = s.channels == 3 && *k != 3;
  *g = split ? outlier_group(s.outlier) : 0;
  *b = split && s.background == CP_BG_FIRST ? 1 : 0;
}
// Which single-stack kernel a stack launches with (an occupancy cache key).
inline int single_variant(const StackDev& s) {
  if (s.mode != CP_MODE_OUTLIER) return 0;
  int k, g, b;
  outlier_variant(s, &k, &g, &b);
  return 1 + k * 8 + g * 2 + b;
}

// Pixel-thread single-stack outlier kernel (cp_outlier_px.cuh): RGB stacks with 16-byte
// aligned frame rows and no crop, distance kind 1 (integer) or 2 (paired f32). A CTA of
// kPxThreads threads; phase A's order statistics reach the pixel threads through PxAux.
constexpr int kPxThreads = 128;
// CTAs per SM the batch routing assumes for the pixel-thread kernel (its 64-frame residency)
constexpr int kPxAloneCtas = 7;
struct PxAux {
  uint32_t lo[4][32], hi[4][32];  // word w of column t; word 3 is zero (funnel padding)
  float wq[12][32];               // rel: w * iqr_inv of byte position q of column t
  uint32_t out[3][32], blend[3][32];
};
// Stage rows of the pixel-thread kernels: n padded to whole 32-sample words. The copies fill
// rows 0..n-1; the kernels zero the rest once, so that the bit planes load every sample of
// a word without bound tests (the sample mask leaves the padding out of every statistic).
inline int px_stage_rows(int n) { return 32 * nw_for(n); }
// header + one or two (double-buffered) stage buffers of the padded rows + PxAux
inline int px_smem_bytes(int n, bool db) {
  return kSmemHeader + (db ? 2 : 1) * px_stage_rows(n) * row_pitch_host(3) +
         static_cast<int>(sizeof(PxAux));
}
// Several outlier settings of one stack in one pass (k_outlier_multi, cp_outlier_multi.cuh):
// the settings' descriptors, kernel parameters; sets[0] also gives the frames, geometry and
// (sub)sample, which all of them share. share_dist[s]: setting s has the distance kind,
// threshold and weights of setting s - 1, so its outlier flags and extreme are the same.
constexpr int kMultiMax = 8;
struct MultiArgs {
  StackDev sets[kMultiMax];
  int32_t count;
  int32_t share_dist[kMultiMax];
  int32_t pad[3];
};
static_assert(sizeof(MultiArgs) <= 32764, "MultiArgs exceeds the kernel parameter limit");
// Launch (occupancy_only: CTAs per SM instead) of the multi-setting kernel for the plane
// words of a.sets[0]; rel: some setting has a rel threshold (quartiles needed).
int px_multi(const MultiArgs& a, bool rel, bool occupancy_only, int grid, int smem, void* stream,
             uint32_t* error);

// (distance kind, outlier group, background) of the compiled pixel-thread kernels; each
// translation unit holds plane-word counts 1 and 2 (single and double buffered) and 4
// (single), each with phase A by word column (pa 0) and by pixel (pa 2).
#define CP_PX_VARIANTS(X)                                                                    \
  X(1, 1, 1) X(1, 2, 1) X(1, 3, 1) X(1, 1, 0) X(1, 2, 0) X(1, 3, 0) X(2, 1, 1) X(2, 2, 1)  \
  X(2, 3, 1) X(2, 1, 0) X(2, 2, 0) X(2, 3, 0)
#define CP_DECLARE_PX(K, G, B)                                                               \
  int px_launch_k##K##_g##G##_b##B(const StackDev& s, int pa, bool db, bool occupancy_only,   \
                                   int grid, int smem, void* stream, uint32_t* error);
CP_PX_VARIANTS(CP_DECLARE_PX)
#undef CP_DECLARE_PX

// Chrono-video windows sliding by one frame (cp_video.cu): the kernel's parameter block.
// Window k of a launch reads frame rows k .. k + n - 1; longer calls are split into
// launches of at most kVideoMaxWin windows.
constexpr int kVideoMaxRows = 768;
constexpr int kVideoMaxWin = 640;
struct VideoArgs {
  StackDev S;      // options of every window (S.n = window length <= 64); frame tables unused
  int32_t n_rows;  // frame rows of this launch
  int32_t n_win;   // windows of this launch
  int32_t npx;     // pixels per frame
  int32_t tiles;   // 32-pixel tiles per frame
  const uint8_t* rows[kVideoMaxRows];
  uint8_t* outs[kVideoMaxWin];
  uint8_t* blends[kVideoMaxWin];  // entries may be null
  unsigned long long* warnings;   // nullable: one counter per window of this launch
};
int video_smem_bytes(int n);
// og: outlier group (1 extreme/first/last, 2 average, 3 forward/backward); bg_first: the
// background is `first`. occupancy_only: returns CTAs per SM instead of launching.
int video_slide(const void* args, int og, int bg_first, bool occupancy_only, int grid, int smem,
                void* stream, uint32_t* error);

// Shake search (cp_shake.cu): diffs[(f-1) * S^2 + oy*S + ox] for frames 1..n-1.
int launch_shake(const uint8_t* const* frames_dev, int32_t n, int32_t width, int32_t height,
                 int32_t channels, const int32_t* anchors_dev, int32_t n_anchors, int32_t r,
                 int32_t s, int32_t* diffs_dev, void* stream);

}  // namespace cp
