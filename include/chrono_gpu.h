/*
 * chrono_gpu.h — C ABI of the GB300 frame-stack compositing library (libchrono_gpu.so).
 *
 * Replaces the stack reduction of chrono-photo 0.6.5 (a Rust CLI/library):
 *   - OutlierProcessor::new/process ............ src/chrono.rs:46-206 (per-pixel calc_pixel :208-494)
 *   - SimpleProcessor::new/process (darker/lighter) src/simple.rs:18-168
 *   - ShakeAnalyzer::analyze / Crop::create .... src/shake.rs:136-176, :190-313
 *   - chrono-video window enumeration .......... src/main.rs:214-331
 * The reference has no FFI; these entry points are what a Rust crate would bind with
 * `extern "C"` in place of the calls at src/main.rs:465-483 (create_frame),
 * :504-511 (create_frame_simple) and :61-74 (shake analysis).
 *
 * Conventions
 *   - Every function returns an int status: CP_OK (0) or a negative CP_ERR_* code.
 *     The reference panics on layout mismatches (src/chrono.rs:126, src/simple.rs:65,
 *     src/shake.rs:336); here those cases return CP_ERR_ARG / CP_ERR_RANGE instead.
 *   - Buffers are caller-owned. Images are interleaved 8-bit, row-major, `channels`
 *     bytes per pixel (1..4), the flat layout of image::FlatSamples used by the reference.
 *   - Stacks are frame-major: frame i of a stack is `frames[i]` (per-frame pointers) or
 *     `base + i * frame_stride`.
 *   - `*_device` entry points take device pointers and a CUDA stream (cudaStream_t passed
 *     as void*, NULL = the context's own stream) and are asynchronous unless noted.
 *     Entry points without the suffix take host memory and are synchronous.
 *   - No CPU fallback: if no usable sm_103 device is present, cp_ctx_create fails.
 */
#ifndef CHRONO_GPU_H
#define CHRONO_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------ */
#define CP_OK 0
#define CP_ERR_ARG (-1)     /* invalid argument or unsupported layout                      */
#define CP_ERR_OOM (-2)     /* device or pinned allocation failed                          */
#define CP_ERR_TIMEOUT (-3) /* a bounded device-side wait gave up (persistent queue)       */
#define CP_ERR_CUDA (-4)    /* CUDA runtime error; see cp_ctx_last_error                   */
#define CP_ERR_BUDGET (-5)  /* request exceeds the HBM budget of the context/server        */
#define CP_ERR_RANGE (-6)   /* shake window outside the image (reference: panic, shake.rs:336) */
#define CP_ERR_STATE (-7)   /* object in the wrong state (stopped server, unknown job)     */
#define CP_ERR_NODEV (-8)   /* no CUDA device with compute capability 10.3                 */
#define CP_ERR_LIMIT (-9)   /* request above a fixed limit (batch_static, composite_multi) */
#define CP_ERR_IO (-10)     /* image file missing, unreadable or not a supported PNG/JPEG  */
#define CP_ERR_CANCELLED (-11) /* server job cancelled before it started                   */

/* ---- option enums (src/options.rs) --------------------------------------------------- */
/* SelectionMode, src/options.rs:8-31 */
#define CP_MODE_OUTLIER 0
#define CP_MODE_DARKER 1
#define CP_MODE_LIGHTER 2
/* OutlierSelectionMode, src/options.rs:284-315 */
#define CP_OUTLIER_FIRST 0
#define CP_OUTLIER_LAST 1
#define CP_OUTLIER_EXTREME 2
#define CP_OUTLIER_AVERAGE 3
#define CP_OUTLIER_FORWARD 4
#define CP_OUTLIER_BACKWARD 5
/* BackgroundMode, src/options.rs:319-344 */
#define CP_BG_FIRST 0
#define CP_BG_RANDOM 1
#define CP_BG_AVERAGE 2
#define CP_BG_MEDIAN 3

/* Largest stack (frames per composite) the kernels accept. */
#define CP_MAX_FRAMES 128

/* Fade, src/options.rs:60-139. Points are (frame, value) pairs ordered by frame, as
 * parsed from `(clamp|repeat)/(abs|rel)/f,v/f,v/...`. enabled = 0 is Fade::none(). */
typedef struct cp_fade {
  int32_t enabled;
  int32_t repeat;   /* 1: FadeMode::Repeat, 0: FadeMode::Clamp */
  int32_t absolute; /* 1: abs (frame index + window offset), 0: rel (counted from the end) */
  int32_t n_points; /* >= 2 when enabled */
  const int32_t* frames;
  const float* values;
} cp_fade;

/* Parsed CLI options for one composite (src/cli.rs:22-136; defaults src/cli.rs:192-216).
 * Threshold values are the raw CLI numbers; the abs scaling by 255 of
 * Threshold::new (src/options.rs:197-213) happens inside. */
typedef struct cp_params {
  int32_t mode;       /* CP_MODE_*                                        */
  int32_t thr_abs;    /* 1: abs/min/max, 0: rel/min/max                   */
  float thr_min;      /* --threshold min                                  */
  float thr_max;      /* --threshold max (the parser copies min if absent) */
  int32_t outlier;    /* CP_OUTLIER_*                                     */
  int32_t background; /* CP_BG_*                                          */
  float weights[4];   /* --weights, per channel                           */
  cp_fade fade;       /* --fade                                           */
  /* --sample: sorted, distinct sample positions (0..n-1) used for the median/quartiles
   * (src/chrono.rs:151-163, :227-235). NULL / 0 = all frames. The reference draws them
   * with an unseeded RNG; cp_sample_indices draws them from a seed. */
  const int32_t* sample;
  int32_t n_sample;
  /* Seed of the counter-based generator that replaces the reference's unseeded
   * ThreadRng for --background random (src/chrono.rs:355-360, :532-555). */
  uint64_t rng_seed;
} cp_params;

/* One frame stack. With `crop` set, output pixel (x, y) of frame i is read from source
 * pixel (x + crop[2i], y + crop[2i+1]) of a src_width x src_height frame: the per-frame
 * crop origins of Crop::create (src/shake.rs:136-176) applied as address offsets. */
typedef struct cp_stack {
  int32_t n;        /* frames (samples) in the stack, 1..CP_MAX_FRAMES               */
  int32_t width;    /* output width  (cropped width when crop != NULL)                */
  int32_t height;   /* output height                                                  */
  int32_t channels; /* bytes per pixel, 1..4 (layout.width_stride)                    */
  const uint8_t* const* frames; /* per-frame base pointers, or NULL to use base/stride */
  const uint8_t* base;
  int64_t frame_stride;         /* bytes between frames when frames == NULL           */
  const int32_t* crop;          /* NULL or 2*n crop origins (x, y)                    */
  int32_t src_width;            /* source frame size when crop != NULL                */
  int32_t src_height;
  /* indices[0] of a chrono-video window: the `frame_offset` that an absolute fade is
   * evaluated at (src/chrono.rs:103, :496-502; src/simple.rs:54-57). 0 for a still. */
  int32_t frame_offset;
} cp_stack;

/* Optional per-pixel diagnostics of the outlier kernel, device (or host for the host
 * entry point) arrays; any member may be NULL. P = width * height. */
typedef struct cp_debug {
  float* median;          /* [P][channels] median (0 for weight-0 channels), chrono.rs:238-255 */
  float* q1;              /* [P][channels] lower quartile (rel threshold only)                 */
  float* q3;              /* [P][channels] upper quartile (rel threshold only)                 */
  uint32_t* outlier_bits; /* [P][words] bit i set iff sample i is an outlier, words = (n+31)/32 */
  int32_t* chosen;        /* [P] sample index blended in (-1: none; forward/backward with >1
                             outliers: -2; average with >1 outliers: 0, the index the reference
                             evaluates the fade at, chrono.rs:467)                              */
  int32_t* background;    /* [P] sample index copied as background (first/random), else -1    */
  int32_t* n_outliers;    /* [P] number of outliers                                           */
} cp_debug;

/* ---- library / options helpers (host only) ------------------------------------------- */
const char* cp_version(void);
const char* cp_status_str(int status);
/* Defaults of src/cli.rs:192-216: outlier, abs/0.05/0.2, background random, outlier
 * extreme, weights 1 1 1 1, fade none. */
void cp_params_default(cp_params* p);
/* Fade factor of every sample of an n-frame stack: out[i] = fade(i, n, frame_offset) with
 * the Fade::new table and Fade::get lookup (src/options.rs:69-139, src/chrono.rs:496-502). */
int cp_fade_lut(const cp_fade* fade, int32_t n, int32_t frame_offset, float* out);
/* Chrono-video windows (src/main.rs:230-286). Ranges are FrameRange start/end/step with
 * has_* = 0 for the `.` placeholder (src/flist.rs:46-79). Writes, for each output frame k,
 * win_start[k] = offset into win_indices and win_len[k] (0 = skipped frame). Pass NULL
 * buffers to query *n_windows and *n_indices first. */
int cp_video_windows(int32_t image_count, int32_t in_has_start, int32_t in_start,
                     int32_t in_has_end, int32_t in_end, int32_t in_step,
                     int32_t out_has_start, int32_t out_start, int32_t out_has_end,
                     int32_t out_end, int32_t out_step, int32_t* n_windows,
                     int64_t* n_indices, int64_t* win_start, int32_t* win_len,
                     int32_t* win_indices, int32_t* win_frame);
/* Crop::create (src/shake.rs:136-176): crops[4i..4i+3] = (x, y, w, h) per frame.
 * *has_crop = 0 (and crops untouched) when every offset is (0, 0) — the reference's None. */
int cp_crop_create(const int32_t* offsets, int32_t n, int32_t width, int32_t height,
                   int32_t* has_crop, int32_t* crops);
/* Seeded replacement for rand::seq::sample_indices + sort (src/chrono.rs:153-158):
 * writes min(count, n) sorted distinct positions. */
int cp_sample_indices(int32_t n, int32_t count, uint64_t seed, int32_t* out, int32_t* n_out);

/* ---- context ------------------------------------------------------------------------- */
typedef struct cp_ctx cp_ctx;
/* hbm_budget: bytes of device memory the context may hold (0 = no limit). */
int cp_ctx_create(int32_t device, uint64_t hbm_budget, cp_ctx** out);
void cp_ctx_destroy(cp_ctx* ctx);
/* Copies the last error message of this context into buf (always NUL-terminated). */
int cp_ctx_last_error(cp_ctx* ctx, char* buf, size_t len);
/* Stream the *_device entry points use when passed NULL. */
void* cp_ctx_stream(cp_ctx* ctx);
int cp_ctx_synchronize(cp_ctx* ctx);
/* Limit, in SM clock cycles, of every bounded device-side wait of this context's later
 * launches (a CTA waiting for its staged frames; 0 = the default, 2^32 cycles, about 2 s).
 * A wait that runs out makes its CTA leave (after its copies in flight have landed) and the
 * call, or the next cp_ctx_synchronize, return CP_ERR_TIMEOUT; the context stays usable.
 * A limit of 1 cycle gives up every wait at once (for tests of that path). No counterpart
 * in the reference, whose loops have no device side. */
int cp_ctx_set_wait_limit(cp_ctx* ctx, uint64_t cycles);
/* Testing aid: the next `count` device or pinned allocations made for this context (its own
 * buffers, cp_dev_alloc, cp_host_alloc, server jobs) fail with CP_ERR_OOM as if memory ran
 * out; 0 cancels what is left. No counterpart in the reference. */
int cp_ctx_fail_allocations(cp_ctx* ctx, int32_t count);
/* The launch configurations the context's autotuner chose for the single-stack outlier
 * kernel, as a JSON array (one object per distance kind, outlier group, background and
 * plane-word count: the choice, its measured time and the static choice's time). The first
 * launch of such a key on a stack that fills the GPU several times times every candidate
 * configuration (results do not depend on it) and caches the fastest in a file keyed by GPU
 * and library version (CP_TUNE_CACHE; CP_AUTOTUNE=0 turns tuning off). CP_ERR_LIMIT if the
 * text did not fit `len`. Replaces the reference's hand-set thread counts
 * (src/main.rs:49-54, :254-261). */
int cp_ctx_tuning_report(cp_ctx* ctx, char* buf, size_t len);
/* Device memory owned by the context (counted against its HBM budget). */
int cp_dev_alloc(cp_ctx* ctx, uint64_t bytes, void** ptr);
int cp_dev_free(cp_ctx* ctx, void* ptr);
/* Pinned (page-locked) host memory: frames staged from it are copied by DMA without an
 * intermediate host copy. */
int cp_host_alloc(cp_ctx* ctx, uint64_t bytes, void** ptr);
int cp_host_free(cp_ctx* ctx, void* ptr);
/* stream NULL: synchronous on the context's stream. */
int cp_memcpy_h2d(cp_ctx* ctx, void* dst_dev, const void* src_host, uint64_t bytes, void* stream);
int cp_memcpy_d2h(cp_ctx* ctx, void* dst_host, const void* src_dev, uint64_t bytes, void* stream);

/* ---- compositing --------------------------------------------------------------------- */
/* One stack per launch (the plain kernel). Device pointers throughout: frames (16-byte
 * aligned, each readable up to the next multiple of 16 bytes past its last pixel), out
 * (P*channels bytes), out_blend (P*channels, nullable; outlier mode only: the blend mask,
 * 255 in channels >= 3, src/chrono.rs:183-191), dbg members. warnings (device uint64,
 * nullable) is incremented by the number of all-outlier pixels (src/chrono.rs:180-203).
 * Replaces OutlierProcessor::process (mode outlier) and SimpleProcessor::process
 * (darker/lighter) for one output frame. */
int cp_composite_device(cp_ctx* ctx, const cp_stack* stack, const cp_params* params,
                        uint8_t* out, uint8_t* out_blend, const cp_debug* dbg,
                        uint64_t* warnings, void* stream);

/* One device-resident stack under `count` parameter sets (at most CP_MAX_SETTINGS), the
 * device form of cp_composite_multi: out[k], out_blend[k] (nullable; outlier settings only)
 * and warnings[k] (device uint64 array of count entries, nullable) as for
 * cp_composite_device with params[k]. Outlier settings that share the stack's order
 * statistics (RGB frames starting 16-byte aligned, integer or paired-f32 distances, the
 * same --sample) run in one multi-setting pass that stages every frame row and selects the
 * medians once for all of them; each setting's results equal cp_composite_device's for it
 * alone. Replaces several OutlierProcessor::process runs over the same files
 * (src/main.rs:465-483 once per setting). */
int cp_composite_device_multi(cp_ctx* ctx, const cp_stack* stack, const cp_params* params,
                              int32_t count, uint8_t* const* out, uint8_t* const* out_blend,
                              uint64_t* warnings, void* stream);
/* Kernel launches the context has made so far (a replayed batch graph counts one), and of
 * them the multi-setting launches and the settings they carried (any pointer nullable). */
int cp_ctx_launch_counts(cp_ctx* ctx, uint64_t* launches, uint64_t* multi_launches,
                         uint64_t* multi_settings);

/* Host-memory form of cp_composite_device: frames in host memory are staged through
 * pinned buffers and copied to the device in row bands that overlap the kernel; results
 * are copied back. Synchronous. n_warnings (host, nullable) receives the warning count.
 * dbg members, when given, are host arrays. */
int cp_composite(cp_ctx* ctx, const cp_stack* stack, const cp_params* params, uint8_t* out,
                 uint8_t* out_blend, const cp_debug* dbg, uint64_t* n_warnings);

/* cp_composite of one host-memory stack under `count` parameter sets (1..CP_MAX_SETTINGS):
 * the frames cross the host link once, band by band, and every setting's kernel runs on
 * each band while the next band is in flight. out[k], out_blend[k] (array and entries
 * nullable) and n_warnings[k] (nullable) belong to params[k]; each equals what cp_composite
 * gives for params[k] alone. The reference composites one setting per run, re-reading its
 * frames each time (src/main.rs:454-517); this is the call for several settings of one
 * stack (e.g. comparing thresholds or outlier modes). CP_ERR_LIMIT above CP_MAX_SETTINGS. */
#define CP_MAX_SETTINGS 16
int cp_composite_multi(cp_ctx* ctx, const cp_stack* stack, const cp_params* params,
                       int32_t count, uint8_t* const* out, uint8_t* const* out_blend,
                       uint64_t* n_warnings);

/* Many stacks of uneven size in ONE persistent launch that pulls (stack, tile) work items
 * from a device queue (chrono-video windows, mixed jobs). Device pointers; params[i]
 * applies to stacks[i]; outs/blends/warnings are per stack (blends/warnings nullable).
 * The launch is captured into a CUDA graph that is replayed while the batch shape is
 * unchanged. Replaces the rayon loop over create_frame calls, src/main.rs:254-330. */
int cp_composite_batch_device(cp_ctx* ctx, const cp_stack* stacks, const cp_params* params,
                              int32_t n_stacks, uint8_t* const* outs,
                              uint8_t* const* out_blends, uint64_t* warnings, void* stream);

/* Chrono-video over frames resident on the device: one composite per window of
 * cp_video_windows (win_start/win_len/win_indices index into `frames`, image_count device
 * frame pointers). Windows of length 0 are skipped (src/main.rs:326-328); outs, out_blends
 * (nullable) and warnings (device, nullable) are indexed by window. Each window's absolute
 * fade is evaluated at its first index (src/chrono.rs:103). One persistent launch, work
 * ordered tile-major so that overlapping windows read shared frame rows while they are in
 * L2. Replaces create_video's loop over create_frame, src/main.rs:254-323. */
int cp_composite_video_device(cp_ctx* ctx, const uint8_t* const* frames, int32_t image_count,
                              int32_t width, int32_t height, int32_t channels,
                              int32_t n_windows, const int64_t* win_start,
                              const int32_t* win_len, const int32_t* win_indices,
                              const cp_params* params, uint8_t* const* outs,
                              uint8_t* const* out_blends, uint64_t* warnings, void* stream);

/* Allocation-free form of cp_composite_batch_device. No counterpart in the reference. For
 * callers that cannot call cudaMalloc: a plug-in inside a host application whose own
 * allocator owns all device memory, or a service that must not grow its device footprint
 * after start-up. It needs no context: it runs on the current device and on `stream`, and
 * keeps its scratch (stack descriptors, tile prefix sums, work counter, error flag) in one
 * fixed __device__ array of about 190 KB that every GPU loading the library holds until the
 * process exits. At most CP_STATIC_MAX_STACKS stacks per call (more: CP_ERR_LIMIT). The
 * first call on a device (with that device current) looks up the array's device address;
 * the address is kept for the life of the process, so a cudaDeviceReset() followed by more
 * calls is not supported. The descriptors are passed to the GPU as kernel parameters, so
 * the call returns without waiting for earlier work on `stream`, reads no host memory after
 * it returns, and can be captured into a CUDA graph. All calls share the array:
 * calls that overlap on the GPU (other streams, other host threads) race, so order them on
 * one stream. Inputs, outputs and warnings (device array of n_stacks counters, nullable)
 * are as for cp_composite_batch_device. */
#define CP_STATIC_MAX_STACKS 64
int cp_composite_batch_static(const cp_stack* stacks, const cp_params* params, int32_t n_stacks,
                              uint8_t* const* outs, uint8_t* const* out_blends,
                              uint64_t* warnings, void* stream);
/* Device-side status of the last cp_composite_batch_static call on the current device:
 * waits for `stream`, then *status = CP_OK, or CP_ERR_TIMEOUT when a tile's bounded wait
 * for its staged frames gave up (that call's outputs are incomplete). Allocates nothing. */
int cp_composite_batch_static_status(int32_t* status, void* stream);

/* ---- camera shake -------------------------------------------------------------------- */
/* ShakeAnalyzer::analyze (src/shake.rs:190-313): anchor windows of radius anchor_radius
 * from frame 0, exhaustive wrapping-i32 sum of squared differences over the
 * (2*search_radius+1)^2 offsets for frames 1..n-1, first minimum. Device frames; offsets
 * (host, 2n int32, frame 0 = (0, 0)) and, nullable, diffs (host, (n-1)*(2s+1)^2 int32) are
 * written on return (synchronous). CP_ERR_RANGE where the reference would panic. */
int cp_shake_analyze_device(cp_ctx* ctx, const uint8_t* const* frames, int32_t n,
                            int32_t width, int32_t height, int32_t channels,
                            const int32_t* anchors, int32_t n_anchors, int32_t anchor_radius,
                            int32_t search_radius, int32_t* offsets, int32_t* diffs);

/* ---- frame ingest ---------------------------------------------------------------------- */
/* Replaces `image::open(path)` + `as_flat_samples_u8()` of the frame readers
 * (src/streams.rs:63-70, src/simple.rs:45-52, src/shake.rs:218-255) for PNG files: 8-bit
 * grayscale (1 channel), RGB (3) or RGBA (4), not interlaced; the decoded samples are the
 * image's flat u8 layout, row-major, channels interleaved. cp_png_info reads the header of
 * one file. cp_load_png decodes n files on `threads` host threads (0: all cores) into
 * out + i * frame_stride (host memory, e.g. from cp_host_alloc, so that cp_composite copies
 * it to the device at full link speed); every file must have the given width, height and
 * channels. ctx (nullable) receives the error message. CP_ERR_IO for a missing, truncated,
 * corrupt (chunk CRC-32, zlib Adler-32 or DEFLATE data) or unsupported file. */
int cp_png_info(cp_ctx* ctx, const char* path, int32_t* width, int32_t* height,
                int32_t* channels);
int cp_load_png(cp_ctx* ctx, const char* const* paths, int32_t n, int32_t threads,
                uint8_t* out, uint64_t frame_stride, int32_t width, int32_t height,
                int32_t channels);

/* The same for JPEG files (the reference's own frames are JPEG: image-%05d.jpg at quality
 * 95, src/util/create_example_data.rs:52-56), decoded on the GPU by nvJPEG's batched
 * decoder (libnvjpeg, loaded at the first call): Huffman-coded DCT, baseline, extended or
 * progressive, 8-bit samples, one component (channels 1, gray) or three (channels 3,
 * interleaved RGB); any chroma subsampling nvJPEG takes. Files are read on `threads` host
 * threads (0: all cores) and their headers checked against width, height and channels.
 * cp_load_jpeg_device writes frame i to out + i * frame_stride in DEVICE memory (the stack
 * of cp_composite_device: only the compressed bytes cross the host link); cp_load_jpeg to
 * host memory (decoded on the device, then copied back). Both return when the frames are
 * written. JPEG decoders differ in their inverse DCT and chroma upsampling, so the samples
 * match those of image's decoder to a tolerance, not bit for bit. CP_ERR_IO for a missing,
 * truncated, corrupt or unsupported file (lossless, hierarchical, arithmetic-coded, 12-bit,
 * CMYK) or when libnvjpeg cannot be loaded. cp_jpeg_info reads a file's header (host only). */
int cp_jpeg_info(cp_ctx* ctx, const char* path, int32_t* width, int32_t* height,
                 int32_t* channels);
int cp_load_jpeg_device(cp_ctx* ctx, const char* const* paths, int32_t n, int32_t threads,
                        uint8_t* out, uint64_t frame_stride, int32_t width, int32_t height,
                        int32_t channels);
int cp_load_jpeg(cp_ctx* ctx, const char* const* paths, int32_t n, int32_t threads,
                 uint8_t* out, uint64_t frame_stride, int32_t width, int32_t height,
                 int32_t channels);

/* ---- output encode ----------------------------------------------------------------------- */
/* Replaces save_image (src/main.rs:519-570: image::save_buffer by file extension, the parent
 * directory created when missing) for PNG output of a composite or blend mask: `image` is
 * height rows of width * channels bytes (1 gray, 3 RGB, 4 RGBA), written losslessly with
 * adaptive scanline filters and zlib `level` 0..9 (0: stored, -1: 6), compressed in 256 KB
 * segments on `threads` host threads (0: all cores; the file does not depend on it).
 * ctx (nullable) receives the error message; CP_ERR_IO when the file cannot be written. */
int cp_save_png(cp_ctx* ctx, const char* path, const uint8_t* image, int32_t width,
                int32_t height, int32_t channels, int32_t level, int32_t threads);

/* Replaces the .jpg branch of save_image (src/main.rs:542-556: image's JPEGEncoder at
 * --quality, 95 by default, src/cli.rs:82-84): baseline JPEG of a host image (channels 1
 * gray, 3 RGB, 4 RGBA with the alpha dropped, as image does), quality 1..100 (0 or less:
 * 95) with the IJG scaling of the Annex K tables, chroma `subsampling` 0 = 4:4:4 (the
 * reference's) or 1 = 4:2:0, Huffman tables built for the image, one restart interval per
 * MCU row so that rows are coded on `threads` host threads (0: all cores; the file does not
 * depend on it). Width and height up to 65535. cp_save_jpeg writes the file (creating a
 * missing parent directory); cp_encode_jpeg writes the bytes to out[0, capacity) and their
 * count to *size (CP_ERR_LIMIT, with *size set, when they do not fit; capacity 0 queries
 * the size). */
int cp_save_jpeg(cp_ctx* ctx, const char* path, const uint8_t* image, int32_t width,
                 int32_t height, int32_t channels, int32_t quality, int32_t subsampling,
                 int32_t threads);
int cp_encode_jpeg(cp_ctx* ctx, const uint8_t* image, int32_t width, int32_t height,
                   int32_t channels, int32_t quality, int32_t subsampling, int32_t threads,
                   uint8_t* out, uint64_t capacity, uint64_t* size);

/* ---- serving ------------------------------------------------------------------------- */
/* A compositing job: a host-memory stack plus options, output buffers in host memory.
 * Frames named by (frame_keys) are kept resident on the device between jobs, so jobs
 * over overlapping windows of the same frames share uploads; key 0 = not shareable. */
typedef struct cp_job {
  cp_stack stack;              /* host frames (frames[] or base/stride)                */
  const uint64_t* frame_keys;  /* nullable: n keys naming the frames for residency    */
  cp_params params;
  uint8_t* out;                /* host, width*height*channels                          */
  uint8_t* out_blend;          /* host, nullable                                       */
} cp_job;

typedef struct cp_job_result {
  int32_t status;              /* CP_OK or the job's error                             */
  uint64_t warnings;
  double submit_s;             /* host clock (s) at submit, admission, completion      */
  double admit_s;
  double done_s;
} cp_job_result;

typedef struct cp_server cp_server;
/* max_inflight: jobs whose work may be on the device at once. The server admits jobs
 * against the context's HBM budget (hbm_budget, 0 = the context's) as memory frees up,
 * uploads each admitted job's frames on copy streams, and launches the jobs whose uploads
 * have landed together in one batched persistent launch per channel count, on rotating
 * compute streams, so that new launches overlap the ones still running. */
int cp_server_create(cp_ctx* ctx, uint64_t hbm_budget, int32_t max_inflight, cp_server** out);
/* Non-blocking; the job's buffers must stay valid until it completes. */
int cp_server_submit(cp_server* srv, const cp_job* job, uint64_t* job_id);
/* Waits up to timeout_ms (-1 = forever; 0 = poll without blocking) for job_id.
 * CP_ERR_TIMEOUT if not done yet. */
int cp_server_wait(cp_server* srv, uint64_t job_id, int32_t timeout_ms, cp_job_result* res);
/* Cancels a job that is still queued (not yet admitted): it completes at once with status
 * CP_ERR_CANCELLED and its buffers are not touched. CP_ERR_STATE if the job has already been
 * admitted or has completed (it then runs to completion), CP_ERR_ARG for an unknown id.
 * The reference's processors run to completion; there is no counterpart. */
int cp_server_cancel(cp_server* srv, uint64_t job_id);
/* Stops accepting jobs, drains the queue and joins the worker. */
int cp_server_destroy(cp_server* srv);

#ifdef __cplusplus
}
#endif
#endif /* CHRONO_GPU_H */
