// cp_host_internal.h — the context object and host helpers shared by the C-ABI sources.
#pragma once
#include <cuda_runtime.h>

#include <atomic>

#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "../../include/chrono_gpu.h"
#include "cp_internal.h"

namespace cp {

struct DevBuffer {
  void* ptr = nullptr;
  uint64_t bytes = 0;
};
struct PinnedBuffer {
  void* ptr = nullptr;
  uint64_t bytes = 0;
};

// One captured batch launch (cp_batch.cpp).
struct BatchPlan {
  std::vector<StackDev> host;  // descriptors the plan was built from
  void* dev = nullptr;         // [StackDev x n][int32 prefix x (n+1)][uint32 counter]
  uint64_t dev_bytes = 0;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  int32_t total = 0;
  int32_t interleave = 0;  // equal-geometry stacks: tile-major work order
  int32_t max_n = 0;
};

// Launch configuration of the pixel-thread outlier kernel (cp_tune.cpp).
struct PxChoice {
  int pa = -1;    // phase A: 0 word columns, 2 per pixel, -1 the static choice of the kind
  int db = 0;     // 1: two staging buffers per CTA
  int ctas = 0;   // CTAs per SM (0: as many as fit)
  float ms = 0.0f, static_ms = 0.0f;  // measured launch times: this choice, the static one
  std::string name;
  bool from_cache = false;
};

}  // namespace cp

struct cp_ctx {
  int device = 0;
  int sm_count = 0;
  int max_smem = 0;
  cudaStream_t stream = nullptr;       // kernels
  cudaStream_t copy_stream = nullptr;  // host -> device staging
  cudaStream_t copy_stream2 = nullptr; // second host -> device stream (copies alternate)
  cudaStream_t d2h_stream = nullptr;   // device -> host results
  uint64_t budget = 0, used = 0;
  std::mutex mu;      // allocations, budget, caches
  std::mutex err_mu;  // last_error
  std::mutex call_mu; // serialises the host-staged entry points (shared staging buffers)
  std::string last_error;
  std::map<void*, uint64_t> allocs;
  std::map<std::pair<int, int>, int> occupancy;  // (kernel key, smem) -> CTAs per SM
  uint32_t* d_error = nullptr;               // device error flags of bounded waits
  int64_t wait_cycles = 0;                   // bounded-wait limit of launches (0: default)
  std::atomic<int> fail_allocs{0};           // injected failures of the next allocations
  // kernel launches made by the context (graph replays count one), multi-setting launches
  // and the settings they carried (cp_ctx_launch_counts)
  std::atomic<uint64_t> n_launches{0}, n_multi{0}, n_multi_settings{0};
  std::string gpu_name;                      // device name (tuning cache key)
  std::map<int, cp::PxChoice> px_tuned;      // pixel-thread kernel choices by key
  bool tune_loaded = false;                  // the tuning cache file has been read
  std::mutex tune_mu;                        // one tuning run at a time
  unsigned long long* d_warn = nullptr;      // device warning counter (host-staged calls)
  // host-staged composite: device copies of the frames and outputs, pinned staging
  cp::DevBuffer frames_dev, out_dev, blend_dev, dbg_dev;
  cp::PinnedBuffer pin_in, pin_out, pin_blend;
  std::vector<cudaEvent_t> band_events;
  // batch plans (graph-captured persistent launches)
  std::vector<std::unique_ptr<cp::BatchPlan>> plans;
  void* jpeg = nullptr;  // the JPEG decoder (cp_jpeg.cpp), created at the first JPEG call
};

namespace cp {

void ctx_error(cp_ctx* ctx, const char* fmt, ...);
int cuda_status(cp_ctx* ctx, cudaError_t e, const char* what);
int fade_lut(const cp_fade* f, int32_t n, int32_t frame_offset, float* out);
int prepare_stack(cp_ctx* ctx, const cp_stack* st, const cp_params* p,
                  const uint8_t* const* dev_frames, StackDev* d);
int launch_single(cp_ctx* ctx, const StackDev& d, cudaStream_t stream);
// The stack takes the pixel-thread kernels (RGB, aligned rows, no crop, integer or paired f32
// distances, shared memory for its frames).
bool px_eligible(cp_ctx* ctx, const StackDev& d);
inline void count_launches(cp_ctx* ctx, uint64_t n) { ctx->n_launches += n; }
// Several settings of one stack (and band): the pixel-kernel settings sharing their order
// statistics in multi-setting launches of up to kMultiMax, the rest one by one.
int launch_multi(cp_ctx* ctx, const std::vector<StackDev>& ds, cudaStream_t stream);
// The pixel-thread kernel with its measured (or cached, forced, static) configuration.
int launch_px(cp_ctx* ctx, const StackDev& d, cudaStream_t stream);
int check_device_error(cp_ctx* ctx);
int budget_reserve(cp_ctx* ctx, uint64_t bytes);
void budget_release(cp_ctx* ctx, uint64_t bytes);
int dev_alloc(cp_ctx* ctx, uint64_t bytes, void** ptr);
// true (and one injected failure used up) when the next allocation must fail
bool injected_alloc_failure(cp_ctx* ctx);
int dev_free(cp_ctx* ctx, void* ptr);
int ensure_buffer(cp_ctx* ctx, DevBuffer& b, uint64_t bytes);
int ensure_pinned(cp_ctx* ctx, PinnedBuffer& b, uint64_t bytes);
bool is_pinned(const void* p);
void release_plans(cp_ctx* ctx);
void jpeg_release(cp_ctx* ctx);  // frees the context's JPEG decoder, if any
// Batched launches (cp_batch.cpp): the specialised batched kernel a stack takes (index in
// CP_BATCH_VARIANTS, -1: the general kernel), and one launch over device descriptors.
int batch_variant_key(const StackDev& d);
int batch_group_key(const StackDev& d);  // stacks with equal keys share a launch
int launch_batch_dispatch(cp_ctx* ctx, const std::vector<StackDev>& host, const StackDev* d_stacks,
                          const int32_t* d_prefix, int32_t total, int32_t interleave,
                          uint32_t* d_counter, int max_n, cudaStream_t st,
                          uint32_t* d_err);  // null: the context's error flag

}  // namespace cp
