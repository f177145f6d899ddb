// cp_static.cu — batched compositing without any device allocation.
//
// Some callers cannot call cudaMalloc: code running while a CUDA graph is being captured,
// plug-ins inside a host application whose allocator owns all device memory, or services
// that must not grow their footprint after start-up. cp_composite_batch_static serves them:
// the batched kernel's scratch (stack descriptors, tile prefix sums, the work counter and an
// error flag) lives in one file-scope __device__ array of fixed size instead of memory from
// a context. The caller passes device inputs and outputs as for cp_composite_batch_device.

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/chrono_gpu.h"
#include "cp_host_internal.h"
#include "cp_internal.h"

namespace cp {
namespace {

constexpr int kMaxStaticDevices = 64;
constexpr size_t kDescBytes = sizeof(StackDev) * CP_STATIC_MAX_STACKS;
constexpr size_t kPrefixOffset = (kDescBytes + 255) / 256 * 256;
constexpr size_t kCounterOffset = kPrefixOffset + 256 * ((sizeof(int32_t) * (CP_STATIC_MAX_STACKS + 1) + 255) / 256);
constexpr size_t kScratchBytes = kCounterOffset + 256;  // counter at +0, error flag at +4

// Held by every GPU that loads the library, for the life of the process.
static __device__ __align__(256) unsigned char g_static_scratch[kScratchBytes];

std::mutex g_setup_mu;
void* g_scratch_ptr[kMaxStaticDevices] = {};

// Device address of the scratch array on `device` (the current device), looked up once.
int scratch_address(int device, unsigned char** out) {
  if (device < 0 || device >= kMaxStaticDevices) return CP_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_ptr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || !p) return CP_ERR_CUDA;
    g_scratch_ptr[device] = p;
  }
  *out = static_cast<unsigned char*>(g_scratch_ptr[device]);
  return CP_OK;
}

}  // namespace
}  // namespace cp

using namespace cp;

extern "C" int cp_composite_batch_static(const cp_stack* stacks, const cp_params* params,
                                         int32_t n_stacks, uint8_t* const* outs,
                                         uint8_t* const* out_blends, uint64_t* warnings,
                                         void* stream) {
  if (!stacks || !params || !outs || n_stacks < 1) return CP_ERR_ARG;
  if (n_stacks > CP_STATIC_MAX_STACKS) return CP_ERR_LIMIT;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return CP_ERR_NODEV;
  int major = 0, minor = 0, sms = 0, max_smem = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  if (major != 10 || minor != 3) return CP_ERR_NODEV;
  unsigned char* scratch = nullptr;
  int rc = scratch_address(device, &scratch);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int channels = stacks[0].channels;
  int32_t prefix[CP_STATIC_MAX_STACKS + 1];
  prefix[0] = 0;
  int max_n = 0;
  StackDev d;  // prepared one at a time and copied into the scratch array
  const uint8_t* fr[CP_MAX_FRAMES];
  for (int i = 0; i < n_stacks; ++i) {
    const cp_stack& s = stacks[i];
    if (s.channels != channels || s.n < 1 || s.n > CP_MAX_FRAMES || !outs[i] ||
        (!s.frames && !s.base))
      return CP_ERR_ARG;
    for (int f = 0; f < s.n; ++f) fr[f] = s.frames ? s.frames[f] : s.base + s.frame_stride * f;
    rc = prepare_stack(nullptr, &s, &params[i], fr, &d);
    if (rc) return rc;
    d.out = outs[i];
    d.blend = (out_blends && params[i].mode == CP_MODE_OUTLIER) ? out_blends[i] : nullptr;
    d.warnings = warnings ? reinterpret_cast<unsigned long long*>(warnings + i) : nullptr;
    if (max_n < s.n) max_n = s.n;
    if (static_cast<int64_t>(prefix[i]) + d.tiles > 0x7FFFFFFF) return CP_ERR_LIMIT;
    prefix[i + 1] = prefix[i] + d.tiles;
    // pageable source: the call returns once `d` has been read, so it can be reused
    const cudaError_t e = cudaMemcpyAsync(scratch + sizeof(StackDev) * i, &d, sizeof(StackDev),
                                          cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return CP_ERR_CUDA;
  }
  const int smem = smem_bytes_for(max_n, channels);
  if (smem > max_smem) return CP_ERR_ARG;
  uint32_t* counter = reinterpret_cast<uint32_t*>(scratch + kCounterOffset);
  uint32_t* error = counter + 1;
  cudaError_t e = cudaMemcpyAsync(scratch + kPrefixOffset, prefix, sizeof(int32_t) * (n_stacks + 1),
                                  cudaMemcpyHostToDevice, st);
  // the work counter and the error flag must start at zero: the array keeps the last call's
  if (e == cudaSuccess) e = cudaMemsetAsync(counter, 0, 2 * sizeof(uint32_t), st);
  if (e != cudaSuccess) return CP_ERR_CUDA;
  int per_sm = 1;
  switch (channels) {
    case 1: per_sm = composite_max_ctas_c1(cta_threads(1), smem); break;
    case 3: per_sm = composite_max_ctas_c3(cta_threads(3), smem); break;
    case 4: per_sm = composite_max_ctas_c4(cta_threads(4), smem); break;
    default: return CP_ERR_ARG;
  }
  const int grid = prefix[n_stacks] < per_sm * sms ? prefix[n_stacks] : per_sm * sms;
  const StackDev* d_stacks = reinterpret_cast<const StackDev*>(scratch);
  const int32_t* d_prefix = reinterpret_cast<const int32_t*>(scratch + kPrefixOffset);
  switch (channels) {
    case 1: rc = launch_batch_c1(d_stacks, d_prefix, n_stacks, prefix[n_stacks], 0, counter, error, grid > 0 ? grid : 1, smem, st); break;
    case 3: rc = launch_batch_c3(d_stacks, d_prefix, n_stacks, prefix[n_stacks], 0, counter, error, grid > 0 ? grid : 1, smem, st); break;
    default: rc = launch_batch_c4(d_stacks, d_prefix, n_stacks, prefix[n_stacks], 0, counter, error, grid > 0 ? grid : 1, smem, st); break;
  }
  return rc == 0 ? CP_OK : CP_ERR_CUDA;
}
