// cp_static.cu — batched compositing without any device allocation.
//
// Some callers cannot call cudaMalloc: plug-ins inside a host application whose allocator
// owns all device memory, or services that must not grow their footprint after start-up.
// cp_composite_batch_static serves them: the batched kernel's scratch (stack descriptors,
// tile prefix sums, the work counter and an error flag) lives in one file-scope __device__
// array of fixed size instead of memory from a context. The caller passes device inputs and
// outputs as for cp_composite_batch_device.
//
// The host-side descriptors reach the array as kernel parameters of a small copy kernel
// (k_static_fill): a launch copies its parameters when it is enqueued, so the call reads no
// host memory later and never waits for earlier work on the stream (a pageable
// cudaMemcpyAsync would do both).

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <cstring>

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
static_assert(sizeof(StackDev) % 16 == 0, "descriptors are copied in 16-byte words");
static_assert(kPrefixOffset % 16 == 0 && kCounterOffset % 16 == 0, "16-byte aligned regions");

// Held by every GPU that loads the library, for the life of the process.
static __device__ __align__(256) unsigned char g_static_scratch[kScratchBytes];

// One copy into the scratch array: `words` 16-byte words to byte offset `offset`. Four
// descriptors per launch keep the parameter block (and the caller's host stack frame that
// builds it) near 12 KB, well inside the 32 KB kernel-parameter limit.
constexpr int kFillDescs = 4;
constexpr int kFillWords = static_cast<int>(sizeof(StackDev) * kFillDescs / 16);
struct FillChunk {
  uint32_t offset;
  uint32_t words;
  uint32_t pad[2];
  uint4 data[kFillWords];
};
static_assert(sizeof(int32_t) * (CP_STATIC_MAX_STACKS + 1) + 16 <= sizeof(uint4) * kFillWords,
              "the prefix sums and the zeroed counter fit one chunk");

__global__ void k_static_fill(const __grid_constant__ FillChunk c, unsigned char* scratch) {
  uint4* dst = reinterpret_cast<uint4*>(scratch + c.offset);
  for (uint32_t i = threadIdx.x; i < c.words; i += blockDim.x) dst[i] = c.data[i];
}

// Device address of the scratch array on `device` (the current device), looked up on every
// call: a cached address would dangle after a device reset or a new primary context, and the
// lookup is cheap. The host-side name of the array is not a device address.
int scratch_address(int device, unsigned char** out) {
  if (device < 0 || device >= kMaxStaticDevices) return CP_ERR_ARG;
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
  if (e != cudaSuccess || !p) return CP_ERR_CUDA;
  *out = static_cast<unsigned char*>(p);
  return CP_OK;
}

int launch_fill(const FillChunk& c, unsigned char* scratch, cudaStream_t st) {
  k_static_fill<<<1, 256, 0, st>>>(c, scratch);
  return cudaGetLastError() == cudaSuccess ? CP_OK : CP_ERR_CUDA;
}

int current_sm103(int* device) {
  if (cudaGetDevice(device) != cudaSuccess) return CP_ERR_NODEV;
  int major = 0, minor = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, *device);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, *device);
  return (major == 10 && minor == 3) ? CP_OK : CP_ERR_NODEV;
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
  int rc = current_sm103(&device);
  if (rc) return rc;
  int sms = 0, max_smem = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  unsigned char* scratch = nullptr;
  rc = scratch_address(device, &scratch);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int channels = stacks[0].channels;
  // every argument is checked before anything is enqueued
  int32_t prefix[CP_STATIC_MAX_STACKS + 1];
  prefix[0] = 0;
  int max_n = 0;
  FillChunk chunk;
  const uint8_t* fr[CP_MAX_FRAMES];
  for (int pass = 0; pass < 2; ++pass) {
    for (int i = 0; i < n_stacks; ++i) {
      const cp_stack& s = stacks[i];
      if (s.channels != channels || s.n < 1 || s.n > CP_MAX_FRAMES || !outs[i] ||
          (!s.frames && !s.base))
        return CP_ERR_ARG;
      for (int f = 0; f < s.n; ++f) fr[f] = s.frames ? s.frames[f] : s.base + s.frame_stride * f;
      StackDev* d = reinterpret_cast<StackDev*>(chunk.data) + (i % kFillDescs);
      rc = prepare_stack(nullptr, &s, &params[i], fr, d);
      if (rc) return rc;
      d->out = outs[i];
      d->blend = (out_blends && params[i].mode == CP_MODE_OUTLIER) ? out_blends[i] : nullptr;
      d->warnings = warnings ? reinterpret_cast<unsigned long long*>(warnings + i) : nullptr;
      if (pass == 0) {
        if (max_n < s.n) max_n = s.n;
        if (static_cast<int64_t>(prefix[i]) + d->tiles > 0x7FFFFFFF) return CP_ERR_LIMIT;
        prefix[i + 1] = prefix[i] + d->tiles;
        continue;
      }
      // descriptors i - i % 4 .. i go up as the parameters of one copy launch
      if (i % kFillDescs == kFillDescs - 1 || i == n_stacks - 1) {
        const int first = i - i % kFillDescs;
        chunk.offset = static_cast<uint32_t>(sizeof(StackDev) * first);
        chunk.words = static_cast<uint32_t>(sizeof(StackDev) * (i - first + 1) / 16);
        rc = launch_fill(chunk, scratch, st);
        if (rc) return rc;
      }
    }
    if (pass == 0 && smem_bytes_for(max_n, channels) > max_smem) return CP_ERR_ARG;
  }
  const int smem = smem_bytes_for(max_n, channels);
  // the prefix sums, and the work counter and error flag, which must start at zero: the
  // array keeps the last call's contents
  std::memset(chunk.data, 0, sizeof(chunk.data));
  std::memcpy(chunk.data, prefix, sizeof(int32_t) * (n_stacks + 1));
  const uint32_t prefix_words = static_cast<uint32_t>((kCounterOffset - kPrefixOffset) / 16);
  chunk.offset = static_cast<uint32_t>(kPrefixOffset);
  chunk.words = prefix_words + 1;
  rc = launch_fill(chunk, scratch, st);
  if (rc) return rc;
  uint32_t* counter = reinterpret_cast<uint32_t*>(scratch + kCounterOffset);
  uint32_t* error = counter + 1;
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

extern "C" int cp_composite_batch_static_status(int32_t* status, void* stream) {
  if (!status) return CP_ERR_ARG;
  int device = 0;
  int rc = current_sm103(&device);
  if (rc) return rc;
  unsigned char* scratch = nullptr;
  rc = scratch_address(device, &scratch);
  if (rc) return rc;
  uint32_t flag = 0;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (cudaMemcpyAsync(&flag, scratch + kCounterOffset + 4, sizeof(flag), cudaMemcpyDeviceToHost,
                      st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return CP_ERR_CUDA;
  *status = flag ? CP_ERR_TIMEOUT : CP_OK;
  return CP_OK;
}
