// cp_memory.cpp — device and pinned memory of a context: the HBM budget, allocation
// bookkeeping, injected allocation failures (cp_ctx_fail_allocations) and the grow-only
// buffers of the host-staged calls.

#include <cuda_runtime.h>

#include <map>
#include <mutex>

#include "../../include/chrono_gpu.h"
#include "cp_host_internal.h"
#include "cp_internal.h"

namespace cp {

int budget_reserve(cp_ctx* ctx, uint64_t bytes) {
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (ctx->budget && ctx->used + bytes > ctx->budget) {
    ctx_error(ctx, "HBM budget exceeded: %llu + %llu > %llu", (unsigned long long)ctx->used,
              (unsigned long long)bytes, (unsigned long long)ctx->budget);
    return CP_ERR_BUDGET;
  }
  ctx->used += bytes;
  return CP_OK;
}
void budget_release(cp_ctx* ctx, uint64_t bytes) {
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->used = bytes > ctx->used ? 0 : ctx->used - bytes;
}

bool injected_alloc_failure(cp_ctx* ctx) {
  if (!ctx) return false;
  int left = ctx->fail_allocs.load();
  while (left > 0) {
    if (ctx->fail_allocs.compare_exchange_weak(left, left - 1)) {
      ctx_error(ctx, "allocation failed (injected by cp_ctx_fail_allocations)");
      return true;
    }
  }
  return false;
}

int dev_alloc(cp_ctx* ctx, uint64_t bytes, void** ptr) {
  if (injected_alloc_failure(ctx)) return CP_ERR_OOM;
  if (!ptr) return CP_ERR_ARG;
  *ptr = nullptr;
  if (bytes == 0) return CP_OK;
  int rc = budget_reserve(ctx, bytes);
  if (rc) return rc;
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaMalloc(ptr, bytes);
  if (e != cudaSuccess) {
    budget_release(ctx, bytes);
    *ptr = nullptr;
    return cuda_status(ctx, e, "cudaMalloc");
  }
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->allocs[*ptr] = bytes;
  return CP_OK;
}

int dev_free(cp_ctx* ctx, void* ptr) {
  if (!ptr) return CP_OK;
  uint64_t bytes = 0;
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->allocs.find(ptr);
    if (it == ctx->allocs.end()) return CP_ERR_ARG;
    bytes = it->second;
    ctx->allocs.erase(it);
  }
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaFree(ptr);
  budget_release(ctx, bytes);
  return cuda_status(ctx, e, "cudaFree");
}

// Grows a context-owned device buffer to at least `bytes`.
int ensure_buffer(cp_ctx* ctx, DevBuffer& b, uint64_t bytes) {
  if (b.bytes >= bytes) return CP_OK;
  if (b.ptr) {
    int rc = dev_free(ctx, b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
    if (rc) return rc;
  }
  void* p = nullptr;
  int rc = dev_alloc(ctx, bytes, &p);
  if (rc) return rc;
  b.ptr = p;
  b.bytes = bytes;
  return CP_OK;
}

int ensure_pinned(cp_ctx* ctx, PinnedBuffer& b, uint64_t bytes) {
  if (b.bytes >= bytes) return CP_OK;
  if (b.ptr) cudaFreeHost(b.ptr);
  b.ptr = nullptr;
  b.bytes = 0;
  if (injected_alloc_failure(ctx)) return CP_ERR_OOM;
  cudaError_t e = cudaHostAlloc(&b.ptr, bytes, cudaHostAllocPortable);
  if (e != cudaSuccess) return cuda_status(ctx, e, "cudaHostAlloc");
  b.bytes = bytes;
  return CP_OK;
}

bool is_pinned(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

}  // namespace cp

extern "C" {

int cp_ctx_fail_allocations(cp_ctx* ctx, int32_t count) {
  if (!ctx || count < 0) return CP_ERR_ARG;
  ctx->fail_allocs.store(count);
  return CP_OK;
}

}  // extern "C"
