// cuda_runtime.h (test double) — the subset of the CUDA runtime API that cp_server.cpp,
// cp_prepare.cpp and cp_memory.cpp call, for compiling those files on a machine without a
// GPU. Found ahead of the toolkit's header by the include path of the mock build
// (tests/test_server_mock.py). mock_device.cpp implements it over host memory: streams are
// in-order queues that a host thread executes, events complete when that thread reaches them,
// and the tests hold, release or fail the queued work through the mock_* controls.
#pragma once

#include <stddef.h>

enum cudaError {
  cudaSuccess = 0,
  cudaErrorInvalidValue = 1,
  cudaErrorMemoryAllocation = 2,
  cudaErrorInvalidResourceHandle = 400,
  cudaErrorNotReady = 600,
  cudaErrorIllegalAddress = 700,
  cudaErrorLaunchTimeout = 702,
};
typedef enum cudaError cudaError_t;

enum cudaMemcpyKind {
  cudaMemcpyHostToHost = 0,
  cudaMemcpyHostToDevice = 1,
  cudaMemcpyDeviceToHost = 2,
  cudaMemcpyDeviceToDevice = 3,
};

enum cudaMemAllocationType { cudaMemAllocationTypeInvalid = 0, cudaMemAllocationTypePinned = 1 };
enum cudaMemLocationType { cudaMemLocationTypeInvalid = 0, cudaMemLocationTypeDevice = 1 };
enum cudaMemPoolAttr { cudaMemPoolAttrReleaseThreshold = 4 };
enum cudaMemoryType {
  cudaMemoryTypeUnregistered = 0,
  cudaMemoryTypeHost = 1,
  cudaMemoryTypeDevice = 2,
};

struct cudaMemLocation {
  enum cudaMemLocationType type;
  int id;
};
struct cudaMemPoolProps {
  enum cudaMemAllocationType allocType;
  int handleTypes;
  struct cudaMemLocation location;
  void* win32SecurityAttributes;
  size_t maxSize;
  unsigned short usage;
  unsigned char reserved[54];
};
struct cudaPointerAttributes {
  enum cudaMemoryType type;
  int device;
  void* devicePointer;
  void* hostPointer;
};

typedef struct MockStream* cudaStream_t;
typedef struct MockEvent* cudaEvent_t;
typedef struct MockPool* cudaMemPool_t;
typedef struct MockGraph* cudaGraph_t;
typedef struct MockGraphExec* cudaGraphExec_t;

#define cudaStreamNonBlocking 0x01
#define cudaEventDisableTiming 0x02
#define cudaHostAllocPortable 0x01

extern "C" {
const char* cudaGetErrorString(cudaError_t e);
cudaError_t cudaGetLastError(void);
cudaError_t cudaSetDevice(int device);
cudaError_t cudaStreamCreateWithFlags(cudaStream_t* s, unsigned int flags);
cudaError_t cudaStreamDestroy(cudaStream_t s);
cudaError_t cudaStreamSynchronize(cudaStream_t s);
cudaError_t cudaStreamWaitEvent(cudaStream_t s, cudaEvent_t e, unsigned int flags);
cudaError_t cudaEventCreateWithFlags(cudaEvent_t* e, unsigned int flags);
cudaError_t cudaEventDestroy(cudaEvent_t e);
cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t s);
cudaError_t cudaEventQuery(cudaEvent_t e);
cudaError_t cudaEventSynchronize(cudaEvent_t e);
cudaError_t cudaMemcpyAsync(void* dst, const void* src, size_t bytes, enum cudaMemcpyKind kind,
                            cudaStream_t s);
cudaError_t cudaMemsetAsync(void* dst, int value, size_t bytes, cudaStream_t s);
cudaError_t cudaMemcpy(void* dst, const void* src, size_t bytes, enum cudaMemcpyKind kind);
cudaError_t cudaMemset(void* dst, int value, size_t bytes);
cudaError_t cudaMalloc(void** p, size_t bytes);
cudaError_t cudaFree(void* p);
cudaError_t cudaHostAlloc(void** p, size_t bytes, unsigned int flags);
cudaError_t cudaFreeHost(void* p);
cudaError_t cudaPointerGetAttributes(struct cudaPointerAttributes* a, const void* p);
cudaError_t cudaMemPoolCreate(cudaMemPool_t* pool, const struct cudaMemPoolProps* props);
cudaError_t cudaMemPoolDestroy(cudaMemPool_t pool);
cudaError_t cudaMemPoolSetAttribute(cudaMemPool_t pool, enum cudaMemPoolAttr attr, void* value);
cudaError_t cudaMallocFromPoolAsync(void** p, size_t bytes, cudaMemPool_t pool, cudaStream_t s);
cudaError_t cudaFreeAsync(void* p, cudaStream_t s);
}
