// mock_device.cpp (test double) — a host-memory stand-in for the CUDA runtime and for the
// batched compositing launch, so that the compositing server (cp_server.cpp), with the real
// option preparation (cp_prepare.cpp) and memory accounting (cp_memory.cpp), runs on a machine
// without a GPU.
//
// Execution model. A stream is an in-order queue of operations; one host thread (the "device")
// runs the front operation of every stream whose turn has come, so copies, kernels and event
// records complete asynchronously with respect to the caller, as on a GPU. A wait on an event
// blocks its stream until the event's last record has run. Tests hold uploads, kernels or
// downloads (mock_hold), make launches report a device-side wait that gave up (their error
// word, mock_fail_launch_words), raise a sticky device fault (mock_fault_launches: every later
// call reports it, as after an illegal address), cap the memory pool (mock_set_pool_limit) and
// fail allocations the way the runtime reports a full device or host (mock_fail_allocs).
//
// Checks. Every copy and kernel checks at run time that its device ranges lie inside live
// allocations; memory freed with cudaFreeAsync is poisoned (0xCD) and kept until mock_reset,
// so a use after free shows up as a misuse count or as wrong output, never as a crash. Events,
// streams and pools are never freed before mock_reset either: a destroyed handle that is used
// again is counted as misuse. mock_stats reports these counts and the live objects.
//
// The mock kernel (launch_batch_dispatch) computes, per stack, the byte-wise maximum of its
// frames into `out` and the byte-wise minimum into `blend`, and adds the frame count to the
// stack's warning counter: enough to check that every frame, output and counter of every job
// went to the right place.

#include "cuda_runtime.h"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/chrono_gpu.h"
#include "../../chrono_photo_gb300/csrc/cp_host_internal.h"
#include "../../chrono_photo_gb300/csrc/cp_internal.h"

using cp::StackDev;

struct MockEvent {
  uint64_t recorded = 0;   // records issued
  uint64_t completed = 0;  // records run by the device
  bool destroyed = false;
};

enum MockOpKind { kUpload, kDownload, kCopyOther, kMemset, kKernel, kRecord, kWait, kFree };

struct MockOp {
  MockOpKind kind;
  std::function<void()> run;  // copies, memsets, kernels, frees (called under the state lock)
  MockEvent* ev = nullptr;    // record, wait
  uint64_t gen = 0;
};

struct MockStream {
  std::deque<MockOp> q;
  bool destroyed = false;
};
struct MockPool {
  bool destroyed = false;
};

namespace {

enum Stat {
  kStUploads,          // host->device copies issued
  kStUploadBytes,
  kStDownloads,        // device->host copies issued
  kStLaunches,         // kernels issued
  kStLaunchesRun,      // kernels run
  kStLiveEvents,
  kStLiveStreams,
  kStLivePools,
  kStPoolBytes,        // live bytes from cudaMallocFromPoolAsync (freed when the free runs)
  kStLiveHost,         // live cudaHostAlloc buffers
  kStLiveDev,          // live cudaMalloc buffers
  kStMisuse,           // bad handle, range outside live memory, double free, sync timeout
  kStMaxPending,       // most kernels issued but not yet run, at any time
  kStStacks,           // stacks over all kernels issued
  kStMaxStacks,        // most stacks in one kernel
  kStCount
};

struct State {
  std::mutex mu;
  std::condition_variable cv;  // signalled when the device ran something
  std::thread device;
  bool stop = false;
  unsigned hold = 0;  // 1 uploads, 2 kernels, 4 downloads
  cudaError_t sticky = cudaSuccess;
  int fail_words = 0, fault_launches = 0;
  unsigned fail_kinds = 0;  // allocations that fail: 1 pool, 2 cudaMalloc, 4 cudaHostAlloc
  int fail_allocs = 0;      // how many more of them fail
  uint64_t pool_limit = 0;  // 0: no limit
  std::vector<MockStream*> streams;
  std::vector<MockEvent*> events;
  std::vector<MockPool*> pools;
  std::map<uintptr_t, size_t> pool_live, dev_live, host_live;
  std::vector<void*> retired;  // freed memory, poisoned, released by mock_reset
  uint64_t pending_launches = 0;
  uint64_t stat[kStCount] = {};
};

State& S() {
  static State* s = new State();  // never destroyed: the device thread may outlive statics
  return *s;
}

bool in_map(const std::map<uintptr_t, size_t>& m, const void* p, size_t bytes) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(p);
  auto it = m.upper_bound(a);
  if (it == m.begin()) return false;
  --it;
  return a >= it->first && a + bytes <= it->first + it->second;
}
// [p, p + bytes) inside live device memory (a pool or cudaMalloc allocation)
bool dev_range(State& s, const void* p, size_t bytes) {
  return in_map(s.pool_live, p, bytes) || in_map(s.dev_live, p, bytes);
}

bool held(const State& s, MockOpKind k) {
  if (k == kUpload) return s.hold & 1u;
  if (k == kKernel) return s.hold & 2u;
  if (k == kDownload) return s.hold & 4u;
  return false;
}

bool runnable(const State& s, const MockStream* st) {
  if (st->q.empty()) return false;
  const MockOp& op = st->q.front();
  if (op.kind == kWait) return op.ev->completed >= op.gen;
  return !held(s, op.kind);
}

void device_loop() {
  State& s = S();
  std::unique_lock<std::mutex> lk(s.mu);
  while (!s.stop) {
    bool any = false;
    for (size_t i = 0; i < s.streams.size() && s.sticky == cudaSuccess; ++i) {
      MockStream* st = s.streams[i];
      while (s.sticky == cudaSuccess && runnable(s, st)) {
        MockOp op = std::move(st->q.front());
        st->q.pop_front();
        if (op.kind == kRecord) op.ev->completed = std::max(op.ev->completed, op.gen);
        if (op.run) op.run();
        any = true;
      }
    }
    if (any)
      s.cv.notify_all();
    else
      s.cv.wait_for(lk, std::chrono::milliseconds(1));
  }
}

void enqueue(State& s, MockStream* st, MockOp op) {
  st->q.push_back(std::move(op));
  s.cv.notify_all();
}

bool bad_stream(State& s, cudaStream_t st) {
  if (st && !st->destroyed) return false;
  s.stat[kStMisuse] += 1;
  return true;
}
bool bad_event(State& s, cudaEvent_t e) {
  if (e && !e->destroyed) return false;
  s.stat[kStMisuse] += 1;
  return true;
}

// Waits (bounded) until `done` holds or the device has faulted.
template <class F>
cudaError_t wait_device(State& s, std::unique_lock<std::mutex>& lk, F done) {
  const auto limit = std::chrono::steady_clock::now() + std::chrono::seconds(10);
  while (!done() && s.sticky == cudaSuccess) {
    if (s.cv.wait_until(lk, limit) == std::cv_status::timeout && !done()) {
      s.stat[kStMisuse] += 1;  // held work never released, or a wait that can never end
      return cudaErrorLaunchTimeout;
    }
  }
  return s.sticky;
}

void* mock_malloc(size_t bytes) { return std::malloc(bytes ? bytes : 1); }

// One failure of an allocation of kind `k` is due (and used up).
bool alloc_fails(State& s, unsigned k) {
  if (!(s.fail_kinds & k) || s.fail_allocs <= 0) return false;
  s.fail_allocs -= 1;
  return true;
}

// Poisons and retires an allocation of `m` (it stays mapped until mock_reset).
bool retire(State& s, std::map<uintptr_t, size_t>& m, void* p) {
  auto it = m.find(reinterpret_cast<uintptr_t>(p));
  if (it == m.end()) {
    s.stat[kStMisuse] += 1;
    return false;
  }
  std::memset(p, 0xCD, it->second);
  s.retired.push_back(p);
  m.erase(it);
  return true;
}

// The kernel: per stack, byte-wise max of the frames into out, min into blend, n warnings.
void run_kernel(State& s, const StackDev* d_stacks, const int32_t* d_prefix, int nb,
                int32_t total, uint32_t* d_err, bool fail_word) {
  if (!dev_range(s, d_stacks, sizeof(StackDev) * nb) ||
      !dev_range(s, d_prefix, sizeof(int32_t) * (nb + 1))) {
    s.stat[kStMisuse] += 1;
    return;
  }
  if (d_prefix[0] != 0 || d_prefix[nb] != total) s.stat[kStMisuse] += 1;
  for (int k = 0; k < nb; ++k) {
    const StackDev& d = d_stacks[k];
    if (d_prefix[k + 1] - d_prefix[k] != d.tiles) s.stat[kStMisuse] += 1;
    const size_t bytes = static_cast<size_t>(d.width) * d.height * d.channels;
    bool ok = dev_range(s, d.out, bytes) && dev_range(s, d.warnings, 8) &&
              (!d.blend || dev_range(s, d.blend, bytes)) && !d.has_crop;
    for (int i = 0; i < d.n && ok; ++i) ok = dev_range(s, d.frames[i], bytes);
    if (!ok) {
      s.stat[kStMisuse] += 1;
      continue;
    }
    for (size_t b = 0; b < bytes; ++b) {
      uint8_t hi = 0, lo = 255;
      for (int i = 0; i < d.n; ++i) {
        hi = std::max(hi, d.frames[i][b]);
        lo = std::min(lo, d.frames[i][b]);
      }
      d.out[b] = hi;
      if (d.blend) d.blend[b] = lo;
    }
    *d.warnings += static_cast<unsigned long long>(d.n);
  }
  if (fail_word) {
    if (dev_range(s, d_err, 4))
      *d_err = 1u;
    else
      s.stat[kStMisuse] += 1;
  }
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// Runtime API
// ---------------------------------------------------------------------------------------------
extern "C" {

const char* cudaGetErrorString(cudaError_t e) {
  switch (e) {
    case cudaSuccess: return "no error";
    case cudaErrorInvalidValue: return "invalid argument";
    case cudaErrorMemoryAllocation: return "out of memory";
    case cudaErrorInvalidResourceHandle: return "invalid resource handle";
    case cudaErrorNotReady: return "device not ready";
    case cudaErrorIllegalAddress: return "an illegal memory access was encountered (mock)";
    case cudaErrorLaunchTimeout: return "the mock device did not finish in time";
    default: return "unknown error";
  }
}

cudaError_t cudaGetLastError(void) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  return s.sticky;  // a sticky fault is not cleared
}

cudaError_t cudaSetDevice(int) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  return s.sticky;
}

cudaError_t cudaStreamCreateWithFlags(cudaStream_t* st, unsigned int) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (s.sticky) return s.sticky;
  *st = new MockStream();
  s.streams.push_back(*st);
  s.stat[kStLiveStreams] += 1;
  return cudaSuccess;
}

cudaError_t cudaStreamDestroy(cudaStream_t st) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (bad_stream(s, st)) return cudaErrorInvalidResourceHandle;
  st->destroyed = true;  // queued work still runs, as on the device
  s.stat[kStLiveStreams] -= 1;
  return cudaSuccess;
}

cudaError_t cudaStreamSynchronize(cudaStream_t st) {
  State& s = S();
  std::unique_lock<std::mutex> lk(s.mu);
  if (bad_stream(s, st)) return cudaErrorInvalidResourceHandle;
  return wait_device(s, lk, [&] { return st->q.empty(); });
}

cudaError_t cudaStreamWaitEvent(cudaStream_t st, cudaEvent_t e, unsigned int) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (bad_stream(s, st) || bad_event(s, e)) return cudaErrorInvalidResourceHandle;
  if (s.sticky) return s.sticky;
  MockOp op{kWait, nullptr, e, e->recorded};
  enqueue(s, st, std::move(op));
  return cudaSuccess;
}

cudaError_t cudaEventCreateWithFlags(cudaEvent_t* e, unsigned int) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (s.sticky) return s.sticky;
  *e = new MockEvent();
  s.events.push_back(*e);
  s.stat[kStLiveEvents] += 1;
  return cudaSuccess;
}

cudaError_t cudaEventDestroy(cudaEvent_t e) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (bad_event(s, e)) return cudaErrorInvalidResourceHandle;
  e->destroyed = true;  // records and waits already queued still run
  s.stat[kStLiveEvents] -= 1;
  return cudaSuccess;
}

cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t st) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (bad_stream(s, st) || bad_event(s, e)) return cudaErrorInvalidResourceHandle;
  if (s.sticky) return s.sticky;
  e->recorded += 1;
  MockOp op{kRecord, nullptr, e, e->recorded};
  enqueue(s, st, std::move(op));
  return cudaSuccess;
}

cudaError_t cudaEventQuery(cudaEvent_t e) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (bad_event(s, e)) return cudaErrorInvalidResourceHandle;
  if (s.sticky) return s.sticky;
  return e->completed >= e->recorded ? cudaSuccess : cudaErrorNotReady;
}

cudaError_t cudaEventSynchronize(cudaEvent_t e) {
  State& s = S();
  std::unique_lock<std::mutex> lk(s.mu);
  if (bad_event(s, e)) return cudaErrorInvalidResourceHandle;
  const uint64_t gen = e->recorded;
  return wait_device(s, lk, [&] { return e->completed >= gen; });
}

cudaError_t cudaMemcpyAsync(void* dst, const void* src, size_t bytes, enum cudaMemcpyKind kind,
                            cudaStream_t st) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (bad_stream(s, st)) return cudaErrorInvalidResourceHandle;
  if (s.sticky) return s.sticky;
  State* ps = &s;
  MockOpKind k = kCopyOther;
  if (kind == cudaMemcpyHostToDevice) {
    k = kUpload;
    s.stat[kStUploads] += 1;
    s.stat[kStUploadBytes] += bytes;
  } else if (kind == cudaMemcpyDeviceToHost) {
    k = kDownload;
    s.stat[kStDownloads] += 1;
  }
  MockOp op{k, [ps, dst, src, bytes, kind] {
              const bool ok = (kind != cudaMemcpyHostToDevice || dev_range(*ps, dst, bytes)) &&
                              (kind != cudaMemcpyDeviceToHost || dev_range(*ps, src, bytes));
              if (ok)
                std::memcpy(dst, src, bytes);
              else
                ps->stat[kStMisuse] += 1;
            }};
  enqueue(s, st, std::move(op));
  return cudaSuccess;
}

cudaError_t cudaMemsetAsync(void* dst, int value, size_t bytes, cudaStream_t st) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (bad_stream(s, st)) return cudaErrorInvalidResourceHandle;
  if (s.sticky) return s.sticky;
  State* ps = &s;
  MockOp op{kMemset, [ps, dst, value, bytes] {
              if (dev_range(*ps, dst, bytes))
                std::memset(dst, value, bytes);
              else
                ps->stat[kStMisuse] += 1;
            }};
  enqueue(s, st, std::move(op));
  return cudaSuccess;
}

cudaError_t cudaMemcpy(void* dst, const void* src, size_t bytes, enum cudaMemcpyKind) {
  State& s = S();
  std::unique_lock<std::mutex> lk(s.mu);
  // synchronous: after all queued work, as on the legacy default stream
  cudaError_t e = wait_device(s, lk, [&] {
    for (MockStream* st : s.streams)
      if (!st->q.empty()) return false;
    return true;
  });
  if (e) return e;
  std::memcpy(dst, src, bytes);
  return cudaSuccess;
}

cudaError_t cudaMemset(void* dst, int value, size_t bytes) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (s.sticky) return s.sticky;
  std::memset(dst, value, bytes);
  return cudaSuccess;
}

cudaError_t cudaMalloc(void** p, size_t bytes) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (s.sticky) return s.sticky;
  if (alloc_fails(s, 2u)) return cudaErrorMemoryAllocation;
  *p = mock_malloc(bytes);
  s.dev_live[reinterpret_cast<uintptr_t>(*p)] = bytes;
  s.stat[kStLiveDev] += 1;
  return cudaSuccess;
}

cudaError_t cudaFree(void* p) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (!p) return cudaSuccess;
  if (!retire(s, s.dev_live, p)) return cudaErrorInvalidValue;
  s.stat[kStLiveDev] -= 1;
  return s.sticky;
}

cudaError_t cudaHostAlloc(void** p, size_t bytes, unsigned int) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (s.sticky) return s.sticky;
  if (alloc_fails(s, 4u)) return cudaErrorMemoryAllocation;
  *p = mock_malloc(bytes);
  s.host_live[reinterpret_cast<uintptr_t>(*p)] = bytes;
  s.stat[kStLiveHost] += 1;
  return cudaSuccess;
}

cudaError_t cudaFreeHost(void* p) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (!p) return cudaSuccess;
  if (!retire(s, s.host_live, p)) return cudaErrorInvalidValue;
  s.stat[kStLiveHost] -= 1;
  return cudaSuccess;
}

cudaError_t cudaPointerGetAttributes(struct cudaPointerAttributes* a, const void* p) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  std::memset(a, 0, sizeof *a);
  a->type = in_map(s.host_live, p, 1) ? cudaMemoryTypeHost
            : dev_range(s, p, 1)      ? cudaMemoryTypeDevice
                                      : cudaMemoryTypeUnregistered;
  return cudaSuccess;
}

cudaError_t cudaMemPoolCreate(cudaMemPool_t* pool, const struct cudaMemPoolProps*) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (s.sticky) return s.sticky;
  *pool = new MockPool();
  s.pools.push_back(*pool);
  s.stat[kStLivePools] += 1;
  return cudaSuccess;
}

cudaError_t cudaMemPoolDestroy(cudaMemPool_t pool) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (!pool || pool->destroyed) {
    s.stat[kStMisuse] += 1;
    return cudaErrorInvalidResourceHandle;
  }
  pool->destroyed = true;
  s.stat[kStLivePools] -= 1;
  return cudaSuccess;
}

cudaError_t cudaMemPoolSetAttribute(cudaMemPool_t pool, enum cudaMemPoolAttr, void*) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (!pool || pool->destroyed) {
    s.stat[kStMisuse] += 1;
    return cudaErrorInvalidResourceHandle;
  }
  return cudaSuccess;
}

cudaError_t cudaMallocFromPoolAsync(void** p, size_t bytes, cudaMemPool_t pool, cudaStream_t st) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (!pool || pool->destroyed || bad_stream(s, st)) return cudaErrorInvalidResourceHandle;
  if (s.sticky) return s.sticky;
  if (alloc_fails(s, 1u) || (s.pool_limit && s.stat[kStPoolBytes] + bytes > s.pool_limit))
    return cudaErrorMemoryAllocation;
  *p = mock_malloc(bytes);
  s.pool_live[reinterpret_cast<uintptr_t>(*p)] = bytes;
  s.stat[kStPoolBytes] += bytes;
  return cudaSuccess;
}

cudaError_t cudaFreeAsync(void* p, cudaStream_t st) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (bad_stream(s, st)) return cudaErrorInvalidResourceHandle;
  State* ps = &s;
  MockOp op{kFree, [ps, p] {
              auto it = ps->pool_live.find(reinterpret_cast<uintptr_t>(p));
              const size_t bytes = it == ps->pool_live.end() ? 0 : it->second;
              if (retire(*ps, ps->pool_live, p)) ps->stat[kStPoolBytes] -= bytes;
            }};
  enqueue(s, st, std::move(op));
  return cudaSuccess;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// The launch the server makes (cp_batch.cpp on a GPU)
// ---------------------------------------------------------------------------------------------
namespace cp {

int batch_group_key(const StackDev& d) { return d.nw; }

int launch_batch_dispatch(cp_ctx* ctx, const std::vector<StackDev>& host, const StackDev* d_stacks,
                          const int32_t* d_prefix, int32_t total, int32_t, uint32_t*, int,
                          cudaStream_t st, uint32_t* d_err) {
  State& s = S();
  cudaError_t fault = cudaSuccess;
  {
    std::lock_guard<std::mutex> lk(s.mu);
    if (bad_stream(s, st)) {
      fault = cudaErrorInvalidResourceHandle;
    } else if (s.sticky) {
      fault = s.sticky;
    } else {
      const int nb = static_cast<int>(host.size());
      const bool fail_word = s.fail_words > 0;
      if (fail_word) s.fail_words -= 1;
      const bool raise = s.fault_launches > 0;
      if (raise) s.fault_launches -= 1;
      State* ps = &s;
      MockOp op{kKernel, [ps, d_stacks, d_prefix, nb, total, d_err, fail_word, raise] {
                  ps->pending_launches -= 1;
                  ps->stat[kStLaunchesRun] += 1;
                  if (raise) {
                    ps->sticky = cudaErrorIllegalAddress;
                    return;
                  }
                  run_kernel(*ps, d_stacks, d_prefix, nb, total, d_err, fail_word);
                }};
      s.stat[kStLaunches] += 1;
      s.stat[kStStacks] += static_cast<uint64_t>(nb);
      s.stat[kStMaxStacks] = std::max<uint64_t>(s.stat[kStMaxStacks], static_cast<uint64_t>(nb));
      s.pending_launches += 1;
      s.stat[kStMaxPending] = std::max(s.stat[kStMaxPending], s.pending_launches);
      enqueue(s, st, std::move(op));
    }
  }
  if (fault) return cuda_status(ctx, fault, "batched launch");
  count_launches(ctx, 1);
  return CP_OK;
}

}  // namespace cp

// ---------------------------------------------------------------------------------------------
// Test controls
// ---------------------------------------------------------------------------------------------
extern "C" {

// A context as cp_ctx_create makes it, without a device (streams and kernels are not used by
// the server; it makes its own).
cp_ctx* mock_ctx_create(uint64_t hbm_budget) {
  cp_ctx* ctx = new cp_ctx();
  ctx->device = 0;
  ctx->sm_count = 152;
  ctx->max_smem = 232448;
  ctx->budget = hbm_budget;
  return ctx;
}
void mock_ctx_destroy(cp_ctx* ctx) { delete ctx; }
uint64_t mock_ctx_used(cp_ctx* ctx) {
  std::lock_guard<std::mutex> lk(ctx->mu);
  return ctx->used;
}
uint64_t mock_ctx_launches(cp_ctx* ctx) { return ctx->n_launches.load(); }

// Stops the device, drops every queued operation and frees everything the mock holds; then
// starts a fresh device. Call only with no server alive.
void mock_reset(void) {
  State& s = S();
  {
    std::lock_guard<std::mutex> lk(s.mu);
    s.stop = true;
    s.cv.notify_all();
  }
  if (s.device.joinable()) s.device.join();
  std::lock_guard<std::mutex> lk(s.mu);
  for (MockStream* st : s.streams) delete st;
  for (MockEvent* e : s.events) delete e;
  for (MockPool* p : s.pools) delete p;
  for (auto& kv : s.pool_live) std::free(reinterpret_cast<void*>(kv.first));
  for (auto& kv : s.dev_live) std::free(reinterpret_cast<void*>(kv.first));
  for (auto& kv : s.host_live) std::free(reinterpret_cast<void*>(kv.first));
  for (void* p : s.retired) std::free(p);
  s.streams.clear();
  s.events.clear();
  s.pools.clear();
  s.pool_live.clear();
  s.dev_live.clear();
  s.host_live.clear();
  s.retired.clear();
  s.hold = 0;
  s.sticky = cudaSuccess;
  s.fail_words = s.fault_launches = 0;
  s.fail_kinds = 0;
  s.fail_allocs = 0;
  s.pool_limit = 0;
  s.pending_launches = 0;
  std::memset(s.stat, 0, sizeof s.stat);
  s.stop = false;
  s.device = std::thread(device_loop);
}

void mock_shutdown(void) {
  State& s = S();
  {
    std::lock_guard<std::mutex> lk(s.mu);
    s.stop = true;
    s.cv.notify_all();
  }
  if (s.device.joinable()) s.device.join();
}

void mock_hold(unsigned mask) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  s.hold = mask;
  s.cv.notify_all();
}
void mock_fail_launch_words(int count) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  s.fail_words = count;
}
void mock_fault_launches(int count) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  s.fault_launches = count;
}
// The next `count` allocations of the kinds in `mask` (1 pool, 2 cudaMalloc, 4 cudaHostAlloc)
// fail with cudaErrorMemoryAllocation, as the runtime reports a full device or host.
void mock_fail_allocs(unsigned mask, int count) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  s.fail_kinds = mask;
  s.fail_allocs = count;
}
void mock_set_pool_limit(uint64_t bytes) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  s.pool_limit = bytes;
}

// prepare_stack's derived descriptor fields for a stack and its options (frames at dummy
// device addresses), for host-only tests of the option semantics. ints: n, nw, n_sub, med_k,
// med_pair, q1_k, q1_pair, q3_k, q3_pair, fast_int, pair_f32, no_fade, unit_fade, wmask,
// thr_abs, thr_int[0..4] (20 values); floats: q1_frac, q3_frac, thr_min, thr_max, thr_scale,
// thr_sq, then fade[0..n-1]. Returns prepare_stack's status.
int mock_prepare(const cp_stack* st, const cp_params* p, int32_t* ints, float* floats) {
  if (!st || st->n < 1 || st->n > CP_MAX_FRAMES) return CP_ERR_ARG;
  std::vector<const uint8_t*> fr(static_cast<size_t>(st->n),
                                 reinterpret_cast<const uint8_t*>(uintptr_t(256)));
  StackDev d;
  const int rc = cp::prepare_stack(nullptr, st, p, fr.data(), &d);
  if (rc) return rc;
  const int32_t iv[] = {d.n, d.nw, d.n_sub, d.med_k, d.med_pair, d.q1_k, d.q1_pair, d.q3_k,
                        d.q3_pair, static_cast<int32_t>(d.fast_int),
                        static_cast<int32_t>(d.pair_f32), static_cast<int32_t>(d.no_fade),
                        static_cast<int32_t>(d.unit_fade), static_cast<int32_t>(d.wmask),
                        d.thr_abs, d.thr_int[0], d.thr_int[1], d.thr_int[2], d.thr_int[3],
                        d.thr_int[4]};
  std::memcpy(ints, iv, sizeof iv);
  const float fv[] = {d.q1_frac, d.q3_frac, d.thr_min, d.thr_max, d.thr_scale, d.thr_sq};
  std::memcpy(floats, fv, sizeof fv);
  for (int i = 0; i < d.n; ++i) floats[6 + i] = d.fade[i];
  return CP_OK;
}

// Copies up to n counters (the Stat order) into out; returns how many there are.
int mock_stats(uint64_t* out, int n) {
  State& s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  for (int i = 0; i < n && i < kStCount; ++i) out[i] = s.stat[i];
  return kStCount;
}

// Waits (up to timeout_ms) until no stream has an operation the device could run now.
int mock_wait_idle(int timeout_ms) {
  State& s = S();
  std::unique_lock<std::mutex> lk(s.mu);
  const auto limit = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms);
  for (;;) {
    bool busy = false;
    for (MockStream* st : s.streams)
      if (runnable(s, st)) busy = true;
    if (!busy || s.sticky) return 0;
    if (s.cv.wait_until(lk, limit) == std::cv_status::timeout) return -1;
  }
}

}  // extern "C"
