// cp_server.cpp — continuous-batching compositing server.
//
// The reference composites one output at a time from temp files (src/main.rs:454-492,
// parallel over video frames with rayon, :254-261). The server instead keeps a queue of
// jobs and one worker thread that, on every turn:
//   1. admits queued jobs while launch slots and HBM budget allow: reserves device memory,
//      reuses frames already resident under the same caller key (shared windows), and
//      issues the host->device copies of the rest on two copy streams (frames alternate:
//      one stream of back-to-back copies leaves the host link idle between copies). Device
//      memory comes from a stream-ordered pool (cudaMallocFromPoolAsync / cudaFreeAsync), so
//      admitting and retiring jobs never synchronises the device;
//   2. gathers every admitted job whose frames have landed and runs all their tiles in one
//      persistent batched launch (per channel count) on the next of several compute streams,
//      so launches of newer jobs overlap older ones still on the device;
//   3. copies finished outputs back on a d2h stream, completes the jobs, releases their
//      memory (keyed frames stay cached until memory is needed) and wakes waiters.
// Per-job results do not depend on what else is in the batch: every (stack, tile) item is
// computed independently by the same kernel code as a single launch.

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/chrono_gpu.h"
#include "cp_host_internal.h"
#include "cp_internal.h"

using namespace cp;

namespace {

constexpr int kStreams = 3;       // compute streams launches rotate over
constexpr int kMaxBatch = 1024;   // stacks per launch

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

uint64_t round_up(uint64_t v, uint64_t a) { return (v + a - 1) / a * a; }

// Stream-ordered device memory from the server's pool, counted against the context budget.
int pool_alloc(cp_ctx* ctx, cudaMemPool_t pool, uint64_t bytes, cudaStream_t st, void** p) {
  *p = nullptr;
  if (injected_alloc_failure(ctx)) return CP_ERR_OOM;
  int rc = budget_reserve(ctx, bytes);
  if (rc) return rc;
  const cudaError_t e = cudaMallocFromPoolAsync(p, bytes, pool, st);
  if (e != cudaSuccess) {
    budget_release(ctx, bytes);
    *p = nullptr;
    return cuda_status(ctx, e, "cudaMallocFromPoolAsync");
  }
  return CP_OK;
}
// The memory's last users have completed (the worker saw their events).
void pool_free(cp_ctx* ctx, void* p, uint64_t bytes, cudaStream_t st) {
  if (!p) return;
  cudaFreeAsync(p, st);
  budget_release(ctx, bytes);
}

struct Frame {  // a device frame, shared by key
  void* dev = nullptr;
  uint64_t bytes = 0;
  int refs = 0;
  uint64_t last_use = 0;
  cudaEvent_t ready = nullptr;  // upload finished
};

struct Job {
  uint64_t id = 0;
  cp_job spec;  // deep-copied pointers below
  std::vector<const uint8_t*> host_frames;
  std::vector<uint64_t> keys;
  std::vector<int32_t> crop;
  std::vector<int32_t> fade_frames;
  std::vector<float> fade_values;
  std::vector<int32_t> sample;
  // device side
  std::vector<Frame*> frames;        // resident frames (keyed or private)
  std::vector<Frame*> private_frames;
  void* out_dev = nullptr;
  void* blend_dev = nullptr;
  unsigned long long* warn_dev = nullptr;
  uint8_t* stage = nullptr;  // pinned host staging of out | blend | warnings
  uint64_t stage_bytes = 0;
  uint64_t reserved = 0;
  int state = 0;  // 0 queued, 1 admitted (uploading), 2 launched, 3 done
  int vkey = -1;  // launch group: batched kernel of the job's settings and plane words
  cudaEvent_t staged = nullptr;   // own uploads and the warning-counter reset finished
  cudaEvent_t done_ev = nullptr;
  cp_job_result res{};
};

struct LaunchSlot {
  void* dev = nullptr;          // StackDev array + prefix + counter
  uint64_t bytes = 0;
  void* pinned = nullptr;       // host staging of the descriptors
  cudaEvent_t ev = nullptr;     // launch finished
  cudaEvent_t freed = nullptr;  // the results and the error word of the launch read back
  bool busy = false;
};

}  // namespace

struct cp_server {
  cp_ctx* ctx = nullptr;
  uint64_t budget = 0, reserved = 0;
  int max_inflight = 4;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  bool stopping = false;
  uint64_t next_id = 1, use_clock = 0;
  std::deque<Job*> queue;
  std::vector<Job*> active;
  std::unordered_map<uint64_t, std::unique_ptr<Job>> jobs;  // by id
  std::unordered_map<uint64_t, std::unique_ptr<Frame>> cache;  // keyed frames
  cudaStream_t compute[kStreams] = {};
  cudaStream_t h2d = nullptr, h2d2 = nullptr, d2h = nullptr;
  cudaMemPool_t pool = nullptr;  // frames and outputs
  int next_stream = 0;
  std::vector<LaunchSlot> slots;
  std::thread worker;
  int error = CP_OK;
  std::multimap<uint64_t, uint8_t*> pinned_free;  // reusable pinned staging buffers by size
};

namespace {

uint64_t frame_bytes_of(const Job& j) {
  const cp_stack& s = j.spec.stack;
  const int sw = s.crop ? s.src_width : s.width, sh = s.crop ? s.src_height : s.height;
  return static_cast<uint64_t>(sw) * sh * s.channels;
}
uint64_t frame_pitch_of(const Job& j) { return round_up(frame_bytes_of(j) + 16, 256); }
uint64_t out_bytes_of(const Job& j) {
  const cp_stack& s = j.spec.stack;
  return round_up(static_cast<uint64_t>(s.width) * s.height * s.channels, 256);
}

// Device bytes a job needs beyond frames already resident.
uint64_t job_need(cp_server* srv, const Job& j) {
  uint64_t need = 2 * out_bytes_of(j) + 256;
  for (int i = 0; i < j.spec.stack.n; ++i) {
    const uint64_t k = j.keys.empty() ? 0 : j.keys[static_cast<size_t>(i)];
    if (k && srv->cache.count(k)) continue;
    need += frame_pitch_of(j);
  }
  return need;
}

// Frees unreferenced cached frames, oldest first, until `need` more bytes fit the budget.
void evict_for(cp_server* srv, uint64_t need) {
  if (!srv->budget) return;
  while (srv->reserved + need > srv->budget) {
    uint64_t best = 0;
    Frame* bf = nullptr;
    for (auto& kv : srv->cache) {
      Frame* f = kv.second.get();
      if (f->refs == 0 && (!bf || f->last_use < bf->last_use)) {
        bf = f;
        best = kv.first;
      }
    }
    if (!bf) return;
    cudaEventSynchronize(bf->ready);
    cudaEventDestroy(bf->ready);
    pool_free(srv->ctx, bf->dev, bf->bytes, srv->h2d);
    srv->reserved -= bf->bytes;
    srv->cache.erase(best);
  }
}

int admit(cp_server* srv, Job* j) {
  cp_ctx* ctx = srv->ctx;
  const uint64_t pitch = frame_pitch_of(*j), fbytes = frame_bytes_of(*j);
  const int n = j->spec.stack.n;
  j->frames.assign(static_cast<size_t>(n), nullptr);
  int uploads = 0;
  for (int i = 0; i < n; ++i) {
    const uint64_t k = j->keys.empty() ? 0 : j->keys[static_cast<size_t>(i)];
    Frame* f = nullptr;
    if (k) {
      auto it = srv->cache.find(k);
      if (it != srv->cache.end()) f = it->second.get();
    }
    if (!f) {
      std::unique_ptr<Frame> nf(new Frame());
      cudaStream_t cs = (uploads++ & 1) ? srv->h2d2 : srv->h2d;
      int rc = pool_alloc(ctx, srv->pool, pitch, cs, &nf->dev);
      if (rc) return rc;
      nf->bytes = pitch;
      srv->reserved += pitch;
      cudaEventCreateWithFlags(&nf->ready, cudaEventDisableTiming);
      cudaMemcpyAsync(nf->dev, j->host_frames[static_cast<size_t>(i)], fbytes,
                      cudaMemcpyHostToDevice, cs);
      cudaEventRecord(nf->ready, cs);
      f = nf.get();
      if (k) {
        srv->cache[k] = std::move(nf);
      } else {
        j->private_frames.push_back(f);
        nf.release();
      }
    }
    f->refs += 1;
    f->last_use = ++srv->use_clock;
    j->frames[static_cast<size_t>(i)] = f;
  }
  const uint64_t ob = out_bytes_of(*j);
  void* p = nullptr;
  int rc = pool_alloc(ctx, srv->pool, 2 * ob + 256, srv->h2d, &p);
  if (rc) return rc;
  srv->reserved += 2 * ob + 256;
  j->reserved = 2 * ob + 256;
  j->out_dev = p;
  j->blend_dev = static_cast<uint8_t*>(p) + ob;
  j->warn_dev = reinterpret_cast<unsigned long long*>(static_cast<uint8_t*>(p) + 2 * ob);
  cudaMemsetAsync(j->warn_dev, 0, 8, srv->h2d);
  // staged: the reset above and this job's uploads on both copy streams
  cudaEvent_t join = nullptr;
  cudaEventCreateWithFlags(&join, cudaEventDisableTiming);
  cudaEventRecord(join, srv->h2d2);
  cudaStreamWaitEvent(srv->h2d, join, 0);
  cudaEventDestroy(join);  // released once the recorded work completes
  cudaEventCreateWithFlags(&j->staged, cudaEventDisableTiming);
  cudaEventRecord(j->staged, srv->h2d);
  // device->host copies go to pinned staging (a copy into pageable memory would block the
  // worker until the launch finishes); the worker copies to the caller's buffers at the end
  j->stage_bytes = 2 * ob + 64;
  auto it = srv->pinned_free.lower_bound(j->stage_bytes);
  if (it != srv->pinned_free.end() && it->first <= 2 * j->stage_bytes) {
    j->stage = it->second;
    j->stage_bytes = it->first;
    srv->pinned_free.erase(it);
  } else {
    void* h = nullptr;
    if (injected_alloc_failure(srv->ctx) ||
        cudaHostAlloc(&h, j->stage_bytes, cudaHostAllocPortable) != cudaSuccess)
      return CP_ERR_OOM;
    j->stage = static_cast<uint8_t*>(h);
  }
  j->state = 1;
  j->res.admit_s = now_s();
  return CP_OK;
}

void release(cp_server* srv, Job* j) {
  for (Frame* f : j->frames)
    if (f) f->refs -= 1;
  if (!j->private_frames.empty() && !j->staged) {
    // admission failed before it joined the second copy stream into the first: uploads of
    // this job may still be queued there, and the frees below (on the first stream) must
    // follow them
    cudaEvent_t join = nullptr;
    cudaEventCreateWithFlags(&join, cudaEventDisableTiming);
    cudaEventRecord(join, srv->h2d2);
    cudaStreamWaitEvent(srv->h2d, join, 0);
    cudaEventDestroy(join);
  }
  for (Frame* f : j->private_frames) {
    cudaEventDestroy(f->ready);
    pool_free(srv->ctx, f->dev, f->bytes, srv->h2d);
    srv->reserved -= f->bytes;
    delete f;
  }
  j->private_frames.clear();
  j->frames.clear();
  if (j->out_dev) {
    pool_free(srv->ctx, j->out_dev, j->reserved, srv->h2d);
    srv->reserved -= j->reserved;
    j->out_dev = nullptr;
  }
  if (j->staged) {
    cudaEventDestroy(j->staged);
    j->staged = nullptr;
  }
  if (j->stage) {
    srv->pinned_free.emplace(j->stage_bytes, j->stage);
    j->stage = nullptr;
  }
}

// 1: every frame of the job is on the device; 0: copies still in flight; -1: a copy failed.
int frames_ready(const Job* j) {
  if (j->staged) {
    const cudaError_t q = cudaEventQuery(j->staged);
    if (q == cudaErrorNotReady) return 0;
    if (q != cudaSuccess) return -1;
  }
  for (const Frame* f : j->frames) {
    const cudaError_t q = cudaEventQuery(f->ready);
    if (q == cudaErrorNotReady) return 0;
    if (q != cudaSuccess) return -1;
  }
  return 1;
}

// One persistent launch over the tiles of `batch` (same channel count).
int launch_jobs(cp_server* srv, std::vector<Job*>& batch) {
  cp_ctx* ctx = srv->ctx;
  LaunchSlot* slot = nullptr;
  for (auto& s : srv->slots)
    if (!s.busy || cudaEventQuery(s.freed) == cudaSuccess) {
      slot = &s;
      break;
    }
  if (!slot) return CP_ERR_STATE;  // caller retries later
  const int nb = static_cast<int>(batch.size());
  std::vector<StackDev> descs(static_cast<size_t>(nb));
  std::vector<int32_t> prefix(static_cast<size_t>(nb) + 1, 0);
  int max_n = 0;
  for (int i = 0; i < nb; ++i) {
    Job* j = batch[static_cast<size_t>(i)];
    std::vector<const uint8_t*> fr;
    for (Frame* f : j->frames) fr.push_back(static_cast<const uint8_t*>(f->dev));
    int rc = prepare_stack(ctx, &j->spec.stack, &j->spec.params, fr.data(), &descs[static_cast<size_t>(i)]);
    if (rc) return rc;
    StackDev& d = descs[static_cast<size_t>(i)];
    d.out = static_cast<uint8_t*>(j->out_dev);
    d.blend = (j->spec.out_blend && j->spec.params.mode == CP_MODE_OUTLIER)
                  ? static_cast<uint8_t*>(j->blend_dev) : nullptr;
    d.warnings = j->warn_dev;
    prefix[static_cast<size_t>(i) + 1] = prefix[static_cast<size_t>(i)] + d.tiles;
    max_n = std::max(max_n, d.n);
  }
  const uint64_t bytes = sizeof(StackDev) * nb + sizeof(int32_t) * (nb + 1) + 64;
  if (slot->bytes < bytes) {
    if (slot->dev) dev_free(ctx, slot->dev);
    if (slot->pinned) cudaFreeHost(slot->pinned);
    slot->dev = nullptr;
    slot->pinned = nullptr;
    slot->bytes = 0;
    const uint64_t want = std::max<uint64_t>(bytes, sizeof(StackDev) * 64 + 4096);
    int rc = dev_alloc(ctx, want, &slot->dev);
    if (rc) return rc;
    if (cudaHostAlloc(&slot->pinned, want, cudaHostAllocPortable) != cudaSuccess) return CP_ERR_OOM;
    slot->bytes = want;
  }
  uint8_t* hp = static_cast<uint8_t*>(slot->pinned);
  std::memcpy(hp, descs.data(), sizeof(StackDev) * nb);
  std::memcpy(hp + sizeof(StackDev) * nb, prefix.data(), sizeof(int32_t) * (nb + 1));
  cudaStream_t st = srv->compute[srv->next_stream];
  srv->next_stream = (srv->next_stream + 1) % kStreams;
  uint8_t* dp = static_cast<uint8_t*>(slot->dev);
  StackDev* d_stacks = reinterpret_cast<StackDev*>(dp);
  int32_t* d_prefix = reinterpret_cast<int32_t*>(dp + sizeof(StackDev) * nb);
  uint32_t* d_counter = reinterpret_cast<uint32_t*>(d_prefix + nb + 1);
  // this launch's own error flag (a bounded wait that gave up), read back with each job's
  // results, so a failed tile fails exactly the jobs of this launch
  uint32_t* d_err = d_counter + 1;
  cudaMemcpyAsync(dp, hp, sizeof(StackDev) * nb + sizeof(int32_t) * (nb + 1),
                  cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(d_err, 0, sizeof(uint32_t), st);
  const int rc = launch_batch_dispatch(ctx, descs, d_stacks, d_prefix, prefix.back(), 0,
                                       d_counter, max_n, st, d_err);
  if (rc) return rc;
  cudaEventRecord(slot->ev, st);
  slot->busy = true;
  // results back on the d2h stream once the launch is done
  cudaStreamWaitEvent(srv->d2h, slot->ev, 0);
  for (Job* j : batch) {
    const uint64_t ob = out_bytes_of(*j);
    cudaMemcpyAsync(j->stage, j->out_dev, 2 * ob + 8, cudaMemcpyDeviceToHost, srv->d2h);
    cudaMemcpyAsync(j->stage + 2 * ob + 8, d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                    srv->d2h);
    cudaEventCreateWithFlags(&j->done_ev, cudaEventDisableTiming);
    cudaEventRecord(j->done_ev, srv->d2h);
    j->state = 2;
  }
  // the slot's memory (descriptors, counter, error word) is reused only after the d2h
  // stream has read the error word: a reuse that only waited for the launch could overwrite
  // it with the next launch's descriptors before this launch's jobs read it
  cudaEventRecord(slot->freed, srv->d2h);
  return CP_OK;
}

void worker_loop(cp_server* srv) {
  cudaSetDevice(srv->ctx->device);
  std::unique_lock<std::mutex> lk(srv->mu);
  for (;;) {
    bool progressed = false;
    // 1. admission
    int inflight = 0;
    for (Job* j : srv->active)
      if (j->state < 3) ++inflight;
    while (!srv->queue.empty() && inflight < srv->max_inflight) {
      Job* j = srv->queue.front();
      const uint64_t need = job_need(srv, *j);
      if (srv->budget && need > srv->budget) {  // can never fit
        srv->queue.pop_front();
        j->res.status = CP_ERR_BUDGET;
        j->res.done_s = now_s();
        j->state = 3;
        srv->cv_done.notify_all();
        progressed = true;
        continue;
      }
      evict_for(srv, need);
      if (srv->budget && srv->reserved + need > srv->budget) break;  // wait for memory
      srv->queue.pop_front();
      const int rc = admit(srv, j);
      if (rc) {
        release(srv, j);
        j->res.status = rc;
        j->res.done_s = now_s();
        j->state = 3;
        srv->cv_done.notify_all();
      } else {
        srv->active.push_back(j);
        ++inflight;
      }
      progressed = true;
    }
    // 2. launch every admitted job whose frames have landed, one launch per channel count
    //    and launch group (batched kernel and plane words, see batch_group_key)
    std::map<std::pair<int, int>, std::vector<Job*>> ready;
    for (Job* j : srv->active) {
      if (j->state != 1) continue;
      const int fr = frames_ready(j);
      if (fr > 0) {
        ready[std::make_pair(j->spec.stack.channels, j->vkey)].push_back(j);
      } else if (fr < 0) {
        cudaGetLastError();
        release(srv, j);
        j->res.status = CP_ERR_CUDA;
        j->res.done_s = now_s();
        j->state = 3;
        srv->cv_done.notify_all();
        progressed = true;
      }
    }
    for (auto& kv : ready) {
      std::vector<Job*>& b = kv.second;
      for (size_t i = 0; i < b.size(); i += kMaxBatch) {
        std::vector<Job*> part(b.begin() + static_cast<long>(i),
                               b.begin() + static_cast<long>(std::min(b.size(), i + kMaxBatch)));
        const int rc = launch_jobs(srv, part);
        if (rc == CP_ERR_STATE) break;  // no free launch slot: retry next turn
        if (rc) {
          for (Job* j : part) {
            release(srv, j);
            j->res.status = rc;
            j->res.done_s = now_s();
            j->state = 3;
          }
          srv->cv_done.notify_all();
        }
        progressed = true;
      }
    }
    // 3. completions
    for (auto it = srv->active.begin(); it != srv->active.end();) {
      Job* j = *it;
      const cudaError_t q = j->state == 2 ? cudaEventQuery(j->done_ev) : cudaErrorNotReady;
      if (j->state == 2 && q != cudaSuccess && q != cudaErrorNotReady) {  // the launch failed
        cudaGetLastError();
        cudaEventDestroy(j->done_ev);
        j->done_ev = nullptr;
        release(srv, j);
        j->res.status = CP_ERR_CUDA;
        j->res.done_s = now_s();
        j->state = 3;
        it = srv->active.erase(it);
        srv->cv_done.notify_all();
        progressed = true;
      } else if (j->state == 2 && q == cudaSuccess) {
        cudaEventDestroy(j->done_ev);
        j->done_ev = nullptr;
        const cp_stack& st = j->spec.stack;
        const uint64_t bytes = static_cast<uint64_t>(st.width) * st.height * st.channels;
        const uint64_t ob = out_bytes_of(*j);
        std::memcpy(j->spec.out, j->stage, bytes);
        if (j->spec.out_blend && j->spec.params.mode == CP_MODE_OUTLIER)
          std::memcpy(j->spec.out_blend, j->stage + ob, bytes);
        std::memcpy(&j->res.warnings, j->stage + 2 * ob, 8);
        uint32_t dev_err = 0;
        std::memcpy(&dev_err, j->stage + 2 * ob + 8, sizeof dev_err);
        release(srv, j);
        // a tile of this job's launch gave up waiting for its frames: the output is partial
        j->res.status = dev_err ? CP_ERR_TIMEOUT : CP_OK;
        j->res.done_s = now_s();
        j->state = 3;
        it = srv->active.erase(it);
        srv->cv_done.notify_all();
        progressed = true;
      } else if (j->state == 3) {
        it = srv->active.erase(it);
      } else {
        ++it;
      }
    }
    if (srv->stopping && srv->queue.empty() && srv->active.empty()) break;
    if (!progressed) {
      if (srv->active.empty() && srv->queue.empty())
        srv->cv_work.wait(lk);
      else
        srv->cv_work.wait_for(lk, std::chrono::microseconds(50));
    }
  }
}

}  // namespace

extern "C" {

int cp_server_create(cp_ctx* ctx, uint64_t hbm_budget, int32_t max_inflight, cp_server** out) {
  if (!ctx || !out) return CP_ERR_ARG;
  *out = nullptr;
  cudaSetDevice(ctx->device);
  std::unique_ptr<cp_server> srv(new cp_server());
  srv->ctx = ctx;
  srv->budget = hbm_budget ? hbm_budget : ctx->budget;
  srv->max_inflight = max_inflight > 0 ? max_inflight : 8;
  for (auto& s : srv->compute)
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return CP_ERR_CUDA;
  if (cudaStreamCreateWithFlags(&srv->h2d, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&srv->h2d2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&srv->d2h, cudaStreamNonBlocking) != cudaSuccess)
    return CP_ERR_CUDA;
  cudaMemPoolProps props;
  std::memset(&props, 0, sizeof props);
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = ctx->device;
  if (cudaMemPoolCreate(&srv->pool, &props) != cudaSuccess) return CP_ERR_CUDA;
  uint64_t keep = ~0ull;  // keep freed memory in the pool for later jobs (the budget bounds it)
  cudaMemPoolSetAttribute(srv->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  srv->slots.resize(static_cast<size_t>(kStreams) * 2);
  for (auto& s : srv->slots) {
    cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&s.freed, cudaEventDisableTiming);
  }
  srv->worker = std::thread(worker_loop, srv.get());
  *out = srv.release();
  return CP_OK;
}

int cp_server_submit(cp_server* srv, const cp_job* job, uint64_t* job_id) {
  if (!srv || !job || !job_id || !job->out) return CP_ERR_ARG;
  const cp_stack& s = job->stack;
  if (s.n < 1 || s.n > CP_MAX_FRAMES || (!s.frames && !s.base) || s.width < 1 || s.height < 1 ||
      (s.channels != 1 && s.channels != 3 && s.channels != 4))
    return CP_ERR_ARG;
  std::unique_ptr<Job> j(new Job());
  j->spec = *job;
  for (int i = 0; i < s.n; ++i)
    j->host_frames.push_back(s.frames ? s.frames[i] : s.base + s.frame_stride * i);
  if (job->frame_keys) j->keys.assign(job->frame_keys, job->frame_keys + s.n);
  if (s.crop) {
    j->crop.assign(s.crop, s.crop + 2 * s.n);
    j->spec.stack.crop = j->crop.data();
  }
  j->spec.stack.frames = nullptr;
  j->spec.stack.base = nullptr;
  const cp_fade& fd = job->params.fade;
  if (fd.enabled && fd.n_points > 0 && fd.frames && fd.values) {
    j->fade_frames.assign(fd.frames, fd.frames + fd.n_points);
    j->fade_values.assign(fd.values, fd.values + fd.n_points);
    j->spec.params.fade.frames = j->fade_frames.data();
    j->spec.params.fade.values = j->fade_values.data();
  }
  if (job->params.sample && job->params.n_sample > 0) {
    j->sample.assign(job->params.sample, job->params.sample + job->params.n_sample);
    j->spec.params.sample = j->sample.data();
  }
  // validate the options now so that a bad job fails at submission
  {
    StackDev probe;
    std::vector<const uint8_t*> fr(static_cast<size_t>(s.n), reinterpret_cast<const uint8_t*>(256));
    int rc = prepare_stack(srv->ctx, &j->spec.stack, &j->spec.params, fr.data(), &probe);
    if (rc) return rc;
    j->vkey = batch_group_key(probe);
  }
  j->res.submit_s = now_s();
  std::lock_guard<std::mutex> lk(srv->mu);
  if (srv->stopping) return CP_ERR_STATE;
  j->id = srv->next_id++;
  *job_id = j->id;
  srv->queue.push_back(j.get());
  srv->jobs[j->id] = std::move(j);
  srv->cv_work.notify_one();
  return CP_OK;
}

int cp_server_wait(cp_server* srv, uint64_t job_id, int32_t timeout_ms, cp_job_result* res) {
  if (!srv || !res) return CP_ERR_ARG;
  std::unique_lock<std::mutex> lk(srv->mu);
  auto it = srv->jobs.find(job_id);
  if (it == srv->jobs.end()) return CP_ERR_STATE;
  Job* j = it->second.get();
  auto done = [&] { return j->state == 3; };
  if (timeout_ms < 0) {
    srv->cv_done.wait(lk, done);
  } else if (!srv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done)) {
    return CP_ERR_TIMEOUT;
  }
  *res = j->res;
  srv->jobs.erase(it);
  return CP_OK;
}

int cp_server_cancel(cp_server* srv, uint64_t job_id) {
  if (!srv) return CP_ERR_ARG;
  std::lock_guard<std::mutex> lk(srv->mu);
  auto it = srv->jobs.find(job_id);
  if (it == srv->jobs.end()) return CP_ERR_ARG;
  Job* j = it->second.get();
  if (j->state != 0) return CP_ERR_STATE;  // admitted or done: it runs to completion
  for (auto q = srv->queue.begin(); q != srv->queue.end(); ++q)
    if (*q == j) {
      srv->queue.erase(q);
      break;
    }
  j->res.status = CP_ERR_CANCELLED;
  j->res.done_s = now_s();
  j->state = 3;
  srv->cv_done.notify_all();
  srv->cv_work.notify_all();
  return CP_OK;
}

int cp_server_destroy(cp_server* srv) {
  if (!srv) return CP_ERR_ARG;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stopping = true;
    srv->cv_work.notify_all();
  }
  if (srv->worker.joinable()) srv->worker.join();
  cudaSetDevice(srv->ctx->device);
  for (auto& s : srv->compute) cudaStreamSynchronize(s);
  cudaStreamSynchronize(srv->h2d);
  cudaStreamSynchronize(srv->h2d2);
  cudaStreamSynchronize(srv->d2h);
  for (auto& kv : srv->cache) {
    cudaEventDestroy(kv.second->ready);
    pool_free(srv->ctx, kv.second->dev, kv.second->bytes, srv->h2d);
  }
  cudaStreamSynchronize(srv->h2d);
  for (auto& s : srv->slots) {
    if (s.dev) dev_free(srv->ctx, s.dev);
    if (s.pinned) cudaFreeHost(s.pinned);
    cudaEventDestroy(s.ev);
    cudaEventDestroy(s.freed);
  }
  for (auto& kv : srv->pinned_free) cudaFreeHost(kv.second);
  for (auto& s : srv->compute) cudaStreamDestroy(s);
  cudaStreamDestroy(srv->h2d);
  cudaStreamDestroy(srv->h2d2);
  cudaStreamDestroy(srv->d2h);
  if (srv->pool) cudaMemPoolDestroy(srv->pool);
  const int err = srv->error;
  delete srv;
  return err;
}

}  // extern "C"
