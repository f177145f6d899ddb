// cp_tune.cpp — launch configuration of the pixel-thread outlier kernel, chosen by measurement.
//
// A launch of k_outlier_px has three free choices that do not change its results: how
// phase A runs (word columns on three warps, or each warp on its own pixel's planes), one or
// two staging buffers per CTA, and how many CTAs per SM the grid fills. Which is fastest
// depends on the frame count (plane words), the distance kind (integer or f32 pairs), the
// outlier group and the background; the reference's own knobs for the same trade-off are its
// thread counts (src/main.rs:49-54, :254-261), set by hand.
//
// The first launch of a key (distance kind, outlier group, background, plane words, size
// class of the stack) on a large enough stack times every candidate on that stack (CUDA events on the caller's
// stream, two runs each, the better kept), keeps the fastest for the context and appends it
// to a cache file of JSON lines (CP_TUNE_CACHE, default ~/.cache/chrono_gpu/tune.jsonl),
// keyed by GPU name and library version, which later contexts read at their first launch.
// CP_AUTOTUNE=0 uses the static choice; CP_PX_CONFIG="pa,db,ctas" forces one candidate.
// Tuning never runs while the stream is being captured into a graph.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "../../include/chrono_gpu.h"
#include "cp_host_internal.h"
#include "cp_internal.h"

namespace cp {
namespace {

// Stack size class: log2 of the tiles per SM, 3 (8-15 tiles per SM, the smallest stack that
// is tuned) to 7 (128 and more). The fastest configuration of a few waves of tiles is not
// that of a hundred.
int size_class(const StackDev& d, int sm_count) {
  const int per_sm = d.tiles / std::max(1, sm_count);
  int c = 0;
  while (c < 7 && (2 << c) <= per_sm) ++c;
  return c;
}

int px_key(const StackDev& d, int sm_count, int* k, int* g, int* b) {
  outlier_variant(d, k, g, b);
  return (((*k * 8 + *g) * 2 + *b) * 8 + d.nw) * 8 + size_class(d, sm_count);
}

std::string key_name(int k, int g, int b, const StackDev& d, int sm_count) {
  char buf[96];
  std::snprintf(buf, sizeof buf, "kind%d group%d bg%d words%d tiles/SM>=%d", k, g, b, d.nw,
                1 << size_class(d, sm_count));
  return buf;
}

int px_call(int k, int g, int b, const StackDev& d, int pa, bool db, bool occ, int grid, int smem,
            cudaStream_t st, uint32_t* err) {
  int rc = -1;
#define CP_PX_CALL(K, G, B) \
  if (k == K && g == G && b == B) rc = px_launch_k##K##_g##G##_b##B(d, pa, db, occ, grid, smem, st, err);
  CP_PX_VARIANTS(CP_PX_CALL)
#undef CP_PX_CALL
  return rc;
}

// CTAs per SM of a variant, cached per context.
int px_occupancy(cp_ctx* ctx, int k, int g, int b, const StackDev& d, int pa, bool db) {
  const int smem = px_smem_bytes(d.n, db);
  const auto key = std::make_pair(5000 + ((k * 8 + g) * 2 + b) * 64 + d.nw * 8 + pa * 2 + db, smem);
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->occupancy.find(key);
    if (it != ctx->occupancy.end()) return it->second;
  }
  int occ = px_call(k, g, b, d, pa, db, true, 0, smem, nullptr, nullptr);
  if (occ < 1) occ = 1;
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->occupancy[key] = occ;
  return occ;
}

int px_run(cp_ctx* ctx, int k, int g, int b, const StackDev& d, const PxChoice& c,
           cudaStream_t st) {
  const int smem = px_smem_bytes(d.n, c.db != 0);
  const int occ = px_occupancy(ctx, k, g, b, d, c.pa, c.db != 0);
  const int per_sm = c.ctas > 0 ? std::min(c.ctas, occ) : occ;
  const int grid = std::max(1, std::min(d.tiles, per_sm * ctx->sm_count));
  const int rc = px_call(k, g, b, d, c.pa, c.db != 0, false, grid, smem, st, ctx->d_error);
  if (rc < 0) {
    ctx_error(ctx, "no pixel-thread kernel for variant %d/%d/%d", k, g, b);
    return CP_ERR_ARG;
  }
  count_launches(ctx, 1);
  return cuda_status(ctx, static_cast<cudaError_t>(rc), "composite launch");
}

std::string cache_path() {
  const char* p = std::getenv("CP_TUNE_CACHE");
  if (p && *p) return p;
  const char* home = std::getenv("HOME");
  if (!home || !*home) return std::string();
  const std::string dir = std::string(home) + "/.cache/chrono_gpu";
  mkdir((std::string(home) + "/.cache").c_str(), 0755);
  mkdir(dir.c_str(), 0755);
  return dir + "/tune.jsonl";
}

std::string json_str(const std::string& line, const char* field) {
  const std::string pat = std::string("\"") + field + "\":\"";
  const size_t a = line.find(pat);
  if (a == std::string::npos) return std::string();
  const size_t s = a + pat.size();
  const size_t e = line.find('"', s);
  return e == std::string::npos ? std::string() : line.substr(s, e - s);
}
double json_num(const std::string& line, const char* field, double dflt) {
  const std::string pat = std::string("\"") + field + "\":";
  const size_t a = line.find(pat);
  if (a == std::string::npos) return dflt;
  return std::atof(line.c_str() + a + pat.size());
}

void load_cache(cp_ctx* ctx) {
  // ctx->mu held
  if (ctx->tune_loaded) return;
  ctx->tune_loaded = true;
  const std::string path = cache_path();
  if (path.empty()) return;
  std::ifstream f(path);
  std::string line;
  while (std::getline(f, line)) {
    if (json_str(line, "gpu") != ctx->gpu_name || json_str(line, "lib") != cp_version()) continue;
    const int key = static_cast<int>(json_num(line, "key", -1));
    if (key < 0) continue;
    PxChoice c;
    c.pa = static_cast<int>(json_num(line, "pa", -1));
    c.db = static_cast<int>(json_num(line, "db", 0));
    c.ctas = static_cast<int>(json_num(line, "ctas", 0));
    c.ms = static_cast<float>(json_num(line, "ms", 0));
    c.static_ms = static_cast<float>(json_num(line, "static_ms", 0));
    c.name = json_str(line, "name");
    c.from_cache = true;
    if (c.pa != 0 && c.pa != 2) continue;
    ctx->px_tuned[key] = c;
  }
}

void append_cache(cp_ctx* ctx, int key, const PxChoice& c) {
  const std::string path = cache_path();
  if (path.empty()) return;
  std::ofstream f(path, std::ios::app);
  if (!f) return;
  char buf[512];
  std::snprintf(buf, sizeof buf,
                "{\"gpu\":\"%s\",\"lib\":\"%s\",\"key\":%d,\"name\":\"%s\",\"pa\":%d,\"db\":%d,"
                "\"ctas\":%d,\"ms\":%.5f,\"static_ms\":%.5f}\n",
                ctx->gpu_name.c_str(), cp_version(), key, c.name.c_str(), c.pa, c.db, c.ctas,
                c.ms, c.static_ms);
  f << buf;
}

// Times every candidate on this stack; outputs are written by each run and again by the
// launch that follows (identical results). Warnings and debug outputs are left out.
PxChoice tune(cp_ctx* ctx, int k, int g, int b, const StackDev& d, cudaStream_t st) {
  StackDev t = d;
  t.warnings = nullptr;
  t.dbg_median = t.dbg_q1 = t.dbg_q3 = nullptr;
  t.dbg_bits = nullptr;
  t.dbg_chosen = t.dbg_bg = t.dbg_nout = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  PxChoice best;
  best.ms = 1e30f;
  const int static_pa = 2;  // kPxPhaseA
  float static_ms = 0.0f;
  for (int pa : {0, 2}) {
    for (int db = 0; db < 2; ++db) {
      if (db && (d.nw > 2 || px_smem_bytes(d.n, true) > ctx->max_smem)) continue;
      const int occ = px_occupancy(ctx, k, g, b, d, pa, db != 0);
      for (int ctas = occ; ctas >= std::max(1, occ - 1); --ctas) {
        PxChoice c;
        c.pa = pa;
        c.db = db;
        c.ctas = ctas;
        float ms = 1e30f;
        for (int rep = 0; rep < 3; ++rep) {
          cudaEventRecord(e0, st);
          if (px_run(ctx, k, g, b, t, c, st) != CP_OK) {
            ms = 1e30f;
            break;
          }
          cudaEventRecord(e1, st);
          cudaEventSynchronize(e1);
          float m = 0.0f;
          cudaEventElapsedTime(&m, e0, e1);
          if (rep > 0) ms = std::min(ms, m);  // the first run warms caches and occupancy
        }
        if (pa == static_pa && db == 0 && ctas == occ) static_ms = ms;
        if (ms < best.ms) {
          best = c;
          best.ms = ms;
        }
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  best.static_ms = static_ms;
  best.name = key_name(k, g, b, d, ctx->sm_count);
  return best;
}

}  // namespace

int launch_px(cp_ctx* ctx, const StackDev& d, cudaStream_t stream) {
  int k, g, b;
  const int key = px_key(d, ctx->sm_count, &k, &g, &b);
  PxChoice c;  // the static choice: phase A per kind, one buffer, full occupancy
  const char* forced = std::getenv("CP_PX_CONFIG");
  const char* at = std::getenv("CP_AUTOTUNE");
  if (forced && *forced) {
    int pa = -1, db = 0, ctas = 0;
    if (std::sscanf(forced, "%d,%d,%d", &pa, &db, &ctas) >= 2 && (pa == 0 || pa == 2)) {
      c.pa = pa;
      c.db = (db && d.nw <= 2 && px_smem_bytes(d.n, true) <= ctx->max_smem) ? 1 : 0;
      c.ctas = ctas;
    }
  } else if (!(at && std::strcmp(at, "0") == 0)) {
    bool have = false;
    {
      std::lock_guard<std::mutex> lk(ctx->mu);
      load_cache(ctx);
      auto it = ctx->px_tuned.find(key);
      if (it != ctx->px_tuned.end()) {
        c = it->second;
        have = true;
      }
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(stream, &cap);
    // tune on stacks that fill the GPU several times over, outside graph capture
    if (!have && cap == cudaStreamCaptureStatusNone && d.tiles >= 8 * ctx->sm_count) {
      std::lock_guard<std::mutex> tl(ctx->tune_mu);
      bool again = false;
      {
        std::lock_guard<std::mutex> lk(ctx->mu);
        auto it = ctx->px_tuned.find(key);
        if (it != ctx->px_tuned.end()) {
          c = it->second;
          again = true;
        }
      }
      if (!again) {
        c = tune(ctx, k, g, b, d, stream);
        if (c.ms < 1e29f) {
          {
            std::lock_guard<std::mutex> lk(ctx->mu);
            ctx->px_tuned[key] = c;
          }
          append_cache(ctx, key, c);
        } else {
          c = PxChoice();
        }
      }
    }
  }
  if (c.pa < 0) c.pa = 2;  // kPxPhaseA
  return px_run(ctx, k, g, b, d, c, stream);
}

std::string tuning_report(cp_ctx* ctx) {
  std::lock_guard<std::mutex> lk(ctx->mu);
  std::ostringstream o;
  o << "[";
  bool first = true;
  for (const auto& kv : ctx->px_tuned) {
    const PxChoice& c = kv.second;
    char buf[320];
    std::snprintf(buf, sizeof buf,
                  "%s{\"key\":\"%s\",\"phase_a\":\"%s\",\"buffers\":%d,\"ctas_per_sm\":%d,"
                  "\"tuned_ms\":%.5f,\"static_ms\":%.5f,\"from\":\"%s\"}",
                  first ? "" : ",", c.name.c_str(), c.pa == 2 ? "per-pixel" : "word-column",
                  c.db + 1, c.ctas, c.ms, c.static_ms, c.from_cache ? "cache" : "measured");
    o << buf;
    first = false;
  }
  o << "]";
  return o.str();
}

}  // namespace cp

extern "C" int cp_ctx_tuning_report(cp_ctx* ctx, char* buf, size_t len) {
  if (!ctx || !buf || len == 0) return CP_ERR_ARG;
  const std::string s = cp::tuning_report(ctx);
  std::snprintf(buf, len, "%s", s.c_str());
  return s.size() < len ? CP_OK : CP_ERR_LIMIT;
}
