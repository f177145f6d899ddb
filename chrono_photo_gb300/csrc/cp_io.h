// cp_io.h — host helpers shared by the image file writers (PNG and JPEG): a small thread
// pool over independent work items, and output-file creation with the reference's
// parent-directory rule.
#pragma once

#include <sys/stat.h>
#include <sys/types.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <new>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace cp {

// Runs fn(0) .. fn(count - 1) on up to `threads` threads (0: all cores), each index once.
// An exception in fn stops the remaining work and is rethrown (as std::bad_alloc) on the
// calling thread after every worker has joined; if fewer threads start than asked for, the
// started ones share the work.
template <typename Fn>
void run_parallel(size_t count, int threads, Fn fn) {
  int workers = threads > 0 ? threads : static_cast<int>(std::thread::hardware_concurrency());
  workers = std::max(1, std::min<int>(workers, static_cast<int>(std::min<size_t>(count, 1024))));
  std::atomic<size_t> next(0);
  std::atomic<bool> failed(false);
  auto work = [&]() {
    for (size_t i = next.fetch_add(1); i < count && !failed.load(); i = next.fetch_add(1)) {
      try {
        fn(i);
      } catch (const std::exception&) {
        failed.store(true);
      }
    }
  };
  std::vector<std::thread> pool;
  try {
    pool.reserve(static_cast<size_t>(workers));
    for (int t = 1; t < workers; ++t) pool.emplace_back(work);
  } catch (const std::exception&) {
  }
  work();
  for (auto& t : pool) t.join();
  if (failed.load()) throw std::bad_alloc();
}

// Opens `path` for writing; when its parent directory is missing, creates it (one level, as
// std::fs::create_dir in the reference's save_image, src/main.rs:533-540) and tries again.
inline FILE* open_output(const char* path) {
  FILE* f = std::fopen(path, "wb");
  if (f) return f;
  std::string dir(path);
  const size_t slash = dir.find_last_of('/');
  if (slash == std::string::npos || slash == 0) return nullptr;
  dir.resize(slash);
  struct stat st;
  if (stat(dir.c_str(), &st) == 0) return nullptr;  // the parent exists: a real error
  if (mkdir(dir.c_str(), 0777) != 0) return nullptr;
  return std::fopen(path, "wb");
}

}  // namespace cp
