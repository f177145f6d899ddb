// cp_jpeg.cpp — frame ingest of JPEG files, decoded on the GPU by nvJPEG.
//
// The reference opens every frame with image::open (src/streams.rs:63-70, src/simple.rs:45,
// src/shake.rs:218-255), and its frames are JPEG files: its example-data writer saves
// image-%05d.jpg at quality 95 (src/util/create_example_data.rs:52-56). image 0.23 decodes
// them on the CPU, one frame at a time, to RGB8 (three components) or L8 (one).
//
// Here the files are read on host threads, their headers checked on the host (baseline,
// extended or progressive Huffman DCT with 8-bit samples, one or three components, the
// caller's size), and the batch is decoded by nvJPEG's batched decoder straight into the
// device frames, interleaved RGB or gray: only the compressed bytes cross the host link,
// and the decoded stack is where the compositing kernels read it (cp_composite_device).
// libnvjpeg is loaded at the first JPEG call (dlopen), so the rest of the library needs
// nothing of it. JPEG is lossy and decoders differ in their inverse DCT and chroma
// upsampling, so the samples are not pinned to image's decoder bit for bit; the tests hold
// nvJPEG's output to a stated tolerance of an exact-IDCT decoder.
//
// Files go to the GPU's JPEG engines (nvJPEG's hardware backend: 64 1080p frames in about
// 19 ms on a GB300) when their header shows a stream those take: baseline (SOF0), all
// components in one interleaved scan, 4:4:4, 4:2:2, 4:2:0, 4:4:0 or gray. The others
// (progressive, extended, multi-scan, 4:1:1 ...) go to nvJPEG's default backend, whose
// Huffman decoding runs on the calling thread, as does everything when the GPU has no JPEG
// engines. CP_JPEG_BACKEND=default (or gpu, the GPU-assisted hybrid) sends every file to
// that software backend.

#include <dlfcn.h>
#include <nvjpeg.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "../../include/chrono_gpu.h"
#include "cp_host_internal.h"
#include "cp_io.h"

namespace {

// ---- header ---------------------------------------------------------------------------------

struct JpegHeader {
  int width = 0, height = 0, components = 0;
  bool baseline = false;     // SOF0
  bool engine_ok = false;    // a stream the hardware decoder takes (see the file header)
  int h[3] = {0, 0, 0}, v[3] = {0, 0, 0};
};

// Sampling factors the JPEG engines take: gray, or chroma 1x1 with luma 1x1, 2x1, 2x2, 1x2.
bool engine_sampling(const JpegHeader& h) {
  if (h.components == 1) return true;
  if (h.h[1] != 1 || h.v[1] != 1 || h.h[2] != 1 || h.v[2] != 1) return false;
  return (h.h[0] == 1 || h.h[0] == 2) && (h.v[0] == 1 || h.v[0] == 2);
}

// Walks the markers up to the first scan header (T.81 B.1-B.2). CP_OK, or CP_ERR_IO with
// *why.
int parse_header(const uint8_t* d, size_t n, JpegHeader* h, std::string* why) {
  if (n < 4 || d[0] != 0xFF || d[1] != 0xD8) {
    *why = "not a JPEG file (no SOI marker)";
    return CP_ERR_IO;
  }
  size_t p = 2;
  for (;;) {
    while (p < n && d[p] != 0xFF) ++p;  // data between segments is not allowed; skip it
    while (p < n && d[p] == 0xFF) ++p;  // fill bytes
    if (p >= n) {
      *why = "no frame header before the end of the file";
      return CP_ERR_IO;
    }
    const uint8_t m = d[p++];
    if (m == 0xD8 || m == 0x01 || (m >= 0xD0 && m <= 0xD7)) continue;  // no length
    if (m == 0xD9 || (m == 0xDA && h->components == 0)) {
      *why = "no frame header before the scan";
      return CP_ERR_IO;
    }
    if (p + 2 > n) break;
    const size_t len = (static_cast<size_t>(d[p]) << 8) | d[p + 1];
    if (len < 2 || p + len > n) break;
    const uint8_t* s = d + p + 2;
    if (m >= 0xC0 && m <= 0xCF && m != 0xC4 && m != 0xC8 && m != 0xCC) {
      if (m != 0xC0 && m != 0xC1 && m != 0xC2) {
        *why = "unsupported JPEG process (lossless, hierarchical or arithmetic coding)";
        return CP_ERR_IO;
      }
      if (len < 8) break;
      h->baseline = m == 0xC0;
      if (s[0] != 8) {
        *why = "unsupported sample precision (only 8 bits)";
        return CP_ERR_IO;
      }
      h->height = (s[1] << 8) | s[2];
      h->width = (s[3] << 8) | s[4];
      h->components = s[5];
      if (h->height == 0) {
        *why = "unsupported: height defined by a DNL marker";
        return CP_ERR_IO;
      }
      if (h->components != 1 && h->components != 3) {
        *why = "unsupported number of components (only 1 or 3)";
        return CP_ERR_IO;
      }
      if (len < 8 + 3u * h->components) break;
      for (int c = 0; c < h->components; ++c) {
        h->h[c] = s[7 + 3 * c] >> 4;
        h->v[c] = s[7 + 3 * c] & 15;
      }
      p += len;
      continue;
    }
    if (m == 0xDA) {  // the first scan: does it hold every component?
      if (len < 3) break;
      h->engine_ok = h->baseline && s[0] == h->components && engine_sampling(*h);
      return CP_OK;
    }
    p += len;
  }
  *why = "truncated JPEG header";
  return CP_ERR_IO;
}

bool read_file(const char* path, std::vector<uint8_t>* data) {
  struct stat st;
  if (stat(path, &st) != 0 || !S_ISREG(st.st_mode)) return false;
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  data->resize(static_cast<size_t>(st.st_size));
  const bool ok = std::fread(data->data(), 1, data->size(), f) == data->size();
  std::fclose(f);
  return ok;
}

// ---- nvJPEG, loaded at first use --------------------------------------------------------------

struct NvJpeg {
  bool ok = false;
  std::string why;
  decltype(&nvjpegCreateEx) create = nullptr;
  decltype(&nvjpegDestroy) destroy = nullptr;
  decltype(&nvjpegJpegStateCreate) state_create = nullptr;
  decltype(&nvjpegJpegStateDestroy) state_destroy = nullptr;
  decltype(&nvjpegDecodeBatchedInitialize) batch_init = nullptr;
  decltype(&nvjpegDecodeBatched) batch_decode = nullptr;
};

const NvJpeg& nvjpeg() {
  static NvJpeg lib;
  static std::once_flag once;
  std::call_once(once, [] {
    void* so = dlopen("libnvjpeg.so.13", RTLD_NOW | RTLD_LOCAL);
    if (!so) so = dlopen("libnvjpeg.so", RTLD_NOW | RTLD_LOCAL);
    if (!so) {
      lib.why = "libnvjpeg cannot be loaded";
      return;
    }
    bool all = true;
    auto sym = [&](const char* name) {
      void* f = dlsym(so, name);
      if (!f) all = false;
      return f;
    };
    lib.create = reinterpret_cast<decltype(lib.create)>(sym("nvjpegCreateEx"));
    lib.destroy = reinterpret_cast<decltype(lib.destroy)>(sym("nvjpegDestroy"));
    lib.state_create = reinterpret_cast<decltype(lib.state_create)>(sym("nvjpegJpegStateCreate"));
    lib.state_destroy =
        reinterpret_cast<decltype(lib.state_destroy)>(sym("nvjpegJpegStateDestroy"));
    lib.batch_init =
        reinterpret_cast<decltype(lib.batch_init)>(sym("nvjpegDecodeBatchedInitialize"));
    lib.batch_decode = reinterpret_cast<decltype(lib.batch_decode)>(sym("nvjpegDecodeBatched"));
    lib.ok = all;
    if (!all) lib.why = "libnvjpeg lacks the batched decoder";
  });
  return lib;
}

// One nvJPEG handle with its batched-decode state.
struct Backend {
  nvjpegHandle_t handle = nullptr;
  nvjpegJpegState_t state = nullptr;
  int batch = 0;  // batch size and output format of the last initialisation
  int format = -1;
  bool tried = false;
};

// A context's decoders, used under `mu`: the JPEG engines and the software backend, each
// created at its first use.
struct JpegDecoder {
  Backend engine, software;
  std::mutex mu;
};

constexpr int kJpegBatch = 64;  // files per nvjpegDecodeBatched call

int nvjpeg_status(cp_ctx* ctx, nvjpegStatus_t s, const char* what) {
  if (s == NVJPEG_STATUS_SUCCESS) return CP_OK;
  cp::ctx_error(ctx, "%s: nvJPEG status %d", what, static_cast<int>(s));
  if (s == NVJPEG_STATUS_BAD_JPEG || s == NVJPEG_STATUS_JPEG_NOT_SUPPORTED ||
      s == NVJPEG_STATUS_INCOMPLETE_BITSTREAM)
    return CP_ERR_IO;
  if (s == NVJPEG_STATUS_ALLOCATOR_FAILURE) return CP_ERR_OOM;
  return CP_ERR_CUDA;
}

int get_decoder(cp_ctx* ctx, JpegDecoder** out) {
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!ctx->jpeg) {
    const NvJpeg& lib = nvjpeg();
    if (!lib.ok) {
      cp::ctx_error(ctx, "JPEG decode: %s", lib.why.c_str());
      return CP_ERR_IO;
    }
    ctx->jpeg = new JpegDecoder;
  }
  *out = static_cast<JpegDecoder*>(ctx->jpeg);
  return CP_OK;
}

// The backend's handle and state, created at the first call (CP_OK), or CP_ERR_STATE when
// this backend cannot be had on this GPU.
int open_backend(cp_ctx* ctx, Backend* b, nvjpegBackend_t kind) {
  if (b->handle) return CP_OK;
  if (b->tried) return CP_ERR_STATE;
  b->tried = true;
  const NvJpeg& lib = nvjpeg();
  nvjpegStatus_t s = lib.create(kind, nullptr, nullptr, 0, &b->handle);
  if (s == NVJPEG_STATUS_SUCCESS) s = lib.state_create(b->handle, &b->state);
  if (s != NVJPEG_STATUS_SUCCESS) {
    if (b->handle) lib.destroy(b->handle);
    b->handle = nullptr;
    b->state = nullptr;
    if (kind == NVJPEG_BACKEND_HARDWARE) return CP_ERR_STATE;  // no JPEG engines here
    return nvjpeg_status(ctx, s, "nvJPEG initialisation");
  }
  return CP_OK;
}

// Decodes files[idx[k]] into dst + idx[k] * stride with one backend, in batches of up to
// kJpegBatch, on the context's stream (not waited for). *unsupported: the backend refused a
// batch as a stream it does not take (nothing of that batch written).
int decode_with(cp_ctx* ctx, Backend* b, const std::vector<std::vector<uint8_t>>& files,
                const std::vector<size_t>& idx, uint8_t* dst, uint64_t stride, int32_t width,
                int32_t channels, bool* unsupported) {
  const NvJpeg& lib = nvjpeg();
  const nvjpegOutputFormat_t fmt = channels == 1 ? NVJPEG_OUTPUT_Y : NVJPEG_OUTPUT_RGBI;
  *unsupported = false;
  for (size_t i0 = 0; i0 < idx.size(); i0 += kJpegBatch) {
    const int nb = static_cast<int>(std::min<size_t>(kJpegBatch, idx.size() - i0));
    if (b->batch != nb || b->format != static_cast<int>(fmt)) {
      const int rc = nvjpeg_status(ctx, lib.batch_init(b->handle, b->state, nb, 1, fmt),
                                   "nvjpegDecodeBatchedInitialize");
      if (rc) {
        b->batch = 0;
        return rc;
      }
      b->batch = nb;
      b->format = static_cast<int>(fmt);
    }
    std::vector<const unsigned char*> data(static_cast<size_t>(nb));
    std::vector<size_t> lengths(static_cast<size_t>(nb));
    std::vector<nvjpegImage_t> dests(static_cast<size_t>(nb));
    for (int k = 0; k < nb; ++k) {
      const size_t i = idx[i0 + static_cast<size_t>(k)];
      data[static_cast<size_t>(k)] = files[i].data();
      lengths[static_cast<size_t>(k)] = files[i].size();
      nvjpegImage_t& d = dests[static_cast<size_t>(k)];
      std::memset(&d, 0, sizeof d);
      d.channel[0] = dst + stride * i;
      d.pitch[0] = static_cast<size_t>(width) * channels;
    }
    const nvjpegStatus_t st = lib.batch_decode(b->handle, b->state, data.data(), lengths.data(),
                                               dests.data(), ctx->stream);
    if (st != NVJPEG_STATUS_SUCCESS) {
      b->batch = 0;  // a failed batch is reset by the next initialisation
      cudaStreamSynchronize(ctx->stream);
      *unsupported = st == NVJPEG_STATUS_JPEG_NOT_SUPPORTED;
      return nvjpeg_status(ctx, st, "nvjpegDecodeBatched");
    }
  }
  return CP_OK;
}

// CP_JPEG_BACKEND=default / gpu: every file to that software backend.
int software_choice() {
  const char* b = std::getenv("CP_JPEG_BACKEND");
  if (!b) return -1;
  if (std::strcmp(b, "default") == 0) return NVJPEG_BACKEND_DEFAULT;
  if (std::strcmp(b, "gpu") == 0) return NVJPEG_BACKEND_GPU_HYBRID;
  return -1;
}

// Reads and checks the n files; CP_ERR_IO names the first bad one.
int read_batch(cp_ctx* ctx, const char* const* paths, int32_t n, int32_t threads, int32_t width,
               int32_t height, int32_t channels, std::vector<std::vector<uint8_t>>* files,
               std::vector<bool>* engine_ok) {
  files->assign(static_cast<size_t>(n), std::vector<uint8_t>());
  std::vector<char> eng(static_cast<size_t>(n), 0);
  std::vector<int> rc(static_cast<size_t>(n), CP_OK);
  std::vector<std::string> why(static_cast<size_t>(n));
  cp::run_parallel(static_cast<size_t>(n), threads, [&](size_t i) {
    if (!read_file(paths[i], &(*files)[i])) {
      rc[i] = CP_ERR_IO;
      why[i] = "cannot read the file";
      return;
    }
    JpegHeader h;
    rc[i] = parse_header((*files)[i].data(), (*files)[i].size(), &h, &why[i]);
    eng[i] = h.engine_ok ? 1 : 0;
    if (rc[i] == CP_OK && (h.width != width || h.height != height || h.components != channels)) {
      char b[160];
      std::snprintf(b, sizeof b, "%dx%d with %d component(s), expected %dx%d with %d",
                    h.width, h.height, h.components, width, height, channels);
      why[i] = b;
      rc[i] = CP_ERR_IO;
    }
  });
  for (int32_t i = 0; i < n; ++i)
    if (rc[static_cast<size_t>(i)] != CP_OK) {
      cp::ctx_error(ctx, "%s: %s", paths[i], why[static_cast<size_t>(i)].c_str());
      return rc[static_cast<size_t>(i)];
    }
  engine_ok->assign(eng.begin(), eng.end());
  return CP_OK;
}

// Decodes the files into dst + i * stride (device memory) on the context's stream and waits:
// files the JPEG engines take go there, the rest (and all of them when the engines are
// missing or refuse the batch as unsupported) to the software backend.
int decode_to_device(cp_ctx* ctx, const std::vector<std::vector<uint8_t>>& files,
                     const std::vector<bool>& engine_ok, uint8_t* dst, uint64_t stride,
                     int32_t width, int32_t channels) {
  JpegDecoder* dec = nullptr;
  int rc = get_decoder(ctx, &dec);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(dec->mu);
  const int forced = software_choice();
  const bool engines =
      forced < 0 && open_backend(ctx, &dec->engine, NVJPEG_BACKEND_HARDWARE) == CP_OK;
  std::vector<size_t> eng, soft;
  for (size_t i = 0; i < files.size(); ++i)
    (engines && engine_ok[i] ? eng : soft).push_back(i);
  if (!eng.empty()) {
    bool unsupported = false;
    rc = decode_with(ctx, &dec->engine, files, eng, dst, stride, width, channels, &unsupported);
    if (rc && unsupported) {  // decode them all again in software
      soft.clear();
      for (size_t i = 0; i < files.size(); ++i) soft.push_back(i);
      rc = CP_OK;
    }
    if (rc) return rc;
  }
  if (!soft.empty()) {
    rc = open_backend(ctx, &dec->software,
                      forced < 0 ? NVJPEG_BACKEND_DEFAULT : static_cast<nvjpegBackend_t>(forced));
    if (rc) return rc == CP_ERR_STATE ? CP_ERR_CUDA : rc;
    bool unsupported = false;
    rc = decode_with(ctx, &dec->software, files, soft, dst, stride, width, channels,
                     &unsupported);
    if (rc) return rc;
  }
  // the host bitstreams stay alive until the decode has finished
  return cp::cuda_status(ctx, cudaStreamSynchronize(ctx->stream), "JPEG decode");
}

bool valid_args(const char* const* paths, int32_t n, const void* out, uint64_t frame_stride,
                int32_t width, int32_t height, int32_t channels) {
  if (!paths || !out || n < 1 || width < 1 || height < 1 || (channels != 1 && channels != 3) ||
      frame_stride < static_cast<uint64_t>(width) * height * channels)
    return false;
  for (int32_t i = 0; i < n; ++i)
    if (!paths[i]) return false;
  return true;
}

}  // namespace

namespace cp {
void jpeg_release(cp_ctx* ctx) {
  auto* dec = static_cast<JpegDecoder*>(ctx->jpeg);
  if (!dec) return;
  const NvJpeg& lib = nvjpeg();
  for (Backend* b : {&dec->engine, &dec->software}) {
    if (b->state) lib.state_destroy(b->state);
    if (b->handle) lib.destroy(b->handle);
  }
  delete dec;
  ctx->jpeg = nullptr;
}
}  // namespace cp

extern "C" int cp_jpeg_info(cp_ctx* ctx, const char* path, int32_t* width, int32_t* height,
                            int32_t* channels) {
  if (!path || !width || !height || !channels) return CP_ERR_ARG;
  try {
    std::vector<uint8_t> data;
    if (!read_file(path, &data)) {
      cp::ctx_error(ctx, "%s: cannot read the file", path);
      return CP_ERR_IO;
    }
    JpegHeader h;
    std::string why;
    const int rc = parse_header(data.data(), data.size(), &h, &why);
    if (rc) {
      cp::ctx_error(ctx, "%s: %s", path, why.c_str());
      return rc;
    }
    *width = h.width;
    *height = h.height;
    *channels = h.components;
    return CP_OK;
  } catch (const std::exception& e) {
    cp::ctx_error(ctx, "cp_jpeg_info: %s", e.what());
    return CP_ERR_OOM;
  }
}

extern "C" int cp_load_jpeg_device(cp_ctx* ctx, const char* const* paths, int32_t n,
                                   int32_t threads, uint8_t* out, uint64_t frame_stride,
                                   int32_t width, int32_t height, int32_t channels) {
  if (!ctx || !valid_args(paths, n, out, frame_stride, width, height, channels))
    return CP_ERR_ARG;
  try {
    cudaSetDevice(ctx->device);
    std::vector<std::vector<uint8_t>> files;
    std::vector<bool> engine_ok;
    int rc = read_batch(ctx, paths, n, threads, width, height, channels, &files, &engine_ok);
    if (rc) return rc;
    return decode_to_device(ctx, files, engine_ok, out, frame_stride, width, channels);
  } catch (const std::exception& e) {
    cp::ctx_error(ctx, "cp_load_jpeg_device: %s", e.what());
    return CP_ERR_OOM;
  }
}

extern "C" int cp_load_jpeg(cp_ctx* ctx, const char* const* paths, int32_t n, int32_t threads,
                            uint8_t* out, uint64_t frame_stride, int32_t width, int32_t height,
                            int32_t channels) {
  if (!ctx || !valid_args(paths, n, out, frame_stride, width, height, channels))
    return CP_ERR_ARG;
  try {
    cudaSetDevice(ctx->device);
    std::vector<std::vector<uint8_t>> files;
    std::vector<bool> engine_ok;
    int rc = read_batch(ctx, paths, n, threads, width, height, channels, &files, &engine_ok);
    if (rc) return rc;
    // decoded into the context's device staging, then copied to the caller's host frames
    std::lock_guard<std::mutex> call(ctx->call_mu);
    const uint64_t fb = static_cast<uint64_t>(width) * height * channels;
    rc = cp::ensure_buffer(ctx, ctx->frames_dev, fb * static_cast<uint64_t>(n));
    if (rc) return rc;
    uint8_t* dev = static_cast<uint8_t*>(ctx->frames_dev.ptr);
    rc = decode_to_device(ctx, files, engine_ok, dev, fb, width, channels);
    if (rc) return rc;
    rc = cp::cuda_status(ctx, cudaMemcpy2DAsync(out, frame_stride, dev, fb, fb,
                                                static_cast<size_t>(n), cudaMemcpyDeviceToHost,
                                                ctx->stream), "d2h");
    if (rc) return rc;
    return cp::cuda_status(ctx, cudaStreamSynchronize(ctx->stream), "d2h");
  } catch (const std::exception& e) {
    cp::ctx_error(ctx, "cp_load_jpeg: %s", e.what());
    return CP_ERR_OOM;
  }
}
