// cp_ingest.cpp — frame ingest: PNG files decoded on a pool of host threads straight into the
// caller's (pinned) staging buffer, frame-major, as the compositing entry points read it.
//
// The reference opens every frame with the `image` crate and takes its flat u8 samples
// (src/streams.rs:63-70, src/simple.rs:45-52, src/shake.rs:218-255): one decoder call per
// frame, inside the slicing loop. Here a batch of files is decoded in parallel (one file per
// task) by a restatement of the PNG format (ISO/IEC 15948): chunk walk with CRC check, zlib
// inflate of the concatenated IDAT data, and the five scanline filters. PNG is lossless, so
// the samples are exactly the image's; 8-bit gray, RGB and RGBA without interlacing are
// accepted (the layouts the compositing kernels take), anything else is CP_ERR_IO.

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#ifndef CP_NO_ZLIB
#include <zlib.h>
#endif

#include "../../include/chrono_gpu.h"
#include "cp_host_internal.h"

namespace {

struct PngHeader {
  int32_t width = 0, height = 0, channels = 0;
};

uint32_t be32(const uint8_t* p) {
  return (static_cast<uint32_t>(p[0]) << 24) | (static_cast<uint32_t>(p[1]) << 16) |
         (static_cast<uint32_t>(p[2]) << 8) | static_cast<uint32_t>(p[3]);
}

bool read_file(const char* path, std::vector<uint8_t>* data) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  data->clear();
  uint8_t buf[1 << 16];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) data->insert(data->end(), buf, buf + got);
  const bool ok = !std::ferror(f);
  std::fclose(f);
  return ok;
}

// The Paeth predictor of the PNG specification (filter type 4).
inline uint8_t paeth(int a, int b, int c) {
  const int p = a + b - c;
  const int pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
  if (pa <= pb && pa <= pc) return static_cast<uint8_t>(a);
  if (pb <= pc) return static_cast<uint8_t>(b);
  return static_cast<uint8_t>(c);
}

// Reverses the per-scanline filters of `raw` (height rows of 1 + stride bytes) into `out`
// (rows of `stride` bytes); bpp = bytes per pixel. False on an unknown filter type.
bool unfilter(const uint8_t* raw, int32_t height, size_t stride, int bpp, uint8_t* out) {
  const uint8_t* prev = nullptr;
  for (int32_t y = 0; y < height; ++y) {
    const uint8_t* in = raw + static_cast<size_t>(y) * (stride + 1);
    const uint8_t ft = in[0];
    ++in;
    uint8_t* row = out + static_cast<size_t>(y) * stride;
    switch (ft) {
      case 0:
        std::memcpy(row, in, stride);
        break;
      case 1:
        for (size_t i = 0; i < stride; ++i)
          row[i] = static_cast<uint8_t>(in[i] + (i >= static_cast<size_t>(bpp) ? row[i - bpp] : 0));
        break;
      case 2:
        for (size_t i = 0; i < stride; ++i) row[i] = static_cast<uint8_t>(in[i] + (prev ? prev[i] : 0));
        break;
      case 3:
        for (size_t i = 0; i < stride; ++i) {
          const int a = i >= static_cast<size_t>(bpp) ? row[i - bpp] : 0;
          const int b = prev ? prev[i] : 0;
          row[i] = static_cast<uint8_t>(in[i] + ((a + b) >> 1));
        }
        break;
      case 4:
        for (size_t i = 0; i < stride; ++i) {
          const int a = i >= static_cast<size_t>(bpp) ? row[i - bpp] : 0;
          const int b = prev ? prev[i] : 0;
          const int c = (prev && i >= static_cast<size_t>(bpp)) ? prev[i - bpp] : 0;
          row[i] = static_cast<uint8_t>(in[i] + paeth(a, b, c));
        }
        break;
      default:
        return false;
    }
    prev = row;
  }
  return true;
}

// Walks the chunks of a PNG file: header into `h`, the IDAT payloads concatenated into
// `idat`. Returns CP_OK or CP_ERR_IO with `why` set.
int parse_png(const std::vector<uint8_t>& d, PngHeader* h, std::vector<uint8_t>* idat,
              std::string* why) {
  static const uint8_t kSig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
  if (d.size() < 8 || std::memcmp(d.data(), kSig, 8) != 0) {
    *why = "not a PNG file";
    return CP_ERR_IO;
  }
  size_t pos = 8;
  bool have_header = false, ended = false;
  if (idat) idat->clear();
  while (!ended) {
    if (pos + 12 > d.size()) {
      *why = "truncated chunk";
      return CP_ERR_IO;
    }
    const uint32_t len = be32(&d[pos]);
    const uint8_t* type = &d[pos + 4];
    if (len > d.size() || pos + 12 + len > d.size()) {
      *why = "truncated chunk";
      return CP_ERR_IO;
    }
    const uint8_t* body = &d[pos + 8];
#ifndef CP_NO_ZLIB
    const uLong crc = crc32(crc32(0L, Z_NULL, 0), type, 4 + len);
    if (crc != be32(body + len)) {
      *why = "chunk CRC mismatch";
      return CP_ERR_IO;
    }
#endif
    if (std::memcmp(type, "IHDR", 4) == 0) {
      if (len != 13 || have_header) {
        *why = "bad IHDR";
        return CP_ERR_IO;
      }
      const uint32_t w = be32(body), hh = be32(body + 4);
      const int depth = body[8], color = body[9], comp = body[10], filt = body[11],
                lace = body[12];
      const int ch = color == 0 ? 1 : (color == 2 ? 3 : (color == 6 ? 4 : 0));
      if (depth != 8 || ch == 0 || comp != 0 || filt != 0 || lace != 0) {
        *why = "unsupported PNG (8-bit gray, RGB or RGBA without interlacing only)";
        return CP_ERR_IO;
      }
      if (w == 0 || hh == 0 || w > (1u << 24) || hh > (1u << 24)) {
        *why = "bad image size";
        return CP_ERR_IO;
      }
      h->width = static_cast<int32_t>(w);
      h->height = static_cast<int32_t>(hh);
      h->channels = ch;
      have_header = true;
      if (!idat) return CP_OK;  // header only
    } else if (std::memcmp(type, "IDAT", 4) == 0) {
      if (!have_header) {
        *why = "IDAT before IHDR";
        return CP_ERR_IO;
      }
      idat->insert(idat->end(), body, body + len);
    } else if (std::memcmp(type, "IEND", 4) == 0) {
      ended = true;
    } else if (!(type[0] & 0x20)) {  // an unknown critical chunk (PLTE: palette images)
      *why = "unsupported critical chunk";
      return CP_ERR_IO;
    }
    pos += 12 + len;
  }
  if (!have_header) {
    *why = "no IHDR";
    return CP_ERR_IO;
  }
  return CP_OK;
}

struct Scratch {
  std::vector<uint8_t> file, idat, raw;
};

// Decodes one file into `out` (height rows of width * channels bytes).
int decode_png(const char* path, const PngHeader& want, uint8_t* out, Scratch* s,
               std::string* why) {
#ifdef CP_NO_ZLIB
  (void)path; (void)want; (void)out; (void)s;
  *why = "built without zlib";
  return CP_ERR_UNSUPPORTED;
#else
  if (!read_file(path, &s->file)) {
    *why = std::string("cannot read ") + path;
    return CP_ERR_IO;
  }
  PngHeader h;
  int rc = parse_png(s->file, &h, &s->idat, why);
  if (rc) {
    *why = std::string(path) + ": " + *why;
    return rc;
  }
  if (h.width != want.width || h.height != want.height || h.channels != want.channels) {
    *why = std::string(path) + ": size or channels differ from the stack's";
    return CP_ERR_IO;
  }
  const size_t stride = static_cast<size_t>(h.width) * h.channels;
  const size_t need = static_cast<size_t>(h.height) * (stride + 1);
  s->raw.resize(need);
  uLongf got = static_cast<uLongf>(need);
  if (uncompress(s->raw.data(), &got, s->idat.data(), static_cast<uLong>(s->idat.size())) != Z_OK ||
      got != need) {
    *why = std::string(path) + ": corrupt image data";
    return CP_ERR_IO;
  }
  if (!unfilter(s->raw.data(), h.height, stride, h.channels, out)) {
    *why = std::string(path) + ": unknown scanline filter";
    return CP_ERR_IO;
  }
  return CP_OK;
#endif
}

}  // namespace

extern "C" int cp_png_info(cp_ctx* ctx, const char* path, int32_t* width, int32_t* height,
                           int32_t* channels) {
  if (!path || !width || !height || !channels) return CP_ERR_ARG;
  std::vector<uint8_t> data;
  if (!read_file(path, &data)) {
    cp::ctx_error(ctx, "cannot read %s", path);
    return CP_ERR_IO;
  }
  PngHeader h;
  std::string why;
  const int rc = parse_png(data, &h, nullptr, &why);
  if (rc) {
    cp::ctx_error(ctx, "%s: %s", path, why.c_str());
    return rc;
  }
  *width = h.width;
  *height = h.height;
  *channels = h.channels;
  return CP_OK;
}

extern "C" int cp_load_png(cp_ctx* ctx, const char* const* paths, int32_t n, int32_t threads,
                           uint8_t* out, uint64_t frame_stride, int32_t width, int32_t height,
                           int32_t channels) {
  if (!paths || !out || n < 1 || width < 1 || height < 1 ||
      (channels != 1 && channels != 3 && channels != 4) ||
      frame_stride < static_cast<uint64_t>(width) * height * channels)
    return CP_ERR_ARG;
  for (int32_t i = 0; i < n; ++i)
    if (!paths[i]) return CP_ERR_ARG;
  int workers = threads > 0 ? threads : static_cast<int>(std::thread::hardware_concurrency());
  if (workers < 1) workers = 1;
  if (workers > n) workers = n;
  PngHeader want;
  want.width = width;
  want.height = height;
  want.channels = channels;
  std::atomic<int32_t> next(0);
  std::atomic<int> status(CP_OK);
  std::string first_why;
  std::atomic_flag why_taken = ATOMIC_FLAG_INIT;
  auto work = [&]() {
    Scratch s;
    std::string why;
    for (;;) {
      const int32_t i = next.fetch_add(1);
      if (i >= n || status.load() != CP_OK) return;
      const int rc = decode_png(paths[i], want, out + frame_stride * static_cast<uint64_t>(i), &s,
                                &why);
      if (rc != CP_OK) {
        int expected = CP_OK;
        if (status.compare_exchange_strong(expected, rc) && !why_taken.test_and_set())
          first_why = why;
        return;
      }
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < workers; ++t) pool.emplace_back(work);
  work();
  for (auto& t : pool) t.join();
  if (status.load() != CP_OK) cp::ctx_error(ctx, "%s", first_why.c_str());
  return status.load();
}
