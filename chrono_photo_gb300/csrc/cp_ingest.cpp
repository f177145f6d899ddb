// cp_ingest.cpp — frame ingest: PNG files decoded on a pool of host threads straight into the
// caller's (pinned) staging buffer, frame-major, as the compositing entry points read it.
//
// The reference opens every frame with the `image` crate and takes its flat u8 samples
// (src/streams.rs:63-70, src/simple.rs:45-52, src/shake.rs:218-255): one decoder call per
// frame, inside the slicing loop. Here a batch of files is decoded in parallel (one file per
// task) by a restatement of the PNG format (ISO/IEC 15948): chunk walk with CRC-32 check,
// zlib/DEFLATE decoding (RFC 1950/1951) of the concatenated IDAT data with its Adler-32
// check, and the five scanline filters. The decoder is self-contained (no zlib dependency),
// so the same code decodes on every host. PNG is lossless, so the samples are exactly the
// image's; 8-bit gray, RGB and RGBA without interlacing are accepted (the layouts the
// compositing kernels take), anything else is CP_ERR_IO.

#include <sys/stat.h>

#include <atomic>
#include <new>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/chrono_gpu.h"
#include "cp_host_internal.h"
#include "cp_png.h"

namespace {

using cp::png::adler32;
using cp::png::be32;
using cp::png::crc32_png;
using cp::png::kCodeLenOrder;
using cp::png::kDistBase;
using cp::png::kDistExtra;
using cp::png::kLenBase;
using cp::png::kLenExtra;

struct PngHeader {
  int32_t width = 0, height = 0, channels = 0;
};

// The whole of a regular file into `data` in one read (anything else, e.g. a directory, is
// not an image file: false).
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

// ---- DEFLATE decoder (RFC 1951) writing into a buffer of known size ----

// Canonical Huffman code: symbols sorted by code length; `fast` maps the next kFast input
// bits (least significant first, as DEFLATE packs codes bit-reversed) to symbol << 4 | length
// for codes of at most kFast bits, 0 for longer codes, which the canonical walk decodes.
constexpr int kFast = 11;
constexpr int kMaxBits = 15;

struct Huffman {
  uint16_t count[kMaxBits + 1];
  uint16_t symbol[288];
  uint16_t fast[1 << kFast];
};

// The counts per code length and the symbols in canonical order from per-symbol code
// lengths. False when the lengths over-subscribe the code space; incomplete codes are
// accepted (an unassigned code then fails at decode time).
bool huffman_counts(Huffman* h, const uint8_t* lengths, int n) {
  std::memset(h->count, 0, sizeof h->count);
  for (int s = 0; s < n; ++s) h->count[lengths[s]]++;
  h->count[0] = 0;
  int left = 1;
  for (int len = 1; len <= kMaxBits; ++len) {
    left = (left << 1) - h->count[len];
    if (left < 0) return false;
  }
  uint16_t offs[kMaxBits + 2];
  offs[1] = 0;
  for (int len = 1; len <= kMaxBits; ++len) offs[len + 1] = offs[len] + h->count[len];
  for (int s = 0; s < n; ++s)
    if (lengths[s]) h->symbol[offs[lengths[s]]++] = static_cast<uint16_t>(s);
  return true;
}

// huffman_counts plus the kFast-bit lookup of symbol << 4 | length (the code-length code).
bool build_huffman(Huffman* h, const uint8_t* lengths, int n) {
  if (!huffman_counts(h, lengths, n)) return false;
  std::memset(h->fast, 0, sizeof h->fast);
  uint32_t code = 0;
  int idx = 0;
  for (int len = 1; len <= kFast; ++len) {
    for (int k = 0; k < h->count[len]; ++k, ++idx, ++code) {
      uint32_t rev = 0;
      for (int b = 0; b < len; ++b) rev |= ((code >> b) & 1u) << (len - 1 - b);
      const uint16_t e = static_cast<uint16_t>((h->symbol[idx] << 4) | len);
      for (uint32_t fill = rev; fill < (1u << kFast); fill += 1u << len) h->fast[fill] = e;
    }
    code <<= 1;
  }
  return true;
}

// Literal/length and distance codes as decode entries: for each kFast-bit lookup, the code
// length (bits 0-3), the extra-bit count (bits 4-7), the kind (bits 8-9) and the value
// (bits 16-31: the literal byte, or the base length / distance of RFC 1951 section 3.2.5).
// An entry of 0 marks a code longer than kFast bits, resolved by the canonical walk.
enum : uint32_t { kEntLiteral = 0, kEntBase = 1, kEntEnd = 2, kEntBad = 3 };
inline uint32_t make_entry(uint32_t kind, uint32_t value, uint32_t extra, uint32_t len) {
  return (value << 16) | (kind << 8) | (extra << 4) | len;
}
inline uint32_t ent_len(uint32_t e) { return e & 15u; }
inline uint32_t ent_extra(uint32_t e) { return (e >> 4) & 15u; }
inline uint32_t ent_kind(uint32_t e) { return (e >> 8) & 3u; }
inline uint32_t ent_value(uint32_t e) { return e >> 16; }

struct DecodeTable {
  Huffman h;
  uint32_t e[1 << kFast];
  bool dist = false;
  // The entry of symbol `sym` whose code is `len` bits long.
  uint32_t entry_of(int sym, uint32_t len) const {
    if (dist) {
      if (sym > 29) return make_entry(kEntBad, 0, 0, len);
      return make_entry(kEntBase, kDistBase[sym], kDistExtra[sym], len);
    }
    if (sym < 256) return make_entry(kEntLiteral, static_cast<uint32_t>(sym), 0, len);
    if (sym == 256) return make_entry(kEntEnd, 0, 0, len);
    if (sym > 285) return make_entry(kEntBad, 0, 0, len);
    return make_entry(kEntBase, kLenBase[sym - 257], kLenExtra[sym - 257], len);
  }
  // False when the lengths over-subscribe the code space. Each symbol's entry is made once
  // and replicated over the lookups that start with its (bit-reversed) code.
  bool build(const uint8_t* lengths, int n, bool is_dist) {
    dist = is_dist;
    if (!huffman_counts(&h, lengths, n)) return false;
    std::memset(e, 0, sizeof e);
    uint32_t code = 0;
    int idx = 0;
    for (int len = 1; len <= kFast; ++len) {
      for (int k = 0; k < h.count[len]; ++k, ++idx, ++code) {
        uint32_t rev = 0;
        for (int b = 0; b < len; ++b) rev |= ((code >> b) & 1u) << (len - 1 - b);
        const uint32_t x = entry_of(h.symbol[idx], static_cast<uint32_t>(len));
        for (uint32_t fill = rev; fill < (1u << kFast); fill += 1u << len) e[fill] = x;
      }
      code <<= 1;
    }
    return true;
  }
  // Entry for the next code in `buf` (at least kMaxBits valid bits); a code the table does
  // not assign gives kEntBad with length 0.
  uint32_t lookup(uint64_t buf) const {
    const uint32_t x = e[buf & ((1u << kFast) - 1)];
    return x ? x : lookup_long(buf);
  }
  // Codes longer than kFast bits: the canonical walk (codes of each length are consecutive
  // integers starting at `first`).
  __attribute__((noinline)) uint32_t lookup_long(uint64_t buf) const {
    int code = 0, first = 0, index = 0;
    for (int len = 1; len <= kMaxBits; ++len) {
      code |= static_cast<int>((buf >> (len - 1)) & 1);
      const int count = h.count[len];
      if (code - first < count) return entry_of(h.symbol[index + code - first], static_cast<uint32_t>(len));
      index += count;
      first = (first + count) << 1;
      code <<= 1;
    }
    return make_entry(kEntBad, 0, 0, 0);
  }
};

// Bytes that the decoder may write past the end of its output (match copies move 8-byte
// words); the output buffer must have this many writable bytes after n_out.
constexpr size_t kCopySlack = 16;

class Inflater {
 public:
  Inflater(const uint8_t* in, size_t n_in, uint8_t* out, size_t n_out)
      : in_(in), n_in_(n_in), out_(out), n_out_(n_out) {}

  // Decodes the whole DEFLATE stream; on success `consumed()` is the number of input bytes
  // it occupied (rounded up to a byte) and `produced()` the output length.
  bool run(std::string* why) {
    bool last = false;
    while (!last) {
      last = bits(1) != 0;
      const uint32_t type = bits(2);
      bool ok;
      if (type == 0) ok = stored(why);
      else if (type == 1) ok = fixed(why);
      else if (type == 2) ok = dynamic(why);
      else {
        *why = "bad DEFLATE block type";
        ok = false;
      }
      if (!ok) return false;
      if (overrun()) {
        *why = "truncated image data";
        return false;
      }
    }
    return true;
  }
  size_t produced() const { return pos_out_; }
  size_t consumed() const { return pos_in_ - nbits_ / 8; }

 private:
  // Tops the bit buffer up to at least 56 bits. Away from the end of the input, one
  // unaligned 8-byte little-endian load: whole bytes are consumed, and the bits above
  // nbits_ that the load also sets are the same input bits the next load ORs in again.
  void refill() {
#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__
    if (pos_in_ + 8 <= n_in_) {
      uint64_t v;
      std::memcpy(&v, in_ + pos_in_, 8);
      buf_ |= v << nbits_;
      pos_in_ += (63 - nbits_) >> 3;
      nbits_ |= 56;
      return;
    }
#endif
    while (nbits_ <= 56) {
      const uint64_t byte = pos_in_ < n_in_ ? in_[pos_in_] : 0;  // zeros past the end
      ++pos_in_;
      buf_ |= byte << nbits_;
      nbits_ += 8;
    }
  }
  bool overrun() const { return pos_in_ - nbits_ / 8 > n_in_; }
  uint32_t bits(int n) {
    if (nbits_ < n) refill();
    return bits_buffered(n);
  }
  uint32_t bits_buffered(int n) {
    const uint32_t v = static_cast<uint32_t>(buf_ & ((1ull << n) - 1));
    buf_ >>= n;
    nbits_ -= n;
    return v;
  }

  // Next symbol of `h`, or -1 for a code that the table does not assign.
  int decode(const Huffman& h) {
    if (nbits_ < kMaxBits) refill();
    return decode_buffered(h);
  }
  // decode() with at least kMaxBits bits already in the buffer.
  int decode_buffered(const Huffman& h) {
    const uint16_t e = h.fast[buf_ & ((1u << kFast) - 1)];
    if (e) {
      buf_ >>= e & 15;
      nbits_ -= e & 15;
      return e >> 4;
    }
    // Canonical walk: codes of each length are consecutive integers starting at `first`.
    int code = 0, first = 0, index = 0;
    for (int len = 1; len <= kMaxBits; ++len) {
      code |= static_cast<int>((buf_ >> (len - 1)) & 1);
      const int count = h.count[len];
      if (code - first < count) {
        buf_ >>= len;
        nbits_ -= len;
        return h.symbol[index + code - first];
      }
      index += count;
      first = (first + count) << 1;
      code <<= 1;
    }
    return -1;
  }

  bool stored(std::string* why) {
    // Drop the bits up to the next byte boundary, then return whole unread bytes to the input.
    buf_ >>= nbits_ & 7;
    nbits_ -= nbits_ & 7;
    pos_in_ -= nbits_ / 8;
    buf_ = 0;
    nbits_ = 0;
    if (pos_in_ + 4 > n_in_) {
      *why = "truncated image data";
      return false;
    }
    const uint32_t len = in_[pos_in_] | (in_[pos_in_ + 1] << 8);
    const uint32_t nlen = in_[pos_in_ + 2] | (in_[pos_in_ + 3] << 8);
    pos_in_ += 4;
    if ((len ^ 0xFFFFu) != nlen) {
      *why = "bad stored block length";
      return false;
    }
    if (pos_in_ + len > n_in_ || pos_out_ + len > n_out_) {
      *why = pos_in_ + len > n_in_ ? "truncated image data" : "image data longer than the image";
      return false;
    }
    std::memcpy(out_ + pos_out_, in_ + pos_in_, len);
    pos_in_ += len;
    pos_out_ += len;
    return true;
  }

  bool fixed(std::string* why) {
    static const struct Fixed {
      DecodeTable lit, dist;
      Fixed() {
        uint8_t l[288];
        for (int s = 0; s < 288; ++s) l[s] = s < 144 ? 8 : (s < 256 ? 9 : (s < 280 ? 7 : 8));
        lit.build(l, 288, false);
        uint8_t d[30];
        std::memset(d, 5, sizeof d);
        dist.build(d, 30, true);
      }
    } F;
    return codes(F.lit, F.dist, why);
  }

  bool dynamic(std::string* why) {
    const int nlen = static_cast<int>(bits(5)) + 257;
    const int ndist = static_cast<int>(bits(5)) + 1;
    const int ncode = static_cast<int>(bits(4)) + 4;
    if (nlen > 286 || ndist > 30) {
      *why = "bad dynamic block header";
      return false;
    }
    uint8_t lengths[320];
    std::memset(lengths, 0, 19);
    for (int i = 0; i < ncode; ++i) lengths[kCodeLenOrder[i]] = static_cast<uint8_t>(bits(3));
    Huffman lencode;
    if (!build_huffman(&lencode, lengths, 19)) {
      *why = "bad code-length code";
      return false;
    }
    int i = 0;
    while (i < nlen + ndist) {
      const int sym = decode(lencode);
      if (sym < 0) {
        *why = "bad code-length code";
        return false;
      }
      if (sym < 16) {
        lengths[i++] = static_cast<uint8_t>(sym);
        continue;
      }
      int rep;
      uint8_t val = 0;
      if (sym == 16) {
        if (i == 0) {
          *why = "repeat without a previous length";
          return false;
        }
        val = lengths[i - 1];
        rep = 3 + static_cast<int>(bits(2));
      } else if (sym == 17) {
        rep = 3 + static_cast<int>(bits(3));
      } else {
        rep = 11 + static_cast<int>(bits(7));
      }
      if (i + rep > nlen + ndist) {
        *why = "code lengths overflow";
        return false;
      }
      while (rep--) lengths[i++] = val;
    }
    if (lengths[256] == 0) {
      *why = "no end-of-block code";
      return false;
    }
    DecodeTable lit, dist;
    if (!lit.build(lengths, nlen, false) || !dist.build(lengths + nlen, ndist, true)) {
      *why = "over-subscribed Huffman code";
      return false;
    }
    return codes(lit, dist, why);
  }

  // Literal/length + distance symbols of one compressed block, up to end-of-block (256).
  bool codes(const DecodeTable& lit, const DecodeTable& dist, std::string* why) {
    for (;;) {
      // One symbol with its match takes at most 15 + 5 + 15 + 13 = 48 bits.
      if (nbits_ < 48) refill();
      uint32_t e = lit.lookup(buf_);
      if (ent_kind(e) == kEntLiteral) {
        if (pos_out_ >= n_out_) return fail(why, "image data longer than the image");
        consume(ent_len(e));
        out_[pos_out_++] = static_cast<uint8_t>(ent_value(e));
        // a second literal needs at most 15 of the >= 33 bits left: no refill
        e = lit.lookup(buf_);
        if (ent_kind(e) == kEntLiteral) {
          if (pos_out_ >= n_out_) return fail(why, "image data longer than the image");
          consume(ent_len(e));
          out_[pos_out_++] = static_cast<uint8_t>(ent_value(e));
          continue;
        }
        if (nbits_ < 48) refill();  // the low bits, and so `e`, are unchanged by a refill
      }
      if (ent_kind(e) != kEntBase) {
        if (ent_kind(e) == kEntEnd) {
          consume(ent_len(e));
          return true;
        }
        return fail(why, "bad literal/length code");
      }
      consume(ent_len(e));
      const size_t len = ent_value(e) + bits_buffered(static_cast<int>(ent_extra(e)));
      const uint32_t de = dist.lookup(buf_);
      if (ent_kind(de) != kEntBase) return fail(why, "bad distance code");
      consume(ent_len(de));
      const size_t d = ent_value(de) + bits_buffered(static_cast<int>(ent_extra(de)));
      if (d > pos_out_) return fail(why, "distance before the start of the data");
      if (len > n_out_ - pos_out_) return fail(why, "image data longer than the image");
      uint8_t* dst = out_ + pos_out_;
      const uint8_t* src = dst - d;
      if (d >= 8) {
        // 8-byte words, each read from bytes already final (d >= 8); the last word may
        // run up to 7 bytes past the match, into bytes written later or the slack.
        uint8_t* const end = dst + len;
        do {
          uint64_t w;
          std::memcpy(&w, src, 8);
          std::memcpy(dst, &w, 8);
          src += 8;
          dst += 8;
        } while (dst < end);
      } else {
        for (size_t k = 0; k < len; ++k) dst[k] = src[k];  // overlapping copy repeats the run
      }
      pos_out_ += len;
      if (overrun()) return fail(why, "truncated image data");
    }
  }

  void consume(uint32_t n) {
    buf_ >>= n;
    nbits_ -= static_cast<int>(n);
  }
  static bool fail(std::string* why, const char* what) {
    *why = what;
    return false;
  }

  const uint8_t* in_;
  size_t n_in_, pos_in_ = 0;
  uint8_t* out_;
  size_t n_out_, pos_out_ = 0;
  uint64_t buf_ = 0;
  int nbits_ = 0;
};

// Decompresses a zlib stream (RFC 1950: header, DEFLATE data, Adler-32 of the output) into
// exactly `n_out` bytes; `out` has kCopySlack writable bytes beyond them.
bool zlib_decode(const uint8_t* in, size_t n_in, uint8_t* out, size_t n_out, std::string* why) {
  if (n_in < 6 || (in[0] & 15) != 8 || (in[0] >> 4) > 7 || ((in[0] << 8) | in[1]) % 31 != 0 ||
      (in[1] & 0x20)) {
    *why = "bad zlib header";
    return false;
  }
  Inflater inf(in + 2, n_in - 2, out, n_out);
  if (!inf.run(why)) return false;
  if (inf.produced() != n_out) {
    *why = "image data shorter than the image";
    return false;
  }
  const size_t tail = 2 + inf.consumed();
  if (tail + 4 > n_in || be32(in + tail) != adler32(out, n_out)) {
    *why = tail + 4 > n_in ? "truncated image data" : "Adler-32 mismatch";
    return false;
  }
  return true;
}

// The Paeth predictor of the PNG specification (filter type 4): of a (left), b (above) and
// c (upper left), the one nearest to a + b - c, ties in the order a, b, c. Written with
// selects rather than branches: on noisy images the choice is unpredictable.
inline int paeth(int a, int b, int c) {
  const int pa = std::abs(b - c), pb = std::abs(a - c), pc = std::abs(a + b - 2 * c);
  const int bc = pb <= pc ? b : c;
  return ((pa <= pb) & (pa <= pc)) ? a : bc;
}

// Reverses the per-scanline filters of `raw` (height rows of 1 + stride bytes) into `out`
// (rows of `stride` bytes) for BPP bytes per pixel. The row above the first is zero, as is
// the pixel left of the first. False on an unknown filter type.
template <int BPP>
bool unfilter_bpp(const uint8_t* raw, int32_t height, size_t stride, uint8_t* out,
                  const uint8_t* zero_row) {
  for (int32_t y = 0; y < height; ++y) {
    const uint8_t* in = raw + static_cast<size_t>(y) * (stride + 1);
    const uint8_t ft = *in++;
    uint8_t* row = out + static_cast<size_t>(y) * stride;
    const uint8_t* prev = y ? row - stride : zero_row;
    switch (ft) {
      case 0:
        std::memcpy(row, in, stride);
        break;
      case 1: {
        uint8_t a[BPP] = {};
        for (size_t i = 0; i < stride; i += BPP)
          for (int k = 0; k < BPP; ++k) row[i + k] = a[k] = static_cast<uint8_t>(in[i + k] + a[k]);
        break;
      }
      case 2:
        for (size_t i = 0; i < stride; ++i) row[i] = static_cast<uint8_t>(in[i] + prev[i]);
        break;
      case 3: {
        int a[BPP] = {};
        for (size_t i = 0; i < stride; i += BPP)
          for (int k = 0; k < BPP; ++k) {
            a[k] = static_cast<uint8_t>(in[i + k] + ((a[k] + prev[i + k]) >> 1));
            row[i + k] = static_cast<uint8_t>(a[k]);
          }
        break;
      }
      case 4: {
        int a[BPP] = {}, c[BPP] = {};
        for (size_t i = 0; i < stride; i += BPP)
          for (int k = 0; k < BPP; ++k) {
            const int b = prev[i + k];
            a[k] = static_cast<uint8_t>(in[i + k] + paeth(a[k], b, c[k]));
            c[k] = b;
            row[i + k] = static_cast<uint8_t>(a[k]);
          }
        break;
      }
      default:
        return false;
    }
  }
  return true;
}

bool unfilter(const uint8_t* raw, int32_t height, size_t stride, int bpp, uint8_t* out) {
  std::vector<uint8_t> zero_row(stride, 0);
  if (bpp == 1) return unfilter_bpp<1>(raw, height, stride, out, zero_row.data());
  if (bpp == 3) return unfilter_bpp<3>(raw, height, stride, out, zero_row.data());
  return unfilter_bpp<4>(raw, height, stride, out, zero_row.data());
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
    if (crc32_png(type, 4 + len) != be32(body + len)) {
      *why = "chunk CRC mismatch";
      return CP_ERR_IO;
    }
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
  s->raw.resize(need + kCopySlack);
  if (!zlib_decode(s->idat.data(), s->idat.size(), s->raw.data(), need, why)) {
    *why = std::string(path) + ": " + *why;
    return CP_ERR_IO;
  }
  if (!unfilter(s->raw.data(), h.height, stride, h.channels, out)) {
    *why = std::string(path) + ": unknown scanline filter";
    return CP_ERR_IO;
  }
  return CP_OK;
}

}  // namespace

// Runs an entry point's body so that no C++ exception crosses the C ABI: allocation and
// thread failures become CP_ERR_OOM with the reason in the context's message.
template <typename Fn>
int guarded(cp_ctx* ctx, const char* what, Fn fn) {
  try {
    return fn();
  } catch (const std::exception& e) {
    cp::ctx_error(ctx, "%s: %s", what, e.what());
    return CP_ERR_OOM;
  }
}

extern "C" int cp_png_info(cp_ctx* ctx, const char* path, int32_t* width, int32_t* height,
                           int32_t* channels) {
  if (!path || !width || !height || !channels) return CP_ERR_ARG;
  return guarded(ctx, "cp_png_info", [&]() {
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
  });
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
      int rc;
      try {
        rc = decode_png(paths[i], want, out + frame_stride * static_cast<uint64_t>(i), &s, &why);
      } catch (const std::exception&) {  // no exception may end a worker thread
        rc = CP_ERR_OOM;
        why.clear();
      }
      if (rc != CP_OK) {
        int expected = CP_OK;
        if (status.compare_exchange_strong(expected, rc) && !why_taken.test_and_set()) {
          try {
            first_why = why.empty() ? std::string(paths[i]) + ": out of host memory" : why;
          } catch (const std::exception&) {
          }
        }
        return;
      }
    }
  };
  std::vector<std::thread> pool;
  try {
    pool.reserve(static_cast<size_t>(workers));
    for (int t = 1; t < workers; ++t) pool.emplace_back(work);
  } catch (const std::exception&) {
    // fewer threads than asked for: the ones started, and this one, share the frames
  }
  work();
  for (auto& t : pool) t.join();
  if (status.load() != CP_OK) cp::ctx_error(ctx, "%s", first_why.c_str());
  return status.load();
}
