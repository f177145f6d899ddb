// cp_png_write.cpp — output encode: composites and blend masks written as PNG files.
//
// The reference saves each output image with image::save_buffer (the JPEG encoder for .jpg),
// picking the format from the file extension and creating a missing parent directory
// (src/main.rs:519-570; the blend mask at :489-491). This writes PNG, which is lossless, so
// the saved samples are exactly the composite's. The published formats are restated here:
// adaptive scanline filters (ISO/IEC 15948: per row, the filter whose output has the
// smallest sum of absolute signed bytes), a zlib stream (RFC 1950) whose DEFLATE data
// (RFC 1951) comes from a hash-chain LZ77 matcher, each block coded as the cheapest of
// stored, fixed-Huffman and dynamic-Huffman, with code lengths limited to 15 bits (7 for the
// code-length code) by the Kraft-preserving adjustment of ISO/IEC 10918-1 Annex K.3.

#include <sys/stat.h>
#include <sys/types.h>

#include <algorithm>
#include <atomic>
#include <new>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/chrono_gpu.h"
#include "cp_host_internal.h"
#include "cp_io.h"
#include "cp_png.h"

namespace {

using cp::open_output;
using cp::run_parallel;

constexpr int kWindow = 32768;
constexpr int kMinMatch = 3, kMaxMatch = 258;
constexpr int kLitLen = 286, kDist = 30, kCodeLen = 19;

using cp::png::kCodeLenOrder;
using cp::png::kDistBase;
using cp::png::kDistExtra;
using cp::png::kLenBase;
using cp::png::kLenExtra;

// Length 3..258 -> length symbol index (0..28); distance 1..32768 -> distance symbol.
struct SymbolTables {
  uint8_t len_sym[kMaxMatch + 1];
  uint8_t dist_sym[kWindow + 1];
  SymbolTables() {
    for (int s = 0; s < 29; ++s) {
      const int hi = s == 28 ? kMaxMatch : kLenBase[s] + (1 << kLenExtra[s]) - 1;
      for (int l = kLenBase[s]; l <= hi && l <= kMaxMatch; ++l) len_sym[l] = static_cast<uint8_t>(s);
    }
    len_sym[kMaxMatch] = 28;  // 258 has its own symbol (285), not 284 + extra 31
    for (int s = 0; s < 30; ++s) {
      const int hi = kDistBase[s] + (1 << kDistExtra[s]) - 1;
      for (int d = kDistBase[s]; d <= hi && d <= kWindow; ++d) dist_sym[d] = static_cast<uint8_t>(s);
    }
  }
};
const SymbolTables& tables() {
  static const SymbolTables T;
  return T;
}

// LSB-first bit writer (DEFLATE packs data elements starting at the least significant bit).
class BitWriter {
 public:
  explicit BitWriter(std::vector<uint8_t>* out) : out_(out) {}
  void put(uint32_t bits, int n) {
    buf_ |= static_cast<uint64_t>(bits) << nbits_;
    nbits_ += n;
    while (nbits_ >= 8) {
      out_->push_back(static_cast<uint8_t>(buf_));
      buf_ >>= 8;
      nbits_ -= 8;
    }
  }
  void align() {
    if (nbits_ > 0) put(0, 8 - nbits_);
  }
  int pending_bits() const { return nbits_; }

 private:
  std::vector<uint8_t>* out_;
  uint64_t buf_ = 0;
  int nbits_ = 0;
};

// Code lengths of at most `limit` bits for `n` symbols with frequencies `freq` (0: unused
// symbol, length 0). Huffman's construction by the two-queue method over the sorted
// leaves; when the deepest leaf exceeds the limit, leaves are moved up pairwise keeping the
// code complete (ISO/IEC 10918-1 Annex K.3), and the lengths are dealt out again in order
// of decreasing frequency.
void huffman_lengths(const uint32_t* freq, int n, int limit, uint8_t* len) {
  std::fill(len, len + n, 0);
  std::vector<int> leaves;
  for (int s = 0; s < n; ++s)
    if (freq[s]) leaves.push_back(s);
  const int m = static_cast<int>(leaves.size());
  if (m == 0) return;
  if (m == 1) {
    len[leaves[0]] = 1;
    return;
  }
  std::sort(leaves.begin(), leaves.end(), [&](int a, int b) {
    return freq[a] != freq[b] ? freq[a] < freq[b] : a < b;
  });
  // nodes 0..m-1 are the leaves in sorted order, m.. the internal nodes in creation order
  std::vector<uint64_t> weight(static_cast<size_t>(2 * m - 1));
  std::vector<int> parent(static_cast<size_t>(2 * m - 1), -1);
  for (int i = 0; i < m; ++i) weight[static_cast<size_t>(i)] = freq[leaves[static_cast<size_t>(i)]];
  int qa = 0, qb = m, next = m;
  auto pop = [&]() {
    if (qa < m && (qb >= next || weight[static_cast<size_t>(qa)] <= weight[static_cast<size_t>(qb)]))
      return qa++;
    return qb++;
  };
  while (next < 2 * m - 1) {
    const int x = pop(), y = pop();
    weight[static_cast<size_t>(next)] = weight[static_cast<size_t>(x)] + weight[static_cast<size_t>(y)];
    parent[static_cast<size_t>(x)] = parent[static_cast<size_t>(y)] = next;
    ++next;
  }
  std::vector<int> depth(static_cast<size_t>(2 * m - 1), 0);
  for (int i = 2 * m - 3; i >= 0; --i)
    depth[static_cast<size_t>(i)] = depth[static_cast<size_t>(parent[static_cast<size_t>(i)])] + 1;
  int maxd = 0;
  std::vector<int> count(static_cast<size_t>(2 * m + 2), 0);
  for (int i = 0; i < m; ++i) {
    const int d = depth[static_cast<size_t>(i)];
    ++count[static_cast<size_t>(d)];
    maxd = std::max(maxd, d);
  }
  for (int i = maxd; i > limit; --i) {
    while (count[static_cast<size_t>(i)] > 0) {
      int j = i - 2;
      while (j > 0 && count[static_cast<size_t>(j)] == 0) --j;
      count[static_cast<size_t>(i)] -= 2;      // two leaves leave the deepest level: their
      count[static_cast<size_t>(i - 1)] += 1;  // parent becomes a leaf, and a leaf at level j
      count[static_cast<size_t>(j + 1)] += 2;  // becomes the parent of one of them and
      count[static_cast<size_t>(j)] -= 1;      // another leaf one level down
    }
  }
  // the most frequent symbols take the shortest lengths
  int k = m - 1;
  for (int d = 1; d <= std::min(maxd, limit); ++d)
    for (int c = 0; c < count[static_cast<size_t>(d)]; ++c, --k)
      len[leaves[static_cast<size_t>(k)]] = static_cast<uint8_t>(d);
}

// Canonical codes (RFC 1951 section 3.2.2), bit-reversed for LSB-first output.
void canonical_codes(const uint8_t* len, int n, uint16_t* code) {
  int bl_count[16] = {0};
  for (int s = 0; s < n; ++s) ++bl_count[len[s]];
  bl_count[0] = 0;
  int next_code[16] = {0};
  int c = 0;
  for (int b = 1; b < 16; ++b) {
    c = (c + bl_count[b - 1]) << 1;
    next_code[b] = c;
  }
  for (int s = 0; s < n; ++s) {
    code[s] = 0;
    if (!len[s]) continue;
    const uint32_t v = static_cast<uint32_t>(next_code[len[s]]++);
    uint32_t r = 0;
    for (int b = 0; b < len[s]; ++b) r |= ((v >> b) & 1u) << (len[s] - 1 - b);
    code[s] = static_cast<uint16_t>(r);
  }
}

// One LZ77 token: a literal byte (dist == 0) or a match of `len` bytes `dist` back.
struct Token {
  uint16_t len;   // the literal byte, or the match length 3..258
  uint16_t dist;  // 0 for a literal, else the distance 1..32768
};

// Effort per zlib level 1..9: hash-chain candidates examined per position, and the match
// length at which the search stops early.
struct Effort {
  int chain, nice;
};
Effort effort(int level) {
  static const Effort kE[10] = {{0, 0},    {4, 16},    {6, 32},    {8, 64},     {12, 128},
                                {16, 128}, {32, 128},  {128, 258}, {1024, 258}, {4096, 258}};
  return kE[std::min(std::max(level, 0), 9)];
}

// Hash-chain LZ77 over the whole input (32 KB window, greedy parse): head[] holds the
// latest position of each 3-byte hash, prev[] the previous position with the same hash.
// Length of the common prefix of a and b, at most max_len (b - a >= 1; both readable for
// max_len bytes). Eight bytes per step on little-endian hosts: the first differing byte is
// the lowest set bit of the XOR.
inline int match_length(const uint8_t* a, const uint8_t* b, int max_len) {
  int l = 0;
#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__
  while (l + 8 <= max_len) {
    uint64_t x, y;
    std::memcpy(&x, a + l, 8);
    std::memcpy(&y, b + l, 8);
    if (x != y) return l + (__builtin_ctzll(x ^ y) >> 3);
    l += 8;
  }
#endif
  while (l < max_len && a[l] == b[l]) ++l;
  return l;
}

class Matcher {
 public:
  Matcher(const uint8_t* data, size_t n, int level)
      : d_(data), n_(n), e_(effort(level)), head_(1u << kHashBits, -1), prev_(kWindow, -1) {}

  // Makes positions [from, to) available as match sources without coding them (the window
  // before a segment).
  void prime(size_t from, size_t to) {
    for (size_t p = from; p < to && p + kMinMatch <= n_; ++p) insert(p, hash(p));
  }

  // Tokens for [pos, end) appended to `out`; returns the position reached (>= end: a match
  // may run past `end`, never past the matcher's own end n).
  size_t parse(size_t pos, size_t end, std::vector<Token>* out) {
    while (pos < end) {
      int best_len = 0, best_dist = 0;
      if (pos + kMinMatch <= n_) {
        const uint32_t h = hash(pos);
        const int max_len = static_cast<int>(std::min<size_t>(kMaxMatch, n_ - pos));
        int64_t cand = head_[h];
        for (int chain = e_.chain; cand >= 0 && chain > 0; --chain) {
          const size_t dist = pos - static_cast<size_t>(cand);
          if (dist > static_cast<size_t>(kWindow)) break;
          const uint8_t* a = d_ + cand;
          const uint8_t* b = d_ + pos;
          if (a[best_len] == b[best_len] && a[0] == b[0] && a[1] == b[1]) {
            const int l = match_length(a, b, max_len);
            if (l > best_len) {
              best_len = l;
              best_dist = static_cast<int>(dist);
              if (l >= e_.nice || l >= max_len) break;
            }
          }
          const int64_t nxt = prev_[static_cast<size_t>(cand) & (kWindow - 1)];
          if (nxt >= cand) break;
          cand = nxt;
        }
        insert(pos, h);
      }
      if (best_len >= kMinMatch) {
        out->push_back(Token{static_cast<uint16_t>(best_len), static_cast<uint16_t>(best_dist)});
        for (size_t q = pos + 1; q < pos + static_cast<size_t>(best_len); ++q)
          if (q + kMinMatch <= n_) insert(q, hash(q));
        pos += static_cast<size_t>(best_len);
      } else {
        out->push_back(Token{d_[pos], 0});
        ++pos;
      }
    }
    return pos;
  }

 private:
  static constexpr int kHashBits = 15;
  uint32_t hash(size_t p) const {
    const uint32_t v = d_[p] | (static_cast<uint32_t>(d_[p + 1]) << 8) |
                       (static_cast<uint32_t>(d_[p + 2]) << 16);
    return (v * 2654435761u) >> (32 - kHashBits);
  }
  void insert(size_t p, uint32_t h) {
    prev_[p & (kWindow - 1)] = head_[h];
    head_[h] = static_cast<int64_t>(p);
  }
  const uint8_t* d_;
  size_t n_;
  Effort e_;
  std::vector<int64_t> head_, prev_;  // positions; -1: none
};

// Fixed Huffman code lengths (RFC 1951 section 3.2.6).
void fixed_lengths(uint8_t* ll, uint8_t* dl) {
  for (int s = 0; s < 288; ++s) ll[s] = s < 144 ? 8 : (s < 256 ? 9 : (s < 280 ? 7 : 8));
  for (int s = 0; s < 30; ++s) dl[s] = 5;
}

// Run-length form of the code lengths of a dynamic block header (symbols 0-15 literal
// lengths, 16 = repeat previous 3-6, 17 = zeros 3-10, 18 = zeros 11-138).
struct ClSym {
  uint8_t sym, extra;
};
std::vector<ClSym> rle_lengths(const uint8_t* lens, int n) {
  std::vector<ClSym> out;
  int i = 0;
  while (i < n) {
    const uint8_t v = lens[i];
    int run = 1;
    while (i + run < n && lens[i + run] == v) ++run;
    int left = run;
    if (v == 0) {
      while (left >= 11) {
        const int r = std::min(left, 138);
        out.push_back(ClSym{18, static_cast<uint8_t>(r - 11)});
        left -= r;
      }
      if (left >= 3) {
        out.push_back(ClSym{17, static_cast<uint8_t>(left - 3)});
        left = 0;
      }
    } else {
      out.push_back(ClSym{v, 0});
      --left;
      while (left >= 3) {
        const int r = std::min(left, 6);
        out.push_back(ClSym{16, static_cast<uint8_t>(r - 3)});
        left -= r;
      }
    }
    for (; left > 0; --left) out.push_back(ClSym{v, 0});
    i += run;
  }
  return out;
}

// Writes the tokens of one block covering input bytes [begin, end) as the cheapest of a
// stored, a fixed-Huffman and a dynamic-Huffman block (exact bit counts); stored only when
// `toks` is null (no parse at level 0).
void write_block(BitWriter& bw, const std::vector<Token>* tok_list, const uint8_t* data,
                 size_t begin, size_t end, bool final) {
  static const std::vector<Token> kNone;
  const std::vector<Token>& toks = tok_list ? *tok_list : kNone;
  const SymbolTables& T = tables();
  uint32_t lf[kLitLen] = {0}, df[kDist] = {0};
  uint64_t extra_bits = 0;
  for (const Token& t : toks) {
    if (!t.dist) {
      ++lf[t.len];
    } else {
      const int ls = T.len_sym[t.len], ds = T.dist_sym[t.dist];
      ++lf[257 + ls];
      ++df[ds];
      extra_bits += kLenExtra[ls] + kDistExtra[ds];
    }
  }
  lf[256] = 1;  // end of block

  // dynamic code
  uint8_t ll[kLitLen], dl[kDist];
  huffman_lengths(lf, kLitLen, 15, ll);
  huffman_lengths(df, kDist, 15, dl);
  bool any_dist = false;
  for (int s = 0; s < kDist; ++s) any_dist = any_dist || dl[s];
  if (!any_dist) dl[0] = 1;  // one distance code of one bit stands for "no distances"
  int hlit = kLitLen, hdist = kDist;
  while (hlit > 257 && !ll[hlit - 1]) --hlit;
  while (hdist > 1 && !dl[hdist - 1]) --hdist;
  uint8_t all[kLitLen + kDist];
  std::memcpy(all, ll, static_cast<size_t>(hlit));
  std::memcpy(all + hlit, dl, static_cast<size_t>(hdist));
  const std::vector<ClSym> cls = rle_lengths(all, hlit + hdist);
  uint32_t cf[kCodeLen] = {0};
  for (const ClSym& c : cls) ++cf[c.sym];
  uint8_t cl[kCodeLen];
  huffman_lengths(cf, kCodeLen, 7, cl);
  // decoders accept an incomplete code only for distances: a code-length code with a single
  // symbol gets a second, unused one-bit code
  int cl_used = 0;
  for (int s = 0; s < kCodeLen; ++s) cl_used += cl[s] ? 1 : 0;
  if (cl_used == 1) cl[cl[0] ? 1 : 0] = 1;
  int hclen = kCodeLen;
  while (hclen > 4 && !cl[kCodeLenOrder[hclen - 1]]) --hclen;
  uint64_t dyn = 3 + 5 + 5 + 4 + 3 * static_cast<uint64_t>(hclen) + extra_bits;
  for (const ClSym& c : cls) dyn += cl[c.sym] + (c.sym == 16 ? 2 : c.sym == 17 ? 3 : c.sym == 18 ? 7 : 0);
  for (int s = 0; s < kLitLen; ++s) dyn += static_cast<uint64_t>(lf[s]) * ll[s];
  for (int s = 0; s < kDist; ++s) dyn += static_cast<uint64_t>(df[s]) * dl[s];

  // fixed code
  uint8_t fll[288], fdl[30];
  fixed_lengths(fll, fdl);
  uint64_t fix = 3 + extra_bits;
  for (int s = 0; s < kLitLen; ++s) fix += static_cast<uint64_t>(lf[s]) * fll[s];
  for (int s = 0; s < kDist; ++s) fix += static_cast<uint64_t>(df[s]) * fdl[s];

  // stored: header bits, padding to a byte, then LEN/NLEN + bytes per 65535-byte piece
  const uint64_t raw = end - begin;
  const uint64_t pieces = std::max<uint64_t>(1, (raw + 65534) / 65535);
  const uint64_t stored = pieces * (3 + 32) + 7 + 8 * raw;

  if (!tok_list || (stored <= dyn && stored <= fix)) {
    for (uint64_t k = 0; k < pieces; ++k) {
      const size_t a = begin + static_cast<size_t>(k * 65535);
      const size_t b = std::min(end, a + 65535);
      bw.put((final && k + 1 == pieces) ? 1u : 0u, 1);
      bw.put(0, 2);
      bw.align();
      const uint32_t len = static_cast<uint32_t>(b - a);
      bw.put(len, 16);
      bw.put(len ^ 0xFFFFu, 16);
      for (size_t i = a; i < b; ++i) bw.put(data[i], 8);
    }
    return;
  }
  const bool use_fixed = fix <= dyn;
  const uint8_t* L = use_fixed ? fll : ll;
  const uint8_t* D = use_fixed ? fdl : dl;
  const int nl = use_fixed ? 288 : kLitLen;
  uint16_t lcode[288], dcode[30];
  canonical_codes(L, nl, lcode);
  canonical_codes(D, 30, dcode);
  bw.put(final ? 1u : 0u, 1);
  bw.put(use_fixed ? 1u : 2u, 2);
  if (!use_fixed) {
    uint16_t ccode[kCodeLen];
    canonical_codes(cl, kCodeLen, ccode);
    bw.put(static_cast<uint32_t>(hlit - 257), 5);
    bw.put(static_cast<uint32_t>(hdist - 1), 5);
    bw.put(static_cast<uint32_t>(hclen - 4), 4);
    for (int i = 0; i < hclen; ++i) bw.put(cl[kCodeLenOrder[i]], 3);
    for (const ClSym& c : cls) {
      bw.put(ccode[c.sym], cl[c.sym]);
      if (c.sym == 16) bw.put(c.extra, 2);
      else if (c.sym == 17) bw.put(c.extra, 3);
      else if (c.sym == 18) bw.put(c.extra, 7);
    }
  }
  for (const Token& t : toks) {
    if (!t.dist) {
      bw.put(lcode[t.len], L[t.len]);
      continue;
    }
    const int ls = T.len_sym[t.len], ds = T.dist_sym[t.dist];
    bw.put(lcode[257 + ls], L[257 + ls]);
    if (kLenExtra[ls]) bw.put(static_cast<uint32_t>(t.len - kLenBase[ls]), kLenExtra[ls]);
    bw.put(dcode[ds], D[ds]);
    if (kDistExtra[ds]) bw.put(static_cast<uint32_t>(t.dist - kDistBase[ds]), kDistExtra[ds]);
  }
  bw.put(lcode[256], L[256]);
}

// Compressed independently: the filtered data is cut into segments of this many bytes, a
// fixed size so that the file does not depend on the number of threads.
constexpr size_t kSegment = 256 * 1024;
constexpr size_t kBlockTokens = 1u << 15;

// DEFLATE data of data[begin, end) whose matches reach back at most into the 32 KB before
// `begin`. A segment other than the last ends with an empty stored block (BFINAL 0, LEN 0),
// which ends it on a byte boundary, so that the segments' bytes concatenate into one stream
// (the method of parallel gzip).
std::vector<uint8_t> deflate_segment(const uint8_t* data, size_t begin, size_t end, int level,
                                     bool last) {
  std::vector<uint8_t> out;
  out.reserve((end - begin) / 2 + 64);
  BitWriter bw(&out);
  if (level <= 0) {
    write_block(bw, nullptr, data, begin, end, last);
  } else {
    Matcher m(data, end, level);
    m.prime(begin > static_cast<size_t>(kWindow) ? begin - kWindow : 0, begin);
    std::vector<Token> toks;
    size_t pos = begin;
    while (pos < end) {
      toks.clear();
      const size_t b = pos;
      while (pos < end && toks.size() < kBlockTokens) pos = m.parse(pos, pos + 1, &toks);
      write_block(bw, &toks, data, b, pos, last && pos >= end);
    }
  }
  if (!last) {
    bw.put(0, 3);
    bw.align();
    bw.put(0, 16);
    bw.put(0xFFFFu, 16);
  }
  bw.align();
  return out;
}

// zlib stream (RFC 1950) of `data` at `level` (0: stored blocks only), its segments
// compressed on `threads` threads.
std::vector<uint8_t> zlib_encode(const uint8_t* data, size_t n, int level, int threads) {
  const size_t nseg = std::max<size_t>(1, (n + kSegment - 1) / kSegment);
  std::vector<std::vector<uint8_t>> segs(nseg);
  run_parallel(nseg, threads, [&](size_t i) {
    const size_t b = i * kSegment, e = std::min(n, b + kSegment);
    segs[i] = deflate_segment(data, b, e, level, i + 1 == nseg);
  });
  std::vector<uint8_t> out;
  size_t total = 6;
  for (const auto& v : segs) total += v.size();
  out.reserve(total);
  out.push_back(0x78);  // deflate, 32 KB window
  out.push_back(level <= 1 ? 0x01 : level <= 5 ? 0x5E : level == 6 ? 0x9C : 0xDA);
  for (const auto& v : segs) out.insert(out.end(), v.begin(), v.end());
  uint8_t a[4];
  cp::png::put_be32(a, cp::png::adler32(data, n));
  out.insert(out.end(), a, a + 4);
  return out;
}

// The Paeth predictor (filter type 4) with selects instead of branches.
inline int paeth_pred(int a, int b, int c) {
  const int pa = std::abs(b - c), pb = std::abs(a - c), pc = std::abs(a + b - 2 * c);
  const int bc = pb <= pc ? b : c;
  return ((pa <= pb) & (pa <= pc)) ? a : bc;
}
inline uint32_t sabs(uint8_t v) { return static_cast<uint32_t>(std::abs(static_cast<int8_t>(v))); }

// Rows [y0, y1) of filter_rows into `out` (rows of 1 + stride bytes).
void filter_band(const uint8_t* img, int w, int c, int y0, int y1, bool adaptive,
                 const uint8_t* zero, uint8_t* out) {
  const size_t stride = static_cast<size_t>(w) * c;
  const size_t bpp = static_cast<size_t>(c);
  std::vector<uint8_t> cand[5];
  for (auto& v : cand) v.resize(stride);
  for (int y = y0; y < y1; ++y) {
    const uint8_t* x = img + static_cast<size_t>(y) * stride;
    const uint8_t* up = y ? x - stride : zero;
    uint8_t* dst = out + static_cast<size_t>(y) * (stride + 1);
    if (!adaptive) {
      dst[0] = 0;
      std::memcpy(dst + 1, x, stride);
      continue;
    }
    uint8_t *o1 = cand[1].data(), *o2 = cand[2].data(), *o3 = cand[3].data(),
            *o4 = cand[4].data();
    uint64_t sum[5] = {0, 0, 0, 0, 0};
    for (size_t i = 0; i < bpp && i < stride; ++i) {  // first pixel: a = c = 0
      o1[i] = x[i];
      o2[i] = static_cast<uint8_t>(x[i] - up[i]);
      o3[i] = static_cast<uint8_t>(x[i] - (up[i] >> 1));
      o4[i] = static_cast<uint8_t>(x[i] - up[i]);  // Paeth(0, b, 0) = b
    }
    for (size_t i = bpp; i < stride; ++i) {
      const int a = x[i - bpp], b = up[i], cc = up[i - bpp];
      o1[i] = static_cast<uint8_t>(x[i] - a);
      o2[i] = static_cast<uint8_t>(x[i] - b);
      o3[i] = static_cast<uint8_t>(x[i] - ((a + b) >> 1));
      o4[i] = static_cast<uint8_t>(x[i] - paeth_pred(a, b, cc));
    }
    for (size_t i = 0; i < stride; ++i) {
      sum[0] += sabs(x[i]);
      sum[1] += sabs(o1[i]);
      sum[2] += sabs(o2[i]);
      sum[3] += sabs(o3[i]);
      sum[4] += sabs(o4[i]);
    }
    int best_f = 0;
    for (int f = 1; f < 5; ++f)
      if (sum[f] < sum[best_f]) best_f = f;
    dst[0] = static_cast<uint8_t>(best_f);
    std::memcpy(dst + 1, best_f ? cand[best_f].data() : x, stride);
  }
}

// Filtered scanlines: per row the filter type (0-4) whose bytes, read as signed, have the
// smallest sum of absolute values, then the filtered bytes. Rows depend only on the image,
// so bands of rows are filtered in parallel.
std::vector<uint8_t> filter_rows(const uint8_t* img, int w, int h, int c, bool adaptive,
                                 int threads) {
  const size_t stride = static_cast<size_t>(w) * c;
  std::vector<uint8_t> out(static_cast<size_t>(h) * (stride + 1));
  const std::vector<uint8_t> zero(stride, 0);
  constexpr int kBand = 32;
  run_parallel(static_cast<size_t>((h + kBand - 1) / kBand), threads, [&](size_t band) {
    const int y0 = static_cast<int>(band) * kBand;
    filter_band(img, w, c, y0, std::min(h, y0 + kBand), adaptive, zero.data(), out.data());
  });
  return out;
}

void put_chunk(std::vector<uint8_t>* png, const char* type, const uint8_t* body, size_t len) {
  uint8_t hdr[8];
  cp::png::put_be32(hdr, static_cast<uint32_t>(len));
  std::memcpy(hdr + 4, type, 4);
  png->insert(png->end(), hdr, hdr + 8);
  if (len) png->insert(png->end(), body, body + len);
  uint32_t crc = cp::png::crc32_update(0, reinterpret_cast<const uint8_t*>(type), 4);
  crc = cp::png::crc32_update(crc, body, len);
  uint8_t tail[4];
  cp::png::put_be32(tail, crc);
  png->insert(png->end(), tail, tail + 4);
}

// The body of cp_save_png (which keeps C++ exceptions from crossing the C ABI).
int save_png(cp_ctx* ctx, const char* path, const uint8_t* image, int32_t width,
             int32_t height, int32_t channels, int32_t level, int32_t threads) {
  if (level < 0) level = 6;
  const std::vector<uint8_t> rows = filter_rows(image, width, height, channels, level > 0,
                                                threads);
  const std::vector<uint8_t> z = zlib_encode(rows.data(), rows.size(), level, threads);
  std::vector<uint8_t> png;
  png.reserve(z.size() + 128);
  static const uint8_t kSig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
  png.insert(png.end(), kSig, kSig + 8);
  uint8_t ihdr[13];
  cp::png::put_be32(ihdr, static_cast<uint32_t>(width));
  cp::png::put_be32(ihdr + 4, static_cast<uint32_t>(height));
  ihdr[8] = 8;                                                       // bit depth
  ihdr[9] = static_cast<uint8_t>(channels == 1 ? 0 : channels == 3 ? 2 : 6);  // colour type
  ihdr[10] = ihdr[11] = ihdr[12] = 0;  // deflate, adaptive filtering, no interlace
  put_chunk(&png, "IHDR", ihdr, 13);
  constexpr size_t kIdat = 1u << 20;
  for (size_t o = 0; o < z.size(); o += kIdat)
    put_chunk(&png, "IDAT", z.data() + o, std::min(kIdat, z.size() - o));
  put_chunk(&png, "IEND", nullptr, 0);
  FILE* f = open_output(path);
  if (!f) {
    cp::ctx_error(ctx, "cannot create %s", path);
    return CP_ERR_IO;
  }
  const bool ok = std::fwrite(png.data(), 1, png.size(), f) == png.size();
  const bool closed = std::fclose(f) == 0;
  if (!ok || !closed) {
    cp::ctx_error(ctx, "cannot write %s", path);
    return CP_ERR_IO;
  }
  return CP_OK;
}

}  // namespace

extern "C" int cp_save_png(cp_ctx* ctx, const char* path, const uint8_t* image, int32_t width,
                           int32_t height, int32_t channels, int32_t level, int32_t threads) {
  if (!path || !image || width < 1 || height < 1 ||
      (channels != 1 && channels != 3 && channels != 4) || level > 9)
    return CP_ERR_ARG;
  try {
    return save_png(ctx, path, image, width, height, channels, level, threads);
  } catch (const std::exception& e) {
    cp::ctx_error(ctx, "cp_save_png: %s", e.what());
    return CP_ERR_OOM;
  }
}
