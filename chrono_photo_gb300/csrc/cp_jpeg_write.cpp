// cp_jpeg_write.cpp — output encode: composites and blend masks written as baseline JPEG.
//
// The reference writes .jpg outputs (and its example frames) with image 0.23's JPEGEncoder
// at a quality in percent, 95 by default (src/main.rs:542-556, src/cli.rs:82-84,
// src/util/create_example_data.rs:56): baseline sequential DCT, 8-bit samples, YCbCr with
// every component sampled 1x1, the alpha channel of RGBA input dropped. This encoder makes
// the same format choices, restated from ISO/IEC 10918-1 (ITU-T T.81) and JFIF 1.02:
//   - RGB -> YCbCr by the JFIF equations, level shift by 128;
//   - forward DCT by its definition (T.81 A.3.3), computed separably in f32;
//   - quantisation by the Annex K.1 example tables scaled by quality as in the IJG library
//     (scale 5000/q below 50, else 200 - 2q, in percent, each entry clamped to 1..255);
//   - Huffman tables built for the image (Annex K.2 code sizes, K.3 limit to 16 bits,
//     canonical codes of Annex C), which the standard allows and every decoder reads;
//   - a restart interval of one MCU row (DRI / RSTn), so that the rows are coded
//     independently on host threads; the bytes do not depend on the number of threads.
// Chroma 4:2:0 (2x2 averaging) is available for files like a camera's; the reference's
// encoder has no such option. The output bytes are not those of image's encoder (its
// Huffman tables and rounding differ); a decoder reconstructs the same image either way, up
// to the quantisation error both share.

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/chrono_gpu.h"
#include "cp_host_internal.h"
#include "cp_io.h"

namespace {

// Annex K.1 example quantisation tables, row-major (natural) order.
const uint8_t kLumaQ[64] = {16, 11, 10, 16, 24,  40,  51,  61,  12, 12, 14, 19, 26,  58,  60,  55,
                            14, 13, 16, 24, 40,  57,  69,  56,  14, 17, 22, 29, 51,  87,  80,  62,
                            18, 22, 37, 56, 68,  109, 103, 77,  24, 35, 55, 64, 81,  104, 113, 92,
                            49, 64, 78, 87, 103, 121, 120, 101, 72, 92, 95, 98, 112, 100, 103, 99};
const uint8_t kChromaQ[64] = {17, 18, 24, 47, 99, 99, 99, 99, 18, 21, 26, 66, 99, 99, 99, 99,
                              24, 26, 56, 99, 99, 99, 99, 99, 47, 66, 99, 99, 99, 99, 99, 99,
                              99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99,
                              99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99};

// zigzag index k -> natural index (row * 8 + col): the anti-diagonals d = row + col in
// turn, even ones walked upwards (row falling), odd ones downwards.
struct Zigzag {
  int nat[64];
  Zigzag() {
    int k = 0;
    for (int d = 0; d < 15; ++d) {
      const int lo = std::max(0, d - 7), hi = std::min(d, 7);
      if (d % 2 == 0)
        for (int r = hi; r >= lo; --r) nat[k++] = r * 8 + (d - r);
      else
        for (int r = lo; r <= hi; ++r) nat[k++] = r * 8 + (d - r);
    }
  }
};
const Zigzag kZz;

// cs[u][x] = C(u)/2 cos((2x+1) u pi / 16), C(0) = 1/sqrt(2), else 1: F = cs f cs^T is the
// two-dimensional DCT of A.3.3.
struct DctBasis {
  float cs[8][8];
  DctBasis() {
    const double pi = 3.14159265358979323846;
    for (int u = 0; u < 8; ++u)
      for (int x = 0; x < 8; ++x)
        cs[u][x] = static_cast<float>((u == 0 ? std::sqrt(0.5) : 1.0) * 0.5 *
                                      std::cos((2 * x + 1) * u * pi / 16.0));
  }
};
const DctBasis kDct;

// Quantised coefficients (zigzag order) of one 8x8 block of level-shifted samples.
void fdct_quantise(const float blk[64], const uint16_t q[64], int16_t out[64]) {
  float tmp[64], F[64];
  for (int y = 0; y < 8; ++y)
    for (int u = 0; u < 8; ++u) {
      float s = 0.0f;
      for (int x = 0; x < 8; ++x) s += kDct.cs[u][x] * blk[y * 8 + x];
      tmp[y * 8 + u] = s;
    }
  for (int v = 0; v < 8; ++v)
    for (int u = 0; u < 8; ++u) {
      float s = 0.0f;
      for (int y = 0; y < 8; ++y) s += kDct.cs[v][y] * tmp[y * 8 + u];
      F[v * 8 + u] = s;
    }
  for (int k = 0; k < 64; ++k) {
    const int n = kZz.nat[k];
    const float r = F[n] / static_cast<float>(q[n]);
    // round half away from zero; |r| <= 2048 / 1 for 8-bit samples
    out[k] = static_cast<int16_t>(r >= 0.0f ? std::floor(r + 0.5f) : -std::floor(-r + 0.5f));
  }
}

int bit_length(int v) {  // magnitude category (T.81 F.1.2.1): bits of |v|
  unsigned a = static_cast<unsigned>(v < 0 ? -v : v);
  int s = 0;
  while (a) {
    ++s;
    a >>= 1;
  }
  return s;
}

// One Huffman table: BITS / HUFFVAL for the DHT segment and the code of each symbol.
struct Huff {
  uint8_t bits[17] = {0};
  std::vector<uint8_t> vals;
  uint16_t code[256] = {0};
  uint8_t size[256] = {0};
};

// Annex K.2 (code sizes from symbol frequencies, with a reserved symbol 256 of frequency 1
// so that no real symbol gets the all-ones code), K.3 (lengths limited to 16 bits) and
// Annex C (canonical codes in the order of HUFFVAL).
Huff build_huff(const std::vector<uint64_t>& counts) {
  std::vector<uint64_t> freq(257, 0);
  for (int i = 0; i < 256; ++i) freq[i] = counts[static_cast<size_t>(i)];
  freq[256] = 1;
  std::vector<int> codesize(257, 0), others(257, -1);
  for (;;) {
    // the two least frequent live entries; among equal ones the highest index, so that the
    // reserved symbol gets a longest code
    int c1 = -1, c2 = -1;
    for (int i = 0; i <= 256; ++i)
      if (freq[i] && (c1 < 0 || freq[i] <= freq[c1])) c1 = i;
    for (int i = 0; i <= 256; ++i)
      if (freq[i] && i != c1 && (c2 < 0 || freq[i] <= freq[c2])) c2 = i;
    if (c2 < 0) break;
    freq[c1] += freq[c2];
    freq[c2] = 0;
    for (int i = c1;; i = others[i]) {
      ++codesize[i];
      if (others[i] < 0) {
        others[i] = c2;
        break;
      }
    }
    for (int i = c2; i >= 0; i = others[i]) ++codesize[i];
  }
  std::vector<int> nbits(300, 0);
  int maxlen = 0;
  for (int i = 0; i <= 256; ++i)
    if (codesize[i]) {
      ++nbits[static_cast<size_t>(codesize[i])];
      maxlen = std::max(maxlen, codesize[i]);
    }
  // K.3: a pair of codes at the longest length i gives way to one code at i - 1 and two
  // below the next shorter length j that has codes
  for (int i = maxlen; i > 16; --i) {
    while (nbits[static_cast<size_t>(i)] > 0) {
      int j = i - 2;
      while (nbits[static_cast<size_t>(j)] == 0) --j;
      nbits[static_cast<size_t>(i)] -= 2;
      nbits[static_cast<size_t>(i - 1)] += 1;
      nbits[static_cast<size_t>(j + 1)] += 2;
      nbits[static_cast<size_t>(j)] -= 1;
    }
  }
  int top = 16;
  while (nbits[static_cast<size_t>(top)] == 0) --top;
  nbits[static_cast<size_t>(top)] -= 1;  // the reserved symbol's code
  Huff h;
  for (int l = 1; l <= 16; ++l) h.bits[l] = static_cast<uint8_t>(nbits[static_cast<size_t>(l)]);
  // K.4: symbols in the order of their K.2 code size, then of value (256 comes last)
  std::vector<int> order;
  for (int l = 1; l < 300; ++l)
    for (int i = 0; i < 256; ++i)
      if (codesize[i] == l) order.push_back(i);
  int total = 0;
  for (int l = 1; l <= 16; ++l) total += h.bits[l];
  order.resize(static_cast<size_t>(total));
  h.vals.assign(order.begin(), order.end());
  // Annex C: canonical codes
  uint32_t code = 0;
  size_t k = 0;
  for (int l = 1; l <= 16; ++l) {
    for (int c = 0; c < h.bits[l]; ++c, ++k) {
      h.code[h.vals[k]] = static_cast<uint16_t>(code);
      h.size[h.vals[k]] = static_cast<uint8_t>(l);
      ++code;
    }
    code <<= 1;
  }
  return h;
}

// Entropy-coded bytes with 0xFF stuffing (T.81 F.1.2.3); flush() pads with 1-bits.
struct BitWriter {
  std::vector<uint8_t>* out;
  uint64_t acc = 0;
  int n = 0;
  void put(uint32_t bits, int len) {
    acc = (acc << len) | (bits & ((1u << len) - 1u));
    n += len;
    while (n >= 8) {
      const uint8_t b = static_cast<uint8_t>(acc >> (n - 8));
      out->push_back(b);
      if (b == 0xFF) out->push_back(0x00);
      n -= 8;
    }
  }
  void flush() {
    if (n > 0) put((1u << (8 - n)) - 1u, 8 - n);
  }
};

struct Layout {
  int comps = 3;              // 1 gray, 3 YCbCr
  int hs = 1, vs = 1;         // luma blocks per MCU across / down (4:2:0: 2 x 2)
  int mcu_w = 8, mcu_h = 8;   // MCU size in pixels
  int mcus_x = 0, mcus_y = 0;
  int blocks = 1;             // blocks per MCU
};

// Quantised blocks of MCU row `r` in MCU order (luma blocks left to right, top to bottom,
// then Cb, then Cr).
void transform_row(const uint8_t* img, int w, int h, int ch, const Layout& L,
                   const uint16_t q[2][64], int r, int16_t* out) {
  const int y0 = r * L.mcu_h;
  // level-shifted planes of this MCU row, edges replicated to the MCU grid
  const int pw = L.mcus_x * L.mcu_w;
  std::vector<float> Y(static_cast<size_t>(pw) * L.mcu_h), Cb, Cr;
  if (L.comps == 3) {
    Cb.resize(Y.size());
    Cr.resize(Y.size());
  }
  for (int yy = 0; yy < L.mcu_h; ++yy) {
    const int sy = std::min(y0 + yy, h - 1);
    const uint8_t* row = img + static_cast<size_t>(sy) * w * ch;
    for (int xx = 0; xx < pw; ++xx) {
      const uint8_t* p = row + static_cast<size_t>(std::min(xx, w - 1)) * ch;
      const size_t o = static_cast<size_t>(yy) * pw + xx;
      if (L.comps == 1) {
        Y[o] = static_cast<float>(p[0]) - 128.0f;
      } else {
        const float R = p[0], G = p[1], B = p[2];
        Y[o] = 0.299f * R + 0.587f * G + 0.114f * B - 128.0f;
        Cb[o] = -0.168736f * R - 0.331264f * G + 0.5f * B;
        Cr[o] = 0.5f * R - 0.418688f * G - 0.081312f * B;
      }
    }
  }
  float blk[64];
  int16_t* o = out;
  for (int mx = 0; mx < L.mcus_x; ++mx) {
    for (int by = 0; by < L.vs; ++by)
      for (int bx = 0; bx < L.hs; ++bx) {
        for (int y = 0; y < 8; ++y)
          for (int x = 0; x < 8; ++x)
            blk[y * 8 + x] = Y[static_cast<size_t>(by * 8 + y) * pw + mx * L.mcu_w + bx * 8 + x];
        fdct_quantise(blk, q[0], o);
        o += 64;
      }
    if (L.comps == 3) {
      for (const std::vector<float>* P : {&Cb, &Cr}) {
        for (int y = 0; y < 8; ++y)
          for (int x = 0; x < 8; ++x) {
            // the mean of the hs x vs samples a chroma sample covers
            float s = 0.0f;
            for (int dy = 0; dy < L.vs; ++dy)
              for (int dx = 0; dx < L.hs; ++dx)
                s += (*P)[static_cast<size_t>(y * L.vs + dy) * pw + mx * L.mcu_w + x * L.hs + dx];
            blk[y * 8 + x] = s / static_cast<float>(L.hs * L.vs);
          }
        fdct_quantise(blk, q[1], o);
        o += 64;
      }
    }
  }
}

// Table of block b of an MCU: 0 luma, 1 chroma.
inline int block_table(const Layout& L, int b) { return b < L.hs * L.vs ? 0 : 1; }

// Symbol statistics (count = true) or entropy-coded bytes of one MCU row; DC predictions
// start at 0 in every row (each row is one restart interval).
template <bool kCount>
void code_row(const int16_t* blocks, const Layout& L, std::vector<uint64_t>* counts,
              const Huff* huff, BitWriter* bw) {
  int pred[3] = {0, 0, 0};
  const int16_t* c = blocks;
  for (int m = 0; m < L.mcus_x; ++m)
    for (int b = 0; b < L.blocks; ++b, c += 64) {
      const int t = block_table(L, b);
      const int comp = t == 0 ? 0 : b - L.hs * L.vs + 1;
      const int diff = c[0] - pred[comp];
      pred[comp] = c[0];
      const int s = bit_length(diff);
      if (kCount) {
        ++counts[2 * t][static_cast<size_t>(s)];
      } else {
        const Huff& hd = huff[2 * t];
        bw->put(hd.code[s], hd.size[s]);
        if (s) bw->put(static_cast<uint32_t>(diff < 0 ? diff - 1 : diff), s);
      }
      int run = 0;
      for (int k = 1; k < 64; ++k) {
        const int v = c[k];
        if (v == 0) {
          ++run;
          continue;
        }
        while (run > 15) {
          if (kCount) ++counts[2 * t + 1][0xF0];
          else bw->put(huff[2 * t + 1].code[0xF0], huff[2 * t + 1].size[0xF0]);
          run -= 16;
        }
        const int sv = bit_length(v);
        const int sym = (run << 4) | sv;
        if (kCount) {
          ++counts[2 * t + 1][static_cast<size_t>(sym)];
        } else {
          const Huff& ha = huff[2 * t + 1];
          bw->put(ha.code[sym], ha.size[sym]);
          bw->put(static_cast<uint32_t>(v < 0 ? v - 1 : v), sv);
        }
        run = 0;
      }
      if (run > 0) {
        if (kCount) ++counts[2 * t + 1][0];
        else bw->put(huff[2 * t + 1].code[0], huff[2 * t + 1].size[0]);
      }
    }
}

void put16(std::vector<uint8_t>* o, int v) {
  o->push_back(static_cast<uint8_t>(v >> 8));
  o->push_back(static_cast<uint8_t>(v));
}
void marker(std::vector<uint8_t>* o, uint8_t m, int len) {  // len counts itself
  o->push_back(0xFF);
  o->push_back(m);
  put16(o, len);
}

}  // namespace

namespace cp {

// The JPEG file of an image (channels 1, 3 or 4; quality 1..100; subsampling 0 = 4:4:4,
// 1 = 4:2:0).
std::vector<uint8_t> encode_jpeg(const uint8_t* img, int w, int h, int ch, int quality,
                                 int subsampling, int threads) {
  Layout L;
  L.comps = ch == 1 ? 1 : 3;
  L.hs = L.vs = (L.comps == 3 && subsampling == 1) ? 2 : 1;
  L.mcu_w = 8 * L.hs;
  L.mcu_h = 8 * L.vs;
  L.mcus_x = (w + L.mcu_w - 1) / L.mcu_w;
  L.mcus_y = (h + L.mcu_h - 1) / L.mcu_h;
  L.blocks = L.hs * L.vs + (L.comps == 3 ? 2 : 0);
  const int scale = quality < 50 ? 5000 / quality : 200 - 2 * quality;
  uint16_t q[2][64];
  for (int i = 0; i < 64; ++i) {
    q[0][i] = static_cast<uint16_t>(std::min(255, std::max(1, (kLumaQ[i] * scale + 50) / 100)));
    q[1][i] = static_cast<uint16_t>(std::min(255, std::max(1, (kChromaQ[i] * scale + 50) / 100)));
  }
  const size_t row_coefs = static_cast<size_t>(L.mcus_x) * L.blocks * 64;
  std::vector<int16_t> coefs(row_coefs * static_cast<size_t>(L.mcus_y));
  const int ntab = L.comps == 3 ? 4 : 2;  // DC/AC luma, DC/AC chroma
  std::vector<std::vector<uint64_t>> row_counts(static_cast<size_t>(L.mcus_y) * ntab,
                                                std::vector<uint64_t>(256, 0));
  run_parallel(static_cast<size_t>(L.mcus_y), threads, [&](size_t r) {
    int16_t* rc = coefs.data() + row_coefs * r;
    transform_row(img, w, h, ch, L, q, static_cast<int>(r), rc);
    code_row<true>(rc, L, &row_counts[r * ntab], nullptr, nullptr);
  });
  std::vector<uint64_t> counts[4];
  for (int t = 0; t < ntab; ++t) {
    counts[t].assign(256, 0);
    for (int r = 0; r < L.mcus_y; ++r)
      for (int s = 0; s < 256; ++s)
        counts[t][static_cast<size_t>(s)] += row_counts[static_cast<size_t>(r) * ntab + t][static_cast<size_t>(s)];
  }
  Huff huff[4];
  for (int t = 0; t < ntab; ++t) huff[t] = build_huff(counts[t]);
  std::vector<std::vector<uint8_t>> rows(static_cast<size_t>(L.mcus_y));
  run_parallel(static_cast<size_t>(L.mcus_y), threads, [&](size_t r) {
    rows[r].reserve(row_coefs / 4);
    BitWriter bw{&rows[r]};
    code_row<false>(coefs.data() + row_coefs * r, L, nullptr, huff, &bw);
    bw.flush();
  });
  std::vector<uint8_t> o;
  size_t body = 0;
  for (const auto& r : rows) body += r.size() + 2;
  o.reserve(body + 1024);
  o.push_back(0xFF);
  o.push_back(0xD8);  // SOI
  // APP0 JFIF 1.01, no density, no thumbnail
  marker(&o, 0xE0, 16);
  const uint8_t jfif[14] = {'J', 'F', 'I', 'F', 0, 1, 1, 0, 0, 1, 0, 1, 0, 0};
  o.insert(o.end(), jfif, jfif + 14);
  for (int t = 0; t < (L.comps == 3 ? 2 : 1); ++t) {  // DQT, 8-bit entries in zigzag order
    marker(&o, 0xDB, 67);
    o.push_back(static_cast<uint8_t>(t));
    for (int k = 0; k < 64; ++k) o.push_back(static_cast<uint8_t>(q[t][kZz.nat[k]]));
  }
  marker(&o, 0xC0, 8 + 3 * L.comps);  // SOF0
  o.push_back(8);
  put16(&o, h);
  put16(&o, w);
  o.push_back(static_cast<uint8_t>(L.comps));
  for (int c = 0; c < L.comps; ++c) {
    o.push_back(static_cast<uint8_t>(c + 1));
    o.push_back(static_cast<uint8_t>(c == 0 ? (L.hs << 4) | L.vs : 0x11));
    o.push_back(static_cast<uint8_t>(c == 0 ? 0 : 1));
  }
  for (int t = 0; t < ntab; ++t) {  // DHT: class 0 DC / 1 AC, destination 0 luma / 1 chroma
    const Huff& hf = huff[t];
    marker(&o, 0xC4, 2 + 1 + 16 + static_cast<int>(hf.vals.size()));
    o.push_back(static_cast<uint8_t>(((t & 1) << 4) | (t >> 1)));
    o.insert(o.end(), hf.bits + 1, hf.bits + 17);
    o.insert(o.end(), hf.vals.begin(), hf.vals.end());
  }
  if (L.mcus_y > 1) {  // DRI: one MCU row per restart interval
    marker(&o, 0xDD, 4);
    put16(&o, L.mcus_x);
  }
  marker(&o, 0xDA, 6 + 2 * L.comps);  // SOS
  o.push_back(static_cast<uint8_t>(L.comps));
  for (int c = 0; c < L.comps; ++c) {
    o.push_back(static_cast<uint8_t>(c + 1));
    o.push_back(static_cast<uint8_t>(c == 0 ? 0x00 : 0x11));
  }
  o.push_back(0);
  o.push_back(63);
  o.push_back(0);
  for (int r = 0; r < L.mcus_y; ++r) {
    o.insert(o.end(), rows[static_cast<size_t>(r)].begin(), rows[static_cast<size_t>(r)].end());
    if (r + 1 < L.mcus_y) {
      o.push_back(0xFF);
      o.push_back(static_cast<uint8_t>(0xD0 + (r & 7)));  // RSTn
    }
  }
  o.push_back(0xFF);
  o.push_back(0xD9);  // EOI
  return o;
}

}  // namespace cp

extern "C" int cp_encode_jpeg(cp_ctx* ctx, const uint8_t* image, int32_t width, int32_t height,
                              int32_t channels, int32_t quality, int32_t subsampling,
                              int32_t threads, uint8_t* out, uint64_t capacity, uint64_t* size) {
  if (!image || !size || width < 1 || height < 1 || width > 65535 || height > 65535 ||
      (channels != 1 && channels != 3 && channels != 4) || quality > 100 ||
      (subsampling != 0 && subsampling != 1) || (capacity && !out))
    return CP_ERR_ARG;
  try {
    const std::vector<uint8_t> j = cp::encode_jpeg(image, width, height, channels,
                                                   quality < 1 ? 95 : quality, subsampling,
                                                   threads);
    *size = j.size();
    if (j.size() > capacity) {
      cp::ctx_error(ctx, "cp_encode_jpeg: %zu bytes do not fit in %llu", j.size(),
                    static_cast<unsigned long long>(capacity));
      return CP_ERR_LIMIT;
    }
    std::memcpy(out, j.data(), j.size());
    return CP_OK;
  } catch (const std::exception& e) {
    cp::ctx_error(ctx, "cp_encode_jpeg: %s", e.what());
    return CP_ERR_OOM;
  }
}

extern "C" int cp_save_jpeg(cp_ctx* ctx, const char* path, const uint8_t* image, int32_t width,
                            int32_t height, int32_t channels, int32_t quality,
                            int32_t subsampling, int32_t threads) {
  if (!path || !image || width < 1 || height < 1 || width > 65535 || height > 65535 ||
      (channels != 1 && channels != 3 && channels != 4) || quality > 100 ||
      (subsampling != 0 && subsampling != 1))
    return CP_ERR_ARG;
  try {
    const std::vector<uint8_t> j = cp::encode_jpeg(image, width, height, channels,
                                                   quality < 1 ? 95 : quality, subsampling,
                                                   threads);
    FILE* f = cp::open_output(path);
    if (!f) {
      cp::ctx_error(ctx, "cannot create %s", path);
      return CP_ERR_IO;
    }
    const bool ok = std::fwrite(j.data(), 1, j.size(), f) == j.size();
    const bool closed = std::fclose(f) == 0;
    if (!ok || !closed) {
      cp::ctx_error(ctx, "cannot write %s", path);
      return CP_ERR_IO;
    }
    return CP_OK;
  } catch (const std::exception& e) {
    cp::ctx_error(ctx, "cp_save_jpeg: %s", e.what());
    return CP_ERR_OOM;
  }
}
