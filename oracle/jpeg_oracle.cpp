// jpeg_oracle.cpp — TEST INFRASTRUCTURE ONLY: a reference JPEG decoder for the ingest tests.
//
// The product decodes JPEG frames on the GPU with nvJPEG; the reference (image 0.23, which
// decodes with the jpeg-decoder crate, pinned in the reference's Cargo.toml through
// `image = "0.23"`) decodes them on the CPU at src/streams.rs:63-70. Decoders differ in
// their inverse DCT and chroma upsampling, so this checker is the decoding process of
// ISO/IEC 10918-1 (ITU-T T.81) Annex F for sequential Huffman DCT with 8-bit samples
// (SOF0 / SOF1), restated with the EXACT inverse DCT of A.3.3 evaluated in double precision:
// every conforming decoder lies within a small distance of it, and the tests state that
// distance. Components are upsampled by replication (each sample covers Hmax/H x Vmax/V
// pixels) and YCbCr is converted to RGB by the JFIF 1.02 equations. Interleaved and
// single-component scans, restart intervals and both quantisation-table precisions are read;
// progressive and arithmetic-coded files are not (the tests do not produce them).
//
// Nothing here is shared with the product's encoder or decoder.

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

struct HuffTable {
  bool present = false;
  int mincode[17], maxcode[18], valptr[17];
  uint8_t vals[256];
};

struct Component {
  int id = 0, h = 1, v = 1, tq = 0;
  int td = 0, ta = 0;   // table selectors of the current scan
  int bw = 0, bh = 0;   // blocks across / down, covering whole MCUs
  int pred = 0;
  std::vector<int> coef;  // bw * bh blocks of 64 coefficients, natural order
};

struct Decoder {
  const uint8_t* d = nullptr;
  size_t n = 0, p = 0;
  uint16_t qt[4][64];
  HuffTable dc[4], ac[4];
  int width = 0, height = 0, ncomp = 0, hmax = 1, vmax = 1, mcux = 0, mcuy = 0;
  int restart = 0;
  bool have_frame = false;
  Component comp[4];
  int zz[64];  // zigzag index -> natural index
  // entropy-coded data reader
  uint32_t acc = 0;
  int cnt = 0;
};

void make_zigzag(int* zz) {
  // walk the anti-diagonals of the 8x8 block; on even diagonals the column grows
  int k = 0;
  for (int s = 0; s < 15; ++s) {
    if (s % 2 == 0) {
      for (int c = (s < 8 ? 0 : s - 7); c <= (s < 8 ? s : 7); ++c) zz[k++] = (s - c) * 8 + c;
    } else {
      for (int c = (s < 8 ? s : 7); c >= (s < 8 ? 0 : s - 7); --c) zz[k++] = (s - c) * 8 + c;
    }
  }
}

int u16(const uint8_t* q) { return (q[0] << 8) | q[1]; }

// Annex C / F.2.2.3: MINCODE, MAXCODE and VALPTR per code length.
bool build_table(HuffTable* t, const uint8_t* bits, const uint8_t* vals, int nvals) {
  int code = 0, k = 0;
  for (int l = 1; l <= 16; ++l) {
    t->valptr[l] = k;
    t->mincode[l] = code;
    code += bits[l - 1];
    k += bits[l - 1];
    t->maxcode[l] = bits[l - 1] ? code - 1 : -1;
    if (code > (1 << l)) return false;  // over-subscribed
    code <<= 1;
  }
  t->maxcode[17] = 0x7FFFFFFF;
  if (k != nvals || k > 256) return false;
  std::memcpy(t->vals, vals, static_cast<size_t>(k));
  t->present = true;
  return true;
}

// Next bit of the entropy-coded segment; a stuffed 0xFF 0x00 reads as 0xFF, a marker reads
// as zero bits without being consumed.
int next_bit(Decoder* s) {
  if (s->cnt == 0) {
    uint8_t b = 0;
    if (s->p < s->n) {
      if (s->d[s->p] == 0xFF) {
        if (s->p + 1 < s->n && s->d[s->p + 1] == 0x00) {
          b = 0xFF;
          s->p += 2;
        }
      } else {
        b = s->d[s->p++];
      }
    }
    s->acc = b;
    s->cnt = 8;
  }
  --s->cnt;
  return (s->acc >> s->cnt) & 1;
}

int receive(Decoder* s, int nbits) {
  int v = 0;
  for (int i = 0; i < nbits; ++i) v = (v << 1) | next_bit(s);
  return v;
}

int extend(int v, int t) { return t && v < (1 << (t - 1)) ? v - (1 << t) + 1 : v; }

int decode_symbol(Decoder* s, const HuffTable* t) {
  int code = next_bit(s), l = 1;
  while (code > t->maxcode[l]) {
    code = (code << 1) | next_bit(s);
    if (++l > 16) return -1;
  }
  return t->vals[t->valptr[l] + code - t->mincode[l]];
}

bool decode_block(Decoder* s, Component* c, int* blk) {
  const HuffTable* dct = &s->dc[c->td];
  const HuffTable* act = &s->ac[c->ta];
  if (!dct->present || !act->present) return false;
  const int t = decode_symbol(s, dct);
  if (t < 0 || t > 11) return false;
  c->pred += extend(receive(s, t), t);
  blk[0] = c->pred;
  for (int k = 1; k < 64;) {
    const int rs = decode_symbol(s, act);
    if (rs < 0) return false;
    const int r = rs >> 4, sz = rs & 15;
    if (sz == 0) {
      if (r != 15) break;  // EOB
      k += 16;
      continue;
    }
    k += r;
    if (k > 63) return false;
    blk[s->zz[k]] = extend(receive(s, sz), sz);
    ++k;
  }
  return true;
}

// At a restart interval's end: drop the partial byte, step over RSTn, reset predictions.
bool restart_marker(Decoder* s, Component** sc, int ns) {
  s->cnt = 0;
  while (s->p + 1 < s->n && !(s->d[s->p] == 0xFF && s->d[s->p + 1] >= 0xD0 && s->d[s->p + 1] <= 0xD7))
    ++s->p;
  if (s->p + 1 >= s->n) return false;
  s->p += 2;
  for (int i = 0; i < ns; ++i) sc[i]->pred = 0;
  return true;
}

bool decode_scan(Decoder* s, Component** sc, int ns) {
  for (int i = 0; i < ns; ++i) sc[i]->pred = 0;
  s->cnt = 0;
  if (ns == 1) {  // non-interleaved: blocks of the component's own extent, row by row
    Component* c = sc[0];
    const int cw = (s->width * c->h + s->hmax - 1) / s->hmax;
    const int ch = (s->height * c->v + s->vmax - 1) / s->vmax;
    const int bx = (cw + 7) / 8, by = (ch + 7) / 8;
    int done = 0;
    for (int y = 0; y < by; ++y)
      for (int x = 0; x < bx; ++x) {
        if (s->restart && done && done % s->restart == 0 && !restart_marker(s, sc, ns))
          return false;
        if (!decode_block(s, c, &c->coef[(static_cast<size_t>(y) * c->bw + x) * 64])) return false;
        ++done;
      }
    return true;
  }
  const int total = s->mcux * s->mcuy;
  for (int m = 0; m < total; ++m) {
    if (s->restart && m && m % s->restart == 0 && !restart_marker(s, sc, ns)) return false;
    const int mx = m % s->mcux, my = m / s->mcux;
    for (int i = 0; i < ns; ++i) {
      Component* c = sc[i];
      for (int v = 0; v < c->v; ++v)
        for (int h = 0; h < c->h; ++h) {
          const size_t b = static_cast<size_t>(my * c->v + v) * c->bw + mx * c->h + h;
          if (!decode_block(s, c, &c->coef[b * 64])) return false;
        }
    }
  }
  return true;
}

bool parse(Decoder* s) {
  if (s->n < 4 || s->d[0] != 0xFF || s->d[1] != 0xD8) return false;
  s->p = 2;
  for (;;) {
    while (s->p < s->n && s->d[s->p] != 0xFF) ++s->p;
    while (s->p < s->n && s->d[s->p] == 0xFF) ++s->p;
    if (s->p >= s->n) return false;
    const uint8_t m = s->d[s->p++];
    if (m == 0xD9) return s->have_frame;  // EOI
    if (m == 0xD8 || (m >= 0xD0 && m <= 0xD7) || m == 0x01) continue;
    if (s->p + 2 > s->n) return false;
    const int len = u16(s->d + s->p);
    if (len < 2 || s->p + static_cast<size_t>(len) > s->n) return false;
    const uint8_t* q = s->d + s->p + 2;
    const int body = len - 2;
    if (m == 0xDB) {  // DQT
      int o = 0;
      while (o < body) {
        const int pq = q[o] >> 4, tq = q[o] & 15;
        if (tq > 3 || o + 1 + 64 * (pq + 1) > body) return false;
        for (int k = 0; k < 64; ++k)
          s->qt[tq][s->zz[k]] = static_cast<uint16_t>(pq ? u16(q + o + 1 + 2 * k) : q[o + 1 + k]);
        o += 1 + 64 * (pq + 1);
      }
    } else if (m == 0xC4) {  // DHT
      int o = 0;
      while (o < body) {
        if (o + 17 > body) return false;
        const int tc = q[o] >> 4, th = q[o] & 15;
        int nv = 0;
        for (int l = 0; l < 16; ++l) nv += q[o + 1 + l];
        if (tc > 1 || th > 3 || o + 17 + nv > body) return false;
        if (!build_table(tc ? &s->ac[th] : &s->dc[th], q + o + 1, q + o + 17, nv)) return false;
        o += 17 + nv;
      }
    } else if (m == 0xDD) {  // DRI
      if (body < 2) return false;
      s->restart = u16(q);
    } else if (m == 0xC0 || m == 0xC1) {  // SOF: sequential Huffman DCT
      if (body < 6 || q[0] != 8) return false;
      s->height = u16(q + 1);
      s->width = u16(q + 3);
      s->ncomp = q[5];
      if (s->width < 1 || s->height < 1 || (s->ncomp != 1 && s->ncomp != 3) ||
          body < 6 + 3 * s->ncomp)
        return false;
      for (int i = 0; i < s->ncomp; ++i) {
        Component& c = s->comp[i];
        c.id = q[6 + 3 * i];
        c.h = q[7 + 3 * i] >> 4;
        c.v = q[7 + 3 * i] & 15;
        c.tq = q[8 + 3 * i];
        if (c.h < 1 || c.h > 4 || c.v < 1 || c.v > 4 || c.tq > 3) return false;
        if (c.h > s->hmax) s->hmax = c.h;
        if (c.v > s->vmax) s->vmax = c.v;
      }
      s->mcux = (s->width + 8 * s->hmax - 1) / (8 * s->hmax);
      s->mcuy = (s->height + 8 * s->vmax - 1) / (8 * s->vmax);
      for (int i = 0; i < s->ncomp; ++i) {
        Component& c = s->comp[i];
        c.bw = s->mcux * c.h;
        c.bh = s->mcuy * c.v;
        c.coef.assign(static_cast<size_t>(c.bw) * c.bh * 64, 0);
      }
      s->have_frame = true;
    } else if (m >= 0xC2 && m <= 0xCF && m != 0xC4 && m != 0xC8 && m != 0xCC) {
      return false;  // progressive, lossless, hierarchical or arithmetic: not read here
    } else if (m == 0xDA) {  // SOS
      if (!s->have_frame || body < 1) return false;
      const int ns = q[0];
      if (ns < 1 || ns > s->ncomp || body < 4 + 2 * ns) return false;
      Component* sc[4];
      for (int i = 0; i < ns; ++i) {
        sc[i] = nullptr;
        for (int j = 0; j < s->ncomp; ++j)
          if (s->comp[j].id == q[1 + 2 * i]) sc[i] = &s->comp[j];
        if (!sc[i]) return false;
        sc[i]->td = q[2 + 2 * i] >> 4;
        sc[i]->ta = q[2 + 2 * i] & 15;
        if (sc[i]->td > 3 || sc[i]->ta > 3) return false;
      }
      if (q[1 + 2 * ns] != 0 || q[2 + 2 * ns] != 63) return false;
      s->p += static_cast<size_t>(len);
      if (!decode_scan(s, sc, ns)) return false;
      continue;
    }
    s->p += static_cast<size_t>(len);
  }
}

// Exact inverse DCT (A.3.3) of dequantised coefficients, level shift, round, clamp.
void idct_block(const int* coef, const uint16_t* q, uint8_t* out, int stride) {
  static double basis[8][8];  // basis[x][u] = C(u)/2 cos((2x+1) u pi / 16)
  static bool init = false;
  if (!init) {
    for (int x = 0; x < 8; ++x)
      for (int u = 0; u < 8; ++u)
        basis[x][u] = (u ? 1.0 : std::sqrt(0.5)) * 0.5 * std::cos((2 * x + 1) * u * M_PI / 16.0);
    init = true;
  }
  double F[64], t[64];
  for (int i = 0; i < 64; ++i) F[i] = static_cast<double>(coef[i]) * q[i];
  for (int v = 0; v < 8; ++v)  // rows: t[v][x] = sum_u basis[x][u] F[v][u]
    for (int x = 0; x < 8; ++x) {
      double a = 0.0;
      for (int u = 0; u < 8; ++u) a += basis[x][u] * F[v * 8 + u];
      t[v * 8 + x] = a;
    }
  for (int y = 0; y < 8; ++y)
    for (int x = 0; x < 8; ++x) {
      double a = 0.0;
      for (int v = 0; v < 8; ++v) a += basis[y][v] * t[v * 8 + x];
      const double r = std::floor(a + 128.0 + 0.5);
      out[y * stride + x] = static_cast<uint8_t>(r < 0 ? 0 : r > 255 ? 255 : r);
    }
}

uint8_t clamp_round(double v) {
  const double r = std::floor(v + 0.5);
  return static_cast<uint8_t>(r < 0 ? 0 : r > 255 ? 255 : r);
}

}  // namespace

extern "C" {

// Width, height and components of a sequential JPEG: 0, or -1 for a file it does not read.
int or_jpeg_info(const uint8_t* data, size_t len, int32_t* w, int32_t* h, int32_t* c) {
  Decoder* s = new Decoder;
  make_zigzag(s->zz);
  s->d = data;
  s->n = len;
  const bool ok = parse(s);
  if (ok) {
    *w = s->width;
    *h = s->height;
    *c = s->ncomp;
  }
  delete s;
  return ok ? 0 : -1;
}

// Decodes into out (h x w x c bytes, c = 1 or 3): 0, or -1.
int or_jpeg_decode(const uint8_t* data, size_t len, uint8_t* out, size_t cap) {
  Decoder* s = new Decoder;
  make_zigzag(s->zz);
  s->d = data;
  s->n = len;
  int rc = -1;
  if (parse(s) && cap >= static_cast<size_t>(s->width) * s->height * s->ncomp) {
    std::vector<std::vector<uint8_t>> planes(static_cast<size_t>(s->ncomp));
    for (int i = 0; i < s->ncomp; ++i) {
      Component& c = s->comp[i];
      const int pw = c.bw * 8;
      planes[i].assign(static_cast<size_t>(pw) * c.bh * 8, 0);
      for (int by = 0; by < c.bh; ++by)
        for (int bx = 0; bx < c.bw; ++bx)
          idct_block(&c.coef[(static_cast<size_t>(by) * c.bw + bx) * 64], s->qt[c.tq],
                     &planes[i][static_cast<size_t>(by) * 8 * pw + bx * 8], pw);
    }
    for (int y = 0; y < s->height; ++y)
      for (int x = 0; x < s->width; ++x) {
        double v[3];
        for (int i = 0; i < s->ncomp; ++i) {
          const Component& c = s->comp[i];
          const int sx = x * c.h / s->hmax, sy = y * c.v / s->vmax;
          v[i] = planes[i][static_cast<size_t>(sy) * c.bw * 8 + sx];
        }
        uint8_t* o = out + (static_cast<size_t>(y) * s->width + x) * s->ncomp;
        if (s->ncomp == 1) {
          o[0] = static_cast<uint8_t>(v[0]);
        } else {
          const double Y = v[0], cb = v[1] - 128.0, cr = v[2] - 128.0;
          o[0] = clamp_round(Y + 1.402 * cr);
          o[1] = clamp_round(Y - 0.344136 * cb - 0.714136 * cr);
          o[2] = clamp_round(Y + 1.772 * cb);
        }
      }
    rc = 0;
  }
  delete s;
  return rc;
}

}  // extern "C"
