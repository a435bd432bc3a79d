// ingest.cpp -- host-side readers of the reference's input formats (plain
// C++, no CUDA, no third-party library):
//
//  * Wavefront OBJ text, turned into the loadOBJ3 face-major SoA layout
//    (main.h:620-679, which reads it through assimp's aiImportFile);
//  * the ACCV binary depth format of loadDepth (main.cu:35-64): int32 rows,
//    int32 cols, then rows*cols uint16 depths in mm, row-major, host byte
//    order;
//  * 16-bit (or 8-bit) greyscale PNG, the "640x480 png images" the
//    reference's usage text names (README.md), decoded with this file's own
//    inflate (RFC 1950/1951) and scanline unfiltering (PNG specification,
//    section 9).
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cctype>
#include <cstring>
#include <string>
#include <vector>

#include "qpso.h"

namespace {

bool read_file(const char* path, std::vector<unsigned char>& out) {
  FILE* fp = std::fopen(path, "rb");
  if (!fp) return false;
  unsigned char buf[1 << 16];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof(buf), fp)) > 0) out.insert(out.end(), buf, buf + n);
  const bool ok = !std::ferror(fp);
  std::fclose(fp);
  return ok;
}

// ---------------------------------------------------------------- OBJ ----
// Vertices are `v x y z [w]` lines; faces are `f` lines whose corners are
// `i`, `i/t`, `i//n` or `i/t/n` with 1-based or negative (relative) vertex
// indices.  A polygon of n > 3 corners becomes the fan (0, k, k+1).  Every
// other statement (normals, texture coordinates, groups, materials, lines,
// comments) is ignored.
bool parse_index(const char*& p, long nverts, long* out) {
  char* end = nullptr;
  errno = 0;
  const long v = std::strtol(p, &end, 10);
  if (end == p || errno) return false;
  p = end;
  while (*p == '/' || (*p >= '0' && *p <= '9') || *p == '-') ++p;  // skip /t/n
  long idx = v > 0 ? v - 1 : nverts + v;
  if (v == 0 || idx < 0 || idx >= nverts) return false;
  *out = idx;
  return true;
}

qpso_status load_obj(const char* path, std::vector<float>& xyz, std::vector<uint32_t>& tri) {
  std::vector<unsigned char> raw;
  if (!read_file(path, raw)) return QPSO_ERR_NOT_FOUND;
  raw.push_back('\n');
  raw.push_back('\0');
  const char* p = reinterpret_cast<const char*>(raw.data());
  const char* end = p + raw.size() - 1;
  std::vector<long> poly;
  while (p < end) {
    const char* eol = static_cast<const char*>(std::memchr(p, '\n', (size_t)(end - p)));
    if (!eol) eol = end;
    while (p < eol && (*p == ' ' || *p == '\t')) ++p;
    if (p + 1 < eol && p[0] == 'v' && (p[1] == ' ' || p[1] == '\t')) {
      p += 2;
      for (int c = 0; c < 3; ++c) {
        char* e = nullptr;
        const float f = std::strtof(p, &e);
        if (e == p || !std::isfinite(f)) return QPSO_ERR_ARG;
        xyz.push_back(f);
        p = e;
      }
    } else if (p + 1 < eol && p[0] == 'f' && (p[1] == ' ' || p[1] == '\t')) {
      p += 2;
      poly.clear();
      const long nv = (long)(xyz.size() / 3);
      for (;;) {
        while (p < eol && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
        if (p >= eol) break;
        long idx;
        if (!parse_index(p, nv, &idx)) return QPSO_ERR_ARG;
        poly.push_back(idx);
      }
      if (poly.size() < 3) return QPSO_ERR_ARG;
      for (size_t k = 1; k + 1 < poly.size(); ++k) {
        tri.push_back((uint32_t)poly[0]);
        tri.push_back((uint32_t)poly[k]);
        tri.push_back((uint32_t)poly[k + 1]);
      }
    }
    p = eol + 1;
  }
  return tri.empty() ? QPSO_ERR_ARG : QPSO_OK;
}

// ------------------------------------------------------------ inflate ----
struct BitReader {
  const unsigned char* p;
  size_t n, pos = 0;  // pos in bits
  bool bad = false;
  uint32_t bits(int k) {  // LSB-first
    uint32_t v = 0;
    for (int i = 0; i < k; ++i) {
      const size_t byte = pos >> 3;
      if (byte >= n) {
        bad = true;
        return 0;
      }
      v |= (uint32_t)((p[byte] >> (pos & 7)) & 1u) << i;
      ++pos;
    }
    return v;
  }
};

// Canonical Huffman code from code lengths (RFC 1951 section 3.2.2).
struct Huffman {
  uint16_t count[16] = {0};
  std::vector<uint16_t> symbol;
  bool build(const uint8_t* len, int n) {
    std::memset(count, 0, sizeof(count));
    for (int i = 0; i < n; ++i) count[len[i]]++;
    count[0] = 0;
    int left = 1;
    for (int l = 1; l < 16; ++l) {
      left <<= 1;
      left -= count[l];
      if (left < 0) return false;  // over-subscribed
    }
    uint16_t offs[16];
    offs[1] = 0;
    for (int l = 1; l < 15; ++l) offs[l + 1] = (uint16_t)(offs[l] + count[l]);
    symbol.assign((size_t)n, 0);
    for (int i = 0; i < n; ++i)
      if (len[i]) symbol[offs[len[i]]++] = (uint16_t)i;
    return true;
  }
  int decode(BitReader& br) const {
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; ++l) {
      code |= (int)br.bits(1);
      if (br.bad) return -1;
      const int c = count[l];
      if (code - c < first) return symbol[(size_t)(index + (code - first))];
      index += c;
      first += c;
      first <<= 1;
      code <<= 1;
    }
    return -1;
  }
};

const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_codes(BitReader& br, const Huffman& lit, const Huffman& dist, std::vector<unsigned char>& out,
                   size_t limit) {
  for (;;) {
    const int sym = lit.decode(br);
    if (sym < 0) return false;
    if (sym < 256) {
      if (out.size() >= limit) return false;
      out.push_back((unsigned char)sym);
    } else if (sym == 256) {
      return true;
    } else {
      const int li = sym - 257;
      if (li >= 29) return false;
      const size_t len = kLenBase[li] + br.bits(kLenExtra[li]);
      const int ds = dist.decode(br);
      if (ds < 0 || ds >= 30 || br.bad) return false;
      const size_t d = kDistBase[ds] + br.bits(kDistExtra[ds]);
      if (br.bad || d > out.size() || out.size() + len > limit) return false;
      const size_t from = out.size() - d;
      for (size_t i = 0; i < len; ++i) out.push_back(out[from + i]);
    }
  }
}

// zlib stream (RFC 1950) holding a deflate stream (RFC 1951); `limit`
// bounds the output size.
bool zlib_inflate(const unsigned char* in, size_t n, std::vector<unsigned char>& out, size_t limit) {
  if (n < 6) return false;
  const unsigned cmf = in[0], flg = in[1];
  if ((cmf & 15) != 8 || ((cmf << 8) | flg) % 31 != 0 || (flg & 0x20)) return false;
  BitReader br{in + 2, n - 6};
  int final = 0;
  while (!final) {
    final = (int)br.bits(1);
    const uint32_t type = br.bits(2);
    if (br.bad) return false;
    if (type == 0) {
      br.pos = (br.pos + 7) & ~(size_t)7;
      const size_t byte = br.pos >> 3;
      if (byte + 4 > br.n) return false;
      const uint32_t len = br.p[byte] | (br.p[byte + 1] << 8);
      const uint32_t nlen = br.p[byte + 2] | (br.p[byte + 3] << 8);
      if ((len ^ 0xffffu) != nlen || byte + 4 + len > br.n || out.size() + len > limit) return false;
      out.insert(out.end(), br.p + byte + 4, br.p + byte + 4 + len);
      br.pos = (byte + 4 + len) * 8;
    } else if (type == 1) {
      uint8_t l[288], d[30];
      for (int i = 0; i < 144; ++i) l[i] = 8;
      for (int i = 144; i < 256; ++i) l[i] = 9;
      for (int i = 256; i < 280; ++i) l[i] = 7;
      for (int i = 280; i < 288; ++i) l[i] = 8;
      for (int i = 0; i < 30; ++i) d[i] = 5;
      Huffman lit, dist;
      lit.build(l, 288);
      dist.build(d, 30);
      if (!inflate_codes(br, lit, dist, out, limit)) return false;
    } else if (type == 2) {
      const int nlen = (int)br.bits(5) + 257, ndist = (int)br.bits(5) + 1, ncode = (int)br.bits(4) + 4;
      if (br.bad || nlen > 286 || ndist > 30) return false;
      static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
      uint8_t cl[19] = {0};
      for (int i = 0; i < ncode; ++i) cl[order[i]] = (uint8_t)br.bits(3);
      Huffman lencode;
      if (br.bad || !lencode.build(cl, 19)) return false;
      uint8_t lens[320] = {0};
      int idx = 0;
      while (idx < nlen + ndist) {
        const int sym = lencode.decode(br);
        if (sym < 0) return false;
        if (sym < 16) {
          lens[idx++] = (uint8_t)sym;
        } else {
          uint8_t val = 0;
          int rep;
          if (sym == 16) {
            if (idx == 0) return false;
            val = lens[idx - 1];
            rep = 3 + (int)br.bits(2);
          } else if (sym == 17) {
            rep = 3 + (int)br.bits(3);
          } else {
            rep = 11 + (int)br.bits(7);
          }
          if (br.bad || idx + rep > nlen + ndist) return false;
          while (rep--) lens[idx++] = val;
        }
      }
      if (lens[256] == 0) return false;  // no end-of-block code
      Huffman lit, dist;
      if (!lit.build(lens, nlen) || !dist.build(lens + nlen, ndist)) return false;
      if (!inflate_codes(br, lit, dist, out, limit)) return false;
    } else {
      return false;
    }
  }
  // Adler-32 of the output (RFC 1950 section 2.2), big-endian after the data
  const size_t end = 2 + ((br.pos + 7) >> 3);
  if (end + 4 > n) return false;
  uint32_t a = 1, b = 0;
  for (unsigned char c : out) {
    a = (a + c) % 65521u;
    b = (b + a) % 65521u;
  }
  const uint32_t want = ((uint32_t)in[end] << 24) | ((uint32_t)in[end + 1] << 16) | ((uint32_t)in[end + 2] << 8) | in[end + 3];
  return ((b << 16) | a) == want;
}

// ---------------------------------------------------------------- PNG ----
uint32_t be32(const unsigned char* p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}

uint32_t crc32_png(const unsigned char* p, size_t n) {
  static uint32_t table[256];
  static bool init = false;
  if (!init) {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t c = i;
      for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      table[i] = c;
    }
    init = true;
  }
  uint32_t c = 0xffffffffu;
  for (size_t i = 0; i < n; ++i) c = table[(c ^ p[i]) & 0xff] ^ (c >> 8);
  return c ^ 0xffffffffu;
}

const unsigned char kPngSig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};

// The unfiltered scanlines of a PNG (not interlaced; colour types 0 grey,
// 2 RGB, 4 grey + alpha, 6 RGBA; bit depth 8 or 16): rows of W * channels *
// depth / 8 bytes, big-endian samples.
qpso_status png_scanlines(const std::vector<unsigned char>& f, uint32_t* w, uint32_t* h, int* depth_out,
                          int* channels_out, std::vector<unsigned char>& pix) {
  if (f.size() < 8 || std::memcmp(f.data(), kPngSig, 8) != 0) return QPSO_ERR_ARG;
  size_t at = 8;
  uint32_t W = 0, H = 0;
  int depth = 0, ctype = -1, interlace = 0;
  std::vector<unsigned char> idat;
  bool seen_end = false;
  while (at + 12 <= f.size()) {
    const uint32_t len = be32(&f[at]);
    if (len > f.size() - at - 12) return QPSO_ERR_ARG;
    const unsigned char* type = &f[at + 4];
    const unsigned char* data = &f[at + 8];
    if (crc32_png(type, (size_t)len + 4) != be32(data + len)) return QPSO_ERR_ARG;
    if (!std::memcmp(type, "IHDR", 4)) {
      if (len != 13) return QPSO_ERR_ARG;
      W = be32(data);
      H = be32(data + 4);
      depth = data[8];
      ctype = data[9];
      if (data[10] != 0 || data[11] != 0) return QPSO_ERR_ARG;
      interlace = data[12];
    } else if (!std::memcmp(type, "IDAT", 4)) {
      idat.insert(idat.end(), data, data + len);
    } else if (!std::memcmp(type, "IEND", 4)) {
      seen_end = true;
      break;
    }
    at += (size_t)len + 12;
  }
  if (!seen_end || W == 0 || H == 0 || W > 16384 || H > 16384) return QPSO_ERR_ARG;
  const int channels = ctype == 0 ? 1 : ctype == 2 ? 3 : ctype == 4 ? 2 : ctype == 6 ? 4 : 0;
  if (channels == 0 || (depth != 8 && depth != 16) || interlace != 0) return QPSO_ERR_ARG;
  const size_t bpp = (size_t)channels * depth / 8, row = (size_t)W * bpp;
  std::vector<unsigned char> raw;
  const size_t want = (row + 1) * H;
  if (!zlib_inflate(idat.data(), idat.size(), raw, want) || raw.size() != want) return QPSO_ERR_ARG;
  std::vector<unsigned char> prev(row, 0), cur(row);
  pix.resize(row * H);
  for (uint32_t y = 0; y < H; ++y) {
    const unsigned char* s = &raw[(size_t)y * (row + 1)];
    const int filter = s[0];
    ++s;
    for (size_t i = 0; i < row; ++i) {
      const int a = i >= bpp ? cur[i - bpp] : 0, b = prev[i], c = i >= bpp ? prev[i - bpp] : 0;
      int pred;
      switch (filter) {
        case 0: pred = 0; break;
        case 1: pred = a; break;
        case 2: pred = b; break;
        case 3: pred = (a + b) >> 1; break;
        case 4: {
          const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
          pred = (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
          break;
        }
        default: return QPSO_ERR_ARG;
      }
      cur[i] = (unsigned char)(s[i] + pred);
    }
    std::memcpy(&pix[(size_t)y * row], cur.data(), row);
    prev.swap(cur);
  }
  *w = W;
  *h = H;
  *depth_out = depth;
  *channels_out = channels;
  return QPSO_OK;
}

// Greyscale PNG (colour type 0, bit depth 8 or 16, not interlaced) to uint16.
qpso_status decode_png_gray(const std::vector<unsigned char>& f, std::vector<uint16_t>& px, uint32_t* w,
                            uint32_t* h) {
  std::vector<unsigned char> pix;
  int depth = 0, channels = 0;
  uint32_t W = 0, H = 0;
  const qpso_status st = png_scanlines(f, &W, &H, &depth, &channels, pix);
  if (st != QPSO_OK) return st;
  if (channels != 1) return QPSO_ERR_ARG;
  px.resize((size_t)W * H);
  for (size_t i = 0; i < px.size(); ++i)
    px[i] = depth == 16 ? (uint16_t)((pix[2 * i] << 8) | pix[2 * i + 1]) : pix[i];
  *w = W;
  *h = H;
  return QPSO_OK;
}

// Colour PNG to 8-bit B, G, R (OpenCV's channel order, as cv::imread gives
// the reference): RGB and RGBA drop alpha, grey is replicated, 16-bit
// samples keep their high byte.
qpso_status decode_png_bgr(const std::vector<unsigned char>& f, std::vector<unsigned char>& bgr, uint32_t* w,
                           uint32_t* h) {
  std::vector<unsigned char> pix;
  int depth = 0, channels = 0;
  uint32_t W = 0, H = 0;
  const qpso_status st = png_scanlines(f, &W, &H, &depth, &channels, pix);
  if (st != QPSO_OK) return st;
  const size_t n = (size_t)W * H, step = (size_t)channels * (depth / 8), sb = depth / 8;
  bgr.resize(3 * n);
  for (size_t i = 0; i < n; ++i) {
    const unsigned char* p = &pix[i * step];
    unsigned char r, g, b;
    if (channels >= 3) {
      r = p[0];
      g = p[sb];
      b = p[2 * sb];
    } else {
      r = g = b = p[0];
    }
    bgr[3 * i] = b;
    bgr[3 * i + 1] = g;
    bgr[3 * i + 2] = r;
  }
  *w = W;
  *h = H;
  return QPSO_OK;
}

// Binary PPM (P6, maxval 255): RGB samples to B, G, R.
qpso_status decode_ppm_bgr(const std::vector<unsigned char>& f, std::vector<unsigned char>& bgr, uint32_t* w,
                           uint32_t* h) {
  if (f.size() < 2 || f[0] != 'P' || f[1] != '6') return QPSO_ERR_ARG;
  size_t at = 2;
  long vals[3];
  for (int k = 0; k < 3; ++k) {
    for (;;) {  // whitespace and comments
      while (at < f.size() && std::isspace(f[at])) ++at;
      if (at < f.size() && f[at] == '#') {
        while (at < f.size() && f[at] != '\n') ++at;
        continue;
      }
      break;
    }
    long v = 0;
    int digits = 0;
    while (at < f.size() && f[at] >= '0' && f[at] <= '9' && digits < 9) v = v * 10 + (f[at++] - '0'), ++digits;
    if (digits == 0) return QPSO_ERR_ARG;
    vals[k] = v;
  }
  if (at >= f.size() || !std::isspace(f[at])) return QPSO_ERR_ARG;
  ++at;
  const long W = vals[0], H = vals[1];
  if (W <= 0 || H <= 0 || W > 16384 || H > 16384 || vals[2] != 255) return QPSO_ERR_ARG;
  const size_t n = (size_t)W * H;
  if (f.size() - at < 3 * n) return QPSO_ERR_ARG;
  bgr.resize(3 * n);
  for (size_t i = 0; i < n; ++i) {
    bgr[3 * i] = f[at + 3 * i + 2];
    bgr[3 * i + 1] = f[at + 3 * i + 1];
    bgr[3 * i + 2] = f[at + 3 * i];
  }
  *w = (uint32_t)W;
  *h = (uint32_t)H;
  return QPSO_OK;
}

// ACCV binary depth (loadDepth, main.cu:35-64).
qpso_status decode_accv(const std::vector<unsigned char>& f, std::vector<uint16_t>& px, uint32_t* w,
                        uint32_t* h) {
  if (f.size() < 8) return QPSO_ERR_ARG;
  int32_t rows, cols;
  std::memcpy(&rows, f.data(), 4);
  std::memcpy(&cols, f.data() + 4, 4);
  if (rows <= 0 || cols <= 0 || rows > 16384 || cols > 16384) return QPSO_ERR_ARG;
  const size_t n = (size_t)rows * (size_t)cols;
  if (f.size() != 8 + 2 * n) return QPSO_ERR_ARG;
  px.resize(n);
  std::memcpy(px.data(), f.data() + 8, 2 * n);
  *w = (uint32_t)cols;
  *h = (uint32_t)rows;
  return QPSO_OK;
}

}  // namespace

extern "C" {

qpso_status qpso_obj_load(const char* path, float* soa_out, uint32_t capacity_faces, uint32_t* num_faces) {
  if (!path || !num_faces) return QPSO_ERR_ARG;
  std::vector<float> xyz;
  std::vector<uint32_t> tri;
  const qpso_status st = load_obj(path, xyz, tri);
  if (st != QPSO_OK) return st;
  const size_t F = tri.size() / 3;
  if (F > (1u << 26)) return QPSO_ERR_ARG;
  *num_faces = (uint32_t)F;
  if (!soa_out) return QPSO_OK;
  if (F > capacity_faces) return QPSO_ERR_ARG;
  // loadOBJ3: soa[f + j*F + c*3F] = coordinate c of corner j of face f
  for (size_t f = 0; f < F; ++f)
    for (int j = 0; j < 3; ++j)
      for (int c = 0; c < 3; ++c) soa_out[f + (size_t)j * F + (size_t)c * 3 * F] = xyz[3 * (size_t)tri[3 * f + j] + c];
  return QPSO_OK;
}

qpso_status qpso_image_u16_load(const char* path, uint16_t* out, uint64_t capacity_px, uint32_t* width,
                                uint32_t* height) {
  if (!path || !width || !height) return QPSO_ERR_ARG;
  std::vector<unsigned char> f;
  if (!read_file(path, f)) return QPSO_ERR_NOT_FOUND;
  std::vector<uint16_t> px;
  uint32_t w = 0, h = 0;
  const bool png = f.size() >= 8 && std::memcmp(f.data(), kPngSig, 8) == 0;
  const qpso_status st = png ? decode_png_gray(f, px, &w, &h) : decode_accv(f, px, &w, &h);
  if (st != QPSO_OK) return st;
  *width = w;
  *height = h;
  if (!out) return QPSO_OK;
  if (px.size() > capacity_px) return QPSO_ERR_ARG;
  std::memcpy(out, px.data(), px.size() * 2);
  return QPSO_OK;
}

qpso_status qpso_image_bgr8_load(const char* path, uint8_t* out, uint64_t capacity_px, uint32_t* width,
                                 uint32_t* height) {
  if (!path || !width || !height) return QPSO_ERR_ARG;
  std::vector<unsigned char> f;
  if (!read_file(path, f)) return QPSO_ERR_NOT_FOUND;
  std::vector<unsigned char> bgr;
  uint32_t w = 0, h = 0;
  const bool png = f.size() >= 8 && std::memcmp(f.data(), kPngSig, 8) == 0;
  const qpso_status st = png ? decode_png_bgr(f, bgr, &w, &h) : decode_ppm_bgr(f, bgr, &w, &h);
  if (st != QPSO_OK) return st;
  *width = w;
  *height = h;
  if (!out) return QPSO_OK;
  if ((uint64_t)w * h > capacity_px) return QPSO_ERR_ARG;
  std::memcpy(out, bgr.data(), bgr.size());
  return QPSO_OK;
}

}  // extern "C"
