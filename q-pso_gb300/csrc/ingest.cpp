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
//    section 9);
// and one writer: baseline JPEG (ITU-T T.81), for the cluster images the
// reference's main writes with cv::imwrite (main.cu:1262-1272).
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


// ---- baseline JPEG writer (ITU-T T.81: sequential DCT, Huffman coding) ----
//
// 4:4:4 YCbCr (JFIF, ITU-T T.871), one 8x8 block per component per MCU,
// edges padded by repeating the last row and column.  The quantisation
// tables are the example tables of T.81 Annex K.1 scaled by quality as the
// IJG software scales them (cv::imwrite's default is quality 95); the
// Huffman tables are the typical tables of Annex K.3, written into the file.

const uint8_t kJpegZig[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                              12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                              35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                              58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};
// Annex K.1, natural (row-major) order
const uint8_t kJpegQLum[64] = {16, 11, 10, 16, 24,  40,  51,  61,  12, 12, 14, 19, 26,  58,  60,  55,
                               14, 13, 16, 24, 40,  57,  69,  56,  14, 17, 22, 29, 51,  87,  80,  62,
                               18, 22, 37, 56, 68,  109, 103, 77,  24, 35, 55, 64, 81,  104, 113, 92,
                               49, 64, 78, 87, 103, 121, 120, 101, 72, 92, 95, 98, 112, 100, 103, 99};
const uint8_t kJpegQChr[64] = {17, 18, 24, 47, 99, 99, 99, 99, 18, 21, 26, 66, 99, 99, 99, 99,
                               24, 26, 56, 99, 99, 99, 99, 99, 47, 66, 99, 99, 99, 99, 99, 99,
                               99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99,
                               99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99};
// Annex K.3: code lengths (BITS, 1..16) and symbols (HUFFVAL)
const uint8_t kDcLumBits[16] = {0, 1, 5, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0};
const uint8_t kDcChrBits[16] = {0, 3, 1, 1, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0};
const uint8_t kDcVals[12] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11};
const uint8_t kAcLumBits[16] = {0, 2, 1, 3, 3, 2, 4, 3, 5, 5, 4, 4, 0, 0, 1, 0x7d};
const uint8_t kAcLumVals[162] = {
    0x01, 0x02, 0x03, 0x00, 0x04, 0x11, 0x05, 0x12, 0x21, 0x31, 0x41, 0x06, 0x13, 0x51, 0x61, 0x07, 0x22, 0x71,
    0x14, 0x32, 0x81, 0x91, 0xa1, 0x08, 0x23, 0x42, 0xb1, 0xc1, 0x15, 0x52, 0xd1, 0xf0, 0x24, 0x33, 0x62, 0x72,
    0x82, 0x09, 0x0a, 0x16, 0x17, 0x18, 0x19, 0x1a, 0x25, 0x26, 0x27, 0x28, 0x29, 0x2a, 0x34, 0x35, 0x36, 0x37,
    0x38, 0x39, 0x3a, 0x43, 0x44, 0x45, 0x46, 0x47, 0x48, 0x49, 0x4a, 0x53, 0x54, 0x55, 0x56, 0x57, 0x58, 0x59,
    0x5a, 0x63, 0x64, 0x65, 0x66, 0x67, 0x68, 0x69, 0x6a, 0x73, 0x74, 0x75, 0x76, 0x77, 0x78, 0x79, 0x7a, 0x83,
    0x84, 0x85, 0x86, 0x87, 0x88, 0x89, 0x8a, 0x92, 0x93, 0x94, 0x95, 0x96, 0x97, 0x98, 0x99, 0x9a, 0xa2, 0xa3,
    0xa4, 0xa5, 0xa6, 0xa7, 0xa8, 0xa9, 0xaa, 0xb2, 0xb3, 0xb4, 0xb5, 0xb6, 0xb7, 0xb8, 0xb9, 0xba, 0xc2, 0xc3,
    0xc4, 0xc5, 0xc6, 0xc7, 0xc8, 0xc9, 0xca, 0xd2, 0xd3, 0xd4, 0xd5, 0xd6, 0xd7, 0xd8, 0xd9, 0xda, 0xe1, 0xe2,
    0xe3, 0xe4, 0xe5, 0xe6, 0xe7, 0xe8, 0xe9, 0xea, 0xf1, 0xf2, 0xf3, 0xf4, 0xf5, 0xf6, 0xf7, 0xf8, 0xf9, 0xfa};
const uint8_t kAcChrBits[16] = {0, 2, 1, 2, 4, 4, 3, 4, 7, 5, 4, 4, 0, 1, 2, 0x77};
const uint8_t kAcChrVals[162] = {
    0x00, 0x01, 0x02, 0x03, 0x11, 0x04, 0x05, 0x21, 0x31, 0x06, 0x12, 0x41, 0x51, 0x07, 0x61, 0x71, 0x13, 0x22,
    0x32, 0x81, 0x08, 0x14, 0x42, 0x91, 0xa1, 0xb1, 0xc1, 0x09, 0x23, 0x33, 0x52, 0xf0, 0x15, 0x62, 0x72, 0xd1,
    0x0a, 0x16, 0x24, 0x34, 0xe1, 0x25, 0xf1, 0x17, 0x18, 0x19, 0x1a, 0x26, 0x27, 0x28, 0x29, 0x2a, 0x35, 0x36,
    0x37, 0x38, 0x39, 0x3a, 0x43, 0x44, 0x45, 0x46, 0x47, 0x48, 0x49, 0x4a, 0x53, 0x54, 0x55, 0x56, 0x57, 0x58,
    0x59, 0x5a, 0x63, 0x64, 0x65, 0x66, 0x67, 0x68, 0x69, 0x6a, 0x73, 0x74, 0x75, 0x76, 0x77, 0x78, 0x79, 0x7a,
    0x82, 0x83, 0x84, 0x85, 0x86, 0x87, 0x88, 0x89, 0x8a, 0x92, 0x93, 0x94, 0x95, 0x96, 0x97, 0x98, 0x99, 0x9a,
    0xa2, 0xa3, 0xa4, 0xa5, 0xa6, 0xa7, 0xa8, 0xa9, 0xaa, 0xb2, 0xb3, 0xb4, 0xb5, 0xb6, 0xb7, 0xb8, 0xb9, 0xba,
    0xc2, 0xc3, 0xc4, 0xc5, 0xc6, 0xc7, 0xc8, 0xc9, 0xca, 0xd2, 0xd3, 0xd4, 0xd5, 0xd6, 0xd7, 0xd8, 0xd9, 0xda,
    0xe2, 0xe3, 0xe4, 0xe5, 0xe6, 0xe7, 0xe8, 0xe9, 0xea, 0xf2, 0xf3, 0xf4, 0xf5, 0xf6, 0xf7, 0xf8, 0xf9, 0xfa};

// the canonical code of a table (Annex C): code and length per symbol
struct HuffCode {
  uint16_t code[256];
  uint8_t len[256];
  bool ok;
};

HuffCode huff_codes(const uint8_t bits[16], const uint8_t* vals) {
  HuffCode h;
  std::memset(&h, 0, sizeof(h));
  uint32_t code = 0;
  int k = 0;
  for (int l = 1; l <= 16; ++l) {
    for (int i = 0; i < bits[l - 1]; ++i, ++k) {
      h.code[vals[k]] = (uint16_t)code;
      h.len[vals[k]] = (uint8_t)l;
      ++code;
    }
    code <<= 1;
  }
  h.ok = true;
  return h;
}

struct BitWriter {
  std::vector<unsigned char>& out;
  uint32_t acc = 0;
  int n = 0;
  explicit BitWriter(std::vector<unsigned char>& o) : out(o) {}
  void put(uint32_t v, int len) {  // len <= 16
    acc = (acc << len) | (v & ((1u << len) - 1u));
    n += len;
    while (n >= 8) {
      const unsigned char b = (unsigned char)(acc >> (n - 8));
      out.push_back(b);
      if (b == 0xFF) out.push_back(0x00);  // byte stuffing
      n -= 8;
    }
    acc &= (1u << n) - 1u;
  }
  void flush() {  // pad with 1-bits
    if (n > 0) put((1u << (8 - n)) - 1u, 8 - n);
  }
};

int bit_size(int v) {  // the magnitude category of v
  v = v < 0 ? -v : v;
  int s = 0;
  while (v) {
    ++s;
    v >>= 1;
  }
  return s;
}

void put_u16(std::vector<unsigned char>& o, uint32_t v) {
  o.push_back((unsigned char)(v >> 8));
  o.push_back((unsigned char)v);
}

// forward DCT of one 8x8 block (level-shifted samples), separable, by the
// definition: F(u,v) = 1/4 C(u) C(v) sum f(x,y) cos((2x+1)u pi/16) cos((2y+1)v pi/16)
void fdct8x8(const double in[64], double out[64]) {
  static double c[8][8];
  static bool init = false;
  if (!init) {
    for (int u = 0; u < 8; ++u)
      for (int x = 0; x < 8; ++x)
        c[u][x] = (u == 0 ? std::sqrt(0.125) : 0.5) * std::cos((2 * x + 1) * u * 3.14159265358979323846 / 16.0);
    init = true;
  }
  double t[64];
  for (int y = 0; y < 8; ++y)
    for (int u = 0; u < 8; ++u) {
      double s = 0.0;
      for (int x = 0; x < 8; ++x) s += c[u][x] * in[y * 8 + x];
      t[y * 8 + u] = s;
    }
  for (int u = 0; u < 8; ++u)
    for (int v = 0; v < 8; ++v) {
      double s = 0.0;
      for (int y = 0; y < 8; ++y) s += c[v][y] * t[y * 8 + u];
      out[v * 8 + u] = s;
    }
}

std::vector<unsigned char> encode_jpeg(const uint8_t* bgr, uint32_t w, uint32_t h, int quality) {
  quality = quality < 1 ? 1 : quality > 100 ? 100 : quality;
  const int scale = quality < 50 ? 5000 / quality : 200 - 2 * quality;
  uint8_t q[2][64];
  for (int i = 0; i < 64; ++i) {
    int a = (kJpegQLum[i] * scale + 50) / 100, b = (kJpegQChr[i] * scale + 50) / 100;
    q[0][i] = (uint8_t)(a < 1 ? 1 : a > 255 ? 255 : a);
    q[1][i] = (uint8_t)(b < 1 ? 1 : b > 255 ? 255 : b);
  }
  const HuffCode dc[2] = {huff_codes(kDcLumBits, kDcVals), huff_codes(kDcChrBits, kDcVals)};
  const HuffCode ac[2] = {huff_codes(kAcLumBits, kAcLumVals), huff_codes(kAcChrBits, kAcChrVals)};
  std::vector<unsigned char> o;
  o.reserve((size_t)w * h + 1024);
  o.push_back(0xFF), o.push_back(0xD8);  // SOI
  // APP0 JFIF 1.01, no density units, no thumbnail
  o.push_back(0xFF), o.push_back(0xE0);
  put_u16(o, 16);
  const unsigned char jfif[] = {'J', 'F', 'I', 'F', 0, 1, 1, 0, 0, 1, 0, 1, 0, 0};
  o.insert(o.end(), jfif, jfif + sizeof(jfif));
  for (int t = 0; t < 2; ++t) {  // DQT, in zigzag order
    o.push_back(0xFF), o.push_back(0xDB);
    put_u16(o, 67);
    o.push_back((unsigned char)t);
    for (int k = 0; k < 64; ++k) o.push_back(q[t][kJpegZig[k]]);
  }
  o.push_back(0xFF), o.push_back(0xC0);  // SOF0
  put_u16(o, 17);
  o.push_back(8);
  put_u16(o, h);
  put_u16(o, w);
  o.push_back(3);
  for (int c = 0; c < 3; ++c) {
    o.push_back((unsigned char)(c + 1));
    o.push_back(0x11);
    o.push_back(c == 0 ? 0 : 1);
  }
  struct Table {
    int tc_th;
    const uint8_t* bits;
    const uint8_t* vals;
    int n;
  };
  const Table tabs[4] = {{0x00, kDcLumBits, kDcVals, 12}, {0x10, kAcLumBits, kAcLumVals, 162},
                         {0x01, kDcChrBits, kDcVals, 12}, {0x11, kAcChrBits, kAcChrVals, 162}};
  for (const Table& t : tabs) {  // DHT
    o.push_back(0xFF), o.push_back(0xC4);
    put_u16(o, (uint32_t)(3 + 16 + t.n));
    o.push_back((unsigned char)t.tc_th);
    o.insert(o.end(), t.bits, t.bits + 16);
    o.insert(o.end(), t.vals, t.vals + t.n);
  }
  o.push_back(0xFF), o.push_back(0xDA);  // SOS
  put_u16(o, 12);
  o.push_back(3);
  for (int c = 0; c < 3; ++c) {
    o.push_back((unsigned char)(c + 1));
    o.push_back(c == 0 ? 0x00 : 0x11);
  }
  o.push_back(0), o.push_back(63), o.push_back(0);
  BitWriter bw(o);
  int pred[3] = {0, 0, 0};
  double blk[64], coef[64];
  for (uint32_t by = 0; by < h; by += 8)
    for (uint32_t bx = 0; bx < w; bx += 8)
      for (int c = 0; c < 3; ++c) {
        for (int y = 0; y < 8; ++y)
          for (int x = 0; x < 8; ++x) {
            const uint32_t sy = by + y < h ? by + y : h - 1, sx = bx + x < w ? bx + x : w - 1;
            const uint8_t* p = bgr + 3 * ((size_t)sy * w + sx);
            const double B = p[0], G = p[1], R = p[2];
            const double v = c == 0   ? 0.299 * R + 0.587 * G + 0.114 * B
                             : c == 1 ? -0.168736 * R - 0.331264 * G + 0.5 * B + 128.0
                                      : 0.5 * R - 0.418688 * G - 0.081312 * B + 128.0;
            blk[y * 8 + x] = v - 128.0;
          }
        fdct8x8(blk, coef);
        const int t = c == 0 ? 0 : 1;
        int zz[64];
        for (int k = 0; k < 64; ++k) {
          const int i = kJpegZig[k];
          zz[k] = (int)std::lround(coef[i] / q[t][i]);
        }
        // the tables code DC differences up to category 11 and AC values up
        // to category 10: clamp (reached only near quality 100)
        for (int k = 1; k < 64; ++k) zz[k] = zz[k] < -1023 ? -1023 : zz[k] > 1023 ? 1023 : zz[k];
        // DC: the difference from the component's previous block
        int diff = zz[0] - pred[c];
        diff = diff < -2047 ? -2047 : diff > 2047 ? 2047 : diff;
        pred[c] += diff;
        const int s = bit_size(diff);
        bw.put(dc[t].code[s], dc[t].len[s]);
        if (s) bw.put((uint32_t)(diff < 0 ? diff - 1 : diff), s);
        // AC: runs of zeros and magnitude categories
        int run = 0;
        for (int k = 1; k < 64; ++k) {
          if (zz[k] == 0) {
            ++run;
            continue;
          }
          while (run > 15) {
            bw.put(ac[t].code[0xF0], ac[t].len[0xF0]);
            run -= 16;
          }
          const int sz = bit_size(zz[k]);
          const int sym = (run << 4) | sz;
          bw.put(ac[t].code[sym], ac[t].len[sym]);
          bw.put((uint32_t)(zz[k] < 0 ? zz[k] - 1 : zz[k]), sz);
          run = 0;
        }
        if (run > 0) bw.put(ac[t].code[0x00], ac[t].len[0x00]);  // end of block
      }
  bw.flush();
  o.push_back(0xFF), o.push_back(0xD9);  // EOI
  return o;
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

qpso_status qpso_image_jpeg_write(const char* path, const uint8_t* bgr, uint32_t width, uint32_t height,
                                  int32_t quality) {
  if (!path || !bgr || width == 0 || height == 0 || width > 65535 || height > 65535 || quality < 1 ||
      quality > 100)
    return QPSO_ERR_ARG;
  const std::vector<unsigned char> jpg = encode_jpeg(bgr, width, height, quality);
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return QPSO_ERR_NOT_FOUND;
  const bool ok = std::fwrite(jpg.data(), 1, jpg.size(), fp) == jpg.size();
  return (std::fclose(fp) == 0 && ok) ? QPSO_OK : QPSO_ERR_NOT_FOUND;
}

}  // extern "C"
