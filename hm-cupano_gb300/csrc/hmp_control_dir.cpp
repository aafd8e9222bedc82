// hmp_control_dir.cpp -- loader of a stitching control directory (host only).
//
// A control directory holds, per image i, Hugin nona's coordinate tables mapping_000i_x.tif /
// mapping_000i_y.tif (16-bit unsigned, canvas pixel -> source column / row, 65535 = unmapped) and
// mapping_000i.tif, whose XPosition / YPosition tags (in resolution units) place the table on the
// canvas, plus seam_file.png (enblend / multiblend): an 8-bit paletted image of per-pixel image
// indices, or a grayscale one. Replaces ControlMasks::load (src/pano/controlMasks.cpp:133-326),
// ControlMasks3::load (src/pano/controlMasks3.cpp:186-300) and ControlMasksN::load
// (src/pano/controlMasksN.cpp:22-193), which use libtiff, libpng and OpenCV; neither machine has
// those libraries, so the TIFF and PNG decoders (with an RFC 1951 inflate) are written here.
//
// Rules kept from the reference:
//   positions : XPosition * XResolution (float products, as libtiff returns the tags), snapped to
//               the nearest integer within 1e-3 (cupano/masks.py:35-51), then shifted so that the
//               smallest is 0 (controlMasks.cpp:42-59)
//   seam, two images : the smallest value -> 1 (weight of image 1), the largest -> 0
//               (controlMasks.cpp:225-250)
//   seam, three images : 8-bit paletted with labels exactly {0, 1, 2} (controlMasks3.cpp:186-196)
//   seam, N images : exactly N distinct values, remapped in order to 0..N-1 (controlMasksN.cpp:150-183)
//   seam decoding : palette indices for an 8-bit paletted PNG, else grayscale (OpenCV's
//               IMREAD_GRAYSCALE: 16-bit samples keep the high byte, colour is weighted
//               0.299 / 0.587 / 0.114)
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include "hmpano.h"

namespace {

using Bytes = std::vector<uint8_t>;

struct LoadError : std::runtime_error {
  int code;
  LoadError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] void fail(const std::string& m, int code = HMP_ERR_INVALID_VALUE) { throw LoadError(code, m); }

// Largest image side and pixel count either decoder accepts; larger headers are rejected before
// anything is sized from them (and keep every byte count below 2^40).
constexpr int64_t kMaxSide = int64_t(1) << 20;
constexpr int64_t kMaxPixels = int64_t(1) << 31;

void check_size(int64_t w, int64_t h, const std::string& path) {
  if (w <= 0 || h <= 0) fail("image without pixels: " + path);
  if (w > kMaxSide || h > kMaxSide || w * h > kMaxPixels)
    fail("image larger than 2^20 pixels per side or 2^31 pixels: " + path, HMP_ERR_NOT_SUPPORTED);
}

Bytes read_file(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) fail("Cannot open file: " + path, HMP_ERR_FILE_NOT_FOUND);
  Bytes b;
  uint8_t buf[1 << 16];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) b.insert(b.end(), buf, buf + n);
  std::fclose(f);
  return b;
}

// ---- inflate (RFC 1951) ----

class Inflate {
 public:
  // `limit`: the most output bytes the caller uses; decoding stops once they are out.
  Inflate(const uint8_t* p, size_t n, Bytes& out, size_t limit) : p_(p), n_(n), out_(out), limit_(limit) {}

  void run() {
    int last;
    do {
      last = int(bits(1));
      const int type = int(bits(2));
      if (type == 0)
        stored();
      else if (type == 1)
        fixed();
      else if (type == 2)
        dynamic();
      else
        fail("corrupt deflate stream (block type 3)");
    } while (!last && out_.size() < limit_);
  }

 private:
  struct Huff {
    uint16_t count[16];
    uint16_t symbol[320];
  };

  uint32_t bits(int need) {
    while (cnt_ < need) {
      if (pos_ >= n_) fail("truncated deflate stream");
      buf_ |= uint32_t(p_[pos_++]) << cnt_;
      cnt_ += 8;
    }
    const uint32_t v = buf_ & ((1u << need) - 1u);
    buf_ >>= need;
    cnt_ -= need;
    return v;
  }

  void stored() {
    buf_ = 0;
    cnt_ = 0;
    if (pos_ + 4 > n_) fail("truncated deflate stream");
    const unsigned len = p_[pos_] | (p_[pos_ + 1] << 8), nlen = p_[pos_ + 2] | (p_[pos_ + 3] << 8);
    pos_ += 4;
    if ((len ^ 0xFFFFu) != nlen) fail("corrupt deflate stream (stored length)");
    if (pos_ + len > n_) fail("truncated deflate stream");
    out_.insert(out_.end(), p_ + pos_, p_ + pos_ + std::min<size_t>(len, limit_ - out_.size()));
    pos_ += len;
  }

  static void build(Huff& h, const uint8_t* len, int n) {
    std::memset(h.count, 0, sizeof(h.count));
    for (int s = 0; s < n; ++s) h.count[len[s]]++;
    h.count[0] = 0;
    uint16_t offs[16];
    offs[1] = 0;
    for (int l = 1; l < 15; ++l) offs[l + 1] = uint16_t(offs[l] + h.count[l]);
    for (int s = 0; s < n; ++s)
      if (len[s]) h.symbol[offs[len[s]]++] = uint16_t(s);
  }

  // Canonical Huffman decode, one bit at a time (codes are stored MSB-first within the LSB-first stream).
  int decode(const Huff& h) {
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; ++l) {
      code |= int(bits(1));
      const int count = h.count[l];
      if (code - count < first) return h.symbol[index + (code - first)];
      index += count;
      first += count;
      first <<= 1;
      code <<= 1;
    }
    fail("corrupt deflate stream (bad code)");
  }

  void codes(const Huff& lit, const Huff& dist) {
    // Base lengths / distances and extra bits of the length and distance codes (RFC 1951 3.2.5).
    static const uint16_t lbase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                       31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
    static const uint8_t lext[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
    static const uint16_t dbase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                       193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
    static const uint8_t dext[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
    for (;;) {
      int sym = decode(lit);
      if (out_.size() >= limit_) return;
      if (sym < 256) {
        out_.push_back(uint8_t(sym));
      } else if (sym == 256) {
        return;
      } else {
        sym -= 257;
        if (sym >= 29) fail("corrupt deflate stream (length code)");
        const size_t len = lbase[sym] + bits(lext[sym]);
        const int ds = decode(dist);
        if (ds >= 30) fail("corrupt deflate stream (distance code)");
        const size_t d = dbase[ds] + bits(dext[ds]);
        if (d > out_.size()) fail("corrupt deflate stream (distance too far)");
        const size_t from = out_.size() - d, copy = std::min<size_t>(len, limit_ - out_.size());
        for (size_t k = 0; k < copy; ++k) {
          const uint8_t v = out_[from + k];
          out_.push_back(v);
        }
      }
    }
  }

  void fixed() {
    uint8_t len[320];
    int s = 0;
    for (; s < 144; ++s) len[s] = 8;
    for (; s < 256; ++s) len[s] = 9;
    for (; s < 280; ++s) len[s] = 7;
    for (; s < 288; ++s) len[s] = 8;
    Huff lit, dist;
    build(lit, len, 288);
    for (s = 0; s < 30; ++s) len[s] = 5;
    build(dist, len, 30);
    codes(lit, dist);
  }

  void dynamic() {
    static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
    const int nlen = int(bits(5)) + 257, ndist = int(bits(5)) + 1, ncode = int(bits(4)) + 4;
    if (nlen > 286 || ndist > 30) fail("corrupt deflate stream (code counts)");
    uint8_t len[320] = {};
    for (int i = 0; i < ncode; ++i) len[order[i]] = uint8_t(bits(3));
    Huff lencode;
    build(lencode, len, 19);
    std::memset(len, 0, sizeof(len));
    int i = 0;
    while (i < nlen + ndist) {
      const int sym = decode(lencode);
      if (sym < 16) {
        len[i++] = uint8_t(sym);
      } else {
        int rep, val = 0;
        if (sym == 16) {
          if (i == 0) fail("corrupt deflate stream (repeat with no length)");
          val = len[i - 1];
          rep = 3 + int(bits(2));
        } else if (sym == 17) {
          rep = 3 + int(bits(3));
        } else {
          rep = 11 + int(bits(7));
        }
        if (i + rep > nlen + ndist) fail("corrupt deflate stream (too many lengths)");
        while (rep--) len[i++] = uint8_t(val);
      }
    }
    if (len[256] == 0) fail("corrupt deflate stream (no end-of-block code)");
    Huff lit, dist;
    build(lit, len, nlen);
    build(dist, len + nlen, ndist);
    codes(lit, dist);
  }

  const uint8_t* p_;
  size_t n_, pos_ = 0;
  uint32_t buf_ = 0;
  int cnt_ = 0;
  Bytes& out_;
  size_t limit_;
};

// zlib stream (RFC 1950): a 2-byte header, deflate data, Adler-32 (not checked). At most `limit`
// output bytes.
Bytes zlib_inflate(const uint8_t* p, size_t n, size_t limit) {
  if (n < 2 || (p[0] & 0x0F) != 8 || ((p[0] << 8) | p[1]) % 31 != 0 || (p[1] & 0x20))
    fail("not a zlib stream");
  Bytes out;
  Inflate(p + 2, n - 2, out, limit).run();
  return out;
}

// ---- PNG ----

uint32_t be32(const uint8_t* p) { return (uint32_t(p[0]) << 24) | (uint32_t(p[1]) << 16) | (uint32_t(p[2]) << 8) | p[3]; }

struct Png {
  int w = 0, h = 0, depth = 0, color = 0;
  std::vector<uint8_t> palette;  // RGB triples
  Bytes pix;                     // unfiltered rows, ceil(w * channels * depth / 8) bytes each
  int channels() const { return color == 0 || color == 3 ? 1 : color == 2 ? 3 : color == 4 ? 2 : 4; }
  size_t row_bytes() const { return (size_t(w) * channels() * depth + 7) / 8; }
};

Png decode_png(const std::string& path) {
  const Bytes b = read_file(path);
  static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
  if (b.size() < 8 || std::memcmp(b.data(), sig, 8) != 0) fail("File is not recognized as a PNG: " + path);
  Png png;
  Bytes idat;
  int interlace = 0;
  size_t pos = 8;
  bool have_header = false;
  while (pos + 12 <= b.size()) {
    const uint32_t len = be32(&b[pos]);
    const std::string type(reinterpret_cast<const char*>(&b[pos + 4]), 4);
    if (pos + 12 + size_t(len) > b.size()) fail("truncated PNG chunk: " + path);
    const uint8_t* d = &b[pos + 8];
    if (type == "IHDR") {
      if (len < 13) fail("bad PNG header: " + path);
      png.w = int(std::min<uint32_t>(be32(d), uint32_t(INT32_MAX)));
      png.h = int(std::min<uint32_t>(be32(d + 4), uint32_t(INT32_MAX)));
      png.depth = d[8];
      png.color = d[9];
      interlace = d[12];
      have_header = true;
    } else if (type == "PLTE") {
      png.palette.assign(d, d + len);
    } else if (type == "IDAT") {
      idat.insert(idat.end(), d, d + len);
    } else if (type == "IEND") {
      break;
    }
    pos += 12 + size_t(len);
  }
  if (!have_header) fail("PNG without a valid header: " + path);
  check_size(int64_t(png.w), int64_t(png.h), path);
  if (interlace) fail("interlaced PNG is not supported: " + path, HMP_ERR_NOT_SUPPORTED);
  const std::set<int> depths = png.color == 0 ? std::set<int>{1, 2, 4, 8, 16}
                               : png.color == 3 ? std::set<int>{1, 2, 4, 8}
                                                : std::set<int>{8, 16};
  if (!(png.color == 0 || png.color == 2 || png.color == 3 || png.color == 4 || png.color == 6) || !depths.count(png.depth))
    fail("unsupported PNG colour type / bit depth: " + path, HMP_ERR_NOT_SUPPORTED);
  const size_t rb = png.row_bytes(), bpp = std::max<size_t>(1, size_t(png.channels()) * png.depth / 8);
  const Bytes raw = zlib_inflate(idat.data(), idat.size(), (rb + 1) * size_t(png.h));
  if (raw.size() < (rb + 1) * size_t(png.h)) fail("truncated PNG image data: " + path);
  png.pix.assign(rb * size_t(png.h), 0);
  for (int y = 0; y < png.h; ++y) {
    const uint8_t filter = raw[(rb + 1) * size_t(y)];
    const uint8_t* src = &raw[(rb + 1) * size_t(y) + 1];
    uint8_t* row = &png.pix[rb * size_t(y)];
    const uint8_t* prev = y ? row - rb : nullptr;
    for (size_t i = 0; i < rb; ++i) {
      const int a = i >= bpp ? row[i - bpp] : 0, up = prev ? prev[i] : 0, c = (prev && i >= bpp) ? prev[i - bpp] : 0;
      int v = src[i];
      switch (filter) {
        case 0: break;
        case 1: v += a; break;
        case 2: v += up; break;
        case 3: v += (a + up) >> 1; break;
        case 4: {
          const int pp = a + up - c, pa = std::abs(pp - a), pb = std::abs(pp - up), pc = std::abs(pp - c);
          v += (pa <= pb && pa <= pc) ? a : (pb <= pc ? up : c);
          break;
        }
        default: fail("bad PNG filter type: " + path);
      }
      row[i] = uint8_t(v);
    }
  }
  return png;
}

uint8_t gray_of(int r, int g, int b) {
  // ITU-R BT.601 weights in 14-bit fixed point, rounded (0.299, 0.587, 0.114).
  return uint8_t((r * 4899 + g * 9617 + b * 1868 + 8192) >> 14);
}

// Seam raster: palette indices of an 8-bit paletted PNG (`paletted` = true), else the grayscale image.
std::vector<uint8_t> read_seam_png(const std::string& path, int& w, int& h, bool& paletted) {
  const Png png = decode_png(path);
  w = png.w;
  h = png.h;
  paletted = png.color == 3 && png.depth == 8;
  std::vector<uint8_t> out(size_t(w) * h);
  const size_t rb = png.row_bytes();
  const auto sample = [&](int y, size_t s) -> int {  // sample s of row y at its bit depth
    const uint8_t* row = &png.pix[rb * size_t(y)];
    if (png.depth == 8) return row[s];
    if (png.depth == 16) return (row[2 * s] << 8) | row[2 * s + 1];
    const int per = 8 / png.depth;
    return (row[s / per] >> (8 - png.depth * (int(s % per) + 1))) & ((1 << png.depth) - 1);
  };
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      int v;
      if (png.color == 3) {
        const int idx = sample(y, size_t(x));
        if (paletted) {
          v = idx;
        } else {
          if (size_t(3 * idx + 2) >= png.palette.size()) fail("PNG palette index out of range: " + path);
          v = gray_of(png.palette[3 * idx], png.palette[3 * idx + 1], png.palette[3 * idx + 2]);
        }
      } else if (png.color == 0 || png.color == 4) {
        const int c = png.channels();
        const int s = sample(y, size_t(x) * c);
        v = png.depth == 16 ? s >> 8 : png.depth == 8 ? s : s * 255 / ((1 << png.depth) - 1);
      } else {
        const int c = png.channels();
        int rgb[3];
        for (int k = 0; k < 3; ++k) {
          const int s = sample(y, size_t(x) * c + k);
          rgb[k] = png.depth == 16 ? s >> 8 : s;
        }
        v = gray_of(rgb[0], rgb[1], rgb[2]);
      }
      out[size_t(y) * w + x] = uint8_t(v);
    }
  return out;
}

// ---- TIFF ----

struct Tiff {
  Bytes b;
  bool be = false;  // big-endian ("MM")
  struct Entry {
    uint16_t type;
    uint32_t count;
    uint32_t at;  // byte offset of the value(s)
  };
  std::map<uint16_t, Entry> tags;

  uint16_t u16(size_t o) const {
    if (o + 2 > b.size()) fail("truncated TIFF");
    return be ? uint16_t((b[o] << 8) | b[o + 1]) : uint16_t(b[o] | (b[o + 1] << 8));
  }
  uint32_t u32(size_t o) const {
    if (o + 4 > b.size()) fail("truncated TIFF");
    return be ? be32(&b[o]) : uint32_t(b[o] | (b[o + 1] << 8) | (b[o + 2] << 16) | (uint32_t(b[o + 3]) << 24));
  }
  static int type_size(uint16_t t) {
    switch (t) {
      case 1: case 2: case 6: case 7: return 1;
      case 3: case 8: return 2;
      case 4: case 9: case 11: return 4;
      case 5: case 10: case 12: return 8;
      default: return 0;
    }
  }
  bool has(uint16_t tag) const { return tags.count(tag) != 0; }
  // Integer value i of a BYTE / SHORT / LONG tag.
  uint32_t uint_at(uint16_t tag, uint32_t i = 0) const {
    if (!has(tag)) fail("TIFF tag " + std::to_string(tag) + " is missing");
    const Entry& e = tags.at(tag);
    if (i >= e.count) fail("TIFF tag " + std::to_string(tag) + " has too few values");
    if (e.type == 3) return u16(e.at + 2 * i);
    if (e.type == 4) return u32(e.at + 4 * i);
    if (e.type == 1) {
      if (size_t(e.at) + i >= b.size()) fail("truncated TIFF");
      return b[size_t(e.at) + i];
    }
    fail("TIFF tag " + std::to_string(tag) + " is not an integer");
  }
  uint32_t uint_or(uint16_t tag, uint32_t dflt) const { return has(tag) ? uint_at(tag) : dflt; }
  // A RATIONAL / FLOAT / DOUBLE / integer tag as float (libtiff hands these tags out as float).
  float real(uint16_t tag) const {
    if (!has(tag)) fail("TIFF tag " + std::to_string(tag) + " is missing");
    const Entry& e = tags.at(tag);
    if (e.type == 5) {
      const uint32_t num = u32(e.at), den = u32(e.at + 4);
      return den ? float(double(num) / double(den)) : 0.f;
    }
    if (e.type == 10) {
      const int32_t num = int32_t(u32(e.at)), den = int32_t(u32(e.at + 4));
      return den ? float(double(num) / double(den)) : 0.f;
    }
    if (e.type == 11) {
      const uint32_t v = u32(e.at);
      float f;
      std::memcpy(&f, &v, 4);
      return f;
    }
    if (e.type == 12) {
      const uint64_t v = (uint64_t(u32(e.at + (be ? 0 : 4))) << 32) | u32(e.at + (be ? 4 : 0));
      double d;
      std::memcpy(&d, &v, 8);
      return float(d);
    }
    return float(uint_at(tag));
  }
};

Tiff parse_tiff(const std::string& path) {
  Tiff t;
  t.b = read_file(path);
  if (t.b.size() < 8) fail("not a TIFF file: " + path);
  if (t.b[0] == 'I' && t.b[1] == 'I')
    t.be = false;
  else if (t.b[0] == 'M' && t.b[1] == 'M')
    t.be = true;
  else
    fail("not a TIFF file: " + path);
  if (t.u16(2) != 42) fail("not a classic TIFF file (BigTIFF is not supported): " + path, HMP_ERR_NOT_SUPPORTED);
  const uint32_t ifd = t.u32(4);
  const uint16_t n = t.u16(ifd);
  for (uint16_t i = 0; i < n; ++i) {
    const size_t e = ifd + 2 + 12 * size_t(i);
    Tiff::Entry en;
    const uint16_t tag = t.u16(e);
    en.type = t.u16(e + 2);
    en.count = t.u32(e + 4);
    const uint64_t bytes = uint64_t(Tiff::type_size(en.type)) * en.count;
    en.at = bytes <= 4 ? uint32_t(e + 8) : t.u32(e + 8);
    if (uint64_t(en.at) + bytes > t.b.size()) fail("TIFF tag data out of range: " + path);
    t.tags[tag] = en;
  }
  return t;
}

// TIFF LZW (compression 5): MSB-first codes of 9..12 bits, the width growing one code early.
Bytes lzw_decode(const uint8_t* p, size_t n, size_t expect) {
  Bytes out;
  out.reserve(expect);
  std::vector<std::pair<int, uint8_t>> table;  // (prefix code, last byte); codes 0..255 implicit
  std::vector<uint8_t> scratch;
  const auto emit = [&](int code) -> uint8_t {  // appends the string of `code`, returns its first byte
    scratch.clear();
    while (code >= 258) {
      const auto& e = table[size_t(code - 258)];
      scratch.push_back(e.second);
      code = e.first;
    }
    scratch.push_back(uint8_t(code));
    out.insert(out.end(), scratch.rbegin(), scratch.rend());
    return uint8_t(code);
  };
  size_t bitpos = 0;
  int width = 9, prev = -1;
  for (;;) {
    if (out.size() >= expect || bitpos + width > n * 8) break;  // nothing past the strip is used
    int code = 0;
    for (int k = 0; k < width; ++k, ++bitpos) code = (code << 1) | ((p[bitpos >> 3] >> (7 - (bitpos & 7))) & 1);
    if (code == 257) break;  // end of information
    if (code == 256) {       // clear
      table.clear();
      width = 9;
      prev = -1;
      continue;
    }
    const int next = 258 + int(table.size());
    if (prev < 0) {
      if (code > 255) fail("corrupt LZW data");
      emit(code);
    } else if (code < next) {
      const uint8_t first = emit(code);
      table.emplace_back(prev, first);
    } else if (code == next) {
      const uint8_t first = emit(prev);
      out.push_back(first);
      table.emplace_back(prev, first);
    } else {
      fail("corrupt LZW data");
    }
    prev = code;
    const int size = 258 + int(table.size());
    if (size + 1 >= (1 << width) && width < 12) ++width;
  }
  return out;
}

Bytes packbits_decode(const uint8_t* p, size_t n, size_t expect) {
  Bytes out;
  out.reserve(expect);
  size_t i = 0;
  while (i < n && out.size() < expect) {
    const int8_t c = int8_t(p[i++]);
    if (c >= 0) {
      const size_t k = size_t(c) + 1;
      if (i + k > n) fail("corrupt PackBits data");
      out.insert(out.end(), p + i, p + i + k);
      i += k;
    } else if (c != -128) {
      if (i >= n) fail("corrupt PackBits data");
      out.insert(out.end(), size_t(1 - c), p[i++]);
    }
  }
  return out;
}

// A single-channel 16-bit unsigned TIFF image (strips or tiles; none / LZW / Deflate / PackBits;
// horizontal predictor).
std::vector<uint16_t> read_tiff_u16(const std::string& path, int& w, int& h) {
  const Tiff t = parse_tiff(path);
  const uint32_t w32 = t.uint_at(256), h32 = t.uint_at(257);
  check_size(int64_t(w32), int64_t(h32), path);
  w = int(w32);
  h = int(h32);
  const uint32_t spp = t.uint_or(277, 1), bits = t.uint_or(258, 1), fmt = t.uint_or(339, 1);
  const uint32_t comp = t.uint_or(259, 1), pred = t.uint_or(317, 1);
  if (spp != 1 || bits != 16 || fmt != 1)
    fail("mapping tables must be single-channel 16-bit unsigned TIFF images: " + path, HMP_ERR_NOT_SUPPORTED);
  if (!(comp == 1 || comp == 5 || comp == 8 || comp == 32946 || comp == 32773))
    fail("unsupported TIFF compression " + std::to_string(comp) + ": " + path, HMP_ERR_NOT_SUPPORTED);
  if (pred != 1 && pred != 2) fail("unsupported TIFF predictor " + std::to_string(pred) + ": " + path, HMP_ERR_NOT_SUPPORTED);
  const bool tiled = t.has(322);
  const uint32_t bw32 = tiled ? t.uint_at(322) : uint32_t(w);
  const uint32_t bh32 = tiled ? t.uint_at(323) : std::min<uint32_t>(t.uint_or(278, uint32_t(h)), uint32_t(h));
  if (bw32 == 0 || bh32 == 0 || bw32 > uint32_t(kMaxSide) || bh32 > uint32_t(kMaxSide) ||
      uint64_t(bw32) * bh32 > uint64_t(kMaxPixels))
    fail("bad TIFF strip or tile size: " + path);
  const int bw = int(bw32), bh = int(bh32);
  const uint16_t off_tag = tiled ? 324 : 273, cnt_tag = tiled ? 325 : 279;
  const int across = (w + bw - 1) / bw, down = (h + bh - 1) / bh;
  const uint64_t nblocks = uint64_t(across) * uint64_t(down);
  if (!t.has(off_tag) || !t.has(cnt_tag) || t.tags.at(off_tag).count < nblocks || t.tags.at(cnt_tag).count < nblocks)
    fail("TIFF strip or tile table missing: " + path);
  std::vector<uint16_t> img(size_t(w) * h);
  for (uint32_t blk = 0; blk < uint32_t(nblocks); ++blk) {
    const int bx = int(blk % uint32_t(across)) * bw, by = int(blk / uint32_t(across)) * bh;
    const int rows = tiled ? bh : std::min(bh, h - by);  // a tile is stored whole; a strip is clipped
    const size_t expect = size_t(bw) * rows * 2;
    const uint32_t off = t.uint_at(off_tag, blk), cnt = t.uint_at(cnt_tag, blk);
    if (uint64_t(off) + cnt > t.b.size()) fail("TIFF data out of range: " + path);
    const uint8_t* src = t.b.data() + off;
    Bytes data;
    if (comp == 1)
      data.assign(src, src + std::min<size_t>(cnt, expect));
    else if (comp == 5)
      data = lzw_decode(src, cnt, expect);
    else if (comp == 32773)
      data = packbits_decode(src, cnt, expect);
    else
      data = zlib_inflate(src, cnt, expect);
    if (data.size() < expect) fail("TIFF strip or tile too short: " + path);
    for (int r = 0; r < rows; ++r) {
      uint16_t acc = 0;
      for (int c = 0; c < bw; ++c) {
        const uint8_t* q = &data[(size_t(r) * bw + c) * 2];
        uint16_t v = t.be ? uint16_t((q[0] << 8) | q[1]) : uint16_t(q[0] | (q[1] << 8));
        if (pred == 2) v = acc = uint16_t(acc + v);
        const int x = bx + c, y = by + r;
        if (x < w && y < h) img[size_t(y) * w + x] = v;
      }
    }
  }
  return img;
}

// Canvas position of a table: XPosition * XResolution (float, as libtiff returns both), snapped
// to the nearest integer within 1e-3.
void tiff_position(const std::string& path, float& x, float& y) {
  const Tiff t = parse_tiff(path);
  const auto get = [&](uint16_t tag) { return t.has(tag) ? t.real(tag) : 0.f; };
  const auto snap = [](float v) {
    const float r = std::nearbyint(v);
    return std::fabs(v - r) < 1e-3f ? r : v;
  };
  x = snap(get(286) * get(282));
  y = snap(get(287) * get(283));
}

}  // namespace

struct hmp_control_dir_impl {
  hmp_control_dir pub{};
  std::vector<std::vector<uint16_t>> maps;
  std::vector<uint8_t> seam;
};

extern "C" {

HMP_API hmp_status hmp_control_dir_load(const char* directory, int kind, int n_images, hmp_control_dir** out) {
  hmp_status s{};
  const auto make = [&](int code, const std::string& m) {
    s.code = code;
    std::snprintf(s.message, sizeof(s.message), "%s", m.c_str());
    return s;
  };
  if (!out || !directory) return make(HMP_ERR_INVALID_VALUE, "null argument");
  *out = nullptr;
  if (kind == HMP_KIND_PANO2) n_images = 2;
  if (kind == HMP_KIND_PANO3) n_images = 3;
  if (!(kind == HMP_KIND_PANO2 || kind == HMP_KIND_PANO3 || kind == HMP_KIND_PANON) || n_images < 2 || n_images > 8)
    return make(HMP_ERR_INVALID_VALUE, "kind must be HMP_KIND_PANO2 / PANO3 / PANON with 2..8 images");
  auto* d = new (std::nothrow) hmp_control_dir_impl;
  if (!d) return make(HMP_ERR_MEMORY_ALLOCATION, "out of host memory");
  try {
    std::string dir(directory);
    if (!dir.empty() && dir.back() != '/') dir += '/';
    d->maps.resize(size_t(2 * n_images));
    float px[8], py[8];
    for (int i = 0; i < n_images; ++i) {
      char stem[32];
      std::snprintf(stem, sizeof(stem), "mapping_%04d", i);
      int wx, hx, wy, hy;
      d->maps[2 * i] = read_tiff_u16(dir + stem + "_x.tif", wx, hx);
      d->maps[2 * i + 1] = read_tiff_u16(dir + stem + "_y.tif", wy, hy);
      if (wx != wy || hx != hy) fail(std::string("x and y tables differ in size: ") + dir + stem);
      d->pub.map_width[i] = wx;
      d->pub.map_height[i] = hx;
      d->pub.map_x[i] = d->maps[2 * i].data();
      d->pub.map_y[i] = d->maps[2 * i + 1].data();
      tiff_position(dir + stem + ".tif", px[i], py[i]);
    }
    const float min_x = *std::min_element(px, px + n_images), min_y = *std::min_element(py, py + n_images);
    for (int i = 0; i < n_images; ++i) {
      d->pub.xpos[i] = px[i] - min_x;
      d->pub.ypos[i] = py[i] - min_y;
    }
    int sw, sh;
    bool paletted;
    d->seam = read_seam_png(dir + "seam_file.png", sw, sh, paletted);
    std::set<int> uniq(d->seam.begin(), d->seam.end());
    if (kind == HMP_KIND_PANO2) {
      const uint8_t lo = uint8_t(*uniq.begin()), hi = uint8_t(*uniq.rbegin());
      for (uint8_t& v : d->seam) v = v == hi ? 0 : (v == lo ? 1 : v);
    } else if (kind == HMP_KIND_PANO3) {
      if (!paletted) fail("three-image seam must be an 8-bit paletted PNG: " + dir + "seam_file.png");
      if (uniq != std::set<int>{0, 1, 2}) fail("three-image seam labels must be exactly 0, 1, 2: " + dir + "seam_file.png");
    } else {
      if (int(uniq.size()) != n_images)
        fail("Seam mask classes (" + std::to_string(uniq.size()) + ") != n_images (" + std::to_string(n_images) +
             "): " + dir + "seam_file.png");
      uint8_t lut[256] = {};
      int k = 0;
      for (int v : uniq) lut[v] = uint8_t(k++);
      for (uint8_t& v : d->seam) v = lut[v];
    }
    d->pub.kind = kind;
    d->pub.n = n_images;
    d->pub.seam_width = sw;
    d->pub.seam_height = sh;
    d->pub.seam = d->seam.data();
  } catch (const LoadError& e) {
    delete d;
    return make(e.code, e.what());
  } catch (const std::bad_alloc&) {
    delete d;
    return make(HMP_ERR_MEMORY_ALLOCATION, "out of host memory");
  } catch (const std::exception& e) {
    delete d;
    return make(HMP_ERR_INVALID_VALUE, std::string("control directory: ") + e.what());
  }
  d->pub.internal = d;
  *out = &d->pub;
  return make(HMP_OK, "");
}

HMP_API void hmp_control_dir_free(hmp_control_dir* d) {
  if (d) delete static_cast<hmp_control_dir_impl*>(d->internal);
}

HMP_API hmp_status hmp_read_seam_png(const char* path, int* width, int* height, int* paletted, uint8_t* out,
                                     size_t capacity) {
  hmp_status s{};
  try {
    if (!path || !width || !height) fail("null argument");
    int w, h;
    bool pal;
    const std::vector<uint8_t> px = read_seam_png(path, w, h, pal);
    *width = w;
    *height = h;
    if (paletted) *paletted = pal ? 1 : 0;
    if (out) {
      if (capacity < px.size()) fail("output buffer too small");
      std::memcpy(out, px.data(), px.size());
    }
    s.code = HMP_OK;
  } catch (const LoadError& e) {
    s.code = e.code;
    std::snprintf(s.message, sizeof(s.message), "%s", e.what());
  } catch (const std::bad_alloc&) {
    s.code = HMP_ERR_MEMORY_ALLOCATION;
    std::snprintf(s.message, sizeof(s.message), "out of host memory");
  } catch (const std::exception& e) {
    s.code = HMP_ERR_INVALID_VALUE;
    std::snprintf(s.message, sizeof(s.message), "%s", e.what());
  }
  return s;
}

HMP_API hmp_status hmp_read_tiff_u16(const char* path, int* width, int* height, uint16_t* out, size_t capacity) {
  hmp_status s{};
  try {
    if (!path || !width || !height) fail("null argument");
    int w, h;
    const std::vector<uint16_t> px = read_tiff_u16(path, w, h);
    *width = w;
    *height = h;
    if (out) {
      if (capacity < px.size()) fail("output buffer too small");
      std::memcpy(out, px.data(), px.size() * 2);
    }
    s.code = HMP_OK;
  } catch (const LoadError& e) {
    s.code = e.code;
    std::snprintf(s.message, sizeof(s.message), "%s", e.what());
  } catch (const std::bad_alloc&) {
    s.code = HMP_ERR_MEMORY_ALLOCATION;
    std::snprintf(s.message, sizeof(s.message), "out of host memory");
  } catch (const std::exception& e) {
    s.code = HMP_ERR_INVALID_VALUE;
    std::snprintf(s.message, sizeof(s.message), "%s", e.what());
  }
  return s;
}

}  // extern "C"
