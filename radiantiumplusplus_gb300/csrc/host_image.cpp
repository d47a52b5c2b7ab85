// Image decoders (see host_image.h for the formats and conventions).
#include "host_image.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>

namespace rad {
namespace img {

namespace {

[[noreturn]] void Fail(const std::string& what) { throw std::runtime_error("image: " + what); }

// ------------------------------------------------------------------ inflate
// RFC 1951: LSB-first bit reader and canonical Huffman codes decoded by code
// length (count of codes per length, symbols in code order).
struct Bits {
  const uint8_t* p;
  size_t n, pos = 0;
  uint32_t buf = 0;
  int cnt = 0;
  uint32_t Get(int k) {
    while (cnt < k) {
      if (pos >= n) Fail("deflate stream truncated");
      buf |= (uint32_t)p[pos++] << cnt;
      cnt += 8;
    }
    uint32_t v = buf & ((1u << k) - 1u);
    buf >>= k;
    cnt -= k;
    return v;
  }
  void AlignByte() {
    buf = 0;
    cnt = 0;
  }
};

struct Huff {
  uint16_t count[16];
  uint16_t sym[320];
};

void BuildHuff(Huff& h, const uint8_t* lens, int n) {
  std::memset(h.count, 0, sizeof(h.count));
  for (int i = 0; i < n; i++) h.count[lens[i]]++;
  h.count[0] = 0;
  uint16_t offs[16];
  offs[1] = 0;
  int left = 1;
  for (int len = 1; len < 16; len++) {
    left = (left << 1) - h.count[len];
    if (left < 0) Fail("over-subscribed Huffman code");
    if (len < 15) offs[len + 1] = (uint16_t)(offs[len] + h.count[len]);
  }
  for (int i = 0; i < n; i++)
    if (lens[i]) h.sym[offs[lens[i]]++] = (uint16_t)i;
}

int Decode(Bits& b, const Huff& h) {
  int code = 0, first = 0, index = 0;
  for (int len = 1; len < 16; len++) {
    code |= (int)b.Get(1);
    int count = h.count[len];
    if (code - first < count) return h.sym[index + (code - first)];
    index += count;
    first = (first + count) << 1;
    code <<= 1;
  }
  Fail("bad Huffman code");
}

// RFC 1951 section 3.2.5 length / distance bases and extra bits
const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

void InflateBlock(Bits& b, std::vector<uint8_t>& out, const Huff& lit, const Huff& dist) {
  for (;;) {
    int s = Decode(b, lit);
    if (s < 256) {
      out.push_back((uint8_t)s);
    } else if (s == 256) {
      return;
    } else {
      s -= 257;
      if (s >= 29) Fail("bad length symbol");
      size_t len = kLenBase[s] + b.Get(kLenExtra[s]);
      int ds = Decode(b, dist);
      if (ds >= 30) Fail("bad distance symbol");
      size_t d = kDistBase[ds] + b.Get(kDistExtra[ds]);
      if (d > out.size()) Fail("distance beyond output");
      size_t from = out.size() - d;
      for (size_t i = 0; i < len; i++) out.push_back(out[from + i]);
    }
  }
}

}  // namespace

std::vector<uint8_t> Inflate(const uint8_t* data, size_t n, bool zlibHeader) {
  size_t start = 0;
  if (zlibHeader) {
    if (n < 2) Fail("zlib stream too short");
    if ((data[0] & 15) != 8 || ((data[0] << 8) | data[1]) % 31 != 0) Fail("bad zlib header");
    if (data[1] & 32) Fail("zlib preset dictionary");
    start = 2;
  }
  Bits b{data + start, n - start};
  std::vector<uint8_t> out;
  int last;
  do {
    last = (int)b.Get(1);
    int type = (int)b.Get(2);
    if (type == 0) {  // stored
      b.AlignByte();
      if (b.pos + 4 > b.n) Fail("stored block truncated");
      uint32_t len = b.p[b.pos] | (b.p[b.pos + 1] << 8);
      uint32_t nlen = b.p[b.pos + 2] | (b.p[b.pos + 3] << 8);
      if ((len ^ 0xffffu) != nlen) Fail("stored block length check");
      b.pos += 4;
      if (b.pos + len > b.n) Fail("stored block truncated");
      out.insert(out.end(), b.p + b.pos, b.p + b.pos + len);
      b.pos += len;
    } else if (type == 1) {  // fixed codes
      uint8_t lens[320];
      for (int i = 0; i < 144; i++) lens[i] = 8;
      for (int i = 144; i < 256; i++) lens[i] = 9;
      for (int i = 256; i < 280; i++) lens[i] = 7;
      for (int i = 280; i < 288; i++) lens[i] = 8;
      Huff lit, dist;
      BuildHuff(lit, lens, 288);
      for (int i = 0; i < 30; i++) lens[i] = 5;
      BuildHuff(dist, lens, 30);
      InflateBlock(b, out, lit, dist);
    } else if (type == 2) {  // dynamic codes
      int nlen = (int)b.Get(5) + 257, ndist = (int)b.Get(5) + 1, ncode = (int)b.Get(4) + 4;
      if (nlen > 286 || ndist > 30) Fail("bad dynamic block counts");
      static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
      uint8_t lens[320];
      std::memset(lens, 0, sizeof(lens));
      for (int i = 0; i < ncode; i++) lens[order[i]] = (uint8_t)b.Get(3);
      Huff lencode;
      BuildHuff(lencode, lens, 19);
      int idx = 0;
      while (idx < nlen + ndist) {
        int s = Decode(b, lencode);
        if (s < 16) {
          lens[idx++] = (uint8_t)s;
        } else {
          int rep;
          uint8_t val = 0;
          if (s == 16) {
            if (idx == 0) Fail("repeat with no previous length");
            val = lens[idx - 1];
            rep = 3 + (int)b.Get(2);
          } else if (s == 17) {
            rep = 3 + (int)b.Get(3);
          } else {
            rep = 11 + (int)b.Get(7);
          }
          if (idx + rep > nlen + ndist) Fail("too many code lengths");
          while (rep--) lens[idx++] = val;
        }
      }
      Huff lit, dist;
      BuildHuff(lit, lens, nlen);
      BuildHuff(dist, lens + nlen, ndist);
      InflateBlock(b, out, lit, dist);
    } else {
      Fail("bad deflate block type");
    }
  } while (!last);
  return out;
}

float HalfToFloat(uint16_t h) {
  uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
  uint32_t e = (h >> 10) & 31u, m = h & 1023u;
  uint32_t bits;
  if (e == 0) {
    if (m == 0) {
      bits = sign;
    } else {  // subnormal: normalise
      int shift = 0;
      while (!(m & 1024u)) {
        m <<= 1;
        shift++;
      }
      m &= 1023u;
      bits = sign | ((uint32_t)(127 - 15 + 1 - shift) << 23) | (m << 13);
    }
  } else if (e == 31) {
    bits = sign | 0x7f800000u | (m << 13);
  } else {
    bits = sign | ((e + 127 - 15) << 23) | (m << 13);
  }
  float f;
  std::memcpy(&f, &bits, 4);
  return f;
}

namespace {

// float -> binary16, round to nearest even (what a FLOAT channel read into a
// HALF frame buffer slice goes through)
uint16_t FloatToHalf(float f) {
  uint32_t x;
  std::memcpy(&x, &f, 4);
  uint32_t sign = (x >> 16) & 0x8000u;
  uint32_t ax = x & 0x7fffffffu;
  if (ax >= 0x7f800000u) return (uint16_t)(sign | 0x7c00u | (ax > 0x7f800000u ? 0x200u : 0u));
  if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);  // rounds to infinity
  if (ax < 0x38800000u) {                                    // subnormal or zero half
    if (ax < 0x33000000u) return (uint16_t)sign;
    // half subnormal = round(|f| * 2^24) = round(significand * 2^(e - 126))
    uint32_t e = ax >> 23;  // 102 .. 112
    uint32_t m = (ax & 0x7fffffu) | 0x800000u;
    int s = 126 - (int)e;  // 14 .. 24
    uint32_t r = m >> s;
    uint32_t rem = m & ((1u << s) - 1u), half = 1u << (s - 1);
    if (rem > half || (rem == half && (r & 1u))) r++;
    return (uint16_t)(sign | r);
  }
  uint32_t r = ((ax >> 13) - ((127 - 15) << 10));
  uint32_t rem = ax & 0x1fffu;
  if (rem > 0x1000u || (rem == 0x1000u && (r & 1u))) r++;
  return (uint16_t)(sign | r);
}

uint32_t BE32(const uint8_t* p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

// stbi__convert_format from n samples to req (1 or 3) samples per pixel.
void ConvertChannels(const std::vector<uint8_t>& in, int n, int req, size_t npx, std::vector<uint8_t>& out) {
  out.resize(npx * req);
  for (size_t i = 0; i < npx; i++) {
    const uint8_t* s = &in[i * n];
    uint8_t* d = &out[i * req];
    if (req == 3) {
      if (n <= 2) {
        d[0] = d[1] = d[2] = s[0];
      } else {
        d[0] = s[0];
        d[1] = s[1];
        d[2] = s[2];
      }
    } else {
      d[0] = n <= 2 ? s[0] : (uint8_t)(((int)s[0] * 77 + (int)s[1] * 150 + 29 * (int)s[2]) >> 8);
    }
  }
}

void FlipRows(uint8_t* p, int h, size_t rowBytes) {
  std::vector<uint8_t> tmp(rowBytes);
  for (int y = 0; y < h / 2; y++) {
    uint8_t* a = p + (size_t)y * rowBytes;
    uint8_t* b = p + (size_t)(h - 1 - y) * rowBytes;
    std::memcpy(tmp.data(), a, rowBytes);
    std::memcpy(a, b, rowBytes);
    std::memcpy(b, tmp.data(), rowBytes);
  }
}

// --------------------------------------------------------------------- PNG
int Paeth(int a, int b, int c) {
  int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
  if (pa <= pb && pa <= pc) return a;
  return pb <= pc ? b : c;
}

// Undo the per-row filters of one (sub-)image of w x h pixels; returns raw rows.
std::vector<uint8_t> Unfilter(const uint8_t* src, size_t avail, int w, int h, int bpp, size_t rowBytes, size_t& used) {
  size_t need = (size_t)h * (rowBytes + 1);
  if (avail < need) Fail("png image data truncated");
  std::vector<uint8_t> out((size_t)h * rowBytes);
  for (int y = 0; y < h; y++) {
    int f = src[(size_t)y * (rowBytes + 1)];
    const uint8_t* in = src + (size_t)y * (rowBytes + 1) + 1;
    uint8_t* cur = &out[(size_t)y * rowBytes];
    const uint8_t* prev = y ? &out[(size_t)(y - 1) * rowBytes] : nullptr;
    for (size_t i = 0; i < rowBytes; i++) {
      int a = i >= (size_t)bpp ? cur[i - bpp] : 0;
      int b = prev ? prev[i] : 0;
      int c = (prev && i >= (size_t)bpp) ? prev[i - bpp] : 0;
      int v;
      switch (f) {
        case 0: v = in[i]; break;
        case 1: v = in[i] + a; break;
        case 2: v = in[i] + b; break;
        case 3: v = in[i] + ((a + b) >> 1); break;
        case 4: v = in[i] + Paeth(a, b, c); break;
        default: Fail("bad png filter type");
      }
      cur[i] = (uint8_t)v;
    }
  }
  (void)w;
  used = need;
  return out;
}

Ldr DecodePng(const std::string& bytes, int req, bool flipY) {
  const uint8_t* p = (const uint8_t*)bytes.data();
  size_t n = bytes.size(), pos = 8;
  uint32_t w = 0, h = 0;
  int depth = 0, ctype = -1, interlace = 0;
  std::vector<uint8_t> idat, plte;
  bool seenEnd = false;
  while (pos + 8 <= n && !seenEnd) {
    uint32_t len = BE32(p + pos);
    std::string type((const char*)p + pos + 4, 4);
    if (pos + 12 + (size_t)len > n) Fail("png chunk truncated");
    const uint8_t* d = p + pos + 8;
    if (type == "IHDR") {
      if (len != 13) Fail("bad IHDR");
      w = BE32(d);
      h = BE32(d + 4);
      depth = d[8];
      ctype = d[9];
      if (d[10] != 0 || d[11] != 0) Fail("unknown png compression / filter method");
      interlace = d[12];
    } else if (type == "PLTE") {
      plte.assign(d, d + len);
    } else if (type == "IDAT") {
      idat.insert(idat.end(), d, d + len);
    } else if (type == "IEND") {
      seenEnd = true;
    } else if (!(type[0] & 0x20)) {
      Fail("unknown critical png chunk " + type);
    }
    pos += 12 + (size_t)len;
  }
  if (w == 0 || h == 0 || w > (1u << 24) || h > (1u << 24)) Fail("bad png size");
  int nch;
  switch (ctype) {
    case 0: nch = 1; break;
    case 2: nch = 3; break;
    case 3: nch = 1; break;
    case 4: nch = 2; break;
    case 6: nch = 4; break;
    default: Fail("bad png colour type");
  }
  bool okDepth = (depth == 8 || depth == 16) || ((ctype == 0 || ctype == 3) && (depth == 1 || depth == 2 || depth == 4));
  if (!okDepth || (ctype == 3 && depth == 16)) Fail("bad png bit depth");
  if (ctype == 3 && plte.empty()) Fail("png palette missing");
  std::vector<uint8_t> raw = Inflate(idat.data(), idat.size(), true);
  int bitsPx = nch * depth;
  int bpp = std::max(1, bitsPx / 8);
  int outN = ctype == 3 ? 3 : nch;  // palette expands to RGB (alpha is dropped by the conversion)
  std::vector<uint8_t> px((size_t)w * h * outN);
  auto store = [&](const std::vector<uint8_t>& rows, int sw, int sh, size_t rowBytes, int x0, int y0, int dx, int dy) {
    for (int y = 0; y < sh; y++) {
      const uint8_t* r = &rows[(size_t)y * rowBytes];
      for (int x = 0; x < sw; x++) {
        uint8_t* o = &px[(((size_t)(y0 + y * dy)) * w + (size_t)(x0 + x * dx)) * outN];
        if (depth < 8) {
          int bit = x * depth;
          int v = (r[bit >> 3] >> (8 - depth - (bit & 7))) & ((1 << depth) - 1);
          if (ctype == 3) {
            if ((size_t)v * 3 + 2 >= plte.size()) Fail("png palette index out of range");
            o[0] = plte[v * 3];
            o[1] = plte[v * 3 + 1];
            o[2] = plte[v * 3 + 2];
          } else {
            static const int scale[9] = {0, 0xff, 0x55, 0, 0x11, 0, 0, 0, 0x01};
            o[0] = (uint8_t)(v * scale[depth]);
          }
        } else if (ctype == 3) {
          int v = r[x];
          if ((size_t)v * 3 + 2 >= plte.size()) Fail("png palette index out of range");
          o[0] = plte[v * 3];
          o[1] = plte[v * 3 + 1];
          o[2] = plte[v * 3 + 2];
        } else {
          int step = depth / 8;
          for (int c = 0; c < nch; c++) o[c] = r[((size_t)x * nch + c) * step];  // 16-bit: high byte
        }
      }
    }
  };
  size_t off = 0;
  if (!interlace) {
    size_t rowBytes = ((size_t)w * bitsPx + 7) / 8, used;
    std::vector<uint8_t> rows = Unfilter(raw.data(), raw.size(), (int)w, (int)h, bpp, rowBytes, used);
    store(rows, (int)w, (int)h, rowBytes, 0, 0, 1, 1);
  } else {
    static const int xo[7] = {0, 4, 0, 2, 0, 1, 0}, yo[7] = {0, 0, 4, 0, 2, 0, 1};
    static const int xs[7] = {8, 8, 4, 4, 2, 2, 1}, ys[7] = {8, 8, 8, 4, 4, 2, 2};
    for (int k = 0; k < 7; k++) {
      int sw = ((int)w - xo[k] + xs[k] - 1) / xs[k], sh = ((int)h - yo[k] + ys[k] - 1) / ys[k];
      if (sw <= 0 || sh <= 0) continue;
      size_t rowBytes = ((size_t)sw * bitsPx + 7) / 8, used;
      std::vector<uint8_t> rows = Unfilter(raw.data() + off, raw.size() - off, sw, sh, bpp, rowBytes, used);
      store(rows, sw, sh, rowBytes, xo[k], yo[k], xs[k], ys[k]);
      off += used;
    }
  }
  Ldr out;
  out.width = (int)w;
  out.height = (int)h;
  out.channels = req;
  ConvertChannels(px, outN, req, (size_t)w * h, out.px);
  if (flipY) FlipRows(out.px.data(), out.height, (size_t)out.width * req);
  return out;
}

// --------------------------------------------------------------------- PNM
Ldr DecodePnm(const std::string& bytes, int req, bool flipY) {
  size_t pos = 2;
  auto token = [&]() {
    for (;;) {
      while (pos < bytes.size() && std::isspace((unsigned char)bytes[pos])) pos++;
      if (pos < bytes.size() && bytes[pos] == '#') {
        while (pos < bytes.size() && bytes[pos] != '\n') pos++;
        continue;
      }
      break;
    }
    long v = 0;
    int digits = 0;
    while (pos < bytes.size() && std::isdigit((unsigned char)bytes[pos])) {
      v = v * 10 + (bytes[pos++] - '0');
      if (++digits > 9) Fail("pnm number too long");
    }
    if (!digits) Fail("bad pnm header");
    return v;
  };
  int nch = bytes[1] == '6' ? 3 : 1;
  long w = token(), h = token(), maxv = token();
  if (maxv != 255) Fail("pnm maxval other than 255");
  pos++;  // one whitespace byte
  if (w <= 0 || h <= 0 || w > (1 << 24) || h > (1 << 24)) Fail("bad pnm size");
  size_t need = (size_t)w * h * nch;
  if (pos + need > bytes.size()) Fail("pnm data truncated");
  std::vector<uint8_t> px(bytes.begin() + pos, bytes.begin() + pos + need);
  Ldr out;
  out.width = (int)w;
  out.height = (int)h;
  out.channels = req;
  ConvertChannels(px, nch, req, (size_t)w * h, out.px);
  if (flipY) FlipRows(out.px.data(), out.height, (size_t)out.width * req);
  return out;
}

// -------------------------------------------------------------------- JPEG
// ITU-T T.81 Huffman JPEG: sequential (SOF0 / SOF1) and progressive (SOF2)
// scans, 8-bit samples, 1, 3 or 4 components, sampling factors 1..4 that
// divide the largest ones, restart intervals. The pixel pipeline restates the
// choices stb_image makes (stbi_load behind the image_default asset):
//  * coefficients are kept as 16-bit integers (progressive scans add their
//    successive-approximation bits to them), multiplied by the quantisation
//    table with 16-bit wrap-around;
//  * the inverse DCT is the integer "islow" factorisation of the Independent
//    JPEG Group (Loeffler-Ligtenberg-Moschytz rotations with constants rounded
//    to 12 fractional bits): columns first, rounded to keep 2 extra bits,
//    then rows with the 0.5 rounding and the +128 level shift folded into one
//    bias before the final shift by 17, clamped to 0..255;
//  * chroma planes subsampled 2x horizontally and/or vertically are upsampled
//    with the triangle filter (3/4 nearest + 1/4 next sample, centred between
//    samples; with both, a 3x3-weighted 2-D version rounded once), the rows
//    stepped so that output row y blends the chroma rows nearest y/2 - 1/4;
//    any other ratio replicates samples;
//  * YCbCr -> RGB in 20-bit fixed point with the constants 1.402, 0.71414,
//    0.34414, 1.772 rounded to 12 bits, the cb term of green truncated to its
//    high 16 bits; 3 components named 'R', 'G', 'B' (or an Adobe marker with
//    transform 0 and no JFIF marker) are RGB already; 4 components are CMYK
//    (Adobe transform 0) or YCCK (transform 2) combined with K by the rounded
//    product x * k / 255, else YCbCr with the fourth ignored;
//  * one requested channel is the Y plane itself for YCbCr files, the integer
//    luma (77 r + 150 g + 29 b) >> 8 otherwise.
struct JHuff {
  bool present = false;
  uint8_t fastLen[512];  // 9-bit lookahead: code length (0: longer code)
  uint8_t fastSym[512];
  int maxcode[18], valptr[17], mincode[17];
  uint8_t vals[256];
};

// T.81 C.2 / F.2.2.3: canonical codes from the counts per length.
void BuildJHuff(JHuff& h, const uint8_t* counts, const uint8_t* vals, int n) {
  std::memcpy(h.vals, vals, n);
  std::memset(h.fastLen, 0, sizeof(h.fastLen));
  int code = 0, k = 0;
  for (int l = 1; l <= 16; l++) {
    h.valptr[l] = k;
    h.mincode[l] = code;
    for (int i = 0; i < counts[l - 1]; i++, k++, code++) {
      if (l <= 9) {
        int first = code << (9 - l);
        for (int j = 0; j < (1 << (9 - l)); j++) {
          h.fastLen[first + j] = (uint8_t)l;
          h.fastSym[first + j] = vals[k];
        }
      }
    }
    h.maxcode[l] = counts[l - 1] ? code - 1 : -1;
    if (code > (1 << l)) Fail("jpeg: bad Huffman code lengths");
    code <<= 1;
  }
  h.present = true;
}

// Entropy-coded segment reader: MSB-first bits, 0xFF 0x00 stuffing removed; a
// marker ends the data (zeros are read after it).
struct JBits {
  const uint8_t* p;
  size_t n, pos;
  uint32_t buf = 0;
  int cnt = 0;
  int marker = -1;
  bool nomore = false;
  uint8_t Byte() { return pos < n ? p[pos++] : 0; }
  void Fill() {
    while (cnt <= 24) {
      uint32_t b = 0;
      if (!nomore) {
        b = Byte();
        if (b == 0xFF) {
          uint32_t c = Byte();
          while (c == 0xFF) c = Byte();
          if (c != 0) {
            marker = (int)c;
            nomore = true;
            b = 0;
          }
        }
      }
      buf |= b << (24 - cnt);
      cnt += 8;
    }
  }
  int Bits(int k) {
    if (k == 0) return 0;
    Fill();
    uint32_t v = buf >> (32 - k);
    buf <<= k;
    cnt -= k;
    return (int)v;
  }
  // EXTEND(RECEIVE(s)), T.81 F.2.2.1
  int Receive(int s) {
    int v = Bits(s);
    return v < (1 << (s - 1)) ? v - (1 << s) + 1 : v;
  }
  int Decode(const JHuff& h) {
    if (!h.present) Fail("jpeg: scan uses an undefined Huffman table");
    Fill();
    uint32_t look = buf >> 23;
    if (h.fastLen[look]) {
      int l = h.fastLen[look];
      buf <<= l;
      cnt -= l;
      return h.fastSym[look];
    }
    for (int l = 10; l <= 16; l++) {
      int code = (int)(buf >> (32 - l));
      if (code <= h.maxcode[l]) {
        buf <<= l;
        cnt -= l;
        return h.vals[h.valptr[l] + code - h.mincode[l]];
      }
    }
    Fail("jpeg: bad Huffman code");
  }
};

struct JComp {
  int id = 0, h = 1, v = 1, tq = 0, td = 0, ta = 0;
  int x = 0, y = 0;        // plane size in samples
  int bw = 0, bh = 0;      // blocks per row / column of the MCU-padded plane
  int dcPred = 0;
  std::vector<int16_t> coef;  // bw * bh blocks of 64, natural order
  std::vector<uint8_t> plane;  // bw * 8 x bh * 8 samples
};

// zigzag index -> natural (row-major) index, T.81 figure A.6
struct JZigzag {
  uint8_t nat[64];
  JZigzag() {
    int k = 0;
    for (int s = 0; s < 15; s++) {
      int lo = s > 7 ? s - 7 : 0, hi = s < 7 ? s : 7;
      if (s & 1) {
        for (int r = lo; r <= hi; r++) nat[k++] = (uint8_t)(r * 8 + (s - r));
      } else {
        for (int r = hi; r >= lo; r--) nat[k++] = (uint8_t)(r * 8 + (s - r));
      }
    }
  }
};
const JZigzag kZz;

inline int F2F(float x) { return (int)(x * 4096.f + 0.5f); }

// One 1-D pass of the islow IDCT on s0..s7 (frequency order); outputs the even
// part x0..x3 and the odd part t0..t3 (outputs i and 7 - i are x_i +- t_(3-i)).
inline void Idct1D(int s0, int s1, int s2, int s3, int s4, int s5, int s6, int s7, int& x0, int& x1, int& x2,
                   int& x3, int& t0, int& t1, int& t2, int& t3) {
  int p2 = s2, p3 = s6;
  int p1 = (p2 + p3) * F2F(0.5411961f);
  t2 = p1 + p3 * F2F(-1.847759065f);
  t3 = p1 + p2 * F2F(0.765366865f);
  p2 = s0;
  p3 = s4;
  t0 = (p2 + p3) * 4096;
  t1 = (p2 - p3) * 4096;
  x0 = t0 + t3;
  x3 = t0 - t3;
  x1 = t1 + t2;
  x2 = t1 - t2;
  t0 = s7;
  t1 = s5;
  t2 = s3;
  t3 = s1;
  p3 = t0 + t2;
  int p4 = t1 + t3;
  p1 = t0 + t3;
  p2 = t1 + t2;
  int p5 = (p3 + p4) * F2F(1.175875602f);
  t0 = t0 * F2F(0.298631336f);
  t1 = t1 * F2F(2.053119869f);
  t2 = t2 * F2F(3.072711026f);
  t3 = t3 * F2F(1.501321110f);
  p1 = p5 + p1 * F2F(-0.899976223f);
  p2 = p5 + p2 * F2F(-2.562915447f);
  p3 = p3 * F2F(-1.961570560f);
  p4 = p4 * F2F(-0.390180644f);
  t3 += p1 + p4;
  t2 += p2 + p3;
  t1 += p2 + p4;
  t0 += p1 + p3;
}

inline uint8_t Clamp255(int v) { return (uint8_t)(v < 0 ? 0 : v > 255 ? 255 : v); }

// Dequantised block d (natural order) -> 8 x 8 samples at out (row stride).
void IdctBlock(const int16_t* d, uint8_t* out, int stride) {
  int val[64];
  for (int c = 0; c < 8; c++) {  // columns, keeping 2 extra bits
    int x0, x1, x2, x3, t0, t1, t2, t3;
    Idct1D(d[c], d[c + 8], d[c + 16], d[c + 24], d[c + 32], d[c + 40], d[c + 48], d[c + 56], x0, x1, x2, x3, t0, t1,
           t2, t3);
    x0 += 512;
    x1 += 512;
    x2 += 512;
    x3 += 512;
    val[c] = (x0 + t3) >> 10;
    val[c + 56] = (x0 - t3) >> 10;
    val[c + 8] = (x1 + t2) >> 10;
    val[c + 48] = (x1 - t2) >> 10;
    val[c + 16] = (x2 + t1) >> 10;
    val[c + 40] = (x2 - t1) >> 10;
    val[c + 24] = (x3 + t0) >> 10;
    val[c + 32] = (x3 - t0) >> 10;
  }
  for (int r = 0; r < 8; r++) {  // rows: remove 12 + 2 + 3 bits, round, shift the level by 128
    const int* v = val + 8 * r;
    int x0, x1, x2, x3, t0, t1, t2, t3;
    Idct1D(v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], x0, x1, x2, x3, t0, t1, t2, t3);
    const int bias = 65536 + (128 << 17);
    x0 += bias;
    x1 += bias;
    x2 += bias;
    x3 += bias;
    uint8_t* o = out + (size_t)r * stride;
    o[0] = Clamp255((x0 + t3) >> 17);
    o[7] = Clamp255((x0 - t3) >> 17);
    o[1] = Clamp255((x1 + t2) >> 17);
    o[6] = Clamp255((x1 - t2) >> 17);
    o[2] = Clamp255((x2 + t1) >> 17);
    o[5] = Clamp255((x2 - t1) >> 17);
    o[3] = Clamp255((x3 + t0) >> 17);
    o[4] = Clamp255((x3 - t0) >> 17);
  }
}

struct JpegDecoder {
  const uint8_t* b;
  size_t n, pos = 2;
  uint16_t q[4][64] = {};  // natural order
  bool qSet[4] = {};
  JHuff dc[4], ac[4];
  std::vector<JComp> comp;
  int X = 0, Y = 0, hmax = 1, vmax = 1, mcux = 0, mcuy = 0;
  bool progressive = false, frame = false, jfif = false;
  int rgbIds = 0, adobe = -1, restart = 0;
  int eobrun = 0;

  uint8_t U8() {
    if (pos >= n) Fail("jpeg: truncated");
    return b[pos++];
  }
  int U16() {
    int hi = U8();
    return (hi << 8) | U8();
  }
  // the next marker: 0xFF then any fill 0xFF bytes; -1 when the byte is not 0xFF
  int Marker() {
    if (pos >= n) Fail("jpeg: no EOI marker");
    if (b[pos] != 0xFF) {
      pos++;
      return -1;
    }
    while (pos < n && b[pos] == 0xFF) pos++;
    return U8();
  }

  void Frame(int m) {
    if (frame) Fail("jpeg: more than one frame");
    frame = true;
    progressive = m == 0xC2;
    int L = U16();
    if (U8() != 8) Fail("jpeg: only 8-bit samples are supported");
    Y = U16();
    X = U16();
    if (Y == 0) Fail("jpeg: no height in the frame header (DNL is not supported)");
    if (X == 0) Fail("jpeg: zero width");
    int nf = U8();
    if (nf != 1 && nf != 3 && nf != 4) Fail("jpeg: 1, 3 or 4 components are supported");
    if (L != 8 + 3 * nf) Fail("jpeg: bad frame header length");
    comp.resize(nf);
    for (int i = 0; i < nf; i++) {
      JComp& c = comp[i];
      c.id = U8();
      int hv = U8();
      c.h = hv >> 4;
      c.v = hv & 15;
      c.tq = U8();
      if (c.h < 1 || c.h > 4 || c.v < 1 || c.v > 4) Fail("jpeg: bad sampling factors");
      if (c.tq > 3) Fail("jpeg: bad quantisation table index");
      if (nf == 3 && c.id == "RGB"[i]) rgbIds++;
      hmax = std::max(hmax, c.h);
      vmax = std::max(vmax, c.v);
    }
    if ((size_t)X * Y * nf > ((size_t)1 << 30)) Fail("jpeg: image too large");
    for (JComp& c : comp)
      if (hmax % c.h || vmax % c.v) Fail("jpeg: sampling factors must divide the largest ones");
    mcux = (X + hmax * 8 - 1) / (hmax * 8);
    mcuy = (Y + vmax * 8 - 1) / (vmax * 8);
    for (JComp& c : comp) {
      c.x = (X * c.h + hmax - 1) / hmax;
      c.y = (Y * c.v + vmax - 1) / vmax;
      c.bw = mcux * c.h;
      c.bh = mcuy * c.v;
      c.coef.assign((size_t)c.bw * c.bh * 64, 0);
    }
  }

  void Tables(int m) {
    int L = U16() - 2;
    if (m == 0xDB) {  // DQT
      while (L > 0) {
        int pq = U8(), t = pq & 15, p = pq >> 4;
        if (p > 1 || t > 3) Fail("jpeg: bad DQT");
        for (int i = 0; i < 64; i++) q[t][kZz.nat[i]] = (uint16_t)(p ? U16() : U8());
        qSet[t] = true;
        L -= p ? 129 : 65;
      }
    } else if (m == 0xC4) {  // DHT
      while (L > 0) {
        int tc = U8(), th = tc & 15;
        tc >>= 4;
        if (tc > 1 || th > 3) Fail("jpeg: bad DHT");
        uint8_t counts[16], vals[256];
        int total = 0;
        for (int i = 0; i < 16; i++) total += counts[i] = U8();
        if (total > 256) Fail("jpeg: bad DHT");
        for (int i = 0; i < total; i++) vals[i] = U8();
        BuildJHuff(tc ? ac[th] : dc[th], counts, vals, total);
        L -= 17 + total;
      }
    }
    if (L != 0) Fail("jpeg: bad table segment length");
  }

  void Skip(int m) {
    int L = U16();
    if (L < 2 || pos + (size_t)(L - 2) > n) Fail("jpeg: bad segment length");
    const uint8_t* s = b + pos;
    if (m == 0xE0 && L >= 7 && std::memcmp(s, "JFIF\0", 5) == 0) jfif = true;
    if (m == 0xEE && L >= 14 && std::memcmp(s, "Adobe\0", 6) == 0) adobe = s[11];
    pos += L - 2;
  }

  // T.81 G.1.2: one block of a scan into the coefficients c (zigzag band ss..se).
  void DecodeBlock(JBits& r, JComp& c, int16_t* d, int ss, int se, int ah, int al) {
    if (!progressive) {
      std::memset(d, 0, 64 * sizeof(int16_t));
      int t = r.Decode(dc[c.td]);
      if (t > 15) Fail("jpeg: bad DC code");
      c.dcPred += t ? r.Receive(t) : 0;
      d[0] = (int16_t)c.dcPred;
      for (int k = 1; k < 64;) {
        int rs = r.Decode(ac[c.ta]), s = rs & 15, run = rs >> 4;
        if (s == 0) {
          if (rs != 0xF0) break;
          k += 16;
        } else {
          k += run;
          if (k > 63) Fail("jpeg: AC run past the block");
          d[kZz.nat[k++]] = (int16_t)r.Receive(s);
        }
      }
      return;
    }
    if (ss == 0) {  // DC scans
      if (ah == 0) {
        std::memset(d, 0, 64 * sizeof(int16_t));
        int t = r.Decode(dc[c.td]);
        if (t > 15) Fail("jpeg: bad DC code");
        c.dcPred += t ? r.Receive(t) : 0;
        d[0] = (int16_t)(c.dcPred * (1 << al));
      } else if (r.Bits(1)) {
        d[0] = (int16_t)(d[0] + (1 << al));
      }
      return;
    }
    if (ah == 0) {  // first AC scan of a band
      if (eobrun > 0) {
        eobrun--;
        return;
      }
      for (int k = ss; k <= se;) {
        int rs = r.Decode(ac[c.ta]), s = rs & 15, run = rs >> 4;
        if (s == 0) {
          if (run < 15) {
            eobrun = (1 << run) - 1 + r.Bits(run);
            break;
          }
          k += 16;
        } else {
          k += run;
          if (k > 63) Fail("jpeg: AC run past the block");
          d[kZz.nat[k++]] = (int16_t)(r.Receive(s) * (1 << al));
        }
      }
      return;
    }
    // AC refinement (T.81 G.1.2.3): one correction bit per nonzero coefficient
    // passed, new coefficients of magnitude 1 << al placed after `run` zeros
    const int16_t bit = (int16_t)(1 << al);
    auto refine = [&](int16_t& v) {
      if (r.Bits(1) && (v & bit) == 0) v = (int16_t)(v > 0 ? v + bit : v - bit);
    };
    if (eobrun > 0) {
      eobrun--;
      for (int k = ss; k <= se; k++) {
        int16_t& v = d[kZz.nat[k]];
        if (v != 0) refine(v);
      }
      return;
    }
    int k = ss;
    do {
      int rs = r.Decode(ac[c.ta]), s = rs & 15, run = rs >> 4;
      int16_t val = 0;
      if (s == 0) {
        if (run < 15) {
          eobrun = (1 << run) - 1 + r.Bits(run);
          run = 64;  // the rest of the band only refines
        }              // else 15 zeros and a zero "coefficient": 16 zeros
      } else {
        if (s != 1) Fail("jpeg: bad AC refinement code");
        val = r.Bits(1) ? bit : (int16_t)-bit;
      }
      while (k <= se) {
        int16_t& v = d[kZz.nat[k++]];
        if (v != 0) {
          refine(v);
        } else {
          if (run == 0) {
            v = val;
            break;
          }
          run--;
        }
      }
    } while (k <= se);
  }

  void Scan() {
    int L = U16();
    int ns = U8();
    if (ns < 1 || ns > 4 || ns > (int)comp.size() || L != 6 + 2 * ns) Fail("jpeg: bad scan header");
    std::vector<JComp*> sc;
    for (int i = 0; i < ns; i++) {
      int id = U8(), tt = U8();
      JComp* c = nullptr;
      for (JComp& k : comp)
        if (k.id == id) c = &k;
      if (!c) Fail("jpeg: scan names an unknown component");
      c->td = tt >> 4;
      c->ta = tt & 15;
      if (c->td > 3 || c->ta > 3) Fail("jpeg: bad Huffman table index");
      sc.push_back(c);
    }
    int ss = U8(), se = U8(), a = U8(), ah = a >> 4, al = a & 15;
    if (progressive) {
      if (ss > 63 || se > 63 || ss > se || ah > 13 || al > 13) Fail("jpeg: bad progressive scan");
      if ((ss == 0) != (se == 0)) Fail("jpeg: a scan mixes DC and AC coefficients");
      if (ss > 0 && ns != 1) Fail("jpeg: AC scans have one component");
    } else {
      if (ss != 0 || ah != 0 || al != 0) Fail("jpeg: bad sequential scan");
      se = 63;
    }
    JBits r{b, n, pos};
    int todo = restart ? restart : 0x7fffffff;
    auto reset = [&]() {
      r.buf = 0;
      r.cnt = 0;
      r.marker = -1;
      r.nomore = false;
      for (JComp* c : sc) c->dcPred = 0;
      eobrun = 0;
      todo = restart ? restart : 0x7fffffff;
    };
    reset();
    // the segment's remaining bytes (padding bits) up to its marker
    auto drain = [&]() {
      while (r.marker < 0 && r.pos < r.n) {
        r.buf = 0;
        r.cnt = 0;
        r.Fill();
      }
    };
    // false: the segment ended without its restart marker (the scan stops)
    auto step = [&]() {
      if (--todo > 0) return true;
      drain();
      if (r.marker < 0xD0 || r.marker > 0xD7) return false;
      reset();
      return true;
    };
    bool more = true;
    if (ns == 1) {  // non-interleaved: the component's own block grid
      JComp& c = *sc[0];
      int w = (c.x + 7) >> 3, h = (c.y + 7) >> 3;
      for (int j = 0; j < h && more; j++)
        for (int i = 0; i < w && more; i++) {
          DecodeBlock(r, c, &c.coef[((size_t)j * c.bw + i) * 64], ss, se, ah, al);
          more = step();
        }
    } else {
      for (int j = 0; j < mcuy && more; j++)
        for (int i = 0; i < mcux && more; i++) {
          for (JComp* c : sc)
            for (int y = 0; y < c->v; y++)
              for (int x = 0; x < c->h; x++) {
                size_t blk = (size_t)(j * c->v + y) * c->bw + (i * c->h + x);
                DecodeBlock(r, *c, &c->coef[blk * 64], ss, se, ah, al);
              }
          more = step();
        }
    }
    drain();
    pos = r.pos;
    if (r.marker >= 0) pendingMarker = r.marker;
  }
  int pendingMarker = -1;

  void Decode() {
    if (n < 2 || b[0] != 0xFF || b[1] != 0xD8) Fail("jpeg: no SOI marker");
    for (;;) {
      int m;
      if (pendingMarker >= 0) {
        m = pendingMarker;
        pendingMarker = -1;
      } else {
        m = Marker();
        if (m < 0) continue;  // padding between segments
      }
      if (m == 0xD9) break;  // EOI
      if (m == 0xC0 || m == 0xC1 || m == 0xC2) {
        Frame(m);
      } else if (m >= 0xC3 && m <= 0xCF && m != 0xC4 && m != 0xC8 && m != 0xCC) {
        Fail("jpeg: only Huffman baseline / extended / progressive frames are supported");
      } else if (m == 0xDB || m == 0xC4) {
        Tables(m);
      } else if (m == 0xDD) {
        if (U16() != 4) Fail("jpeg: bad DRI length");
        restart = U16();
      } else if (m == 0xDA) {
        if (!frame) Fail("jpeg: scan before the frame header");
        Scan();
      } else if ((m >= 0xE0 && m <= 0xEF) || m == 0xFE) {
        Skip(m);
      } else if (m >= 0xD0 && m <= 0xD7) {
        // a stray restart marker between segments
      } else {
        Fail("jpeg: unknown marker");
      }
    }
    if (!frame) Fail("jpeg: no frame header");
    for (JComp& c : comp) {  // dequantise (16-bit wrap) and transform every block
      if (!qSet[c.tq]) Fail("jpeg: undefined quantisation table");
      c.plane.assign((size_t)c.bw * 8 * c.bh * 8, 0);
      const uint16_t* qt = q[c.tq];
      int16_t blk[64];
      for (int j = 0; j < c.bh; j++)
        for (int i = 0; i < c.bw; i++) {
          const int16_t* d = &c.coef[((size_t)j * c.bw + i) * 64];
          for (int k = 0; k < 64; k++) blk[k] = (int16_t)(d[k] * qt[k]);
          IdctBlock(blk, &c.plane[(size_t)j * 8 * c.bw * 8 + (size_t)i * 8], c.bw * 8);
        }
    }
  }
};

inline uint8_t Div4(int x) { return (uint8_t)(x >> 2); }
inline uint8_t Div16(int x) { return (uint8_t)(x >> 4); }
inline uint8_t Blinn(int x, int y) {  // x * y / 255, rounded
  unsigned t = (unsigned)(x * y + 128);
  return (uint8_t)((t + (t >> 8)) >> 8);
}
inline uint8_t LumaY(int r, int g, int b) { return (uint8_t)((r * 77 + g * 150 + 29 * b) >> 8); }

// One output row of a component plane at hs x vs subsampling (w input samples).
const uint8_t* Upsample(uint8_t* out, const uint8_t* nearRow, const uint8_t* farRow, int w, int hs, int vs) {
  if (hs == 1 && vs == 1) return nearRow;
  if (hs == 1 && vs == 2) {
    for (int i = 0; i < w; i++) out[i] = Div4(3 * nearRow[i] + farRow[i] + 2);
  } else if (hs == 2 && vs == 1) {
    const uint8_t* in = nearRow;
    if (w == 1) {
      out[0] = out[1] = in[0];
      return out;
    }
    out[0] = in[0];
    out[1] = Div4(in[0] * 3 + in[1] + 2);
    int i = 1;
    for (; i < w - 1; i++) {
      int c = 3 * in[i] + 2;
      out[2 * i] = Div4(c + in[i - 1]);
      out[2 * i + 1] = Div4(c + in[i + 1]);
    }
    out[2 * i] = Div4(in[w - 2] * 3 + in[w - 1] + 2);  // stb's last pair: 3/4 of the left sample (kept)
    out[2 * i + 1] = in[w - 1];
  } else if (hs == 2 && vs == 2) {
    if (w == 1) {
      out[0] = out[1] = Div4(3 * nearRow[0] + farRow[0] + 2);
      return out;
    }
    int t1 = 3 * nearRow[0] + farRow[0];
    out[0] = Div4(t1 + 2);
    for (int i = 1; i < w; i++) {
      int t0 = t1;
      t1 = 3 * nearRow[i] + farRow[i];
      out[2 * i - 1] = Div16(3 * t0 + t1 + 8);
      out[2 * i] = Div16(3 * t1 + t0 + 8);
    }
    out[2 * w - 1] = Div4(t1 + 2);
  } else {
    for (int i = 0; i < w; i++)
      for (int j = 0; j < hs; j++) out[i * hs + j] = nearRow[i];
  }
  return out;
}

void YCbCrRow(uint8_t* out, const uint8_t* y, const uint8_t* cb, const uint8_t* cr, int count) {
  const int kCr = F2F(1.40200f) << 8, kCrG = F2F(0.71414f) << 8, kCbG = F2F(0.34414f) << 8,
            kCb = F2F(1.77200f) << 8;
  for (int i = 0; i < count; i++) {
    int yf = (y[i] << 20) + (1 << 19);
    int vr = cr[i] - 128, vb = cb[i] - 128;
    int r = yf + vr * kCr;
    int g = (int)((uint32_t)(yf + vr * -kCrG) + ((uint32_t)(vb * -kCbG) & 0xffff0000u));
    int b = yf + vb * kCb;
    out[3 * i] = Clamp255(r >> 20);
    out[3 * i + 1] = Clamp255(g >> 20);
    out[3 * i + 2] = Clamp255(b >> 20);
  }
}

Ldr DecodeJpeg(const std::string& bytes, int req, bool flipY) {
  JpegDecoder z;
  z.b = (const uint8_t*)bytes.data();
  z.n = bytes.size();
  z.Decode();
  const int nc = (int)z.comp.size();
  const bool isRgb = nc == 3 && (z.rgbIds == 3 || (z.adobe == 0 && !z.jfif));
  const int decodeN = (nc == 3 && req < 3 && !isRgb) ? 1 : nc;
  struct Line {
    const uint8_t *l0, *l1;
    int hs, vs, ystep, ypos, wl;
    std::vector<uint8_t> buf;
  };
  std::vector<Line> ln(decodeN);
  for (int k = 0; k < decodeN; k++) {
    const JComp& c = z.comp[k];
    Line& L = ln[k];
    L.hs = z.hmax / c.h;
    L.vs = z.vmax / c.v;
    L.ystep = L.vs >> 1;
    L.ypos = 0;
    L.wl = (z.X + L.hs - 1) / L.hs;
    L.l0 = L.l1 = c.plane.data();
    L.buf.resize((size_t)z.X + 3);
  }
  Ldr out;
  out.width = z.X;
  out.height = z.Y;
  out.channels = req;
  out.px.resize((size_t)z.X * z.Y * req);
  std::vector<uint8_t> rgb((size_t)z.X * 3);
  const uint8_t* co[4] = {};
  for (int j = 0; j < z.Y; j++) {
    for (int k = 0; k < decodeN; k++) {
      Line& L = ln[k];
      bool bot = L.ystep >= (L.vs >> 1);
      co[k] = Upsample(L.buf.data(), bot ? L.l1 : L.l0, bot ? L.l0 : L.l1, L.wl, L.hs, L.vs);
      if (++L.ystep >= L.vs) {
        L.ystep = 0;
        L.l0 = L.l1;
        if (++L.ypos < z.comp[k].y) L.l1 += (size_t)z.comp[k].bw * 8;
      }
    }
    uint8_t* o = &out.px[(size_t)j * z.X * req];
    if (req == 3) {
      if (nc == 3) {
        if (isRgb) {
          for (int i = 0; i < z.X; i++) {
            o[3 * i] = co[0][i];
            o[3 * i + 1] = co[1][i];
            o[3 * i + 2] = co[2][i];
          }
        } else {
          YCbCrRow(o, co[0], co[1], co[2], z.X);
        }
      } else if (nc == 4) {
        if (z.adobe == 0) {  // CMYK
          for (int i = 0; i < z.X; i++) {
            int m = co[3][i];
            o[3 * i] = Blinn(co[0][i], m);
            o[3 * i + 1] = Blinn(co[1][i], m);
            o[3 * i + 2] = Blinn(co[2][i], m);
          }
        } else if (z.adobe == 2) {  // YCCK
          YCbCrRow(o, co[0], co[1], co[2], z.X);
          for (int i = 0; i < z.X; i++) {
            int m = co[3][i];
            for (int c = 0; c < 3; c++) o[3 * i + c] = Blinn(255 - o[3 * i + c], m);
          }
        } else {  // YCbCr, the fourth component ignored
          YCbCrRow(o, co[0], co[1], co[2], z.X);
        }
      } else {
        for (int i = 0; i < z.X; i++) o[3 * i] = o[3 * i + 1] = o[3 * i + 2] = co[0][i];
      }
    } else {
      if (isRgb) {
        for (int i = 0; i < z.X; i++) o[i] = LumaY(co[0][i], co[1][i], co[2][i]);
      } else if (nc == 4 && z.adobe == 0) {
        for (int i = 0; i < z.X; i++) {
          int m = co[3][i];
          o[i] = LumaY(Blinn(co[0][i], m), Blinn(co[1][i], m), Blinn(co[2][i], m));
        }
      } else if (nc == 4 && z.adobe == 2) {
        for (int i = 0; i < z.X; i++) o[i] = Blinn(255 - co[0][i], co[3][i]);
      } else {
        for (int i = 0; i < z.X; i++) o[i] = co[0][i];
      }
    }
  }
  if (flipY) FlipRows(out.px.data(), out.height, (size_t)out.width * req);
  return out;
}

bool IsJpeg(const std::string& b) { return b.size() >= 3 && (uint8_t)b[0] == 0xFF && (uint8_t)b[1] == 0xD8 && (uint8_t)b[2] == 0xFF; }

// ---------------------------------------------------------------------- BMP
// Windows / OS2 bitmaps as stb_image reads them: BITMAPCOREHEADER (12 bytes)
// and the 40 / 56 / 108 / 124-byte info headers, 1 / 4 / 8-bit palettes,
// 24-bit BGR, 16 / 32-bit pixels through channel masks (BI_RGB defaults 5-5-5 and
// 8-8-8-8, or BI_BITFIELDS), each field widened to 8 bits by bit replication;
// rows are bottom-up unless the height is negative. RLE compression is refused.
// A 32-bit image whose alpha field is zero everywhere reads as opaque.
uint32_t LE32(const uint8_t* p) { return p[0] | (p[1] << 8) | (p[2] << 16) | ((uint32_t)p[3] << 24); }
int LE16(const uint8_t* p) { return p[0] | (p[1] << 8); }

int HighBit(uint32_t z) {
  int n = -1;
  while (z) {
    n++;
    z >>= 1;
  }
  return n;
}
int BitCount(uint32_t a) {
  int n = 0;
  for (; a; a &= a - 1) n++;
  return n;
}
// the field (v & mask) >> shift, `bits` wide, widened to 8 bits by replicating its bits
int MaskField(uint32_t v, uint32_t mask, int shift, int bits) {
  if (!mask) return 0;
  v &= mask;
  if (shift < 0)
    v <<= -shift;
  else
    v >>= shift;
  if (bits >= 8) return (int)(v & 255);
  v >>= 8 - bits;  // the field's top `bits` bits of the 8-bit window
  int r = 0;
  for (int got = 0; got < 8; got += bits) r = (r << bits) | (int)v;  // replicate ...
  int total = ((8 + bits - 1) / bits) * bits;
  return r >> (total - 8);  // ... and keep the top 8 bits
}

Ldr DecodeBmp(const std::string& bytes, int req, bool flipY) {
  const uint8_t* b = (const uint8_t*)bytes.data();
  size_t n = bytes.size();
  if (n < 26) Fail("bmp: truncated header");
  uint32_t offset = LE32(b + 10), hsz = LE32(b + 14);
  if (hsz != 12 && hsz != 40 && hsz != 56 && hsz != 108 && hsz != 124) Fail("bmp: unknown header size");
  if (14 + (size_t)hsz > n) Fail("bmp: truncated header");
  const uint8_t* h = b + 14;
  int64_t w, ht;
  int bpp;
  uint32_t compress = 0, mr = 0, mg = 0, mb = 0, ma = 0;
  if (hsz == 12) {
    w = LE16(h + 4);
    ht = LE16(h + 6);
    bpp = LE16(h + 10);
  } else {
    w = (int32_t)LE32(h + 4);
    ht = (int32_t)LE32(h + 8);
    bpp = LE16(h + 14);
    compress = LE32(h + 16);
  }
  if (LE16(h + (hsz == 12 ? 8 : 12)) != 1) Fail("bmp: planes must be 1");
  bool topDown = ht < 0;
  if (topDown) ht = -ht;
  if (w <= 0 || ht <= 0 || w > (1 << 24) || ht > (1 << 24)) Fail("bmp: bad size");
  if (compress == 1 || compress == 2) Fail("bmp: RLE compression is not supported");
  if (compress != 0 && compress != 3) Fail("bmp: unsupported compression");
  size_t extra = 14 + hsz;
  if (bpp == 16 || bpp == 32) {
    if (compress == 0) {
      if (bpp == 32) {
        mr = 0xffu << 16;
        mg = 0xffu << 8;
        mb = 0xffu;
        ma = 0xffu << 24;
      } else {
        mr = 31u << 10;
        mg = 31u << 5;
        mb = 31u;
      }
    } else if (hsz == 40) {  // BI_BITFIELDS: three masks follow the header
      if (extra + 12 > n) Fail("bmp: truncated masks");
      mr = LE32(b + extra);
      mg = LE32(b + extra + 4);
      mb = LE32(b + extra + 8);
      extra += 12;
      if (mr == mg && mg == mb) Fail("bmp: bad masks");
    } else {
      mr = LE32(h + 40);
      mg = LE32(h + 44);
      mb = LE32(h + 48);
      ma = hsz >= 56 ? LE32(h + 52) : 0;
    }
  } else if (bpp != 1 && bpp != 4 && bpp != 8 && bpp != 24) {
    Fail("bmp: unsupported bit depth");
  } else if (compress == 3) {
    Fail("bmp: bitfields need 16 or 32-bit pixels");
  }
  const int src = ma ? 4 : 3;  // samples per pixel before the requested conversion
  std::vector<uint8_t> px((size_t)w * ht * src);
  uint8_t pal[256][4] = {};
  if (bpp < 16) {
    int esz = hsz == 12 ? 3 : 4;
    int64_t psize = offset > extra ? (int64_t)(offset - extra) / esz : 0;
    if (psize <= 0 || psize > 256) Fail("bmp: bad palette");
    if (extra + (size_t)psize * esz > n) Fail("bmp: truncated palette");
    for (int i = 0; i < psize; i++) {
      const uint8_t* e = b + extra + (size_t)i * esz;
      pal[i][0] = e[2];
      pal[i][1] = e[1];
      pal[i][2] = e[0];
      pal[i][3] = 255;
    }
  }
  size_t rowBytes = (((size_t)w * bpp + 31) / 32) * 4;
  if (offset > n || (size_t)ht * rowBytes > n - offset) Fail("bmp: pixel data truncated");
  int rs = HighBit(mr) - 7, gs = HighBit(mg) - 7, bs = HighBit(mb) - 7, as = HighBit(ma) - 7;
  int rc = BitCount(mr), gc = BitCount(mg), bc = BitCount(mb), ac = BitCount(ma);
  bool anyAlpha = false;
  for (int64_t y = 0; y < ht; y++) {
    const uint8_t* row = b + offset + (size_t)y * rowBytes;
    int64_t oy = topDown ? y : ht - 1 - y;  // output rows top to bottom
    uint8_t* o = &px[(size_t)oy * w * src];
    for (int64_t x = 0; x < w; x++, o += src) {
      if (bpp < 16) {
        int idx;
        if (bpp == 8) {
          idx = row[x];
        } else if (bpp == 4) {
          idx = (row[x >> 1] >> ((x & 1) ? 0 : 4)) & 15;
        } else {
          idx = (row[x >> 3] >> (7 - (x & 7))) & 1;
        }
        o[0] = pal[idx][0];
        o[1] = pal[idx][1];
        o[2] = pal[idx][2];
      } else if (bpp == 24) {
        const uint8_t* p = row + 3 * x;
        o[0] = p[2];
        o[1] = p[1];
        o[2] = p[0];
      } else {
        uint32_t v = bpp == 16 ? (uint32_t)LE16(row + 2 * x) : LE32(row + 4 * x);
        o[0] = (uint8_t)MaskField(v, mr, rs, rc);
        o[1] = (uint8_t)MaskField(v, mg, gs, gc);
        o[2] = (uint8_t)MaskField(v, mb, bs, bc);
        if (src == 4) {
          o[3] = (uint8_t)(ma ? MaskField(v, ma, as, ac) : 255);
          anyAlpha |= o[3] != 0;
        }
      }
    }
  }
  if (src == 4 && !anyAlpha)
    for (size_t i = 3; i < px.size(); i += 4) px[i] = 255;
  Ldr out;
  out.width = (int)w;
  out.height = (int)ht;
  out.channels = req;
  ConvertChannels(px, src, req, (size_t)w * ht, out.px);
  if (flipY) FlipRows(out.px.data(), out.height, (size_t)out.width * req);
  return out;
}

// ---------------------------------------------------------------------- TGA
// Truevision TGA as stb_image reads it: colour-mapped (type 1 / 9), true-colour
// (2 / 10) and grey (3 / 11) images, run-length packets for the 9..11 types,
// 8-bit grey or indices, 15 / 16-bit 5-5-5 colour (each field scaled by
// 255 / 31, no alpha), 24-bit BGR and 32-bit BGRA; rows bottom-up unless the
// descriptor's top-to-bottom bit is set.
Ldr DecodeTga(const std::string& bytes, int req, bool flipY) {
  const uint8_t* b = (const uint8_t*)bytes.data();
  size_t n = bytes.size();
  if (n < 18) Fail("tga: truncated header");
  int idLen = b[0], cmapType = b[1], type = b[2];
  int cmapFirst = LE16(b + 3), cmapLen = LE16(b + 5), cmapBits = b[7];
  int w = LE16(b + 12), ht = LE16(b + 14), bits = b[16], desc = b[17];
  bool rle = type >= 8;
  int base = rle ? type - 8 : type;
  if (cmapType > 1 || (base != 1 && base != 2 && base != 3)) Fail("tga: unsupported image type");
  if ((base == 1) != (cmapType == 1)) Fail("tga: colour map and image type disagree");
  if (w == 0 || ht == 0) Fail("tga: zero size");
  auto compOf = [](int bitsPer, bool grey) {  // stbi__tga_get_comp
    if (bitsPer == 8) return grey ? 1 : 0;
    if (bitsPer == 15 || bitsPer == 16) return bitsPer == 16 && grey ? 2 : 3;
    if (bitsPer == 24) return 3;
    if (bitsPer == 32) return 4;
    return 0;
  };
  int comp;
  if (base == 1) {
    if (bits != 8 && bits != 16) Fail("tga: colour-map indices must be 8 or 16 bits");
    comp = compOf(cmapBits, false);
  } else {
    comp = compOf(bits, base == 3);
  }
  if (comp == 0 || comp == 2) Fail("tga: unsupported pixel format");
  size_t pos = 18 + (size_t)idLen;
  const bool rgb16 = (base == 1 ? cmapBits : bits) == 15 || (base == 1 ? cmapBits : bits) == 16;
  auto readPixel = [&](const uint8_t* p, int nbits, uint8_t* o) {
    if (nbits == 15 || nbits == 16) {
      int v = LE16(p);
      int r = (v >> 10) & 31, g = (v >> 5) & 31, bl = v & 31;
      o[0] = (uint8_t)((r * 255) / 31);
      o[1] = (uint8_t)((g * 255) / 31);
      o[2] = (uint8_t)((bl * 255) / 31);
    } else {
      for (int i = 0; i < nbits / 8; i++) o[i] = p[i];
    }
  };
  std::vector<uint8_t> cmap;
  int cmapBytes = (cmapBits + 1) >> 3;
  if (cmapType == 1) {
    // stb_image refuses an empty palette ("bad palette"); every index would fall back to entry 0
    if (cmapLen == 0) Fail("tga: empty colour map");
    if (pos + (size_t)cmapLen * cmapBytes > n) Fail("tga: truncated colour map");
    cmap.resize((size_t)cmapLen * comp);
    for (int i = 0; i < cmapLen; i++) readPixel(b + pos + (size_t)i * cmapBytes, cmapBits, &cmap[(size_t)i * comp]);
    pos += (size_t)cmapLen * cmapBytes;
  }
  const int pixBytes = (bits + 1) >> 3;
  std::vector<uint8_t> px((size_t)w * ht * comp);
  size_t total = (size_t)w * ht;
  uint8_t cur[4] = {};
  int runLeft = 0;
  bool repeat = false, first = true;
  for (size_t i = 0; i < total; i++) {
    bool read = true;
    if (rle) {
      if (runLeft == 0) {
        if (pos >= n) Fail("tga: truncated data");
        int hdr = b[pos++];
        runLeft = 1 + (hdr & 127);
        repeat = (hdr & 128) != 0;
        read = true;
      } else if (repeat) {
        read = false;
      }
      runLeft--;
    }
    if (read || first) {
      if (pos + pixBytes > n) Fail("tga: truncated data");
      const uint8_t* p = b + pos;
      pos += pixBytes;
      if (base == 1) {
        int idx = pixBytes == 1 ? p[0] : LE16(p);
        idx -= cmapFirst;
        if (idx < 0 || idx >= cmapLen) idx = 0;
        std::memcpy(cur, &cmap[(size_t)idx * comp], comp);
      } else {
        readPixel(p, bits, cur);
      }
      first = false;
    }
    std::memcpy(&px[i * comp], cur, comp);
  }
  if (comp >= 3 && !rgb16)  // BGR(A) -> RGB(A)
    for (size_t i = 0; i < total; i++) std::swap(px[i * comp], px[i * comp + 2]);
  if (!((desc >> 5) & 1)) FlipRows(px.data(), ht, (size_t)w * comp);  // stored bottom-up
  Ldr out;
  out.width = w;
  out.height = ht;
  out.channels = req;
  ConvertChannels(px, comp, req, total, out.px);
  if (flipY) FlipRows(out.px.data(), out.height, (size_t)out.width * req);
  return out;
}

bool IsBmp(const std::string& b) { return b.size() >= 2 && b[0] == 'B' && b[1] == 'M'; }
// stbi__tga_test: a plausible header (no magic number)
bool IsTga(const std::string& s) {
  if (s.size() < 18) return false;
  const uint8_t* b = (const uint8_t*)s.data();
  int cmapType = b[1], type = b[2];
  if (cmapType > 1) return false;
  if (cmapType == 1) {
    if (type != 1 && type != 9) return false;
    if (b[7] != 8 && b[7] != 15 && b[7] != 16 && b[7] != 24 && b[7] != 32) return false;
    if (b[16] != 8 && b[16] != 16) return false;
  } else {
    if (type != 2 && type != 3 && type != 10 && type != 11) return false;
    int bits = b[16];
    if (bits != 8 && bits != 15 && bits != 16 && bits != 24 && bits != 32) return false;
  }
  return LE16(b + 12) >= 1 && LE16(b + 14) >= 1;
}

// stbi_load of a Radiance file (stbi__hdr_load + stbi__hdr_to_ldr): one
// requested channel is (r + g + b) / 3 of the decoded RGBE values; each value v
// becomes (v ^ (1 / 2.2)) * 255 + 0.5, clamped to 0..255 and truncated.
bool IsHdrFile(const std::string& b) { return b.rfind("#?RADIANCE", 0) == 0 || b.rfind("#?RGBE", 0) == 0; }
Ldr HdrToLdr(const std::string& bytes, int req, bool flipY) {
  Hdr h = LoadHdr(bytes, flipY);
  Ldr out;
  out.width = h.width;
  out.height = h.height;
  out.channels = req;
  size_t npx = (size_t)h.width * h.height;
  out.px.resize(npx * req);
  const float gamma = 1.0f / 2.2f;
  for (size_t i = 0; i < npx; i++)
    for (int k = 0; k < req; k++) {
      const float* c = &h.px[i * 3];
      float v = req == 3 ? c[k] : (c[0] + c[1] + c[2]) / 3;
      float z = (float)std::pow((double)v, (double)gamma) * 255 + 0.5f;
      z = z < 0 ? 0 : z > 255 ? 255 : z;
      out.px[i * req + k] = (uint8_t)z;
    }
  return out;
}

bool IsPng(const std::string& b) { return b.size() >= 8 && std::memcmp(b.data(), "\x89PNG\r\n\x1a\n", 8) == 0; }
bool IsPnm(const std::string& b) { return b.size() >= 3 && b[0] == 'P' && (b[1] == '5' || b[1] == '6'); }

}  // namespace

Ldr LoadLdr(const std::string& bytes, int reqChannels, bool flipY) {
  if (reqChannels != 1 && reqChannels != 3) Fail("channel must be 1 or 3");
  if (IsPng(bytes)) return DecodePng(bytes, reqChannels, flipY);
  if (IsPnm(bytes)) return DecodePnm(bytes, reqChannels, flipY);
  if (IsJpeg(bytes)) return DecodeJpeg(bytes, reqChannels, flipY);
  if (IsBmp(bytes)) return DecodeBmp(bytes, reqChannels, flipY);
  if (IsHdrFile(bytes)) return HdrToLdr(bytes, reqChannels, flipY);
  if (IsTga(bytes)) return DecodeTga(bytes, reqChannels, flipY);  // last: TGA has no signature
  Fail("unsupported image format (PNG, JPEG, BMP, TGA, Radiance HDR and binary PNM are read)");
}

// --------------------------------------------------------------------- HDR
Hdr LoadHdr(const std::string& bytes, bool flipY) {
  Hdr out;
  if (IsPng(bytes) || IsPnm(bytes) || IsJpeg(bytes) || IsBmp(bytes) || (!IsHdrFile(bytes) && IsTga(bytes))) {
    // stbi_loadf of an LDR file
    Ldr l = LoadLdr(bytes, 3, flipY);
    out.width = l.width;
    out.height = l.height;
    out.px.resize(l.px.size());
    for (size_t i = 0; i < l.px.size(); i++)
      out.px[i] = (float)(std::pow((double)(l.px[i] / 255.0f), (double)2.2f) * (double)1.0f);
    return out;
  }
  size_t pos = 0;
  auto line = [&]() {
    size_t e = bytes.find('\n', pos);
    if (e == std::string::npos) Fail("hdr header truncated");
    std::string s = bytes.substr(pos, e - pos);
    pos = e + 1;
    return s;
  };
  std::string magic = line();
  if (magic != "#?RADIANCE" && magic != "#?RGBE") Fail("not a Radiance hdr file");
  bool fmt = false;
  for (;;) {
    std::string s = line();
    if (s.empty()) break;
    if (s == "FORMAT=32-bit_rle_rgbe") fmt = true;
  }
  if (!fmt) Fail("unsupported hdr format");
  std::string res = line();
  int w = 0, h = 0;
  if (std::sscanf(res.c_str(), "-Y %d +X %d", &h, &w) != 2) Fail("unsupported hdr orientation");
  if (w <= 0 || h <= 0 || w > (1 << 24) || h > (1 << 24)) Fail("bad hdr size");
  const uint8_t* p = (const uint8_t*)bytes.data();
  size_t n = bytes.size();
  std::vector<uint8_t> rgbe((size_t)w * h * 4);
  bool rle = w >= 8 && w < 32768 && pos + 4 <= n && p[pos] == 2 && p[pos + 1] == 2 && !(p[pos + 2] & 0x80);
  if (!rle) {
    if (pos + rgbe.size() > n) Fail("hdr data truncated");
    std::memcpy(rgbe.data(), p + pos, rgbe.size());
  } else {
    std::vector<uint8_t> sc((size_t)w * 4);
    for (int y = 0; y < h; y++) {
      if (pos + 4 > n || p[pos] != 2 || p[pos + 1] != 2 || ((p[pos + 2] << 8) | p[pos + 3]) != w)
        Fail("bad hdr scanline header");
      pos += 4;
      for (int c = 0; c < 4; c++) {
        int x = 0;
        while (x < w) {
          if (pos >= n) Fail("hdr data truncated");
          int cnt = p[pos++];
          if (cnt > 128) {
            cnt -= 128;
            if (pos >= n || x + cnt > w) Fail("bad hdr run");
            uint8_t v = p[pos++];
            for (int k = 0; k < cnt; k++) sc[(size_t)(x++) * 4 + c] = v;
          } else {
            if (cnt == 0 || pos + cnt > n || x + cnt > w) Fail("bad hdr literal");
            for (int k = 0; k < cnt; k++) sc[(size_t)(x++) * 4 + c] = p[pos++];
          }
        }
      }
      std::memcpy(&rgbe[(size_t)y * w * 4], sc.data(), sc.size());
    }
  }
  out.width = w;
  out.height = h;
  out.px.resize((size_t)w * h * 3);
  for (size_t i = 0; i < (size_t)w * h; i++) {
    const uint8_t* q = &rgbe[i * 4];
    if (q[3]) {
      float f = (float)std::ldexp(1.0f, (int)q[3] - (int)(128 + 8));
      out.px[i * 3] = q[0] * f;
      out.px[i * 3 + 1] = q[1] * f;
      out.px[i * 3 + 2] = q[2] * f;
    } else {
      out.px[i * 3] = out.px[i * 3 + 1] = out.px[i * 3 + 2] = 0.f;
    }
  }
  if (flipY) FlipRows((uint8_t*)out.px.data(), h, (size_t)w * 3 * sizeof(float));
  return out;
}

// --------------------------------------------------------------------- EXR
namespace {

void ExrUnpredict(std::vector<uint8_t>& t, size_t size, std::vector<uint8_t>& out) {
  for (size_t i = 1; i < size; i++) t[i] = (uint8_t)((int)t[i - 1] + (int)t[i] - 128);
  out.resize(size);
  size_t a = 0, b = (size + 1) / 2, s = 0;
  while (s < size) {
    out[s++] = t[a++];
    if (s < size) out[s++] = t[b++];
  }
}

std::vector<uint8_t> ExrRle(const uint8_t* in, size_t n, size_t expect) {
  std::vector<uint8_t> t;
  t.reserve(expect);
  size_t i = 0;
  while (i < n) {
    int c = (int8_t)in[i++];
    if (c < 0) {
      if (i + (size_t)(-c) > n) Fail("exr rle literal truncated");
      t.insert(t.end(), in + i, in + i + (-c));
      i += (size_t)(-c);
    } else {
      if (i >= n) Fail("exr rle run truncated");
      t.insert(t.end(), (size_t)c + 1, in[i++]);
    }
    if (t.size() > expect) Fail("exr rle overflow");
  }
  return t;
}

}  // namespace

Hdr LoadExr(const std::string& bytes) {
  const uint8_t* p = (const uint8_t*)bytes.data();
  size_t n = bytes.size();
  if (n < 8 || p[0] != 0x76 || p[1] != 0x2f || p[2] != 0x31 || p[3] != 0x01) Fail("not an OpenEXR file");
  uint32_t ver = p[4] | (p[5] << 8) | (p[6] << 16) | ((uint32_t)p[7] << 24);
  if ((ver & 0xff) != 2) Fail("unsupported OpenEXR version");
  if (ver & 0x200) Fail("tiled OpenEXR files are not supported");
  if (ver & (0x800 | 0x1000)) Fail("deep / multi-part OpenEXR files are not supported");
  auto rd32 = [&](size_t at) -> int32_t {
    if (at + 4 > n) Fail("exr truncated");
    return (int32_t)(p[at] | (p[at + 1] << 8) | (p[at + 2] << 16) | ((uint32_t)p[at + 3] << 24));
  };
  auto cstr = [&](size_t& at) {
    size_t e = at;
    while (e < n && p[e]) e++;
    if (e >= n) Fail("exr string truncated");
    std::string s((const char*)p + at, e - at);
    at = e + 1;
    return s;
  };
  struct Ch {
    std::string name;
    int type, xs, ys;
  };
  std::vector<Ch> chans;
  int comp = -1;
  int32_t box[4] = {0, 0, -1, -1};
  bool haveBox = false;
  size_t pos = 8;
  for (;;) {
    if (pos >= n) Fail("exr header truncated");
    if (p[pos] == 0) {
      pos++;
      break;
    }
    std::string name = cstr(pos), type = cstr(pos);
    int32_t size = rd32(pos);
    pos += 4;
    if (size < 0 || pos + (size_t)size > n) Fail("exr attribute truncated");
    size_t end = pos + (size_t)size;
    if (name == "channels" && type == "chlist") {
      size_t q = pos;
      while (q < end && p[q]) {
        Ch c;
        c.name = cstr(q);
        c.type = rd32(q);
        c.xs = rd32(q + 8);
        c.ys = rd32(q + 12);
        q += 16;
        chans.push_back(c);
      }
    } else if (name == "compression") {
      comp = p[pos];
    } else if (name == "dataWindow" && type == "box2i") {
      for (int k = 0; k < 4; k++) box[k] = rd32(pos + 4 * k);
      haveBox = true;
    }
    pos = end;
  }
  if (chans.empty() || !haveBox) Fail("exr header lacks channels / dataWindow");
  for (const Ch& c : chans) {
    if (c.xs != 1 || c.ys != 1) Fail("subsampled exr channels are not supported");
    if (c.type != 1 && c.type != 2) Fail("exr UINT channels are not supported");
  }
  int linesPer;
  switch (comp) {
    case 0: case 1: case 2: linesPer = 1; break;
    case 3: linesPer = 16; break;
    default: Fail("exr compression other than NONE / RLE / ZIPS / ZIP is not supported");
  }
  int64_t w = (int64_t)box[2] - box[0] + 1, h = (int64_t)box[3] - box[1] + 1;
  if (w <= 0 || h <= 0 || w > (1 << 24) || h > (1 << 24)) Fail("bad exr size");
  // R, G, B by the name after the last '.', first one wins (image_reader.cpp:133-160)
  int pick[3] = {-1, -1, -1};
  for (size_t i = 0; i < chans.size(); i++) {
    std::string s = chans[i].name;
    size_t d = s.rfind('.');
    if (d != std::string::npos) s = s.substr(d + 1);
    for (char& ch : s) ch = (char)std::tolower((unsigned char)ch);
    int k = s == "r" ? 0 : s == "g" ? 1 : s == "b" ? 2 : -1;
    if (k >= 0 && pick[k] < 0) pick[k] = (int)i;
  }
  bool halfSlice = chans[0].type == 1;  // the frame buffer takes the first channel's type
  size_t lineBytes = 0;
  std::vector<size_t> chOff(chans.size());
  for (size_t i = 0; i < chans.size(); i++) {
    chOff[i] = lineBytes;
    lineBytes += (size_t)w * (chans[i].type == 1 ? 2 : 4);
  }
  size_t nChunks = (size_t)((h + linesPer - 1) / linesPer);
  if (pos + nChunks * 8 > n) Fail("exr offset table truncated");
  Hdr out;
  out.width = (int)w;
  out.height = (int)h;
  out.px.assign((size_t)w * h * 3, 0.f);
  std::vector<uint8_t> tmp, blk;
  for (size_t c = 0; c < nChunks; c++) {
    uint64_t off = 0;
    for (int k = 7; k >= 0; k--) off = (off << 8) | p[pos + c * 8 + k];
    if (off + 8 > n) Fail("exr chunk offset out of range");
    int32_t y = rd32((size_t)off), size = rd32((size_t)off + 4);
    int64_t row0 = (int64_t)y - box[1];
    if (row0 < 0 || row0 >= h || size < 0 || off + 8 + (uint64_t)size > n) Fail("bad exr chunk");
    int lines = (int)std::min<int64_t>(linesPer, h - row0);
    size_t expect = lineBytes * lines;
    const uint8_t* d = p + off + 8;
    const uint8_t* data;
    if ((size_t)size == expect || comp == 0) {
      if ((size_t)size < expect) Fail("exr chunk too short");
      data = d;
    } else {
      if (comp == 1) {
        tmp = ExrRle(d, (size_t)size, expect);
      } else {
        tmp = Inflate(d, (size_t)size, true);
      }
      if (tmp.size() != expect) Fail("exr chunk size mismatch");
      ExrUnpredict(tmp, expect, blk);
      data = blk.data();
    }
    for (int l = 0; l < lines; l++) {
      const uint8_t* line = data + (size_t)l * lineBytes;
      float* o = &out.px[(size_t)(row0 + l) * w * 3];
      for (int k = 0; k < 3; k++) {
        if (pick[k] < 0) continue;
        const Ch& ch = chans[pick[k]];
        const uint8_t* s = line + chOff[pick[k]];
        for (int64_t x = 0; x < w; x++) {
          float v;
          if (ch.type == 1) {
            v = HalfToFloat((uint16_t)(s[x * 2] | (s[x * 2 + 1] << 8)));
          } else {
            uint32_t bits = s[x * 4] | (s[x * 4 + 1] << 8) | (s[x * 4 + 2] << 16) | ((uint32_t)s[x * 4 + 3] << 24);
            std::memcpy(&v, &bits, 4);
            if (halfSlice) v = HalfToFloat(FloatToHalf(v));
          }
          o[x * 3 + k] = v;
        }
      }
    }
  }
  return out;
}

}  // namespace img
}  // namespace rad
