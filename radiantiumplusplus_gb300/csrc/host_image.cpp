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

bool IsPng(const std::string& b) { return b.size() >= 8 && std::memcmp(b.data(), "\x89PNG\r\n\x1a\n", 8) == 0; }
bool IsPnm(const std::string& b) { return b.size() >= 3 && b[0] == 'P' && (b[1] == '5' || b[1] == '6'); }

}  // namespace

Ldr LoadLdr(const std::string& bytes, int reqChannels, bool flipY) {
  if (reqChannels != 1 && reqChannels != 3) Fail("channel must be 1 or 3");
  if (IsPng(bytes)) return DecodePng(bytes, reqChannels, flipY);
  if (IsPnm(bytes)) return DecodePnm(bytes, reqChannels, flipY);
  Fail("unsupported image format (PNG and binary PNM are read)");
}

// --------------------------------------------------------------------- HDR
Hdr LoadHdr(const std::string& bytes, bool flipY) {
  Hdr out;
  if (IsPng(bytes) || IsPnm(bytes)) {  // stbi_loadf of an LDR file
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
