// Image decoders behind the reference's image assets (rad.core asset/image_stb.cpp,
// image_hdr.cpp, image_exr.cpp; image_reader.cpp:44-216). The reference links
// stb_image and OpenEXR; neither is available here, so the formats are read by
// this file from their published specifications:
//  * PNG (ISO/IEC 15948; zlib / deflate per RFC 1950 / 1951): all colour types,
//    bit depths 1..16, Adam7 interlacing, PLTE / tRNS;
//  * baseline and progressive Huffman JPEG (ITU-T T.81) with stb_image's
//    integer IDCT, chroma upsampling and colour conversion;
//  * BMP (palette, 24-bit, 16 / 32-bit masked; not RLE) and TGA (colour-mapped,
//    true-colour and grey, raw or run-length);
//  * binary PNM (P5 / P6, maxval <= 255);
//  * Radiance RGBE .hdr (flat and adaptive run-length scanlines);
//  * OpenEXR scanline images with NONE, RLE, ZIPS or ZIP compression and HALF or
//    FLOAT channels.
// Results follow stb's conventions where the reference relies on them: 16-bit
// samples keep their high byte, channel counts are converted the way stbi_load
// converts them (grey replicated, alpha dropped, RGB -> grey by the integer
// luma (77 r + 150 g + 29 b) >> 8), and rows are flipped bottom-up on request.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace rad {
namespace img {

// 8-bit image, `channels` interleaved samples per pixel, rows top to bottom
// unless flipped.
struct Ldr {
  int width = 0, height = 0, channels = 0;
  std::vector<uint8_t> px;
};
// float image (3 channels), rows top to bottom unless flipped.
struct Hdr {
  int width = 0, height = 0;
  std::vector<float> px;
};

// stbi_load(..., req_comp) for PNG / JPEG / BMP / TGA / PNM files (and Radiance
// files mapped to 8 bits as stb does): req_comp is 1 or 3.
Ldr LoadLdr(const std::string& bytes, int reqChannels, bool flipY);
// stbi_loadf(..., 3) for Radiance .hdr files (and, like stb, LDR files mapped
// through (v / 255) ^ 2.2).
Hdr LoadHdr(const std::string& bytes, bool flipY);
// ImageReader::ReadExr: R, G, B channels by name (missing ones read 0).
Hdr LoadExr(const std::string& bytes);

// zlib stream (RFC 1950) -> bytes; throws on malformed input.
std::vector<uint8_t> Inflate(const uint8_t* data, size_t n, bool zlibHeader);
// IEEE 754 binary16 bit pattern -> float.
float HalfToFloat(uint16_t h);

}  // namespace img
}  // namespace rad
