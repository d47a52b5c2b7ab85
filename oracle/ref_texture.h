// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_core.h).
// Textures: Texture<T> with its constant fast path (texture.h:47-90),
// ConfigNodeReadTexture (config_node_ext.h:17-45), Bitmap over a MipMap with
// nearest / bilinear / trilinear / anisotropic (EWA) filtering
// (bitmap.cpp:24-344), Chessboard (chessboard.cpp:15-63), and the image assets
// behind bitmaps (rad.core asset/image_stb.cpp, image_hdr.cpp, image_exr.cpp).
// Image files are decoded by the library's decoder
// (radiantiumplusplus_gb300/csrc/host_image.cpp, compiled into this library:
// the reference's stb_image / OpenEXR are absent); the decoder's output is
// pinned on its own by tests/test_images.py against images encoded in Python.
#pragma once
#include "ref_core.h"

namespace orc {

// What a texture lookup reads from the SurfaceInteraction: UV and its
// screen-space derivatives (interaction.h: UV, dUVdX, dUVdY).
struct TexSi {
  V2 uv, duvdx, duvdy;
  // BsdfContext::Mode == TransportMode::Importance (light tracing, particle_tracer.cpp:161, :199); BSDF calls
  // carry it with the surface point
  bool importance = false;
};

// RGB textures return (r, g, b); mono textures return (v, 0, 0).
struct Texture {
  int channels = 3;
  uint32_t width = 1, height = 1;  // texture.h:30-31 (1 x 1 for constants and chessboards)
  virtual ~Texture() = default;
  virtual V3 Eval(const TexSi& si) const = 0;
  virtual V3 Read(uint32_t x, uint32_t y) const = 0;
};

struct ImageAsset {
  int width = 0, height = 0, channels = 0;
  std::vector<float> px;  // texel (x, y) at (y * width + x) * channels
  std::string type;
};
ImageAsset LoadImageAsset(const Json& cfg, const std::string& type, const std::string& path);

struct TexEnv {
  const std::map<std::string, ImageAsset>* images = nullptr;
  std::vector<const Texture*>* created = nullptr;  // every texture, in creation order
};

// ConfigNodeReadTexture for a present key: numbers / arrays are constants.
std::shared_ptr<Texture> MakeTexture(const Json& node, int channels, TexEnv* env);
std::shared_ptr<Texture> ConstTexture(const V3& v, int channels);

}  // namespace orc
