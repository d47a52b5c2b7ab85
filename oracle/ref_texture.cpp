// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_core.h). Textures; see ref_texture.h.
#include "ref_texture.h"

#include <algorithm>
#include <fstream>
#include <sstream>

#include "../radiantiumplusplus_gb300/csrc/host_image.h"

namespace orc {

namespace {

// texture.h:44-50: a constant colour
struct ConstTex final : Texture {
  V3 value;
  V3 Eval(const TexSi&) const override { return value; }
  V3 Read(uint32_t, uint32_t) const override { return value; }
};

// One mip level: width x height texels of `channels` floats.
struct Level {
  uint32_t w = 0, h = 0;
  std::vector<float> px;
  V3 At(uint32_t x, uint32_t y, int c) const {
    const float* p = &px[((size_t)y * w + x) * c];
    return c == 3 ? V3(p[0], p[1], p[2]) : V3(p[0], 0, 0);
  }
};

// bitmap.cpp:24-261
struct MipMap {
  std::vector<Level> mips;
  int wrap = 0;  // 0 clamp, 1 repeat
  int C = 3;

  MipMap(Level image, int maxLevel, int wrapMode, int channels) : wrap(wrapMode), C(channels) {
    if (maxLevel != 0 && ((image.w % 2 != 0) || (image.h % 2 != 0))) maxLevel = 0;
    uint32_t realMaxLevel;
    if (maxLevel < 0) {
      realMaxLevel = 1 + (uint32_t)std::log2(std::max(image.w, image.h));
    } else {
      realMaxLevel = (uint32_t)maxLevel;
    }
    realMaxLevel = std::max(realMaxLevel, 1u);
    mips.push_back(std::move(image));
    for (uint32_t a = 1; a < realMaxLevel; a++) {
      Level map;
      map.w = std::max(1u, mips[a - 1].w / 2);
      map.h = std::max(1u, mips[a - 1].h / 2);
      map.px.resize((size_t)map.w * map.h * C);
      const Level& last = mips[a - 1];
      for (uint32_t j = 0; j < map.h; j++) {
        for (uint32_t i = 0; i < map.w; i++) {
          V3 u0v0 = FilterBilinearInt(last, i * 2, j * 2);
          V3 u1v0 = FilterBilinearInt(last, i * 2 + 1, j * 2);
          V3 u0v1 = FilterBilinearInt(last, i * 2, j * 2 + 1);
          V3 u1v1 = FilterBilinearInt(last, i * 2 + 1, j * 2 + 1);
          V3 color = (u0v0 + u1v0 + u0v1 + u1v1) * Float(0.25);
          for (int c = 0; c < C; c++) map.px[((size_t)j * map.w + i) * C + c] = color[c];
        }
      }
      mips.push_back(std::move(map));
    }
  }
  size_t MaxLevel() const { return mips.size(); }

  V3 EvalNearest(const V2& uv) const { return FilterNearest(mips[0], uv); }
  V3 EvalBilinear(const V2& uv) const { return FilterBilinear(mips[0], uv); }

  // bitmap.cpp:78-101
  V3 EvalTrilinear(const V2& uv, const V2& duvdx, const V2& duvdy) const {
    Float x = duvdx.x * duvdx.x + duvdx.y * duvdx.y;
    Float y = duvdy.x * duvdy.x + duvdy.y * duvdy.y;
    Float width = std::sqrt(std::max(x, y));
    Float level = MaxLevel() - 1 + std::log2(std::max(width, Float(1e-8)));
    if (level < 0) return EvalIsotropic(uv, 0);
    if (level >= MaxLevel() - 1) return EvalIsotropic(uv, MaxLevel() - 1);
    size_t down = (size_t)std::floor(level);
    Float weight = level - down;
    V3 low = EvalIsotropic(uv, down);
    V3 high = EvalIsotropic(uv, down + 1);
    return low * (1 - weight) + (high * weight);
  }

  // bitmap.cpp:106-145
  V3 EvalAnisotropic(const V2& uv, const V2& duvdx, const V2& duvdy, Float anisoLevel) const {
    Float x = duvdx.x * duvdx.x + duvdx.y * duvdx.y;
    Float y = duvdy.x * duvdy.x + duvdy.y * duvdy.y;
    Float big = std::sqrt(std::max(x, y));
    Float small = std::sqrt(std::min(x, y));
    V2 bigduv = x < y ? duvdy : duvdx;
    V2 smallduv = x < y ? duvdx : duvdy;
    if ((small * anisoLevel < big) && (small > 0)) {
      Float scale = big / (small * anisoLevel);
      smallduv = V2(smallduv.x * scale, smallduv.y * scale);
      small *= scale;
    }
    if (small == 0) return EvalIsotropic(uv, 0);
    Float level = MaxLevel() - 1 + std::log2(std::max(small, Float(1e-8)));
    if (level < 0) return EvalEWA(uv, 0, bigduv, smallduv);
    if (level >= MaxLevel() - 1) return EvalIsotropic(uv, MaxLevel() - 1);
    size_t down = (size_t)std::floor(level);
    Float weight = level - down;
    V3 low = EvalEWA(uv, down, bigduv, smallduv);
    V3 high(0);
    if (weight != 0) high = EvalEWA(uv, down + 1, bigduv, smallduv);
    return low * (1 - weight) + (high * weight);
  }

  // bitmap.cpp:149-157
  Float Wrap(Float v) const {
    if (wrap == 1) return std::clamp(v - std::floor(v), Float(0), Float(1));
    return std::clamp(v, Float(0), Float(1));
  }
  // bitmap.cpp:159-170
  void WrapInt(const Level& img, uint32_t u, uint32_t v, uint32_t& x, uint32_t& y) const {
    if (wrap == 1) {
      x = u % img.w;
      y = v % img.h;
    } else {
      x = std::clamp(u, uint32_t(0), img.w - 1);
      y = std::clamp(v, uint32_t(0), img.h - 1);
    }
  }
  // bitmap.cpp:172-178
  V3 FilterBilinearInt(const Level& img, uint32_t u, uint32_t v) const {
    uint32_t pu, pv;
    WrapInt(img, u, v, pu, pv);
    Float fu = pu + Float(1);
    Float fv = pv + Float(1);
    return FilterBilinear(img, pu, pv, fu, fv);
  }
  // The continuous coordinate's integer part. A NaN uv (undefined conversion
  // in the reference) reads texel 0.
  static uint32_t Index(Float f, uint32_t n) {
    uint32_t p = f >= 0 ? (uint32_t)f : 0u;
    return std::min(p, n - 1);
  }
  // bitmap.cpp:179-188
  V3 FilterNearest(const Level& img, const V2& uv) const {
    Float u = Wrap(uv.x);
    Float v = Wrap(uv.y);
    Float fu = u * (img.w - 1);
    Float fv = v * (img.h - 1);
    return img.At(Index(fu, img.w), Index(fv, img.h), C);
  }
  // bitmap.cpp:190-198
  V3 FilterBilinear(const Level& img, const V2& uv) const {
    Float u = Wrap(uv.x);
    Float v = Wrap(uv.y);
    Float fu = u * (img.w - 1);
    Float fv = v * (img.h - 1);
    return FilterBilinear(img, Index(fu, img.w), Index(fv, img.h), fu, fv);
  }
  // bitmap.cpp:200-214
  V3 FilterBilinear(const Level& img, uint32_t pu, uint32_t pv, Float fu, Float fv) const {
    int32_t dpu = (fu > pu + 0.5f) ? 1 : -1;
    int32_t dpv = (fv > pv + 0.5f) ? 1 : -1;
    uint32_t apu = std::clamp(pu + dpu, 0u, img.w - 1);
    uint32_t apv = std::clamp(pv + dpv, 0u, img.h - 1);
    Float du = std::min(std::abs(fu - pu - Float(0.5)), Float(1));
    Float dv = std::min(std::abs(fv - pv - Float(0.5)), Float(1));
    V3 u0v0 = img.At(pu, pv, C);
    V3 u1v0 = img.At(apu, pv, C);
    V3 u0v1 = img.At(pu, apv, C);
    V3 u1v1 = img.At(apu, apv, C);
    return (u0v0 * (1 - du) + u1v0 * du) * (1 - dv) + (u0v1 * (1 - du) + u1v1 * du) * dv;
  }
  // bitmap.cpp:216-220: bilinear whatever the filter argument
  V3 EvalIsotropic(const V2& uv, size_t level) const {
    size_t l = std::clamp(level, size_t(0), MaxLevel() - 1);
    return FilterBilinear(mips[l], uv);
  }
  // bitmap.cpp:222-258 (reads level 0 through EvalNearest)
  V3 EvalEWA(const V2& uv_, size_t level, const V2& dst0_, const V2& dst1_) const {
    const Level& map = mips[level];
    V2 st(uv_.x * (map.w), uv_.y * (map.h));
    V2 dst0(dst0_.x * map.w, dst0_.y * map.h);
    V2 dst1(dst1_.x * map.w, dst1_.y * map.h);
    Float A = dst0[1] * dst0[1] + dst1[1] * dst1[1] + 1;
    Float B = -2 * (dst0[0] * dst0[1] + dst1[0] * dst1[1]);
    Float Cc = dst0[0] * dst0[0] + dst1[0] * dst1[0] + 1;
    Float invF = 1 / (A * Cc - B * B * Float(0.25));
    A *= invF;
    B *= invF;
    Cc *= invF;
    Float det = -B * B + 4 * A * Cc;
    Float invDet = 1 / det;
    Float uSqrt = std::sqrt(det * Cc), vSqrt = std::sqrt(det * A);
    int32_t s0 = (int32_t)std::ceil(st[0] - 2 * invDet * uSqrt);
    int32_t s1 = (int32_t)std::floor(st[0] + 2 * invDet * uSqrt);
    int32_t t0 = (int32_t)std::ceil(st[1] - 2 * invDet * vSqrt);
    int32_t t1 = (int32_t)std::floor(st[1] + 2 * invDet * vSqrt);
    const V2 invR(1 / Float(map.w), 1 / Float(map.h));
    V3 sum(0);
    Float sumWts = 0;
    for (int it = t0; it <= t1; ++it) {
      Float tt = it - st[1];
      for (int is = s0; is <= s1; ++is) {
        Float ss = is - st[0];
        Float r2 = A * ss * ss + B * ss * tt + Cc * tt * tt;
        if (r2 < 1) {
          Float weight = std::exp(Float(-2) * r2) - std::exp(Float(-2));
          V3 value = EvalNearest(V2(is * invR.x, it * invR.y));
          sum = sum + value * weight;
          sumWts += weight;
        }
      }
    }
    return sum / sumWts;
  }
};

// bitmap.cpp:263-344
struct BitmapTex final : Texture {
  std::unique_ptr<MipMap> mip;
  int filter = 1;  // 0 nearest, 1 bilinear, 2 trilinear, 3 anisotropic
  Float anisoLevel = 0;
  V3 Eval(const TexSi& si) const override {
    switch (filter) {
      case 0: return mip->EvalNearest(si.uv);
      case 1: return mip->EvalBilinear(si.uv);
      case 2: return mip->EvalTrilinear(si.uv, si.duvdx, si.duvdy);
      case 3: return mip->EvalAnisotropic(si.uv, si.duvdx, si.duvdy, anisoLevel);
      default: return V3(0);
    }
  }
  V3 Read(uint32_t x, uint32_t y) const override { return mip->mips[0].At(x, y, channels); }
};

// chessboard.cpp:15-63
struct ChessTex final : Texture {
  Transform transform;
  std::shared_ptr<Texture> a, b;
  bool remap = false;
  V3 Eval(const TexSi& si) const override {
    V3 t = transform.ApplyAffineToWorld(V3(si.uv.x, si.uv.y, 0));
    V2 tuv(t.x, t.y);
    V2 floorUV(std::floor(tuv.x), std::floor(tuv.y));
    V2 ab(tuv.x - floorUV.x, tuv.y - floorUV.y);
    bool isRight = ab.x > 0.5f;
    bool isUp = ab.y > 0.5f;
    TexSi tsi = si;
    if (isRight == isUp) {
      if (remap) tsi.uv = V2((tuv.x - Float(0.5)) * 2, (tuv.y - Float(0.5)) * 2);
      return a->Eval(tsi);
    }
    if (remap) tsi.uv = V2(tuv.x * 2, tuv.y * 2);
    return b->Eval(tsi);
  }
  V3 Read(uint32_t, uint32_t) const override { return V3(0); }
};

std::string ReadFileBytes(const std::string& path) {
  std::ifstream in(path, std::ios::binary);
  if (!in) throw std::runtime_error("cannot open " + path);
  std::stringstream ss;
  ss << in.rdbuf();
  return ss.str();
}

}  // namespace

std::shared_ptr<Texture> ConstTexture(const V3& v, int channels) {
  auto t = std::make_shared<ConstTex>();
  t->channels = channels;
  t->value = channels == 3 ? v : V3(v.x, 0, 0);
  return t;
}

// image_stb.cpp:48-104 (8-bit RGB / mono, /255, optional sRGB -> linear),
// image_hdr.cpp:33-57 and image_exr.cpp:29-94 (float RGB)
ImageAsset LoadImageAsset(const Json& cfg, const std::string& type, const std::string& path) {
  ImageAsset im;
  im.type = type;
  std::string bytes = ReadFileBytes(path);
  if (type == "image_default") {
    int ch = ReadI(&cfg, "channel", 3);
    bool flip = ReadB(&cfg, "is_flip_y", true);
    bool toLinear = ReadB(&cfg, "is_to_linear", ch == 3);
    if (ch != 1 && ch != 3) throw std::runtime_error("channel must be 1 or 3");
    rad::img::Ldr l = rad::img::LoadLdr(bytes, ch, flip);
    im.width = l.width;
    im.height = l.height;
    im.channels = ch;
    im.px.resize(l.px.size());
    for (size_t i = 0; i < l.px.size(); i++) {
      Float v = Float(l.px[i]) / 255;
      if (ch == 3 && toLinear)  // Color24f::ToLinear (color.h:41-46)
        v = v <= 0.04045f ? v * (1.0f / 12.92f) : std::pow((v + 0.055f) * (1.0f / 1.055f), 2.4f);
      im.px[i] = v;
    }
  } else if (type == "image_hdr") {
    rad::img::Hdr h = rad::img::LoadHdr(bytes, ReadB(&cfg, "is_flip_y", false));
    im.width = h.width;
    im.height = h.height;
    im.channels = 3;
    im.px = std::move(h.px);
  } else {
    rad::img::Hdr h = rad::img::LoadExr(bytes);
    im.width = h.width;
    im.height = h.height;
    im.channels = 3;
    im.px = std::move(h.px);
  }
  return im;
}

std::shared_ptr<Texture> MakeTexture(const Json& node, int channels, TexEnv* env) {
  if (node.is_number() || node.is_array()) {
    V3 v = channels == 3 ? JVec3(node) : V3((Float)JNum(node), 0, 0);
    auto t = ConstTexture(v, channels);
    if (env && env->created) env->created->push_back(t.get());
    return t;
  }
  if (!env || !env->images) throw std::runtime_error("textured parameters need a scene");
  std::string type = ReadS(&node, "type", "");
  if (type == "bitmap") {
    auto t = std::make_shared<BitmapTex>();
    t->channels = channels;
    if (env->created) env->created->push_back(t.get());
    const Json* an = node.find("asset_name");
    if (!an || an->kind != Json::String) throw std::runtime_error("no child: asset_name");
    auto it = env->images->find(an->str);
    if (it == env->images->end()) throw std::runtime_error("unknown asset: " + an->str);
    const ImageAsset& im = it->second;
    if (im.channels != channels) throw std::runtime_error("image asset channel count does not match");
    std::string f = ReadS(&node, "filter", "bilinear");
    t->filter = f == "nearest" ? 0 : f == "trilinear" ? 2 : f == "anisotropic" ? 3 : 1;
    int wrap = ReadS(&node, "wrap", "clamp") == "repeat" ? 1 : 0;
    bool enableMipMap = t->filter == 2 || t->filter == 3;
    int maxLevel = ReadI(&node, "max_level", enableMipMap ? -1 : 0);
    t->anisoLevel = ReadF(&node, "anisotropic_level", t->filter == 3 ? Float(8) : 0);
    t->width = (uint32_t)im.width;
    t->height = (uint32_t)im.height;
    if (!enableMipMap && maxLevel < 0) maxLevel = 0;
    Level l0;
    l0.w = (uint32_t)im.width;
    l0.h = (uint32_t)im.height;
    l0.px = im.px;
    t->mip = std::make_unique<MipMap>(std::move(l0), maxLevel, wrap, channels);
    return t;
  }
  if (type == "chessboard") {
    auto t = std::make_shared<ChessTex>();
    t->channels = channels;
    if (env->created) env->created->push_back(t.get());
    const Json* tu = node.find("to_uv");
    t->transform = Transform(tu ? JsonAsTransform(*tu) : M4::Identity());
    const Json* a = node.find("color_a");
    const Json* b = node.find("color_b");
    t->a = a ? MakeTexture(*a, channels, env) : MakeTexture(Json::Num(0.4f), channels, env);
    t->b = b ? MakeTexture(*b, channels, env) : MakeTexture(Json::Num(0.2f), channels, env);
    t->remap = ReadB(&node, "remap", false);
    return t;
  }
  throw std::runtime_error("cannot find factory: " + type);
}

}  // namespace orc
