// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_core.h).
// BSDF restatement: rad.offline/include/rad/offline/render/bsdf.h:10-142 and
// src/bsdf/{diffuse,rough_metal,rough_glass,disney,two_side,perfect_mirror,perfect_glass,
// plastic,rough_plastic,mask}.cpp.
#pragma once
#include <functional>

#include "ref_core.h"
#include "ref_texture.h"

namespace orc {

// bsdf.h:32-50
enum BsdfType : uint32_t {
  BT_Empty = 0,
  BT_Diffuse = 1,
  BT_Glossy = 2,
  BT_Delta = 4,
  BT_Reflection = 8,
  BT_Transmission = 16,
  BT_Null = 32,
  BT_All = 1 | 2 | 4 | 8 | 16,
  BT_NoDelta = 1 | 2,
};

struct BsdfSample {
  V3 Wo;
  Float Pdf = 0;
  Float Eta = 1;
  uint32_t Type = BT_Empty;
};

struct Bsdf;
// A textured parameter (ConfigNodeReadTexture, config_node_ext.h:17-45): the
// texture and how its value is written into a copy of the BSDF.
struct TexParam {
  std::shared_ptr<Texture> tex;
  std::function<void(Bsdf&, const V3&)> set;
};

// The integrators only ever use the default BsdfContext (Radiance, All lobes),
// path.cpp:139 and vol_path.cpp:38, so the context is not a parameter here.
// The reference evaluates a BSDF's textures inside Sample / Eval / Pdf at the
// SurfaceInteraction's UV; here the public calls take that UV (ts, null = no
// surface point) and run the constant-parameter code on a copy whose textured
// parameters hold the looked-up values -- the same values, in the same order
// of arithmetic.
struct Bsdf {
  uint32_t flags = 0;
  std::vector<TexParam> texParams;
  virtual ~Bsdf() = default;
  bool HasAnyTypeExceptDelta() const { return (flags & BT_NoDelta) != 0; }
  std::pair<BsdfSample, Spectrum> Sample(const V3& wi, Float lobeXi, const V2& dirXi, const TexSi* ts = nullptr) const {
    if (ts && !texParams.empty()) return Bound(*ts)->SampleImpl(wi, lobeXi, dirXi, ts);
    return SampleImpl(wi, lobeXi, dirXi, ts);
  }
  Spectrum Eval(const V3& wi, const V3& wo, const TexSi* ts = nullptr) const {
    if (ts && !texParams.empty()) return Bound(*ts)->EvalImpl(wi, wo, ts);
    return EvalImpl(wi, wo, ts);
  }
  Float Pdf(const V3& wi, const V3& wo, const TexSi* ts = nullptr) const {
    if (ts && !texParams.empty()) return Bound(*ts)->PdfImpl(wi, wo, ts);
    return PdfImpl(wi, wo, ts);
  }

 protected:
  virtual std::unique_ptr<Bsdf> Clone() const = 0;
  virtual std::pair<BsdfSample, Spectrum> SampleImpl(const V3& wi, Float lobeXi, const V2& dirXi,
                                                     const TexSi* ts) const = 0;
  virtual Spectrum EvalImpl(const V3& wi, const V3& wo, const TexSi* ts) const = 0;
  virtual Float PdfImpl(const V3& wi, const V3& wo, const TexSi* ts) const = 0;
  std::unique_ptr<Bsdf> Bound(const TexSi& ts) const {
    std::unique_ptr<Bsdf> b = Clone();
    for (const TexParam& p : texParams) p.set(*b, p.tex->Eval(ts));
    return b;
  }
  // An RGB / mono parameter: a constant is stored in the member, a texture is
  // recorded (the member is then filled per lookup). Returns the texture or null.
  template <class T>
  std::shared_ptr<Texture> ColorParam(const Json* cfg, const char* k, const V3& def, Spectrum T::*m, TexEnv* env) {
    const Json* j = cfg ? cfg->find(k) : nullptr;
    if (j && !(j->is_number() || j->is_array())) {
      TexParam p{MakeTexture(*j, 3, env), [m](Bsdf& b, const V3& v) { static_cast<T&>(b).*m = v; }};
      texParams.push_back(p);
      return p.tex;
    }
    static_cast<T*>(this)->*m = j ? JVec3(*j) : def;
    return nullptr;
  }
  template <class T>
  std::shared_ptr<Texture> MonoParam(const Json* cfg, const char* k, Float def, Float T::*m, TexEnv* env) {
    const Json* j = cfg ? cfg->find(k) : nullptr;
    if (j && !j->is_number()) {
      TexParam p{MakeTexture(*j, 1, env), [m](Bsdf& b, const V3& v) { static_cast<T&>(b).*m = v.x; }};
      texParams.push_back(p);
      return p.tex;
    }
    static_cast<T*>(this)->*m = j ? (Float)j->num : def;
    return nullptr;
  }
};

// Factory by the reference's names: diffuse, rough_metal, rough_glass, disney, two_side,
// perfect_mirror, perfect_glass, plastic, rough_plastic, mask. env: the scene's
// image assets (null: textured parameters are an error).
std::unique_ptr<Bsdf> MakeBsdf(const Json* cfg, TexEnv* env = nullptr);

// Warps: rad.offline/src/warp.cpp:10-99
V2 SquareToUniformDisk(const V2& u);
V3 SquareToCosineHemisphere(const V2& u);
Float SquareToCosineHemispherePdf(const V3& v);
V2 SquareToUniformTriangle(const V2& u);
V3 SquareToUniformSphere(const V2& u);
Float SquareToUniformSpherePdf();
Float SquareToUniformConePdf(Float cosCutoff);

// Fresnel: rad.offline/src/fresnel.cpp:10-84
V3 FresnelReflect(const V3& wi, const V3& wh);
V3 FresnelRefract(const V3& wi, const V3& wh, Float cosThetaT, Float etaTI);
void FresnelDielectric(Float cosThetaI, Float eta, Float& r, Float& cosThetaT, Float& etaIT, Float& etaTI);
Spectrum FresnelConductor(Float cosThetaI, const Spectrum& eta, const Spectrum& k);

// Microfacet distributions: rad.offline/src/microfacet.cpp:12-285 (mitsuba variant)
struct Microfacet {
  bool ggx = true;
  Float alphaX = 0.1f, alphaY = 0.1f;
  bool sampleVisible = true;
  Float D(const V3& wh) const;
  Float SmithG1(const V3& v, const V3& wh) const;
  Float G(const V3& wi, const V3& wo, const V3& wh) const { return SmithG1(wi, wh) * SmithG1(wo, wh); }
  Float Pdf(const V3& wi, const V3& wh) const;
  std::pair<V3, Float> Sample(const V3& wi, const V2& xi) const;
};

}  // namespace orc
