// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_core.h).
// BSDF restatement: rad.offline/include/rad/offline/render/bsdf.h:10-142 and
// src/bsdf/{diffuse,rough_metal,rough_glass,disney,two_side,perfect_mirror,perfect_glass,
// plastic,rough_plastic,mask}.cpp.
#pragma once
#include "ref_core.h"

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

// The integrators only ever use the default BsdfContext (Radiance, All lobes),
// path.cpp:139 and vol_path.cpp:38, so the context is not a parameter here.
struct Bsdf {
  uint32_t flags = 0;
  virtual ~Bsdf() = default;
  bool HasAnyTypeExceptDelta() const { return (flags & BT_NoDelta) != 0; }
  virtual std::pair<BsdfSample, Spectrum> Sample(const V3& wi, Float lobeXi, const V2& dirXi) const = 0;
  virtual Spectrum Eval(const V3& wi, const V3& wo) const = 0;
  virtual Float Pdf(const V3& wi, const V3& wo) const = 0;
};

// Factory by the reference's names: diffuse, rough_metal, rough_glass, disney, two_side,
// perfect_mirror, perfect_glass, plastic, rough_plastic, mask.
std::unique_ptr<Bsdf> MakeBsdf(const Json* cfg);

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
