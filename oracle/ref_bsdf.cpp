// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_core.h).
#include "ref_bsdf.h"

#include <algorithm>

namespace orc {

// ---------------------------------------------------------------- warps
// warp.cpp:22-27
V2 SquareToUniformDisk(const V2& u) {
  Float r = std::sqrt(u.x);
  Float angle = 2 * PI * u.y;
  return V2(r * std::cos(angle), r * std::sin(angle));
}
// warp.cpp:33-47 (the live #else branch)
V3 SquareToCosineHemisphere(const V2& u) {
  V2 bottom = SquareToUniformDisk(u);
  Float x = bottom.x, y = bottom.y;
  Float z = SafeSqrt(1 - Sqr(x) - Sqr(y));
  return V3(x, y, z);
}
// warp.cpp:48-50
Float SquareToCosineHemispherePdf(const V3& v) { return v.z * (1 / PI); }
// warp.cpp:52-55
V2 SquareToUniformTriangle(const V2& u) {
  Float t = SafeSqrt(1 - u.x);
  return V2(1 - t, t * u.y);
}
// warp.cpp:60-66
V3 SquareToUniformSphere(const V2& u) {
  Float z = Fmadd(-2, u.y, 1);
  Float r = SafeSqrt(Fmadd(-z, z, 1));
  Float a = 2 * PI * u.x;
  Float s = std::sin(a), c = std::cos(a);
  return V3(r * c, r * s, z);
}
// warp.cpp:67-69
Float SquareToUniformSpherePdf() { return 1 / (4 * PI); }
// warp.cpp:78-80
Float SquareToUniformConePdf(Float cosCutoff) { return 1 / (2 * PI) / (1 - cosCutoff); }

// -------------------------------------------------------------- fresnel
// fresnel.cpp:14-16
V3 FresnelReflect(const V3& wi, const V3& wh) {
  Float k = 2 * dot(wi, wh);
  return Fmadd(wh, V3(k), -wi);
}
// fresnel.cpp:22-24
V3 FresnelRefract(const V3& wi, const V3& wh, Float cosThetaT, Float etaTI) {
  Float k = Fmadd(dot(wi, wh), etaTI, cosThetaT);
  return Fmadd(wh, V3(k), -(wi * etaTI));
}
// fresnel.cpp:38-59
void FresnelDielectric(Float cosThetaI, Float eta, Float& r, Float& cosThetaT, Float& etaIT, Float& etaTI) {
  bool isOutside = cosThetaI >= 0;
  Float rcpEta = Rcp(eta);
  etaIT = isOutside ? eta : rcpEta;
  etaTI = isOutside ? rcpEta : eta;
  Float sqrCosThetaT = Fmadd(-Fmadd(-cosThetaI, cosThetaI, 1), etaTI * etaTI, 1);
  Float absCosThetaI = std::abs(cosThetaI);
  Float absCosThetaT = SafeSqrt(sqrCosThetaT);
  bool indexMatched = eta == 1;
  bool specialCase = indexMatched || absCosThetaI == 0;
  Float rSC = indexMatched ? Float(0.f) : Float(1.f);
  Float aS = Fmadd(-etaIT, absCosThetaT, absCosThetaI) / Fmadd(etaIT, absCosThetaT, absCosThetaI);
  Float aP = Fmadd(-etaIT, absCosThetaI, absCosThetaT) / Fmadd(etaIT, absCosThetaI, absCosThetaT);
  r = Float(0.5) * (Sqr(aS) + Sqr(aP));
  if (specialCase) r = rSC;
  cosThetaT = cosThetaI >= 0 ? -absCosThetaT : absCosThetaT;
}
// fresnel.cpp:61-77
Spectrum FresnelConductor(Float cosThetaI, const Spectrum& eta, const Spectrum& k) {
  Float cosThetaI2 = cosThetaI * cosThetaI, sinThetaI2 = Float(1) - cosThetaI2,
        sinThetaI4 = sinThetaI2 * sinThetaI2;
  Spectrum out;
  for (int c = 0; c < 3; c++) {
    Float etaR = eta[c], etaI = k[c];
    Float temp1 = etaR * etaR - etaI * etaI - sinThetaI2;
    Float a2pb2 = temp1 * temp1 + etaI * etaI * etaR * etaR * 4;
    a2pb2 = std::sqrt(std::max(a2pb2, Float(0)));
    Float a = std::sqrt(std::max((a2pb2 + temp1) * Float(0.5), Float(0)));
    Float term1 = a2pb2 + cosThetaI2;
    Float term2 = a * 2 * cosThetaI;
    Float rs = (term1 - term2) * (1 / (term1 + term2));
    Float term3 = a2pb2 * cosThetaI2 + sinThetaI4;
    Float term4 = term2 * sinThetaI2;
    Float rp = rs * (term3 - term4) * (1 / (term3 + term4));
    out[c] = (rs + rp) * Float(0.5);
  }
  return out;
}

// ----------------------------------------------------------- microfacet
// Beckmann ErfInv polynomial: math_ext.h:116-142 (reference source).
static Float ErfInv(Float a) {
  float p;
  float t = (float)std::log(std::max(Fmadd(a, -a, 1), std::numeric_limits<Float>::min()));
  if (std::abs(t) > 6.125f) {
    p = 3.03697567e-10f;
    p = Fmadd(p, t, 2.93243101e-8f);
    p = Fmadd(p, t, 1.22150334e-6f);
    p = Fmadd(p, t, 2.84108955e-5f);
    p = Fmadd(p, t, 3.93552968e-4f);
    p = Fmadd(p, t, 3.02698812e-3f);
    p = Fmadd(p, t, 4.83185798e-3f);
    p = Fmadd(p, t, -2.64646143e-1f);
    p = Fmadd(p, t, 8.40016484e-1f);
  } else {
    p = 5.43877832e-9f;
    p = Fmadd(p, t, 1.43286059e-7f);
    p = Fmadd(p, t, 1.22775396e-6f);
    p = Fmadd(p, t, 1.12962631e-7f);
    p = Fmadd(p, t, -5.61531961e-5f);
    p = Fmadd(p, t, -1.47697705e-4f);
    p = Fmadd(p, t, 2.31468701e-3f);
    p = Fmadd(p, t, 1.15392562e-2f);
    p = Fmadd(p, t, -2.32015476e-1f);
    p = Fmadd(p, t, 8.86226892e-1f);
  }
  return a * p;
}

Float Microfacet::D(const V3& wh) const {
  Float alphaXY = alphaX * alphaY;
  Float cosTheta = wh.z;
  if (ggx) {  // microfacet.cpp:149-154
    Float result = Rcp(PI * alphaXY * Sqr(Sqr(wh.x / alphaX) + Sqr(wh.y / alphaY) + Sqr(wh.z)));
    return result * cosTheta > 1e-20f ? result : 0;
  }
  // microfacet.cpp:20-26
  Float cosTheta2 = Sqr(cosTheta);
  Float result = std::exp(-(Sqr(wh.x / alphaX) + Sqr(wh.y / alphaY)) / cosTheta2) / (PI * alphaXY * Sqr(cosTheta2));
  return result * cosTheta > 1e-20f ? result : 0;
}

Float Microfacet::SmithG1(const V3& v, const V3& wh) const {
  Float xyAlpha2 = Sqr(alphaX * v.x) + Sqr(alphaY * v.y);
  Float tanThetaAlpha2 = xyAlpha2 / Sqr(v.z);
  Float result;
  if (ggx) {  // microfacet.cpp:180-190
    result = 2 / (1 + std::sqrt(1 + tanThetaAlpha2));
  } else {  // microfacet.cpp:53-63
    Float a = Rsqrt(tanThetaAlpha2);
    Float aSqr = Sqr(a);
    result = a >= 1.6f ? 1.f : (3.535f * a + 2.181f * aSqr) / (1.f + 2.276f * a + 2.577f * aSqr);
  }
  if (xyAlpha2 == 0) result = 1;
  if (dot(v, wh) * v.z <= 0) result = 0;
  return result;
}

// microfacet.cpp:70-78 / 198-206
Float Microfacet::Pdf(const V3& wi, const V3& wh) const {
  Float result = D(wh);
  if (sampleVisible) {
    result *= SmithG1(wi, wh) * AbsDot(wi, wh) / wi.z;
  } else {
    result *= wh.z;
  }
  return result;
}

// microfacet.cpp:208-243 (PBRT's visible-slope sampler, float math)
static V2 SampleVisibleGGX(Float cosThetaI, V2 sample) {
  if (cosThetaI > 0.9999) {
    Float r = std::sqrt(sample.x / (1 - sample.x));
    Float phi = Float(6.28318530718) * sample.y;
    return V2(r * std::cos(phi), r * std::sin(phi));
  }
  Float sinTheta = std::sqrt(std::max((Float)0, (Float)1 - Sqr(cosThetaI)));
  Float tanTheta = sinTheta / cosThetaI;
  Float a = 1 / tanTheta;
  Float G1 = 2 / (1 + std::sqrt(1 + 1 / Sqr(a)));
  Float A = 2 * sample.x / G1 - 1;
  Float tmp = 1.f / Fmadd(A, A, -1);
  if (tmp > 1e10) tmp = Float(1e10);
  Float B = tanTheta;
  Float Dd = std::sqrt(std::max(Float(Sqr(B) * Sqr(tmp) - (Sqr(A) - Sqr(B)) * tmp), Float(0)));
  Float slopeX1 = Fmadd(B, tmp, -Dd);
  Float slopeX2 = Fmadd(B, tmp, Dd);
  Float slopeX = (A < 0 || slopeX2 > 1 / tanTheta) ? slopeX1 : slopeX2;
  Float S;
  if (sample.y > 0.5f) {
    S = 1;
    sample.y = 2 * (sample.y - Float(0.5));
  } else {
    S = -1;
    sample.y = 2 * (Float(0.5) - sample.y);
  }
  Float z = (sample.y * (sample.y * (sample.y * 0.27385f - 0.73369f) + 0.46341f)) /
            (sample.y * (sample.y * (sample.y * 0.093073f + 0.309420f) - 1) + 0.597999f);
  Float slopeY = S * z * std::sqrt(1 + slopeX * slopeX);
  return V2(slopeX, slopeY);
}

// microfacet.cpp:80-97 (mitsuba visible Beckmann sampler)
static V2 SampleVisibleBeckmann(Float cosThetaI, V2 sample) {
  Float tanThetaI = SafeSqrt(Fmadd(-cosThetaI, cosThetaI, Float(1))) / cosThetaI;
  Float cotThetaI = Rcp(tanThetaI);
  Float maxval = std::erf(cotThetaI);
  // cwiseMin(1 - 1e-6) then cwiseMax(1e-6)
  sample.x = std::max(std::min(sample.x, Float(1 - 1e-6)), Float(1e-6));
  sample.y = std::max(std::min(sample.y, Float(1 - 1e-6)), Float(1e-6));
  Float x = maxval - (maxval + 1) * std::erf(std::sqrt(-std::log(sample.x)));
  sample.x *= 1 + maxval + (1 / std::sqrt(PI)) * tanThetaI * std::exp(-Sqr(cotThetaI));
  for (int i = 0; i < 3; i++) {
    Float slope = ErfInv(x);
    Float value = 1 + x + (1 / std::sqrt(PI)) * tanThetaI * std::exp(-Sqr(slope)) - sample.x;
    Float derivative = 1 - slope * tanThetaI;
    x -= value / derivative;
  }
  return V2(ErfInv(x), ErfInv(Fmadd(Float(2), sample.y, Float(-1))));
}

// microfacet.cpp:99-136 / 245-277
std::pair<V3, Float> Microfacet::Sample(const V3& wi, const V2& xi) const {
  if (sampleVisible) {
    V3 wiP = normalized(V3(alphaX * wi.x, alphaY * wi.y, wi.z));
    Float sinPhi, cosPhi;
    Frame::SinCosPhi(wiP, sinPhi, cosPhi);
    Float cosTheta = wiP.z;
    V2 slope = ggx ? SampleVisibleGGX(cosTheta, xi) : SampleVisibleBeckmann(cosTheta, xi);
    slope = V2(Fmadd(cosPhi, slope.x, -(sinPhi * slope.y)) * alphaX,
               Fmadd(sinPhi, slope.x, cosPhi * slope.y) * alphaY);
    V3 m = normalized(V3(-slope.x, -slope.y, 1));
    Float pdf = D(m) * SmithG1(wi, m) * AbsDot(wi, m) / wi.z;
    return {m, pdf};
  }
  Float sinPhi, cosPhi, alpha2;
  if (alphaX == alphaY) {
    Float a = (2 * PI) * xi.y;
    sinPhi = std::sin(a);
    cosPhi = std::cos(a);
    alpha2 = alphaX * alphaY;
  } else {
    Float ratio = alphaY / alphaX;
    Float tmp = ratio * std::tan((2 * PI) * xi.y);
    cosPhi = Rsqrt(Fmadd(tmp, tmp, 1));
    cosPhi = MulSign(cosPhi, std::abs(xi.y - Float(0.5)) - Float(0.25));
    sinPhi = cosPhi * tmp;
    alpha2 = Rcp(Sqr(cosPhi / alphaX) + Sqr(sinPhi / alphaY));
  }
  Float cosTheta, pdf;
  if (ggx) {
    Float tanThetaM2 = alpha2 * xi.x / (1.f - xi.x);
    cosTheta = Rsqrt(1.f + tanThetaM2);
    Float cos2Theta = Sqr(cosTheta);
    Float temp = 1 + tanThetaM2 / alpha2;
    Float cos3Theta = std::max(cos2Theta * cosTheta, Float(1e-20));
    pdf = Rcp(PI * alphaX * alphaY * cos3Theta * Sqr(temp));
  } else {
    cosTheta = Rsqrt(Fmadd(-alpha2, std::log(1 - xi.x), 1));
    Float cos2Theta = Sqr(cosTheta);
    Float cos3Theta = std::max(cos2Theta * cosTheta, Float(1e-20));
    pdf = (1.f - xi.x) / (PI * alphaX * alphaY * cos3Theta);
  }
  Float sinTheta = std::sqrt(1 - Sqr(cosTheta));
  return {V3(cosPhi * sinTheta, sinPhi * sinTheta, cosTheta), pdf};
}

// ----------------------------------------------------------------- helpers
// Microfacet parameters (rough_metal.cpp:30-45, rough_glass.cpp:35-50) with
// textured alpha / alpha_u / alpha_v recorded as TexParams of the owning BSDF.
template <class T>
static void DistParam(T* self, const Json* cfg, Microfacet T::*m, TexEnv* env) {
  Microfacet& d = self->*m;
  std::string dist = ReadS(cfg, "distribution", "ggx");
  d.ggx = dist != "beckmann";
  auto alpha = [&](const char* k, int which) {
    const Json* j = cfg ? cfg->find(k) : nullptr;
    if (j && !j->is_number()) {
      self->texParams.push_back(TexParam{MakeTexture(*j, 1, env), [m, which](Bsdf& b, const V3& v) {
                                           Microfacet& x = static_cast<T&>(b).*m;
                                           if (which != 2) x.alphaX = v.x;
                                           if (which != 1) x.alphaY = v.x;
                                         }});
      return;
    }
    Float a = j ? (Float)j->num : Float(0.1f);
    if (which != 2) d.alphaX = a;
    if (which != 1) d.alphaY = a;
  };
  if (cfg && cfg->has("alpha")) {
    alpha("alpha", 0);
  } else {
    alpha("alpha_u", 1);
    alpha("alpha_v", 2);
  }
  d.sampleVisible = ReadB(cfg, "sample_visible", true);
}

// ----------------------------------------------------------------- diffuse
// diffuse.cpp:46-99
struct DiffuseBsdf final : Bsdf {
  Spectrum R;
  explicit DiffuseBsdf(const Json* cfg, TexEnv* env) {
    flags = BT_Diffuse | BT_Reflection;
    ColorParam(cfg, "reflectance", V3(0.5f), &DiffuseBsdf::R, env);
  }
  std::unique_ptr<Bsdf> Clone() const override { return std::make_unique<DiffuseBsdf>(*this); }
  std::pair<BsdfSample, Spectrum> SampleImpl(const V3& wi, Float, const V2& dirXi, const TexSi*) const override {
    Float cosThetaI = wi.z;
    if (cosThetaI <= 0) return {{}, Spectrum(0)};
    BsdfSample bsr;
    bsr.Wo = SquareToCosineHemisphere(dirXi);
    bsr.Pdf = SquareToCosineHemispherePdf(bsr.Wo);
    bsr.Eta = 1;
    bsr.Type = flags;
    Float cosThetaO = bsr.Wo.z;
    return {bsr, R * (1 / PI) * cosThetaO};
  }
  Spectrum EvalImpl(const V3& wi, const V3& wo, const TexSi*) const override {
    if (wi.z <= 0 || wo.z <= 0) return Spectrum(0);
    return R * (1 / PI) * wo.z;
  }
  Float PdfImpl(const V3& wi, const V3& wo, const TexSi*) const override {
    if (wi.z <= 0 || wo.z <= 0) return 0;
    return SquareToCosineHemispherePdf(wo);
  }
};

// ------------------------------------------------------------ rough_metal
// rough_metal.cpp:22-176
struct RoughMetalBsdf final : Bsdf {
  Spectrum R, eta, k;
  Microfacet dist;
  explicit RoughMetalBsdf(const Json* cfg, TexEnv* env) {
    flags = BT_Glossy | BT_Reflection;
    ColorParam(cfg, "reflectance", V3(1), &RoughMetalBsdf::R, env);
    ColorParam(cfg, "eta", V3(0.1999899f, 0.9220823f, 1.0998751f), &RoughMetalBsdf::eta, env);
    ColorParam(cfg, "k", V3(3.9046354f, 2.4476316f, 2.1376500f), &RoughMetalBsdf::k, env);
    DistParam(this, cfg, &RoughMetalBsdf::dist, env);
  }
  std::unique_ptr<Bsdf> Clone() const override { return std::make_unique<RoughMetalBsdf>(*this); }
  std::pair<BsdfSample, Spectrum> SampleImpl(const V3& wi, Float, const V2& dirXi, const TexSi*) const override {
    Float cosThetaI = wi.z;
    if (cosThetaI <= 0) return {{}, Spectrum(0)};
    BsdfSample bsr;
    auto mp = dist.Sample(wi, dirXi);
    V3 m = mp.first;
    bsr.Pdf = mp.second;
    bsr.Wo = FresnelReflect(wi, m);
    bsr.Eta = 1;
    bsr.Type = flags;
    if (bsr.Pdf <= 0 || bsr.Wo.z <= 0) return {{}, Spectrum(0)};
    bsr.Pdf /= 4 * dot(bsr.Wo, m);
    Float Dv = dist.D(m);
    Float Gv = dist.G(wi, bsr.Wo, m);
    Spectrum F = FresnelConductor(dot(wi, m), eta, k);
    Float denom = 4 * wi.z * bsr.Wo.z;
    Spectrum brdf((F.x * Dv * Gv) / denom, (F.y * Dv * Gv) / denom, (F.z * Dv * Gv) / denom);
    return {bsr, cmul(R, brdf) * bsr.Wo.z};
  }
  Spectrum EvalImpl(const V3& wi, const V3& wo, const TexSi*) const override {
    Float cosThetaI = wi.z, cosThetaO = wo.z;
    if (cosThetaI <= 0 || cosThetaO <= 0) return Spectrum(0);
    V3 wh = normalized(wo + wi);
    Spectrum F = FresnelConductor(dot(wi, wh), eta, k);
    Float Dv = dist.D(wh);
    Float Gv = dist.G(wi, wo, wh);
    Float denom = cosThetaI * cosThetaO * 4;
    Spectrum brdf(std::abs(F.x * Dv * Gv) / denom, std::abs(F.y * Dv * Gv) / denom,
                  std::abs(F.z * Dv * Gv) / denom);
    return cmul(R, brdf) * cosThetaO;
  }
  Float PdfImpl(const V3& wi, const V3& wo, const TexSi*) const override {
    if (wi.z <= 0 || wo.z <= 0) return 0;
    V3 wh = normalized(wo + wi);
    return dist.Pdf(wi, wh) / (4 * dot(wo, wh));
  }
};

// ------------------------------------------------------------ rough_glass
// rough_glass.cpp:22-221
struct RoughGlassBsdf final : Bsdf {
  Spectrum R, T;
  Float eta, invEta;
  Microfacet dist;
  explicit RoughGlassBsdf(const Json* cfg, TexEnv* env) {
    flags = BT_Glossy | BT_Reflection | BT_Transmission;
    ColorParam(cfg, "reflectance", V3(1), &RoughGlassBsdf::R, env);
    ColorParam(cfg, "transmittance", V3(1), &RoughGlassBsdf::T, env);
    Float intIor = ReadF(cfg, "int_ior", Float(1.5046));
    Float extIor = ReadF(cfg, "ext_ior", Float(1.000277));
    eta = intIor / extIor;
    invEta = extIor / intIor;
    DistParam(this, cfg, &RoughGlassBsdf::dist, env);
  }
  std::unique_ptr<Bsdf> Clone() const override { return std::make_unique<RoughGlassBsdf>(*this); }
  std::pair<BsdfSample, Spectrum> SampleImpl(const V3& wi, Float lobeXi, const V2& dirXi, const TexSi* ts) const override {
    BsdfSample bsr;
    Float cosThetaI = wi.z;
    if (cosThetaI == 0) return {{}, Spectrum(0)};
    auto mp = dist.Sample(MulSign(wi, cosThetaI), dirXi);
    V3 wh = mp.first;
    if (mp.second == 0) return {{}, Spectrum(0)};
    Float F, cosThetaT, etaIT, etaTI;
    FresnelDielectric(dot(wi, wh), eta, F, cosThetaT, etaIT, etaTI);
    bool selectedR = lobeXi <= F;
    bsr.Wo = selectedR ? FresnelReflect(wi, wh) : FresnelRefract(wi, wh, cosThetaT, etaTI);
    bool isReflect = Frame::IsSameHemisphere(wi, bsr.Wo);
    bsr.Eta = isReflect ? 1 : etaIT;
    bsr.Type = BT_Glossy | (isReflect ? BT_Reflection : BT_Transmission);
    bsr.Pdf = PdfImpl(wi, bsr.Wo, ts);
    if (bsr.Pdf <= 0) return {{}, Spectrum(0)};
    return {bsr, EvalImpl(wi, bsr.Wo, ts)};
  }
  Spectrum EvalImpl(const V3& wi, const V3& wo, const TexSi* ts) const override {
    Float cosThetaI = wi.z, cosThetaO = wo.z;
    if (cosThetaI == 0) return Spectrum(0);
    bool reflect = cosThetaI * cosThetaO > 0;
    Float e = cosThetaI > 0 ? eta : invEta;
    Float ie = cosThetaI > 0 ? invEta : eta;
    V3 m = normalized(wi + wo * (reflect ? 1 : e));
    m = MulSign(m, m.z);
    Float Dv = dist.D(m);
    Float F, cT, eIT, eTI;
    FresnelDielectric(dot(wi, m), eta, F, cT, eIT, eTI);
    Float Gv = dist.G(wi, wo, m);
    Spectrum result(0);
    if (reflect) {
      Float brdf = std::abs(F * Dv * Gv / (cosThetaI * 4));
      result = R * brdf;
    } else {
      Float scale = (ts && ts->importance) ? Float(1) : Sqr(ie);  // rough_glass.cpp:143
      Float idm = dot(wi, m);
      Float odm = dot(wo, m);
      Float btdf = std::abs((scale * (1 - F) * Dv * Gv * e * e * idm * odm) / (cosThetaI * Sqr(idm + e * odm)));
      result = T * btdf;
    }
    return result;
  }
  Float PdfImpl(const V3& wi, const V3& wo, const TexSi*) const override {
    Float cosThetaI = wi.z, cosThetaO = wo.z;
    if (cosThetaI == 0) return 0;
    bool reflect = cosThetaI * cosThetaO > 0;
    Float e = cosThetaI > 0 ? eta : invEta;
    V3 m = normalized(wi + wo * (reflect ? 1 : e));
    m = MulSign(m, m.z);
    Float idm = dot(wi, m);
    Float odm = dot(wo, m);
    if (idm * cosThetaI <= 0 || odm * cosThetaO <= 0) return 0;
    Float dwhdwo = reflect ? Rcp(odm * 4) : ((e * e * odm) / (Sqr(idm + e * odm)));
    Float pdf = dist.Pdf(MulSign(wi, cosThetaI), m);
    Float F, cT, eIT, eTI;
    FresnelDielectric(idm, eta, F, cT, eIT, eTI);
    pdf *= reflect ? F : (1 - F);
    return std::abs(pdf * dwhdwo);
  }
};

// ----------------------------------------------------------------- disney
// disney.cpp:28-642
struct DisneyBsdf final : Bsdf {
  Spectrum baseColor;
  Float roughness, anisotropic, specTrans, sheen, sheenTint, flatness, specTint, metallic, clearcoat,
      clearcoatGloss;
  Float eta, specularSample, clearcoatSample, diffuseReflectSample;
  bool hasClearcoat, hasSheen, hasSpecTrans, hasMetallic, hasSpecTint, hasSheenTint, hasAnisotropic,
      hasFlatness;

  // disney.cpp:459-471: a key counts as present when it exists and is not the number 0.
  static bool HasValue(const Json* cfg, const char* k) {
    const Json* j = cfg ? cfg->find(k) : nullptr;
    if (!j) return false;
    if (j->is_number()) return (Float)j->num != 0;
    return true;
  }

  explicit DisneyBsdf(const Json* cfg, TexEnv* env) {
    ColorParam(cfg, "base_color", V3(0.5f), &DisneyBsdf::baseColor, env);
    MonoParam(cfg, "roughness", 0.5f, &DisneyBsdf::roughness, env);
    hasAnisotropic = HasValue(cfg, "anisotropic");
    MonoParam(cfg, "anisotropic", 0, &DisneyBsdf::anisotropic, env);
    hasSpecTrans = HasValue(cfg, "spec_trans");
    MonoParam(cfg, "spec_trans", 0, &DisneyBsdf::specTrans, env);
    hasSheen = HasValue(cfg, "sheen");
    MonoParam(cfg, "sheen", 0, &DisneyBsdf::sheen, env);
    hasSheenTint = HasValue(cfg, "sheen_tint");
    MonoParam(cfg, "sheen_tint", 0, &DisneyBsdf::sheenTint, env);
    hasFlatness = HasValue(cfg, "flatness");
    MonoParam(cfg, "flatness", 0, &DisneyBsdf::flatness, env);
    hasSpecTint = HasValue(cfg, "spec_tint");
    MonoParam(cfg, "spec_tint", 0, &DisneyBsdf::specTint, env);
    hasMetallic = HasValue(cfg, "metallic");
    MonoParam(cfg, "metallic", 0, &DisneyBsdf::metallic, env);
    hasClearcoat = HasValue(cfg, "clearcoat");
    MonoParam(cfg, "clearcoat", 0, &DisneyBsdf::clearcoat, env);
    MonoParam(cfg, "clearcoat_gloss", 0, &DisneyBsdf::clearcoatGloss, env);
    specularSample = ReadF(cfg, "main_specular_sampling_rate", 1);
    clearcoatSample = ReadF(cfg, "clearcoat_sampling_rate", 1);
    diffuseReflectSample = ReadF(cfg, "diffuse_reflectance_sampling_rate", 1);
    bool hasEta = cfg && cfg->has("eta");
    bool hasSpecular = cfg && cfg->has("specular");
    if (hasEta && hasSpecular) throw std::runtime_error("eta cannot set with specular at same time");
    if (hasEta) {
      eta = ReadF(cfg, "eta", 1.5f);
      if (hasSpecTrans && eta == Float(1)) eta = Float(1.001);
    } else {
      Float specular = ReadF(cfg, "specular", 0.5f);
      if (hasSpecTrans && specular == Float(0)) specular = Float(0.001);
      eta = Float(2) * Rcp(Float(1) - std::sqrt(Float(0.08) * specular)) - Float(1);
    }
    flags = BT_Diffuse | BT_Reflection;
    if (hasClearcoat) flags |= BT_Glossy;
    if (hasSpecTrans) flags |= BT_Transmission;
  }
  std::unique_ptr<Bsdf> Clone() const override { return std::make_unique<DisneyBsdf>(*this); }

  // disney.cpp:474-486
  void RoughnessToAlpha(Float& ax, Float& ay) const {
    Float roughness2 = Sqr(roughness);
    if (!hasAnisotropic) {
      Float a = std::max(Float(0.001), roughness2);
      ax = ay = a;
      return;
    }
    Float aspect = std::sqrt(Float(1) - Float(0.9) * anisotropic);
    ax = std::max(Float(0.001), roughness2 / aspect);
    ay = std::max(Float(0.001), roughness2 * aspect);
  }
  // disney.cpp:488-500
  static bool CheckMacMicNormal(const V3& m, const V3& wi, const V3& wo, Float cosThetaI, bool reflection) {
    if (reflection) {
      return (dot(wi, MulSign(m, cosThetaI)) > Float(0)) && (dot(wo, MulSign(m, cosThetaI)) > Float(0));
    }
    return (dot(wi, MulSign(m, cosThetaI)) > Float(0)) && (dot(wo, cosThetaI >= 0 ? -m : m) > Float(0));
  }
  // disney.cpp:502-505
  static Float SchlickWeight(Float cosI) {
    Float m = std::clamp(Float(1) - cosI, Float(0), Float(1));
    return Sqr(Sqr(m)) * m;
  }
  // disney.cpp:514-525
  static Float SchlickF(Float R0, Float cosThetaI, Float eta) {
    bool isOutside = cosThetaI >= Float(0);
    Float rcpEta = Rcp(eta);
    Float etaIT = isOutside ? eta : rcpEta;
    Float etaTI = isOutside ? rcpEta : eta;
    Float sqrCosThetaT = Fmadd(-Fmadd(-cosThetaI, cosThetaI, Float(1)), Sqr(etaTI), Float(1));
    Float cosThetaT = SafeSqrt(sqrCosThetaT);
    return etaIT > Float(1) ? Lerp(SchlickWeight(std::abs(cosThetaI)), Float(1), R0)
                            : Lerp(SchlickWeight(cosThetaT), Float(1), R0);
  }
  // disney.cpp:534-545; LerpSpectrum(a, b, t) = a + t .* (b - a) (spectrum.h:72-74)
  static Spectrum SchlickF(const Spectrum& R0, Float cosThetaI, Float eta) {
    bool isOutside = cosThetaI >= Float(0);
    Float rcpEta = Rcp(eta);
    Float etaIT = isOutside ? eta : rcpEta;
    Float etaTI = isOutside ? rcpEta : eta;
    Float sqrCosThetaT = Fmadd(-Fmadd(-cosThetaI, cosThetaI, Float(1)), Sqr(etaTI), Float(1));
    Float cosThetaT = SafeSqrt(sqrCosThetaT);
    Float w = etaIT > Float(1) ? SchlickWeight(std::abs(cosThetaI)) : SchlickWeight(cosThetaT);
    return Spectrum(w + R0.x * (Float(1) - w), w + R0.y * (Float(1) - w), w + R0.z * (Float(1) - w));
  }
  static Float SchlickR0Eta(Float eta) { return Sqr((eta - Float(1)) / (eta + Float(1))); }
  // disney.cpp:567-590
  Spectrum DisneyFresnel(Float dielectricF, Float lum, Float cosThetaI, bool isFrontSide, Float bsdf) const {
    bool isOutside = cosThetaI >= Float(0);
    Float rcpEta = Rcp(eta);
    Float etaIT = isOutside ? eta : rcpEta;
    Spectrum schlickF(0);
    if (hasMetallic) schlickF = schlickF + metallic * SchlickF(baseColor, cosThetaI, eta);
    Float st = hasSpecTint ? specTint : Float(0);
    if (hasSpecTint) {
      Spectrum cTint = lum > Float(0) ? baseColor / lum : Spectrum(1);
      Spectrum F0 = cTint * SchlickR0Eta(etaIT);
      schlickF = schlickF + (Float(1) - metallic) * st * SchlickF(F0, cosThetaI, eta);
    }
    Float fd = (Float(1) - metallic) * (Float(1) - st) * dielectricF;
    Spectrum frontF = Spectrum(fd) + schlickF;
    return isFrontSide ? frontF : Spectrum(bsdf * dielectricF);
  }
  // disney.cpp:592-612
  static Float SmithGGX1(const V3& v, const V3& wh, Float alpha) {
    Float alpha2 = Sqr(alpha);
    Float cosTheta = std::abs(v.z);
    Float cosTheta2 = Sqr(cosTheta);
    Float tanTheta2 = (Float(1) - cosTheta2) / cosTheta2;
    Float result = Float(2) * Rcp(Float(1) + std::sqrt(Float(1) + alpha2 * tanTheta2));
    if (v.z == 1) result = 1;
    if (dot(v, wh) * v.z <= Float(0)) result = Float(0);
    return result;
  }
  static Float ClearcoatG(const V3& wi, const V3& wo, const V3& wh, Float alpha) {
    return SmithGGX1(wi, wh, alpha) * SmithGGX1(wo, wh, alpha);
  }
  // GTR1, disney.cpp:37-60
  struct GTR1 {
    Float alpha;
    V3 Sample(const V2& xi) const {
      Float a = (Float(2) * PI) * xi.x;
      Float sinPhi = std::sin(a), cosPhi = std::cos(a);
      Float alpha2 = Sqr(alpha);
      Float cosTheta2 = (Float(1) - std::pow(alpha2, Float(1) - xi.y)) / (Float(1) - alpha2);
      Float sinTheta = std::sqrt(std::max(Float(0), Float(1) - cosTheta2));
      Float cosTheta = std::sqrt(std::max(Float(0), cosTheta2));
      return V3(cosPhi * sinTheta, sinPhi * sinTheta, cosTheta);
    }
    Float Eval(const V3& m) const {
      Float cosTheta = m.z;
      Float cosTheta2 = Sqr(cosTheta), alpha2 = Sqr(alpha);
      Float result = (alpha2 - Float(1)) / (PI * std::log(alpha2) * (Float(1) + (alpha2 - Float(1)) * cosTheta2));
      return result * cosTheta > Float(1e-20f) ? result : Float(0);
    }
    Float Pdf(const V3& m) const { return m.z < Float(0) ? Float(0) : m.z * Eval(m); }
  };

  // disney.cpp:113-235
  std::pair<BsdfSample, Spectrum> SampleImpl(const V3& wi, Float lobeXi, const V2& dirXi, const TexSi* ts) const override {
    Float cosThetaI = wi.z;
    BsdfSample bsr;
    if (cosThetaI == 0) return {bsr, Spectrum(0)};
    Float aniso = hasAnisotropic ? anisotropic : 0;
    (void)aniso;
    Float st = hasSpecTrans ? specTrans : Float(0);
    Float met = hasMetallic ? metallic : Float(0);
    Float cc = hasClearcoat ? clearcoat : Float(0);
    Float brdf = (Float(1) - met) * (Float(1) - st);
    Float bsdf = hasSpecTrans ? (Float(1) - met) * st : Float(0);
    bool isFrontSide = cosThetaI > Float(0);
    Microfacet spec;
    spec.ggx = true;
    spec.sampleVisible = true;
    RoughnessToAlpha(spec.alphaX, spec.alphaY);
    V3 mSpec = spec.Sample(MulSign(wi, cosThetaI), dirXi).first;
    Float frSpecDielectric, cosThetaT, etaIT, etaTI;
    FresnelDielectric(dot(wi, mSpec), eta, frSpecDielectric, cosThetaT, etaIT, etaTI);
    if (!isFrontSide && (bsdf <= 0)) return {bsr, Spectrum(0)};
    Float probSpecReflect = isFrontSide ? specularSample * (Float(1) - bsdf * (Float(1) - frSpecDielectric))
                                        : frSpecDielectric;
    Float probSpecTrans =
        hasSpecTrans ? (isFrontSide ? specularSample * bsdf * (Float(1) - frSpecDielectric) : (Float(1) - frSpecDielectric))
                     : Float(0);
    Float probClearcoat = hasClearcoat ? (isFrontSide ? Float(0.25) * cc * clearcoatSample : Float(0)) : Float(0);
    Float probDiffuse = isFrontSide ? brdf * diffuseReflectSample : Float(0);
    Float rcpTotalProb = Rcp(probSpecReflect + probSpecTrans + probClearcoat + probDiffuse);
    probSpecTrans *= rcpTotalProb;
    probClearcoat *= rcpTotalProb;
    probDiffuse *= rcpTotalProb;
    Float currentProb = 0;
    bool sampleDiffuse = (lobeXi < probDiffuse);
    currentProb += probDiffuse;
    bool sampleClearcoat = hasClearcoat && (lobeXi >= currentProb) && (lobeXi < currentProb + probClearcoat);
    currentProb += probClearcoat;
    bool sampleSpecTrans = hasSpecTrans && (lobeXi >= currentProb) && (lobeXi < currentProb + probSpecTrans);
    currentProb += probSpecTrans;
    bool sampleSpecReflect = (lobeXi >= currentProb);
    bsr.Eta = Float(1);
    if (sampleSpecReflect) {
      V3 wo = FresnelReflect(wi, mSpec);
      bsr.Wo = wo;
      bsr.Type = BT_Reflection | BT_Glossy;
      bool reflect = cosThetaI * wo.z > Float(0);
      bool isValid = CheckMacMicNormal(mSpec, wi, wo, cosThetaI, true) && reflect;
      if (!isValid) return {bsr, Spectrum(0)};
    }
    if (sampleSpecTrans) {
      V3 wo = FresnelRefract(wi, mSpec, cosThetaT, etaTI);
      bsr.Wo = wo;
      bsr.Type = BT_Transmission | BT_Glossy;
      bsr.Eta = etaIT;
      bool refract = cosThetaI * wo.z < Float(0);
      bool isValid = CheckMacMicNormal(mSpec, wi, wo, cosThetaI, false) && refract;
      if (!isValid) return {bsr, Spectrum(0)};
    }
    if (hasClearcoat && sampleClearcoat) {
      GTR1 ccDist{Lerp(Float(0.1), Float(0.001), clearcoatGloss)};
      V3 mCC = ccDist.Sample(dirXi);
      V3 wo = FresnelReflect(wi, mCC);
      bsr.Wo = wo;
      bsr.Type = BT_Reflection | BT_Glossy;
      bool reflect = cosThetaI * wo.z > Float(0);
      bool isValid = CheckMacMicNormal(mCC, wi, wo, cosThetaI, true) && reflect;
      if (!isValid) return {bsr, Spectrum(0)};
    }
    if (sampleDiffuse) {
      V3 wo = SquareToCosineHemisphere(dirXi);
      bsr.Wo = wo;
      bsr.Type = BT_Reflection | BT_Diffuse;
      bool reflect = cosThetaI * wo.z > Float(0);
      if (!reflect) return {bsr, Spectrum(0)};
    }
    bsr.Pdf = PdfImpl(wi, bsr.Wo, ts);
    if (bsr.Pdf <= 0) return {bsr, Spectrum(0)};
    return {bsr, EvalImpl(wi, bsr.Wo, ts)};
  }

  // disney.cpp:237-361
  Spectrum EvalImpl(const V3& wi, const V3& wo, const TexSi* ts) const override {
    Float cosThetaI = wi.z;
    if (cosThetaI == 0) return Spectrum(0);
    Float rough = roughness;
    Float flat = hasFlatness ? flatness : Float(0);
    Float st = hasSpecTrans ? specTrans : Float(0);
    Float met = hasMetallic ? metallic : Float(0);
    Float cc = hasClearcoat ? clearcoat : Float(0);
    Float sh = hasSheen ? sheen : Float(0);
    Float brdf = (Float(1) - met) * (Float(1) - st);
    Float bsdf = (Float(1) - met) * st;
    Float cosThetaO = wo.z;
    bool reflect = cosThetaI * cosThetaO > Float(0);
    bool refract = cosThetaI * cosThetaO < Float(0);
    bool isFrontSide = cosThetaI > Float(0);
    Float invEta = Rcp(eta);
    Float etaPath = isFrontSide ? eta : invEta;
    Float invEtaPath = isFrontSide ? invEta : eta;
    Microfacet spec;
    spec.ggx = true;
    spec.sampleVisible = true;
    RoughnessToAlpha(spec.alphaX, spec.alphaY);
    V3 wh = normalized(wi + wo * (reflect ? Float(1) : etaPath));
    wh = MulSign(wh, wh.z);
    Float frSpecDielectric, cosThetaT, etaIT, etaTI;
    FresnelDielectric(dot(wi, wh), eta, frSpecDielectric, cosThetaT, etaIT, etaTI);
    bool canReflection = CheckMacMicNormal(wh, wi, wo, cosThetaI, true);
    bool canRefraction = CheckMacMicNormal(wh, wi, wo, cosThetaI, false);
    bool hasSpecReflectLobe = reflect && canReflection && (frSpecDielectric > Float(0));
    bool hasClearcoatLobe = hasClearcoat && (cc > Float(0)) && reflect && canReflection && isFrontSide;
    bool hasSpecTransLobe =
        hasSpecTrans && (bsdf > Float(0)) && refract && canRefraction && (frSpecDielectric < Float(1));
    bool hasDiffuseLobe = (brdf > Float(0)) && reflect && isFrontSide;
    bool hasSheenLobe = hasSheen && (sh > Float(0)) && reflect && (Float(1) - met > Float(0)) && isFrontSide;
    Float Dv = spec.D(wh);
    Float Gv = spec.G(wi, wo, wh);
    Spectrum value(0);
    if (hasSpecReflectLobe) {
      Float lum = hasSpecTint ? Luminance(baseColor) : Float(1);
      Spectrum dF = DisneyFresnel(frSpecDielectric, lum, dot(wi, wh), isFrontSide, bsdf);
      Float den = Float(4) * std::abs(cosThetaI);
      value = value + Spectrum(dF.x * Dv * Gv / den, dF.y * Dv * Gv / den, dF.z * Dv * Gv / den);
    }
    if (hasSpecTrans && hasSpecTransLobe) {
      Float scale = (ts && ts->importance) ? Float(1) : Sqr(invEtaPath);  // disney.cpp:304
      Float idh = dot(wi, wh), odh = dot(wo, wh);
      Float t = std::abs((scale * (Float(1) - frSpecDielectric) * Dv * Gv * etaPath * etaPath * idh * odh) /
                         (cosThetaI * Sqr(idh + etaPath * odh)));
      Spectrum sq(std::sqrt(baseColor.x), std::sqrt(baseColor.y), std::sqrt(baseColor.z));
      value = value + (sq * bsdf) * t;
    }
    if (hasClearcoat && hasClearcoatLobe) {
      Float ccF = SchlickF(Float(0.04), dot(wi, wh), eta);
      GTR1 ccDistr{Lerp(Float(0.1), Float(0.001), clearcoatGloss)};
      Float ccD = ccDistr.Eval(wh);
      Float ccG = ClearcoatG(wi, wo, wh, Float(0.25));
      value = value + Spectrum((cc * Float(0.25)) * ccF * ccD * ccG * std::abs(cosThetaO));
    }
    if (hasDiffuseLobe) {
      Float Fo = SchlickWeight(std::abs(cosThetaO));
      Float Fi = SchlickWeight(std::abs(cosThetaI));
      Float fsDiff = (Float(1) - Float(0.5) * Fi) * (Float(1) - Float(0.5) * Fo);
      Float cosThetaD = dot(wh, wo);
      Float Rr = Float(2) * rough * Sqr(cosThetaD);
      Float fsRetro = Rr * (Fo + Fi + Fo * Fi * (Rr - Float(1)));
      if (hasFlatness) {
        Float Fss90 = Rr / Float(2);
        Float Fss = Lerp(Float(1), Fss90, Fo) * Lerp(Float(1), Fss90, Fi);
        Float fsSSS = Float(1.25) * (Fss * (Float(1) / (std::abs(cosThetaO) + std::abs(cosThetaI)) - Float(0.5)) + Float(0.5));
        Float s = brdf * std::abs(cosThetaO);
        Float l = Lerp(fsDiff + fsRetro, fsSSS, flat);
        value = value + ((baseColor * s) * (1 / PI)) * l;
      } else {
        Float s = brdf * std::abs(cosThetaO);
        value = value + ((baseColor * s) * (1 / PI)) * (fsDiff + fsRetro);
      }
      if (hasSheen && hasSheenLobe) {
        Float Fd = SchlickWeight(std::abs(cosThetaD));
        if (hasSheenTint) {
          Float lum = Luminance(baseColor);
          Spectrum cTint = lum > Float(0) ? baseColor / lum : Spectrum(1);
          Spectrum cSheen(1 + sheenTint * (cTint.x - 1), 1 + sheenTint * (cTint.y - 1), 1 + sheenTint * (cTint.z - 1));
          Float s = sh * (Float(1) - met) * Fd;
          value = value + (cSheen * s) * std::abs(cosThetaO);
        } else {
          value = value + Spectrum(sh * (Float(1) - met) * Fd * std::abs(cosThetaO));
        }
      }
    }
    return value;
  }

  // disney.cpp:363-456
  Float PdfImpl(const V3& wi, const V3& wo, const TexSi*) const override {
    Float cosThetaI = wi.z;
    if (cosThetaI == 0) return 0;
    Float st = hasSpecTrans ? specTrans : Float(0);
    Float met = hasMetallic ? metallic : Float(0);
    Float cc = hasClearcoat ? clearcoat : Float(0);
    Float brdf = (Float(1) - met) * (Float(1) - st);
    Float bsdf = (Float(1) - met) * st;
    bool isFrontSide = cosThetaI > Float(0);
    Float etaPath = isFrontSide ? eta : Rcp(eta);
    Float cosThetaO = wo.z;
    bool reflect = cosThetaI * cosThetaO > Float(0);
    bool refract = cosThetaI * cosThetaO < Float(0);
    V3 wh = normalized(wi + wo * (reflect ? Float(1) : etaPath));
    wh = MulSign(wh, wh.z);
    Microfacet spec;
    spec.ggx = true;
    spec.sampleVisible = true;
    RoughnessToAlpha(spec.alphaX, spec.alphaY);
    Float frSpecDielectric, cosThetaT, etaIT, etaTI;
    FresnelDielectric(dot(wi, wh), eta, frSpecDielectric, cosThetaT, etaIT, etaTI);
    Float probSpecReflect = isFrontSide ? specularSample * (Float(1) - bsdf * (Float(1) - frSpecDielectric))
                                        : frSpecDielectric;
    Float probSpecTrans =
        hasSpecTrans ? (isFrontSide ? specularSample * bsdf * (Float(1) - frSpecDielectric) : (Float(1) - frSpecDielectric))
                     : Float(0);
    Float probClearcoat = hasClearcoat ? (isFrontSide ? Float(0.25) * cc * clearcoatSample : Float(0)) : Float(0);
    Float probDiffuse = isFrontSide ? brdf * diffuseReflectSample : Float(0);
    Float rcpTotalProb = Rcp(probSpecReflect + probSpecTrans + probClearcoat + probDiffuse);
    probSpecReflect *= rcpTotalProb;
    probSpecTrans *= rcpTotalProb;
    probClearcoat *= rcpTotalProb;
    probDiffuse *= rcpTotalProb;
    Float dwhdwoAbs;
    if (hasSpecTrans) {
      Float wiDotH = dot(wi, wh);
      Float woDotH = dot(wo, wh);
      dwhdwoAbs = std::abs(reflect ? Rcp(Float(4) * woDotH) : (Sqr(etaPath) * woDotH) / Sqr(wiDotH + etaPath * woDotH));
    } else {
      dwhdwoAbs = std::abs(Rcp(Float(4) * dot(wo, wh)));
    }
    Float pdf = 0;
    bool canReflection = CheckMacMicNormal(wh, wi, wo, cosThetaI, true) && reflect;
    if (canReflection) pdf += probSpecReflect * spec.Pdf(MulSign(wi, cosThetaI), wh) * dwhdwoAbs;
    if (reflect) pdf += probDiffuse * SquareToCosineHemispherePdf(wo);
    if (hasSpecTrans) {
      bool canRefr = CheckMacMicNormal(wh, wi, wo, cosThetaI, false) && refract;
      if (canRefr) pdf += probSpecTrans * spec.Pdf(MulSign(wi, cosThetaI), wh) * dwhdwoAbs;
    }
    if (hasClearcoat) {
      GTR1 ccDistr{Lerp(Float(0.1), Float(0.001), clearcoatGloss)};
      if (canReflection) pdf += probClearcoat * ccDistr.Pdf(wh) * dwhdwoAbs;
    }
    return pdf;
  }
};

// --------------------------------------------------------- perfect_mirror
// perfect_mirror.cpp:17-62
struct PerfectMirrorBsdf final : Bsdf {
  Spectrum R, eta, k;
  explicit PerfectMirrorBsdf(const Json* cfg, TexEnv* env) {
    flags = BT_Delta | BT_Reflection;
    ColorParam(cfg, "reflectance", V3(1), &PerfectMirrorBsdf::R, env);
    ColorParam(cfg, "eta", V3(0), &PerfectMirrorBsdf::eta, env);
    ColorParam(cfg, "k", V3(1), &PerfectMirrorBsdf::k, env);
  }
  std::unique_ptr<Bsdf> Clone() const override { return std::make_unique<PerfectMirrorBsdf>(*this); }
  std::pair<BsdfSample, Spectrum> SampleImpl(const V3& wi, Float, const V2&, const TexSi*) const override {
    Float cosThetaI = wi.z;
    if (cosThetaI <= 0) return {{}, Spectrum(0)};
    BsdfSample bsr;
    bsr.Wo = V3(-wi.x, -wi.y, wi.z);  // fresnel.cpp:10-12
    bsr.Eta = 1;
    bsr.Type = flags;
    bsr.Pdf = 1;
    Spectrum F = FresnelConductor(wi.z, eta, k);
    return {bsr, cmul(R, F)};
  }
  Spectrum EvalImpl(const V3&, const V3&, const TexSi*) const override { return Spectrum(0); }
  Float PdfImpl(const V3&, const V3&, const TexSi*) const override { return 0; }
};

// ---------------------------------------------------------- perfect_glass
// perfect_glass.cpp:17-87 (radiance transport)
struct PerfectGlassBsdf final : Bsdf {
  Spectrum R, T;
  Float eta;
  std::unique_ptr<Bsdf> Clone() const override { return std::make_unique<PerfectGlassBsdf>(*this); }
  explicit PerfectGlassBsdf(const Json* cfg, TexEnv* env) {
    flags = BT_Delta | BT_Reflection | BT_Transmission;
    ColorParam(cfg, "reflectance", V3(1), &PerfectGlassBsdf::R, env);
    ColorParam(cfg, "transmittance", V3(1), &PerfectGlassBsdf::T, env);
    Float intIor = ReadF(cfg, "int_ior", Float(1.5046));
    Float extIor = ReadF(cfg, "ext_ior", Float(1.000277));
    eta = intIor / extIor;
  }
  std::pair<BsdfSample, Spectrum> SampleImpl(const V3& wi, Float lobeXi, const V2&, const TexSi* ts) const override {
    Float ri, cosThetaT, etaIT, etaTI;
    FresnelDielectric(wi.z, eta, ri, cosThetaT, etaIT, etaTI);
    Float ti = 1 - ri;
    BsdfSample bsr;
    Spectrum f;
    if (lobeXi <= ri) {
      bsr.Wo = V3(-wi.x, -wi.y, wi.z);
      bsr.Eta = 1;
      bsr.Pdf = ri;
      bsr.Type = BT_Delta | BT_Reflection;
      f = R * ri;
    } else {
      bsr.Wo = V3(-etaTI * wi.x, -etaTI * wi.y, cosThetaT);  // fresnel.cpp:18-20
      bsr.Eta = etaIT;
      bsr.Pdf = ti;
      bsr.Type = BT_Delta | BT_Transmission;
      f = T * ti;
      Float factor = (ts && ts->importance) ? Float(1) : etaTI;  // perfect_glass.cpp:64-65
      f = f * Sqr(factor);
    }
    return {bsr, f};
  }
  Spectrum EvalImpl(const V3&, const V3&, const TexSi*) const override { return Spectrum(0); }
  Float PdfImpl(const V3&, const V3&, const TexSi*) const override { return 0; }
};

// ------------------------------------------------- plastic / rough_plastic
// fresnel.cpp:79-84
static Float DiffuseReflectance(Float eta) {
  Float invEta = Rcp(eta);
  if (eta < 1) return Fmadd(Float(0.0636f), invEta, Fmadd(eta, Fmadd(eta, Float(-1.4399f), Float(0.7099f)), Float(0.6681f)));
  // Horner(invEta, 0.919317, -3.4793, 6.75335, -7.80989, 4.98554, -1.36881) (math_base.h:90-105)
  Float acc = Float(-1.36881f);
  acc = Fmadd(invEta, acc, Float(4.98554f));
  acc = Fmadd(invEta, acc, Float(-7.80989f));
  acc = Fmadd(invEta, acc, Float(6.75335f));
  acc = Fmadd(invEta, acc, Float(-3.4793f));
  acc = Fmadd(invEta, acc, Float(0.919317f));
  return acc;
}
static Float DielectricR(Float cosThetaI, Float eta) {
  Float r, ct, eit, eti;
  FresnelDielectric(cosThetaI, eta, r, ct, eit, eti);
  return r;
}
// Constructor state shared by plastic.cpp:18-44 and rough_plastic.cpp:20-56.
struct PlasticBase : Bsdf {
  Float eta, fdrInt, invEta2, specularSampleWeight;
  Spectrum diffuse, specular;
  bool noLinear;
  PlasticBase(const Json* cfg, TexEnv* env) {
    flags = BT_Diffuse | BT_Reflection | BT_Delta;
    Float intIor = ReadF(cfg, "int_ior", Float(1.49f));
    Float extIor = ReadF(cfg, "ext_ior", Float(1.000277f));
    eta = intIor / extIor;
    std::shared_ptr<Texture> dt = ColorParam(cfg, "diffuse", V3(0.5f), &PlasticBase::diffuse, env);
    std::shared_ptr<Texture> st = ColorParam(cfg, "specular", V3(1), &PlasticBase::specular, env);
    noLinear = ReadB(cfg, "no_linear", false);
    fdrInt = DiffuseReflectance(Float(1) / eta);
    invEta2 = Float(1) / (eta * eta);
    // the mean luminance of Texture::Read over each texture's texels
    // (constants and chessboards are 1 x 1; a chessboard reads 0)
    std::shared_ptr<Texture> dc = dt ? dt : ConstTexture(diffuse, 3), sc = st ? st : ConstTexture(specular, 3);
    double diffMean = 0, specMean = 0;
    for (uint32_t y = 0; y < dc->height; y++)
      for (uint32_t x = 0; x < dc->width; x++) diffMean += Luminance(dc->Read(x, y));
    diffMean /= (dc->height * dc->width);
    for (uint32_t y = 0; y < sc->height; y++)
      for (uint32_t x = 0; x < sc->width; x++) specMean += Luminance(sc->Read(x, y));
    specMean /= (sc->height * sc->width);
    specularSampleWeight = (Float)(specMean / (diffMean + specMean));
  }
  Spectrum DiffuseTerm(Float fi, Float fo, Float cosThetaO) const {  // plastic.cpp:83-88
    V3 num = diffuse * (1 / PI) * invEta2 * (1 - fi) * (1 - fo) * cosThetaO;
    if (noLinear) {
      V3 inv(Rcp(1 - diffuse.x * fdrInt), Rcp(1 - diffuse.y * fdrInt), Rcp(1 - diffuse.z * fdrInt));
      return cmul(num, inv);
    }
    return num / (1 - fdrInt);
  }
};

// plastic.cpp:16-139
struct PlasticBsdf final : PlasticBase {
  PlasticBsdf(const Json* cfg, TexEnv* env) : PlasticBase(cfg, env) {}
  std::unique_ptr<Bsdf> Clone() const override { return std::make_unique<PlasticBsdf>(*this); }
  std::pair<BsdfSample, Spectrum> SampleImpl(const V3& wi, Float lobeXi, const V2& dirXi, const TexSi*) const override {
    Float cosThetaI = wi.z;
    if (cosThetaI <= 0) return {{}, Spectrum(0)};
    Float fi = DielectricR(cosThetaI, eta);
    Float probSpec = fi * specularSampleWeight;
    Float probDiff = (1 - fi) * (1 - specularSampleWeight);
    probSpec = probSpec / (probSpec + probDiff);  // Delta and Diffuse both enabled
    probDiff = 1 - probSpec;
    BsdfSample bsr;
    bsr.Eta = 1;
    Spectrum f;
    if (lobeXi < probSpec) {
      bsr.Wo = V3(-wi.x, -wi.y, wi.z);
      bsr.Pdf = probSpec;
      bsr.Type = BT_Reflection | BT_Delta;
      f = specular * fi;
    } else {
      bsr.Wo = SquareToCosineHemisphere(dirXi);
      bsr.Pdf = SquareToCosineHemispherePdf(bsr.Wo) * probDiff;
      bsr.Type = BT_Reflection | BT_Diffuse;
      Float cosThetaO = bsr.Wo.z;
      Float fo = DielectricR(cosThetaO, eta);
      f = DiffuseTerm(fi, fo, cosThetaO);
    }
    return {bsr, f};
  }
  Spectrum EvalImpl(const V3& wi, const V3& wo, const TexSi*) const override {
    Float cosThetaI = wi.z, cosThetaO = wo.z;
    if (cosThetaI <= 0 || cosThetaO <= 0) return Spectrum(0);
    Float fi = DielectricR(cosThetaI, eta);
    Float fo = DielectricR(cosThetaO, eta);
    return DiffuseTerm(fi, fo, cosThetaO);
  }
  Float PdfImpl(const V3& wi, const V3& wo, const TexSi*) const override {
    Float cosThetaI = wi.z, cosThetaO = wo.z;
    if (cosThetaI <= 0 || cosThetaO <= 0) return 0;
    Float fi = DielectricR(cosThetaI, eta);
    Float probSpec = fi * specularSampleWeight;
    Float probDiff = (1 - fi) * (1 - specularSampleWeight);
    probDiff = probDiff / (probDiff + probSpec);
    return SquareToCosineHemispherePdf(wo) * probDiff;
  }
};

// rough_plastic.cpp:17-241 (default context: Glossy and Diffuse both enabled)
struct RoughPlasticBsdf final : PlasticBase {
  Microfacet dist;
  std::unique_ptr<Bsdf> Clone() const override { return std::make_unique<RoughPlasticBsdf>(*this); }
  RoughPlasticBsdf(const Json* cfg, TexEnv* env) : PlasticBase(cfg, env) {
    std::string d = ReadS(cfg, "distribution", "ggx");
    dist.ggx = d != "beckmann";
    const Json* aj = cfg ? cfg->find("alpha") : nullptr;
    if (aj && !aj->is_number()) {  // one alpha texture for both axes (rough_plastic.cpp:28, :104-118)
      texParams.push_back(TexParam{MakeTexture(*aj, 1, env), [](Bsdf& b, const V3& v) {
                                     auto& r = static_cast<RoughPlasticBsdf&>(b);
                                     r.dist.alphaX = r.dist.alphaY = v.x;
                                   }});
    } else {
      dist.alphaX = dist.alphaY = aj ? (Float)aj->num : Float(0.1f);
    }
    dist.sampleVisible = ReadB(cfg, "sample_visible", true);
  }
  std::pair<BsdfSample, Spectrum> SampleImpl(const V3& wi, Float lobeXi, const V2& dirXi, const TexSi* ts) const override {
    Float cosThetaI = wi.z;
    if (cosThetaI <= 0) return {{}, Spectrum(0)};
    Float fi = DielectricR(cosThetaI, eta);
    Float probSpec = fi * specularSampleWeight;
    Float probDiff = (1 - fi) * (1 - specularSampleWeight);
    probSpec = probSpec / (probSpec + probDiff);
    BsdfSample bsr;
    bsr.Eta = 1;
    if (lobeXi < probSpec) {
      auto whp = dist.Sample(wi, dirXi);
      if (whp.second <= 0) return {bsr, Spectrum(0)};
      bsr.Wo = FresnelReflect(wi, whp.first);
      bsr.Type = BT_Glossy | BT_Reflection;
    } else {
      bsr.Wo = SquareToCosineHemisphere(dirXi);
      bsr.Type = BT_Diffuse | BT_Reflection;
    }
    bsr.Pdf = PdfImpl(wi, bsr.Wo, ts);
    if (bsr.Pdf <= 0) return {bsr, Spectrum(0)};
    return {bsr, EvalImpl(wi, bsr.Wo, ts)};
  }
  Spectrum EvalImpl(const V3& wi, const V3& wo, const TexSi*) const override {
    Float cosThetaI = wi.z, cosThetaO = wo.z;
    if (cosThetaI <= 0 || cosThetaO <= 0) return Spectrum(0);
    V3 wh = normalized(wo + wi);
    Float F = DielectricR(dot(wi, wh), eta);
    Float Dv = dist.D(wh);
    Float Gv = dist.G(wi, wo, wh);
    Spectrum spec = specular * Dv * Gv * F / (4 * cosThetaI);
    Float fo = DielectricR(dot(wo, wh), eta);
    Spectrum diff = DiffuseTerm(F, fo, cosThetaO);
    return spec + diff;
  }
  Float PdfImpl(const V3& wi, const V3& wo, const TexSi*) const override {
    Float cosThetaI = wi.z, cosThetaO = wo.z;
    if (cosThetaI <= 0 || cosThetaO <= 0) return 0;
    Float fi = DielectricR(cosThetaI, eta);
    Float probSpec = fi * specularSampleWeight;
    Float probDiff = (1 - fi) * (1 - specularSampleWeight);
    probSpec = probSpec / (probSpec + probDiff);
    probDiff = 1 - probSpec;
    V3 wh = normalized(wo + wi);
    Float specPdf = dist.Pdf(wi, wh) / (4 * dot(wo, wh)) * probSpec;
    Float diffPdf = SquareToCosineHemispherePdf(wo) * probDiff;
    return specPdf + diffPdf;
  }
};

// ------------------------------------------------------------------- mask
// mask.cpp:10-69
struct MaskBsdf final : Bsdf {
  Float opacity;
  std::shared_ptr<Bsdf> nested;
  MaskBsdf(const Json* cfg, TexEnv* env) {
    MonoParam(cfg, "opacity", 0.5f, &MaskBsdf::opacity, env);
    if (!cfg || !cfg->has("nested")) throw std::runtime_error("mask needs a nested bsdf");
    nested = MakeBsdf(cfg->find("nested"), env);
    flags = nested->flags;
  }
  std::unique_ptr<Bsdf> Clone() const override { return std::make_unique<MaskBsdf>(*this); }
  Float EvalOpacity() const { return std::clamp(opacity, Float(0), Float(1)); }
  std::pair<BsdfSample, Spectrum> SampleImpl(const V3& wi, Float lobeXi, const V2& dirXi,
                                             const TexSi* ts) const override {
    Float op = EvalOpacity();
    BsdfSample bsr;
    Spectrum result;
    if (lobeXi < op) {
      lobeXi /= op;
      auto r = nested->Sample(wi, lobeXi, dirXi, ts);
      bsr = r.first;
      bsr.Pdf *= op;
      result = r.second * op;
    } else {
      result = Spectrum(1);
      bsr.Pdf = 1 - op;
      bsr.Eta = 1;
      bsr.Wo = -wi;
      bsr.Type = BT_Null;
    }
    return {bsr, result};
  }
  Spectrum EvalImpl(const V3& wi, const V3& wo, const TexSi* ts) const override {
    return nested->Eval(wi, wo, ts) * EvalOpacity();
  }
  Float PdfImpl(const V3& wi, const V3& wo, const TexSi* ts) const override {
    return nested->Pdf(wi, wo, ts) * EvalOpacity();
  }
};

// --------------------------------------------------------------- two_side
// two_side.cpp:64-129
struct TwoSideBsdf final : Bsdf {
  std::shared_ptr<Bsdf> outside, inside;
  TwoSideBsdf(const Json* cfg, TexEnv* env) {
    if (cfg && cfg->has("two_side")) {
      outside = inside = MakeBsdf(cfg->find("two_side"), env);
    } else {
      // two_side.cpp:34-52: the out_side / in_side form. The reference reads its
      // (uninitialised) pointers before assigning them; the intent, kept here,
      // is outside = out_side and inside = in_side, both required.
      if (cfg && cfg->has("out_side")) outside = MakeBsdf(cfg->find("out_side"), env);
      if (cfg && cfg->has("in_side")) inside = MakeBsdf(cfg->find("in_side"), env);
      if (!outside || !inside) throw std::runtime_error("config must contains out_side and in_side");
    }
    flags = inside->flags | outside->flags;
  }
  std::unique_ptr<Bsdf> Clone() const override { return std::make_unique<TwoSideBsdf>(*this); }
  std::pair<BsdfSample, Spectrum> SampleImpl(const V3& wi, Float lobeXi, const V2& dirXi,
                                             const TexSi* ts) const override {
    if (wi.z > 0) return outside->Sample(wi, lobeXi, dirXi, ts);
    if (wi.z < 0) {
      V3 twi(wi.x, wi.y, -wi.z);
      auto r = inside->Sample(twi, lobeXi, dirXi, ts);
      r.first.Wo.z *= -1;
      return r;
    }
    return {BsdfSample{}, Spectrum(0)};
  }
  Spectrum EvalImpl(const V3& wi, const V3& wo, const TexSi* ts) const override {
    if (wi.z > 0) return outside->Eval(wi, wo, ts);
    if (wi.z < 0) return inside->Eval(V3(wi.x, wi.y, -wi.z), V3(wo.x, wo.y, -wo.z), ts);
    return Spectrum(0);
  }
  Float PdfImpl(const V3& wi, const V3& wo, const TexSi* ts) const override {
    if (wi.z > 0) return outside->Pdf(wi, wo, ts);
    if (wi.z < 0) return inside->Pdf(V3(wi.x, wi.y, -wi.z), V3(wo.x, wo.y, -wo.z), ts);
    return 0;
  }
};

std::unique_ptr<Bsdf> MakeBsdf(const Json* cfg, TexEnv* env) {
  std::string type = ReadS(cfg, "type", "");
  if (type == "diffuse") return std::make_unique<DiffuseBsdf>(cfg, env);
  if (type == "rough_metal") return std::make_unique<RoughMetalBsdf>(cfg, env);
  if (type == "rough_glass") return std::make_unique<RoughGlassBsdf>(cfg, env);
  if (type == "disney") return std::make_unique<DisneyBsdf>(cfg, env);
  if (type == "two_side") return std::make_unique<TwoSideBsdf>(cfg, env);
  if (type == "perfect_mirror") return std::make_unique<PerfectMirrorBsdf>(cfg, env);
  if (type == "perfect_glass") return std::make_unique<PerfectGlassBsdf>(cfg, env);
  if (type == "plastic") return std::make_unique<PlasticBsdf>(cfg, env);
  if (type == "rough_plastic") return std::make_unique<RoughPlasticBsdf>(cfg, env);
  if (type == "mask") return std::make_unique<MaskBsdf>(cfg, env);
  throw std::runtime_error("cannot find factory: " + type);
}

}  // namespace orc
