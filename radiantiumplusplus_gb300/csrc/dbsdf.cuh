// Device BSDFs: diffuse (diffuse.cpp:46-99), rough_metal (rough_metal.cpp:22-176),
// rough_glass (rough_glass.cpp:22-221), disney (disney.cpp:28-613),
// perfect_mirror (perfect_mirror.cpp:17-70), perfect_glass (perfect_glass.cpp:17-87),
// plastic (plastic.cpp:16-139), rough_plastic (rough_plastic.cpp:17-241) and the
// wrappers two_side (two_side.cpp:64-129) and mask (mask.cpp:10-69). Eval and Pdf
// are fused into one call that shares the half vector, D and G between the value
// and the density; each result equals the reference's separate Eval / Pdf for the
// same inputs.
#pragma once
#include "dmath.cuh"
#include "dtex.cuh"

namespace rad {

// BsdfSampleResult (bsdf.h:77-98): a sample that fails keeps the defaults,
// pdf 0 and eta 1.
struct BsdfSampleRes {
  V3 wo{0.f, 0.f, 0.f};
  float pdf = 0.f;
  float eta = 1.f;
  uint32_t type = 0;
  V3 f{0.f, 0.f, 0.f};
};

RD Microfacet MatDist(const MatRec& m) {
  Microfacet d;
  d.ax = m.p[9];
  d.ay = m.p[10];
  d.ggx = m.p[11] != 0.f;
  d.visible = m.p[12] != 0.f;
  return d;
}

// ----------------------------------------------------------------- diffuse
RD void DiffuseEvalPdf(const MatRec& m, V3 wi, V3 wo, V3& f, float& pdf) {
  if (wi.z <= 0.f || wo.z <= 0.f) {
    f = v3s(0.f);
    pdf = 0.f;
    return;
  }
  V3 R = ld3(m.p);
  f = R * (1.f / kPi) * wo.z;
  pdf = SquareToCosineHemispherePdf(wo);
}
RD BsdfSampleRes DiffuseSample(const MatRec& m, V3 wi, V2 dirXi) {
  BsdfSampleRes r{};
  if (wi.z <= 0.f) return r;
  r.wo = SquareToCosineHemisphere(dirXi);
  r.pdf = SquareToCosineHemispherePdf(r.wo);
  r.eta = 1.f;
  r.type = m.flags;
  V3 R = ld3(m.p);
  r.f = R * (1.f / kPi) * r.wo.z;
  return r;
}

// ------------------------------------------------------------- rough_metal
RD void MetalEvalPdf(const MatRec& m, V3 wi, V3 wo, V3& f, float& pdf) {
  float cosThetaI = wi.z, cosThetaO = wo.z;
  if (cosThetaI <= 0.f || cosThetaO <= 0.f) {
    f = v3s(0.f);
    pdf = 0.f;
    return;
  }
  Microfacet d = MatDist(m);
  V3 wh = normalized(wo + wi);
  V3 F = FresnelConductor(dot(wi, wh), ld3(m.p + 3), ld3(m.p + 6));
  float D = MfD(d, wh);
  float G = MfG(d, wi, wo, wh);
  float den = cosThetaI * cosThetaO * 4.f;
  V3 brdf{fabsf(F.x * D * G) / den, fabsf(F.y * D * G) / den, fabsf(F.z * D * G) / den};
  f = cmul(ld3(m.p), brdf) * cosThetaO;
  pdf = MfPdf(d, wi, wh) / (4.f * dot(wo, wh));
}
RD BsdfSampleRes MetalSample(const MatRec& m, V3 wi, V2 dirXi) {
  BsdfSampleRes r{};
  if (wi.z <= 0.f) return r;
  Microfacet d = MatDist(m);
  float pdf;
  V3 mm = MfSample(d, wi, dirXi, pdf);
  V3 wo = Reflect(wi, mm);
  if (pdf <= 0.f || wo.z <= 0.f) return r;
  pdf /= 4.f * dot(wo, mm);
  float D = MfD(d, mm);
  float G = MfG(d, wi, wo, mm);
  V3 F = FresnelConductor(dot(wi, mm), ld3(m.p + 3), ld3(m.p + 6));
  float den = 4.f * wi.z * wo.z;
  V3 brdf{(F.x * D * G) / den, (F.y * D * G) / den, (F.z * D * G) / den};
  r.wo = wo;
  r.pdf = pdf;
  r.eta = 1.f;
  r.type = m.flags;
  r.f = cmul(ld3(m.p), brdf) * wo.z;
  return r;
}

// ------------------------------------------------------------- rough_glass
RD void GlassEvalPdf(const MatRec& m, V3 wi, V3 wo, V3& f, float& pdf, bool imp = false) {
  f = v3s(0.f);
  pdf = 0.f;
  float cosThetaI = wi.z, cosThetaO = wo.z;
  if (cosThetaI == 0.f) return;
  Microfacet d = MatDist(m);
  float etaM = m.p[6], invEtaM = m.p[7];
  bool reflect = cosThetaI * cosThetaO > 0.f;
  float e = cosThetaI > 0.f ? etaM : invEtaM;
  float ie = cosThetaI > 0.f ? invEtaM : etaM;
  V3 mm = normalized(wi + wo * (reflect ? 1.f : e));
  mm = MulSign(mm, mm.z);
  // Eval (rough_glass.cpp:109-150)
  float D = MfD(d, mm);
  float F = FresnelDielectric(dot(wi, mm), etaM).r;
  float G = MfG(d, wi, wo, mm);
  float idm = dot(wi, mm), odm = dot(wo, mm);
  if (reflect) {
    float brdf = fabsf(F * D * G / (cosThetaI * 4.f));
    f = ld3(m.p) * brdf;
  } else {
    float scale = imp ? 1.f : Sqr(ie);  // TransportMode::Importance: no eta^2 (rough_glass.cpp:143)
    float btdf = fabsf((scale * (1.f - F) * D * G * e * e * idm * odm) / (cosThetaI * Sqr(idm + e * odm)));
    f = ld3(m.p + 3) * btdf;
  }
  // Pdf (rough_glass.cpp:168-201)
  if (idm * cosThetaI <= 0.f || odm * cosThetaO <= 0.f) return;
  float dwhdwo = reflect ? Rcp(odm * 4.f) : ((e * e * odm) / (Sqr(idm + e * odm)));
  float p = MfPdf(d, MulSign(wi, cosThetaI), mm);
  float Fp = FresnelDielectric(idm, etaM).r;
  p *= reflect ? Fp : (1.f - Fp);
  pdf = fabsf(p * dwhdwo);
}
RD BsdfSampleRes GlassSample(const MatRec& m, V3 wi, float lobeXi, V2 dirXi, bool imp = false) {
  BsdfSampleRes r{};
  float cosThetaI = wi.z;
  if (cosThetaI == 0.f) return r;
  Microfacet d = MatDist(m);
  float mpdf;
  V3 wh = MfSample(d, MulSign(wi, cosThetaI), dirXi, mpdf);
  if (mpdf == 0.f) return r;
  Dielectric fr = FresnelDielectric(dot(wi, wh), m.p[6]);
  bool selectedR = lobeXi <= fr.r;
  V3 wo = selectedR ? Reflect(wi, wh) : Refract(wi, wh, fr.cosThetaT, fr.etaTI);
  bool isReflect = wi.z * wo.z > 0.f;
  V3 f;
  float pdf;
  GlassEvalPdf(m, wi, wo, f, pdf, imp);
  if (pdf <= 0.f) return BsdfSampleRes{};
  r.wo = wo;
  r.eta = isReflect ? 1.f : fr.etaIT;
  r.type = BT_GLOSSY | (isReflect ? BT_REFLECTION : BT_TRANSMISSION);
  r.pdf = pdf;
  r.f = f;
  return r;
}

// ------------------------------------------------------------------ disney
struct DisneyP {
  V3 base;
  float rough, aniso, specTrans, sheen, sheenTint, flatness, specTint, metallic, clearcoat, ccGloss, eta;
  float specSample, ccSample, diffSample;
  uint32_t fl;
};
RD DisneyP LoadDisney(const MatRec& m) {
  DisneyP d;
  d.base = ld3(m.p);
  d.rough = m.p[3];
  d.aniso = m.p[4];
  d.specTrans = m.p[5];
  d.sheen = m.p[6];
  d.sheenTint = m.p[7];
  d.flatness = m.p[8];
  d.specTint = m.p[9];
  d.metallic = m.p[10];
  d.clearcoat = m.p[11];
  d.ccGloss = m.p[12];
  d.eta = m.p[13];
  d.specSample = m.p[14];
  d.ccSample = m.p[15];
  d.diffSample = m.aux;
  d.fl = m.dflags;
  return d;
}
RD Microfacet DisneyDist(const DisneyP& d) {  // disney.cpp:474-486
  Microfacet mf;
  mf.ggx = true;
  mf.visible = true;
  float r2 = Sqr(d.rough);
  if (!(d.fl & DF_ANISO)) {
    float a = fmaxr(0.001f, r2);
    mf.ax = mf.ay = a;
  } else {
    float aspect = sqrtf(1.f - 0.9f * d.aniso);
    mf.ax = fmaxr(0.001f, r2 / aspect);
    mf.ay = fmaxr(0.001f, r2 * aspect);
  }
  return mf;
}
RD bool CheckMacMic(V3 mm, V3 wi, V3 wo, float cosThetaI, bool reflection) {
  if (reflection) return (dot(wi, MulSign(mm, cosThetaI)) > 0.f) && (dot(wo, MulSign(mm, cosThetaI)) > 0.f);
  return (dot(wi, MulSign(mm, cosThetaI)) > 0.f) && (dot(wo, cosThetaI >= 0.f ? -mm : mm) > 0.f);
}
RD float SchlickWeight(float cosI) {
  float m = clampr(1.f - cosI, 0.f, 1.f);
  return Sqr(Sqr(m)) * m;
}
RD float SchlickWeightFor(float cosThetaI, float eta) {
  bool isOutside = cosThetaI >= 0.f;
  float rcpEta = Rcp(eta);
  float etaIT = isOutside ? eta : rcpEta;
  float etaTI = isOutside ? rcpEta : eta;
  float sqrCosThetaT = fmaf(-fmaf(-cosThetaI, cosThetaI, 1.f), Sqr(etaTI), 1.f);
  float cosThetaT = SafeSqrt(sqrCosThetaT);
  return etaIT > 1.f ? SchlickWeight(fabsf(cosThetaI)) : SchlickWeight(cosThetaT);
}
RD float SchlickF1(float R0, float cosThetaI, float eta) {  // disney.cpp:514-525
  return Lerp(SchlickWeightFor(cosThetaI, eta), 1.f, R0);
}
RD V3 SchlickF3(V3 R0, float cosThetaI, float eta) {  // disney.cpp:534-545
  float w = SchlickWeightFor(cosThetaI, eta);
  return V3{w + R0.x * (1.f - w), w + R0.y * (1.f - w), w + R0.z * (1.f - w)};
}
RD float GTR1Eval(float alpha, V3 mm) {  // disney.cpp:49-54
  float cosTheta = mm.z;
  float cosTheta2 = Sqr(cosTheta), alpha2 = Sqr(alpha);
  float result = (alpha2 - 1.f) / (kPi * logf(alpha2) * (1.f + (alpha2 - 1.f) * cosTheta2));
  return result * cosTheta > 1e-20f ? result : 0.f;
}
RD float GTR1Pdf(float alpha, V3 mm) { return mm.z < 0.f ? 0.f : mm.z * GTR1Eval(alpha, mm); }
RD V3 GTR1Sample(float alpha, V2 xi) {  // disney.cpp:39-47
  float a = (2.f * kPi) * xi.x;
  float sinPhi = sinf(a), cosPhi = cosf(a);
  float alpha2 = Sqr(alpha);
  float cosTheta2 = (1.f - powf(alpha2, 1.f - xi.y)) / (1.f - alpha2);
  float sinTheta = sqrtf(fmaxr(0.f, 1.f - cosTheta2));
  float cosTheta = sqrtf(fmaxr(0.f, cosTheta2));
  return V3{cosPhi * sinTheta, sinPhi * sinTheta, cosTheta};
}
RD float SmithGGX1(V3 v, V3 wh, float alpha) {  // disney.cpp:596-612
  float alpha2 = Sqr(alpha);
  float cosTheta = fabsf(v.z);
  float cosTheta2 = Sqr(cosTheta);
  float tanTheta2 = (1.f - cosTheta2) / cosTheta2;
  float result = 2.f * Rcp(1.f + sqrtf(1.f + alpha2 * tanTheta2));
  if (v.z == 1.f) result = 1.f;
  if (dot(v, wh) * v.z <= 0.f) result = 0.f;
  return result;
}

// disney.cpp:237-456: value and density for one (wi, wo).
RD void DisneyEvalPdf(const MatRec& m, V3 wi, V3 wo, V3& f, float& pdf, bool imp = false) {
  f = v3s(0.f);
  pdf = 0.f;
  float cosThetaI = wi.z;
  if (cosThetaI == 0.f) return;
  DisneyP d = LoadDisney(m);
  float diffSample = d.diffSample;
  float ccSample = d.ccSample;
  float specSample = d.specSample;
  bool hasST = d.fl & DF_SPECTRANS, hasMet = d.fl & DF_METALLIC, hasCC = d.fl & DF_CLEARCOAT;
  bool hasSheen = d.fl & DF_SHEEN, hasST2 = d.fl & DF_SPECTINT, hasFlat = d.fl & DF_FLATNESS;
  float specTrans = hasST ? d.specTrans : 0.f;
  float metallic = hasMet ? d.metallic : 0.f;
  float clearcoat = hasCC ? d.clearcoat : 0.f;
  float sheen = hasSheen ? d.sheen : 0.f;
  float flatness = hasFlat ? d.flatness : 0.f;
  float brdf = (1.f - metallic) * (1.f - specTrans);
  float bsdf = (1.f - metallic) * specTrans;
  float cosThetaO = wo.z;
  bool reflect = cosThetaI * cosThetaO > 0.f;
  bool refract = cosThetaI * cosThetaO < 0.f;
  bool isFront = cosThetaI > 0.f;
  float invEta = Rcp(d.eta);
  float etaPath = isFront ? d.eta : invEta;
  float invEtaPath = isFront ? invEta : d.eta;
  Microfacet spec = DisneyDist(d);
  V3 wh = normalized(wi + wo * (reflect ? 1.f : etaPath));
  wh = MulSign(wh, wh.z);
  float frD = FresnelDielectric(dot(wi, wh), d.eta).r;
  bool canR = CheckMacMic(wh, wi, wo, cosThetaI, true);
  bool canT = CheckMacMic(wh, wi, wo, cosThetaI, false);
  float D = MfD(spec, wh);
  float G = MfG(spec, wi, wo, wh);
  // ---- value (disney.cpp:237-361)
  bool lobeSR = reflect && canR && (frD > 0.f);
  bool lobeCC = hasCC && (clearcoat > 0.f) && reflect && canR && isFront;
  bool lobeST = hasST && (bsdf > 0.f) && refract && canT && (frD < 1.f);
  bool lobeDiff = (brdf > 0.f) && reflect && isFront;
  bool lobeSheen = hasSheen && (sheen > 0.f) && reflect && (1.f - metallic > 0.f) && isFront;
  V3 value = v3s(0.f);
  if (lobeSR) {
    float lum = hasST2 ? Luminance(d.base) : 1.f;
    float specTint = hasST2 ? d.specTint : 0.f;
    float cI = dot(wi, wh);
    // DisneyFresnel (disney.cpp:567-590)
    bool isOutside = cI >= 0.f;
    float etaIT = isOutside ? d.eta : Rcp(d.eta);
    V3 schlickF = v3s(0.f);
    if (hasMet) schlickF = schlickF + metallic * SchlickF3(d.base, cI, d.eta);
    if (hasST2) {
      V3 cTint = lum > 0.f ? d.base / lum : v3s(1.f);
      float r0 = Sqr((etaIT - 1.f) / (etaIT + 1.f));
      V3 F0 = cTint * r0;
      schlickF = schlickF + (1.f - metallic) * specTint * SchlickF3(F0, cI, d.eta);
    }
    V3 frontF = v3s((1.f - metallic) * (1.f - specTint) * frD) + schlickF;
    V3 dF = isFront ? frontF : v3s(bsdf * frD);
    float den = 4.f * fabsf(cosThetaI);
    value = value + V3{dF.x * D * G / den, dF.y * D * G / den, dF.z * D * G / den};
  }
  if (hasST && lobeST) {
    float scale = imp ? 1.f : Sqr(invEtaPath);  // disney.cpp:304
    float idh = dot(wi, wh), odh = dot(wo, wh);
    float t = fabsf((scale * (1.f - frD) * D * G * etaPath * etaPath * idh * odh) /
                    (cosThetaI * Sqr(idh + etaPath * odh)));
    V3 sq{sqrtf(d.base.x), sqrtf(d.base.y), sqrtf(d.base.z)};
    value = value + (sq * bsdf) * t;
  }
  float ccAlpha = Lerp(0.1f, 0.001f, d.ccGloss);
  if (hasCC && lobeCC) {
    float ccF = SchlickF1(0.04f, dot(wi, wh), d.eta);
    float ccD = GTR1Eval(ccAlpha, wh);
    float ccG = SmithGGX1(wi, wh, 0.25f) * SmithGGX1(wo, wh, 0.25f);
    value = value + v3s((clearcoat * 0.25f) * ccF * ccD * ccG * fabsf(cosThetaO));
  }
  if (lobeDiff) {
    float Fo = SchlickWeight(fabsf(cosThetaO));
    float Fi = SchlickWeight(fabsf(cosThetaI));
    float fsDiff = (1.f - 0.5f * Fi) * (1.f - 0.5f * Fo);
    float cosThetaD = dot(wh, wo);
    float Rr = 2.f * d.rough * Sqr(cosThetaD);
    float fsRetro = Rr * (Fo + Fi + Fo * Fi * (Rr - 1.f));
    float s = brdf * fabsf(cosThetaO);
    if (hasFlat) {
      float Fss90 = Rr / 2.f;
      float Fss = Lerp(1.f, Fss90, Fo) * Lerp(1.f, Fss90, Fi);
      float fsSSS = 1.25f * (Fss * (1.f / (fabsf(cosThetaO) + fabsf(cosThetaI)) - 0.5f) + 0.5f);
      float l = Lerp(fsDiff + fsRetro, fsSSS, flatness);
      value = value + ((d.base * s) * (1.f / kPi)) * l;
    } else {
      value = value + ((d.base * s) * (1.f / kPi)) * (fsDiff + fsRetro);
    }
    if (hasSheen && lobeSheen) {
      float Fd = SchlickWeight(fabsf(cosThetaD));
      if (d.fl & DF_SHEENTINT) {
        float lum = Luminance(d.base);
        V3 cTint = lum > 0.f ? d.base / lum : v3s(1.f);
        V3 cSheen{1.f + d.sheenTint * (cTint.x - 1.f), 1.f + d.sheenTint * (cTint.y - 1.f),
                  1.f + d.sheenTint * (cTint.z - 1.f)};
        float ss = sheen * (1.f - metallic) * Fd;
        value = value + (cSheen * ss) * fabsf(cosThetaO);
      } else {
        value = value + v3s(sheen * (1.f - metallic) * Fd * fabsf(cosThetaO));
      }
    }
  }
  f = value;
  // ---- density (disney.cpp:363-456)
  float pSR = isFront ? specSample * (1.f - bsdf * (1.f - frD)) : frD;
  float pST = hasST ? (isFront ? specSample * bsdf * (1.f - frD) : (1.f - frD)) : 0.f;
  float pCC = hasCC ? (isFront ? 0.25f * clearcoat * ccSample : 0.f) : 0.f;
  float pDf = isFront ? brdf * diffSample : 0.f;
  float rcpTotal = Rcp(pSR + pST + pCC + pDf);
  pSR *= rcpTotal;
  pST *= rcpTotal;
  pCC *= rcpTotal;
  pDf *= rcpTotal;
  float dwhdwoAbs;
  if (hasST) {
    float wiDotH = dot(wi, wh), woDotH = dot(wo, wh);
    dwhdwoAbs = fabsf(reflect ? Rcp(4.f * woDotH) : (Sqr(etaPath) * woDotH) / Sqr(wiDotH + etaPath * woDotH));
  } else {
    dwhdwoAbs = fabsf(Rcp(4.f * dot(wo, wh)));
  }
  float p = 0.f;
  bool canReflection = canR && reflect;
  if (canReflection) p += pSR * MfPdf(spec, MulSign(wi, cosThetaI), wh) * dwhdwoAbs;
  if (reflect) p += pDf * SquareToCosineHemispherePdf(wo);
  if (hasST) {
    if (canT && refract) p += pST * MfPdf(spec, MulSign(wi, cosThetaI), wh) * dwhdwoAbs;
  }
  if (hasCC) {
    if (canReflection) p += pCC * GTR1Pdf(ccAlpha, wh) * dwhdwoAbs;
  }
  pdf = p;
}

// disney.cpp:113-235
RD BsdfSampleRes DisneySample(const MatRec& m, V3 wi, float lobeXi, V2 dirXi, bool imp = false) {
  BsdfSampleRes r{};
  float cosThetaI = wi.z;
  if (cosThetaI == 0.f) return r;
  DisneyP d = LoadDisney(m);
  float diffSample = d.diffSample;
  bool hasST = d.fl & DF_SPECTRANS, hasMet = d.fl & DF_METALLIC, hasCC = d.fl & DF_CLEARCOAT;
  float specTrans = hasST ? d.specTrans : 0.f;
  float metallic = hasMet ? d.metallic : 0.f;
  float clearcoat = hasCC ? d.clearcoat : 0.f;
  float brdf = (1.f - metallic) * (1.f - specTrans);
  float bsdf = hasST ? (1.f - metallic) * specTrans : 0.f;
  bool isFront = cosThetaI > 0.f;
  Microfacet spec = DisneyDist(d);
  float mp;
  V3 mSpec = MfSample(spec, MulSign(wi, cosThetaI), dirXi, mp);
  Dielectric fr = FresnelDielectric(dot(wi, mSpec), d.eta);
  if (!isFront && (bsdf <= 0.f)) return r;
  float pSR = isFront ? d.specSample * (1.f - bsdf * (1.f - fr.r)) : fr.r;
  float pST = hasST ? (isFront ? d.specSample * bsdf * (1.f - fr.r) : (1.f - fr.r)) : 0.f;
  float pCC = hasCC ? (isFront ? 0.25f * clearcoat * d.ccSample : 0.f) : 0.f;
  float pDf = isFront ? brdf * diffSample : 0.f;
  float rcpTotal = Rcp(pSR + pST + pCC + pDf);
  pST *= rcpTotal;
  pCC *= rcpTotal;
  pDf *= rcpTotal;
  float cur = 0.f;
  bool sDiff = lobeXi < pDf;
  cur += pDf;
  bool sCC = hasCC && (lobeXi >= cur) && (lobeXi < cur + pCC);
  cur += pCC;
  bool sST = hasST && (lobeXi >= cur) && (lobeXi < cur + pST);
  cur += pST;
  bool sSR = lobeXi >= cur;
  V3 wo = v3s(0.f);
  r.eta = 1.f;
  if (sSR) {
    wo = Reflect(wi, mSpec);
    r.type = BT_REFLECTION | BT_GLOSSY;
    bool refl = cosThetaI * wo.z > 0.f;
    if (!(CheckMacMic(mSpec, wi, wo, cosThetaI, true) && refl)) return BsdfSampleRes{wo, 0.f, 1.f, r.type, v3s(0.f)};
  }
  if (sST) {
    wo = Refract(wi, mSpec, fr.cosThetaT, fr.etaTI);
    r.type = BT_TRANSMISSION | BT_GLOSSY;
    r.eta = fr.etaIT;
    bool refr = cosThetaI * wo.z < 0.f;
    if (!(CheckMacMic(mSpec, wi, wo, cosThetaI, false) && refr)) return BsdfSampleRes{wo, 0.f, r.eta, r.type, v3s(0.f)};
  }
  if (hasCC && sCC) {
    V3 mCC = GTR1Sample(Lerp(0.1f, 0.001f, d.ccGloss), dirXi);
    wo = Reflect(wi, mCC);
    r.type = BT_REFLECTION | BT_GLOSSY;
    bool refl = cosThetaI * wo.z > 0.f;
    if (!(CheckMacMic(mCC, wi, wo, cosThetaI, true) && refl)) return BsdfSampleRes{wo, 0.f, r.eta, r.type, v3s(0.f)};
  }
  if (sDiff) {
    wo = SquareToCosineHemisphere(dirXi);
    r.type = BT_REFLECTION | BT_DIFFUSE;
    if (!(cosThetaI * wo.z > 0.f)) return BsdfSampleRes{wo, 0.f, r.eta, r.type, v3s(0.f)};
  }
  V3 f;
  float pdf;
  DisneyEvalPdf(m, wi, wo, f, pdf, imp);
  r.wo = wo;
  r.pdf = pdf;
  if (pdf <= 0.f) {
    r.f = v3s(0.f);
    return r;
  }
  r.f = f;
  return r;
}

// ---------------------------------------------------------- perfect_mirror
// perfect_mirror.cpp:27-48; Eval and Pdf are 0 (:50-62).
RD BsdfSampleRes MirrorSample(const MatRec& m, V3 wi) {
  BsdfSampleRes r{};
  if (wi.z <= 0.f) return r;
  r.wo = V3{-wi.x, -wi.y, wi.z};
  r.eta = 1.f;
  r.type = m.flags;
  r.pdf = 1.f;
  r.f = cmul(ld3(m.p), FresnelConductor(wi.z, ld3(m.p + 3), ld3(m.p + 6)));
  return r;
}

// ----------------------------------------------------------- perfect_glass
// perfect_glass.cpp:29-72 (radiance transport); Eval and Pdf are 0.
RD BsdfSampleRes PerfectGlassSample(const MatRec& m, V3 wi, float lobeXi, bool imp = false) {
  BsdfSampleRes r{};
  Dielectric fr = FresnelDielectric(wi.z, m.p[6]);
  float ti = 1.f - fr.r;
  if (lobeXi <= fr.r) {
    r.wo = V3{-wi.x, -wi.y, wi.z};
    r.eta = 1.f;
    r.pdf = fr.r;
    r.type = BT_DELTA | BT_REFLECTION;
    r.f = ld3(m.p) * fr.r;
  } else {
    r.wo = V3{-fr.etaTI * wi.x, -fr.etaTI * wi.y, fr.cosThetaT};
    r.eta = fr.etaIT;
    r.pdf = ti;
    r.type = BT_DELTA | BT_TRANSMISSION;
    r.f = ld3(m.p + 3) * ti;
    if (!imp) r.f = r.f * Sqr(fr.etaTI);  // radiance transport (perfect_glass.cpp:63-65)
  }
  return r;
}

// ------------------------------------------------- plastic / rough_plastic
// Shared layout: p0..2 diffuse, p3..5 specular, p6 eta, p7 1/eta^2, p8 the
// internal diffuse Fresnel reflectance, p13 specular sampling weight, p14 no_linear.
// The diffuse term of plastic.cpp:80-88 / rough_plastic.cpp:143-153.
RD V3 PlasticDiffuse(const MatRec& m, float fi, float fo, float cosThetaO) {
  V3 diff = ld3(m.p);
  float a = 1.f - fi, b = 1.f - fo;
  V3 num{((((diff.x * (1.f / kPi)) * m.p[7]) * a) * b) * cosThetaO,
         ((((diff.y * (1.f / kPi)) * m.p[7]) * a) * b) * cosThetaO,
         ((((diff.z * (1.f / kPi)) * m.p[7]) * a) * b) * cosThetaO};
  if (m.p[14] != 0.f)
    return V3{num.x * Rcp(1.f - diff.x * m.p[8]), num.y * Rcp(1.f - diff.y * m.p[8]),
              num.z * Rcp(1.f - diff.z * m.p[8])};
  float den = 1.f - m.p[8];
  return V3{num.x / den, num.y / den, num.z / den};
}
// Probability of the specular lobe (plastic.cpp:58-66, rough_plastic.cpp:72-80).
RD float PlasticSpecProb(const MatRec& m, float fi) {
  float probSpec = fi * m.p[13];
  float probDiff = (1.f - fi) * (1.f - m.p[13]);
  return probSpec / (probSpec + probDiff);
}
// plastic.cpp:93-139: only the diffuse lobe has a density.
RD void PlasticEvalPdf(const MatRec& m, V3 wi, V3 wo, V3& f, float& pdf) {
  float cosThetaI = wi.z, cosThetaO = wo.z;
  if (cosThetaI <= 0.f || cosThetaO <= 0.f) {
    f = v3s(0.f);
    pdf = 0.f;
    return;
  }
  float fi = FresnelDielectric(cosThetaI, m.p[6]).r;
  float fo = FresnelDielectric(cosThetaO, m.p[6]).r;
  f = PlasticDiffuse(m, fi, fo, cosThetaO);
  float probSpec = fi * m.p[13];
  float probDiff = (1.f - fi) * (1.f - m.p[13]);
  probDiff = probDiff / (probDiff + probSpec);
  pdf = SquareToCosineHemispherePdf(wo) * probDiff;
}
// plastic.cpp:47-91
RD BsdfSampleRes PlasticSample(const MatRec& m, V3 wi, float lobeXi, V2 dirXi) {
  BsdfSampleRes r{};
  float cosThetaI = wi.z;
  if (cosThetaI <= 0.f) return r;
  float fi = FresnelDielectric(cosThetaI, m.p[6]).r;
  float probSpec = PlasticSpecProb(m, fi);
  float probDiff = 1.f - probSpec;
  r.eta = 1.f;
  if (lobeXi < probSpec) {
    r.wo = V3{-wi.x, -wi.y, wi.z};
    r.pdf = probSpec;
    r.type = BT_REFLECTION | BT_DELTA;
    r.f = ld3(m.p + 3) * fi;
  } else {
    r.wo = SquareToCosineHemisphere(dirXi);
    r.pdf = SquareToCosineHemispherePdf(r.wo) * probDiff;
    r.type = BT_REFLECTION | BT_DIFFUSE;
    float cosThetaO = r.wo.z;
    float fo = FresnelDielectric(cosThetaO, m.p[6]).r;
    r.f = PlasticDiffuse(m, fi, fo, cosThetaO);
  }
  return r;
}
// rough_plastic.cpp:122-158 (value) and :183-214 (density) for one (wi, wo).
RD void RoughPlasticEvalPdf(const MatRec& m, V3 wi, V3 wo, V3& f, float& pdf) {
  float cosThetaI = wi.z, cosThetaO = wo.z;
  if (cosThetaI <= 0.f || cosThetaO <= 0.f) {
    f = v3s(0.f);
    pdf = 0.f;
    return;
  }
  Microfacet d = MatDist(m);
  V3 wh = normalized(wo + wi);
  float F = FresnelDielectric(dot(wi, wh), m.p[6]).r;
  float D = MfD(d, wh);
  float G = MfG(d, wi, wo, wh);
  V3 spec = ld3(m.p + 3);
  float den = 4.f * cosThetaI;
  V3 specular{(((spec.x * D) * G) * F) / den, (((spec.y * D) * G) * F) / den, (((spec.z * D) * G) * F) / den};
  float fo = FresnelDielectric(dot(wo, wh), m.p[6]).r;
  f = specular + PlasticDiffuse(m, F, fo, cosThetaO);
  float fi = FresnelDielectric(cosThetaI, m.p[6]).r;
  float probSpec = PlasticSpecProb(m, fi);
  float probDiff = 1.f - probSpec;
  float specPdf = MfPdf(d, wi, wh) / (4.f * dot(wo, wh)) * probSpec;
  float diffPdf = SquareToCosineHemispherePdf(wo) * probDiff;
  pdf = specPdf + diffPdf;
}
// rough_plastic.cpp:58-98
RD BsdfSampleRes RoughPlasticSample(const MatRec& m, V3 wi, float lobeXi, V2 dirXi) {
  BsdfSampleRes r{};
  float cosThetaI = wi.z;
  if (cosThetaI <= 0.f) return r;
  float fi = FresnelDielectric(cosThetaI, m.p[6]).r;
  float probSpec = PlasticSpecProb(m, fi);
  r.eta = 1.f;
  if (lobeXi < probSpec) {
    Microfacet d = MatDist(m);
    float mpdf;
    V3 wh = MfSample(d, wi, dirXi, mpdf);
    if (mpdf <= 0.f) return r;
    r.wo = Reflect(wi, wh);
    r.type = BT_GLOSSY | BT_REFLECTION;
  } else {
    r.wo = SquareToCosineHemisphere(dirXi);
    r.type = BT_DIFFUSE | BT_REFLECTION;
  }
  V3 f;
  float pdf;
  RoughPlasticEvalPdf(m, wi, r.wo, f, pdf);
  r.pdf = pdf;
  if (pdf <= 0.f) return r;
  r.f = f;
  return r;
}

// ---------------------------------------------------------------- dispatch
RD void LeafEvalPdf(const MatRec& m, V3 wi, V3 wo, V3& f, float& pdf, bool imp = false) {
  switch (m.kind) {
    case MAT_DIFFUSE: DiffuseEvalPdf(m, wi, wo, f, pdf); return;
    case MAT_ROUGH_METAL: MetalEvalPdf(m, wi, wo, f, pdf); return;
    case MAT_ROUGH_GLASS: GlassEvalPdf(m, wi, wo, f, pdf, imp); return;
    case MAT_DISNEY: DisneyEvalPdf(m, wi, wo, f, pdf, imp); return;
    case MAT_PLASTIC: PlasticEvalPdf(m, wi, wo, f, pdf); return;
    case MAT_ROUGH_PLASTIC: RoughPlasticEvalPdf(m, wi, wo, f, pdf); return;
    default: f = v3s(0.f); pdf = 0.f; return;  // delta-only BSDFs: Eval = Pdf = 0
  }
}
RD BsdfSampleRes LeafSample(const MatRec& m, V3 wi, float lobeXi, V2 dirXi, bool imp = false) {
  switch (m.kind) {
    case MAT_DIFFUSE: return DiffuseSample(m, wi, dirXi);
    case MAT_ROUGH_METAL: return MetalSample(m, wi, dirXi);
    case MAT_ROUGH_GLASS: return GlassSample(m, wi, lobeXi, dirXi, imp);
    case MAT_DISNEY: return DisneySample(m, wi, lobeXi, dirXi, imp);
    case MAT_PERFECT_MIRROR: return MirrorSample(m, wi);
    case MAT_PERFECT_GLASS: return PerfectGlassSample(m, wi, lobeXi, imp);
    case MAT_PLASTIC: return PlasticSample(m, wi, lobeXi, dirXi);
    case MAT_ROUGH_PLASTIC: return RoughPlasticSample(m, wi, lobeXi, dirXi);
    default: return BsdfSampleRes{};
  }
}
// Wrappers resolve to a leaf: two_side (two_side.cpp:64-129) picks the outside
// or inside BSDF by the sign of wi.z and mirrors z for the inside one; mask
// (mask.cpp:24-60) scales the nested BSDF by its opacity, or, for the share of
// samples beyond the opacity, passes the ray straight through (a Null event).
// Scales are applied innermost first, as the nested calls would apply them; the
// host limits wrapper nesting to kMaxBsdfNest levels. With a texture context,
// textured parameters are looked up at its uv (dtex.cuh).
RD void BsdfEvalPdf(const MatRec* mats, uint32_t mi, V3 wi, V3 wo, V3& f, float& pdf, const TexCtx* tc = nullptr,
                    bool imp = false) {
  float ops[kMaxBsdfNest];
  int nops = 0;
  f = v3s(0.f);
  pdf = 0.f;
  for (int lvl = 0; lvl <= kMaxBsdfNest; lvl++) {
    const MatRec& m = mats[mi];
    if (m.kind == MAT_TWO_SIDE) {
      if (wi.z > 0.f) {
        mi = m.ref0;
      } else if (wi.z < 0.f) {
        mi = m.ref1;
        wi.z = -wi.z;
        wo.z = -wo.z;
      } else {
        break;
      }
    } else if (m.kind == MAT_MASK) {
      if (nops == kMaxBsdfNest) break;
      MatRec tmp;
      ops[nops++] = TexturedMat(m, tc, tmp).p[0];
      mi = m.ref0;
    } else {
      MatRec tmp;
      LeafEvalPdf(TexturedMat(m, tc, tmp), wi, wo, f, pdf, imp);
      break;
    }
  }
  for (int k = nops - 1; k >= 0; k--) {
    f = f * ops[k];
    pdf = pdf * ops[k];
  }
}
RD BsdfSampleRes BsdfSample(const MatRec* mats, uint32_t mi, V3 wi, float lobeXi, V2 dirXi,
                            const TexCtx* tc = nullptr, bool imp = false) {
  float ops[kMaxBsdfNest];
  int nops = 0;
  bool flip = false;
  BsdfSampleRes r{};
  for (int lvl = 0; lvl <= kMaxBsdfNest; lvl++) {
    const MatRec& m = mats[mi];
    if (m.kind == MAT_TWO_SIDE) {
      if (wi.z > 0.f) {
        mi = m.ref0;
      } else if (wi.z < 0.f) {
        mi = m.ref1;
        wi.z = -wi.z;
        flip = !flip;
      } else {
        break;
      }
    } else if (m.kind == MAT_MASK) {
      MatRec tmp;
      float op = TexturedMat(m, tc, tmp).p[0];
      if (lobeXi < op && nops < kMaxBsdfNest) {
        lobeXi /= op;
        ops[nops++] = op;
        mi = m.ref0;
      } else {
        r.f = v3s(1.f);
        r.pdf = 1.f - op;
        r.eta = 1.f;
        r.wo = -wi;
        r.type = BT_NULL;
        break;
      }
    } else {
      MatRec tmp;
      r = LeafSample(TexturedMat(m, tc, tmp), wi, lobeXi, dirXi, imp);
      break;
    }
  }
  for (int k = nops - 1; k >= 0; k--) {
    r.pdf *= ops[k];
    r.f = r.f * ops[k];
  }
  if (flip) r.wo.z = -r.wo.z;
  return r;
}

}  // namespace rad

namespace rad {

// Class-specialised dispatch for the material-sorted shade kernels: the leaf
// kind K is known at compile time, so each kernel carries one BSDF's code.
// A two-sided wrapper resolves to its outside / inside leaf as two_side.cpp does.
template <int K>
RD void LeafEvalPdfK(const MatRec& m, V3 wi, V3 wo, V3& f, float& pdf) {
  if constexpr (K == MAT_DIFFUSE) DiffuseEvalPdf(m, wi, wo, f, pdf);
  else if constexpr (K == MAT_ROUGH_METAL) MetalEvalPdf(m, wi, wo, f, pdf);
  else if constexpr (K == MAT_ROUGH_GLASS) GlassEvalPdf(m, wi, wo, f, pdf);
  else if constexpr (K == MAT_DISNEY) DisneyEvalPdf(m, wi, wo, f, pdf);
  else LeafEvalPdf(m, wi, wo, f, pdf);
}
template <int K>
RD BsdfSampleRes LeafSampleK(const MatRec& m, V3 wi, float lobeXi, V2 dirXi) {
  if constexpr (K == MAT_DIFFUSE) return DiffuseSample(m, wi, dirXi);
  else if constexpr (K == MAT_ROUGH_METAL) return MetalSample(m, wi, dirXi);
  else if constexpr (K == MAT_ROUGH_GLASS) return GlassSample(m, wi, lobeXi, dirXi);
  else if constexpr (K == MAT_DISNEY) return DisneySample(m, wi, lobeXi, dirXi);
  else return LeafSample(m, wi, lobeXi, dirXi);
}
template <int K>
RD void ClassEvalPdf(const MatRec* mats, uint32_t mi, V3 wi, V3 wo, V3& f, float& pdf, const TexCtx* tc = nullptr) {
  if constexpr (K == SC_GENERIC) {
    BsdfEvalPdf(mats, mi, wi, wo, f, pdf, tc);
    return;
  }
  const MatRec& m = mats[mi];
  if (m.kind != MAT_TWO_SIDE) {
    LeafEvalPdfK<K>(m, wi, wo, f, pdf);
  } else if (wi.z > 0.f) {
    LeafEvalPdfK<K>(mats[m.ref0], wi, wo, f, pdf);
  } else if (wi.z < 0.f) {
    LeafEvalPdfK<K>(mats[m.ref1], V3{wi.x, wi.y, -wi.z}, V3{wo.x, wo.y, -wo.z}, f, pdf);
  } else {
    f = v3s(0.f);
    pdf = 0.f;
  }
}
template <int K>
RD BsdfSampleRes ClassSample(const MatRec* mats, uint32_t mi, V3 wi, float lobeXi, V2 dirXi,
                             const TexCtx* tc = nullptr) {
  if constexpr (K == SC_GENERIC) return BsdfSample(mats, mi, wi, lobeXi, dirXi, tc);
  const MatRec& m = mats[mi];
  if (m.kind != MAT_TWO_SIDE) return LeafSampleK<K>(m, wi, lobeXi, dirXi);
  if (wi.z > 0.f) return LeafSampleK<K>(mats[m.ref0], wi, lobeXi, dirXi);
  if (wi.z < 0.f) {
    BsdfSampleRes r = LeafSampleK<K>(mats[m.ref1], V3{wi.x, wi.y, -wi.z}, lobeXi, dirXi);
    r.wo.z *= -1.f;
    return r;
  }
  return BsdfSampleRes{};
}

}  // namespace rad
