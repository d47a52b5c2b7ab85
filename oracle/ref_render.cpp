// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_core.h).
// Integrators: Path::Li (rad.offline/src/renderer/path.cpp:131-236) and
// VolPath::Li (src/renderer/vol_path.cpp:27-349); film loop
// SampleRenderer::Start (src/renderer/sample_renderer.cpp:60-122).
// Exposed through a small C ABI (orc_*) that the tests load with ctypes.
#include <atomic>
#include <thread>

#include "ref_scene.h"

namespace orc {

struct RayCounter {
  uint64_t closest = 0, shadow = 0;
};
static thread_local RayCounter* g_rays = nullptr;

static inline Float MisWeight(Float a, Float b) {  // path.cpp:231-236
  a *= a;
  b *= b;
  Float w = a / (a + b);
  return std::isfinite(w) ? w : 0;
}

static bool Trace(const Scene& S, const Ray& r, SurfaceInteraction& si) {
  if (g_rays) g_rays->closest++;
  return S.RayIntersect(r, si);
}
static bool Occl(const Scene& S, const V3& P, const V3& N, const V3& p) {
  if (g_rays) g_rays->shadow++;
  return S.IsOcclude(P, N, p);
}

// ------------------------------------------------------------------ path
Spectrum PathLi(const Scene& S, const Ray& ray0, const RayDiff& diff0, Pcg32& rng) {
  Ray ray = ray0;
  RayDiff diff = diff0;  // only the camera ray has differentials (path.cpp:132, :208)
  Spectrum throughput(1), result(0);
  Float eta = 1;
  int depth = 0;
  bool isSpecularPath = true;
  V3 prevP;
  Float prevBsdfPdf = 1;
  for (;; depth++) {
    SurfaceInteraction si;
    bool anyHit = Trace(S, ray, si);
    int hitLight = S.LightOf(si);
    if (hitLight >= 0) {
      Float weight;
      if (isSpecularPath) {
        weight = 1;
      } else {
        // SurfaceInteraction::ToDsr (interaction.cpp:68-74)
        DirectionSample dsr;
        dsr.P = si.P;
        dsr.N = si.Shading.N;
        dsr.UV = si.UV;
        V3 rel = si.P - prevP;
        dsr.Dist = norm(rel);
        dsr.Dir = si.IsValid() ? rel / dsr.Dist : -si.Wi;
        Float lightPdf = S.PdfLightDirection(hitLight, prevP, dsr);
        weight = MisWeight(prevBsdfPdf, lightPdf);
      }
      Spectrum li = S.EvalLight(hitLight, si);
      result = result + cmul(throughput, li) * weight;
    }
    if (!anyHit || (S.maxDepth >= 0 && depth + 1 >= S.maxDepth)) break;
    const Shape& sh = S.shapes[si.shape];
    if (sh.light >= 0) break;
    if (sh.bsdf < 0) break;  // the reference dereferences a null BSDF here
    const Bsdf& bsdf = *S.bsdfs[sh.bsdf];
    si.ComputeDifferentials(diff);  // si.BSDF(ray) (path.cpp:172)
    TexSi ts = si.Tex();
    if (bsdf.HasAnyTypeExceptDelta()) {
      Float xl = rng.Next1D();
      V2 xd = rng.Next2D();
      auto dl = S.SampleLightDirection(si.P, xl, xd);
      const DirectionSample& dsr = dl.first;
      if (dsr.Pdf > 0) {
        V3 wo = si.ToLocal(dsr.Dir);
        Spectrum f = bsdf.Eval(si.Wi, wo, &ts);
        Float bsdfPdf = bsdf.Pdf(si.Wi, wo, &ts);
        if (!Occl(S, si.P, si.N, dsr.P)) {
          Float weight = dsr.IsDelta ? 1 : MisWeight(dsr.Pdf, bsdfPdf);
          result = result + cmul(cmul(throughput, f), dl.second) * weight / dsr.Pdf;
        }
      }
    }
    {
      Float xl = rng.Next1D();
      V2 xd = rng.Next2D();
      auto bs = bsdf.Sample(si.Wi, xl, xd, &ts);
      if (bs.first.Pdf <= 0) break;
      throughput = cmul(throughput, bs.second) / bs.first.Pdf;
      eta *= bs.first.Eta;
      ray = SpawnRay(si.P, si.N, si.ToWorld(bs.first.Wo));
      diff.has = false;
      prevBsdfPdf = bs.first.Pdf;
      prevP = si.P;
      isSpecularPath = (bs.first.Type & BT_Delta) != 0;
    }
    if (depth >= S.rrDepth) {
      Float maxThroughput = max_comp(throughput);
      Float rr = std::min(maxThroughput * Sqr(eta), Float(0.95));
      if (rng.Next1D() > rr) break;
      throughput = throughput * Rcp(rr);
    }
  }
  return result;
}

// ---------------------------------------------------------------- media
// medium.cpp:19-43
static MediumInteraction SampleInteraction(const Medium& md, const Ray& ray, Float sample, int channel) {
  MediumInteraction mei;
  mei.Wi = -ray.D;
  mei.Shading = Frame(mei.Wi);
  bool aabbIts;
  Float mint, maxt;
  md.IntersectAABB(ray, aabbIts, mint, maxt);
  aabbIts = aabbIts && (std::isfinite(mint) || std::isfinite(maxt));
  bool active = aabbIts;
  if (!active) {
    mint = 0;
    maxt = std::numeric_limits<Float>::infinity();
  }
  mint = std::max(Float(0), mint);
  maxt = std::min(ray.MaxT, maxt);
  Spectrum combined = md.Majorant();
  Float m = combined[channel];
  Float sampledT = mint + (-std::log(1 - sample) / m);
  bool validMi = active && (sampledT <= maxt);
  mei.T = validMi ? sampledT : std::numeric_limits<Float>::infinity();
  mei.P = ray.At(sampledT);
  mei.MinT = mint;
  md.Coefficients(mei.P, mei.SigmaS, mei.SigmaN, mei.SigmaT);
  mei.CombinedExtinction = combined;
  return mei;
}

static inline V3 ExpSpectrum(const V3& v) { return V3(std::exp(v.x), std::exp(v.y), std::exp(v.z)); }

// medium.cpp:45-59
static void EvalTrAndPdf(const MediumInteraction& mi, const SurfaceInteraction& si, Spectrum& tr, Spectrum& pdf) {
  Float t = std::min(mi.T, si.T) - mi.MinT;
  if (t <= 0) {
    tr = pdf = Spectrum(1);
    return;
  }
  tr = ExpSpectrum(mi.CombinedExtinction * -t);
  pdf = si.T < mi.T ? tr : cmul(tr, mi.CombinedExtinction);
  if (tr.x == pdf.x && tr.y == pdf.y && tr.z == pdf.z) tr = pdf = Spectrum(1);
}

// henyey_greenstein.cpp:37-40 / isotropic.cpp:16-18
static Float PhaseEval(const Medium& md, const MediumInteraction& mi, const V3& wo) {
  if (!md.hg) return SquareToUniformSpherePdf();
  Float c = dot(wo, mi.Wi);
  Float temp = Float(1) + md.g * md.g + Float(2) * md.g * c;
  return (1 / (4 * PI)) * (1 - md.g * md.g) / (temp * std::sqrt(temp));
}
// henyey_greenstein.cpp:18-35 / isotropic.cpp:11-15
static std::pair<V3, Float> PhaseSample(const Medium& md, const MediumInteraction& mi, const V2& xi) {
  if (!md.hg) return {SquareToUniformSphere(xi), SquareToUniformSpherePdf()};
  Float g = md.g;
  Float sqrTerm = (1 - g * g) / (1 - g + 2 * g * xi.x);
  Float cosTheta = (1 + g * g - sqrTerm * sqrTerm) / (2 * g);
  if (std::abs(g) < Float32Epsilon) cosTheta = 1 - 2 * xi.x;
  Float sinTheta = SafeSqrt(1 - cosTheta * cosTheta);
  Float a = 2 * PI * xi.y;
  Float sinPhi = std::sin(a), cosPhi = std::cos(a);
  V3 wo(sinTheta * cosPhi, sinTheta * sinPhi, -cosTheta);
  wo = mi.Shading.ToWorld(wo);
  Float c = -cosTheta;
  Float temp = Float(1) + g * g + Float(2) * g * c;
  Float pdf = (1 / (4 * PI)) * (1 - g * g) / (temp * std::sqrt(temp));
  return {wo, pdf};
}

static int MediumOf(const Scene& S, const SurfaceInteraction& si, const Ray& ray) {  // interaction.cpp:113-115
  const Shape& sh = S.shapes[si.shape];
  return dot(ray.D, si.N) > 0 ? sh.outMedium : sh.inMedium;
}

// vol_path.cpp:224-342. refN is the reference interaction's geometric normal
// (zero for a medium interaction, so SpawnRay leaves the origin in place).
static std::pair<Spectrum, DirectionSample> VolSampleLight(const Scene& S, Pcg32& rng, int medium, int channel,
                                                           const V3& refP, const V3& refN) {
  Float xl = rng.Next1D();
  V2 xd = rng.Next2D();
  auto dl = S.SampleLightDirection(refP, xl, xd);
  DirectionSample dsr = dl.first;
  Spectrum li = dl.second;
  if (dsr.Pdf <= 0) return {Spectrum(0), dsr};
  Ray ray = SpawnRay(refP, refN, dsr.Dir);
  Float totalDist = 0;
  Spectrum resultTr(1);
  bool active = true;
  bool needsIntersection = true;
  SurfaceInteraction si;
  while (active) {
    Float remainingDist = dsr.Dist * (1 - ShadowEpsilon) - totalDist;
    ray.MaxT = remainingDist;
    active = active && remainingDist > 0;
    if (!active) break;
    bool escapedMedium = false;
    bool activeMedium = active && medium >= 0;
    bool activeSurface = active && !activeMedium;
    if (activeMedium) {
      const Medium& md = S.media[medium];
      MediumInteraction mei = SampleInteraction(md, ray, rng.Next1D(), channel);
      if (md.kind == Medium::Homogeneous && mei.IsValid()) ray.MaxT = std::min(mei.T, remainingDist);
      bool intersect = needsIntersection && activeMedium;
      if (intersect) Trace(S, ray, si);
      if (si.T < mei.T) mei.T = std::numeric_limits<Float>::infinity();
      bool isSpectral = activeMedium;  // both media report spectral extinction
      bool notSpectral = !isSpectral && activeMedium;
      if (isSpectral) {
        Float t = std::min(remainingDist, std::min(mei.T, si.T)) - mei.MinT;
        if (t >= 0) {
          Spectrum tr = ExpSpectrum(mei.CombinedExtinction * -t);
          Spectrum freeFlightPdf = (si.T < mei.T || mei.T > remainingDist) ? tr : cmul(tr, mei.CombinedExtinction);
          Float trPdf = freeFlightPdf[channel];
          Spectrum mTr = trPdf > 0 ? tr / trPdf : Spectrum(0);
          resultTr = cmul(resultTr, mTr);
        }
      }
      if (activeMedium && (mei.T > remainingDist) && mei.IsValid()) totalDist = dsr.Dist;
      if (activeMedium && (mei.T > remainingDist)) mei.T = std::numeric_limits<Float>::infinity();
      escapedMedium = activeMedium && !mei.IsValid();
      activeMedium = activeMedium && mei.IsValid();
      isSpectral = isSpectral && activeMedium;
      notSpectral = notSpectral && activeMedium;
      if (activeMedium) totalDist += mei.T;
      if (activeMedium) {
        ray.O = mei.P;
        si.T = si.T - mei.T;
        if (isSpectral) resultTr = cmul(resultTr, mei.SigmaN);
        if (notSpectral) resultTr = cdiv(cmul(resultTr, mei.SigmaN), mei.CombinedExtinction);
      }
    }
    bool intersect = activeSurface && needsIntersection;
    if (intersect) Trace(S, ray, si);
    needsIntersection = needsIntersection && !intersect;
    activeSurface = activeSurface || escapedMedium;
    if (activeSurface) totalDist += si.T;
    activeSurface = activeSurface && si.IsValid() && active && !activeMedium;
    if (activeSurface) {
      if (S.shapes[si.shape].bsdf >= 0) resultTr = Spectrum(0);
      ray = SpawnRay(si.P, si.N, ray.D);
    }
    ray.MaxT = remainingDist;
    needsIntersection = needsIntersection || activeSurface;
    active = active && (activeMedium || activeSurface) && !is_zero(resultTr);
    bool hasMedium = activeSurface && (S.shapes[si.shape].inMedium >= 0 || S.shapes[si.shape].outMedium >= 0);
    if (hasMedium) medium = MediumOf(S, si, ray);
  }
  return {cmul(li, resultTr), dsr};
}

// vol_path.cpp:27-217
Spectrum VolPathLi(const Scene& S, const Ray& ray0, Pcg32& rng) {
  Ray ray = ray0;
  int medium = S.globalMedium;
  Spectrum throughput(1), result(0);
  Float eta = 1;
  int depth = 0;
  bool isSpecularPath = true;
  V3 prevP;
  Float prevPdf = 1;
  int channel = (int)std::min((uint32_t)(rng.Next1D() * 3), 2u);  // vol_path.cpp:219-222
  SurfaceInteraction si;
  for (;; depth++) {
    if (depth >= S.rrDepth) {
      Float maxThroughput = max_comp(throughput);
      Float rr = std::min(maxThroughput * Sqr(eta), Float(0.95));
      if (rng.Next1D() > rr) break;
      throughput = throughput * Rcp(rr);
    }
    if (S.maxDepth >= 0 && depth + 1 >= S.maxDepth) break;
    bool isSampleMedium = medium >= 0;
    bool isSampleSurface = !isSampleMedium;
    bool isNullScatter = false, isMediumScatter = false, isMediumEscaped = false;
    bool isSpectral = isSampleMedium;
    bool notSpectral = false;
    MediumInteraction mei;
    if (isSampleMedium) {
      const Medium& md = S.media[medium];
      mei = SampleInteraction(md, ray, rng.Next1D(), channel);
      if (md.kind == Medium::Homogeneous && mei.IsValid()) ray.MaxT = mei.T;
      Trace(S, ray, si);
      if (si.T < mei.T) mei.T = std::numeric_limits<Float>::infinity();
      if (isSpectral) {
        Spectrum tr, freeFlightPdf;
        EvalTrAndPdf(mei, si, tr, freeFlightPdf);
        Float pdf = freeFlightPdf[channel];
        Spectrum after = cmul(throughput, tr) / pdf;
        throughput = pdf <= 0 ? Spectrum(0) : after;
      }
      isMediumEscaped = isSampleMedium && !mei.IsValid();
      isSampleMedium = isSampleMedium && mei.IsValid();
      bool nullScatter = rng.Next1D() > mei.SigmaT[channel] / mei.CombinedExtinction[channel];
      isNullScatter = isNullScatter || (nullScatter && isSampleMedium);
      isMediumScatter = isMediumScatter || (!isNullScatter && isSampleMedium);
      if (isSpectral && isNullScatter) {
        throughput = cmul(throughput, mei.SigmaN) * mei.CombinedExtinction[channel] / mei.SigmaN[channel];
      }
      if (isMediumScatter) {
        prevP = mei.P;
      }
    }
    if (isNullScatter) {
      ray.O = mei.P;
      si.T = si.T - mei.T;
    }
    if (isMediumScatter) {
      const Medium& md = S.media[medium];
      if (isSpectral) {
        throughput = cmul(throughput, mei.SigmaS) * mei.CombinedExtinction[channel] / mei.SigmaT[channel];
      }
      if (notSpectral) throughput = cdiv(cmul(throughput, mei.SigmaS), mei.SigmaT);
      auto sl = VolSampleLight(S, rng, medium, channel, mei.P, V3(0));
      const DirectionSample& dsr = sl.second;
      if (dsr.Pdf > 0) {
        Float phaseVal = PhaseEval(md, mei, dsr.Dir);
        Float weight = dsr.IsDelta ? 1 : MisWeight(dsr.Pdf, phaseVal);
        result = result + cmul(throughput, sl.first) * weight * phaseVal / dsr.Pdf;
      }
      auto ps = PhaseSample(md, mei, rng.Next2D());
      ray = SpawnRay(mei.P, V3(0), ps.first);
      isSpecularPath = false;
      prevPdf = ps.second;
    }
    isSampleSurface = isSampleSurface || isMediumEscaped;
    if (isSampleSurface) {
      Trace(S, ray, si);
      int hitLight = S.LightOf(si);
      if (hitLight >= 0) {
        Float weight;
        if (isSpecularPath) {
          weight = 1;
        } else {
          DirectionSample dsr;
          dsr.P = si.P;
          dsr.N = si.Shading.N;
          dsr.UV = si.UV;
          V3 rel = si.P - prevP;
          dsr.Dist = norm(rel);
          dsr.Dir = si.IsValid() ? rel / dsr.Dist : -si.Wi;
          Float lightPdf = S.PdfLightDirection(hitLight, prevP, dsr);
          weight = MisWeight(prevPdf, lightPdf);
        }
        Spectrum li = S.EvalLight(hitLight, si);
        result = result + cmul(throughput, li) * weight;
      }
      if (!si.IsValid()) break;
      const Shape& sh = S.shapes[si.shape];
      if (sh.light >= 0) break;
      if (sh.bsdf < 0) {
        ray = SpawnRay(si.P, si.N, ray.D);
        medium = MediumOf(S, si, ray);
        depth--;
        continue;
      }
      const Bsdf& bsdf = *S.bsdfs[sh.bsdf];
      TexSi ts = si.Tex();  // vol_path traces plain rays: uv derivatives stay 0 (vol_path.cpp:28, :177)
      if (bsdf.HasAnyTypeExceptDelta()) {
        auto sl = VolSampleLight(S, rng, medium, channel, si.P, si.N);
        const DirectionSample& dsr = sl.second;
        if (dsr.Pdf > 0) {
          V3 wo = si.ToLocal(dsr.Dir);
          Spectrum f = bsdf.Eval(si.Wi, wo, &ts);
          Float bsdfPdf = bsdf.Pdf(si.Wi, wo, &ts);
          Float weight = dsr.IsDelta ? 1 : MisWeight(dsr.Pdf, bsdfPdf);
          result = result + cmul(cmul(throughput, f), sl.first) * weight / dsr.Pdf;
        }
      }
      Float xl = rng.Next1D();
      V2 xd = rng.Next2D();
      auto bs = bsdf.Sample(si.Wi, xl, xd, &ts);
      if (bs.first.Pdf <= 0) break;
      throughput = cmul(throughput, bs.second) / bs.first.Pdf;
      eta *= bs.first.Eta;
      ray = SpawnRay(si.P, si.N, si.ToWorld(bs.first.Wo));
      prevPdf = bs.first.Pdf;
      prevP = si.P;
      isSpecularPath = (bs.first.Type & BT_Delta) != 0;
      medium = MediumOf(S, si, ray);
    }
    if (!(isSampleSurface || isSampleMedium)) break;
  }
  return result;
}

// ao.cpp:22-36
Spectrum AOLi(const Scene& S, const Ray& ray, Pcg32& rng) {
  SurfaceInteraction si;
  if (!Trace(S, ray, si)) return Spectrum(0);
  V3 wo = SquareToCosineHemisphere(rng.Next2D());
  Float pdf = SquareToCosineHemispherePdf(wo);
  Ray shadowRay = SpawnRay(si.P, si.N, si.ToWorld(wo));
  if (g_rays) g_rays->shadow++;
  bool visibility = S.Occluded(shadowRay);
  Spectrum l(0);
  if (!visibility && wo.z > 0) l = Spectrum(wo.z / PI / pdf);
  return l;
}

// ------------------------------------------------------ particle tracer
// particle_tracer.cpp:135-175
static void ConnectCamera(const Scene& S, const SurfaceInteraction& si, bool hasShape, const Bsdf* bsdf,
                          const TexSi* ts, const DirectionSample& cam, const Spectrum& weight, Float sampleScale,
                          std::vector<Spectrum>& image) {
  if (cam.Pdf <= 0 || is_zero(weight)) return;
  if (Occl(S, si.P, si.N, cam.P)) return;
  V3 o = OffsetP(si.P, si.N, cam.P - si.P);  // SpawnRayTo (interaction.cpp:20-26)
  V3 toCamera = cam.P - o;
  toCamera = toCamera / norm(toCamera);
  V3 wo = si.ToLocal(toCamera);
  Spectrum fs(1);
  if (!hasShape) {
    if (wo.z <= 0) fs = Spectrum(0);
  } else if (!bsdf) {
    fs = fs * std::max(Float(0), wo.z);
  } else {
    Float idn = dot(si.N, si.ToWorld(si.Wi));
    Float odn = dot(si.N, toCamera);
    if (idn * si.Wi.z <= 0 || odn * wo.z <= 0) {
      fs = Spectrum(0);
    } else {
      Float correction = (si.Wi.z * odn) / (wo.z * idn);
      Spectrum bsdfVal = bsdf->Eval(si.Wi, wo, ts);
      fs = cmul(fs, bsdfVal) * std::abs(correction) / cam.Pdf;
    }
  }
  Spectrum ij = cmul(weight, fs) * sampleScale;
  int x = (int)cam.UV.x, y = (int)cam.UV.y;
  Spectrum& px = image[(size_t)y * S.camera.width + x];
  px = px + ij;
}

// One light path (particle_tracer.cpp:97-226): the emitter point seen by the
// camera, then the emitted ray with a camera connection at every vertex.
static void ParticleSample(const Scene& S, uint64_t id, uint32_t seed, Float sampleScale, std::vector<Spectrum>& image) {
  Pcg32 rng = Pcg32::ForSample((uint32_t)id, (uint32_t)(id >> 32), seed);
  if (S.lights.empty()) return;
  if (S.maxDepth != 0) {  // SampleLight (:104-133)
    int index;
    Float lightPdf;
    S.SampleLight(rng.Next1D(), index, lightPdf);
    const Light& L = S.lights[index];
    if (!L.IsDelta()) {
      SurfaceInteraction si;
      Spectrum li;
      bool hasShape = L.kind == Light::Area;
      if (!hasShape) {
        V3 camPos = S.camera.cameraToWorld.ApplyAffineToWorld(V3(0, 0, 0));
        auto r = S.SampleOneLightDirection(index, camPos, rng.Next2D());
        li = r.second;
        lightPdf *= r.first.Pdf > 0 ? (r.first.Pdf * Sqr(r.first.Dist)) : 0;
        si.P = r.first.P;
        si.N = r.first.N;
      } else {  // Light::SamplePosition, then Eval(SurfaceInteraction(psr))
        auto pp = S.LightSamplePosition(index, rng.Next2D());
        lightPdf *= pp.second;
        si.P = pp.first.P;
        si.N = pp.first.N;
        si.UV = pp.first.UV;
        li = S.AreaRadiance(L, si.UV);
      }
      si.Shading = Frame(si.N);
      rng.Next2D();  // Perspective::SampleDirection's sample
      DirectionSample cam;
      Float we = S.camera.SampleDirection(si.P, cam);
      Spectrum weight = li * we / lightPdf;
      si.Wi = si.ToLocal(cam.Dir);
      ConnectCamera(S, si, hasShape, nullptr, nullptr, cam, weight, sampleScale, image);
    }
  }
  int index;
  Float lightPdf;
  S.SampleLight(rng.Next1D(), index, lightPdf);
  V2 xi2 = rng.Next2D(), xi3 = rng.Next2D();
  Ray ray;
  Spectrum li;
  if (!S.LightSampleRay(index, xi2, xi3, ray, li)) return;
  Spectrum throughput = li / lightPdf;
  // TraceLightRay (:177-226)
  Float eta = 1;
  int depth = 1;
  SurfaceInteraction si;
  bool isHit = Trace(S, ray, si);
  if (!isHit || S.shapes[si.shape].bsdf < 0) return;
  if (S.maxDepth >= 0 && depth >= S.maxDepth) return;
  for (;;) {
    const Bsdf& bsdf = *S.bsdfs[S.shapes[si.shape].bsdf];
    TexSi ts = si.Tex();
    ts.importance = true;
    rng.Next2D();
    DirectionSample cam;
    Float we = S.camera.SampleDirection(si.P, cam);
    ConnectCamera(S, si, true, &bsdf, &ts, cam, throughput * we, sampleScale, image);
    Float bl = rng.Next1D();
    V2 bd = rng.Next2D();
    auto bs = bsdf.Sample(si.Wi, bl, bd, &ts);
    // Decision kept with the GPU path: a failed sample (pdf 0) ends the light path,
    // where the reference divides by the zero pdf (particle_tracer.cpp:206) and
    // writes NaN into the film.
    if (!(bs.first.Pdf > 0)) break;
    V3 woW = si.ToWorld(bs.first.Wo);
    Float idn = dot(si.N, -ray.D), odn = dot(si.N, woW);
    if (idn * si.Wi.z <= 0 || odn * bs.first.Wo.z <= 0) break;
    Float correction = (si.Wi.z * odn) / (bs.first.Wo.z * idn);
    throughput = cmul(throughput, bs.second) * std::abs(correction) / bs.first.Pdf;
    eta *= bs.first.Eta;
    if (is_zero(throughput)) break;
    ray = SpawnRay(si.P, si.N, woW);
    isHit = Trace(S, ray, si);
    depth++;
    if (!isHit || S.shapes[si.shape].bsdf < 0) break;
    if (S.maxDepth >= 0 && depth >= S.maxDepth) return;
    if (depth >= S.rrDepth) {
      Float rr = std::min(max_comp(throughput) * Sqr(eta), Float(0.95));
      if (rng.Next1D() > rr) break;
      throughput = throughput * Rcp(rr);
    }
  }
}

Spectrum BdptSample(const Scene& S, uint32_t x, uint32_t y, uint32_t s, uint32_t seed, std::vector<Spectrum>* film);

// sample_renderer.cpp:93-106: one pixel sample. The jitter takes the first two
// draws of the sample's stream (the reference uses a separate per-tile mt19937).
static Spectrum RenderSample(const Scene& S, uint32_t x, uint32_t y, uint32_t s, uint32_t seed) {
  if (S.renderer == "bdpt") return BdptSample(S, x, y, s, seed, nullptr);  // camera side only
  Pcg32 rng = Pcg32::ForSample(x + y * (uint32_t)S.camera.width, s, seed);
  Float jx = rng.Next1D();
  Float jy = rng.Next1D();
  V2 scr(Float(x) + jx, Float(y) + jy);
  RayDiff diff;
  Ray ray = S.camera.SampleRayDifferential(scr, diff);
  if (S.renderer == "ao") return AOLi(S, ray, rng);
  return S.renderer == "vol_path" ? VolPathLi(S, ray, rng) : PathLi(S, ray, diff, rng);
}

// sample_renderer.cpp:101-105: HasInfinity / HasNegative test only the first
// channel (spectrum.h:28-29), HasNaN tests all three.
static inline bool InvalidSample(const Spectrum& li) {
  bool nan = std::isnan(li.x) || std::isnan(li.y) || std::isnan(li.z);
  return nan || std::isinf(li.x) || li.x < 0;
}

}  // namespace orc

using namespace orc;

static thread_local std::string g_err;

extern "C" {

const char* orc_last_error() { return g_err.c_str(); }

void* orc_scene_load(const char* json, const char* baseDir) {
  try {
    return Scene::FromJson(json, baseDir ? baseDir : "").release();
  } catch (const std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}
void orc_scene_free(void* s) { delete (Scene*)s; }

// info: width, height, spp, seed, maxDepth, rrDepth, nShapes, nPrims, nLights, isVol
void orc_scene_info(void* sp, int64_t* info) {
  Scene& S = *(Scene*)sp;
  info[0] = S.camera.width;
  info[1] = S.camera.height;
  info[2] = S.spp;
  info[3] = S.seed;
  info[4] = S.maxDepth;
  info[5] = S.rrDepth;
  info[6] = (int64_t)S.shapes.size();
  info[7] = (int64_t)S.prims.size();
  info[8] = (int64_t)S.lights.size();
  info[9] = S.renderer == "vol_path" ? 1 : 0;
}

// rays: n x 8 (ox, oy, oz, tmin, dx, dy, dz, tmax); hits: n x 5 (t, u, v, prim bits, front bits)
int orc_trace(void* sp, const float* rays, int64_t n, float* hits, int anyHit) {
  Scene& S = *(Scene*)sp;
  for (int64_t i = 0; i < n; i++) {
    const float* r = rays + i * 8;
    Ray ray;
    ray.O = V3(r[0], r[1], r[2]);
    ray.MinT = r[3];
    ray.D = V3(r[4], r[5], r[6]);
    ray.MaxT = r[7];
    float* h = hits + i * 5;
    if (anyHit) {
      uint32_t occ = S.Occluded(ray) ? 1u : 0u;
      h[0] = 0; h[1] = 0; h[2] = 0;
      std::memcpy(&h[3], &occ, 4);
      std::memset(&h[4], 0, 4);
    } else {
      Hit hit = S.Intersect(ray);
      h[0] = hit.t; h[1] = hit.u; h[2] = hit.v;
      std::memcpy(&h[3], &hit.prim, 4);
      std::memcpy(&h[4], &hit.front, 4);
    }
  }
  return 0;
}

// Camera rays for pixel samples (jitter from the sample stream): out n x 8.
int orc_camera_rays(void* sp, const uint32_t* pix, int64_t n, uint32_t sample, uint32_t seed, float* out) {
  Scene& S = *(Scene*)sp;
  for (int64_t i = 0; i < n; i++) {
    uint32_t p = pix[i];
    uint32_t x = p % (uint32_t)S.camera.width, y = p / (uint32_t)S.camera.width;
    Pcg32 rng = Pcg32::ForSample(p, sample, seed);
    Float jx = rng.Next1D(), jy = rng.Next1D();
    Ray r = S.camera.SampleRay(V2(Float(x) + jx, Float(y) + jy));
    float* o = out + i * 8;
    o[0] = r.O.x; o[1] = r.O.y; o[2] = r.O.z; o[3] = r.MinT;
    o[4] = r.D.x; o[5] = r.D.y; o[6] = r.D.z; o[7] = r.MaxT;
  }
  return 0;
}

// Renders rows [row0, row1) with stride rowStep, samples [s0, s1), into film
// (W*H*3, untouched rows left as they are). stats: [closest rays, shadow rays,
// samples, invalid samples]. Returns 0 or -1 with orc_last_error().
int orc_render(void* sp, int row0, int row1, int rowStep, int s0, int s1, int seedOverride, int threads,
               float* film, uint64_t* stats) {
  Scene& S = *(Scene*)sp;
  uint32_t seed = seedOverride >= 0 ? (uint32_t)seedOverride : S.seed;
  int W = S.camera.width;
  std::vector<int> rows;
  for (int y = row0; y < row1; y += rowStep) rows.push_back(y);
  std::atomic<size_t> next{0};
  std::atomic<uint64_t> nC{0}, nS{0}, nSamp{0}, nBad{0};
  int spp = s1 - s0;
  Float coeff = 1.0f / (Float)S.spp;
  auto worker = [&]() {
    RayCounter rc;
    g_rays = &rc;
    uint64_t samp = 0, bad = 0;
    for (;;) {
      size_t k = next.fetch_add(1);
      if (k >= rows.size()) break;
      int y = rows[k];
      for (int x = 0; x < W; x++) {
        Spectrum acc(0);
        for (int s = s0; s < s1; s++) {
          Spectrum li = RenderSample(S, (uint32_t)x, (uint32_t)y, (uint32_t)s, seed);
          samp++;
          if (InvalidSample(li)) {
            bad++;
          } else {
            acc = acc + li;
          }
        }
        float* f = film + (size_t(y) * W + x) * 3;
        if (spp == S.spp) {
          f[0] = acc.x * coeff;
          f[1] = acc.y * coeff;
          f[2] = acc.z * coeff;
        } else {
          f[0] = acc.x;
          f[1] = acc.y;
          f[2] = acc.z;
        }
      }
    }
    nC += rc.closest;
    nS += rc.shadow;
    nSamp += samp;
    nBad += bad;
    g_rays = nullptr;
  };
  try {
    int nt = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
    std::vector<std::thread> ts;
    for (int i = 1; i < nt; i++) ts.emplace_back(worker);
    worker();
    for (auto& t : ts) t.join();
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
  if (stats) {
    stats[0] = nC;
    stats[1] = nS;
    stats[2] = nSamp;
    stats[3] = nBad;
  }
  return 0;
}

// particle_tracer: light paths [first, first + count) of `spp` splatted into
// film (W x H x 3, accumulated onto its contents).
// `threads` workers (0: all host threads) take contiguous ranges of light paths.
int orc_render_particle(void* sp, uint64_t first, uint64_t count, uint64_t spp, uint32_t seed, int threads,
                        float* film) {
  Scene& S = *(Scene*)sp;
  size_t npix = (size_t)S.camera.width * S.camera.height;
  int nt = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
  if (nt < 1) nt = 1;
  std::vector<std::vector<Spectrum>> images(nt, std::vector<Spectrum>(npix, Spectrum(0)));
  Float sampleScale = npix / ((Float)spp);
  std::atomic<bool> failed{false};
  auto worker = [&](int w) {
    try {
      uint64_t a = count * (uint64_t)w / (uint64_t)nt, b = count * (uint64_t)(w + 1) / (uint64_t)nt;
      for (uint64_t i = a; i < b; i++) ParticleSample(S, first + i, seed, sampleScale, images[w]);
    } catch (const std::exception& e) {
      g_err = e.what();
      failed = true;
    }
  };
  std::vector<std::thread> ts;
  for (int i = 1; i < nt; i++) ts.emplace_back(worker, i);
  worker(0);
  for (auto& t : ts) t.join();
  if (failed) return -1;
  for (size_t p = 0; p < npix; p++) {
    for (int w = 0; w < nt; w++) {
      film[3 * p] += images[w][p].x;
      film[3 * p + 1] += images[w][p].y;
      film[3 * p + 2] += images[w][p].z;
    }
  }
  return 0;
}

// bdpt: samples [s0, s1) of the pixels of rows [row0, row1) step rowStep; film
// (W x H x 3) receives, per pixel, (sum of valid camera-side samples + the t = 1
// splats landing there) / spp (bdpt.cpp:261-305). Returns the number of samples
// run, or -1.
int64_t orc_render_bdpt(void* sp, int row0, int row1, int rowStep, int s0, int s1, uint32_t seed, int threads,
                        float* film) {
  Scene& S = *(Scene*)sp;
  if (S.renderer != "bdpt") {
    g_err = "orc_render_bdpt: the scene's renderer is not bdpt";
    return -1;
  }
  const int W = S.camera.width, H = S.camera.height;
  const size_t npix = (size_t)W * H;
  int nt = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
  std::vector<std::vector<Spectrum>> images(nt, std::vector<Spectrum>(npix, Spectrum(0)));
  std::vector<int> rows;
  for (int y = row0; y < row1 && y < H; y += rowStep) rows.push_back(y);
  std::atomic<size_t> next{0};
  std::atomic<bool> failed{false};
  auto worker = [&](int w) {
    try {
      std::vector<Spectrum>& img = images[w];
      for (;;) {
        size_t k = next.fetch_add(1);
        if (k >= rows.size()) break;
        int y = rows[k];
        for (int x = 0; x < W; x++) {
          Spectrum acc(0);
          for (int s = s0; s < s1; s++) {
            Spectrum li = BdptSample(S, (uint32_t)x, (uint32_t)y, (uint32_t)s, seed, &img);
            if (!InvalidSample(li)) acc = acc + li;
          }
          img[(size_t)y * W + x] = img[(size_t)y * W + x] + acc;
        }
      }
    } catch (const std::exception& e) {
      g_err = e.what();
      failed = true;
    }
  };
  std::vector<std::thread> ts;
  for (int i = 1; i < nt; i++) ts.emplace_back(worker, i);
  worker(0);
  for (auto& t : ts) t.join();
  if (failed) return -1;
  Float coeff = Float(1) / (Float)S.spp;
  for (size_t p = 0; p < npix; p++) {
    Spectrum sum(0);
    for (int i = 0; i < nt; i++) sum = sum + images[i][p];
    film[3 * p] = sum.x * coeff;
    film[3 * p + 1] = sum.y * coeff;
    film[3 * p + 2] = sum.z * coeff;
  }
  return (int64_t)rows.size() * W * (s1 - s0);
}

// Per-sample radiance for a list of (pixel, sample) pairs: out n x 3.
int orc_render_samples(void* sp, const uint32_t* pix, const uint32_t* smp, int64_t n, uint32_t seed, float* out) {
  Scene& S = *(Scene*)sp;
  try {
    for (int64_t i = 0; i < n; i++) {
      uint32_t p = pix[i];
      Spectrum li = RenderSample(S, p % (uint32_t)S.camera.width, p / (uint32_t)S.camera.width, smp[i], seed);
      out[i * 3] = li.x;
      out[i * 3 + 1] = li.y;
      out[i * 3 + 2] = li.z;
    }
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
  return 0;
}

// Texture<T>::Eval of the scene's texture number `tex` (creation order), at
// uv (n x 2) with derivatives duv (n x 4: du/dx, dv/dx, du/dy, dv/dy); out n x 3.
int orc_texture_eval(void* sp, uint32_t tex, const float* uv, const float* duv, int64_t n, float* out) {
  Scene& S = *(Scene*)sp;
  if (tex >= S.textures.size()) {
    g_err = "texture index out of range";
    return -1;
  }
  const Texture* t = S.textures[tex];
  for (int64_t i = 0; i < n; i++) {
    TexSi si{V2(uv[2 * i], uv[2 * i + 1]), V2(duv[4 * i], duv[4 * i + 1]), V2(duv[4 * i + 2], duv[4 * i + 3])};
    V3 v = t->Eval(si);
    out[3 * i] = v.x;
    out[3 * i + 1] = v.y;
    out[3 * i + 2] = v.z;
  }
  return 0;
}
int orc_texture_count(void* sp) { return (int)((Scene*)sp)->textures.size(); }

// An image asset as the texture factory sees it (type: image_default /
// image_hdr / image_exr, options as the asset's JSON). Writes width, height,
// channels to dims and, when px is not null, the texels (at most cap floats).
int orc_image_load(const char* assetJson, const char* path, int32_t* dims, float* px, int64_t cap) {
  try {
    Json a = Json::parse(assetJson);
    ImageAsset im = LoadImageAsset(a, ReadS(&a, "type", ""), path);
    dims[0] = im.width;
    dims[1] = im.height;
    dims[2] = im.channels;
    if (px) {
      if ((int64_t)im.px.size() > cap) throw std::runtime_error("buffer too small");
      std::memcpy(px, im.px.data(), im.px.size() * sizeof(float));
    }
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
  return 0;
}

// BSDF batch: the BSDF is given in the reference's JSON form. wi, wo: n x 3
// local directions. f: n x 3 (cosine-weighted value), pdf: n.
int orc_bsdf_eval(const char* bsdfJson, const float* wi, const float* wo, int64_t n, float* f, float* pdf) {
  try {
    Json j = Json::parse(bsdfJson);
    auto b = MakeBsdf(&j);
    for (int64_t i = 0; i < n; i++) {
      V3 a(wi[i * 3], wi[i * 3 + 1], wi[i * 3 + 2]), o(wo[i * 3], wo[i * 3 + 1], wo[i * 3 + 2]);
      Spectrum v = b->Eval(a, o);
      f[i * 3] = v.x;
      f[i * 3 + 1] = v.y;
      f[i * 3 + 2] = v.z;
      pdf[i] = b->Pdf(a, o);
    }
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
  return 0;
}

// u: n x 3 (lobe, dir.x, dir.y). Out: wo n x 3, pdf n, f n x 3, eta n, type n.
int orc_bsdf_sample(const char* bsdfJson, const float* wi, const float* u, int64_t n, float* wo, float* pdf,
                    float* f, float* eta, uint32_t* type) {
  try {
    Json j = Json::parse(bsdfJson);
    auto b = MakeBsdf(&j);
    for (int64_t i = 0; i < n; i++) {
      V3 a(wi[i * 3], wi[i * 3 + 1], wi[i * 3 + 2]);
      auto r = b->Sample(a, u[i * 3], V2(u[i * 3 + 1], u[i * 3 + 2]));
      wo[i * 3] = r.first.Wo.x;
      wo[i * 3 + 1] = r.first.Wo.y;
      wo[i * 3 + 2] = r.first.Wo.z;
      pdf[i] = r.first.Pdf;
      f[i * 3] = r.second.x;
      f[i * 3 + 1] = r.second.y;
      f[i * 3 + 2] = r.second.z;
      eta[i] = r.first.Eta;
      type[i] = r.first.Type;
    }
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
  return 0;
}

// Fresnel known-answer hooks.
void orc_fresnel_dielectric(float cosThetaI, float eta, float* out4) {
  FresnelDielectric(cosThetaI, eta, out4[0], out4[1], out4[2], out4[3]);
}
void orc_fresnel_conductor(float cosThetaI, const float* eta, const float* k, float* out3) {
  Spectrum r = FresnelConductor(cosThetaI, V3(eta[0], eta[1], eta[2]), V3(k[0], k[1], k[2]));
  out3[0] = r.x;
  out3[1] = r.y;
  out3[2] = r.z;
}
// GGX / Beckmann D and G1 for normalisation checks.
float orc_microfacet_d(int ggx, float ax, float ay, const float* wh) {
  Microfacet m;
  m.ggx = ggx != 0;
  m.alphaX = ax;
  m.alphaY = ay;
  return m.D(V3(wh[0], wh[1], wh[2]));
}
uint32_t orc_pcg_u32(uint32_t pixel, uint32_t sample, uint32_t seed, int skip) {
  Pcg32 r = Pcg32::ForSample(pixel, sample, seed);
  for (int i = 0; i < skip; i++) r.NextU32();
  return r.NextU32();
}

}  // extern "C"
