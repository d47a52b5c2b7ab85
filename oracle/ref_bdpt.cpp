// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_core.h).
// Renderer "bdpt" (rad.offline/src/renderer/bdpt.cpp:21-670): a camera subpath
// and a light subpath per pixel sample, every (s, t) connection between them,
// weighted by the multiple-importance weight over all strategies that could
// have made the same path (MISWeight, bdpt.cpp:555-634). Connections with one
// camera vertex (t = 1) are splatted into the film at the pixel they project
// to. Subpaths stop at kMaxBdptVertices vertices, as on the GPU.
#include "ref_scene.h"

namespace orc {

constexpr int kMaxBdptVertices = 64;

struct PathVertex {  // bdpt.cpp:29-44
  enum Kind { Camera, Light, Surface } type = Camera;
  SurfaceInteraction si;
  Spectrum thr = Spectrum(0);
  Float pdfFwd = 0, pdfRev = 0;
  bool isDelta = false;
  int light = -1;
  const V3& p() const { return si.P; }
  const V3& ng() const { return si.N; }
};

// SurfaceInteraction(psr) (interaction.cpp:32-43)
static SurfaceInteraction FromPsr(const PositionSample& psr) {
  SurfaceInteraction si;
  si.P = psr.P;
  si.N = psr.N;
  si.UV = psr.UV;
  si.Shading = Frame(psr.N);
  si.T = 0;
  si.Wi = V3(0);
  return si;
}
// SurfaceInteraction::ToPsr (interaction.cpp:59-67)
static PositionSample ToPsr(const SurfaceInteraction& si) {
  PositionSample psr;
  psr.P = si.P;
  psr.N = si.Shading.N;
  psr.UV = si.UV;
  return psr;
}

static bool IsOnSurface(const PathVertex& v) { return !(v.si.N.x == 0 && v.si.N.y == 0 && v.si.N.z == 0); }
static bool IsInfiniteLight(const Scene& S, const PathVertex& v) {
  return v.type == PathVertex::Light && S.lights[v.light].kind == Light::Skybox;
}
static bool IsLight(const Scene& S, const PathVertex& v) {
  return v.type == PathVertex::Light || (v.type == PathVertex::Surface && S.shapes[v.si.shape].light >= 0);
}
static int GetLight(const Scene& S, const PathVertex& v) {
  return v.type == PathVertex::Light ? v.light : S.shapes[v.si.shape].light;
}
static bool IsConnectible(const Scene& S, const PathVertex& v) {
  if (v.type == PathVertex::Surface) return S.bsdfs[S.shapes[v.si.shape].bsdf]->HasAnyTypeExceptDelta();
  return true;  // the camera, and every light but a DeltaDirection one (none is built)
}
static const Bsdf& BsdfOf(const Scene& S, const PathVertex& v) { return *S.bsdfs[S.shapes[v.si.shape].bsdf]; }
static TexSi TexOf(const SurfaceInteraction& si, bool importance) {
  TexSi ts{si.UV, V2(), V2()};
  ts.importance = importance;
  return ts;
}

// PathVertex::ConvertDensity (bdpt.cpp:46-60): solid angle -> area density at next
static Float ConvertDensity(const Scene& S, const PathVertex& v, Float pdf, const PathVertex& next) {
  if (IsInfiniteLight(S, next)) return pdf;
  V3 w = next.p() - v.p();
  Float dist2 = sqnorm(w);
  if (dist2 == 0) return 0;
  Float invDist2 = Rcp(dist2);
  if (IsOnSurface(next)) pdf *= std::abs(dot(next.ng(), w * std::sqrt(invDist2)));
  return pdf * invDist2;
}

// BDPT::CorrectShadingNormal (bdpt.cpp:636-645)
static Float CorrectShadingNormal(const SurfaceInteraction& si, const V3& wo) {
  Float idn = dot(si.N, si.ToWorld(si.Wi));
  Float odn = dot(si.N, si.ToWorld(wo));
  if (idn * Frame::CosTheta(si.Wi) <= 0 || odn * Frame::CosTheta(wo) <= 0) return 0;
  Float correction = (Frame::CosTheta(si.Wi) * odn) / (Frame::CosTheta(wo) * idn);
  return std::abs(correction);
}

// PathVertex::fs (bdpt.cpp:83-98)
static Spectrum Fs(const Scene& S, const PathVertex& v, const PathVertex& next, bool importance) {
  if (v.type != PathVertex::Surface) return Spectrum(0);
  V3 toNext = normalized(next.p() - v.p());
  V3 wo = v.si.ToLocal(toNext);
  Float correction = importance ? CorrectShadingNormal(v.si, wo) : Float(1);
  TexSi ts = TexOf(v.si, importance);
  Spectrum f = BsdfOf(S, v).Eval(v.si.Wi, wo, &ts);
  return f * correction;
}

// PathVertex::Le (bdpt.cpp:99-117)
static Spectrum Le(const Scene& S, const PathVertex& v, const PathVertex& other) {
  if (!IsLight(S, v)) return Spectrum(0);
  int l = GetLight(S, v);
  V3 toV = normalized(other.p() - v.p());
  if (IsInfiniteLight(S, v)) {
    SurfaceInteraction si;
    si.Wi = -toV;
    return S.EvalLight(l, si);
  }
  SurfaceInteraction tsi = v.si;
  tsi.Wi = v.si.ToLocal(toV);
  return S.EvalLight(l, tsi);
}

// BDPT::InfiniteLightDensity (bdpt.cpp:658-663)
static Float InfiniteLightDensity(const Scene& S, const V3& w) {
  DirectionSample dsr;
  dsr.Dir = -w;
  return S.PdfLightDirection(S.envLight, V3(0), dsr);
}

// PathVertex::PdfLightOrigin (bdpt.cpp:118-131)
static Float PdfLightOrigin(const Scene& S, const PathVertex& v, const PathVertex& other) {
  int l = GetLight(S, v);
  if (IsInfiniteLight(S, v)) return InfiniteLightDensity(S, normalized(other.p() - v.p()));
  Float pdfChoice = S.lightPdf;  // Scene::PdfLight (scene.cpp:83-85)
  V3 w = normalized(other.p() - v.p());
  Float pdfPos = S.LightPdfLe(l, ToPsr(v.si), w).first;
  return pdfPos * pdfChoice;
}

// PathVertex::PdfLight (bdpt.cpp:133-157)
static Float PdfLight(const Scene& S, const PathVertex& v, const PathVertex& next) {
  int l = GetLight(S, v);
  V3 w = next.p() - v.p();
  Float invDist2 = 1 / sqnorm(w);
  w = w * std::sqrt(invDist2);
  Float pdf;
  if (IsInfiniteLight(S, v)) {
    pdf = S.LightPdfLe(l, PositionSample(), -w).first;
  } else {
    pdf = S.LightPdfLe(l, ToPsr(v.si), w).second * invDist2;
  }
  if (IsOnSurface(next)) pdf *= std::abs(dot(next.ng(), w));
  return pdf;
}

// PathVertex::Pdf (bdpt.cpp:158-187): density of sampling next from v, having come from prev
static Float Pdf(const Scene& S, const PathVertex& v, const PathVertex* prev, const PathVertex& next) {
  if (v.type == PathVertex::Light) return PdfLight(S, v, next);
  V3 wn = next.p() - v.p();
  if (sqnorm(wn) == 0) return 0;
  wn = normalized(wn);
  V3 wp;
  if (prev) {
    wp = prev->p() - v.p();
    if (sqnorm(wp) == 0) return 0;
    wp = normalized(wp);
  } else {
    return ConvertDensity(S, v, S.camera.PdfWe(wn), next);
  }
  TexSi ts = TexOf(v.si, false);
  Float pdf = BsdfOf(S, v).Pdf(v.si.ToLocal(wp), v.si.ToLocal(wn), &ts);
  return ConvertDensity(S, v, pdf, next);
}

// BDPT::RandomWalk (bdpt.cpp:409-476)
static void RandomWalk(const Scene& S, Pcg32& rng, Ray ray, Spectrum throughput, Float pdf, bool importance,
                       std::vector<PathVertex>& path) {
  Float pdfFwd = pdf, pdfRev = 0;
  Float rr = 1, eta = 1;
  for (int depth = 0;; depth++) {
    if (is_zero(throughput)) break;
    if (depth >= S.rrDepth) {
      Float rrVal = std::min(max_comp(throughput) * Sqr(eta), Float(0.95));
      if (rng.Next1D() > rrVal) break;
      throughput = throughput * Rcp(rrVal);
      rr *= rrVal;
    }
    SurfaceInteraction si;
    bool isHit = S.RayIntersect(ray, si);
    if (!isHit) {
      if (S.envLight >= 0 && !importance && path.size() < (size_t)kMaxBdptVertices) {
        PathVertex vex;
        vex.type = PathVertex::Light;
        vex.light = S.envLight;
        vex.si.P = ray.At(-1);
        vex.si.N = -ray.D;
        vex.thr = throughput;
        vex.pdfFwd = pdfFwd;
        path.push_back(vex);
      }
      break;
    }
    const Shape& sh = S.shapes[si.shape];
    if (sh.bsdf < 0) break;
    if (path.size() >= (size_t)kMaxBdptVertices) break;
    PathVertex now;
    now.type = PathVertex::Surface;
    now.si = si;
    now.thr = throughput;
    now.pdfRev = 0;
    now.pdfFwd = ConvertDensity(S, path.back(), pdfFwd * rr, now);
    path.push_back(now);
    PathVertex& cur = path[path.size() - 1];
    PathVertex& prev = path[path.size() - 2];
    if (S.maxDepth >= 0 && (depth + 1) > S.maxDepth) break;
    if (sh.light >= 0) break;
    const Bsdf& bsdf = *S.bsdfs[sh.bsdf];
    TexSi ts = TexOf(si, importance);
    Float bl = rng.Next1D();
    V2 bd = rng.Next2D();
    auto bs = bsdf.Sample(si.Wi, bl, bd, &ts);
    if (bs.first.Pdf <= 0) break;
    bool isDelta = (bs.first.Type & BT_Delta) != 0;
    Float correction = importance ? CorrectShadingNormal(si, bs.first.Wo) : Float(1);
    throughput = cmul(throughput, bs.second) * correction / bs.first.Pdf;
    eta *= bs.first.Eta;
    ray = SpawnRay(si.P, si.N, si.ToWorld(bs.first.Wo));
    pdfFwd = bs.first.Pdf;
    if (isDelta) {
      pdfRev = pdfFwd;
      cur.isDelta = true;
    } else {
      pdfRev = bsdf.Pdf(bs.first.Wo, si.Wi, &ts);  // BsdfRevPdf (bdpt.cpp:647-651)
      cur.isDelta = false;
    }
    prev.pdfRev = ConvertDensity(S, cur, pdfRev * rr, prev);
  }
}

// BDPT::GenerateCameraPath (bdpt.cpp:351-369)
static void GenerateCameraPath(const Scene& S, Pcg32& rng, const Ray& ray, std::vector<PathVertex>& path) {
  Float pdfDir = S.camera.PdfWe(ray.D);
  PathVertex c;
  c.type = PathVertex::Camera;
  c.thr = Spectrum(1);
  c.si.P = ray.O;
  path.push_back(c);
  RandomWalk(S, rng, ray, c.thr, pdfDir, false, path);
}

// BDPT::GenerateLightPath (bdpt.cpp:371-407). A scene without lights has no
// light subpath (the reference indexes light -1).
static void GenerateLightPath(const Scene& S, Pcg32& rng, std::vector<PathVertex>& path) {
  if (S.lights.empty()) return;
  int index;
  Float selectPdf;
  S.SampleLight(rng.Next1D(), index, selectPdf);
  V2 xi2 = rng.Next2D();
  V2 xi3 = rng.Next2D();
  Scene::LeSample r = S.LightSampleLe(index, xi2, xi3);
  if (r.pdfPos <= 0 || r.pdfDir <= 0 || is_zero(r.le)) return;
  Spectrum throughput = r.le * std::abs(dot(r.psr.N, r.ray.D)) / (selectPdf * r.pdfPos * r.pdfDir);
  PathVertex lv;
  lv.type = PathVertex::Light;
  lv.thr = r.le;
  lv.pdfFwd = r.pdfPos * selectPdf;
  lv.si = FromPsr(r.psr);
  lv.isDelta = r.psr.IsDelta;
  lv.light = index;
  path.push_back(lv);
  RandomWalk(S, rng, r.ray, throughput, r.pdfDir, true, path);
  if (IsInfiniteLight(S, lv)) {
    if (path.size() > 1) {
      path[1].pdfFwd = r.pdfPos;
      if (IsOnSurface(path[1])) path[1].pdfFwd *= std::abs(dot(r.ray.D, path[1].ng()));
    }
    path[0].pdfFwd = InfiniteLightDensity(S, r.ray.D);
  }
}

// BDPT::MISWeight (bdpt.cpp:555-634). The reference assigns the strategy's
// temporary vertex values in place and restores them on return; so does this.
static Float MISWeight(const Scene& S, std::vector<PathVertex>& lightV, std::vector<PathVertex>& camV,
                       const PathVertex& sampled, int s, int t) {
  if (s + t == 2) return 1;
  Float sumRi = 0;
  if (!S.useMis) {
    for (int i = t - 1; i > 0; --i)
      if (!camV[i].isDelta && !camV[i - 1].isDelta) sumRi++;
    for (int i = s - 1; i >= 0; --i) {
      bool deltaLightvertex = i > 0 ? lightV[i - 1].isDelta : lightV[0].isDelta;
      if (!lightV[i].isDelta && !deltaLightvertex) sumRi++;
    }
    return 1 / (1 + sumRi);
  }
  auto remap0 = [](Float f) -> Float { return f != 0 ? f : 1; };
  PathVertex* qs = s > 0 ? &lightV[s - 1] : nullptr;
  PathVertex* pt = t > 0 ? &camV[t - 1] : nullptr;
  PathVertex* qsMinus = s > 1 ? &lightV[s - 2] : nullptr;
  PathVertex* ptMinus = t > 1 ? &camV[t - 2] : nullptr;
  // saved originals of every vertex touched below (ScopedAssignment)
  PathVertex saveQs, savePt, saveQsMinus, savePtMinus;
  if (qs) saveQs = *qs;
  if (pt) savePt = *pt;
  if (qsMinus) saveQsMinus = *qsMinus;
  if (ptMinus) savePtMinus = *ptMinus;
  if (s == 1)
    *qs = sampled;
  else if (t == 1)
    *pt = sampled;
  if (pt) pt->isDelta = false;
  if (qs) qs->isDelta = false;
  if (pt) pt->pdfRev = s > 0 ? Pdf(S, *qs, qsMinus, *pt) : PdfLightOrigin(S, *pt, *ptMinus);
  if (ptMinus) ptMinus->pdfRev = s > 0 ? Pdf(S, *pt, qs, *ptMinus) : PdfLight(S, *pt, *ptMinus);
  if (qs) qs->pdfRev = Pdf(S, *pt, ptMinus, *qs);
  if (qsMinus) qsMinus->pdfRev = Pdf(S, *qs, pt, *qsMinus);
  Float ri = 1;
  for (int i = t - 1; i > 0; --i) {
    ri *= remap0(camV[i].pdfRev) / remap0(camV[i].pdfFwd);
    if (!camV[i].isDelta && !camV[i - 1].isDelta) sumRi += ri;
  }
  ri = 1;
  for (int i = s - 1; i >= 0; --i) {
    ri *= remap0(lightV[i].pdfRev) / remap0(lightV[i].pdfFwd);
    bool deltaLightvertex = i > 0 ? lightV[i - 1].isDelta : lightV[0].isDelta;
    if (!lightV[i].isDelta && !deltaLightvertex) sumRi += ri;
  }
  if (qsMinus) *qsMinus = saveQsMinus;
  if (ptMinus) *ptMinus = savePtMinus;
  if (qs) *qs = saveQs;
  if (pt) *pt = savePt;
  return 1 / (1 + sumRi);
}

// BDPT::ConnectBdpt (bdpt.cpp:478-553)
static Spectrum ConnectBdpt(const Scene& S, Pcg32& rng, std::vector<PathVertex>& lightV,
                            std::vector<PathVertex>& camV, int s, int t, V2& scrPos) {
  Spectrum l(0);
  if (t > 1 && s != 0 && camV[t - 1].type == PathVertex::Light) return l;
  PathVertex sampled;
  if (s == 0) {
    const PathVertex& pt = camV[t - 1];
    if (IsLight(S, pt)) {
      Spectrum le = Le(S, pt, camV[t - 2]);
      l = l + cmul(le, pt.thr);
    }
  } else if (t == 1) {
    const PathVertex& qs = lightV[s - 1];
    if (IsConnectible(S, qs)) {
      rng.Next2D();  // Perspective::SampleDirection's sample (unused by a pinhole)
      DirectionSample dsr;
      Float we = S.camera.SampleDirection(qs.p(), dsr);
      if (dsr.Pdf > 0) {
        sampled.type = PathVertex::Camera;
        sampled.thr = Spectrum(we / dsr.Pdf);
        sampled.si = FromPsr(dsr);
        sampled.isDelta = true;
        Spectrum fs = Fs(S, qs, sampled, true);
        Spectrum result = cmul(cmul(qs.thr, fs), sampled.thr);
        scrPos = dsr.UV;
        if (!is_zero(result) && !S.IsOcclude(qs.si.P, qs.si.N, dsr.P)) l = l + result;
      }
    }
  } else if (s == 1) {
    const PathVertex& pt = camV[t - 1];
    if (IsConnectible(S, pt)) {
      Float xl = rng.Next1D();
      V2 xd = rng.Next2D();
      int index;
      Float pick;
      S.SampleLight(xl, index, pick);
      if (index >= 0) {
        auto r = S.SampleOneLightDirection(index, pt.p(), xd);
        DirectionSample& dsr = r.first;
        dsr.Pdf *= pick;
        if (dsr.Pdf > 0) {
          sampled.type = PathVertex::Light;
          sampled.thr = r.second / dsr.Pdf;
          sampled.si = FromPsr(dsr);
          sampled.isDelta = dsr.IsDelta;
          sampled.light = index;
          sampled.pdfFwd = PdfLightOrigin(S, sampled, pt);
          Spectrum fs = Fs(S, pt, sampled, false);
          Spectrum result = cmul(cmul(pt.thr, fs), sampled.thr);
          if (!is_zero(result) && !S.IsOcclude(pt.si.P, pt.si.N, dsr.P)) l = l + result;
        }
      }
    }
  } else {
    const PathVertex& qs = lightV[s - 1];
    const PathVertex& pt = camV[t - 1];
    if (IsConnectible(S, qs) && IsConnectible(S, pt)) {
      Spectrum lightFs = Fs(S, qs, pt, true);
      Spectrum cameraFs = Fs(S, pt, qs, false);
      Float g = 1 / sqnorm(qs.p() - pt.p());  // BDPT::G (bdpt.cpp:652-656)
      Spectrum result = cmul(cmul(cmul(qs.thr, lightFs), cameraFs), pt.thr) * g;
      if (!is_zero(result) && !S.IsOcclude(pt.si.P, pt.si.N, qs.p())) l = l + result;
    }
  }
  if (is_zero(l)) return l;
  Float mis = MISWeight(S, lightV, camV, sampled, s, t);
  return l * mis;
}

// One pixel sample (BDPT::Render + Li, bdpt.cpp:261-349): returns the camera-side
// sum (t >= 2) and adds the t = 1 splats into `film` (W x H, may be null).
Spectrum BdptSample(const Scene& S, uint32_t x, uint32_t y, uint32_t s, uint32_t seed, std::vector<Spectrum>* film) {
  const int W = S.camera.width;
  Pcg32 rng = Pcg32::ForSample(x + y * (uint32_t)W, s, seed);
  Float jx = rng.Next1D();
  Float jy = rng.Next1D();
  Ray ray = S.camera.SampleRay(V2(Float(x) + jx, Float(y) + jy));
  std::vector<PathVertex> camV, lightV;
  camV.reserve(kMaxBdptVertices);
  lightV.reserve(kMaxBdptVertices);
  GenerateCameraPath(S, rng, ray, camV);
  GenerateLightPath(S, rng, lightV);
  Spectrum l(0);
  for (int t = 1; t <= (int)camV.size(); ++t) {
    for (int s = 0; s <= (int)lightV.size(); ++s) {
      int depth = t + s - 2;
      if ((s == 1 && t == 1) || depth < 0) continue;
      V2 scrPos((Float)x, (Float)y);
      Spectrum pathL = ConnectBdpt(S, rng, lightV, camV, s, t, scrPos);
      if (t == 1) {
        if (film && !is_zero(pathL)) {
          Spectrum& px = (*film)[(size_t)(int)scrPos.y * W + (int)scrPos.x];
          px = px + pathL;
        }
      } else {
        l = l + pathL;
      }
    }
  }
  return l;
}

}  // namespace orc
