// Renderer "bdpt" (bdpt.cpp:21-670): per pixel sample, a camera subpath and a
// light subpath, then every (s, t) connection between their vertices, each
// weighted by the multiple-importance weight over the strategies that could
// have made the same path. Connections with one camera vertex (t = 1) project
// to another pixel and are splatted into the film there.
//
// One thread runs one pixel sample; both subpaths live in the thread's local
// memory (kMaxBdptVertices each; a subpath stops there).
#pragma once
#include "dlight.cuh"

namespace rad {

constexpr int kMaxBdptVertices = 64;

enum : uint32_t { BV_CAMERA = 0, BV_LIGHT = 1, BV_SURFACE = 2 };

struct BVert {  // bdpt.cpp:29-44
  V3 P, N;     // position, geometric normal (zero: not on a surface)
  Frame sh;    // shading frame
  V3 Wi;       // surface: local incident direction
  V2 uv;       // surface: texture coordinates (textured scenes)
  V3 thr;      // throughput up to this vertex
  float pdfFwd, pdfRev;
  int32_t id;  // surface: shape; light: light
  uint32_t type;
  uint32_t delta;
};

RD bool VIsOnSurface(const BVert& v) { return !(v.N.x == 0.f && v.N.y == 0.f && v.N.z == 0.f); }
RD bool VIsInfinite(const DevScene& S, const BVert& v) {
  return v.type == BV_LIGHT && S.lights[v.id].kind == LIGHT_SKYBOX;
}
RD bool VIsLight(const DevScene& S, const BVert& v) {
  return v.type == BV_LIGHT || (v.type == BV_SURFACE && S.shapes[v.id].light >= 0);
}
RD int VLight(const DevScene& S, const BVert& v) { return v.type == BV_LIGHT ? v.id : S.shapes[v.id].light; }
RD uint32_t VMat(const DevScene& S, const BVert& v) { return (uint32_t)S.shapes[v.id].bsdf; }
// the camera, every light (no DeltaDirection light is built), BSDFs with a non-delta lobe
RD bool VConnectible(const DevScene& S, const BVert& v) {
  return v.type != BV_SURFACE || (S.mats[VMat(S, v)].flags & (BT_DIFFUSE | BT_GLOSSY)) != 0u;
}
RD TexCtx VTex(const DevScene& S, const BVert& v) {
  return TexCtx{S.tex, S.texels, S.texBind, v.uv, V2{0.f, 0.f}, V2{0.f, 0.f}};
}
// SurfaceInteraction(psr) (interaction.cpp:32-43)
RD BVert VFromPsr(uint32_t type, V3 P, V3 N) {
  BVert v{};
  v.type = type;
  v.P = P;
  v.N = N;
  v.sh = FrameFromN(N);
  v.Wi = v3s(0.f);
  v.thr = v3s(0.f);
  return v;
}

// PathVertex::ConvertDensity (bdpt.cpp:46-60)
RD float ConvertDensity(const DevScene& S, const BVert& v, float pdf, const BVert& next) {
  if (VIsInfinite(S, next)) return pdf;
  V3 w = next.P - v.P;
  float dist2 = sqnorm(w);
  if (dist2 == 0.f) return 0.f;
  float invDist2 = Rcp(dist2);
  if (VIsOnSurface(next)) pdf *= AbsDot(next.N, w * sqrtf(invDist2));
  return pdf * invDist2;
}

// BDPT::CorrectShadingNormal (bdpt.cpp:636-645)
RD float CorrectShadingNormal(const BVert& v, V3 wo) {
  float idn = dot(v.N, ToWorld(v.sh, v.Wi));
  float odn = dot(v.N, ToWorld(v.sh, wo));
  if (idn * v.Wi.z <= 0.f || odn * wo.z <= 0.f) return 0.f;
  float correction = (v.Wi.z * odn) / (wo.z * idn);
  return fabsf(correction);
}

// PathVertex::fs (bdpt.cpp:83-98)
RDN V3 VFs(const DevScene& S, const BVert& v, const BVert& next, bool imp) {
  if (v.type != BV_SURFACE) return v3s(0.f);
  V3 toNext = normalized(next.P - v.P);
  V3 wo = ToLocal(v.sh, toNext);
  float correction = imp ? CorrectShadingNormal(v, wo) : 1.f;
  TexCtx tcx = VTex(S, v);
  V3 f;
  float pdf;
  BsdfEvalPdf(S.mats, VMat(S, v), v.Wi, wo, f, pdf, S.nTex ? &tcx : nullptr, imp);
  return f * correction;
}

// PathVertex::Le (bdpt.cpp:99-117)
RD V3 VLe(const DevScene& S, const BVert& v, const BVert& other) {
  if (!VIsLight(S, v)) return v3s(0.f);
  int l = VLight(S, v);
  V3 toV = normalized(other.P - v.P);
  SurfInt si{};
  if (VIsInfinite(S, v)) {
    si.Wi = -toV;
  } else {
    si.N = v.N;
    si.sh = v.sh;
    si.Wi = ToLocal(v.sh, toV);
  }
  return EvalLightAt(S, l, &si);
}

// BDPT::InfiniteLightDensity (bdpt.cpp:658-663)
RD float InfiniteLightDensity(const DevScene& S, V3 w) {
  return PdfLightDirection(S, S.envLight, v3s(0.f), -w, v3s(0.f), 0.f);
}

// Shape::PdfPosition (mesh_base.cpp, rectangle.cpp, sphere.cpp): uniform by area
RD float ShapePdfPosition(const ShapeRec& sh) { return sh.kind == SHAPE_MESH ? sh.cdfNorm : 1.f / sh.surfaceArea; }

// Light::PdfLe (area.cpp:142-147, point.cpp:87-91, projection.cpp:122-133,
// skybox.cpp:206-212) for an emitting position (P, N) and direction.
RD void LightPdfLe(const DevScene& S, int light, V3 P, V3 N, V3 dir, float& pdfPos, float& pdfDir) {
  const LightRec& L = S.lights[light];
  if (L.kind == LIGHT_AREA) {
    Frame fr = FrameFromN(N);
    pdfPos = ShapePdfPosition(S.shapes[L.shape]);
    pdfDir = fabsf(SquareToCosineHemispherePdf(ToLocal(fr, dir)));
  } else if (L.kind == LIGHT_POINT) {
    pdfPos = 0.f;
    pdfDir = fabsf(SquareToUniformSpherePdf());
  } else if (L.kind == LIGHT_PROJECTION) {
    V3 refP = Affine4(L.m, P);
    V3 ndc = Affine4(L.m + 16, refP);
    float pd;
    if (ndc.x < 0.f || ndc.x >= 1.f || ndc.y < 0.f || ndc.y >= 1.f || ndc.z <= 0.f)
      pd = 0.f;
    else
      pd = 1.f / (L.m2[28] * kPi);
    pdfPos = 0.f;
    pdfDir = fabsf(pd);
  } else {  // skybox
    pdfPos = 1.f / (kPi * Sqr(L.world[3]));
    pdfDir = L.distW ? EnvDirPdf(S, L, dir) : SquareToUniformSpherePdf();
  }
}

// PathVertex::PdfLightOrigin (bdpt.cpp:118-131)
RD float PdfLightOrigin(const DevScene& S, const BVert& v, const BVert& other) {
  int l = VLight(S, v);
  if (VIsInfinite(S, v)) return InfiniteLightDensity(S, normalized(other.P - v.P));
  float pdfChoice = S.lightPdf;
  V3 w = normalized(other.P - v.P);
  float pdfPos, pdfDir;
  LightPdfLe(S, l, v.P, v.sh.N, w, pdfPos, pdfDir);
  return pdfPos * pdfChoice;
}

// PathVertex::PdfLight (bdpt.cpp:133-157)
RD float PdfLightV(const DevScene& S, const BVert& v, const BVert& next) {
  int l = VLight(S, v);
  V3 w = next.P - v.P;
  float invDist2 = 1.f / sqnorm(w);
  w = w * sqrtf(invDist2);
  float pdf, pdfPos, pdfDir;
  if (VIsInfinite(S, v)) {
    LightPdfLe(S, l, v3s(0.f), v3s(0.f), -w, pdfPos, pdfDir);
    pdf = pdfPos;
  } else {
    LightPdfLe(S, l, v.P, v.sh.N, w, pdfPos, pdfDir);
    pdf = pdfDir * invDist2;
  }
  if (VIsOnSurface(next)) pdf *= AbsDot(next.N, w);
  return pdf;
}

// Perspective::Importance / PdfWe (perspective.cpp:124-146)
RD float CameraPdfWe(const CameraRec& c, V3 worldDir) { return CameraImportance(c, LinearRows(c.worldToCam, worldDir)); }

// PathVertex::Pdf (bdpt.cpp:158-187): density of sampling next from v, coming from prev
RDN float VPdf(const DevScene& S, const BVert& v, const BVert* prev, const BVert& next) {
  if (v.type == BV_LIGHT) return PdfLightV(S, v, next);
  V3 wn = next.P - v.P;
  if (sqnorm(wn) == 0.f) return 0.f;
  wn = normalized(wn);
  V3 wp;
  if (prev) {
    wp = prev->P - v.P;
    if (sqnorm(wp) == 0.f) return 0.f;
    wp = normalized(wp);
  } else {
    return ConvertDensity(S, v, CameraPdfWe(S.cam, wn), next);
  }
  TexCtx tcx = VTex(S, v);
  V3 f;
  float pdf;
  BsdfEvalPdf(S.mats, VMat(S, v), ToLocal(v.sh, wp), ToLocal(v.sh, wn), f, pdf, S.nTex ? &tcx : nullptr, false);
  return ConvertDensity(S, v, pdf, next);
}

// BDPT::RandomWalk (bdpt.cpp:409-476)
RDN void RandomWalk(const DevScene& S, Pcg32& rng, V3 O, V3 D, float tmin, float tmax, V3 thr, float pdf, bool imp,
                   BVert* path, int& n, uint32_t* err) {
  float pdfFwd = pdf, pdfRev = 0.f;
  float rr = 1.f, eta = 1.f;
  for (int depth = 0;; depth++) {
    if (thr.x == 0.f && thr.y == 0.f && thr.z == 0.f) break;
    if (depth >= S.rrDepth) {
      float rrVal = fminr(max_comp(thr) * Sqr(eta), 0.95f);
      if (Next1D(rng) > rrVal) break;
      thr = thr * Rcp(rrVal);
      rr *= rrVal;
    }
    RayPre r = MakeRayPre(O, D, tmin);
    TraceHit h;
    if (!TraceBvh8<false>(S, r, tmax, h, err)) {
      if (S.envLight >= 0 && !imp && n < kMaxBdptVertices) {
        BVert& e = path[n++];
        e = BVert{};
        e.type = BV_LIGHT;
        e.id = S.envLight;
        e.P = D * -1.f + O;  // ray(-1)
        e.N = -D;
        e.thr = thr;
        e.pdfFwd = pdfFwd;
      }
      break;
    }
    SurfInt si = ComputeSI(S, O, D, h);
    const ShapeRec& shp = S.shapes[si.shape];
    if (shp.bsdf < 0) break;
    if (n >= kMaxBdptVertices) break;
    BVert& now = path[n];
    now.type = BV_SURFACE;
    now.id = si.shape;
    now.P = si.P;
    now.N = si.N;
    now.sh = si.sh;
    now.Wi = si.Wi;
    now.uv = S.nTex ? ComputeUV(S, h, si).uv : V2{0.f, 0.f};
    now.thr = thr;
    now.pdfRev = 0.f;
    now.delta = 0u;
    now.pdfFwd = ConvertDensity(S, path[n - 1], pdfFwd * rr, now);
    BVert& prev = path[n - 1];
    n++;
    if (S.maxDepth >= 0 && (depth + 1) > S.maxDepth) break;
    if (shp.light >= 0) break;
    const uint32_t mi = (uint32_t)shp.bsdf;
    TexCtx tcx = VTex(S, now);
    const TexCtx* tc = S.nTex ? &tcx : nullptr;
    float bl = Next1D(rng);
    V2 bd = Next2D(rng);
    BsdfSampleRes bs = BsdfSample(S.mats, mi, si.Wi, bl, bd, tc, imp);
    if (bs.pdf <= 0.f) break;
    bool isDelta = (bs.type & BT_DELTA) != 0u;
    float correction = imp ? CorrectShadingNormal(now, bs.wo) : 1.f;
    thr = cmul(thr, bs.f) * correction / bs.pdf;
    eta *= bs.eta;
    D = ToWorld(si.sh, bs.wo);
    O = OffsetP(si.P, si.N, D);
    tmin = 0.f;
    tmax = kFloatMax;
    pdfFwd = bs.pdf;
    if (isDelta) {
      pdfRev = pdfFwd;
      now.delta = 1u;
    } else {
      V3 f;
      BsdfEvalPdf(S.mats, mi, bs.wo, si.Wi, f, pdfRev, tc, imp);  // BsdfRevPdf (bdpt.cpp:647-651)
      now.delta = 0u;
    }
    prev.pdfRev = ConvertDensity(S, now, pdfRev * rr, prev);
  }
}

// Light::SampleLe (area.cpp:130-140, point.cpp:75-85, projection.cpp:107-120,
// skybox.cpp:170-204): emitted ray, radiance, emitting position and densities.
struct LeSample {
  V3 O, D, le, P, N;
  float pdfPos, pdfDir;
  bool delta;
};
RDN LeSample LightSampleLe(const DevScene& S, const LightRec& L, V2 xi2, V2 xi3) {
  LeSample r{};
  if (L.kind == LIGHT_AREA) {  // constant radiance
    const ShapeRec& sh = S.shapes[L.shape];
    float pdf;
    ShapeSamplePosition(S, sh, xi2, r.P, r.N, pdf);
    r.delta = sh.kind == SHAPE_SPHERE && sh.m[3] == 0.f;
    r.pdfPos = pdf > 0.f ? pdf : 0.f;
    V3 local = SquareToCosineHemisphere(xi3);
    r.pdfDir = SquareToCosineHemispherePdf(local);
    Frame fr = FrameFromN(r.N);
    r.D = ToWorld(fr, local);
    r.O = OffsetP(r.P, r.N, r.D);
    r.le = V3{L.radiance[0], L.radiance[1], L.radiance[2]};
  } else if (L.kind == LIGHT_POINT) {
    r.P = V3{L.dir[0], L.dir[1], L.dir[2]};
    r.N = v3s(0.f);
    r.delta = true;
    r.pdfPos = 1.f;
    V3 local = SquareToUniformSphere(xi3);
    r.pdfDir = SquareToUniformSpherePdf();
    Frame fr = FrameFromN(r.N);
    r.D = ToWorld(fr, local);
    r.O = OffsetP(r.P, r.N, r.D);
    r.le = V3{L.radiance[0], L.radiance[1], L.radiance[2]};
  } else if (L.kind == LIGHT_PROJECTION) {
    r.P = V3{L.dir[0], L.dir[1], L.dir[2]};
    r.N = ld3(L.lin);
    r.delta = true;
    r.pdfPos = 1.f;
    V3 nearP = Affine4(L.m2, V3{xi3.x, xi3.y, 0.f});
    V3 nearDir = normalized(nearP);
    r.O = r.P;
    r.D = LinearRows(L.m2 + 16, nearDir);
    r.le = V3{L.m2[29], L.m2[30], L.m2[31]};  // irradiance without the light's scale
    r.pdfDir = 1.f / (L.m2[28] * kPi);
  } else if (L.kind == LIGHT_SKYBOX) {
    V3 wc{L.world[0], L.world[1], L.world[2]};
    float R = L.world[3];
    V2 off = SquareToUniformDiskConcentric(xi2);
    float pdfDir;
    V2 uv;
    if (!L.distW) {
      pdfDir = SquareToUniformSpherePdf();
      uv = xi3;
    } else {
      V3 unused;
      if (!EnvSampleDir(S, L, xi3, unused, pdfDir, uv)) return LeSample{};
    }
    if (pdfDir <= 0.f) return LeSample{};
    float theta = uv.y * kPi, phi = uv.x * kPi * 2.f;
    float sinTheta = sinf(theta), cosTheta = cosf(theta), sinPhi = sinf(phi), cosPhi = cosf(phi);
    V3 sph{cosPhi * sinTheta, sinPhi * sinTheta, cosTheta};
    V3 d{sph.y, sph.z, -sph.x};
    V3 worldD = AffineRows(L.lin, -d);
    Frame fr = FrameFromN(d);
    V3 perp = ToWorld(fr, V3{off.x, off.y, 0.f});
    r.O = wc + (perp - worldD) * R;
    r.D = worldD;
    r.le = V3{L.radiance[0], L.radiance[1], L.radiance[2]};
    if (L.tex) {
      TexCtx x{S.tex, S.texels, S.texBind, uv, V2{0.f, 0.f}, V2{0.f, 0.f}};
      TexVal t = TexEval(x, L.tex - 1u, uv);
      r.le = V3{t.c[0], t.c[1], t.c[2]};
    }
    r.pdfPos = 1.f / (kPi * Sqr(R));
    r.pdfDir = pdfDir;
    r.P = r.O;
    r.N = r.D;
    r.delta = false;
  }
  return r;
}

// BDPT::GenerateLightPath (bdpt.cpp:371-407); a scene without lights has no light subpath
RD void GenerateLightPath(const DevScene& S, Pcg32& rng, BVert* path, int& n, uint32_t* err) {
  if (S.nLights == 0) return;
  int index;
  float selectPdf;
  PickLight(S, Next1D(rng), index, selectPdf);
  V2 xi2 = Next2D(rng);
  V2 xi3 = Next2D(rng);
  LeSample r = LightSampleLe(S, S.lights[index], xi2, xi3);
  if (r.pdfPos <= 0.f || r.pdfDir <= 0.f || (r.le.x == 0.f && r.le.y == 0.f && r.le.z == 0.f)) return;
  V3 thr = r.le * AbsDot(r.N, r.D) / (selectPdf * r.pdfPos * r.pdfDir);
  BVert& lv = path[n++];
  lv = VFromPsr(BV_LIGHT, r.P, r.N);
  lv.thr = r.le;
  lv.pdfFwd = r.pdfPos * selectPdf;
  lv.pdfRev = 0.f;
  lv.delta = r.delta ? 1u : 0u;
  lv.id = index;
  RandomWalk(S, rng, r.O, r.D, 0.f, kFloatMax, thr, r.pdfDir, true, path, n, err);
  if (VIsInfinite(S, path[0])) {
    if (n > 1) {
      path[1].pdfFwd = r.pdfPos;
      if (VIsOnSurface(path[1])) path[1].pdfFwd *= AbsDot(r.D, path[1].N);
    }
    path[0].pdfFwd = InfiniteLightDensity(S, r.D);
  }
}

// BDPT::MISWeight (bdpt.cpp:555-634): the strategy's vertex values are set in
// place and restored before returning, as the reference's scoped assignments do.
RDN float MISWeight(const DevScene& S, BVert* lightV, BVert* camV, const BVert& sampled, int s, int t) {
  if (s + t == 2) return 1.f;
  float sumRi = 0.f;
  if (!S.bdptMis) {
    for (int i = t - 1; i > 0; --i)
      if (!camV[i].delta && !camV[i - 1].delta) sumRi += 1.f;
    for (int i = s - 1; i >= 0; --i) {
      bool deltaLightvertex = i > 0 ? lightV[i - 1].delta != 0u : lightV[0].delta != 0u;
      if (!lightV[i].delta && !deltaLightvertex) sumRi += 1.f;
    }
    return 1.f / (1.f + sumRi);
  }
  BVert* qs = s > 0 ? &lightV[s - 1] : nullptr;
  BVert* pt = t > 0 ? &camV[t - 1] : nullptr;
  BVert* qsMinus = s > 1 ? &lightV[s - 2] : nullptr;
  BVert* ptMinus = t > 1 ? &camV[t - 2] : nullptr;
  BVert saveQs, savePt, saveQsMinus, savePtMinus;
  if (qs) saveQs = *qs;
  if (pt) savePt = *pt;
  if (qsMinus) saveQsMinus = *qsMinus;
  if (ptMinus) savePtMinus = *ptMinus;
  if (s == 1)
    *qs = sampled;
  else if (t == 1)
    *pt = sampled;
  if (pt) pt->delta = 0u;
  if (qs) qs->delta = 0u;
  if (pt) pt->pdfRev = s > 0 ? VPdf(S, *qs, qsMinus, *pt) : PdfLightOrigin(S, *pt, *ptMinus);
  if (ptMinus) ptMinus->pdfRev = s > 0 ? VPdf(S, *pt, qs, *ptMinus) : PdfLightV(S, *pt, *ptMinus);
  if (qs) qs->pdfRev = VPdf(S, *pt, ptMinus, *qs);
  if (qsMinus) qsMinus->pdfRev = VPdf(S, *qs, pt, *qsMinus);
  float ri = 1.f;
  for (int i = t - 1; i > 0; --i) {
    float rv = camV[i].pdfRev != 0.f ? camV[i].pdfRev : 1.f, fw = camV[i].pdfFwd != 0.f ? camV[i].pdfFwd : 1.f;
    ri *= rv / fw;
    if (!camV[i].delta && !camV[i - 1].delta) sumRi += ri;
  }
  ri = 1.f;
  for (int i = s - 1; i >= 0; --i) {
    float rv = lightV[i].pdfRev != 0.f ? lightV[i].pdfRev : 1.f, fw = lightV[i].pdfFwd != 0.f ? lightV[i].pdfFwd : 1.f;
    ri *= rv / fw;
    bool deltaLightvertex = i > 0 ? lightV[i - 1].delta != 0u : lightV[0].delta != 0u;
    if (!lightV[i].delta && !deltaLightvertex) sumRi += ri;
  }
  if (qsMinus) *qsMinus = saveQsMinus;
  if (ptMinus) *ptMinus = savePtMinus;
  if (qs) *qs = saveQs;
  if (pt) *pt = savePt;
  return 1.f / (1.f + sumRi);
}

RD bool IsBlack(V3 v) { return v.x == 0.f && v.y == 0.f && v.z == 0.f; }

// BDPT::ConnectBdpt (bdpt.cpp:478-553)
RDN V3 ConnectBdpt(const DevScene& S, Pcg32& rng, BVert* lightV, BVert* camV, int s, int t, V2& scrPos,
                  uint32_t* err) {
  V3 l = v3s(0.f);
  if (t > 1 && s != 0 && camV[t - 1].type == BV_LIGHT) return l;
  BVert sampled{};
  if (s == 0) {
    const BVert& pt = camV[t - 1];
    if (VIsLight(S, pt)) {
      V3 le = VLe(S, pt, camV[t - 2]);
      l = l + cmul(le, pt.thr);
    }
  } else if (t == 1) {
    const BVert& qs = lightV[s - 1];
    if (VConnectible(S, qs)) {
      Next2D(rng);  // Perspective::SampleDirection's sample (unused by a pinhole)
      V3 camP, camDir, camN;
      float camDist, we;
      V2 pixel;
      if (CameraSampleDirection(S.cam, qs.P, camP, camDir, camDist, pixel, we)) {
        camN = LinearRows(S.cam.camToWorld, V3{0.f, 0.f, 1.f});
        sampled = VFromPsr(BV_CAMERA, camP, camN);
        sampled.thr = v3s(we / 1.f);
        sampled.delta = 1u;
        V3 fs = VFs(S, qs, sampled, true);
        V3 result = cmul(cmul(qs.thr, fs), sampled.thr);
        scrPos = pixel;
        if (!IsBlack(result) && !LOccluded(S, qs.P, qs.N, camP, err)) l = l + result;
      }
    }
  } else if (s == 1) {
    const BVert& pt = camV[t - 1];
    if (VConnectible(S, pt)) {
      float xl = Next1D(rng);
      V2 xd = Next2D(rng);
      int index;
      float pick;
      if (PickLight(S, xl, index, pick)) {
        V3 li;
        DirSample dsr = LightSampleDirection(S, S.lights[index], pt.P, xd, li);
        dsr.Pdf *= pick;
        if (dsr.Pdf > 0.f) {
          sampled = VFromPsr(BV_LIGHT, dsr.P, dsr.N);
          sampled.thr = li / dsr.Pdf;
          sampled.delta = dsr.IsDelta ? 1u : 0u;
          sampled.id = index;
          sampled.pdfFwd = PdfLightOrigin(S, sampled, pt);
          V3 fs = VFs(S, pt, sampled, false);
          V3 result = cmul(cmul(pt.thr, fs), sampled.thr);
          if (!IsBlack(result) && !LOccluded(S, pt.P, pt.N, dsr.P, err)) l = l + result;
        }
      }
    }
  } else {
    const BVert& qs = lightV[s - 1];
    const BVert& pt = camV[t - 1];
    if (VConnectible(S, qs) && VConnectible(S, pt)) {
      V3 lightFs = VFs(S, qs, pt, true);
      V3 cameraFs = VFs(S, pt, qs, false);
      float g = 1.f / sqnorm(qs.P - pt.P);  // BDPT::G (bdpt.cpp:652-656)
      V3 result = cmul(cmul(cmul(qs.thr, lightFs), cameraFs), pt.thr) * g;
      if (!IsBlack(result) && !LOccluded(S, pt.P, pt.N, qs.P, err)) l = l + result;
    }
  }
  if (IsBlack(l)) return l;
  float mis = MISWeight(S, lightV, camV, sampled, s, t);
  return l * mis;
}

// One pixel sample (BDPT::Render + Li, bdpt.cpp:261-349): returns the camera-side
// sum (t >= 2); t = 1 connections are splatted into `film` when it is set.
RDN V3 BdptSample(const DevScene& S, const ParticleFilm* film, uint32_t pix, uint32_t smp, uint32_t seed,
                 uint32_t* err) {
  Pcg32 rng = PcgForSample(pix, smp, seed);
  uint32_t x = pix % (uint32_t)S.cam.width, y = pix / (uint32_t)S.cam.width;
  float jx = Next1D(rng);
  float jy = Next1D(rng);
  V3 O, D;
  float tmin, tmax;
  CameraRay(S.cam, (float)x + jx, (float)y + jy, O, D, tmin, tmax);
  BVert camV[kMaxBdptVertices];
  BVert lightV[kMaxBdptVertices];
  int nc = 0, nl = 0;
  // BDPT::GenerateCameraPath (bdpt.cpp:351-369)
  float pdfDir = CameraPdfWe(S.cam, D);
  camV[0] = BVert{};
  camV[0].type = BV_CAMERA;
  camV[0].thr = v3s(1.f);
  camV[0].P = O;
  nc = 1;
  RandomWalk(S, rng, O, D, tmin, tmax, v3s(1.f), pdfDir, false, camV, nc, err);
  GenerateLightPath(S, rng, lightV, nl, err);
  V3 l = v3s(0.f);
  for (int t = 1; t <= nc; ++t) {
    for (int s = 0; s <= nl; ++s) {
      int depth = t + s - 2;
      if ((s == 1 && t == 1) || depth < 0) continue;
      V2 scrPos{(float)x, (float)y};
      V3 pathL = ConnectBdpt(S, rng, lightV, camV, s, t, scrPos, err);
      if (t == 1) {
        if (film && !IsBlack(pathL)) Splat(*film, scrPos, pathL);
      } else {
        l = l + pathL;
      }
    }
  }
  return l;
}

}  // namespace rad
