// Renderer "bdpt" (bdpt.cpp:21-670): per pixel sample, a camera subpath and a
// light subpath, then every (s, t) connection between their vertices, each
// weighted by the multiple-importance weight over the strategies that could
// have made the same path. Connections with one camera vertex (t = 1) project
// to another pixel and are splatted into the film there.
//
// The functions here are the per-sample steps of that algorithm; the kernels
// (k_bdpt.cu) run them as a wavefront: each subpath bounce between two
// launches of the BVH8 closest-hit kernel, the connections of one camera
// vertex index per launch, their visibility rays through the any-hit kernel.
// A subpath's vertices live in device memory strided by the wave size; a
// subpath stops at kMaxBdptVertices vertices.
#pragma once
#include "dlight.cuh"

namespace rad {

enum : uint32_t { BV_CAMERA = 0, BV_LIGHT = 1, BV_SURFACE = 2 };

struct BVert {  // bdpt.cpp:29-44, 112 bytes
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

// One sample's subpath: vertex k at v[k * stride].
struct VPath {
  BVert* v;
  uint32_t stride;
  RD BVert& operator[](int k) const { return v[(size_t)k * stride]; }
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
  return EvalLightAt(S, l, &si, v.uv);
}

// BDPT::InfiniteLightDensity (bdpt.cpp:658-663)
RD float InfiniteLightDensity(const DevScene& S, V3 w) {
  return PdfLightDirection(S, S.envLight, v3s(0.f), -w, v3s(0.f), 0.f, V2{0.f, 0.f});
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

// Walk state of one subpath between two traces (BDPT::RandomWalk's locals).
struct WalkState {
  V3 thr;
  float eta, pdfFwd, rr;
  int n;  // vertices so far
};

// Top of RandomWalk's loop for bounce `depth` (bdpt.cpp:418-428): a black
// throughput ends the walk, then Russian roulette from rr_depth.
RD bool WalkContinue(const DevScene& S, Pcg32& rng, WalkState& w, int depth) {
  if (IsBlack(w.thr)) return false;
  if (depth >= S.rrDepth) {
    float rrVal = fminr(max_comp(w.thr) * Sqr(w.eta), 0.95f);
    if (Next1D(rng) > rrVal) return false;
    w.thr = w.thr * Rcp(rrVal);
    w.rr *= rrVal;
  }
  return true;
}

// The rest of RandomWalk's bounce `depth` (bdpt.cpp:429-475) once ray (O, D)
// has been traced: the miss (an environment vertex on camera subpaths) or the
// surface vertex, the BSDF sample and the reverse density of the previous
// vertex. Returns true with the next ray in (O, D) when the walk goes on.
RDN bool WalkStep(const DevScene& S, Pcg32& rng, VPath path, int cap, WalkState& w, int depth, bool imp, bool hit,
                  const TraceHit& h, V3& O, V3& D) {
  if (!hit) {
    if (S.envLight >= 0 && !imp && w.n < cap) {
      BVert e{};
      e.type = BV_LIGHT;
      e.id = S.envLight;
      e.P = D * -1.f + O;  // ray(-1)
      e.N = -D;
      e.thr = w.thr;
      e.pdfFwd = w.pdfFwd;
      path[w.n++] = e;
    }
    return false;
  }
  SurfInt si = ComputeSI(S, O, D, h);
  const ShapeRec& shp = S.shapes[si.shape];
  if (shp.bsdf < 0) return false;
  if (w.n >= cap) return false;
  BVert now;
  now.type = BV_SURFACE;
  now.id = si.shape;
  now.P = si.P;
  now.N = si.N;
  now.sh = si.sh;
  now.Wi = si.Wi;
  now.uv = S.nTex ? ComputeUV(S, h, si).uv : V2{0.f, 0.f};
  now.thr = w.thr;
  now.pdfRev = 0.f;
  now.delta = 0u;
  const BVert prev = path[w.n - 1];
  now.pdfFwd = ConvertDensity(S, prev, w.pdfFwd * w.rr, now);
  const int k = w.n++;
  bool go = !(S.maxDepth >= 0 && (depth + 1) > S.maxDepth) && shp.light < 0;
  BsdfSampleRes bs{};
  const uint32_t mi = (uint32_t)shp.bsdf;
  TexCtx tcx = VTex(S, now);
  const TexCtx* tc = S.nTex ? &tcx : nullptr;
  if (go) {
    float bl = Next1D(rng);
    V2 bd = Next2D(rng);
    bs = BsdfSample(S.mats, mi, si.Wi, bl, bd, tc, imp);
    go = !(bs.pdf <= 0.f);
  }
  if (!go) {
    path[k] = now;
    return false;
  }
  bool isDelta = (bs.type & BT_DELTA) != 0u;
  float correction = imp ? CorrectShadingNormal(now, bs.wo) : 1.f;
  w.thr = cmul(w.thr, bs.f) * correction / bs.pdf;
  w.eta *= bs.eta;
  D = ToWorld(si.sh, bs.wo);
  O = OffsetP(si.P, si.N, D);
  w.pdfFwd = bs.pdf;
  float pdfRev;
  if (isDelta) {
    pdfRev = w.pdfFwd;
    now.delta = 1u;
  } else {
    V3 f;
    BsdfEvalPdf(S.mats, mi, bs.wo, si.Wi, f, pdfRev, tc, imp);  // BsdfRevPdf (bdpt.cpp:647-651)
  }
  path[k] = now;
  path[k - 1].pdfRev = ConvertDensity(S, now, pdfRev * w.rr, prev);
  return true;
}

// BDPT::GenerateCameraPath (bdpt.cpp:351-369) up to its first trace: the
// jittered camera ray of pixel sample (pix, smp) and the camera vertex.
RD void CameraPathStart(const DevScene& S, Pcg32& rng, uint32_t pix, VPath path, WalkState& w, V3& O, V3& D,
                        float& tmin, float& tmax) {
  uint32_t x = pix % (uint32_t)S.cam.width, y = pix / (uint32_t)S.cam.width;
  float jx = Next1D(rng);
  float jy = Next1D(rng);
  CameraRay(S.cam, (float)x + jx, (float)y + jy, O, D, tmin, tmax);
  BVert c{};
  c.type = BV_CAMERA;
  c.thr = v3s(1.f);
  c.P = O;
  path[0] = c;
  w.thr = v3s(1.f);
  w.eta = 1.f;
  w.pdfFwd = CameraPdfWe(S.cam, D);
  w.rr = 1.f;
  w.n = 1;
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
  if (L.kind == LIGHT_AREA) {
    const ShapeRec& sh = S.shapes[L.shape];
    V2 uv;
    AreaSamplePosition(S, L, xi2, r.P, r.N, uv, r.pdfPos);
    r.delta = !L.tex && sh.kind == SHAPE_SPHERE && sh.m[3] == 0.f;
    V3 local = SquareToCosineHemisphere(xi3);
    r.pdfDir = SquareToCosineHemispherePdf(local);
    Frame fr = FrameFromN(r.N);
    r.D = ToWorld(fr, local);
    r.O = OffsetP(r.P, r.N, r.D);
    r.le = AreaRadiance(S, L, uv);  // Eval(si) with no incident direction: dot(0, N) >= 0
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
    if (L.tex) {
      r.le = LightTex(S, L.tex, xi3);
    }
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
      r.le = LightTex(S, L.tex, uv);
    }
    r.pdfPos = 1.f / (kPi * Sqr(R));
    r.pdfDir = pdfDir;
    r.P = r.O;
    r.N = r.D;
    r.delta = false;
  }
  return r;
}

// Direction and position density of the emitted ray, kept for the fix-up of
// infinite-light subpaths once the walk is over (bdpt.cpp:398-406).
struct LightFix {
  V3 D;
  float pdfPos;
};

// BDPT::GenerateLightPath (bdpt.cpp:371-397) up to its first trace: the light
// pick, the emitted ray and the light vertex. False when there is no light
// subpath (no light, or a zero density or radiance).
RD bool LightPathStart(const DevScene& S, Pcg32& rng, VPath path, WalkState& w, V3& O, V3& D, LightFix& fix) {
  w.n = 0;
  if (S.nLights == 0) return false;
  int index;
  float selectPdf;
  PickLight(S, Next1D(rng), index, selectPdf);
  V2 xi2 = Next2D(rng);
  V2 xi3 = Next2D(rng);
  LeSample r = LightSampleLe(S, S.lights[index], xi2, xi3);
  if (r.pdfPos <= 0.f || r.pdfDir <= 0.f || IsBlack(r.le)) return false;
  BVert lv = VFromPsr(BV_LIGHT, r.P, r.N);
  lv.thr = r.le;
  lv.pdfFwd = r.pdfPos * selectPdf;
  lv.pdfRev = 0.f;
  lv.delta = r.delta ? 1u : 0u;
  lv.id = index;
  path[0] = lv;
  w.thr = r.le * AbsDot(r.N, r.D) / (selectPdf * r.pdfPos * r.pdfDir);
  w.eta = 1.f;
  w.pdfFwd = r.pdfDir;
  w.rr = 1.f;
  w.n = 1;
  O = r.O;
  D = r.D;
  fix.D = r.D;
  fix.pdfPos = r.pdfPos;
  return true;
}

// bdpt.cpp:398-406: an infinite light's subpath takes area densities that
// the walk could not know.
RD void LightPathFinish(const DevScene& S, VPath path, int n, const LightFix& fix) {
  if (n == 0 || !VIsInfinite(S, path[0])) return;
  if (n > 1) {
    float pf = fix.pdfPos;
    if (VIsOnSurface(path[1])) pf *= AbsDot(fix.D, path[1].N);
    path[1].pdfFwd = pf;
  }
  path[0].pdfFwd = InfiniteLightDensity(S, fix.D);
}

// BDPT::MISWeight (bdpt.cpp:555-634). The reference assigns the strategy's
// values into the subpaths (the sampled end vertex, the connection vertices'
// delta flags and the four reverse densities) and restores them afterwards;
// here they are overrides read in place of the stored values.
RDN float MISWeight(const DevScene& S, VPath lightV, VPath camV, const BVert& sampled, int s, int t) {
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
  const BVert* qs = s > 0 ? (s == 1 ? &sampled : &lightV[s - 1]) : nullptr;
  const BVert* pt = t > 0 ? (t == 1 ? &sampled : &camV[t - 1]) : nullptr;
  const BVert* qsMinus = s > 1 ? &lightV[s - 2] : nullptr;
  const BVert* ptMinus = t > 1 ? &camV[t - 2] : nullptr;
  float ptRev = 0.f, ptMinusRev = 0.f, qsRev = 0.f, qsMinusRev = 0.f;
  if (pt) ptRev = s > 0 ? VPdf(S, *qs, qsMinus, *pt) : PdfLightOrigin(S, *pt, *ptMinus);
  if (ptMinus) ptMinusRev = s > 0 ? VPdf(S, *pt, qs, *ptMinus) : PdfLightV(S, *pt, *ptMinus);
  if (qs) qsRev = VPdf(S, *pt, ptMinus, *qs);
  if (qsMinus) qsMinusRev = VPdf(S, *qs, pt, *qsMinus);
  float ri = 1.f;
  for (int i = t - 1; i > 0; --i) {
    const BVert& v = camV[i];
    float rev = i == t - 1 ? ptRev : (i == t - 2 ? ptMinusRev : v.pdfRev);
    rev = rev != 0.f ? rev : 1.f;
    float fwd = v.pdfFwd != 0.f ? v.pdfFwd : 1.f;
    ri *= rev / fwd;
    bool dI = i == t - 1 ? false : v.delta != 0u;
    if (!dI && !camV[i - 1].delta) sumRi += ri;
  }
  ri = 1.f;
  for (int i = s - 1; i >= 0; --i) {
    const BVert& v = (s == 1 && i == 0) ? sampled : lightV[i];
    float rev = i == s - 1 ? qsRev : (i == s - 2 ? qsMinusRev : v.pdfRev);
    rev = rev != 0.f ? rev : 1.f;
    float fwd = v.pdfFwd != 0.f ? v.pdfFwd : 1.f;
    ri *= rev / fwd;
    bool dI = i == s - 1 ? false : v.delta != 0u;
    bool deltaLightvertex = i > 0 ? lightV[i - 1].delta != 0u : dI;
    if (!dI && !deltaLightvertex) sumRi += ri;
  }
  return 1.f / (1.f + sumRi);
}

// Random numbers the t = 1 connections (s = 2 .. sEnd - 1) draw before
// connection sEnd: Perspective::SampleDirection's 2D sample for each light
// vertex s - 1 that can connect (ConnectBdpt, bdpt.cpp:500-503).
RD uint64_t Round1Draws(const DevScene& S, VPath lightV, int sEnd) {
  uint64_t n = 0;
  for (int s = 2; s < sEnd; ++s)
    if (VConnectible(S, lightV[s - 1])) n += 2u;
  return n;
}

// One connection's result: contribution c (MIS-weighted); with `vis`, it
// counts only if the segment from (P, N) to `target` is unoccluded
// (Scene::IsOcclude, scene.cpp:53-63); `splat` connections (t = 1) land on
// film position `pixel` instead of the sample's own pixel.
struct ConnOut {
  V3 c, P, N, target;
  V2 pixel;
  bool vis, splat;
};

// BDPT::ConnectBdpt (bdpt.cpp:478-553) with the visibility test deferred:
// false when the connection contributes nothing whatever the visibility. The
// weight is computed for every candidate; the reference computes it only for
// unoccluded ones, to the same value.
RDN bool ConnectBdpt(const DevScene& S, Pcg32& rng, VPath lightV, VPath camV, int s, int t, ConnOut& o) {
  if (t > 1 && s != 0 && camV[t - 1].type == BV_LIGHT) return false;
  BVert sampled{};
  V3 l = v3s(0.f);
  o.vis = false;
  o.splat = false;
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
      V3 camP, camDir;
      float camDist, we;
      V2 pixel;
      if (CameraSampleDirection(S.cam, qs.P, camP, camDir, camDist, pixel, we)) {
        sampled = VFromPsr(BV_CAMERA, camP, LinearRows(S.cam.camToWorld, V3{0.f, 0.f, 1.f}));
        sampled.thr = v3s(we / 1.f);  // dsr.Pdf is 1
        sampled.delta = 1u;
        V3 fs = VFs(S, qs, sampled, true);
        V3 result = cmul(cmul(qs.thr, fs), sampled.thr);
        if (!IsBlack(result)) {
          l = l + result;
          o.vis = true;
          o.splat = true;
          o.pixel = pixel;
          o.P = qs.P;
          o.N = qs.N;
          o.target = camP;
        }
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
          if (!IsBlack(result)) {
            l = l + result;
            o.vis = true;
            o.P = pt.P;
            o.N = pt.N;
            o.target = dsr.P;
          }
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
      if (!IsBlack(result)) {
        l = l + result;
        o.vis = true;
        o.P = pt.P;
        o.N = pt.N;
        o.target = qs.P;
      }
    }
  }
  if (IsBlack(l)) return false;
  float mis = MISWeight(S, lightV, camV, sampled, s, t);
  o.c = l * mis;
  return true;
}

}  // namespace rad
