// Renderer "particle_tracer" (particle_tracer.cpp:97-232): one light path,
// traced from an emitter, every vertex (and the emitter point itself)
// connected to the camera and splatted into the film with weight x importance
// x (pixels / light paths).
#pragma once
#include "dbsdf.cuh"
#include "dscene.cuh"

namespace rad {

// Unbounded light paths (max_depth -1) are capped like camera paths.
constexpr int kMaxLightBounces = 256;

struct ParticleFilm {
  float4* accum;
  int32_t width, height;
};

// Scene::IsOcclude (scene.cpp:53-63)
RD bool LOccluded(const DevScene& S, V3 P, V3 N, V3 target, uint32_t* err) {
  V3 o = OffsetP(P, N, target - P);
  V3 d = target - o;
  float dist = norm(d);
  if (dist < kShadowEps) return true;
  d = d / dist;
  RayPre r = MakeRayPre(o, d, 0.f);
  TraceHit h;
  return TraceBvh8<true>(S, r, dist * (1.f - kShadowEps), h, err);
}

RD bool LTrace(const DevScene& S, V3 O, V3 D, SurfInt& si, TraceHit& h, uint32_t* err) {
  RayPre r = MakeRayPre(O, D, 0.f);
  if (!TraceBvh8<false>(S, r, kFloatMax, h, err)) return false;
  si = ComputeSI(S, O, D, h);
  return true;
}

RD void Splat(const ParticleFilm& film, V2 pixel, V3 v) {
  int x = (int)pixel.x, y = (int)pixel.y;
  if (x < 0 || y < 0 || x >= film.width || y >= film.height) return;  // the frustum test keeps pixel inside
  float4* a = film.accum + (size_t)y * film.width + x;
  atomicAdd(&a->x, v.x);
  atomicAdd(&a->y, v.y);
  atomicAdd(&a->z, v.z);
}

// ConnetCamera (particle_tracer.cpp:135-175). mi < 0: an emitter point with no
// BSDF (cosine-weighted on a surface; onShape false: the sky, one-sided).
RD void ConnectCamera(const DevScene& S, const ParticleFilm& film, const SurfInt& si, bool onShape, int mi,
                      const TexCtx* tc, V3 camP, V2 pixel, V3 weight, float sampleScale, uint32_t* err) {
  if (weight.x == 0.f && weight.y == 0.f && weight.z == 0.f) return;
  if (LOccluded(S, si.P, si.N, camP, err)) return;
  V3 o = OffsetP(si.P, si.N, camP - si.P);  // SpawnRayTo (interaction.cpp:20-26)
  V3 toCamera = camP - o;
  toCamera = toCamera / norm(toCamera);
  V3 wo = ToLocal(si.sh, toCamera);
  V3 fs = v3s(1.f);
  if (!onShape) {
    if (wo.z <= 0.f) fs = v3s(0.f);
  } else if (mi < 0) {
    fs = fs * fmaxr(0.f, wo.z);
  } else {
    float idn = dot(si.N, ToWorld(si.sh, si.Wi));
    float odn = dot(si.N, toCamera);
    if (idn * si.Wi.z <= 0.f || odn * wo.z <= 0.f) {
      fs = v3s(0.f);
    } else {
      float correction = (si.Wi.z * odn) / (wo.z * idn);
      V3 f;
      float pdf;
      BsdfEvalPdf(S.mats, (uint32_t)mi, si.Wi, wo, f, pdf, tc, true);
      fs = cmul(fs, f) * fabsf(correction);  // / cameraSample.Pdf, which is 1 for the pinhole
    }
  }
  Splat(film, pixel, cmul(weight, fs) * sampleScale);
}

// One light path `id` of a job (seed, pixels / light paths).
RD void ParticlePath(const DevScene& S, const ParticleFilm& film, uint64_t id, uint32_t seed, float sampleScale,
                     uint32_t* err) {
  Pcg32 rng = PcgForSample((uint32_t)id, (uint32_t)(id >> 32), seed);
  if (S.nLights == 0) return;
  // ---- SampleLight (particle_tracer.cpp:104-133): the emitter itself seen by the camera
  if (S.maxDepth != 0) {
    int li0;
    float lightPdf;
    PickLight(S, Next1D(rng), li0, lightPdf);
    const LightRec& L = S.lights[li0];
    bool delta = L.kind == LIGHT_POINT || L.kind == LIGHT_PROJECTION || L.kind == LIGHT_DIRECTIONAL;
    if (!delta) {
      SurfInt si;
      V3 le;
      bool onShape = L.kind == LIGHT_AREA;
      V2 xi = Next2D(rng);
      if (!onShape) {  // sky: a direction seen from the camera's position
        V3 camPos = Affine4(S.cam.camToWorld, v3s(0.f));
        DirSample dsr = LightSampleDirection(S, L, camPos, xi, le);
        lightPdf *= dsr.Pdf > 0.f ? (dsr.Pdf * Sqr(dsr.Dist)) : 0.f;
        si.P = dsr.P;
        si.N = dsr.N;
      } else {  // area: a point on the emitter, radiance Eval(si) (area.cpp:42-45)
        float pdf;
        ShapeSamplePosition(S, S.shapes[L.shape], xi, si.P, si.N, pdf);
        lightPdf *= pdf;
        le = V3{L.radiance[0], L.radiance[1], L.radiance[2]};
      }
      si.sh = FrameFromN(si.N);  // SurfaceInteraction(psr) (interaction.cpp:30-41)
      V3 camP, camDir;
      float camDist, we;
      V2 pixel;
      Next2D(rng);  // Perspective::SampleDirection's sample (unused by a pinhole)
      if (CameraSampleDirection(S.cam, si.P, camP, camDir, camDist, pixel, we)) {
        V3 weight = le * we / lightPdf;
        si.Wi = ToLocal(si.sh, camDir);
        ConnectCamera(S, film, si, onShape, -1, nullptr, camP, pixel, weight, sampleScale, err);
      }
    }
  }
  // ---- Sample (particle_tracer.cpp:97-102): an emitted ray
  int lidx;
  float lightPdf;
  PickLight(S, Next1D(rng), lidx, lightPdf);
  V2 xi2 = Next2D(rng), xi3 = Next2D(rng);
  V3 O, D, li;
  if (!LightSampleRay(S, S.lights[lidx], xi2, xi3, O, D, li)) return;
  V3 thr = li / lightPdf;
  // ---- TraceLightRay (particle_tracer.cpp:177-226)
  float eta = 1.f;
  int depth = 1;
  SurfInt si;
  TraceHit h;
  bool hit = LTrace(S, O, D, si, h, err);
  if (!hit || S.shapes[si.shape].bsdf < 0) return;
  if (S.maxDepth >= 0 && depth >= S.maxDepth) return;
  for (int guard = 0; guard < kMaxLightBounces; guard++) {
    const int mi = S.shapes[si.shape].bsdf;
    TexCtx tcx;
    const TexCtx* tc = nullptr;
    if (S.nTex) {
      tcx = TexCtx{S.tex, S.texels, S.texBind, ComputeUV(S, h, si).uv, V2{0.f, 0.f}, V2{0.f, 0.f}};
      tc = &tcx;
    }
    V3 camP, camDir;
    float camDist, we;
    V2 pixel;
    Next2D(rng);
    if (CameraSampleDirection(S.cam, si.P, camP, camDir, camDist, pixel, we))
      ConnectCamera(S, film, si, true, mi, tc, camP, pixel, thr * we, sampleScale, err);
    float bl = Next1D(rng);
    V2 bd = Next2D(rng);
    BsdfSampleRes bs = BsdfSample(S.mats, (uint32_t)mi, si.Wi, bl, bd, tc, true);
    // A failed sample (pdf 0, e.g. Disney's macro/micro-surface rejection) ends
    // the path; the reference divides by its zero pdf and writes NaN splats.
    if (!(bs.pdf > 0.f)) break;
    V3 woW = ToWorld(si.sh, bs.wo);
    float idn = dot(si.N, -D), odn = dot(si.N, woW);
    if (idn * si.Wi.z <= 0.f || odn * bs.wo.z <= 0.f) break;
    float correction = (si.Wi.z * odn) / (bs.wo.z * idn);
    thr = cmul(thr, bs.f) * fabsf(correction) / bs.pdf;
    eta *= bs.eta;
    if (thr.x == 0.f && thr.y == 0.f && thr.z == 0.f) break;
    D = woW;
    O = OffsetP(si.P, si.N, D);
    hit = LTrace(S, O, D, si, h, err);
    depth++;
    if (!hit || S.shapes[si.shape].bsdf < 0) break;
    if (S.maxDepth >= 0 && depth >= S.maxDepth) break;
    if (depth >= S.rrDepth) {
      float rr = fminr(max_comp(thr) * Sqr(eta), 0.95f);
      if (Next1D(rng) > rr) break;
      thr = thr * Rcp(rr);
    }
  }
}

}  // namespace rad
