// Renderer "particle_tracer" (particle_tracer.cpp:97-232): a light path traced
// from an emitter; every vertex (and the emitter point itself) is connected to
// the camera and splatted into the film with weight x importance x (pixels /
// light paths). The functions here are the per-light-path steps; the kernels
// (k_light.cu) run them as a wavefront between launches of the BVH8
// closest-hit kernel, the camera connections' visibility rays going through
// the any-hit kernel.
#pragma once
#include "dbsdf.cuh"
#include "dscene.cuh"

namespace rad {

RD bool IsBlack(V3 v) { return v.x == 0.f && v.y == 0.f && v.z == 0.f; }

// The visibility ray of Scene::IsOcclude (scene.cpp:53-63) from (P, N) to
// target: false when the points are closer than the shadow epsilon (occluded).
RD bool ShadowRay(V3 P, V3 N, V3 target, V3& o, V3& d, float& tmax) {
  o = OffsetP(P, N, target - P);
  d = target - o;
  float dist = norm(d);
  if (dist < kShadowEps) return false;
  d = d / dist;
  tmax = dist * (1.f - kShadowEps);
  return true;
}

// A camera connection whose splat waits for its visibility ray (o, d, tmax):
// contribution c into film pixel `pixel`.
struct CamSplat {
  V3 o, d, c;
  float tmax;
  uint32_t pixel;
};

// ConnetCamera (particle_tracer.cpp:135-175) with the visibility test
// deferred. mi < 0: an emitter point with no BSDF (cosine-weighted on a
// surface; onShape false: the sky, one-sided). False when nothing would be
// splatted whatever the visibility.
RD bool CameraConnection(const DevScene& S, const SurfInt& si, bool onShape, int mi, const TexCtx* tc, V3 camP,
                         V2 pixel, V3 weight, float sampleScale, CamSplat& out) {
  if (IsBlack(weight)) return false;
  int x = (int)pixel.x, y = (int)pixel.y;
  if (x < 0 || y < 0 || x >= S.cam.width || y >= S.cam.height) return false;  // the frustum test keeps it inside
  V3 o, d;
  float tmax;
  if (!ShadowRay(si.P, si.N, camP, o, d, tmax)) return false;
  V3 toCamera = camP - o;  // SpawnRayTo (interaction.cpp:20-26) starts at the same offset point
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
  out.c = cmul(weight, fs) * sampleScale;
  if (IsBlack(out.c)) return false;
  out.o = o;
  out.d = d;
  out.tmax = tmax;
  out.pixel = (uint32_t)(y * S.cam.width + x);
  return true;
}

// Light path `id` of a job up to its first trace (particle_tracer.cpp:97-133):
// the emitter point seen by the camera (`em`, when hasEm) and the emitted ray
// (O, D) with its weight. False when there is no emitted ray.
RD bool ParticleStart(const DevScene& S, uint64_t id, uint32_t seed, float sampleScale, Pcg32& rng, CamSplat& em,
                      bool& hasEm, V3& O, V3& D, V3& thr) {
  rng = PcgForSample((uint32_t)id, (uint32_t)(id >> 32), seed);
  hasEm = false;
  if (S.nLights == 0) return false;
  // ---- SampleLight (particle_tracer.cpp:104-133)
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
      } else {  // area: Light::SamplePosition, radiance Eval(si) (area.cpp:42-45)
        float pdf;
        V2 uv;
        AreaSamplePosition(S, L, xi, si.P, si.N, uv, pdf);
        lightPdf *= pdf;
        le = AreaRadiance(S, L, uv);
      }
      si.sh = FrameFromN(si.N);  // SurfaceInteraction(psr) (interaction.cpp:30-41)
      V3 camP, camDir;
      float camDist, we;
      V2 pixel;
      Next2D(rng);  // Perspective::SampleDirection's sample (unused by a pinhole)
      if (CameraSampleDirection(S.cam, si.P, camP, camDir, camDist, pixel, we)) {
        V3 weight = le * we / lightPdf;
        si.Wi = ToLocal(si.sh, camDir);
        hasEm = CameraConnection(S, si, onShape, -1, nullptr, camP, pixel, weight, sampleScale, em);
      }
    }
  }
  // ---- Sample (particle_tracer.cpp:97-102): an emitted ray
  int lidx;
  float lightPdf;
  PickLight(S, Next1D(rng), lidx, lightPdf);
  V2 xi2 = Next2D(rng), xi3 = Next2D(rng);
  V3 li;
  if (!LightSampleRay(S, S.lights[lidx], xi2, xi3, O, D, li)) return false;
  thr = li / lightPdf;
  return true;
}

// TraceLightRay (particle_tracer.cpp:177-226) once the ray (O, D) of bounce d
// has been traced: the tests after the trace (Russian roulette from the second
// vertex on), the vertex's camera connection (`cs`, when hasCs) and the
// importance-transport BSDF sample. True with the next ray in (O, D).
RD bool ParticleBounce(const DevScene& S, Pcg32& rng, int d, bool hit, const TraceHit& h, V3& O, V3& D, V3& thr,
                       float& eta, float sampleScale, CamSplat& cs, bool& hasCs) {
  hasCs = false;
  if (!hit) return false;
  SurfInt si = ComputeSI(S, O, D, h);
  const int mi = S.shapes[si.shape].bsdf;
  if (mi < 0) return false;
  const int depth = d + 1;
  if (S.maxDepth >= 0 && depth >= S.maxDepth) return false;
  if (d >= 1 && depth >= S.rrDepth) {
    float rr = fminr(max_comp(thr) * Sqr(eta), 0.95f);
    if (Next1D(rng) > rr) return false;
    thr = thr * Rcp(rr);
  }
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
    hasCs = CameraConnection(S, si, true, mi, tc, camP, pixel, thr * we, sampleScale, cs);
  float bl = Next1D(rng);
  V2 bd = Next2D(rng);
  BsdfSampleRes bs = BsdfSample(S.mats, (uint32_t)mi, si.Wi, bl, bd, tc, true);
  // A failed sample (pdf 0, e.g. Disney's macro/micro-surface rejection) ends
  // the path; the reference divides by its zero pdf and writes NaN splats.
  if (!(bs.pdf > 0.f)) return false;
  V3 woW = ToWorld(si.sh, bs.wo);
  float idn = dot(si.N, -D), odn = dot(si.N, woW);
  if (idn * si.Wi.z <= 0.f || odn * bs.wo.z <= 0.f) return false;
  float correction = (si.Wi.z * odn) / (bs.wo.z * idn);
  thr = cmul(thr, bs.f) * fabsf(correction) / bs.pdf;
  eta *= bs.eta;
  if (IsBlack(thr)) return false;
  D = woW;
  O = OffsetP(si.P, si.N, D);
  return true;
}

}  // namespace rad
