// `vol_path` integrator (VolPath::Li, rad.offline/src/renderer/vol_path.cpp:27-349):
// free flights against the medium majorant (medium.cpp:19-43), null / real
// collisions with hero-channel spectral MIS, phase-function NEE with the
// ratio-tracking transmittance loop (vol_path.cpp:224-342) and index-matched
// boundaries. The loop is cut into parts that a path runs in order (VolAct);
// two schedules run them: a per-event wavefront (one kernel per part over a
// queue of the paths at that part, state in HBM between parts) and a
// persistent kernel (lanes vote on the part to run each warp step). Camera
// rays and PCG streams come from the generate stage; the radiance goes to the
// path's L slot for the accumulate stage.
#include <algorithm>

#include "dbsdf.cuh"
#include "dscene.cuh"
#include "dvol.cuh"
#include "kernels.h"

namespace rad {

constexpr int kVolBlock = 128;
constexpr int kMaxTrLoop = 1 << 20;  // bound on transmittance-loop iterations (device check)
constexpr int kMaxVolIter = 1 << 22; // bound on free-flight iterations per path

RD V3 ExpV(V3 v) { return V3{expf(v.x), expf(v.y), expf(v.z)}; }

// Majorant transmittance relative to the hero channel, exp(-(cE - cE[ch]) t),
// without forming exp(-cE t) itself: the reference's tr / pdf ratios
// (medium.cpp:45-59, vol_path.cpp:262-272) underflow to 0 / 0 once cE t passes
// ~100 (a long shadow segment), which drops the contribution. Used by the
// non-reference estimators (realDepth / BRICKS); 1 for a scalar majorant.
RD V3 RelTr(V3 cE, int ch, float t) {
  float c = comp(cE, ch);
  auto f = [&](float v) {
    float d = v - c;
    return (d == 0.f || !isfinite(t)) ? 1.f : expf(-d * t);
  };
  return V3{f(cE.x), f(cE.y), f(cE.z)};
}

RD float PhaseEval(const MediumRec& md, const MedInt& mi, V3 wo) {
  if (!md.hg) return SquareToUniformSpherePdf();
  float g = md.g;
  float c = dot(wo, mi.Wi);
  float temp = 1.f + g * g + 2.f * g * c;
  return (1.f / (4.f * kPi)) * (1.f - g * g) / (temp * sqrtf(temp));
}
RD V3 PhaseSample(const MediumRec& md, const MedInt& mi, V2 xi, float& pdf) {
  if (!md.hg) {
    pdf = SquareToUniformSpherePdf();
    return SquareToUniformSphere(xi);
  }
  float g = md.g;
  float sqrTerm = (1.f - g * g) / (1.f - g + 2.f * g * xi.x);
  float cosTheta = (1.f + g * g - sqrTerm * sqrTerm) / (2.f * g);
  if (fabsf(g) < kEps32) cosTheta = 1.f - 2.f * xi.x;
  float sinTheta = SafeSqrt(1.f - cosTheta * cosTheta);
  float a = 2.f * kPi * xi.y;
  V3 wo{sinTheta * cosf(a), sinTheta * sinf(a), -cosTheta};
  wo = ToWorld(mi.sh, wo);
  float c = -cosTheta;
  float temp = 1.f + g * g + 2.f * g * c;
  pdf = (1.f / (4.f * kPi)) * (1.f - g * g) / (temp * sqrtf(temp));
  return wo;
}

RD float VMis(float a, float b) {
  a *= a;
  b *= b;
  float w = a / (a + b);
  return isfinite(w) ? w : 0.f;
}

RD bool VTrace(const DevScene& S, const VRay& ray, SurfInt& si, uint32_t* err, V2* uv) {
  RayPre r = MakeRayPre(ray.O, ray.D, ray.MinT);
  TraceHit h;
  if (!TraceBvh8<false>(S, r, ray.MaxT, h, err)) {
    si.T = kInf;
    si.P = v3s(0.f);
    si.N = v3s(0.f);
    si.shape = -1;
    si.sh.S = si.sh.T = si.sh.N = v3s(0.f);
    si.Wi = -ray.D;
    return false;
  }
  si = ComputeSI(S, ray.O, ray.D, h);
  if (uv) *uv = ComputeUV(S, h, si).uv;
  return true;
}

RD VRay Spawn(V3 P, V3 N, V3 d) { return VRay{OffsetP(P, N, d), d, 0.f, kFloatMax}; }

// Out-of-line copies of the large pieces: one body each in the kernel instead
// of one per call site keeps the loop within the instruction cache.
#ifdef RAD_HOST_EMULATION
#define RDN inline
#else
#define RDN __device__ __noinline__
#endif
// uv: where to put the hit's texture coordinates, or null.
RDN bool VTraceCall(const DevScene& S, const VRay& ray, SurfInt& si, uint32_t* err, V2* uv) {
  return VTrace(S, ray, si, err, uv);
}
RDN void VBsdfEvalPdf(const MatRec* mats, uint32_t b, V3 wi, V3 wo, V3& f, float& pdf, const TexCtx* tc) {
  BsdfEvalPdf(mats, b, wi, wo, f, pdf, tc);
}
RDN BsdfSampleRes VBsdfSample(const MatRec* mats, uint32_t b, V3 wi, float xl, V2 xd, const TexCtx* tc) {
  return BsdfSample(mats, b, wi, xl, xd, tc);
}

RD int MediumOfHit(const DevScene& S, const SurfInt& si, V3 D) {
  const ShapeRec& sh = S.shapes[si.shape];
  return dot(D, si.N) > 0.f ? sh.outMedium : sh.inMedium;
}

// Next-event estimation of vol_path (vol_path.cpp:224-342) as resumable steps:
// NeeBegin draws the light sample, each NeeStep is one iteration of the
// transmittance loop (a ratio-tracking step in a medium, or a surface segment),
// so that a warp can run the loop's iterations of many lanes together.
// stable: RelTr ratios instead of the reference's (see RelTr).
struct NeeState {
  DirSample dsr;
  V3 li, tr;        // the light's radiance, the transmittance so far
  VRay ray;
  float total;      // distance covered
  int medium, guard;
  bool active, needsIsect;
  float siT;        // the last surface hit of the shadow ray (SurfInt fields the loop reads)
  V3 siP, siN;
  int siShape;
};

RD void NeeBegin(const DevScene& S, Pcg32& rng, int medium, V3 refP, V3 refN, NeeState& n) {
  float xl = Next1D(rng);
  V2 xd = Next2D(rng);
  n.dsr = SampleLightDirection(S, refP, xl, xd, n.li);
  n.active = n.dsr.Pdf > 0.f;
  if (!n.active) return;
  n.ray = Spawn(refP, refN, n.dsr.Dir);
  n.total = 0.f;
  n.tr = v3s(1.f);
  n.needsIsect = true;
  n.siT = kInf;
  n.siShape = -1;
  n.medium = medium;
  n.guard = 0;
}

// One iteration of the transmittance loop; false once it has ended.
template <bool BRICKS, bool HALF>
RDN bool NeeStep(const DevScene& S, Pcg32& rng, int channel, NeeState& n, uint32_t* err, uint32_t& nRays,
                 bool stable) {
  if (n.guard++ >= kMaxTrLoop) {
    atomicOr(err, 2u);
    n.tr = v3s(0.f);
    return n.active = false;
  }
  VRay& ray = n.ray;
  SurfInt si;
  si.T = n.siT;
  si.P = n.siP;
  si.N = n.siN;
  si.shape = n.siShape;
  float remainingDist = n.dsr.Dist * (1.f - kShadowEps) - n.total;
  ray.MaxT = remainingDist;
  bool active = remainingDist > 0.f;
  if (!active) return n.active = false;
  bool escapedMedium = false;
  bool activeMedium = active && n.medium >= 0;
  bool activeSurface = active && !activeMedium;
  if (activeMedium) {
    const MediumRec& md = S.media[n.medium];
    MedInt mei = SampleInteraction<BRICKS, HALF>(S, md, ray, Next1D(rng), channel);
    if (md.kind == MED_HOMOGENEOUS && mei.T != kInf) ray.MaxT = fminr(mei.T, remainingDist);
    if (n.needsIsect) {
      VTraceCall(S, ray, si, err, nullptr);
      nRays++;
    }
    if (si.T < mei.T) mei.T = kInf;
    bool isSpectral = true;
    {
      float t = fminr(remainingDist, fminr(mei.T, si.T)) - mei.MinT;
      if (t >= 0.f) {
        bool pass = si.T < mei.T || mei.T > remainingDist;
        V3 mTr;
        if (stable) {
          float m = comp(mei.cE, channel);
          V3 rel = RelTr(mei.cE, channel, t);
          mTr = pass ? rel : (m > 0.f ? rel / m : v3s(0.f));
        } else {
          V3 tr = ExpV(mei.cE * -t);
          V3 ffp = pass ? tr : cmul(tr, mei.cE);
          float trPdf = comp(ffp, channel);
          mTr = trPdf > 0.f ? tr / trPdf : v3s(0.f);
        }
        n.tr = cmul(n.tr, mTr);
      }
    }
    if ((mei.T > remainingDist) && mei.T != kInf) n.total = n.dsr.Dist;
    if (mei.T > remainingDist) mei.T = kInf;
    escapedMedium = mei.T == kInf;
    activeMedium = mei.T != kInf;
    isSpectral = isSpectral && activeMedium;
    if (activeMedium) {
      n.total += mei.T;
      ray.O = mei.P;
      si.T = si.T - mei.T;
      if (isSpectral) n.tr = cmul(n.tr, mei.sN);
    }
  }
  bool intersect = activeSurface && n.needsIsect;
  if (intersect) {
    VTraceCall(S, ray, si, err, nullptr);
    nRays++;
  }
  n.needsIsect = n.needsIsect && !intersect;
  activeSurface = activeSurface || escapedMedium;
  if (activeSurface) n.total += si.T;
  activeSurface = activeSurface && si.T != kInf && active && !activeMedium;
  if (activeSurface) {
    if (S.shapes[si.shape].bsdf >= 0) n.tr = v3s(0.f);
    ray = Spawn(si.P, si.N, ray.D);
  }
  ray.MaxT = remainingDist;
  n.needsIsect = n.needsIsect || activeSurface;
  active = active && (activeMedium || activeSurface) && !is_zero(n.tr);
  if (activeSurface) {
    const ShapeRec& sh = S.shapes[si.shape];
    if (sh.inMedium >= 0 || sh.outMedium >= 0) n.medium = MediumOfHit(S, si, ray.D);
  }
  n.siT = si.T;
  n.siP = si.P;
  n.siN = si.N;
  n.siShape = si.shape;
  return n.active = active;
}

// Per-path state of the `vol_path` loop (VolPath::Li's locals), so that a lane
// can run a path one loop iteration at a time and take a new path when its own
// ends (KVolPath).
struct alignas(16) VolPathState {
  VRay ray;
  V3 thr, result, prevP;
  float eta, prevPdf;
  int medium, channel, depth, guard;
  bool isSpecular, siValid, afterNull;
  int act;      // next part of the loop iteration (kAct*)
  V3 scatterP;  // kActScatter / kActScatterEnd: the real collision
  SurfInt si;
  Pcg32 rng;
  uint32_t nRays, nShadow;
  NeeState nee;  // kActNee: the next-event estimation in progress
  int neeRet;    // the part that follows it
  V2 uvHit;      // kActSurfaceEnd: the hit's texture coordinates
};
// Parts of one iteration of the VolPath::Li loop (vol_path.cpp:40-215): the top
// (Russian roulette, depth test, free flight, null / real decision); the medium
// scatter (the light sample of the phase NEE), its transmittance steps and its
// end (NEE contribution, phase sampling); the surface part (trace, emission,
// the light sample of the BSDF NEE), its transmittance steps and its end (NEE
// contribution, BSDF sampling). A path runs them in this order, so its
// arithmetic and random numbers are those of the loop; KVolPath runs one kind
// per warp step.
constexpr int kActTop = 0, kActScatter = 1, kActSurface = 2, kActNee = 3, kActScatterEnd = 4, kActSurfaceEnd = 5;
constexpr int kActs = 6;
static_assert(kActs == kVolActs, "one wavefront queue per loop part");

RD void VolInit(const DevScene& S, VolPathState& p, VRay ray, Pcg32 rng) {
  p.ray = ray;
  p.rng = rng;
  p.medium = S.globalMedium;
  p.thr = v3s(1.f);
  p.result = v3s(0.f);
  p.eta = 1.f;
  p.isSpecular = true;
  p.prevP = v3s(0.f);
  p.prevPdf = 1.f;
  uint32_t ch3 = (uint32_t)(Next1D(p.rng) * 3.f);
  p.channel = (int)(ch3 < 2u ? ch3 : 2u);
  p.si.T = kInf;
  p.si.shape = -1;
  p.siValid = false;
  p.afterNull = false;
  p.depth = 0;
  p.guard = 0;
  p.act = kActTop;
  p.nRays = p.nShadow = 0;
}

// End of a loop iteration (the loop's increment).
RD bool VolNextIteration(VolPathState& p) {
  p.depth++;
  p.guard++;
  p.act = kActTop;
  return true;
}

// Top of an iteration. BRICKS: brick majorants, and no re-trace after a null
// collision (the surface ahead along the same line is unchanged; its distance
// shrinks by the flight). HALF: fp16 grid. realDepth (mode bit kVolRealDepth,
// implied by BRICKS): null collisions count neither toward max_depth nor for
// Russian roulette; the reference counts them (vol_path.cpp:40-52 run once per
// loop iteration), which ties its truncation to the majorant. All off = the
// reference's algorithm. Returns false when the path has ended.
template <bool BRICKS, bool HALF>
RD bool VolTop(const DevScene& S, VolPathState& p, uint32_t mode, uint32_t* err) {
  const bool realDepth = BRICKS || (mode & kVolRealDepth);
  Pcg32& rng = p.rng;
  VRay& ray = p.ray;
  SurfInt& si = p.si;
  V3& thr = p.thr;
  const int channel = p.channel;
  if (p.guard >= kMaxVolIter) {
    atomicOr(err, 4u);
    return false;
  }
  if (p.afterNull) p.depth--;  // realDepth: the null collision was free
  if (p.depth >= S.rrDepth && !p.afterNull) {
    float rr = fminr(max_comp(thr) * Sqr(p.eta), 0.95f);
    if (Next1D(rng) > rr) return false;
    thr = thr * Rcp(rr);
  }
  if (S.maxDepth >= 0 && p.depth + 1 >= S.maxDepth) return false;
  p.afterNull = false;
  if (p.medium < 0) {
    p.act = kActSurface;
    return true;
  }
  const MediumRec& md = S.media[p.medium];
  MedInt mei = SampleInteraction<BRICKS, HALF>(S, md, ray, Next1D(rng), channel);
  if (md.kind == MED_HOMOGENEOUS && mei.T != kInf) ray.MaxT = mei.T;
  if (!(BRICKS && p.siValid)) {
    VTraceCall(S, ray, si, err, nullptr);
    p.nRays++;
  }
  p.siValid = false;
  if (si.T < mei.T) mei.T = kInf;
  {
    // medium.cpp:45-59
    V3 tr, ffp;
    float t = fminr(mei.T, si.T) - mei.MinT;
    if (realDepth) {
      // tr / pdf formed as RelTr ratios (no underflow)
      if (t <= 0.f) {
        tr = ffp = v3s(1.f);
      } else {
        tr = RelTr(mei.cE, channel, t);
        ffp = si.T < mei.T ? v3s(1.f) : v3s(comp(mei.cE, channel));
      }
    } else if (t <= 0.f) {
      tr = ffp = v3s(1.f);
    } else {
      tr = ExpV(mei.cE * -t);
      ffp = si.T < mei.T ? tr : cmul(tr, mei.cE);
      if (tr.x == ffp.x && tr.y == ffp.y && tr.z == ffp.z) tr = ffp = v3s(1.f);
    }
    float pdf = comp(ffp, channel);
    V3 after = cmul(thr, tr) / pdf;
    thr = pdf <= 0.f ? v3s(0.f) : after;
  }
  const bool escaped = mei.T == kInf;
  bool nullScatter = Next1D(rng) > comp(mei.sT, channel) / comp(mei.cE, channel);
  if (escaped) {
    p.act = kActSurface;
    return true;
  }
  if (nullScatter) {
    thr = cmul(thr, mei.sN) * comp(mei.cE, channel) / comp(mei.sN, channel);
    ray.O = mei.P;
    si.T = si.T - mei.T;
    p.siValid = BRICKS;
    p.afterNull = realDepth;
    return VolNextIteration(p);
  }
  // real collision: the scatter part follows
  p.prevP = mei.P;
  thr = cmul(thr, mei.sS) * comp(mei.cE, channel) / comp(mei.sT, channel);
  p.scatterP = mei.P;
  p.act = kActScatter;
  return true;
}

// Medium scatter: the light sample of the phase-function NEE.
RD bool VolScatter(const DevScene& S, VolPathState& p) {
  NeeBegin(S, p.rng, p.medium, p.scatterP, v3s(0.f), p.nee);
  p.neeRet = kActScatterEnd;
  p.act = p.nee.active ? kActNee : kActScatterEnd;
  return true;
}

// After the NEE: its contribution and the next direction.
RD bool VolScatterEnd(const DevScene& S, VolPathState& p) {
  const MediumRec& md = S.media[p.medium];
  MedInt mei;  // the phase functions read the incident direction and its frame
  mei.Wi = -p.ray.D;
  mei.sh = FrameFromN(mei.Wi);
  mei.P = p.scatterP;
  const DirSample& dsr = p.nee.dsr;
  if (dsr.Pdf > 0.f) {
    V3 li = cmul(p.nee.li, p.nee.tr);
    float phaseVal = PhaseEval(md, mei, dsr.Dir);
    float weight = dsr.IsDelta ? 1.f : VMis(dsr.Pdf, phaseVal);
    p.result = p.result + cmul(p.thr, li) * weight * phaseVal / dsr.Pdf;
  }
  float phasePdf;
  V3 wo = PhaseSample(md, mei, Next2D(p.rng), phasePdf);
  p.ray = Spawn(mei.P, v3s(0.f), wo);
  p.isSpecular = false;
  p.prevPdf = phasePdf;
  return VolNextIteration(p);
}

// One step of the NEE's transmittance loop.
template <bool BRICKS, bool HALF>
RD bool VolNee(const DevScene& S, VolPathState& p, uint32_t mode, uint32_t* err) {
  const bool realDepth = BRICKS || (mode & kVolRealDepth);
  if (!NeeStep<BRICKS, HALF>(S, p.rng, p.channel, p.nee, err, p.nShadow, realDepth)) p.act = p.neeRet;
  return true;
}

// Surface part: trace, emission with MIS, the light sample of the BSDF NEE.
template <bool BRICKS, bool HALF>
RD bool VolSurface(const DevScene& S, VolPathState& p, uint32_t mode, uint32_t* err) {
  VRay& ray = p.ray;
  SurfInt& si = p.si;
  V3& thr = p.thr;
  // texture coordinates of the hit, for scenes with textures (vol_path traces
  // plain rays: no differentials, uv derivatives 0)
  const bool textured = S.nTex != 0u;
  V2 uvHit{0.f, 0.f};
  bool hit = VTraceCall(S, ray, si, err, textured ? &uvHit : nullptr);
  p.nRays++;
  int hitLight = hit ? S.shapes[si.shape].light : S.envLight;
  if (hitLight >= 0) {
    float weight;
    if (p.isSpecular) {
      weight = 1.f;
    } else {
      V3 rel = si.P - p.prevP;
      float dist = norm(rel);
      V3 dir = hit ? rel / dist : -si.Wi;
      weight = VMis(p.prevPdf, PdfLightDirection(S, hitLight, p.prevP, dir, si.sh.N, dist, uvHit));
    }
    V3 li = EvalLightAt(S, hitLight, &si, uvHit);
    p.result = p.result + cmul(thr, li) * weight;
  }
  if (!hit) return false;
  const ShapeRec& shp = S.shapes[si.shape];
  if (shp.light >= 0) return false;
  if (shp.bsdf < 0) {
    ray = Spawn(si.P, si.N, ray.D);
    p.medium = MediumOfHit(S, si, ray.D);
    // depth-- then the loop increment: the index-matched boundary is free
    p.guard++;
    p.act = kActTop;
    return true;
  }
  p.uvHit = uvHit;
  p.neeRet = kActSurfaceEnd;
  if (S.mats[shp.bsdf].flags & BT_NODELTA) {
    NeeBegin(S, p.rng, p.medium, si.P, si.N, p.nee);
    p.act = p.nee.active ? kActNee : kActSurfaceEnd;
  } else {
    p.nee.dsr.Pdf = 0.f;  // no NEE at a delta-only BSDF
    p.act = kActSurfaceEnd;
  }
  return true;
}

// After the NEE: its contribution, BSDF sampling.
RD bool VolSurfaceEnd(const DevScene& S, VolPathState& p) {
  VRay& ray = p.ray;
  SurfInt& si = p.si;
  V3& thr = p.thr;
  const ShapeRec& shp = S.shapes[si.shape];
  const MatRec* mats = S.mats;
  TexCtx tcx;
  const TexCtx* tc = nullptr;
  if (S.nTex != 0u) {
    tcx = TexCtx{S.tex, S.texels, S.texBind, p.uvHit, V2{0.f, 0.f}, V2{0.f, 0.f}};
    tc = &tcx;
  }
  const DirSample& dsr = p.nee.dsr;
  if (dsr.Pdf > 0.f) {
    V3 li = cmul(p.nee.li, p.nee.tr);
    V3 wo = ToLocal(si.sh, dsr.Dir);
    V3 f;
    float bsdfPdf;
    VBsdfEvalPdf(mats, (uint32_t)shp.bsdf, si.Wi, wo, f, bsdfPdf, tc);
    float weight = dsr.IsDelta ? 1.f : VMis(dsr.Pdf, bsdfPdf);
    p.result = p.result + cmul(cmul(thr, f), li) * weight / dsr.Pdf;
  }
  float xl = Next1D(p.rng);
  V2 xd = Next2D(p.rng);
  BsdfSampleRes bs = VBsdfSample(mats, (uint32_t)shp.bsdf, si.Wi, xl, xd, tc);
  if (bs.pdf <= 0.f) return false;
  thr = cmul(thr, bs.f) / bs.pdf;
  p.eta *= bs.eta;
  V3 nd = ToWorld(si.sh, bs.wo);
  ray = Spawn(si.P, si.N, nd);
  p.prevPdf = bs.pdf;
  p.prevP = si.P;
  p.isSpecular = (bs.type & BT_DELTA) != 0u;
  p.medium = MediumOfHit(S, si, ray.D);
  return VolNextIteration(p);
}

// The next part of the path's current iteration; false when the path has ended
// (its radiance is in p.result).
template <bool BRICKS, bool HALF>
RD bool VolAct(const DevScene& S, VolPathState& p, int act, uint32_t mode, uint32_t* err) {
  switch (act) {
    case kActScatter: return VolScatter(S, p);
    case kActSurface: return VolSurface<BRICKS, HALF>(S, p, mode, err);
    case kActNee: return VolNee<BRICKS, HALF>(S, p, mode, err);
    case kActScatterEnd: return VolScatterEnd(S, p);
    case kActSurfaceEnd: return VolSurfaceEnd(S, p);
    default: return VolTop<BRICKS, HALF>(S, p, mode, err);
  }
}
template <bool BRICKS, bool HALF>
RD bool VolStep(const DevScene& S, VolPathState& p, uint32_t mode, uint32_t* err) {
  return VolAct<BRICKS, HALF>(S, p, p.act, mode, err);
}

// The whole loop for one path (host-side checks and equivalence tests).
template <bool BRICKS, bool HALF>
RD V3 VolLi(const DevScene& S, Pcg32& rng, VRay ray, uint32_t mode, uint32_t* err, uint64_t& nRays,
            uint64_t& nShadow) {
  VolPathState p;
  VolInit(S, p, ray, rng);
  while (VolStep<BRICKS, HALF>(S, p, mode, err)) {
  }
  rng = p.rng;
  nRays += p.nRays;
  nShadow += p.nShadow;
  return p.result;
}

// Persistent lanes: each thread runs its path one part of a loop iteration at a
// time and takes the next unstarted path (counter B.counters[kMiscBase + 4],
// reset by the generate stage) when its own ends. Each warp step runs the part
// (top / medium scatter / surface) that most of the warp's live lanes are at, so
// a warp executes one code path at a time while paths stay in different phases.
template <bool BRICKS, bool HALF>
__global__ void __launch_bounds__(kVolBlock, 5)
    KVolPath(DevScene S, PathBuffers B, uint32_t count, uint32_t* err, uint32_t mode) {
  uint32_t* next = B.counters + kMiscBase + 4;
  const uint32_t lane = threadIdx.x & 31u;
  VolPathState p;
  uint32_t idx = 0;
  bool live = false, drained = false;
  unsigned long long nRays = 0, nShadow = 0;
  for (;;) {
    uint32_t need = __ballot_sync(0xffffffffu, !live);
    if (need && !drained) {
      int leader = __ffs(need) - 1;
      uint32_t base = 0;
      if ((int)lane == leader) base = atomicAdd(next, (uint32_t)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (base + (uint32_t)__popc(need) >= count) drained = true;
      if (!live) {
        uint32_t i = base + __popc(need & ((1u << lane) - 1u));
        if (i < count) {
          idx = i;
          float4 ro = B.rayO[idx], rd = B.rayD[idx];
          uint2 rs = B.rng[idx];
          Pcg32 rng;
          rng.state = ((uint64_t)rs.y << 32) | rs.x;
          VolInit(S, p, VRay{V3{ro.x, ro.y, ro.z}, V3{rd.x, rd.y, rd.z}, ro.w, rd.w}, rng);
          live = true;
        }
      }
    }
    int act = -1, best = 0;
    for (int a = 0; a < kActs; a++) {
      const int c = __popc(__ballot_sync(0xffffffffu, live && p.act == a));
      if (c > best) {
        best = c;
        act = a;
      }
    }
    if (act < 0) break;
    if (live && p.act == act) {
      bool alive = VolAct<BRICKS, HALF>(S, p, act, mode, err);
      if (!alive) {
        B.L[idx] = make_float4(p.result.x, p.result.y, p.result.z, 0.f);
        nRays += p.nRays;
        nShadow += p.nShadow;
        live = false;
      }
    }
  }
  // ray counters: closest in [kMiscBase + 2], shadow-side traces in [kMiscBase + 3]
  if (nRays) atomicAdd(B.counters + kMiscBase + 2, (uint32_t)nRays);
  if (nShadow) atomicAdd(B.counters + kMiscBase + 3, (uint32_t)nShadow);
}

// ---- per-event wavefront ------------------------------------------------------
// Part order within a round: top, scatter, surface, NEE, scatter end, surface
// end. A part hands its paths to a later part of the same round (queues of
// parity `cur`), except the loop's increment (scatter end, surface end, an
// index-matched boundary), which queues the path for the next round's top, and
// a repeating part (top through null collisions, the NEE's transmittance steps)
// that has run `chunk` steps of a path in this launch, which queues it to
// continue in the next round (parity cur ^ 1). The chunk bounds how long the
// last lanes of a launch run on after its queue has drained.
size_t VolStateBytes() { return sizeof(VolPathState); }

// Queue of a path moving from part `from` to part `act`.
RD uint32_t VolQueueOf(int from, int act, uint32_t cur) {
  return (act <= from ? (cur ^ 1u) : cur) * kVolActs + (uint32_t)act;
}

// Appends idx to queue `dst` for every lane with dst >= 0; all lanes of the warp
// call it. One atomic per destination and warp.
RD void VolPush(const VolWave& V, int dst, uint32_t idx) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t same = __match_any_sync(0xffffffffu, (uint32_t)dst);
  const int leader = __ffs(same) - 1;
  uint32_t base = 0;
  if ((int)lane == leader && dst >= 0) base = atomicAdd(V.cnt + dst, (uint32_t)__popc(same));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (dst >= 0) V.q[(size_t)dst * V.capacity + base + __popc(same & ((1u << lane) - 1u))] = idx;
}

// One loop part over its queue. A lane runs its path's part (the top repeats
// through null collisions, the NEE through its transmittance steps) until the
// path ends, moves to another part or has run `chunk` steps of this one. Lanes
// are topped up in batches: once at most `refillBelow` lanes of the warp still
// run a path (or none do), the lanes whose paths moved store their states and
// queue them at their next part, and the idle lanes take the next paths of
// this part's queue -- so the state copies run with many lanes at once instead
// of one lane at a time. FRESH (first round's top): the queue is the wave's
// paths 0..count-1, started from the generate stage's rays.
// 128 registers (4 blocks per SM): capping the top, surface and NEE parts at 80
// registers (6 blocks) spills little but ran 5% slower on the 1024^2 fBm frame.
template <int ACT, bool FRESH, bool BRICKS, bool HALF>
__global__ void __launch_bounds__(kVolBlock, 4)
    KVolEvent(DevScene S, PathBuffers B, VolWave V, uint32_t count, uint32_t cur, uint32_t* err, uint32_t mode,
              int refillBelow, int chunk) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t in = cur * kVolActs + (uint32_t)ACT;
  const uint32_t n = FRESH ? count : V.cnt[in];
  // blocks past one thread per queued path leave at once (their first fetch
  // would be an atomic on the one queue head)
  if (blockIdx.x * blockDim.x >= n) return;
  uint32_t* head = V.cnt + 2 * kVolActs + ACT;
  VolPathState* states = static_cast<VolPathState*>(V.state);
  VolPathState p;
  uint32_t idx = 0, ended = 0;
  int steps = 0;  // of this part, for the lane's path in this launch
  int dst = -1;   // a path that moved on, held until the next batch hand-off
  bool live = false, drained = n == 0;
  unsigned long long nRays = 0, nShadow = 0;
  for (;;) {
    const uint32_t liveMask = __ballot_sync(0xffffffffu, live);
    if (liveMask == 0u || (!drained && __popc(liveMask) <= refillBelow)) {
      if (__ballot_sync(0xffffffffu, dst >= 0) != 0u) {
        if (dst >= 0) states[idx] = p;
        VolPush(V, dst, idx);
        dst = -1;
      }
      const uint32_t need = __ballot_sync(0xffffffffu, !live);
      if (!drained && need != 0u) {
        const int leader = __ffs(need) - 1;
        uint32_t base = 0;
        if ((int)lane == leader) base = atomicAdd(head, (uint32_t)__popc(need));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (base + (uint32_t)__popc(need) >= n) drained = true;
        if (!live) {
          const uint32_t i = base + __popc(need & ((1u << lane) - 1u));
          if (i < n) {
            if (FRESH) {
              idx = i;
              const float4 ro = B.rayO[idx], rd = B.rayD[idx];
              const uint2 rs = B.rng[idx];
              Pcg32 rng;
              rng.state = ((uint64_t)rs.y << 32) | rs.x;
              VolInit(S, p, VRay{V3{ro.x, ro.y, ro.z}, V3{rd.x, rd.y, rd.z}, ro.w, rd.w}, rng);
            } else {
              idx = V.q[(size_t)in * V.capacity + i];
              p = states[idx];
            }
            steps = 0;
            live = true;
          }
        }
      }
      if (__ballot_sync(0xffffffffu, live) == 0u) break;
    }
    if (live) {
      if (!VolAct<BRICKS, HALF>(S, p, ACT, mode, err)) {
        B.L[idx] = make_float4(p.result.x, p.result.y, p.result.z, 0.f);
        nRays += p.nRays;
        nShadow += p.nShadow;
        ended++;
        live = false;
      } else if (p.act != ACT || ++steps >= chunk) {
        dst = (int)VolQueueOf(ACT, p.act, cur);
        live = false;
      }
    }
  }
  if (nRays) atomicAdd(B.counters + kMiscBase + 2, (uint32_t)nRays);
  if (nShadow) atomicAdd(B.counters + kMiscBase + 3, (uint32_t)nShadow);
  if (ended) atomicAdd(V.cnt + kVolEndedWord, ended);
}

// End of a round: the current parity's queues and every head start empty.
__global__ void KVolRoundEnd(VolWave V, uint32_t cur) {
  const uint32_t t = threadIdx.x;
  if (t < (uint32_t)kVolActs) {
    V.cnt[cur * kVolActs + t] = 0u;
    V.cnt[2 * kVolActs + t] = 0u;
  }
}

#ifndef RAD_HOST_EMULATION
cudaError_t LaunchVolPath(const DevScene& S, const PathBuffers& B, const WaveParams& w, uint32_t* err,
                          cudaStream_t st, uint32_t mode) {
  if (w.count == 0) return cudaSuccess;
  int perSm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, KVolPath<true, true>, kVolBlock, 0);
  int cap = PathGridBlocks() / 8 * (perSm > 0 ? perSm : 4);
  int blocks = (int)std::min<uint32_t>((w.count + kVolBlock - 1) / kVolBlock, (uint32_t)cap);
  switch (mode & (kVolBricks | kVolHalf)) {
    case 0: KVolPath<false, false><<<blocks, kVolBlock, 0, st>>>(S, B, w.count, err, mode); break;
    case kVolBricks: KVolPath<true, false><<<blocks, kVolBlock, 0, st>>>(S, B, w.count, err, mode); break;
    case kVolHalf: KVolPath<false, true><<<blocks, kVolBlock, 0, st>>>(S, B, w.count, err, mode); break;
    default: KVolPath<true, true><<<blocks, kVolBlock, 0, st>>>(S, B, w.count, err, mode); break;
  }
  return cudaGetLastError();
}

// Blocks of each part kernel: the SMs x min(blocks per SM asked for, the
// kernel's occupancy), at most one thread per path.
template <bool BRICKS, bool HALF>
static void VolGrids(uint32_t count, int perSmAsked, int* blocks) {
  const void* k[kVolActs] = {(const void*)KVolEvent<kActTop, false, BRICKS, HALF>,
                             (const void*)KVolEvent<kActScatter, false, BRICKS, HALF>,
                             (const void*)KVolEvent<kActSurface, false, BRICKS, HALF>,
                             (const void*)KVolEvent<kActNee, false, BRICKS, HALF>,
                             (const void*)KVolEvent<kActScatterEnd, false, BRICKS, HALF>,
                             (const void*)KVolEvent<kActSurfaceEnd, false, BRICKS, HALF>};
  for (int a = 0; a < kVolActs; a++) {
    int perSm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k[a], kVolBlock, 0);
    perSm = std::max(1, std::min(perSm > 0 ? perSm : 4, perSmAsked));
    const uint32_t cap = (uint32_t)(PathGridBlocks() / 8 * perSm);
    blocks[a] = (int)std::min<uint32_t>((count + kVolBlock - 1) / kVolBlock, cap);
  }
}

template <bool BRICKS, bool HALF>
static cudaError_t VolRound(const DevScene& S, const PathBuffers& B, const VolWave& V, uint32_t count, uint32_t r,
                            const int* blocks, uint32_t* err, cudaStream_t st, uint32_t mode, int refillBelow,
                            int chunk) {
  const uint32_t cur = r & 1u;
  const int g0 = blocks[kActTop];
  if (r == 0)
    KVolEvent<kActTop, true, BRICKS, HALF><<<g0, kVolBlock, 0, st>>>(S, B, V, count, cur, err, mode, refillBelow, chunk);
  else
    KVolEvent<kActTop, false, BRICKS, HALF><<<g0, kVolBlock, 0, st>>>(S, B, V, count, cur, err, mode, refillBelow,
                                                                      chunk);
  KVolEvent<kActScatter, false, BRICKS, HALF><<<blocks[kActScatter], kVolBlock, 0, st>>>(S, B, V, count, cur, err, mode,
                                                                                       refillBelow, chunk);
  KVolEvent<kActSurface, false, BRICKS, HALF><<<blocks[kActSurface], kVolBlock, 0, st>>>(S, B, V, count, cur, err, mode,
                                                                                       refillBelow, chunk);
  KVolEvent<kActNee, false, BRICKS, HALF><<<blocks[kActNee], kVolBlock, 0, st>>>(S, B, V, count, cur, err, mode,
                                                                               refillBelow, chunk);
  KVolEvent<kActScatterEnd, false, BRICKS, HALF><<<blocks[kActScatterEnd], kVolBlock, 0, st>>>(
      S, B, V, count, cur, err, mode, refillBelow, chunk);
  KVolEvent<kActSurfaceEnd, false, BRICKS, HALF><<<blocks[kActSurfaceEnd], kVolBlock, 0, st>>>(
      S, B, V, count, cur, err, mode, refillBelow, chunk);
  KVolRoundEnd<<<1, 32, 0, st>>>(V, cur);
  return cudaGetLastError();
}

cudaError_t LaunchVolWavefront(const DevScene& S, const PathBuffers& B, const VolWave& V, const WaveParams& w,
                               uint32_t* err, cudaStream_t st, uint32_t mode, const TraceTune& tu,
                               uint32_t* hostCounts, uint64_t* launches) {
  if (w.count == 0) return cudaSuccess;
  if (w.count > V.capacity) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(V.cnt, 0, kVolCountWords * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  int blocks[kVolActs];
  switch (mode & (kVolBricks | kVolHalf)) {
    case 0: VolGrids<false, false>(w.count, tu.blocksPerSm, blocks); break;
    case kVolBricks: VolGrids<true, false>(w.count, tu.blocksPerSm, blocks); break;
    case kVolHalf: VolGrids<false, true>(w.count, tu.blocksPerSm, blocks); break;
    default: VolGrids<true, true>(w.count, tu.blocksPerSm, blocks); break;
  }
  const int refillBelow = std::max(0, std::min(31, tu.refillBusy - 1));
  const int chunk = std::max(1, tu.volChunk);
  // At the end of a round every live path waits in a queue of the next round,
  // so ended + queued = count, and the wave is done when those are empty.
  // The counters are read back every 4 rounds from round 8 on. Every round
  // advances each live path by at least one step of its part, and the steps of
  // a path are bounded (loop iterations, transmittance steps), so the rounds
  // are too; the host loop's own bound turns a runaway into an error.
  for (uint32_t r = 0; r <= (uint32_t)kMaxVolIter; r++) {
    switch (mode & (kVolBricks | kVolHalf)) {
      case 0: e = VolRound<false, false>(S, B, V, w.count, r, blocks, err, st, mode, refillBelow, chunk); break;
      case kVolBricks: e = VolRound<true, false>(S, B, V, w.count, r, blocks, err, st, mode, refillBelow, chunk); break;
      case kVolHalf: e = VolRound<false, true>(S, B, V, w.count, r, blocks, err, st, mode, refillBelow, chunk); break;
      default: e = VolRound<true, true>(S, B, V, w.count, r, blocks, err, st, mode, refillBelow, chunk); break;
    }
    if (e != cudaSuccess) return e;
    if (launches) *launches += kVolActs + 1;
    if (r + 1 >= 8 && (r + 1) % 4 == 0) {
      e = cudaMemcpyAsync(hostCounts, V.cnt, kVolCountWords * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) return e;
      uint32_t queued = 0;
      for (int a = 0; a < kVolActs; a++) queued += hostCounts[((r & 1u) ^ 1u) * kVolActs + a];
      if ((uint64_t)hostCounts[kVolEndedWord] + queued != w.count) return cudaErrorIllegalState;
      if (queued == 0) return cudaSuccess;
    }
  }
  return cudaErrorIllegalState;
}

#endif  // RAD_HOST_EMULATION

}  // namespace rad
