// `vol_path` integrator (VolPath::Li, rad.offline/src/renderer/vol_path.cpp:27-349)
// as one thread per path sample running the whole delta-tracking loop: free
// flights against the medium majorant (medium.cpp:19-43), null / real
// collisions with hero-channel spectral MIS, phase-function NEE with the
// ratio-tracking transmittance loop (vol_path.cpp:224-342) and index-matched
// boundaries. Camera rays and PCG streams come from the wavefront generate
// stage; the radiance goes to the path's L slot for the accumulate stage.
#include "dbsdf.cuh"
#include "dscene.cuh"
#include "kernels.h"

namespace rad {

constexpr int kVolBlock = 128;
constexpr int kMaxTrLoop = 1 << 20;  // bound on transmittance-loop iterations (device check)
constexpr int kMaxVolIter = 1 << 22; // bound on free-flight iterations per path

struct MedInt {
  float T;
  V3 P;
  Frame sh;
  V3 Wi;
  float MinT;
  V3 sS, sN, sT, cE;
};

struct VRay {
  V3 O, D;
  float MinT, MaxT;
};

// grid.cpp:41-75 (trilinear with the half-texel neighbour rule), :88-103
RD V3 EvalGrid(const DevScene& S, const MediumRec& md, V3 p) {
  auto wrap = [&](float v) {
    if (md.repeatWrap) return clampr(v - floorf(v), 0.f, 1.f);
    return clampr(v, 0.f, 1.f);
  };
  V3 wp{wrap(p.x), wrap(p.y), wrap(p.z)};
  V3 fp{wp.x * ((float)md.nx - 1.f), wp.y * ((float)md.ny - 1.f), wp.z * ((float)md.nz - 1.f)};
  int ix = (int)fp.x, iy = (int)fp.y, iz = (int)fp.z;
  int dpu = (fp.x > ((float)ix + 0.5f)) ? 1 : -1;
  int dpv = (fp.y > ((float)iy + 0.5f)) ? 1 : -1;
  int dpw = (fp.z > ((float)iz + 0.5f)) ? 1 : -1;
  int apu = min(max(ix + dpu, 0), md.nx - 1);
  int apv = min(max(iy + dpv, 0), md.ny - 1);
  int apw = min(max(iz + dpw, 0), md.nz - 1);
  float du = fminr(fabsf(fp.x - (float)ix - 0.5f), 1.f);
  float dv = fminr(fabsf(fp.y - (float)iy - 0.5f), 1.f);
  float dw = fminr(fabsf(fp.z - (float)iz - 0.5f), 1.f);
  const float* g = S.volume + md.gridOffset;
  int ch = md.channels;
  auto rd = [&](int u, int v, int w) -> V3 {
    size_t st = (((size_t)w * (size_t)md.ny + (size_t)v) * (size_t)md.nx + (size_t)u) * (size_t)ch;
    if (ch == 1) return v3s(__ldg(g + st));
    return V3{__ldg(g + st), __ldg(g + st + 1), __ldg(g + st + 2)};
  };
  V3 c000 = rd(ix, iy, iz), c100 = rd(apu, iy, iz), c010 = rd(ix, apv, iz), c001 = rd(ix, iy, apw);
  V3 c110 = rd(apu, apv, iz), c011 = rd(ix, apv, apw), c101 = rd(apu, iy, apw), c111 = rd(apu, apv, apw);
  V3 a = Fmadd(c000, v3s(1.f - du), c100 * du);
  V3 b = Fmadd(c010, v3s(1.f - du), c110 * du);
  V3 e = Fmadd(a, v3s(1.f - dv), b * dv);
  V3 f = Fmadd(c001, v3s(1.f - du), c101 * du);
  V3 g2 = Fmadd(c011, v3s(1.f - du), c111 * du);
  V3 h = Fmadd(f, v3s(1.f - dv), g2 * dv);
  return Fmadd(e, v3s(1.f - dw), h * dw);
}

// medium.cpp:19-43 with heterogeneous.cpp / homogeneous.cpp
RD MedInt SampleInteraction(const DevScene& S, const MediumRec& md, const VRay& ray, float sample, int channel) {
  MedInt mei;
  mei.Wi = -ray.D;
  mei.sh = FrameFromN(mei.Wi);
  bool aabbIts;
  float mint, maxt;
  if (md.kind == MED_HOMOGENEOUS) {
    aabbIts = true;
    mint = 0.f;
    maxt = kInf;
  } else {
    V3 lo{md.bbMin[0], md.bbMin[1], md.bbMin[2]}, hi{md.bbMax[0], md.bbMax[1], md.bbMax[2]};
    bool contains = ray.O.x >= lo.x && ray.O.y >= lo.y && ray.O.z >= lo.z && ray.O.x <= hi.x && ray.O.y <= hi.y &&
                    ray.O.z <= hi.z;
    aabbIts = !is_zero(ray.D) || contains;
    V3 rcp{1.f / ray.D.x, 1.f / ray.D.y, 1.f / ray.D.z};
    V3 t1 = cmul(lo - ray.O, rcp), t2 = cmul(hi - ray.O, rcp);
    V3 t1p{fminr(t1.x, t2.x), fminr(t1.y, t2.y), fminr(t1.z, t2.z)};
    V3 t2p{fmaxr(t1.x, t2.x), fmaxr(t1.y, t2.y), fmaxr(t1.z, t2.z)};
    mint = max_comp(t1p);
    maxt = min_comp(t2p);
    aabbIts = aabbIts && maxt >= mint;
  }
  aabbIts = aabbIts && (isfinite(mint) || isfinite(maxt));
  bool active = aabbIts;
  if (!active) {
    mint = 0.f;
    maxt = kInf;
  }
  mint = fmaxr(0.f, mint);
  maxt = fminr(ray.MaxT, maxt);
  V3 combined = md.kind == MED_HOMOGENEOUS ? V3{md.sigmaT[0], md.sigmaT[1], md.sigmaT[2]} * md.scale
                                           : v3s(md.maxDensity);
  float m = comp(combined, channel);
  float sampledT = mint + (-logf(1.f - sample) / m);
  bool validMi = active && (sampledT <= maxt);
  mei.T = validMi ? sampledT : kInf;
  mei.P = ray.D * sampledT + ray.O;
  mei.MinT = mint;
  V3 alb{md.albedo[0], md.albedo[1], md.albedo[2]};
  if (md.kind == MED_HOMOGENEOUS) {
    mei.sT = V3{md.sigmaT[0], md.sigmaT[1], md.sigmaT[2]} * md.scale;
    mei.sS = cmul(mei.sT, alb);
    mei.sN = v3s(0.f);
  } else {
    V3 local = AffineRows(md.toLocal, mei.P);
    V3 e = md.gridSigma ? EvalGrid(S, md, local) : V3{md.sigmaT[0], md.sigmaT[1], md.sigmaT[2]};
    mei.sT = e * md.scale;
    mei.sS = cmul(mei.sT, alb);
    mei.sN = v3s(md.maxDensity) - mei.sT;
  }
  mei.cE = combined;
  return mei;
}

RD V3 ExpV(V3 v) { return V3{expf(v.x), expf(v.y), expf(v.z)}; }

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

RD bool VTrace(const DevScene& S, const VRay& ray, SurfInt& si, uint32_t* err) {
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
  return true;
}

RD VRay Spawn(V3 P, V3 N, V3 d) { return VRay{OffsetP(P, N, d), d, 0.f, kFloatMax}; }

RD int MediumOfHit(const DevScene& S, const SurfInt& si, V3 D) {
  const ShapeRec& sh = S.shapes[si.shape];
  return dot(D, si.N) > 0.f ? sh.outMedium : sh.inMedium;
}

// vol_path.cpp:224-342
RD V3 VolSampleLight(const DevScene& S, Pcg32& rng, int medium, int channel, V3 refP, V3 refN, DirSample& dsr,
                     uint32_t* err, uint64_t& nRays) {
  float xl = Next1D(rng);
  V2 xd = Next2D(rng);
  V3 li;
  dsr = SampleLightDirection(S, refP, xl, xd, li);
  if (dsr.Pdf <= 0.f) return v3s(0.f);
  VRay ray = Spawn(refP, refN, dsr.Dir);
  float totalDist = 0.f;
  V3 resultTr = v3s(1.f);
  bool active = true, needsIntersection = true;
  SurfInt si;
  si.T = kInf;
  si.shape = -1;
  for (int guard = 0; active; guard++) {
    if (guard >= kMaxTrLoop) {
      atomicOr(err, 2u);
      return v3s(0.f);
    }
    float remainingDist = dsr.Dist * (1.f - kShadowEps) - totalDist;
    ray.MaxT = remainingDist;
    active = active && remainingDist > 0.f;
    if (!active) break;
    bool escapedMedium = false;
    bool activeMedium = active && medium >= 0;
    bool activeSurface = active && !activeMedium;
    if (activeMedium) {
      const MediumRec& md = S.media[medium];
      MedInt mei = SampleInteraction(S, md, ray, Next1D(rng), channel);
      if (md.kind == MED_HOMOGENEOUS && mei.T != kInf) ray.MaxT = fminr(mei.T, remainingDist);
      if (needsIntersection) {
        VTrace(S, ray, si, err);
        nRays++;
      }
      if (si.T < mei.T) mei.T = kInf;
      bool isSpectral = true;
      {
        float t = fminr(remainingDist, fminr(mei.T, si.T)) - mei.MinT;
        if (t >= 0.f) {
          V3 tr = ExpV(mei.cE * -t);
          V3 ffp = (si.T < mei.T || mei.T > remainingDist) ? tr : cmul(tr, mei.cE);
          float trPdf = comp(ffp, channel);
          V3 mTr = trPdf > 0.f ? tr / trPdf : v3s(0.f);
          resultTr = cmul(resultTr, mTr);
        }
      }
      if ((mei.T > remainingDist) && mei.T != kInf) totalDist = dsr.Dist;
      if (mei.T > remainingDist) mei.T = kInf;
      escapedMedium = mei.T == kInf;
      activeMedium = mei.T != kInf;
      isSpectral = isSpectral && activeMedium;
      if (activeMedium) {
        totalDist += mei.T;
        ray.O = mei.P;
        si.T = si.T - mei.T;
        if (isSpectral) resultTr = cmul(resultTr, mei.sN);
      }
    }
    bool intersect = activeSurface && needsIntersection;
    if (intersect) {
      VTrace(S, ray, si, err);
      nRays++;
    }
    needsIntersection = needsIntersection && !intersect;
    activeSurface = activeSurface || escapedMedium;
    if (activeSurface) totalDist += si.T;
    activeSurface = activeSurface && si.T != kInf && active && !activeMedium;
    if (activeSurface) {
      if (S.shapes[si.shape].bsdf >= 0) resultTr = v3s(0.f);
      ray = Spawn(si.P, si.N, ray.D);
    }
    ray.MaxT = remainingDist;
    needsIntersection = needsIntersection || activeSurface;
    active = active && (activeMedium || activeSurface) && !is_zero(resultTr);
    if (activeSurface) {
      const ShapeRec& sh = S.shapes[si.shape];
      if (sh.inMedium >= 0 || sh.outMedium >= 0) medium = MediumOfHit(S, si, ray.D);
    }
  }
  return cmul(li, resultTr);
}

__global__ void __launch_bounds__(kVolBlock) KVolPath(DevScene S, PathBuffers B, uint32_t count, uint32_t* err) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  float4 ro = B.rayO[i], rd = B.rayD[i];
  uint2 rs = B.rng[i];
  Pcg32 rng;
  rng.state = ((uint64_t)rs.y << 32) | rs.x;
  VRay ray{V3{ro.x, ro.y, ro.z}, V3{rd.x, rd.y, rd.z}, ro.w, rd.w};
  int medium = S.globalMedium;
  V3 thr = v3s(1.f), result = v3s(0.f);
  float eta = 1.f;
  bool isSpecular = true;
  V3 prevP = v3s(0.f);
  float prevPdf = 1.f;
  uint64_t nRays = 0, nShadow = 0;
  int channel = (int)min((uint32_t)(Next1D(rng) * 3.f), 2u);
  SurfInt si;
  si.T = kInf;
  si.shape = -1;
  for (int depth = 0, guard = 0;; depth++, guard++) {
    if (guard >= kMaxVolIter) {
      atomicOr(err, 4u);
      break;
    }
    if (depth >= S.rrDepth) {
      float rr = fminr(max_comp(thr) * Sqr(eta), 0.95f);
      if (Next1D(rng) > rr) break;
      thr = thr * Rcp(rr);
    }
    if (S.maxDepth >= 0 && depth + 1 >= S.maxDepth) break;
    bool isSampleMedium = medium >= 0;
    bool isSampleSurface = !isSampleMedium;
    bool isNullScatter = false, isMediumScatter = false, isMediumEscaped = false;
    bool isSpectral = isSampleMedium;
    MedInt mei;
    mei.T = kInf;
    if (isSampleMedium) {
      const MediumRec& md = S.media[medium];
      mei = SampleInteraction(S, md, ray, Next1D(rng), channel);
      if (md.kind == MED_HOMOGENEOUS && mei.T != kInf) ray.MaxT = mei.T;
      VTrace(S, ray, si, err);
      nRays++;
      if (si.T < mei.T) mei.T = kInf;
      if (isSpectral) {
        // medium.cpp:45-59
        V3 tr, ffp;
        float t = fminr(mei.T, si.T) - mei.MinT;
        if (t <= 0.f) {
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
      isMediumEscaped = mei.T == kInf;
      isSampleMedium = mei.T != kInf;
      bool nullScatter = Next1D(rng) > comp(mei.sT, channel) / comp(mei.cE, channel);
      isNullScatter = nullScatter && isSampleMedium;
      isMediumScatter = !isNullScatter && isSampleMedium;
      if (isSpectral && isNullScatter) thr = cmul(thr, mei.sN) * comp(mei.cE, channel) / comp(mei.sN, channel);
      if (isMediumScatter) prevP = mei.P;
    }
    if (isNullScatter) {
      ray.O = mei.P;
      si.T = si.T - mei.T;
    }
    if (isMediumScatter) {
      const MediumRec& md = S.media[medium];
      if (isSpectral) thr = cmul(thr, mei.sS) * comp(mei.cE, channel) / comp(mei.sT, channel);
      DirSample dsr;
      V3 li = VolSampleLight(S, rng, medium, channel, mei.P, v3s(0.f), dsr, err, nShadow);
      if (dsr.Pdf > 0.f) {
        float phaseVal = PhaseEval(md, mei, dsr.Dir);
        float weight = dsr.IsDelta ? 1.f : VMis(dsr.Pdf, phaseVal);
        result = result + cmul(thr, li) * weight * phaseVal / dsr.Pdf;
      }
      float phasePdf;
      V3 wo = PhaseSample(md, mei, Next2D(rng), phasePdf);
      ray = Spawn(mei.P, v3s(0.f), wo);
      isSpecular = false;
      prevPdf = phasePdf;
    }
    isSampleSurface = isSampleSurface || isMediumEscaped;
    if (isSampleSurface) {
      bool hit = VTrace(S, ray, si, err);
      nRays++;
      int hitLight = hit ? S.shapes[si.shape].light : S.envLight;
      if (hitLight >= 0) {
        float weight;
        if (isSpecular) {
          weight = 1.f;
        } else {
          V3 rel = si.P - prevP;
          float dist = norm(rel);
          V3 dir = hit ? rel / dist : -si.Wi;
          weight = VMis(prevPdf, PdfLightDirection(S, hitLight, prevP, dir, si.sh.N, dist));
        }
        V3 li = EvalLightAt(S, hitLight, &si);
        result = result + cmul(thr, li) * weight;
      }
      if (!hit) break;
      const ShapeRec& shp = S.shapes[si.shape];
      if (shp.light >= 0) break;
      if (shp.bsdf < 0) {
        ray = Spawn(si.P, si.N, ray.D);
        medium = MediumOfHit(S, si, ray.D);
        depth--;
        continue;
      }
      const MatRec* mats = S.mats;
      if (mats[shp.bsdf].flags & BT_NODELTA) {
        DirSample dsr;
        V3 li = VolSampleLight(S, rng, medium, channel, si.P, si.N, dsr, err, nShadow);
        if (dsr.Pdf > 0.f) {
          V3 wo = ToLocal(si.sh, dsr.Dir);
          V3 f;
          float bsdfPdf;
          BsdfEvalPdf(mats, (uint32_t)shp.bsdf, si.Wi, wo, f, bsdfPdf);
          float weight = dsr.IsDelta ? 1.f : VMis(dsr.Pdf, bsdfPdf);
          result = result + cmul(cmul(thr, f), li) * weight / dsr.Pdf;
        }
      }
      float xl = Next1D(rng);
      V2 xd = Next2D(rng);
      BsdfSampleRes bs = BsdfSample(mats, (uint32_t)shp.bsdf, si.Wi, xl, xd);
      if (bs.pdf <= 0.f) break;
      thr = cmul(thr, bs.f) / bs.pdf;
      eta *= bs.eta;
      V3 nd = ToWorld(si.sh, bs.wo);
      ray = Spawn(si.P, si.N, nd);
      prevPdf = bs.pdf;
      prevP = si.P;
      isSpecular = (bs.type & BT_DELTA) != 0u;
      medium = MediumOfHit(S, si, ray.D);
    }
    if (!(isSampleSurface || isSampleMedium)) break;
  }
  B.L[i] = make_float4(result.x, result.y, result.z, 0.f);
  // ray counters: closest in [kMiscBase + 2], shadow-side traces in [kMiscBase + 3]
  atomicAdd(B.counters + kMiscBase + 2, (uint32_t)nRays);
  atomicAdd(B.counters + kMiscBase + 3, (uint32_t)nShadow);
}

cudaError_t LaunchVolPath(const DevScene& S, const PathBuffers& B, const WaveParams& w, uint32_t* err,
                          cudaStream_t st) {
  if (w.count == 0) return cudaSuccess;
  KVolPath<<<(w.count + kVolBlock - 1) / kVolBlock, kVolBlock, 0, st>>>(S, B, w.count, err);
  return cudaGetLastError();
}

}  // namespace rad
