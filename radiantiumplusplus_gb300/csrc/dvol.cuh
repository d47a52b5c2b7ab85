// Medium sampling of the `vol_path` integrator (medium.cpp:19-43,
// heterogeneous.cpp, homogeneous.cpp, grid.cpp:41-103) plus the brick-majorant
// free flight; shared by the kernel (k_vol.cu) and host-side checks.
#pragma once
#ifndef RAD_HOST_EMULATION
#include <cuda_fp16.h>
#endif
#include "dmath.cuh"
#include "records.h"

namespace rad {

// vol_path mode bits: kVolBricks (16^3-brick majorants, implies kVolRealDepth), kVolHalf
// (fp16 grid), kVolRealDepth (null collisions count neither toward max_depth nor for
// Russian roulette); 0 = the reference's algorithm
constexpr uint32_t kVolBricks = 1u, kVolHalf = 2u, kVolRealDepth = 4u;

RD int IMin(int a, int b) { return a < b ? a : b; }
RD int IMax(int a, int b) { return a < b ? b : a; }

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

// grid.cpp:41-75 (trilinear with the half-texel neighbour rule), :88-103.
// HALF reads the fp16 copy of the grid instead of the fp32 one.
template <bool HALF>
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
  int apu = IMin(IMax(ix + dpu, 0), md.nx - 1);
  int apv = IMin(IMax(iy + dpv, 0), md.ny - 1);
  int apw = IMin(IMax(iz + dpw, 0), md.nz - 1);
  float du = fminr(fabsf(fp.x - (float)ix - 0.5f), 1.f);
  float dv = fminr(fabsf(fp.y - (float)iy - 0.5f), 1.f);
  float dw = fminr(fabsf(fp.z - (float)iz - 0.5f), 1.f);
  const float* g = S.volume + md.gridOffset;
  const uint16_t* gh = S.volumeHalf + md.gridOffset;
  int ch = md.channels;
  auto at = [&](size_t i) -> float {
#ifndef RAD_HOST_EMULATION
    if constexpr (HALF) return __half2float(__ushort_as_half(__ldg(gh + i)));
#endif
    return __ldg(g + i);
  };
  auto rd = [&](int u, int v, int w) -> V3 {
    size_t st = (((size_t)w * (size_t)md.ny + (size_t)v) * (size_t)md.nx + (size_t)u) * (size_t)ch;
    if (ch == 1) return v3s(at(st));
    return V3{at(st), at(st + 1), at(st + 2)};
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

// Free flight against the 16^3-brick majorants (BRICKS mode; no counterpart in
// the reference, which uses one global majorant): the optical depth
// tau = -ln(1 - u) from the same single random number is consumed brick by
// brick along [mint, maxt] by a 3D DDA over the brick lattice in voxel
// coordinates f = local * (n - 1). Returns the collision distance, or kInf, and
// the majorant of the brick the collision lies in.
RD float BrickFreeFlight(const DevScene& S, const MediumRec& md, V3 O, V3 D, float mint, float maxt, float u,
                         float& mLocal) {
  mLocal = 0.f;
  V3 lo = AffineRows(md.toLocal, O);
  V3 ld = LinearRows(md.toLocal, D);
  const float sc[3] = {(float)(md.nx - 1), (float)(md.ny - 1), (float)(md.nz - 1)};
  const float f0[3] = {lo.x * sc[0], lo.y * sc[1], lo.z * sc[2]};
  const float fd[3] = {ld.x * sc[0], ld.y * sc[1], ld.z * sc[2]};
  const int nb[3] = {IMax(1, (md.nx - 1 + 15) / 16), IMax(1, (md.ny - 1 + 15) / 16), IMax(1, (md.nz - 1 + 15) / 16)};
  float tau = -logf(1.f - u);
  float t = mint;
  int b[3], step[3];
  float tMax[3], tDelta[3];
  for (int a = 0; a < 3; a++) {
    float pa = f0[a] + fd[a] * t;
    b[a] = IMin(IMax((int)floorf(pa * (1.f / 16.f)), 0), nb[a] - 1);
    if (fd[a] > 0.f) {
      step[a] = 1;
      tMax[a] = (16.f * (float)(b[a] + 1) - f0[a]) / fd[a];
      tDelta[a] = 16.f / fd[a];
    } else if (fd[a] < 0.f) {
      step[a] = -1;
      tMax[a] = (16.f * (float)b[a] - f0[a]) / fd[a];
      tDelta[a] = -16.f / fd[a];
    } else {
      step[a] = 0;
      tMax[a] = kInf;
      tDelta[a] = kInf;
    }
  }
  const float* maj = S.brickMaj + md.brickOffset;
  const int steps = nb[0] + nb[1] + nb[2] + 4;  // a line crosses at most this many bricks
  for (int k = 0; k < steps; k++) {
    float t1 = fminf(fminf(tMax[0], tMax[1]), fminf(tMax[2], maxt));
    float m = __ldg(maj + ((size_t)b[2] * nb[1] + b[1]) * nb[0] + b[0]);
    if (t1 > t) {
      float dt = t1 - t;
      if (m > 0.f && tau <= m * dt) {
        mLocal = m;
        return t + tau / m;
      }
      tau -= m * dt;
      t = t1;
    }
    if (t >= maxt) break;
    int a = (tMax[0] <= tMax[1] && tMax[0] <= tMax[2]) ? 0 : (tMax[1] <= tMax[2] ? 1 : 2);
    b[a] += step[a];
    if (b[a] < 0 || b[a] >= nb[a]) break;
    tMax[a] += tDelta[a];
  }
  return kInf;
}

// medium.cpp:19-43 with heterogeneous.cpp / homogeneous.cpp. BRICKS: the
// majorant is the brick's (BrickFreeFlight) instead of the global one.
template <bool BRICKS, bool HALF>
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
  V3 alb{md.albedo[0], md.albedo[1], md.albedo[2]};
  if (BRICKS && md.kind == MED_HETEROGENEOUS && md.hasBricks) {
    float mLocal = 0.f;
    float T = active ? BrickFreeFlight(S, md, ray.O, ray.D, mint, maxt, sample, mLocal) : kInf;
    mei.T = T;
    mei.MinT = mint;
    mei.cE = v3s(mLocal);
    if (T != kInf) {
      mei.P = ray.D * T + ray.O;
      V3 local = AffineRows(md.toLocal, mei.P);
      mei.sT = EvalGrid<HALF>(S, md, local) * md.scale;
    } else {
      mei.P = ray.O;
      mei.sT = v3s(0.f);
    }
    mei.sS = cmul(mei.sT, alb);
    mei.sN = mei.cE - mei.sT;
    return mei;
  }
  V3 combined = md.kind == MED_HOMOGENEOUS ? V3{md.sigmaT[0], md.sigmaT[1], md.sigmaT[2]} * md.scale
                                           : v3s(md.maxDensity);
  float m = comp(combined, channel);
  float sampledT = mint + (-logf(1.f - sample) / m);
  bool validMi = active && (sampledT <= maxt);
  mei.T = validMi ? sampledT : kInf;
  mei.P = ray.D * sampledT + ray.O;
  mei.MinT = mint;
  if (md.kind == MED_HOMOGENEOUS) {
    mei.sT = V3{md.sigmaT[0], md.sigmaT[1], md.sigmaT[2]} * md.scale;
    mei.sS = cmul(mei.sT, alb);
    mei.sN = v3s(0.f);
  } else {
    V3 local = AffineRows(md.toLocal, mei.P);
    V3 e = md.gridSigma ? EvalGrid<HALF>(S, md, local) : V3{md.sigmaT[0], md.sigmaT[1], md.sigmaT[2]};
    mei.sT = e * md.scale;
    mei.sS = cmul(mei.sT, alb);
    mei.sN = v3s(md.maxDensity) - mei.sT;
  }
  mei.cE = combined;
  return mei;
}

}  // namespace rad
