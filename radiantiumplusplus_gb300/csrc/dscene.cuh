// Device scene functions: hit -> SurfaceInteraction (mesh_base.cpp:38-82,
// rectangle.cpp:186-199, sphere.cpp:215-249, interaction.cpp:45-53), light
// sampling and densities (scene.cpp:65-113, area.cpp, skybox.cpp, shape.cpp,
// sphere.cpp:265-328), spawn offsets (interaction.cpp:10-26) and the
// perspective camera (perspective.cpp:73-82).
#pragma once
#include "dtex.cuh"
#include "dtrace.cuh"

namespace rad {

struct SurfInt {
  float T;
  V3 P, N;  // geometric normal
  int shape;
  Frame sh;
  V3 Wi;
};

// interaction.cpp:10-16
RD V3 OffsetP(V3 P, V3 N, V3 d) {
  float m = fmaxr(fmaxr(fabsf(P.x), fabsf(P.y)), fabsf(P.z));
  float mag = (1.f + m) * kRayEps;
  mag = MulSign(mag, dot(N, d));
  return Fmadd(v3s(mag), N, P);
}

RD V3 ShapeM3(const ShapeRec& s, int i) { return V3{s.m[i], s.m[i + 1], s.m[i + 2]}; }

// HitShapeRecord::ComputeSurfaceInteraction for a hit of ray (O, D).
RD SurfInt ComputeSI(const DevScene& S, V3 O, V3 D, const TraceHit& h) {
  SurfInt si;
  const ShapeRec& sh = S.shapes[h.shape];
  si.T = h.t;
  si.shape = (int)h.shape;
  V3 dPdU;
  V3 shN;
  if (sh.kind == SHAPE_MESH) {
    uint32_t tri = (h.prim - sh.primOffset) + sh.triOffset;
    uint32_t f0 = __ldg(S.idx + 3 * (size_t)tri), f1 = __ldg(S.idx + 3 * (size_t)tri + 1),
             f2 = __ldg(S.idx + 3 * (size_t)tri + 2);
    V3 p0 = ld3(S.pos + 3 * (size_t)f0), p1 = ld3(S.pos + 3 * (size_t)f1), p2 = ld3(S.pos + 3 * (size_t)f2);
    float b0 = 1.f - h.u - h.v, b1 = h.u, b2 = h.v;
    V3 dp0 = p1 - p0, dp1 = p2 - p0;
    si.P = p0 * b0 + (p1 * b1 + (p2 * b2));
    si.N = normalized(cross(dp0, dp1));
    if (!sh.hasUV) {
      V3 X, Y;
      CoordinateSystem(si.N, X, Y);
      dPdU = X;
    } else {
      const float* uvp = S.uv;
      float u0x = uvp[2 * f0], u0y = uvp[2 * f0 + 1], u1x = uvp[2 * f1], u1y = uvp[2 * f1 + 1];
      float u2x = uvp[2 * f2], u2y = uvp[2 * f2 + 1];
      float d0x = u1x - u0x, d0y = u1y - u0y, d1x = u2x - u0x, d1y = u2y - u0y;
      float det = d0x * d1y - (d0y * d1x);
      float invDet = det == 0.f ? 0.f : Rcp(det);
      dPdU = invDet == 0.f ? v3s(0.f) : (d1y * dp0 - (d0y * dp1)) * invDet;
    }
    if (!sh.hasNormals) {
      shN = si.N;
    } else {
      V3 n0 = ld3(S.nrm + 3 * (size_t)f0), n1 = ld3(S.nrm + 3 * (size_t)f1), n2 = ld3(S.nrm + 3 * (size_t)f2);
      V3 n = n0 * b0 + (n1 * b1 + (n2 * b2));
      float il = Rsqrt(sqnorm(n));
      shN = n * il;
    }
  } else if (sh.kind == SHAPE_RECT) {
    V3 N = ShapeM3(sh, 18), Tr = ShapeM3(sh, 21);
    V3 p = D * h.t + O;
    si.P = N * dot(Tr - p, N) + p;
    si.N = N;
    shN = N;
    dPdU = ShapeM3(sh, 12);
  } else {
    V3 c{sh.m[0], sh.m[1], sh.m[2]};
    float rad = sh.m[3];
    V3 gn = normalized((D * h.t + O) - c);
    shN = gn;
    si.P = Fmadd(gn, v3s(rad), c);
    V3 local = AffineRows(sh.m + 4, si.P);
    V3 du{-local.y, local.x, 0.f};
    dPdU = LinearRows(sh.m + 16, du * (2.f * kPi));
    si.N = gn;
  }
  // interaction.cpp:45-53
  si.sh.N = shN;
  if (is_zero(dPdU)) {
    V3 X, Y;
    CoordinateSystem(shN, X, Y);
    si.sh.S = X;
  } else {
    si.sh.S = normalized(shN * (-dot(shN, dPdU)) + dPdU);
  }
  si.sh.T = cross(shN, si.sh.S);
  si.Wi = ToLocal(si.sh, -D);
  return si;
}

// uv and position derivatives of a hit (mesh_base.cpp:38-66, rectangle.cpp:204-218,
// sphere.cpp:215-240); needed only where textures are looked up.
struct SurfUV {
  V2 uv;
  V3 dPdU, dPdV;
};
RD SurfUV ComputeUV(const DevScene& S, const TraceHit& h, const SurfInt& si) {
  SurfUV r;
  const ShapeRec& sh = S.shapes[h.shape];
  if (sh.kind == SHAPE_MESH) {
    if (!sh.hasUV) {
      r.uv = V2{h.u, h.v};
      CoordinateSystem(si.N, r.dPdU, r.dPdV);
      return r;
    }
    uint32_t tri = (h.prim - sh.primOffset) + sh.triOffset;
    uint32_t f0 = __ldg(S.idx + 3 * (size_t)tri), f1 = __ldg(S.idx + 3 * (size_t)tri + 1),
             f2 = __ldg(S.idx + 3 * (size_t)tri + 2);
    V3 p0 = ld3(S.pos + 3 * (size_t)f0), p1 = ld3(S.pos + 3 * (size_t)f1), p2 = ld3(S.pos + 3 * (size_t)f2);
    V3 dp0 = p1 - p0, dp1 = p2 - p0;
    float b0 = 1.f - h.u - h.v, b1 = h.u, b2 = h.v;
    const float* uvp = S.uv;
    float u0x = uvp[2 * f0], u0y = uvp[2 * f0 + 1], u1x = uvp[2 * f1], u1y = uvp[2 * f1 + 1];
    float u2x = uvp[2 * f2], u2y = uvp[2 * f2 + 1];
    r.uv = V2{u0x * b0 + (u1x * b1 + (u2x * b2)), u0y * b0 + (u1y * b1 + (u2y * b2))};
    float d0x = u1x - u0x, d0y = u1y - u0y, d1x = u2x - u0x, d1y = u2y - u0y;
    float det = d0x * d1y - (d0y * d1x);
    float invDet = det == 0.f ? 0.f : Rcp(det);
    if (invDet == 0.f) {
      r.dPdU = r.dPdV = v3s(0.f);
    } else {
      r.dPdU = (d1y * dp0 - (d0y * dp1)) * invDet;
      r.dPdV = (-d1x * dp0 + (d0x * dp1)) * invDet;
    }
  } else if (sh.kind == SHAPE_RECT) {
    r.uv = V2{h.u * 0.5f + 0.5f, h.v * 0.5f + 0.5f};
    r.dPdU = ShapeM3(sh, 12);
    r.dPdV = ShapeM3(sh, 15);
  } else {
    V3 local = AffineRows(sh.m + 4, si.P);
    float rd2 = Sqr(local.x) + Sqr(local.y);
    // UnitAngleZ (math_ext.h:101-104)
    float temp = asinf(0.5f * norm(V3{local.x, local.y, local.z - MulSign(1.f, local.z)})) * 2.f;
    float theta = local.z >= 0.f ? temp : kPi - temp;
    float phi = atan2f(local.y, local.x);
    if (phi < 0.f) phi += 2.f * kPi;
    r.uv = V2{phi / (2.f * kPi), theta / kPi};
    V3 du{-local.y, local.x, 0.f};
    float rd = sqrtf(rd2);
    float invRd = Rcp(rd);
    float cosPhi = local.x * invRd, sinPhi = local.y * invRd;
    V3 dv{local.z * cosPhi, local.z * sinPhi, -rd};
    if (rd == 0.f) dv = V3{1.f, 0.f, 0.f};
    r.dPdU = LinearRows(sh.m + 16, du * (2.f * kPi));
    r.dPdV = LinearRows(sh.m + 16, dv * kPi);
  }
  return r;
}

// uv derivatives of the first hit of a camera ray: the pixel-offset rays of
// Perspective::SampleRayDifferential (perspective.cpp:84-97) intersected with
// the tangent plane, then solved for (du, dv) as SurfaceInteraction::BSDF(ray)
// does (interaction.cpp:83-109). (sx, sy): the ray's screen position; O: its origin.
RD void CameraUVDerivs(const CameraRec& c, float sx, float sy, V3 O, const SurfInt& si, const SurfUV& su, V2& duvdx,
                       V2& duvdy) {
  float tx = sx * (1.f / (float)c.width), ty = sy * (1.f / (float)c.height);
  V3 nearP = Affine4(c.clipToCamera, V3{tx, ty, 0.f});
  V3 ax = normalized(nearP + V3{c.dx[0], c.dx[1], c.dx[2]});
  V3 ay = normalized(nearP + V3{c.dy[0], c.dy[1], c.dy[2]});
  const float* m = c.camToWorld;
  V3 Dx{(m[0] * ax.x + m[1] * ax.y) + m[2] * ax.z, (m[4] * ax.x + m[5] * ax.y) + m[6] * ax.z,
        (m[8] * ax.x + m[9] * ax.y) + m[10] * ax.z};
  V3 Dy{(m[0] * ay.x + m[1] * ay.y) + m[2] * ay.z, (m[4] * ay.x + m[5] * ay.y) + m[6] * ay.z,
        (m[8] * ay.x + m[9] * ay.y) + m[10] * ay.z};
  float d = dot(si.N, si.P);
  float tX = (d - dot(si.N, O)) / dot(si.N, Dx);
  float tY = (d - dot(si.N, O)) / dot(si.N, Dy);
  V3 dpdx = (Dx * tX + O) - si.P;
  V3 dpdy = (Dy * tY + O) - si.P;
  float a00 = dot(su.dPdU, su.dPdU), a01 = dot(su.dPdU, su.dPdV), a11 = dot(su.dPdV, su.dPdV);
  float invDet = Rcp(fmaf(a00, a11, -(a01 * a01)));
  float b0x = dot(su.dPdU, dpdx), b1x = dot(su.dPdV, dpdx), b0y = dot(su.dPdU, dpdy), b1y = dot(su.dPdV, dpdy);
  invDet = isfinite(invDet) ? invDet : 0.f;
  duvdx = V2{fmaf(a11, b0x, -(a01 * b1x)) * invDet, fmaf(a00, b1x, -(a01 * b0x)) * invDet};
  duvdy = V2{fmaf(a11, b0y, -(a01 * b1y)) * invDet, fmaf(a00, b1y, -(a01 * b0y)) * invDet};
}

// ---------------------------------------------------------------- lights
struct DirSample {
  V3 P, N, Dir;
  float Pdf, Dist;
  bool IsDelta;
};

// Mesh area CDF: DiscreteDistribution1D::SampleReuse (distribution.cpp:36-53).
RD uint32_t CdfLowerBound(const float* cdf, uint32_t n, float value) {
  uint32_t lo = 0, len = n;
  while (len > 0) {
    uint32_t half = len >> 1;
    uint32_t mid = lo + half;
    if (cdf[2 * (size_t)mid] < value) {
      lo = mid + 1;
      len = len - half - 1;
    } else {
      len = half;
    }
  }
  return lo;
}

// Shape::SamplePosition (mesh_base.cpp:84-110, rectangle.cpp:221-230,
// sphere.cpp:250-258): position, normal, area density and the sample's uv (a
// mesh's interpolated uv, else its barycentrics; a rectangle's xi; a sphere
// leaves it unset, here 0).
RD void ShapeSamplePosition(const DevScene& S, const ShapeRec& sh, V2 xi, V3& P, V3& N, float& pdf, V2& uv) {
  uv = V2{0.f, 0.f};
  if (sh.kind == SHAPE_SPHERE) {
    V3 local = SquareToUniformSphere(xi);
    P = Fmadd(local, v3s(sh.m[3]), V3{sh.m[0], sh.m[1], sh.m[2]});
    N = local;
    pdf = 1.f / sh.surfaceArea;
    return;
  }
  if (sh.kind == SHAPE_MESH) {
    const float* cdf = S.cdf + 2 * (size_t)sh.cdfOffset;
    float value = xi.y * sh.cdfSum;
    uint32_t idx = CdfLowerBound(cdf, sh.primCount, value);
    float pm = cdf[2 * (size_t)idx + 1] * sh.cdfNorm;
    float cd = idx == 0 ? 0.f : cdf[2 * (size_t)(idx - 1)] * sh.cdfNorm;
    V2 txi{xi.x, (xi.y - cd) / pm};
    uint32_t tri = idx + sh.triOffset;
    uint32_t f0 = S.idx[3 * (size_t)tri], f1 = S.idx[3 * (size_t)tri + 1], f2 = S.idx[3 * (size_t)tri + 2];
    V3 p0 = ld3(S.pos + 3 * (size_t)f0), p1 = ld3(S.pos + 3 * (size_t)f1), p2 = ld3(S.pos + 3 * (size_t)f2);
    V3 e0 = p1 - p0, e1 = p2 - p0;
    V2 b = SquareToUniformTriangle(txi);
    P = e0 * b.x + (e1 * b.y + p0);
    pdf = sh.cdfNorm;
    if (!sh.hasUV) {
      uv = b;
    } else {
      const float* t = S.uv;
      float b0 = 1.f - b.x - b.y;
      uv = V2{t[2 * f0] * b0 + (t[2 * f1] * b.x + (t[2 * f2] * b.y)),
              t[2 * f0 + 1] * b0 + (t[2 * f1 + 1] * b.x + (t[2 * f2 + 1] * b.y))};
    }
    if (!sh.hasNormals) {
      N = normalized(cross(e0, e1));
    } else {
      V3 n0 = ld3(S.nrm + 3 * (size_t)f0), n1 = ld3(S.nrm + 3 * (size_t)f1), n2 = ld3(S.nrm + 3 * (size_t)f2);
      N = normalized(n0 * (1.f - b.x - b.y) + (n1 * b.x + (n2 * b.y)));
    }
  } else {
    float sx = xi.x * 2.f - 1.f, sy = xi.y * 2.f - 1.f;
    P = AffineRows(sh.m, V3{sx, sy, 0.f});
    N = ShapeM3(sh, 18);
    pdf = 1.f / sh.surfaceArea;
    uv = xi;
  }
}

// Shape::SamplePosition + SampleDirection (shape.cpp:7-19, mesh_base.cpp:84-110,
// rectangle.cpp:204-214, sphere.cpp:251-320); uv as ShapeSamplePosition's.
RD DirSample ShapeSampleDirection(const DevScene& S, const ShapeRec& sh, V3 refP, V2 xi, V2& uv) {
  DirSample d;
  uv = V2{0.f, 0.f};
  if (sh.kind != SHAPE_SPHERE) {
    V3 P, N;
    float pdf;
    ShapeSamplePosition(S, sh, xi, P, N, pdf, uv);
    d.P = P;
    d.N = N;
    d.IsDelta = false;
    V3 dir = P - refP;
    float distanceSquared = sqnorm(dir);
    d.Dist = sqrtf(distanceSquared);
    d.Dir = dir / d.Dist;
    float dp = fabsf(dot(d.Dir, N));
    float x = distanceSquared / dp;
    d.Pdf = pdf * (isfinite(x) ? x : 0.f);
    return d;
  }
  V3 c{sh.m[0], sh.m[1], sh.m[2]};
  float radius = sh.m[3];
  V3 dcv = c - refP;
  float dc2 = sqnorm(dcv);
  float radiusAdj = radius * (1.f - kRayEps);
  if (dc2 > Sqr(radiusAdj)) {
    float invDc = Rsqrt(dc2);
    float sinThetaMax = radius * invDc;
    float sinThetaMax2 = Sqr(sinThetaMax);
    float invSinThetaMax = Rcp(sinThetaMax);
    float cosThetaMax = SafeSqrt(1.f - sinThetaMax2);
    float sinTheta2 = sinThetaMax2 > 0.00068523262f ? 1.f - Sqr(fmaf(cosThetaMax - 1.f, xi.x, 1.f))
                                                   : sinThetaMax2 * xi.x;
    float cosTheta = SafeSqrt(1.f - sinTheta2);
    float cosAlpha = sinTheta2 * invSinThetaMax + cosTheta * SafeSqrt(fmaf(-sinTheta2, Sqr(invSinThetaMax), 1.f));
    float sinAlpha = SafeSqrt(fmaf(-cosAlpha, cosAlpha, 1.f));
    float ph = xi.y * (2.f * kPi);
    float sinPhi = sinf(ph), cosPhi = cosf(ph);
    Frame fr = FrameFromN(dcv * -invDc);
    V3 dd = ToWorld(fr, V3{cosPhi * sinAlpha, sinPhi * sinAlpha, cosAlpha});
    d.P = Fmadd(dd, v3s(radius), c);
    d.N = dd;
    V3 dir = d.P - refP;
    float dist2 = sqnorm(dir);
    d.Dist = sqrtf(dist2);
    d.Dir = dir / d.Dist;
    d.Pdf = SquareToUniformConePdf(cosThetaMax);
  } else {
    V3 dd = SquareToUniformSphere(xi);
    d.P = Fmadd(dd, v3s(radius), c);
    d.N = dd;
    V3 dir = d.P - refP;
    float dist2 = sqnorm(dir);
    d.Dist = sqrtf(dist2);
    d.Dir = dir / d.Dist;
    d.Pdf = (1.f / sh.surfaceArea) * dist2 / AbsDot(d.Dir, d.N);
  }
  d.IsDelta = radius == 0.f;
  return d;
}

// shape.cpp:21-25 / sphere.cpp:322-328
RD float ShapePdfDirection(const ShapeRec& sh, V3 refP, V3 dir, V3 n, float dist) {
  if (sh.kind == SHAPE_SPHERE) {
    V3 c{sh.m[0], sh.m[1], sh.m[2]};
    float sinAlpha = sh.m[3] * Rcp(norm(c - refP));
    float cosAlpha = SafeSqrt(1.f - sinAlpha * sinAlpha);
    return sinAlpha < kOneMinusEps ? SquareToUniformConePdf(cosAlpha)
                                   : (1.f / sh.surfaceArea) * Sqr(dist) / AbsDot(dir, n);
  }
  float pdf = sh.kind == SHAPE_MESH ? sh.cdfNorm : 1.f / sh.surfaceArea;
  float dp = fabsf(dot(dir, n));
  pdf *= dp == 0.f ? 0.f : Sqr(dist) / dp;
  return pdf;
}

// ContinuousDistribution1D::Sample (distribution.cpp:84-97) over one row of a
// 2D distribution laid out as pdf[n], cdf[n + 1], normalization. The bin is
// lower_bound(cdf, xi) - 1 in unsigned arithmetic clamped to n - 1, so xi = 0
// (lower_bound 0) selects the last bin, as in the reference.
RD uint32_t Dist1DSample(const float* row, uint32_t n, float xi, float& pdf) {
  const float* cdf = row + n;
  uint32_t lo = 0, len = n + 1;
  while (len > 0) {
    uint32_t half = len >> 1, mid = lo + half;
    if (cdf[mid] < xi) {
      lo = mid + 1;
      len = len - half - 1;
    } else {
      len = half;
    }
  }
  uint32_t idx = lo == 0u ? n - 1u : (lo - 1u < n - 1u ? lo - 1u : n - 1u);
  pdf = row[idx] * row[2 * n + 1];
  return idx;
}
// Skybox::SampleLightDir / PdfDirection on a bitmap radiance map (skybox.cpp:112-131,
// 213-233) with ContinuousDistribution2D (distribution.cpp:103-129): rows of
// 2 nu + 2 floats, then the marginal (pdf, cdf, normalization, sum).
// ContinuousDistribution2D::Sample / Pdf (distribution.cpp:103-129) of a
// light's luminance distribution (a bitmap skybox or area light).
RD float Dist2DSample(const DevScene& S, const LightRec& L, V2 xi, uint32_t& iu, uint32_t& iv) {
  const uint32_t nu = L.distW, nv = L.distH;
  const float* base = S.lightDist + L.dist;
  const float* marg = base + (size_t)nv * (2 * nu + 2);
  float pdf1, pdf0;
  iv = Dist1DSample(marg, nv, xi.y, pdf1);
  iu = Dist1DSample(base + (size_t)iv * (2 * nu + 2), nu, xi.x, pdf0);
  return pdf0 * pdf1;
}
RD float Dist2DPdf(const DevScene& S, const LightRec& L, V2 uv) {
  const uint32_t nu = L.distW, nv = L.distH;
  const float* base = S.lightDist + L.dist;
  const float* marg = base + (size_t)nv * (2 * nu + 2);
  float fu = uv.x * (float)nu, fv = uv.y * (float)nv;
  uint32_t iu = fu >= 0.f ? (uint32_t)fu : 0u, iv = fv >= 0.f ? (uint32_t)fv : 0u;
  iu = iu < nu - 1u ? iu : nu - 1u;
  iv = iv < nv - 1u ? iv : nv - 1u;
  return base[(size_t)iv * (2 * nu + 2) + iu] / marg[2 * nv + 2];
}

RD bool EnvSampleDir(const DevScene& S, const LightRec& L, V2 xi, V3& worldDir, float& pdf, V2& uv) {
  uint32_t vi, vj;
  pdf = Dist2DSample(S, L, xi, vi, vj);
  if (pdf <= 0.f) return false;
  float y = (float)vj / (float)L.distH, x = (float)vi / (float)L.distW;
  uv = V2{x, y};
  float theta = y * kPi, phi = x * 2.f * kPi;
  float sinTheta = sinf(theta);
  if (sinTheta == 0.f) return false;
  pdf /= (2.f * kPi * kPi * sinTheta);
  float cosTheta = cosf(theta), sinPhi = sinf(phi), cosPhi = cosf(phi);
  V3 sph{cosPhi * sinTheta, sinPhi * sinTheta, cosTheta};
  worldDir = LinearRows(L.lin, V3{sph.y, sph.z, -sph.x});
  return true;
}
RD float EnvDirPdf(const DevScene& S, const LightRec& L, V3 dir) {
  V3 v = Affine4(L.m, dir);
  float theta = acosf(clampr(v.y, -1.f, 1.f));
  float sinTheta = sinf(theta);
  if (sinTheta == 0.f) return 0.f;
  float phi = atan2f(v.x, -v.z);
  phi = phi < 0.f ? phi + 2.f * kPi : phi;
  V2 uv{phi / (2.f * kPi), theta / kPi};
  float pdf = Dist2DPdf(S, L, uv);
  return pdf / (2.f * kPi * kPi * sinTheta);
}
// A light's texture at uv with zero derivatives (lights are looked up without
// ray differentials). One out-of-line copy serves every light lookup, so the
// texture filters' code is not repeated inside each kernel's light sampling.
static RDN V3 LightTex(const DevScene& S, uint32_t tex1, V2 uv) {
  TexCtx x{S.tex, S.texels, S.texBind, uv, V2{0.f, 0.f}, V2{0.f, 0.f}};
  TexVal r = TexEval(x, tex1 - 1u, uv);
  return V3{r.c[0], r.c[1], r.c[2]};
}

// The sky's radiance towards world direction d (skybox.cpp:53-63): the map's
// value at the direction's latitude-longitude uv.
RD V3 EnvRadiance(const DevScene& S, const LightRec& L, V3 d) {
  if (!L.tex) return V3{L.radiance[0], L.radiance[1], L.radiance[2]};
  V3 v = LinearRows(L.m, d);
  float phi = atan2f(v.x, -v.z);
  phi = phi < 0.f ? phi + 2.f * kPi : phi;
  float theta = acosf(clampr(v.y, -1.f, 1.f));
  return LightTex(S, L.tex, V2{phi / (2.f * kPi), theta / kPi});
}

// An area light's radiance at uv: its texture, else the constant (area.cpp:42-45).
RD V3 AreaRadiance(const DevScene& S, const LightRec& L, V2 uv) {
  if (!L.tex) return V3{L.radiance[0], L.radiance[1], L.radiance[2]};
  return LightTex(S, L.tex, uv);
}

// DiffuseArea::SamplePosition (area.cpp:93-115): a bitmap light samples its
// luminance distribution at texel corners uv of its rectangle
// (Rectangle::EvalParamSurface, rectangle.cpp:236-250; |dPdU x dPdV| is the
// rectangle's area). A constant or a chessboard (a 1 x 1 texture,
// chessboard.cpp:30-31) samples the shape, uv the shape sample's. pdf is the
// area density, 0 for a failed sample.
RD void AreaSamplePosition(const DevScene& S, const LightRec& L, V2 xi, V3& P, V3& N, V2& uv, float& pdf) {
  const ShapeRec& sh = S.shapes[L.shape];
  if (!L.distW) {
    ShapeSamplePosition(S, sh, xi, P, N, pdf, uv);
    pdf = pdf > 0.f ? pdf : 0.f;
    return;
  }
  uint32_t iu, iv;
  float p = Dist2DSample(S, L, xi, iu, iv);
  if (p <= 0.f) {
    P = N = v3s(0.f);
    uv = V2{0.f, 0.f};
    pdf = 0.f;
    return;
  }
  uv = V2{(float)iu / (float)L.distW, (float)iv / (float)L.distH};
  P = AffineRows(sh.m, V3{uv.x * 2.f - 1.f, uv.y * 2.f - 1.f, 0.f});
  N = ShapeM3(sh, 18);
  p /= sh.surfaceArea;
  pdf = p > 0.f ? p : 0.f;
}

// Scene::SampleLight (scene.cpp:65-77): uniform pick; false without lights.
RD bool PickLight(const DevScene& S, float xiL, int& index, float& pick) {
  if (S.nLights < 2) {
    index = 0;
    pick = 1.f;
    return S.nLights == 1;
  }
  float lf = xiL * (float)S.nLights;
  uint32_t iu = (uint32_t)lf;
  index = (int)(iu < S.nLights - 1 ? iu : S.nLights - 1);
  pick = S.lightPdf;
  return true;
}

// Light::SampleDirection of one light (area.cpp:47-75, skybox.cpp:65-106,
// point.cpp:33-49, projection.cpp:52-74, the directional extension).
RD DirSample LightSampleDirection(const DevScene& S, const LightRec& L, V3 refP, V2 xi, V3& li) {
  DirSample d{};
  li = v3s(0.f);
  V3 rad{L.radiance[0], L.radiance[1], L.radiance[2]};
  if (L.kind == LIGHT_AREA) {
    if (L.distW) return d;  // area.cpp:59-72: the bitmap branch's SurfaceInteraction::ToDsr leaves Pdf 0
    V2 uv;  // area.cpp:55-58: a chessboard is read at the shape sample's uv
    d = ShapeSampleDirection(S, S.shapes[L.shape], refP, xi, uv);
    li = dot(-d.Dir, d.N) >= 0.f ? AreaRadiance(S, L, uv) : v3s(0.f);
  } else if (L.kind == LIGHT_POINT) {  // point.cpp:33-49
    d.P = V3{L.dir[0], L.dir[1], L.dir[2]};
    d.N = v3s(0.f);
    d.Pdf = 1.f;
    d.IsDelta = true;
    V3 dir = d.P - refP;
    d.Dist = sqrtf(sqnorm(dir));
    float invDist = Rcp(d.Dist);
    d.Dir = dir * invDist;
    li = rad * Sqr(invDist);
  } else if (L.kind == LIGHT_PROJECTION) {  // projection.cpp:52-74 (constant irradiance)
    V3 local = Affine4(L.m, refP);
    V3 uv = Affine4(L.m + 16, local);
    bool inRange = uv.x >= 0.f && uv.x <= 1.f && uv.y >= 0.f && uv.y <= 1.f && local.z > 0.f;
    if (!inRange) return d;  // Pdf 0: no light sample
    d.P = V3{L.dir[0], L.dir[1], L.dir[2]};
    d.N = ld3(L.lin);
    d.Pdf = 1.f;
    d.IsDelta = true;
    V3 dir = d.P - refP;
    d.Dist = sqrtf(sqnorm(dir));
    d.Dir = dir * Rcp(d.Dist);
    float den = Sqr(local.z) * dot(-d.Dir, d.N);
    if (L.tex) {  // irradiance texture at the light-space uv, times the scale
      rad = cmul(LightTex(S, L.tex, V2{uv.x, uv.y}), rad);
    }
    li = V3{(rad.x * kPi) / den, (rad.y * kPi) / den, (rad.z * kPi) / den};
  } else {
    V3 wc{L.world[0], L.world[1], L.world[2]};
    float radius = fmaxr(L.world[3], norm(refP - wc));
    float dist = 2.f * radius;
    V3 worldDir;
    if (L.kind == LIGHT_SKYBOX) {
      if (L.distW) {  // bitmap radiance: luminance importance sampling (skybox.cpp:88-103)
        float pdf;
        V2 uv;
        if (!EnvSampleDir(S, L, xi, worldDir, pdf, uv)) {
          d.Pdf = 0.f;
          return d;
        }
        d.Pdf = pdf;
        rad = LightTex(S, L.tex, uv);
      } else {  // skybox.cpp:70-87
        V3 dir = normalized(SquareToUniformSphere(xi));
        worldDir = LinearRows(L.lin, dir);
        d.Pdf = SquareToUniformSpherePdf();
        if (L.tex) {
          float phi = atan2f(dir.x, -dir.z);
          phi = phi < 0.f ? phi + 2.f * kPi : phi;
          float theta = acosf(clampr(dir.y, -1.f, 1.f));
          rad = LightTex(S, L.tex, V2{phi / (2.f * kPi), theta / kPi});
        }
      }
      d.N = -worldDir;
      d.IsDelta = false;
    } else {
      V3 ld{L.dir[0], L.dir[1], L.dir[2]};
      worldDir = -ld;
      d.N = ld;
      d.Pdf = 1.f;
      d.IsDelta = true;
    }
    d.P = worldDir * dist + refP;
    d.Dir = worldDir;
    d.Dist = dist;
    li = rad;
  }
  return d;
}


// scene.cpp:87-96: uniform light pick, then the light's direction sample.
RD DirSample SampleLightDirection(const DevScene& S, V3 refP, float xiL, V2 xi, V3& li) {
  int index;
  float pick;
  if (!PickLight(S, xiL, index, pick)) {
    DirSample d{};
    li = v3s(0.f);
    d.Pdf = 0.f;
    return d;
  }
  DirSample d = LightSampleDirection(S, S.lights[index], refP, xi, li);
  d.Pdf *= pick;
  return d;
}

// scene.cpp:98-103
RD float PdfLightDirection(const DevScene& S, int light, V3 refP, V3 dir, V3 n, float dist, V2 uv) {
  const LightRec& L = S.lights[light];
  float p = 0.f;
  if (L.kind == LIGHT_AREA && L.distW) {  // area.cpp:81-90 (no facing test)
    float pdf = Dist2DPdf(S, L, uv);
    if (pdf > 0.f) p = pdf * Sqr(dist) / (S.shapes[L.shape].surfaceArea * -dot(dir, n));
  } else if (L.kind == LIGHT_AREA) {
    p = dot(-dir, n) >= 0.f ? ShapePdfDirection(S.shapes[L.shape], refP, dir, n, dist) : 0.f;
  } else if (L.kind == LIGHT_SKYBOX) {
    p = L.distW ? EnvDirPdf(S, L, dir) : SquareToUniformSpherePdf();
  }
  return p * S.lightPdf;
}

// area.cpp:42-45 / skybox.cpp:53-63; point and projection
// lights have no surface to hit and evaluate to 0 (point.cpp:29-31, projection.cpp:48-50).
RD V3 EvalLightAt(const DevScene& S, int light, const SurfInt* si, V2 uv) {
  const LightRec& L = S.lights[light];
  if (L.kind == LIGHT_AREA) return dot(ToWorld(si->sh, si->Wi), si->N) >= 0.f ? AreaRadiance(S, L, uv) : v3s(0.f);
  if (L.kind == LIGHT_SKYBOX) return EnvRadiance(S, L, -si->Wi);
  return v3s(0.f);
}

// ------------------------------------------------------- light tracing parts
// Perspective::Importance (perspective.cpp:124-139) of camera-space direction d.
RD float CameraImportance(const CameraRec& c, V3 d) {
  float cosTheta = d.z;
  if (cosTheta <= 0.f) return 0.f;
  float invCosTheta = Rcp(cosTheta);
  float px = d.x * invCosTheta, py = d.y * invCosTheta;
  if (!(c.rect[0] <= px && c.rect[1] <= py && px <= c.rect[2] && py <= c.rect[3])) return 0.f;
  return c.normalization * invCosTheta * invCosTheta * invCosTheta;
}

// Perspective::SampleDirection + Importance (perspective.cpp:101-137): the
// camera seen from a world point. Returns false (pdf 0) outside the frustum.
RD bool CameraSampleDirection(const CameraRec& c, V3 ref, V3& camP, V3& dir, float& dist, V2& pixel,
                              float& importance) {
  V3 refP = Affine4(c.worldToCam, ref);
  if (refP.z < c.nearZ || refP.z > c.farZ) return false;
  V3 ndc = Affine4(c.camToClip, refP);
  if (ndc.x < 0.f || ndc.x >= 1.f || ndc.y < 0.f || ndc.y >= 1.f) return false;
  pixel = V2{ndc.x * (float)c.width, ndc.y * (float)c.height};
  dist = norm(refP);
  float invDist = Rcp(dist);
  V3 d = refP * invDist;
  camP = Affine4(c.camToWorld, v3s(0.f));
  dir = (camP - ref) * invDist;
  importance = CameraImportance(c, d) * invDist * invDist;
  return true;
}

// Light::SampleRay (area.cpp:120-128, skybox.cpp:135-163, point.cpp:67-71,
// projection.cpp:93-104): an emitted ray and its weight. `ok` false when the
// light cannot emit (a map with zero density). The `directional` extension
// emits parallel rays through a disk covering the world sphere.
RD bool LightSampleRay(const DevScene& S, const LightRec& L, V2 xi2, V2 xi3, V3& O, V3& D, V3& li) {
  V3 rad{L.radiance[0], L.radiance[1], L.radiance[2]};
  if (L.kind == LIGHT_AREA) {
    V3 P, N;
    V2 uv;
    float pdf;
    AreaSamplePosition(S, L, xi2, P, N, uv, pdf);
    Frame fr = FrameFromN(N);
    V3 local = SquareToCosineHemisphere(xi3);
    D = ToWorld(fr, local);
    O = OffsetP(P, N, D);
    li = AreaRadiance(S, L, uv) * kPi / pdf;  // Eval(si) of a point with no incident direction
    return true;
  }
  if (L.kind == LIGHT_POINT) {
    O = V3{L.dir[0], L.dir[1], L.dir[2]};
    D = SquareToUniformSphere(xi3);
    li = rad * 4.f * kPi;
    return true;
  }
  if (L.kind == LIGHT_PROJECTION) {
    V3 nearP = Affine4(L.m2, V3{xi3.x, xi3.y, 0.f});
    V3 nearDir = normalized(nearP);
    O = V3{L.dir[0], L.dir[1], L.dir[2]};
    D = LinearRows(L.m2 + 16, nearDir);
    V3 irr{L.m2[29], L.m2[30], L.m2[31]};
    if (L.tex) {
      irr = LightTex(S, L.tex, xi3);
    }
    li = irr * kPi * L.m2[28];  // SampleRay leaves out the light's scale
    return true;
  }
  V3 wc{L.world[0], L.world[1], L.world[2]};
  float R = L.world[3];
  V2 off = SquareToUniformDiskConcentric(xi2);
  if (L.kind == LIGHT_SKYBOX) {
    float pdfDir;
    V2 uv;
    if (!L.distW) {
      pdfDir = SquareToUniformSpherePdf();
      uv = xi3;
    } else {
      V3 unused;
      if (!EnvSampleDir(S, L, xi3, unused, pdfDir, uv)) return false;
    }
    float theta = uv.y * kPi, phi = uv.x * kPi * 2.f;
    float sinTheta = sinf(theta), cosTheta = cosf(theta), sinPhi = sinf(phi), cosPhi = cosf(phi);
    V3 sph{cosPhi * sinTheta, sinPhi * sinTheta, cosTheta};
    V3 d{sph.y, sph.z, -sph.x};
    V3 worldD = AffineRows(L.lin, -d);  // ApplyAffineToWorld of a direction, as the reference writes it
    Frame fr = FrameFromN(d);
    V3 perp = ToWorld(fr, V3{off.x, off.y, 0.f});
    O = wc + (perp - worldD) * R;
    D = worldD;
    V3 c = rad;
    if (L.tex) {
      c = LightTex(S, L.tex, uv);
    }
    li = ((c * kPi) * Sqr(R)) / pdfDir;
    return true;
  }
  // directional (extension): parallel rays along the light's direction
  V3 ld{L.dir[0], L.dir[1], L.dir[2]};
  Frame fr = FrameFromN(ld);
  V3 perp = ToWorld(fr, V3{off.x, off.y, 0.f});
  O = wc + (perp - ld) * R;
  D = ld;
  li = rad * kPi * Sqr(R);
  return true;
}

// ---------------------------------------------------------------- camera
RD void CameraRay(const CameraRec& c, float sx, float sy, V3& O, V3& D, float& tmin, float& tmax) {
  float tx = sx * (1.f / (float)c.width), ty = sy * (1.f / (float)c.height);
  V3 nearP = Affine4(c.clipToCamera, V3{tx, ty, 0.f});
  V3 dir = normalized(nearP);
  float invZ = Rcp(dir.z);
  O = Affine4(c.camToWorld, V3{0.f, 0.f, 0.f});
  V3 lw{(c.camToWorld[0] * dir.x + c.camToWorld[1] * dir.y) + c.camToWorld[2] * dir.z,
        (c.camToWorld[4] * dir.x + c.camToWorld[5] * dir.y) + c.camToWorld[6] * dir.z,
        (c.camToWorld[8] * dir.x + c.camToWorld[9] * dir.y) + c.camToWorld[10] * dir.z};
  D = normalized(lw);
  tmin = c.nearZ * invZ;
  tmax = c.farZ * invZ;
}

}  // namespace rad
