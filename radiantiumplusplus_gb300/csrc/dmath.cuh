// Device math for the sm_103a kernels. Compiled with --fmad=false so that the
// only fused multiply-adds are the explicit fmaf() calls written where the
// reference writes Math::Fmadd (rad.core math_base.h:68); +,-,*,/ and sqrt
// are IEEE round-to-nearest, so the arithmetic matches the reference's FP32
// expression order. Transcendentals are CUDA's own sinf/cosf/expf/logf/...
#pragma once
#include <stdint.h>

#if defined(RAD_HOST_EMULATION)
// Host build of the device functions and kernels: a CPU harness runs the same
// traversal, BSDF, scene and integrator code (bit for bit the device
// arithmetic, with the host's libm for transcendentals). A kernel runs as a
// loop over its grid, one thread at a time, each thread the only active lane
// of its warp: ballots hold the calling lane's bit, shuffles from the leader
// return the lane's own value, and warp sums see no other lanes.
#include <cuda_runtime.h>
#include <cmath>
#include <cstring>
#define RD inline
#define RDN inline
#undef __global__
#define __global__
#undef __launch_bounds__
#define __launch_bounds__(...)
#undef __device__
#define __device__
#undef __forceinline__
#define __forceinline__ inline
struct HemuDim3 {
  unsigned x, y, z;
};
inline HemuDim3 threadIdx{0u, 0u, 0u}, blockIdx{0u, 0u, 0u}, blockDim{1u, 1u, 1u}, gridDim{1u, 1u, 1u};
inline float __uint_as_float(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
inline uint32_t __float_as_uint(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline int __ffs(uint32_t x) { return __builtin_ffs((int)x); }
inline int __popc(uint32_t x) { return __builtin_popcount(x); }
template <typename T> inline T __ldg(const T* p) { return *p; }
inline uint32_t HemuLane() { return threadIdx.x & 31u; }
inline uint32_t __ballot_sync(uint32_t, bool p) { return p ? 1u << HemuLane() : 0u; }
inline uint32_t __match_any_sync(uint32_t, uint32_t) { return 1u << HemuLane(); }
template <typename T> inline T __shfl_sync(uint32_t, T v, int) { return v; }
template <typename T> inline T __shfl_down_sync(uint32_t, T, unsigned) { return T(0); }
inline uint32_t atomicOr(uint32_t* p, uint32_t v) { uint32_t o = *p; *p |= v; return o; }
inline float atomicAdd(float* p, float v) { float o = *p; *p += v; return o; }
inline uint32_t atomicAdd(uint32_t* p, uint32_t v) { uint32_t o = *p; *p += v; return o; }
inline unsigned long long atomicAdd(unsigned long long* p, unsigned long long v) {
  unsigned long long o = *p;
  *p += v;
  return o;
}
inline uint32_t atomicMax(uint32_t* p, uint32_t v) { uint32_t o = *p; if (v > o) *p = v; return o; }
using std::isfinite;
using std::isnan;
using std::isinf;
#else
#include <cuda_runtime.h>
#define RD __device__ __forceinline__
// large device functions called from several places: one copy in the code
#define RDN __device__ __noinline__
#endif

#include "records.h"

namespace rad {

struct V3 {
  float x, y, z;
};
struct V2 {
  float x, y;
};

RD V3 v3(float a, float b, float c) { return V3{a, b, c}; }
RD V3 v3s(float a) { return V3{a, a, a}; }
RD V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
RD V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
RD V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
RD V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
RD V3 operator*(float s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
RD V3 operator/(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }
RD V3 cmul(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
RD V3 cdiv(V3 a, V3 b) { return V3{a.x / b.x, a.y / b.y, a.z / b.z}; }
RD float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
RD V3 cross(V3 a, V3 b) { return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
RD float sqnorm(V3 a) { return dot(a, a); }
RD float norm(V3 a) { return sqrtf(sqnorm(a)); }
RD V3 normalized(V3 a) {
  float n = sqnorm(a);
  if (n > 0.f) {
    float s = sqrtf(n);
    return V3{a.x / s, a.y / s, a.z / s};
  }
  return a;
}
RD bool is_zero(V3 a) { return a.x == 0.f && a.y == 0.f && a.z == 0.f; }
RD float max_comp(V3 a) {
  float m = a.x;
  m = (m < a.y) ? a.y : m;
  m = (m < a.z) ? a.z : m;
  return m;
}
RD float min_comp(V3 a) {
  float m = a.x;
  m = (a.y < m) ? a.y : m;
  m = (a.z < m) ? a.z : m;
  return m;
}
RD float comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
RD V3 ld3(const float* p) { return V3{p[0], p[1], p[2]}; }

constexpr float kPi = 3.14159265358979323846f;
constexpr float kEps32 = 5.9604644775390625e-08f;  // 2^-24
constexpr float kRayEps = kEps32 * 1500.0f;         // math_ext.h:12
constexpr float kShadowEps = kRayEps * 10.0f;       // math_ext.h:16
constexpr float kOneMinusEps = 0.99999994039535522f;
constexpr float kFloatMax = 3.402823466e+38f;
constexpr float kInf = __builtin_huge_valf();

RD float Sqr(float v) { return v * v; }
RD float Sign(float v) { return v >= 0.f ? 1.f : -1.f; }
RD float MulSign(float a, float b) { return b >= 0.f ? a : -a; }
RD V3 MulSign(V3 a, float b) { return b >= 0.f ? a : -a; }
RD float Rcp(float v) { return 1.f / v; }
RD float Rsqrt(float v) { return 1.f / sqrtf(v); }
RD float SafeSqrt(float v) { return sqrtf(v > 0.f ? v : 0.f); }
RD float AbsDot(V3 a, V3 b) { return fabsf(dot(a, b)); }
RD float Lerp(float a, float b, float t) { return fmaf(b, t, fmaf(-a, t, a)); }
RD V3 Fmadd(V3 a, V3 b, V3 c) { return V3{fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y), fmaf(a.z, b.z, c.z)}; }
RD float Luminance(V3 c) { return (c.x * 0.212671f) + (c.y * 0.715160f) + (c.z * 0.072169f); }
RD float fminr(float a, float b) { return (b < a) ? b : a; }  // std::min
RD float fmaxr(float a, float b) { return (a < b) ? b : a; }  // std::max
// fmaxf(fmaxf(a, b), c) and fminf(fminf(a, b), c) as one instruction each
// (three-input max.f32 / min.f32, sm_100 and later); min and max do not round,
// so the values are the same.
#if defined(RAD_HOST_EMULATION)
RD float Max3(float a, float b, float c) { return fmaxf(fmaxf(a, b), c); }
RD float Min3(float a, float b, float c) { return fminf(fminf(a, b), c); }
#else
RD float Max3(float a, float b, float c) {
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
RD float Min3(float a, float b, float c) {
  float d;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
#endif
RD float clampr(float v, float lo, float hi) { return v < lo ? lo : (hi < v ? hi : v); }

// math_ext.h:48-61
RD void CoordinateSystem(V3 n, V3& X, V3& Y) {
  float sign = Sign(n.z);
  float a = -1.f / (sign + n.z);
  float b = n.x * n.y * a;
  X = V3{MulSign(Sqr(n.x) * a, n.z) + 1.0f, MulSign(b, n.z), MulSign(n.x, -n.z)};
  Y = V3{b, sign + Sqr(n.y) * a, -n.y};
}

struct Frame {
  V3 S, T, N;
};
RD Frame FrameFromN(V3 n) {
  Frame f;
  CoordinateSystem(n, f.S, f.T);
  f.N = n;
  return f;
}
RD V3 ToWorld(const Frame& f, V3 v) { return f.N * v.z + (f.T * v.y + (f.S * v.x)); }
RD V3 ToLocal(const Frame& f, V3 v) { return V3{dot(v, f.S), dot(v, f.T), dot(v, f.N)}; }

// frame.cpp:48-56, including its clamp that returns (1, 1) away from the pole.
RD void SinCosPhi(V3 v, float& sinPhi, float& cosPhi) {
  float sin2Theta = fmaf(v.x, v.x, Sqr(v.y));
  float invSinTheta = Rsqrt(sin2Theta);
  float rx = v.x * invSinTheta, ry = v.y * invSinTheta;
  if (fabsf(sin2Theta) <= 4.f * kEps32) {
    rx = 1.f;
    ry = 0.f;
  } else {
    rx = (-1.f < rx) ? -1.f : rx;
    ry = (-1.f < ry) ? -1.f : ry;
    rx = (rx < 1.f) ? 1.f : rx;
    ry = (ry < 1.f) ? 1.f : ry;
  }
  sinPhi = ry;
  cosPhi = rx;
}

// Row-major 3x4 / 4x4 transforms (transform.cpp:51-95); row dots evaluated
// ((m0 v0 + m1 v1) + m2 v2) + m3.
RD V3 AffineRows(const float* m, V3 v) {  // 3 rows of 4, w == 1
  return V3{((m[0] * v.x + m[1] * v.y) + m[2] * v.z) + m[3], ((m[4] * v.x + m[5] * v.y) + m[6] * v.z) + m[7],
            ((m[8] * v.x + m[9] * v.y) + m[10] * v.z) + m[11]};
}
RD V3 LinearRows(const float* m, V3 v) {  // 3 rows of 4
  return V3{(m[0] * v.x + m[1] * v.y) + m[2] * v.z, (m[4] * v.x + m[5] * v.y) + m[6] * v.z,
            (m[8] * v.x + m[9] * v.y) + m[10] * v.z};
}
RD V3 Affine4(const float* m, V3 v) {  // full 4x4 with perspective divide
  float r0 = ((m[0] * v.x + m[1] * v.y) + m[2] * v.z) + m[3];
  float r1 = ((m[4] * v.x + m[5] * v.y) + m[6] * v.z) + m[7];
  float r2 = ((m[8] * v.x + m[9] * v.y) + m[10] * v.z) + m[11];
  float r3 = ((m[12] * v.x + m[13] * v.y) + m[14] * v.z) + m[15];
  return V3{r0 / r3, r1 / r3, r2 / r3};
}
RD V3 Affine4w1(const float* m, V3 v) {  // 4x4 known affine: divide by the computed w as the reference does
  return Affine4(m, v);
}

// ------------------------------------------------------------------- RNG
// PCG32 stream per (pixel, sample, seed); the same definition as the CPU oracle.
RD uint64_t SplitMix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ULL;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}
struct Pcg32 {
  uint64_t state;
};
RD uint32_t PcgNext(Pcg32& r) {
  uint64_t old = r.state;
  r.state = old * 6364136223846793005ULL + 1442695040888963407ULL;
  uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
  uint32_t rot = (uint32_t)(old >> 59u);
  return (xs >> rot) | (xs << ((32u - rot) & 31u));
}
RD Pcg32 PcgForSample(uint32_t pixel, uint32_t sample, uint32_t seed) {
  Pcg32 r;
  uint64_t init = SplitMix64(SplitMix64(seed) ^ (((uint64_t)pixel << 32) | (uint64_t)sample));
  r.state = 0;
  PcgNext(r);
  r.state += init;
  PcgNext(r);
  return r;
}
// Advances the stream by `delta` draws in O(log delta) (Brown, "Random Number
// Generation with Arbitrary Strides", 1994: the LCG's k-step map is again affine).
RD void PcgAdvance(Pcg32& r, uint64_t delta) {
  uint64_t curMult = 6364136223846793005ULL, curPlus = 1442695040888963407ULL, accMult = 1u, accPlus = 0u;
  while (delta) {
    if (delta & 1u) {
      accMult *= curMult;
      accPlus = accPlus * curMult + curPlus;
    }
    curPlus = (curMult + 1u) * curPlus;
    curMult *= curMult;
    delta >>= 1;
  }
  r.state = accMult * r.state + accPlus;
}
RD float Next1D(Pcg32& r) { return (float)(PcgNext(r) >> 8) * 5.9604644775390625e-08f; }
RD V2 Next2D(Pcg32& r) {
  float a = Next1D(r);
  float b = Next1D(r);
  return V2{a, b};
}

// ------------------------------------------------------------------ warps
// warp.cpp:22-80
RD V2 SquareToUniformDisk(V2 u) {
  float r = sqrtf(u.x);
  float angle = 2.f * kPi * u.y;
  return V2{r * cosf(angle), r * sinf(angle)};
}
RD V3 SquareToCosineHemisphere(V2 u) {
  V2 b = SquareToUniformDisk(u);
  return V3{b.x, b.y, SafeSqrt(1.f - Sqr(b.x) - Sqr(b.y))};
}
RD float SquareToCosineHemispherePdf(V3 v) { return v.z * (1.f / kPi); }
RD V2 SquareToUniformTriangle(V2 u) {
  float t = SafeSqrt(1.f - u.x);
  return V2{1.f - t, t * u.y};
}
RD V3 SquareToUniformSphere(V2 u) {
  float z = fmaf(-2.f, u.y, 1.f);
  float r = SafeSqrt(fmaf(-z, z, 1.f));
  float a = 2.f * kPi * u.x;
  return V3{r * cosf(a), r * sinf(a), z};
}
RD float SquareToUniformSpherePdf() { return 1.f / (4.f * kPi); }
// warp.cpp:80-95 (Shirley-Chiu concentric mapping)
RD V2 SquareToUniformDiskConcentric(V2 u) {
  float x = fmaf(2.f, u.x, -1.f);
  float y = fmaf(2.f, u.y, -1.f);
  bool quadrant = fabsf(x) < fabsf(y);
  float r = quadrant ? y : x;
  float rp = quadrant ? x : y;
  float phi = 0.25f * kPi * rp / r;
  if (quadrant) phi = 0.5f * kPi - phi;
  if (x == 0.f && y == 0.f) phi = 0.f;
  return V2{r * cosf(phi), r * sinf(phi)};
}
RD float SquareToUniformConePdf(float cosCutoff) { return 1.f / (2.f * kPi) / (1.f - cosCutoff); }

// ---------------------------------------------------------------- fresnel
// fresnel.cpp:14-77
RD V3 Reflect(V3 wi, V3 wh) {
  float k = 2.f * dot(wi, wh);
  return Fmadd(wh, v3s(k), -wi);
}
RD V3 Refract(V3 wi, V3 wh, float cosThetaT, float etaTI) {
  float k = fmaf(dot(wi, wh), etaTI, cosThetaT);
  return Fmadd(wh, v3s(k), -(wi * etaTI));
}
struct Dielectric {
  float r, cosThetaT, etaIT, etaTI;
};
RD Dielectric FresnelDielectric(float cosThetaI, float eta) {
  Dielectric d;
  bool isOutside = cosThetaI >= 0.f;
  float rcpEta = Rcp(eta);
  d.etaIT = isOutside ? eta : rcpEta;
  d.etaTI = isOutside ? rcpEta : eta;
  float sqrCosThetaT = fmaf(-fmaf(-cosThetaI, cosThetaI, 1.f), d.etaTI * d.etaTI, 1.f);
  float absCosThetaI = fabsf(cosThetaI);
  float absCosThetaT = SafeSqrt(sqrCosThetaT);
  bool indexMatched = eta == 1.f;
  bool specialCase = indexMatched || absCosThetaI == 0.f;
  float rSC = indexMatched ? 0.f : 1.f;
  float aS = fmaf(-d.etaIT, absCosThetaT, absCosThetaI) / fmaf(d.etaIT, absCosThetaT, absCosThetaI);
  float aP = fmaf(-d.etaIT, absCosThetaI, absCosThetaT) / fmaf(d.etaIT, absCosThetaI, absCosThetaT);
  d.r = 0.5f * (Sqr(aS) + Sqr(aP));
  if (specialCase) d.r = rSC;
  d.cosThetaT = cosThetaI >= 0.f ? -absCosThetaT : absCosThetaT;
  return d;
}
RD float ConductorChannel(float cosThetaI2, float sinThetaI2, float sinThetaI4, float cosThetaI, float etaR,
                          float etaI) {
  float temp1 = etaR * etaR - etaI * etaI - sinThetaI2;
  float a2pb2 = temp1 * temp1 + etaI * etaI * etaR * etaR * 4.f;
  a2pb2 = sqrtf(fmaxr(a2pb2, 0.f));
  float a = sqrtf(fmaxr((a2pb2 + temp1) * 0.5f, 0.f));
  float term1 = a2pb2 + cosThetaI2;
  float term2 = a * 2.f * cosThetaI;
  float rs = (term1 - term2) * (1.f / (term1 + term2));
  float term3 = a2pb2 * cosThetaI2 + sinThetaI4;
  float term4 = term2 * sinThetaI2;
  float rp = rs * (term3 - term4) * (1.f / (term3 + term4));
  return (rs + rp) * 0.5f;
}
RD V3 FresnelConductor(float cosThetaI, V3 eta, V3 k) {
  float c2 = cosThetaI * cosThetaI, s2 = 1.f - c2, s4 = s2 * s2;
  return V3{ConductorChannel(c2, s2, s4, cosThetaI, eta.x, k.x), ConductorChannel(c2, s2, s4, cosThetaI, eta.y, k.y),
            ConductorChannel(c2, s2, s4, cosThetaI, eta.z, k.z)};
}

// ------------------------------------------------------------- microfacet
// microfacet.cpp:12-285 (mitsuba variant)
struct Microfacet {
  float ax, ay;
  bool ggx, visible;
};
RD float MfD(const Microfacet& m, V3 wh) {
  float alphaXY = m.ax * m.ay;
  float cosTheta = wh.z;
  if (m.ggx) {
    float result = Rcp(kPi * alphaXY * Sqr(Sqr(wh.x / m.ax) + Sqr(wh.y / m.ay) + Sqr(wh.z)));
    return result * cosTheta > 1e-20f ? result : 0.f;
  }
  float cosTheta2 = Sqr(cosTheta);
  float result = expf(-(Sqr(wh.x / m.ax) + Sqr(wh.y / m.ay)) / cosTheta2) / (kPi * alphaXY * Sqr(cosTheta2));
  return result * cosTheta > 1e-20f ? result : 0.f;
}
RD float MfG1(const Microfacet& m, V3 v, V3 wh) {
  float xyAlpha2 = Sqr(m.ax * v.x) + Sqr(m.ay * v.y);
  float tanThetaAlpha2 = xyAlpha2 / Sqr(v.z);
  float result;
  if (m.ggx) {
    result = 2.f / (1.f + sqrtf(1.f + tanThetaAlpha2));
  } else {
    float a = Rsqrt(tanThetaAlpha2);
    float aSqr = Sqr(a);
    result = a >= 1.6f ? 1.f : (3.535f * a + 2.181f * aSqr) / (1.f + 2.276f * a + 2.577f * aSqr);
  }
  if (xyAlpha2 == 0.f) result = 1.f;
  if (dot(v, wh) * v.z <= 0.f) result = 0.f;
  return result;
}
RD float MfG(const Microfacet& m, V3 wi, V3 wo, V3 wh) { return MfG1(m, wi, wh) * MfG1(m, wo, wh); }
RD float MfPdf(const Microfacet& m, V3 wi, V3 wh) {
  float result = MfD(m, wh);
  if (m.visible) {
    result *= MfG1(m, wi, wh) * AbsDot(wi, wh) / wi.z;
  } else {
    result *= wh.z;
  }
  return result;
}
// math_ext.h:116-142 (the reference's own inverse-erf polynomial)
RD float ErfInvRef(float a) {
  float p;
  float t = logf(fmaxr(fmaf(a, -a, 1.f), 1.17549435e-38f));
  if (fabsf(t) > 6.125f) {
    p = 3.03697567e-10f;
    p = fmaf(p, t, 2.93243101e-8f);
    p = fmaf(p, t, 1.22150334e-6f);
    p = fmaf(p, t, 2.84108955e-5f);
    p = fmaf(p, t, 3.93552968e-4f);
    p = fmaf(p, t, 3.02698812e-3f);
    p = fmaf(p, t, 4.83185798e-3f);
    p = fmaf(p, t, -2.64646143e-1f);
    p = fmaf(p, t, 8.40016484e-1f);
  } else {
    p = 5.43877832e-9f;
    p = fmaf(p, t, 1.43286059e-7f);
    p = fmaf(p, t, 1.22775396e-6f);
    p = fmaf(p, t, 1.12962631e-7f);
    p = fmaf(p, t, -5.61531961e-5f);
    p = fmaf(p, t, -1.47697705e-4f);
    p = fmaf(p, t, 2.31468701e-3f);
    p = fmaf(p, t, 1.15392562e-2f);
    p = fmaf(p, t, -2.32015476e-1f);
    p = fmaf(p, t, 8.86226892e-1f);
  }
  return a * p;
}
// microfacet.cpp:208-243
RD V2 SampleVisibleGGX(float cosThetaI, V2 s) {
  if ((double)cosThetaI > 0.9999) {
    float r = sqrtf(s.x / (1.f - s.x));
    float phi = 6.28318530718f * s.y;
    return V2{r * cosf(phi), r * sinf(phi)};
  }
  float sinTheta = sqrtf(fmaxr(0.f, 1.f - Sqr(cosThetaI)));
  float tanTheta = sinTheta / cosThetaI;
  float a = 1.f / tanTheta;
  float G1 = 2.f / (1.f + sqrtf(1.f + 1.f / Sqr(a)));
  float A = 2.f * s.x / G1 - 1.f;
  float tmp = 1.f / fmaf(A, A, -1.f);
  if ((double)tmp > 1e10) tmp = 1e10f;
  float B = tanTheta;
  float D = sqrtf(fmaxr(Sqr(B) * Sqr(tmp) - (Sqr(A) - Sqr(B)) * tmp, 0.f));
  float slopeX1 = fmaf(B, tmp, -D);
  float slopeX2 = fmaf(B, tmp, D);
  float slopeX = (A < 0.f || slopeX2 > 1.f / tanTheta) ? slopeX1 : slopeX2;
  float S;
  float sy = s.y;
  if (sy > 0.5f) {
    S = 1.f;
    sy = 2.f * (sy - 0.5f);
  } else {
    S = -1.f;
    sy = 2.f * (0.5f - sy);
  }
  float z = (sy * (sy * (sy * 0.27385f - 0.73369f) + 0.46341f)) / (sy * (sy * (sy * 0.093073f + 0.309420f) - 1.f) + 0.597999f);
  float slopeY = S * z * sqrtf(1.f + slopeX * slopeX);
  return V2{slopeX, slopeY};
}
// microfacet.cpp:80-97
RD V2 SampleVisibleBeckmann(float cosThetaI, V2 s) {
  float tanThetaI = SafeSqrt(fmaf(-cosThetaI, cosThetaI, 1.f)) / cosThetaI;
  float cotThetaI = Rcp(tanThetaI);
  float maxval = erff(cotThetaI);
  s.x = fmaxr(fminr(s.x, (float)(1 - 1e-6)), (float)1e-6);
  s.y = fmaxr(fminr(s.y, (float)(1 - 1e-6)), (float)1e-6);
  float x = maxval - (maxval + 1.f) * erff(sqrtf(-logf(s.x)));
  s.x *= 1.f + maxval + (1.f / sqrtf(kPi)) * tanThetaI * expf(-Sqr(cotThetaI));
  for (int i = 0; i < 3; i++) {
    float slope = ErfInvRef(x);
    float value = 1.f + x + (1.f / sqrtf(kPi)) * tanThetaI * expf(-Sqr(slope)) - s.x;
    float derivative = 1.f - slope * tanThetaI;
    x -= value / derivative;
  }
  return V2{ErfInvRef(x), ErfInvRef(fmaf(2.f, s.y, -1.f))};
}
// microfacet.cpp:99-136 / 245-277
RD V3 MfSample(const Microfacet& m, V3 wi, V2 xi, float& pdf) {
  if (m.visible) {
    V3 wiP = normalized(V3{m.ax * wi.x, m.ay * wi.y, wi.z});
    float sinPhi, cosPhi;
    SinCosPhi(wiP, sinPhi, cosPhi);
    float cosTheta = wiP.z;
    V2 slope = m.ggx ? SampleVisibleGGX(cosTheta, xi) : SampleVisibleBeckmann(cosTheta, xi);
    V2 s2{fmaf(cosPhi, slope.x, -(sinPhi * slope.y)) * m.ax, fmaf(sinPhi, slope.x, cosPhi * slope.y) * m.ay};
    V3 mm = normalized(V3{-s2.x, -s2.y, 1.f});
    pdf = MfD(m, mm) * MfG1(m, wi, mm) * AbsDot(wi, mm) / wi.z;
    return mm;
  }
  float sinPhi, cosPhi, alpha2;
  if (m.ax == m.ay) {
    float a = (2.f * kPi) * xi.y;
    sinPhi = sinf(a);
    cosPhi = cosf(a);
    alpha2 = m.ax * m.ay;
  } else {
    float ratio = m.ay / m.ax;
    float tmp = ratio * tanf((2.f * kPi) * xi.y);
    cosPhi = Rsqrt(fmaf(tmp, tmp, 1.f));
    cosPhi = MulSign(cosPhi, fabsf(xi.y - 0.5f) - 0.25f);
    sinPhi = cosPhi * tmp;
    alpha2 = Rcp(Sqr(cosPhi / m.ax) + Sqr(sinPhi / m.ay));
  }
  float cosTheta;
  if (m.ggx) {
    float tanThetaM2 = alpha2 * xi.x / (1.f - xi.x);
    cosTheta = Rsqrt(1.f + tanThetaM2);
    float cos2Theta = Sqr(cosTheta);
    float temp = 1.f + tanThetaM2 / alpha2;
    float cos3Theta = fmaxr(cos2Theta * cosTheta, 1e-20f);
    pdf = Rcp(kPi * m.ax * m.ay * cos3Theta * Sqr(temp));
  } else {
    cosTheta = Rsqrt(fmaf(-alpha2, logf(1.f - xi.x), 1.f));
    float cos2Theta = Sqr(cosTheta);
    float cos3Theta = fmaxr(cos2Theta * cosTheta, 1e-20f);
    pdf = (1.f - xi.x) / (kPi * m.ax * m.ay * cos3Theta);
  }
  float sinTheta = sqrtf(1.f - Sqr(cosTheta));
  return V3{cosPhi * sinTheta, sinPhi * sinTheta, cosTheta};
}

}  // namespace rad
