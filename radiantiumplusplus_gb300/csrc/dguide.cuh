// Learned path guiding. The reference has no counterpart: its integrators
// sample directions from the BSDF only (path.cpp:189-205). Here a guide network
//   multiresolution hash grid over the shading position (16 levels x 2 fp16
//   features, 2^log2T entries per level) ++ shading normal ++ outgoing
//   direction ++ 1  ->  3 hidden layers of 64 (ReLU, fp16 weights and
//   activations, fp32 accumulation on the tensor cores)  ->  41 outputs
// parameterises an 8-lobe von Mises-Fisher mixture q over world directions and
// the probability c of sampling it instead of the BSDF. Shading draws from the
// one-sample MIS density
//   p(wi) = c q(wi) + (1 - c) p_bsdf(wi),
// so the estimator is unbiased for every network state, and BSDF sampling stays
// the fallback (c <= cMax < 1). Training minimises the KL divergence from the
// product f cos Li to p, with the tracer's own radiance estimates as weights.
#pragma once
#include <cuda_fp16.h>

#include "dmath.cuh"

namespace rad {

constexpr int kGLevels = 16;
constexpr int kGFeat = 2;
constexpr int kGIn = 48;    // 32 grid features, normal xyz, wo xyz, 1, 9 zeros
constexpr int kGHid = 64;
constexpr int kGOut = 48;   // 8 x (mu xyz, log kappa, logit), selection logit, 7 unused
constexpr int kGLobes = 8;
constexpr int kGOutUsed = 5 * kGLobes + 1;
constexpr int kGMixF4 = 11;  // per path slot: 8 x (mu, kappa), pi[0..3], pi[4..7], (c, 0, 0, 0)
constexpr int kGRecF4 = 6;   // training record, see GuideRecord
// MLP weights follow the hash table in the parameter vector; each matrix is
// stored [out][in] (row-major by output).
constexpr int kGW0 = 0;
constexpr int kGW1 = kGW0 + kGHid * kGIn;
constexpr int kGW2 = kGW1 + kGHid * kGHid;
constexpr int kGW3 = kGW2 + kGHid * kGHid;
constexpr int kGWCount = kGW3 + kGOut * kGHid;  // 14336
constexpr float kGLogKMin = -6.f;   // kappa >= exp(-6); the upper bound is a setting (logKMax)
constexpr float kGCBias = 2.f;      // c = cMax * sigmoid(o - kGCBias); cMax is a setting (<= 0.95)
constexpr float kGGradClamp = 1024.f;  // per-output gradient clip before fp16

// Device view of a guide network and its per-wave buffers.
struct GuideDev {
  const __half* table;    // fp16 copy, [level][entry][feature]
  const __half* weights;  // fp16 copy of the MLP weights (kGWCount)
  uint32_t log2T;
  uint32_t res[kGLevels];  // grid resolution per level
  float lo[3], inv[3];     // world position -> [0,1]^3
  float4* mix;             // kGMixF4 per path slot
  float4* rec;             // training records, kGRecF4 each
  uint32_t* ctl;           // [0] records appended, [1] float bits: sum of weights, [2] loss sum bits
  uint32_t recCap;
  uint32_t train;          // append training records in this wave
  uint32_t trainSalt;      // per-wave salt of the training-path selection hash
  uint32_t trainShift;     // a path trains when Hash(path slot ^ salt) >> (32 - shift) == 0
  uint32_t trainDepth;     // only vertices with depth < trainDepth train
  unsigned long long* recTotal;  // optional job counter of training records
  float logKMax;           // kappa <= exp(logKMax)
  float cMax;              // c <= cMax: 1 - cMax of the samples always come from the BSDF
};

// Training record (kGRecF4 float4), appended at a guided vertex:
//  r0 (P, p_bsdf(wi))  r1 (shading N, path slot bits)  r2 (wo world, p_mix(wi))
//  r3 (wi world, weight)  r4 (radiance of the path before this vertex's NEE)
//  r5 (throughput before this vertex)
// The shadow stage adds this vertex's unoccluded NEE into r4; the finalize
// stage sets weight = lum((L_final - r4) / r5) = lum(f cos Li) / p_mix(wi).

__host__ __device__ inline uint32_t GuideHash32(uint32_t x) {  // Wang-style integer mix
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

// Entry of grid vertex (x, y, z) at a level of resolution `res`: dense
// indexing while (res + 1)^3 fits the table, else the spatial hash of
// Teschner et al. 2003 (primes 1, 2654435761, 805459861) modulo 2^log2T.
RD uint32_t GuideGridIndex(uint32_t x, uint32_t y, uint32_t z, uint32_t res, uint32_t log2T) {
  uint64_t s = (uint64_t)res + 1u;
  if (s * s * s <= (1ull << log2T)) return (uint32_t)(x + s * (y + s * z));
  return (x ^ (y * 2654435761u) ^ (z * 805459861u)) & ((1u << log2T) - 1u);
}

// Cell and trilinear fractions of u in [0,1] at resolution res.
RD void GuideCell(float u, uint32_t res, uint32_t& c0, float& t) {
  float f = u * (float)res;
  float fl = floorf(f);
  if (fl < 0.f) fl = 0.f;
  if (fl > (float)(res - 1u)) fl = (float)(res - 1u);
  c0 = (uint32_t)fl;
  t = f - fl;
}

RD float GuideSigmoid(float x) { return 1.f / (1.f + expf(-x)); }

// vMF normalisation kappa / (2 pi (1 - exp(-2 kappa))).
RD float VmfNorm(float kappa) { return kappa / (2.f * kPi * (-expm1f(-2.f * kappa))); }
RD float VmfPdf(V3 mu, float kappa, V3 w) { return VmfNorm(kappa) * expf(kappa * (dot(mu, w) - 1.f)); }
// Langevin function coth(k) - 1/k = mean cosine of a vMF lobe.
RD float Langevin(float k) {
  if (k < 0.05f) return k * (1.f / 3.f) - k * k * k * (1.f / 45.f);
  return 1.f / tanhf(k) - 1.f / k;
}

// Raw network outputs -> mixture parameters.
struct GuideMix {
  V3 mu[kGLobes];
  float kappa[kGLobes], pi[kGLobes];
  float c;
};
RD void GuideMixFromRaw(const float* o, float logKMax, float cMax, GuideMix& m) {
  float zmax = o[4];
  for (int k = 1; k < kGLobes; k++) zmax = fmaxf(zmax, o[5 * k + 4]);
  float s = 0.f;
  for (int k = 0; k < kGLobes; k++) {
    m.pi[k] = expf(o[5 * k + 4] - zmax);
    s += m.pi[k];
  }
  for (int k = 0; k < kGLobes; k++) {
    m.pi[k] = m.pi[k] / s;
    V3 v{o[5 * k], o[5 * k + 1], o[5 * k + 2]};
    float len = sqrtf(dot(v, v));
    m.mu[k] = len > 1e-6f ? v / len : V3{0.f, 0.f, 1.f};
    m.kappa[k] = expf(clampr(o[5 * k + 3], kGLogKMin, logKMax));
  }
  m.c = cMax * GuideSigmoid(o[40] - kGCBias);
}

RD float GuideMixPdf(const GuideMix& m, V3 w) {
  float q = 0.f;
  for (int k = 0; k < kGLobes; k++) q += m.pi[k] * VmfPdf(m.mu[k], m.kappa[k], w);
  return q;
}

// Mixture pdf from the packed per-slot form (kGMixF4 float4).
RD float GuideMixPdfPacked(const float4* mx, V3 w) {
  float4 pa = mx[8], pb = mx[9];
  float pi[8] = {pa.x, pa.y, pa.z, pa.w, pb.x, pb.y, pb.z, pb.w};
  float q = 0.f;
  for (int k = 0; k < kGLobes; k++) {
    float4 l = mx[k];
    q += pi[k] * VmfPdf(V3{l.x, l.y, l.z}, l.w, w);
  }
  return q;
}

// Samples a vMF lobe around mu (Jakob 2012, "Numerically stable sampling of
// the von Mises-Fisher distribution on S^2"): cos = 1 + log(1 + (1 - u1)
// expm1(-2 kappa)) / kappa, azimuth 2 pi u2, in a frame around mu.
RD V3 VmfSample(V3 mu, float kappa, V2 u) {
  float ct = 1.f + log1pf((1.f - u.x) * expm1f(-2.f * kappa)) / kappa;
  ct = clampr(ct, -1.f, 1.f);
  float st = sqrtf(fmaxf(0.f, 1.f - ct * ct));
  float phi = 2.f * kPi * u.y;
  Frame f = FrameFromN(mu);
  return ToWorld(f, V3{st * cosf(phi), st * sinf(phi), ct});
}

// Lobe chosen by ul against the cumulative weights, direction from u.
RD V3 GuideMixSamplePacked(const float4* mx, float ul, V2 u) {
  float4 pa = mx[8], pb = mx[9];
  float pi[8] = {pa.x, pa.y, pa.z, pa.w, pb.x, pb.y, pb.z, pb.w};
  int k = 0;
  float acc = pi[0];
  while (k < kGLobes - 1 && ul >= acc) {
    k++;
    acc += pi[k];
  }
  float4 l = mx[k];
  return VmfSample(V3{l.x, l.y, l.z}, l.w, u);
}

// Loss -w log p(wi) of one record and its gradient with respect to the raw
// outputs o (dO[0..47]; unused outputs get 0). b = p_bsdf(wi). Returns the loss.
//   p = c q + (1 - c) b,  q = sum_k pi_k v_k,  v_k = vMF(wi; mu_k, kappa_k)
//   dL/dc = -w/p (q - b),  dL/dz_k = -w c/p pi_k (v_k - q)        (softmax)
//   dL/da_k = -w c/p pi_k v_k (mu_k.wi - Langevin(kappa_k)) kappa_k (a = log kappa)
//   dL/dm_k = -w c/p pi_k v_k kappa_k (wi - (mu_k.wi) mu_k) / |m_k|
RD float GuideLossGrad(const float* o, V3 wi, float b, float w, float logKMax, float cMax, float* dO) {
  for (int i = 0; i < kGOut; i++) dO[i] = 0.f;
  float zmax = o[4];
  for (int k = 1; k < kGLobes; k++) zmax = fmaxf(zmax, o[5 * k + 4]);
  float pi[kGLobes], v[kGLobes], s = 0.f;
  for (int k = 0; k < kGLobes; k++) {
    pi[k] = expf(o[5 * k + 4] - zmax);
    s += pi[k];
  }
  float q = 0.f;
  for (int k = 0; k < kGLobes; k++) {
    pi[k] = pi[k] / s;
    V3 m{o[5 * k], o[5 * k + 1], o[5 * k + 2]};
    float len = sqrtf(dot(m, m));
    V3 mu = len > 1e-6f ? m / len : V3{0.f, 0.f, 1.f};
    float kap = expf(clampr(o[5 * k + 3], kGLogKMin, logKMax));
    v[k] = VmfPdf(mu, kap, wi);
    q += pi[k] * v[k];
  }
  float sg = GuideSigmoid(o[40] - kGCBias);
  float c = cMax * sg;
  float p = c * q + (1.f - c) * b;
  if (!(p > 0.f) || !(w > 0.f)) return 0.f;
  float gp = -w / p;
  dO[40] = gp * (q - b) * cMax * sg * (1.f - sg);
  float gq = gp * c;
  for (int k = 0; k < kGLobes; k++) {
    V3 m{o[5 * k], o[5 * k + 1], o[5 * k + 2]};
    float len = sqrtf(dot(m, m));
    V3 mu = len > 1e-6f ? m / len : V3{0.f, 0.f, 1.f};
    float a = o[5 * k + 3];
    float kap = expf(clampr(a, kGLogKMin, logKMax));
    float d = dot(mu, wi);
    float gv = gq * pi[k] * v[k];
    dO[5 * k + 4] = gq * pi[k] * (v[k] - q);
    dO[5 * k + 3] = (a > kGLogKMin && a < logKMax) ? gv * (d - Langevin(kap)) * kap : 0.f;
    if (len > 1e-6f) {
      V3 g = (wi - mu * d) * (gv * kap / len);
      dO[5 * k] = g.x;
      dO[5 * k + 1] = g.y;
      dO[5 * k + 2] = g.z;
    }
  }
  for (int i = 0; i < kGOutUsed; i++) dO[i] = clampr(dO[i], -kGGradClamp, kGGradClamp);
  return -w * logf(p);
}

}  // namespace rad
