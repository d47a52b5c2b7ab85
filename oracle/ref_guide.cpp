// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_core.h for the rules).
//
// CPU restatement of the learned path-guiding network of the GPU library. The
// reference has no path guiding, so this oracle is not a restatement of
// reference code: it is an independent implementation of the same
// specification, checked by finite differences (tests/test_guide_oracle.py).
//
// Network: 16-level hash grid (2 features per level) over the position mapped
// to [0,1]^3, then [grid features, normal, wo, 1, 0 x 9] (48 inputs) ->
// 64 -> 64 -> 64 (ReLU) -> 48 outputs (41 used: 8 lobes x (mu xyz, log kappa,
// logit) and the selection logit). Weights are [out][in].
//
// Two arithmetic modes:
//   exact = 0  mirrors the GPU's rounding points: table values, weights,
//              inputs and hidden activations are rounded to fp16 (round to
//              nearest even), sums are fp32, output gradients are clipped and
//              rounded to fp16, hidden-layer gradients are rounded to fp16.
//   exact = 1  double precision everywhere, no fp16 rounding (for finite
//              differences of the analytic gradient).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

constexpr int L = 16, NIN = 48, NH = 64, NOUT = 48, NLOBE = 8, NUSED = 41;
constexpr int OW0 = 0, OW1 = OW0 + NH * NIN, OW2 = OW1 + NH * NH, OW3 = OW2 + NH * NH, NW = OW3 + NOUT * NH;
constexpr double PI = 3.14159265358979323846;

// IEEE binary16 round to nearest even, returned as float.
float Half(float f) {
  if (!std::isfinite(f)) return f;
  float a = std::fabs(f);
  if (a >= 65520.f) return std::copysign(INFINITY, f);
  float q;
  if (a < 6.103515625e-05f) {
    q = std::nearbyint(a * 16777216.f) / 16777216.f;
  } else {
    int e;
    std::frexp(a, &e);  // a = m 2^e, m in [0.5, 1)
    float quantum = std::ldexp(1.f, e - 11);
    q = std::nearbyint(a / quantum) * quantum;
  }
  return std::copysign(q, f);
}

struct Cfg {
  uint32_t log2T;
  uint32_t res[L];
  float lo[3], inv[3];
  float logKMax;  // kappa <= exp(logKMax)
  float cMax;     // c = cMax sigmoid(o - 2)
};

uint32_t GridIndex(uint32_t x, uint32_t y, uint32_t z, uint32_t res, uint32_t log2T) {
  uint64_t s = (uint64_t)res + 1;
  if (s * s * s <= (1ull << log2T)) return (uint32_t)(x + s * (y + s * z));
  return (x ^ (y * 2654435761u) ^ (z * 805459861u)) & ((1u << log2T) - 1u);
}

// Corner entries and trilinear weights of one level (fp32, as the device).
void Corners(const Cfg& c, const float u[3], int l, uint32_t idx[8], float w[8]) {
  uint32_t res = c.res[l];
  uint32_t cell[3];
  float t[3];
  for (int a = 0; a < 3; a++) {
    float f = u[a] * (float)res;
    float fl = std::floor(f);
    if (fl < 0.f) fl = 0.f;
    if (fl > (float)(res - 1)) fl = (float)(res - 1);
    cell[a] = (uint32_t)fl;
    t[a] = f - fl;
  }
  for (int k = 0; k < 8; k++) {
    uint32_t bx = k & 1, by = (k >> 1) & 1, bz = (k >> 2) & 1;
    w[k] = (bx ? t[0] : 1.f - t[0]) * (by ? t[1] : 1.f - t[1]) * (bz ? t[2] : 1.f - t[2]);
    idx[k] = GridIndex(cell[0] + bx, cell[1] + by, cell[2] + bz, res, c.log2T);
  }
}

void Unit(const Cfg& c, const float* P, float u[3]) {
  for (int a = 0; a < 3; a++) {
    float v = (P[a] - c.lo[a]) * c.inv[a];
    u[a] = v < 0.f ? 0.f : (v > 1.f ? 1.f : v);
  }
}

template <typename T>
struct Net {
  const Cfg& c;
  const float* p;  // parameters (table, weights)
  bool exact;
  uint64_t nTable;
  T R(T v) const { return exact ? v : (T)Half((float)v); }
  T Tab(uint64_t i) const { return exact ? (T)p[i] : (T)Half(p[i]); }
  T Wt(int i) const { return exact ? (T)p[nTable + i] : (T)Half(p[nTable + i]); }

  void Input(const float* q, T x[NIN]) const {
    float u[3];
    Unit(c, q, u);
    for (int l = 0; l < L; l++) {
      uint32_t idx[8];
      float w[8];
      Corners(c, u, l, idx, w);
      T f0 = 0, f1 = 0;
      uint64_t base = ((uint64_t)l << c.log2T) * 2;
      for (int k = 0; k < 8; k++) {
        f0 += (T)w[k] * Tab(base + 2 * (uint64_t)idx[k]);
        f1 += (T)w[k] * Tab(base + 2 * (uint64_t)idx[k] + 1);
      }
      x[2 * l] = R(f0);
      x[2 * l + 1] = R(f1);
    }
    for (int a = 0; a < 3; a++) {
      x[32 + a] = R((T)q[3 + a]);
      x[35 + a] = R((T)q[6 + a]);
    }
    x[38] = 1;
    for (int k = 39; k < NIN; k++) x[k] = 0;
  }

  // y[n] = sum_k W[n][k] x[k]
  void Layer(int off, int nin, int nout, const T* x, T* y) const {
    for (int n = 0; n < nout; n++) {
      T s = 0;
      for (int k = 0; k < nin; k++) s += Wt(off + n * nin + k) * x[k];
      y[n] = s;
    }
  }

  void Forward(const float* q, T x[NIN], T h1[NH], T h2[NH], T h3[NH], T o[NOUT]) const {
    Input(q, x);
    Layer(OW0, NIN, NH, x, h1);
    for (int i = 0; i < NH; i++) h1[i] = R(h1[i] > 0 ? h1[i] : 0);
    Layer(OW1, NH, NH, h1, h2);
    for (int i = 0; i < NH; i++) h2[i] = R(h2[i] > 0 ? h2[i] : 0);
    Layer(OW2, NH, NH, h2, h3);
    for (int i = 0; i < NH; i++) h3[i] = R(h3[i] > 0 ? h3[i] : 0);
    Layer(OW3, NH, NOUT, h3, o);
  }
};

template <typename T>
struct Mixture {
  T mu[NLOBE][3], len[NLOBE], kappa[NLOBE], pi[NLOBE], c, sig;
  bool kin[NLOBE];
};

template <typename T>
void MakeMixture(const T* o, T logKMax, T cMax, Mixture<T>& m) {
  T zmax = o[4];
  for (int k = 1; k < NLOBE; k++) zmax = std::max(zmax, o[5 * k + 4]);
  T s = 0;
  for (int k = 0; k < NLOBE; k++) s += (m.pi[k] = std::exp(o[5 * k + 4] - zmax));
  for (int k = 0; k < NLOBE; k++) {
    m.pi[k] /= s;
    T v[3] = {o[5 * k], o[5 * k + 1], o[5 * k + 2]};
    T len = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    m.len[k] = len;
    for (int a = 0; a < 3; a++) m.mu[k][a] = len > (T)1e-6 ? v[a] / len : (a == 2 ? (T)1 : (T)0);
    T a = o[5 * k + 3];
    m.kin[k] = a > (T)-6 && a < logKMax;
    T ac = a < (T)-6 ? (T)-6 : (a > logKMax ? logKMax : a);
    m.kappa[k] = std::exp(ac);
  }
  m.sig = (T)1 / ((T)1 + std::exp(-(o[40] - (T)2)));
  m.c = cMax * m.sig;
}

template <typename T>
T Vmf(const T mu[3], T kappa, const T w[3]) {
  T d = mu[0] * w[0] + mu[1] * w[1] + mu[2] * w[2];
  return kappa / ((T)(2 * PI) * -std::expm1((T)-2 * kappa)) * std::exp(kappa * (d - 1));
}

template <typename T>
T MeanCos(T k) {  // Langevin function
  if (k < (T)0.05) return k / 3 - k * k * k / 45;
  return (T)1 / std::tanh(k) - (T)1 / k;
}

// loss = -w log(c q + (1 - c) b) and its gradient dO with respect to the raw outputs.
template <typename T>
T LossGrad(const T* o, const T wi[3], T b, T w, T logKMax, T cMax, T dO[NOUT]) {
  for (int i = 0; i < NOUT; i++) dO[i] = 0;
  Mixture<T> m;
  MakeMixture(o, logKMax, cMax, m);
  T v[NLOBE], q = 0;
  for (int k = 0; k < NLOBE; k++) q += m.pi[k] * (v[k] = Vmf(m.mu[k], m.kappa[k], wi));
  T p = m.c * q + (1 - m.c) * b;
  if (!(p > 0) || !(w > 0)) return 0;
  T gp = -w / p;
  dO[40] = gp * (q - b) * cMax * m.sig * (1 - m.sig);
  T gq = gp * m.c;
  for (int k = 0; k < NLOBE; k++) {
    T d = m.mu[k][0] * wi[0] + m.mu[k][1] * wi[1] + m.mu[k][2] * wi[2];
    T gv = gq * m.pi[k] * v[k];
    dO[5 * k + 4] = gq * m.pi[k] * (v[k] - q);
    dO[5 * k + 3] = m.kin[k] ? gv * (d - MeanCos(m.kappa[k])) * m.kappa[k] : (T)0;
    if (m.len[k] > (T)1e-6)
      for (int a = 0; a < 3; a++) dO[5 * k + a] = gv * m.kappa[k] * (wi[a] - d * m.mu[k][a]) / m.len[k];
  }
  for (int i = 0; i < NUSED; i++) dO[i] = dO[i] < (T)-1024 ? (T)-1024 : (dO[i] > (T)1024 ? (T)1024 : dO[i]);
  return -w * std::log(p);
}

template <typename T>
void Forward(const Cfg& c, const float* params, const float* q, int64_t n, float* raw, float* mix, bool exact) {
  const T logKMax = (T)c.logKMax, cMax = (T)c.cMax;
  Net<T> net{c, params, exact, (uint64_t)L * (1ull << c.log2T) * 2};
  std::vector<T> x(NIN), h1(NH), h2(NH), h3(NH), o(NOUT);
  for (int64_t i = 0; i < n; i++) {
    net.Forward(q + 9 * i, x.data(), h1.data(), h2.data(), h3.data(), o.data());
    if (raw)
      for (int k = 0; k < NOUT; k++) raw[i * NOUT + k] = k < NUSED ? (float)o[k] : 0.f;
    if (mix) {
      Mixture<T> m;
      MakeMixture(o.data(), logKMax, cMax, m);
      float* out = mix + 44 * i;
      for (int k = 0; k < NLOBE; k++) {
        for (int a = 0; a < 3; a++) out[4 * k + a] = (float)m.mu[k][a];
        out[4 * k + 3] = (float)m.kappa[k];
        out[32 + k] = (float)m.pi[k];
      }
      out[40] = (float)m.c;
      out[41] = out[42] = out[43] = 0.f;
    }
  }
}

template <typename T>
double Grad(const Cfg& c, const float* params, const float* recs, int64_t n, double* grad, bool exact) {
  uint64_t nTable = (uint64_t)L * (1ull << c.log2T) * 2;
  Net<T> net{c, params, exact, nTable};
  const T logKMax = (T)c.logKMax, cMax = (T)c.cMax;
  double lossSum = 0;
  std::vector<T> x(NIN), h1(NH), h2(NH), h3(NH), o(NOUT), d3(NH), d2(NH), d1(NH), dOut(NOUT);
  for (int64_t i = 0; i < n; i++) {
    const float* r = recs + 16 * i;
    float q[9] = {r[0], r[1], r[2], r[4], r[5], r[6], r[8], r[9], r[10]};
    T wi[3] = {(T)r[12], (T)r[13], (T)r[14]};
    T b = (T)r[3], w = (T)r[15];
    if (!(w > 0)) continue;
    net.Forward(q, x.data(), h1.data(), h2.data(), h3.data(), o.data());
    T ol[NOUT];
    for (int k = 0; k < NOUT; k++) ol[k] = k < NUSED ? o[k] : (T)0;
    lossSum += (double)LossGrad(ol, wi, b, w, logKMax, cMax, dOut.data());
    for (int k = 0; k < NOUT; k++) dOut[k] = net.R(dOut[k]);
    // layer 3
    for (int nn = 0; nn < NOUT; nn++)
      for (int k = 0; k < NH; k++) grad[nTable + OW3 + nn * NH + k] += (double)(dOut[nn] * h3[k]);
    for (int k = 0; k < NH; k++) {
      T s = 0;
      for (int nn = 0; nn < NOUT; nn++) s += dOut[nn] * net.Wt(OW3 + nn * NH + k);
      d3[k] = net.R(h3[k] > 0 ? s : (T)0);
    }
    // layer 2
    for (int nn = 0; nn < NH; nn++)
      for (int k = 0; k < NH; k++) grad[nTable + OW2 + nn * NH + k] += (double)(d3[nn] * h2[k]);
    for (int k = 0; k < NH; k++) {
      T s = 0;
      for (int nn = 0; nn < NH; nn++) s += d3[nn] * net.Wt(OW2 + nn * NH + k);
      d2[k] = net.R(h2[k] > 0 ? s : (T)0);
    }
    // layer 1
    for (int nn = 0; nn < NH; nn++)
      for (int k = 0; k < NH; k++) grad[nTable + OW1 + nn * NH + k] += (double)(d2[nn] * h1[k]);
    for (int k = 0; k < NH; k++) {
      T s = 0;
      for (int nn = 0; nn < NH; nn++) s += d2[nn] * net.Wt(OW1 + nn * NH + k);
      d1[k] = net.R(h1[k] > 0 ? s : (T)0);
    }
    // layer 0 and the grid features
    for (int nn = 0; nn < NH; nn++)
      for (int k = 0; k < NIN; k++) grad[nTable + OW0 + nn * NIN + k] += (double)(d1[nn] * x[k]);
    float u[3];
    Unit(c, q, u);
    for (int l = 0; l < L; l++) {
      T g[2];
      for (int f = 0; f < 2; f++) {
        T s = 0;
        for (int nn = 0; nn < NH; nn++) s += d1[nn] * net.Wt(OW0 + nn * NIN + 2 * l + f);
        g[f] = s;
      }
      uint32_t idx[8];
      float wc[8];
      Corners(c, u, l, idx, wc);
      uint64_t base = ((uint64_t)l << c.log2T) * 2;
      for (int k = 0; k < 8; k++)
        for (int f = 0; f < 2; f++) grad[base + 2 * (uint64_t)idx[k] + f] += (double)((T)wc[k] * g[f]);
    }
  }
  return lossSum;
}

Cfg MakeCfg(uint32_t log2T, const uint32_t* res, const float* lo, const float* inv, float logKMax, float cMax) {
  Cfg c{};
  c.logKMax = logKMax;
  c.cMax = cMax;
  c.log2T = log2T;
  for (int l = 0; l < L; l++) c.res[l] = res[l];
  for (int a = 0; a < 3; a++) {
    c.lo[a] = lo[a];
    c.inv[a] = inv[a];
  }
  return c;
}

}  // namespace

extern "C" {

// Level resolutions floor(minRes b^l), b = (maxRes / minRes)^(1/15), in double.
void orc_guide_level_res(uint32_t minRes, uint32_t maxRes, uint32_t* res) {
  double b = std::exp((std::log((double)maxRes) - std::log((double)minRes)) / (L - 1));
  for (int l = 0; l < L; l++) {
    double r = std::floor((double)minRes * std::pow(b, (double)l));
    res[l] = r < 1.0 ? 1u : (uint32_t)r;
  }
}

// queries n x 9 (P, N, wo); raw n x 48 and mix n x 44 optional.
int orc_guide_forward(uint32_t log2T, const uint32_t* res, const float* lo, const float* inv, float logKMax,
                      float cMax, const float* params, const float* queries, int64_t n, float* raw, float* mix,
                      int exact) {
  Cfg c = MakeCfg(log2T, res, lo, inv, logKMax, cMax);
  if (exact)
    Forward<double>(c, params, queries, n, raw, mix, true);
  else
    Forward<float>(c, params, queries, n, raw, mix, false);
  return 0;
}

// records n x 16 (P, b | N, - | wo, - | wi, w); grad (n_params doubles) is
// accumulated into; returns the summed loss.
double orc_guide_grad(uint32_t log2T, const uint32_t* res, const float* lo, const float* inv, float logKMax,
                      float cMax, const float* params, const float* records, int64_t n, double* grad, int exact) {
  Cfg c = MakeCfg(log2T, res, lo, inv, logKMax, cMax);
  if (exact) return Grad<double>(c, params, records, n, grad, true);
  return Grad<float>(c, params, records, n, grad, false);
}

// Mixture pdf of packed mixtures (n x 44) at dirs (n x 3), double precision.
void orc_guide_mix_pdf(const float* mix, const float* dirs, int64_t n, double* pdf) {
  for (int64_t i = 0; i < n; i++) {
    const float* m = mix + 44 * i;
    double w[3] = {dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]};
    double q = 0;
    for (int k = 0; k < NLOBE; k++) {
      double mu[3] = {m[4 * k], m[4 * k + 1], m[4 * k + 2]};
      q += (double)m[32 + k] * Vmf<double>(mu, (double)m[4 * k + 3], w);
    }
    pdf[i] = q;
  }
}

float orc_half_round(float f) { return Half(f); }

}  // extern "C"
