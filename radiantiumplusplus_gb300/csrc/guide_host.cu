// Guide network state on the host side: allocation, seeded initialisation,
// checkpoints and configuration (dguide.cuh describes the method).
#include <cmath>
#include <cstring>
#include <stdexcept>

#include "guide_net.h"
#include "host_json.h"
#include "kernels.h"

namespace rad {

namespace {
void CheckG(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}
uint64_t Mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
float Uniform(uint64_t seed, uint64_t i) {  // [-1, 1)
  return (float)((Mix64(seed * 0x100000001b3ull + i) >> 40) * (1.0 / 8388608.0) - 1.0);
}
}  // namespace

void GuideLevelRes(uint32_t minRes, uint32_t maxRes, uint32_t res[kGLevels]) {
  double b = std::exp((std::log((double)maxRes) - std::log((double)minRes)) / (kGLevels - 1));
  for (int l = 0; l < kGLevels; l++) {
    double r = std::floor((double)minRes * std::pow(b, (double)l));
    res[l] = r < 1.0 ? 1u : (uint32_t)r;
  }
}

static GuideNet* Alloc(const GuideConfig& cfg, const float lo[3], const float hi[3]) {
  if (cfg.log2T < 8 || cfg.log2T > 24) throw std::runtime_error("guide log2_table must be in [8, 24]");
  if (cfg.minRes < 1 || cfg.maxRes < cfg.minRes) throw std::runtime_error("guide resolutions invalid");
  GuideNet* n = new GuideNet();
  n->cfg = cfg;
  n->nTable = (uint64_t)kGLevels * (1ull << cfg.log2T) * kGFeat;
  n->nParams = n->nTable + kGWCount;
  GuideLevelRes(cfg.minRes, cfg.maxRes, n->res);
  for (int a = 0; a < 3; a++) {
    n->lo[a] = lo[a];
    n->hi[a] = hi[a];
  }
  size_t fb = n->nParams * sizeof(float);
  try {
    CheckG(cudaMalloc(&n->p, fb), "guide params");
    CheckG(cudaMalloc(&n->m, fb), "guide moments");
    CheckG(cudaMalloc(&n->v, fb), "guide moments");
    CheckG(cudaMalloc(&n->g, fb), "guide gradients");
    CheckG(cudaMalloc(&n->ph, n->nParams * sizeof(__half)), "guide fp16 params");
    CheckG(cudaMalloc(&n->ctl, 4 * sizeof(uint32_t)), "guide control");
  } catch (...) {
    GuideDestroy(n);
    throw;
  }
  n->bytes = 4 * fb + n->nParams * sizeof(__half) + 16;
  return n;
}

GuideNet* GuideCreate(const GuideConfig& cfg, const float lo[3], const float hi[3]) {
  GuideNet* n = Alloc(cfg, lo, hi);
  std::vector<float> h(n->nParams);
  for (uint64_t i = 0; i < n->nTable; i++) h[i] = 1e-4f * Uniform(cfg.seed, i);
  float* w = h.data() + n->nTable;
  const float s0 = std::sqrt(6.f / kGIn), s1 = std::sqrt(6.f / kGHid), s3 = 0.1f * std::sqrt(6.f / kGHid);
  for (int i = 0; i < kGWCount; i++) {
    float s = i < kGW1 ? s0 : (i < kGW3 ? s1 : s3);
    w[i] = s * Uniform(cfg.seed + 1u, (uint64_t)i);
  }
  // unused output rows stay zero (their gradients are zero too)
  for (int o = kGOutUsed; o < kGOut; o++)
    for (int k = 0; k < kGHid; k++) w[kGW3 + o * kGHid + k] = 0.f;
  try {
    size_t fb = n->nParams * sizeof(float);
    CheckG(cudaMemcpy(n->p, h.data(), fb, cudaMemcpyHostToDevice), "guide upload");
    CheckG(cudaMemset(n->m, 0, fb), "memset");
    CheckG(cudaMemset(n->v, 0, fb), "memset");
    CheckG(cudaMemset(n->g, 0, fb), "memset");
    CheckG(cudaMemset(n->ctl, 0, 16), "memset");
    CheckG(LaunchFloatToHalf(n->p, n->ph, n->nParams, 0), "fp16 copy");
    CheckG(cudaDeviceSynchronize(), "sync");
  } catch (...) {
    GuideDestroy(n);
    throw;
  }
  return n;
}

void GuideDestroy(GuideNet* n) {
  if (!n) return;
  cudaFree(n->p);
  cudaFree(n->m);
  cudaFree(n->v);
  cudaFree(n->g);
  cudaFree(n->ph);
  cudaFree(n->ctl);
  delete n;
}

GuideDev GuideView(const GuideNet& n) {
  GuideDev G{};
  G.table = n.ph;
  G.weights = n.ph + n.nTable;
  G.log2T = n.cfg.log2T;
  for (int l = 0; l < kGLevels; l++) G.res[l] = n.res[l];
  for (int a = 0; a < 3; a++) {
    G.lo[a] = n.lo[a];
    float e = n.hi[a] - n.lo[a];
    G.inv[a] = e > 1e-6f ? 1.f / e : 1.f;
  }
  G.ctl = n.ctl;
  G.trainShift = n.cfg.trainShift;
  G.trainDepth = n.cfg.trainDepth;
  G.logKMax = n.cfg.logKappaMax;
  G.cMax = n.cfg.cMax;
  return G;
}

size_t GuideCheckpointBytes(const GuideNet& n) { return 128 + 3 * n.nParams * sizeof(float); }

void GuideCheckpoint(const GuideNet& n, void* buf, cudaStream_t st) {
  uint32_t hd[32] = {};
  std::memcpy(hd, "RADGUID1", 8);
  hd[2] = 1;
  hd[3] = n.cfg.log2T;
  hd[4] = kGLevels;
  hd[5] = n.cfg.minRes;
  hd[6] = n.cfg.maxRes;
  hd[7] = n.step;
  hd[8] = (uint32_t)n.nParams;
  hd[9] = (uint32_t)(n.nParams >> 32);
  std::memcpy(hd + 10, n.lo, 12);
  std::memcpy(hd + 13, n.hi, 12);
  std::memcpy(hd + 16, n.res, 64);
  unsigned char* b = static_cast<unsigned char*>(buf);
  std::memcpy(b, hd, 128);
  size_t fb = n.nParams * sizeof(float);
  CheckG(cudaMemcpyAsync(b + 128, n.p, fb, cudaMemcpyDeviceToHost, st), "checkpoint copy");
  CheckG(cudaMemcpyAsync(b + 128 + fb, n.m, fb, cudaMemcpyDeviceToHost, st), "checkpoint copy");
  CheckG(cudaMemcpyAsync(b + 128 + 2 * fb, n.v, fb, cudaMemcpyDeviceToHost, st), "checkpoint copy");
  CheckG(cudaStreamSynchronize(st), "sync");
}

GuideNet* GuideFromCheckpoint(const void* buf, size_t size, const GuideConfig& base, cudaStream_t st) {
  if (!buf || size < 128) throw std::runtime_error("guide checkpoint too small");
  uint32_t hd[32];
  std::memcpy(hd, buf, 128);
  if (std::memcmp(hd, "RADGUID1", 8) != 0 || hd[2] != 1 || hd[4] != (uint32_t)kGLevels)
    throw std::runtime_error("not a version-1 guide checkpoint");
  GuideConfig cfg = base;
  cfg.log2T = hd[3];
  cfg.minRes = hd[5];
  cfg.maxRes = hd[6];
  float lo[3], hi[3];
  std::memcpy(lo, hd + 10, 12);
  std::memcpy(hi, hd + 13, 12);
  uint64_t np = (uint64_t)hd[8] | ((uint64_t)hd[9] << 32);
  if (cfg.log2T < 8 || cfg.log2T > 24) throw std::runtime_error("guide checkpoint: bad table size");
  uint64_t expect = (uint64_t)kGLevels * (1ull << cfg.log2T) * kGFeat + kGWCount;
  if (np != expect) throw std::runtime_error("guide checkpoint: parameter count does not match its table size");
  if (size < 128 + 3 * np * sizeof(float)) throw std::runtime_error("guide checkpoint truncated");
  GuideNet* n = Alloc(cfg, lo, hi);
  try {
    n->step = hd[7];
    const unsigned char* b = static_cast<const unsigned char*>(buf);
    size_t fb = np * sizeof(float);
    CheckG(cudaMemcpyAsync(n->p, b + 128, fb, cudaMemcpyHostToDevice, st), "checkpoint upload");
    CheckG(cudaMemcpyAsync(n->m, b + 128 + fb, fb, cudaMemcpyHostToDevice, st), "checkpoint upload");
    CheckG(cudaMemcpyAsync(n->v, b + 128 + 2 * fb, fb, cudaMemcpyHostToDevice, st), "checkpoint upload");
    CheckG(cudaMemsetAsync(n->g, 0, fb, st), "memset");
    CheckG(cudaMemsetAsync(n->ctl, 0, 16, st), "memset");
    CheckG(LaunchFloatToHalf(n->p, n->ph, np, st), "fp16 copy");
    CheckG(cudaStreamSynchronize(st), "sync");
  } catch (...) {
    GuideDestroy(n);
    throw;
  }
  return n;
}

void GuideParseConfig(const char* json, GuideConfig& c) {
  if (!json || !*json) return;
  JValue j = JsonReader::Parse(json);
  auto u = [&](const char* k, uint32_t& dst) {
    if (const JValue* v = j.get(k)) dst = (uint32_t)v->n;
  };
  auto f = [&](const char* k, float& dst) {
    if (const JValue* v = j.get(k)) dst = (float)v->n;
  };
  u("log2_table", c.log2T);
  u("min_res", c.minRes);
  u("max_res", c.maxRes);
  f("lr", c.lr);
  f("train_fraction", c.trainFraction);
  u("train_path_shift", c.trainShift);
  u("train_depth", c.trainDepth);
  u("steps_per_wave", c.stepsPerWave);
  u("record_capacity", c.recCap);
  f("weight_clamp", c.weightClamp);
  f("log_kappa_max", c.logKappaMax);
  f("c_max", c.cMax);
  f("lr_mlp", c.lrMlp);
  u("seed", c.seed);
  u("lazy_table", c.lazyTable);
  if (c.trainShift > 31) throw std::runtime_error("train_path_shift must be <= 31");
  if (!(c.logKappaMax > kGLogKMin) || c.logKappaMax > 12.f) throw std::runtime_error("log_kappa_max must be in (-6, 12]");
  if (!(c.cMax >= 0.f) || c.cMax > 0.95f) throw std::runtime_error("c_max must be in [0, 0.95]");
  if (c.stepsPerWave < 1) c.stepsPerWave = 1;
  if (c.recCap < 1024) c.recCap = 1024;
}

}  // namespace rad
