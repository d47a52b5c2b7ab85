// Host-side state of a guide network (device parameters, Adam moments,
// gradient buffers) and its checkpoint format. See dguide.cuh for the method.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "dguide.cuh"

namespace rad {

struct GuideConfig {
  uint32_t log2T = 19;        // entries per level = 2^log2T
  uint32_t minRes = 16, maxRes = 512;
  float lr = 1e-2f, beta1 = 0.9f, beta2 = 0.99f, eps = 1e-10f;  // lr: hash table
  float lrMlp = 1e-3f;          // MLP weights (1e-2 there drives c into sigmoid saturation)
  float trainFraction = 0.25f;  // a guided job trains during its first fraction of samples
  uint32_t trainShift = 4;      // 1 in 2^shift paths records training vertices
  uint32_t trainDepth = 8;
  uint32_t stepsPerWave = 8;    // Adam steps per wave, each on a strided batch of its records
  uint32_t recCap = 1u << 20;
  float weightClamp = 32.f;     // normalised training weights are clipped to this
  float logKappaMax = 5.f;      // vMF concentration cap, log scale (kappa <= ~148: lobes of ~5 degrees)
  float cMax = 0.6f;            // guide selection probability cap (weights grow at most 1 / (1 - cMax))
  uint32_t seed = 5;
  uint32_t lazyTable = 1;       // Adam leaves table entries without a gradient in the batch untouched
};

struct GuideNet {
  GuideConfig cfg;
  uint64_t nTable = 0, nParams = 0;
  float* p = nullptr;   // fp32 master parameters: table, then MLP weights
  float* m = nullptr;   // Adam first moment
  float* v = nullptr;   // Adam second moment
  float* g = nullptr;   // gradient accumulator (zeroed by each Adam step)
  __half* ph = nullptr; // fp16 copy used by the kernels
  uint32_t* ctl = nullptr;  // [0] records, [1] weight sum bits, [2] loss sum bits, [3] spare
  uint32_t step = 0;
  uint32_t res[kGLevels];
  float lo[3], hi[3];
  uint64_t bytes = 0;
};

// Level resolutions floor(minRes * b^l), b = (maxRes / minRes)^(1 / (levels - 1)).
void GuideLevelRes(uint32_t minRes, uint32_t maxRes, uint32_t res[kGLevels]);
// Allocates and initialises (seeded uniform table in +-1e-4, He-uniform hidden
// layers, small output layer) on the current device.
GuideNet* GuideCreate(const GuideConfig& cfg, const float lo[3], const float hi[3]);
void GuideDestroy(GuideNet* net);
GuideDev GuideView(const GuideNet& net);
// Checkpoint: 32-word header (magic "RADGUID1", version, log2T, levels, minRes,
// maxRes, step, nParams (2 words), lo, hi, level resolutions), then fp32
// parameters, first and second moments.
size_t GuideCheckpointBytes(const GuideNet& net);
void GuideCheckpoint(const GuideNet& net, void* buf, cudaStream_t st);
// Parses a checkpoint into a new network (throws std::runtime_error on a bad buffer).
GuideNet* GuideFromCheckpoint(const void* buf, size_t size, const GuideConfig& base, cudaStream_t st);
// Parses the rad_guide_enable JSON keys into cfg.
void GuideParseConfig(const char* json, GuideConfig& cfg);

}  // namespace rad
