// rad_render_samples_noalloc: per-sample radiance through the same wavefront
// (or vol_path) kernels as rad_render_samples, for callers that cannot call
// cudaMalloc -- for example a host that has already given every free byte of
// device memory to its own pool allocator, or a frame loop that must not let an
// allocation or free synchronise the device. The caller passes device
// pointers for the inputs and the output; the path state the kernels need is a
// file-scope __device__ array of fixed size (kNoAllocMaxSamples paths), which
// every GPU that loads this library holds until the process exits.
//
// Set-up: the first call on a device looks up the array's device address
// with cudaGetSymbolAddress (the host-side name of the array is only a stand-in,
// not a device address) and caches it; make that first call before any stream
// capture. All calls share the one array and it keeps the last call's contents:
// the per-call counters are cleared on every call, and calls that overlap on the
// GPU (different streams, or other host threads) race on it.
#include <mutex>

#include "../../include/radgpu.h"
#include "kernels.h"

namespace rad {

constexpr uint32_t kNoAllocMaxSamples = 16384;

struct NoAllocScratch {
  float4 rayO[kNoAllocMaxSamples];
  float4 rayD[kNoAllocMaxSamples];
  float4 thr[kNoAllocMaxSamples];
  float4 L[kNoAllocMaxSamples];
  float4 prev[kNoAllocMaxSamples];
  float4 shO[kNoAllocMaxSamples];
  float4 shD[kNoAllocMaxSamples];
  float4 shC[kNoAllocMaxSamples];
  HitRec hit[kNoAllocMaxSamples];
  uint2 rng[kNoAllocMaxSamples];
  uint32_t pixel[kNoAllocMaxSamples];
  uint32_t q0[kNoAllocMaxSamples];
  uint32_t q1[kNoAllocMaxSamples];
  uint32_t classQ[kShadeClasses * kNoAllocMaxSamples];
  uint32_t counters[kCounterWords];
};

// About 3.4 MB per device (204 bytes of path state per sample).
static __device__ __align__(256) NoAllocScratch g_noallocScratch;

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
NoAllocScratch* g_addr[kMaxDevices] = {nullptr};
int g_sms[kMaxDevices] = {0};  // SM count per device, read with the address

PathBuffers ScratchBuffers(NoAllocScratch* s) {
  PathBuffers B{};
  B.rayO = s->rayO;
  B.rayD = s->rayD;
  B.thr = s->thr;
  B.L = s->L;
  B.prev = s->prev;
  B.rng = s->rng;
  B.pixel = s->pixel;
  B.hit = s->hit;
  B.q[0] = s->q0;
  B.q[1] = s->q1;
  B.shO = s->shO;
  B.shD = s->shD;
  B.shC = s->shC;
  B.classQ = s->classQ;
  B.counters = s->counters;
  B.capacity = kNoAllocMaxSamples;
  return B;
}

}  // namespace

// Scene access and error reporting live with the rest of the C ABI (runtime.cu).
const DevScene* SceneDevice(const rad_scene* scene);
const TraceTune* SceneTune(const rad_scene* scene);
int SceneDeviceIndex();
int ReportError(int code, const char* msg);

}  // namespace rad

using namespace rad;

extern "C" RAD_API int rad_render_samples_noalloc(rad_scene* scene, const uint32_t* d_pixels,
                                                  const uint32_t* d_samples, int64_t n, uint32_t seed,
                                                  float* d_radiance, void* stream) {
  if (!scene || n < 0 || (n > 0 && (!d_pixels || !d_samples || !d_radiance)))
    return ReportError(RAD_ERR_INVALID_ARG, "bad argument");
  if (n > (int64_t)kNoAllocMaxSamples)
    return ReportError(RAD_ERR_INVALID_ARG,
                       "rad_render_samples_noalloc: n exceeds the fixed scratch capacity of 16384 samples");
  if (n == 0) return RAD_OK;
  const DevScene& S = *SceneDevice(scene);
  if (S.isParticle) return ReportError(RAD_ERR_UNSUPPORTED, "particle_tracer has no per-pixel samples");
  if (S.isBdpt) return ReportError(RAD_ERR_UNSUPPORTED, "bdpt keeps its subpaths in device scratch it allocates");
  int dev = SceneDeviceIndex();
  if (dev < 0 || dev >= kMaxDevices) return ReportError(RAD_ERR_INVALID_ARG, "device index out of range");
  int prevDev = 0;
  if (cudaGetDevice(&prevDev) != cudaSuccess) return ReportError(RAD_ERR_CUDA, "cudaGetDevice failed");
  if (prevDev != dev && cudaSetDevice(dev) != cudaSuccess) return ReportError(RAD_ERR_CUDA, "cudaSetDevice failed");
  auto done = [&](int code, const char* msg) {
    if (prevDev != dev) cudaSetDevice(prevDev);
    return code == RAD_OK ? RAD_OK : ReportError(code, msg);
  };
  NoAllocScratch* addr;
  {
    std::lock_guard<std::mutex> g(g_mu);
    if (!g_addr[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
      if (e != cudaSuccess || !p) return done(RAD_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed");
      int sms = 0;
      if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        return done(RAD_ERR_CUDA, "cudaDeviceGetAttribute failed");
      g_sms[dev] = sms;
      g_addr[dev] = static_cast<NoAllocScratch*>(p);
    }
    addr = g_addr[dev];
  }
  const int sms = g_sms[dev];
  const TraceTune& tu = *SceneTune(scene);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  PathBuffers B = ScratchBuffers(addr);
  uint32_t count = (uint32_t)n;
  // the device-error word is sticky: clear it; generate clears the queue counters
  if (cudaMemsetAsync(addr->counters + kMiscBase + 1, 0, sizeof(uint32_t), st) != cudaSuccess)
    return done(RAD_ERR_CUDA, "cudaMemsetAsync failed");
  WaveParams w{0, count, 0, seed, d_pixels, d_samples};
  if (LaunchGenerate(S, B, w, st) != cudaSuccess) return done(RAD_ERR_CUDA, "generate launch failed");
  if (S.isVol) {
    if (LaunchVolPath(S, B, w, addr->counters + kMiscBase + 1, st) != cudaSuccess)
      return done(RAD_ERR_CUDA, "vol_path launch failed");
  } else {
    // launch shapes and traversal parameters as rad_render_samples uses them (rad_autotune's choice)
    int grid = std::max(1, std::min(sms * 8, (int)((count + 127) / 128)));
    int tgrid = std::max(1, std::min(sms * tu.blocksPerSm, (int)((count + 127) / 128)));
    int iters = S.maxDepth >= 0 ? std::max(1, S.maxDepth) : kMaxBounce;
    if (iters > kMaxBounce) iters = kMaxBounce;
    if (S.isAO) {  // renderer "ao": first hit and one visibility ray
      if (LaunchExtend(S, B, 0, tgrid, st, nullptr, tu.refillBusy, tu.leafFrac8) != cudaSuccess ||
          LaunchShadeAO(S, B, grid, st) != cudaSuccess ||
          LaunchShadow(S, B, 0, tgrid, st, nullptr, tu.refillBusy, tu.leafFrac8) != cudaSuccess)
        return done(RAD_ERR_CUDA, "ao launch failed");
      iters = 0;
    }
    for (int d = 0; d < iters; d++) {
      if (LaunchExtend(S, B, d, tgrid, st, nullptr, tu.refillBusy, tu.leafFrac8) != cudaSuccess ||
          LaunchShade(S, B, d, grid, st, nullptr, false, tu.shadeBlock) != cudaSuccess ||
          LaunchShadow(S, B, d, tgrid, st, nullptr, tu.refillBusy, tu.leafFrac8) != cudaSuccess)
        return done(RAD_ERR_CUDA, "bounce launch failed");
      if (S.maxDepth < 0 && (d % 8) == 7) {
        uint32_t next = 0;
        if (cudaMemcpyAsync(&next, addr->counters + d + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st) !=
                cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
          return done(RAD_ERR_CUDA, "queue readback failed");
        if (next == 0) break;
      }
    }
  }
  if (LaunchGatherRadiance(B, count, d_radiance, st) != cudaSuccess) return done(RAD_ERR_CUDA, "gather launch failed");
  uint32_t err = 0;
  if (cudaMemcpyAsync(&err, addr->counters + kMiscBase + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st) !=
          cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return done(RAD_ERR_CUDA, "stream synchronisation failed");
  if (err & kErrPixelRange) return done(RAD_ERR_DEVICE_CHECK, "a pixel index lies outside the film");
  if (err) return done(RAD_ERR_DEVICE_CHECK, "a device-side bound was exceeded");
  return done(RAD_OK, "");
}
