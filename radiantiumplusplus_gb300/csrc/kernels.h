// Host-side launchers of the sm_103a kernels (implemented in k_*.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "dguide.cuh"
#include "dvol.cuh"
#include "records.h"

namespace rad {

struct MixJob;

// Wavefront path state, structure of arrays, one slot per path in flight.
struct PathBuffers {
  float4* rayO;    // origin xyz, tmin
  float4* rayD;    // direction xyz, tmax
  float4* thr;     // throughput rgb, eta
  float4* L;       // radiance rgb, previous BSDF pdf
  float4* prev;    // previous shading point xyz, flags (bit 0 specular path) | depth << 8
  uint2* rng;      // PCG32 state
  uint32_t* pixel; // film pixel index
  HitRec* hit;
  uint32_t* q[2];  // active path queues (ping-pong)
  float4* shO;     // shadow ray origin xyz, tmax
  float4* shD;     // shadow ray direction xyz, path slot bits
  float4* shC;     // shadow contribution rgb
  uint32_t* classQ;    // kShadeClasses queues of `capacity` slots, filled by extend, read by shade
  uint32_t* counters;  // [0, kMaxBounce]: active counts; [kShadowBase, +kMaxBounce]: shadow counts; kMisc..;
                       // [kClassBase + depth * kShadeClasses + class]: shade-class counts
  uint32_t capacity;
  float4* guideRec;    // guide training records (shadow stage adds NEE into them), or null
  // mixed waves: the job (index into `mix`) of each path slot, and the wave's job table
  uint8_t* job;
  const MixJob* mix;
};

// One job's share of a mixed wave (several jobs' paths in one launch of each
// stage). Its paths occupy slots [pathBegin, pathBegin + count): spw
// consecutive samples (from `sample`) of the npc pixels [pixelBegin,
// pixelBegin + npc), path pathBegin + s * npc + j being pixel pixelBegin + j,
// sample sample + s -- the layout of a one-job wave.
constexpr int kMaxMix = 16;
struct MixJob {
  DevScene S;
  float4* film;
  unsigned long long* stats;
  uint32_t pathBegin, count, pixelBegin, npc, spw, sample, seed, pad;
};

constexpr int kMaxBounce = 256;
constexpr int kShadowBase = kMaxBounce + 1;
constexpr int kMiscBase = 2 * kMaxBounce + 2;  // [0] spare, [1] device error word (sticky),
                                               // [2] vol closest rays, [3] vol shadow-side rays,
                                               // [4] vol paths taken (KVolPath's refill counter)
// bits of the device error word: 1 traversal stack, 2 / 4 vol_path iteration
// bounds, 8 bdpt visibility buffer, kErrPixelRange a pixel index beyond the film
constexpr uint32_t kErrPixelRange = 16u;
constexpr uint32_t kErrGuideTc = 32u;  // a tensor-core wait of the guide network gave up
constexpr int kClassBase = kMiscBase + 8;
// per-bounce ray-fetch counters of the persistent extend / shadow kernels
constexpr int kFetchBase = kClassBase + (kMaxBounce + 1) * kShadeClasses;
constexpr int kCounterWords = kFetchBase + 2 * (kMaxBounce + 1);

#if defined(__CUDACC__)
// Entry i of bounce `depth`'s hits taken class by class from the shade-class
// queues the closest-hit kernel fills (each queued path appears in exactly one),
// so that neighbouring threads shade the same kind of material. `start` holds
// the classes' prefix sums (ClassQueueStarts).
__device__ __forceinline__ void ClassQueueStarts(const PathBuffers& B, int depth, uint32_t* start) {
  const uint32_t* cc = B.counters + kClassBase + depth * kShadeClasses;
  start[0] = 0;
  for (int c = 0; c < kShadeClasses; c++) start[c + 1] = start[c] + cc[c];
}
__device__ __forceinline__ uint32_t ClassQueueEntry(const PathBuffers& B, const uint32_t* start, uint32_t i) {
  int c = 0;
  while (c + 1 < kShadeClasses && i >= start[c + 1]) c++;
  return B.classQ[(size_t)c * B.capacity + (i - start[c])];
}
#endif

struct FilmView {
  float4* accum;  // rgb sum, sample count in w
  int32_t width, height;
  // job counters (64-bit, device): [0] closest rays, [1] shadow rays,
  // [2] invalid samples, [3] samples, [4..7] traversal counts (see LaunchExtend)
  unsigned long long* stats;
};

// ---- parity kernels (k_parity.cu)
cudaError_t LaunchTexEval(const DevScene& S, uint32_t tex, const float* uv, const float* duv, int64_t n, float* out,
                          cudaStream_t st);
cudaError_t LaunchBsdfEval(const MatRec* mats, const float* wi, const float* wo, int64_t n, float* f, float* pdf,
                           cudaStream_t st);
cudaError_t LaunchBsdfSample(const MatRec* mats, const float* wi, const float* u, int64_t n, float* wo, float* pdf,
                             float* f, float* eta, uint32_t* type, cudaStream_t st);
cudaError_t LaunchTrace(const DevScene& S, const float* rays, int64_t n, float* hits, int anyHit, uint32_t* err,
                        cudaStream_t st);
cudaError_t LaunchCameraRays(const DevScene& S, const uint32_t* pix, int64_t n, uint32_t sample, uint32_t seed,
                             float* out, cudaStream_t st);

// ---- wavefront path tracer (k_path.cu)
struct WaveParams {
  uint32_t pixelBegin, count;  // pixels [pixelBegin, pixelBegin + count) of the film
  uint32_t sample, seed;
  const uint32_t* pixelList;   // optional explicit pixel list (parity hook)
  const uint32_t* sampleList;  // optional explicit per-path sample indices
  // Optional device-side wave context (graph replay): when set, the sample index,
  // seed, film and stats come from here, and the accumulate stage advances the
  // sample index, so one captured graph renders consecutive samples.
  const struct WaveCtx* ctx;
  // Samples per wave (0 or 1: one). With spw > 1 the wave holds spw consecutive
  // samples of the same count / spw pixels: path i is pixel pixelBegin + i % (count / spw),
  // sample sample + i / (count / spw). Small frames thus fill the wave.
  uint32_t spw;
};

// Per-job wave context in device memory, read by generate and accumulate.
struct WaveCtx {
  float4* film;
  unsigned long long* stats;
  uint32_t sample;  // next sample index; advanced by accumulate
  uint32_t seed;
  uint32_t pad[2];
};
int PathGridBlocks();
cudaError_t LaunchGenerate(const DevScene& S, const PathBuffers& B, const WaveParams& w, cudaStream_t st);
// Launch parameters of the persistent traversal kernels, chosen per scene by
// the autotuner (rad_autotune): a warp refills its idle lanes once fewer than
// refillBusy lanes are still tracing; it tests pending leaves once at least
// leafFrac8 / 8 of its busy lanes hold some; grids hold blocksPerSm blocks per SM.
// The shade-class kernels run blocks of shadeBlock threads (64, 128 or 256).
struct TraceTune {
  int32_t refillBusy = 20;
  int32_t blocksPerSm = 8;
  int32_t leafFrac8 = 4;
  int32_t shadeBlock = 128;
  int32_t volChunk = 16;  // vol_path wavefront: loop steps of one part a lane runs per launch
};
// trav (optional, 4 x u64): extend node visits, extend prim tests, shadow node visits, shadow prim tests
cudaError_t LaunchExtend(const DevScene& S, const PathBuffers& B, int depth, int grid, cudaStream_t st,
                         unsigned long long* trav = nullptr, int refillBusy = 20, int leafFrac8 = 4, bool mix = false);
// G (optional): guide network; its classes then sample the one-sample MIS mixture.
// grid counts blocks of 128 threads; with block != 128 the grid keeps the same number of threads.
cudaError_t LaunchShade(const DevScene& S, const PathBuffers& B, int depth, int grid, cudaStream_t st,
                        const GuideDev* G = nullptr, bool mix = false, int block = 128);
// Mixed waves: generate (w.count = paths of all jobs, w.spw = number of jobs in
// B.mix) and accumulate (into each job's film, in sample order per pixel).
cudaError_t LaunchGenerateMix(const PathBuffers& B, uint32_t total, uint32_t nJobs, cudaStream_t st);
cudaError_t LaunchAccumulateMix(const PathBuffers& B, uint32_t totalPixels, uint32_t total, uint32_t nJobs,
                                cudaStream_t st);
// renderer "particle_tracer": light paths [first, first + count), splatted into `film`
struct ParticleParams {
  uint64_t first, count;
  uint32_t seed;
  float sampleScale;  // pixels / light paths of the job (particle_tracer.cpp:55)
};
// ---- renderer "bdpt" (k_bdpt.cu): wavefront stages of one wave of pixel samples
struct BVert;
constexpr size_t kBVertBytes = 112;  // sizeof(BVert) (dbdpt.cuh)
constexpr int kBdptBuckets = kShadeClasses * kShadeClasses;  // (camera vertex class, light vertex class)
struct BdptBuffers {
  BVert* vert;         // [2 * cap][nw]: camera subpath vertices, then light subpath vertices
  float4* walkA;       // per sample: walk throughput rgb, eta
  float4* walkB;       // per sample: pdfFwd, rr, vertex count (bits)
  float4* fix;         // per sample: emitted direction xyz, position density (light subpath fix-up)
  uint32_t* nCam;      // per sample: camera / light subpath vertex counts
  uint32_t* nLight;
  float4 *shO, *shD, *shC;  // visibility rays of one connection round: origin + tmax, direction + tag, contribution
  // samples ordered by (camera, light) subpath length, so that a connection round runs over the
  // suffix of samples with a long enough camera subpath, neighbours looping over as many light vertices
  uint32_t* order;     // nw sample slots
  uint32_t* keyStart;  // (cap + 1)^2 + 1: first slot of each key (exclusive scan of the key counts)
  uint32_t* keyFill;   // (cap + 1)^2: per-key counts, then scatter cursors
  uint32_t* itemStart; // (cap + 1)^2 + 1: exclusive scan over keys of the s >= 2 connections (nl - 1 a sample)
  uint2* rng1;         // per sample: PCG state before connection round t = 1
  // the s >= 2 connections of one round ordered by the shade classes of their two vertices
  uint32_t* items;     // nw * cap: sample | s << 24, bucket by bucket
  uint32_t* bucket;    // 2 * kBdptBuckets + 1: counts, then starts, then scatter cursors
  uint32_t cap, nw, shCap;
};
// Camera subpaths: jittered camera rays of the wave's samples into queue 0.
cudaError_t LaunchBdptCamera(const DevScene& S, const PathBuffers& B, const BdptBuffers& V, const WaveParams& w,
                             cudaStream_t st);
// Light subpaths: light pick and emitted rays of the wave's `count` samples into queue 0.
cudaError_t LaunchBdptLight(const DevScene& S, const PathBuffers& B, const BdptBuffers& V, uint32_t count,
                            cudaStream_t st);
// One subpath bounce for the queue of `depth` (after LaunchExtend): vertex, BSDF sample, next ray.
// Longest camera subpath of the wave: B.counters[kMiscBase] (atomic max).
cudaError_t LaunchBdptWalk(const DevScene& S, const PathBuffers& B, const BdptBuffers& V, int depth, bool light,
                           int grid, cudaStream_t st);
// Infinite-light fix-up of the light subpaths, then the samples' order by subpath lengths
// (V.keyFill zeroed beforehand).
cudaError_t LaunchBdptLightFix(const DevScene& S, const BdptBuffers& V, uint32_t count, cudaStream_t st);
// Round t >= 2 of the connections (camera vertex t - 1 with every light vertex): s = 0 / 1 per
// sample (s = 1 draws the round's random numbers; s = 0 adds into B.L directly), then the s >= 2
// ones one per thread; visibility rays into V.sh* (count in B.counters[kShadowBase + t - 1]).
cudaError_t LaunchBdptConnectSplit(const DevScene& S, const PathBuffers& B, const BdptBuffers& V, uint32_t count,
                                   int t, int grid, cudaStream_t st);
// Round t = 1 (splats), one thread per connection: each starts from the sample's stream advanced past the
// draws of the connections before it; the sample's stream is advanced past them all. Without splats
// only the advance runs.
cudaError_t LaunchBdptRound1(const DevScene& S, const PathBuffers& B, const BdptBuffers& V, uint32_t count,
                             bool splats, int grid, cudaStream_t st);
// Visibility rays of round t: unoccluded contributions into B.L (atomic) or the film (splats).
cudaError_t LaunchBdptShadow(const DevScene& S, const PathBuffers& B, const BdptBuffers& V, int t, float4* film,
                             int grid, cudaStream_t st, int refillBusy, int leafFrac8);
// Per sample: camera-side radiance into `out` (n x 3) and / or valid samples into the film.
cudaError_t LaunchBdptAccumulate(const PathBuffers& B, const FilmView& film, uint32_t count, float* out,
                                 cudaStream_t st);
// Renderer "particle_tracer" (k_light.cu): light path starts (emitter connections into
// visibility round 0 of B.sh*, emitted rays into queue 0) and one bounce per launch after
// LaunchExtend (camera connections into round d + 1); the rounds are traced by LaunchBdptShadow.
cudaError_t LaunchParticleStart(const DevScene& S, const PathBuffers& B, const ParticleParams& pp,
                                unsigned long long* stats, cudaStream_t st);
cudaError_t LaunchParticleBounce(const DevScene& S, const PathBuffers& B, int d, float sampleScale, int grid,
                                 cudaStream_t st);
// renderer "ao": for every path of bounce 0 with a hit, one cosine-sampled visibility ray
cudaError_t LaunchShadeAO(const DevScene& S, const PathBuffers& B, int grid, cudaStream_t st);
cudaError_t LaunchShadow(const DevScene& S, const PathBuffers& B, int depth, int grid, cudaStream_t st,
                         unsigned long long* trav = nullptr, int refillBusy = 20, int leafFrac8 = 4, bool mix = false);
// spw: samples per wave of the generate stage (per pixel, in sample order, as
// spw one-sample waves would add them).
cudaError_t LaunchAccumulate(const PathBuffers& B, const FilmView& film, uint32_t count, cudaStream_t st,
                             struct WaveCtx* ctx = nullptr, uint32_t spw = 1);
cudaError_t LaunchGatherRadiance(const PathBuffers& B, uint32_t count, float* out, cudaStream_t st);
cudaError_t LaunchResolveFilm(const FilmView& film, float scale, float* out, cudaStream_t st);

// ---- volumetric path tracer (k_vol.cu)
// mode bits kVolBricks / kVolHalf / kVolRealDepth: see dvol.cuh
// Persistent kernel: lanes run their paths one part of a loop iteration at a
// time, every warp step the part most lanes are at; needs no memory beyond B.
cudaError_t LaunchVolPath(const DevScene& S, const PathBuffers& B, const WaveParams& w, uint32_t* err,
                          cudaStream_t st, uint32_t mode = 0);
// Per-event wavefront: the loop parts (top / medium scatter / surface / NEE
// transmittance / scatter end / surface end) as kernels over queues of the
// paths at each part, path state in HBM between them. The same arithmetic per
// path as LaunchVolPath, so the same radiance bit for bit.
constexpr int kVolActs = 6;
// counter words: [par * kVolActs + act] queue lengths (two parities: a path
// moving to a later part of the round goes to the current parity, one moving
// back or continuing its part to the next round's),
// [2 kVolActs + act] queue heads, [3 kVolActs] paths ended
constexpr int kVolEndedWord = 3 * kVolActs;
constexpr int kVolCountWords = 3 * kVolActs + 1;
struct VolWave {
  void* state;        // capacity per-path loop states (VolStateBytes() each, 16-byte aligned)
  uint32_t* q;        // [2 * kVolActs][capacity] path indices
  uint32_t* cnt;      // kVolCountWords counters
  uint32_t capacity;
};
size_t VolStateBytes();
// Runs the wave's rounds; host-side it waits on the stream every few rounds to
// see whether every path has ended (hostCounts: pinned, kVolCountWords words).
// launches: kernels run. cudaErrorIllegalState if the path count is not
// conserved (a path neither ended nor queued).
// tu.refillBusy: a warp tops up its lanes once fewer than this many run a path;
// tu.blocksPerSm: resident blocks per SM of the part kernels (at most their occupancy);
// tu.volChunk: steps of the repeating parts (null collisions, NEE transmittance)
// a lane runs per path and launch before the path continues in the next round.
cudaError_t LaunchVolWavefront(const DevScene& S, const PathBuffers& B, const VolWave& V, const WaveParams& w,
                               uint32_t* err, cudaStream_t st, uint32_t mode, const TraceTune& tu,
                               uint32_t* hostCounts, uint64_t* launches);

// ---- guide network (k_guide.cu)
cudaError_t GuideKernelsInit();
cudaError_t LaunchGuideInfer(const DevScene& S, const PathBuffers& B, const GuideDev& G, int depth, uint32_t maxCount,
                             cudaStream_t st);
cudaError_t LaunchGuideQuery(const GuideDev& G, const float* queries, uint32_t n, float* raw, float4* mix, uint32_t* err,
                             cudaStream_t st);
cudaError_t LaunchGuideMixEval(const float4* mix, const float* dirs, const float* u, uint32_t n, float* pdf,
                               float* outDirs, cudaStream_t st);
cudaError_t LaunchGuideFinalize(const PathBuffers& B, const GuideDev& G, cudaStream_t st);
// One training batch: records j * steps + step. With ctl, the count and the
// mean weight come from the device (ctl[0], ctl[1]); else `count`, weights as given.
// err: kErrGuideTc is or'ed in if a tensor-core wait gave up.
cudaError_t LaunchGuideTrain(const GuideDev& G, const float4* rec, const uint32_t* ctl, uint32_t count, uint32_t cap,
                             uint32_t steps, uint32_t step, float wClamp, float* gradTable, float* gradW,
                             float* lossOut, uint32_t maxBatch, uint32_t* err, cudaStream_t st);
// Adam step t (1-based). With ctl, the gradient scale is 1 / (size of batch `step`
// of `steps`) from the device record count, and an empty batch changes nothing.
// Parameters [0, split) step with lr, [split, n) with lr2.
cudaError_t LaunchGuideAdam(float* p, float* m, float* v, float* g, __half* ph, uint64_t n, float lr, uint64_t split,
                            float lr2, float b1, float b2, float eps, float gscale, uint32_t t, const uint32_t* ctl,
                            uint32_t cap, uint32_t steps, uint32_t step, bool lazyTable, cudaStream_t st);
cudaError_t LaunchFloatToHalf(const float* src, __half* dst, uint64_t n, cudaStream_t st);

}  // namespace rad
