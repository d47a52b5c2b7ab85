// C ABI of include/radgpu.h: library state, resident scenes, render jobs and
// the serving loop. The reference's Renderer::Start spawns one render thread
// that walks TBB tiles (sample_renderer.cpp:60-122); here one worker thread
// owns the CUDA stream, admits submitted jobs against a device-memory budget,
// and interleaves their waves (one wave = one sample index over a job's
// pixels) round-robin, so jobs that arrive while others run are admitted as
// soon as memory allows and share the device at wave granularity.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "../../include/radgpu.h"
#include "guide_net.h"
#include "host_scene.h"
#include "kernels.h"

using namespace rad;

namespace {

thread_local std::string t_err;

struct Error {
  int code;
  std::string msg;
};

void Check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    if (e == cudaErrorMemoryAllocation) {
      cudaGetLastError();
      throw Error{RAD_ERR_OUT_OF_MEMORY, std::string(what) + ": " + cudaGetErrorString(e)};
    }
    throw Error{RAD_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e)};
  }
}

int Fail(int code, const std::string& msg) {
  t_err = msg;
  return code;
}

template <typename F>
int Guard(F&& f) {
  try {
    f();
    return RAD_OK;
  } catch (const Error& e) {
    return Fail(e.code, e.msg);
  } catch (const JsonError& e) {
    return Fail(RAD_ERR_JSON, e.what());
  } catch (const FactoryError& e) {
    return Fail(RAD_ERR_UNKNOWN_FACTORY, e.what());
  } catch (const IoError& e) {
    return Fail(RAD_ERR_IO, e.what());
  } catch (const ConfigError& e) {
    return Fail(RAD_ERR_INVALID_ARG, e.what());
  } catch (const std::bad_alloc&) {
    return Fail(RAD_ERR_OUT_OF_MEMORY, "host allocation failed");
  } catch (const std::exception& e) {
    return Fail(RAD_ERR_INVALID_ARG, e.what());
  }
}

double NowMs() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

void FreeAll(std::vector<void*>& v) {
  for (void* p : v) cudaFree(p);
  v.clear();
}

template <typename T>
T* DevAlloc(size_t count, std::vector<void*>& owner, uint64_t& bytes) {
  if (count == 0) return nullptr;
  void* p = nullptr;
  Check(cudaMalloc(&p, count * sizeof(T)), "cudaMalloc");
  owner.push_back(p);
  bytes += count * sizeof(T);
  return static_cast<T*>(p);
}

enum JobState { kQueued, kRunning, kCompleting, kDone };
// device job counters: [0..3] rays, invalid, samples; [4..7] traversal; [8] guide records
constexpr int kJobStatWords = 10;

}  // namespace

// The device buffers of a finished job (film, statistics, resolve target,
// events) and, for a `path` job, its instantiated per-chunk wave graphs with
// their wave contexts: kept by the scene for its next job of the same film, so
// a stream of short jobs does not allocate, free (a device-wide sync) and
// capture per job. The graphs are reused when the samples per wave and the
// scene's traversal parameters match; the job's wave contexts are rewritten.
struct JobSpare {
  bool valid = false;
  float4* accum = nullptr;
  unsigned long long *dStats = nullptr, *hStats = nullptr;
  float* resolve = nullptr;
  cudaEvent_t evStart = nullptr, evEnd = nullptr;
  WaveCtx* ctx = nullptr;
  std::vector<cudaGraphExec_t> graphs;
  std::vector<uint64_t> graphKernels;
  uint32_t spw = 0;
  uint64_t tuneEpoch = 0;
  uint64_t bytes = 0;  // film bytes, still counted in the library's used bytes
};

struct rad_scene {
  DevScene dev{};
  std::vector<void*> allocs;
  uint64_t bytes = 0;
  rad_scene_info info{};
  std::atomic<int> jobs{0};
  float worldLo[3] = {0, 0, 0}, worldHi[3] = {1, 1, 1};
  GuideNet* guide = nullptr;  // learned proposal, created by rad_guide_enable / _load or a guided job
  GuideConfig guideCfg;
  TraceTune tune;  // traversal launch parameters (rad_autotune)
  uint64_t tuneEpoch = 0;  // bumped when `tune` changes (captured graphs bake it in)
  JobSpare spare;          // guarded by the library's GPU mutex
};

struct rad_job {
  rad_scene* scene = nullptr;
  uint32_t spp = 0, seed = 0, first = 0, flags = 0;
  uint64_t total = 0;
  uint32_t nextSample = 0;
  uint32_t chunkCursor = 0;
  float4* accum = nullptr;
  unsigned long long* dStats = nullptr;
  unsigned long long* hStats = nullptr;  // pinned
  float* resolve = nullptr;
  uint64_t filmBytes = 0;
  JobState state = kQueued;
  int status = RAD_OK;
  std::string err;
  bool cancel = false;
  std::atomic<uint64_t> launched{0};
  cudaEvent_t evStart = nullptr, evEnd = nullptr;
  double tSubmit = 0, tStart = 0, tEnd = 0;
  double deadline = 0;  // earliest-deadline-first mixing: submit time + samples x the per-sample allowance (ms)
  rad_stats stats{};
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> profEv;
  std::vector<int> profKind;
  uint32_t trainSamples = 0;  // guided jobs train during their first trainSamples samples
  uint32_t spw = 0;           // samples per wave (0 = not chosen yet; see WaveSamples)
  uint32_t mixCursor = 0;     // mixed waves: next pixel of the current sample (0: at a sample boundary)
  // CUDA graph per pixel chunk: one captured wave replayed once per sample
  WaveCtx* ctx = nullptr;  // device, one per chunk
  bool ctxStale = false;   // graphs taken over from an earlier job: contexts not yet written
  std::vector<cudaGraphExec_t> graphs;
  std::vector<uint64_t> graphKernels;
  std::mutex m;
  std::condition_variable cv;
};

namespace {

// Waves the worker may have queued on the stream ahead of the GPU (see WorkerMain),
// and the mixed-wave job tables kept for them.
constexpr size_t kMaxWavesInFlight = 2;
constexpr int kMixRing = (int)kMaxWavesInFlight + 1;

// Device bytes the bdpt scratch may take by default (rad_init
// "bdpt_scratch_bytes"): the wave size follows from the scene's vertex cap
// (2 subpaths x cap vertices + cap visibility rays a sample).
constexpr uint64_t kBdptScratchBytes = 4ull << 30;

struct Lib {
  bool inited = false;
  int device = 0;
  int sms = 0;
  cudaStream_t stream = nullptr;
  uint64_t budget = 150ull * 1000 * 1000 * 1000;
  std::atomic<uint64_t> used{0};
  // films parked with their scenes for the next job (JobSpare): counted in
  // `used`, and released when an admission would otherwise fail
  std::atomic<uint64_t> spareBytes{0};
  std::vector<rad_scene*> spareScenes;  // guarded by gpuMu
  uint32_t maxPaths = 1u << 21;
  PathBuffers paths{};
  std::vector<void*> pathAllocs;
  uint64_t pathBytes = 0;
  uint32_t* hCounters = nullptr;  // pinned
  // mixed waves: a ring of job tables (device, with pinned staging), one per wave in flight
  bool mixJobs = true;
  float shareExp = 0.f;  // mixed-wave shares ~ remaining samples ^ shareExp (0: equal shares)
  double edfNsPerSample = 0;  // > 0: earliest-deadline-first mixing, deadline = submit + samples x this
  double slowNsPerSample = 0;  // > 0: highest-slowdown-first mixing, slowdown = age / (samples x this + 20 ms)
  MixJob* mixDev = nullptr;
  MixJob* mixHost = nullptr;
  uint32_t mixSlot = 0;
  std::mutex gpuMu;
  // serving loop
  std::thread worker;
  std::mutex qmu;
  std::condition_variable qcv;
  std::deque<rad_job*> pending;
  std::vector<rad_job*> running;
  size_t rr = 0;
  bool stop = false;
  std::vector<cudaEvent_t> evPool;
  // guide buffers, allocated with the first guided wave
  float4* guideMix = nullptr;  // kGMixF4 per path slot
  float4* guideRec = nullptr;
  uint32_t guideRecCap = 0;
  uint64_t guideBytes = 0;
  // bdpt wavefront scratch, allocated with the first bdpt wave for its scene's vertex cap
  BdptBuffers bdpt{};
  std::vector<void*> bdptAllocs;
  uint64_t bdptBytes = 0;
  uint64_t bdptScratch = kBdptScratchBytes;
  // vol_path wavefront: per-path loop states and part queues, allocated with the first vol_path wave
  VolWave vol{};
  std::vector<void*> volAllocs;
  uint64_t volBytes = 0;
  uint32_t* hVolWord = nullptr;  // pinned, kVolCountWords words
};

// Never destroyed: at process exit the worker thread may still be parked on
// `qcv`, and destroying a condition variable with a waiter blocks forever.
// rad_shutdown() is the orderly teardown (the Python package calls it atexit).
Lib& L() {
  static Lib* lib = new Lib();
  return *lib;
}
std::mutex g_initMu;

cudaEvent_t GetEvent() {
  Lib& lib = L();
  if (!lib.evPool.empty()) {
    cudaEvent_t e = lib.evPool.back();
    lib.evPool.pop_back();
    return e;
  }
  cudaEvent_t e;
  Check(cudaEventCreate(&e), "cudaEventCreate");
  return e;
}

void AllocPaths(Lib& lib) {
  uint32_t P = lib.maxPaths;
  // refuse path buffers the device cannot hold before allocating any of them
  const uint64_t perPath = 8 * sizeof(float4) + sizeof(uint2) + sizeof(uint32_t) + sizeof(HitRec) +
                           (2 + kShadeClasses) * sizeof(uint32_t) + sizeof(uint8_t);
  size_t freeB = 0, totalB = 0;
  if (cudaMemGetInfo(&freeB, &totalB) == cudaSuccess && (uint64_t)P * perPath > (uint64_t)freeB)
    throw Error{RAD_ERR_INVALID_ARG, "max_paths " + std::to_string(P) + " needs " +
                                         std::to_string((uint64_t)P * perPath) + " bytes of path buffers; " +
                                         std::to_string((uint64_t)freeB) + " free on the device"};
  PathBuffers& B = lib.paths;
  auto& o = lib.pathAllocs;
  uint64_t& b = lib.pathBytes;
  B.rayO = DevAlloc<float4>(P, o, b);
  B.rayD = DevAlloc<float4>(P, o, b);
  B.thr = DevAlloc<float4>(P, o, b);
  B.L = DevAlloc<float4>(P, o, b);
  B.prev = DevAlloc<float4>(P, o, b);
  B.rng = DevAlloc<uint2>(P, o, b);
  B.pixel = DevAlloc<uint32_t>(P, o, b);
  B.hit = DevAlloc<HitRec>(P, o, b);
  B.q[0] = DevAlloc<uint32_t>(P, o, b);
  B.q[1] = DevAlloc<uint32_t>(P, o, b);
  B.shO = DevAlloc<float4>(P, o, b);
  B.shD = DevAlloc<float4>(P, o, b);
  B.shC = DevAlloc<float4>(P, o, b);
  B.classQ = DevAlloc<uint32_t>((size_t)P * kShadeClasses, o, b);
  B.counters = DevAlloc<uint32_t>(kCounterWords, o, b);
  B.job = DevAlloc<uint8_t>(P, o, b);
  B.mix = nullptr;
  lib.mixDev = DevAlloc<MixJob>((size_t)kMixRing * kMaxMix, o, b);
  Check(cudaMemset(B.counters, 0, kCounterWords * sizeof(uint32_t)), "cudaMemset");
  B.capacity = P;
  Check(cudaMallocHost(&lib.hCounters, kCounterWords * sizeof(uint32_t)), "cudaMallocHost");
  Check(cudaMallocHost(&lib.mixHost, (size_t)kMixRing * kMaxMix * sizeof(MixJob)), "cudaMallocHost");
  lib.used += b;
}

void WorkerMain();

void InitLocked(const char* cfg) {
  Lib& lib = L();
  if (lib.inited) {
    // a running library takes a new admission budget; the other keys are fixed at first init
    if (cfg && *cfg) {
      JValue c = JsonReader::Parse(cfg);
      if (const JValue* v = c.get("budget_bytes")) lib.budget = (uint64_t)v->n;
      if (const JValue* v = c.get("mix_jobs")) lib.mixJobs = v->n != 0;
      if (const JValue* v = c.get("share_exponent")) lib.shareExp = (float)v->n;
      if (const JValue* v = c.get("deadline_ns_per_sample")) lib.edfNsPerSample = v->n;
      if (const JValue* v = c.get("slowdown_ns_per_sample")) lib.slowNsPerSample = v->n;
    }
    return;
  }
  const uint32_t maxPaths0 = lib.maxPaths;
  const uint64_t bdptScratch0 = lib.bdptScratch;
  if (cfg && *cfg) {
    JValue c = JsonReader::Parse(cfg);
    if (const JValue* v = c.get("device")) lib.device = (int)v->n;
    if (const JValue* v = c.get("budget_bytes")) lib.budget = (uint64_t)v->n;
    if (const JValue* v = c.get("max_paths")) lib.maxPaths = (uint32_t)v->n;
    if (const JValue* v = c.get("bdpt_scratch_bytes")) lib.bdptScratch = (uint64_t)v->n;
    if (const JValue* v = c.get("mix_jobs")) lib.mixJobs = v->n != 0;
    if (const JValue* v = c.get("share_exponent")) lib.shareExp = (float)v->n;
    if (const JValue* v = c.get("deadline_ns_per_sample")) lib.edfNsPerSample = v->n;
    if (const JValue* v = c.get("slowdown_ns_per_sample")) lib.slowNsPerSample = v->n;
  }
  if (lib.maxPaths < 1024) lib.maxPaths = 1024;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    throw Error{RAD_ERR_NO_DEVICE, "no CUDA device available"};
  }
  if (lib.device < 0 || lib.device >= n) throw Error{RAD_ERR_INVALID_ARG, "device index out of range"};
  Check(cudaSetDevice(lib.device), "cudaSetDevice");
  Check(cudaDeviceGetAttribute(&lib.sms, cudaDevAttrMultiProcessorCount, lib.device), "attribute");
  Check(cudaStreamCreateWithFlags(&lib.stream, cudaStreamNonBlocking), "cudaStreamCreate");
  try {
    Check(GuideKernelsInit(), "guide kernel attributes");
    AllocPaths(lib);
  } catch (...) {
    // a failed first init (e.g. path buffers larger than the device) leaves
    // nothing behind, and a later rad_init starts from the default sizes
    FreeAll(lib.pathAllocs);
    lib.pathBytes = 0;
    lib.paths = PathBuffers{};
    lib.mixDev = nullptr;
    if (lib.hCounters) cudaFreeHost(lib.hCounters);
    if (lib.mixHost) cudaFreeHost(lib.mixHost);
    lib.hCounters = nullptr;
    lib.mixHost = nullptr;
    cudaStreamDestroy(lib.stream);
    lib.stream = nullptr;
    lib.maxPaths = maxPaths0;
    lib.bdptScratch = bdptScratch0;
    cudaGetLastError();
    throw;
  }
  lib.stop = false;
  lib.worker = std::thread(WorkerMain);
  lib.inited = true;
}

void EnsureInit() {
  std::lock_guard<std::mutex> g(g_initMu);
  InitLocked(nullptr);
}

// ---- one wave of a job (caller holds gpuMu) --------------------------------
struct ProfSink {
  rad_job* job;
  void Begin(int kind, cudaEvent_t& a) {
    if (!job || !(job->flags & RAD_JOB_PROFILE_KERNELS)) return;
    a = GetEvent();
    cudaEventRecord(a, L().stream);
    (void)kind;
  }
  void End(int kind, cudaEvent_t a) {
    if (!job || !(job->flags & RAD_JOB_PROFILE_KERNELS)) return;
    cudaEvent_t b = GetEvent();
    cudaEventRecord(b, L().stream);
    job->profEv.push_back({a, b});
    job->profKind.push_back(kind);
  }
};

// ---- bdpt ---------------------------------------------------------------------

int BdptCap(const DevScene& S) {
  return S.maxDepth >= 0 ? std::min(kMaxBdptVertices, S.maxDepth + 2) : kMaxBdptVertices;
}

const VolWave& EnsureVolWave() {
  Lib& lib = L();
  if (lib.vol.state) return lib.vol;
  const uint32_t P = lib.maxPaths;
  VolWave V{};
  std::vector<void*> o;
  uint64_t b = 0;
  try {
    V.state = DevAlloc<uint8_t>((size_t)P * VolStateBytes(), o, b);
    V.q = DevAlloc<uint32_t>((size_t)2 * kVolActs * P, o, b);
    V.cnt = DevAlloc<uint32_t>(kVolCountWords, o, b);
    if (!lib.hVolWord) Check(cudaMallocHost(&lib.hVolWord, kVolCountWords * sizeof(uint32_t)), "cudaMallocHost");
  } catch (...) {
    FreeAll(o);  // nothing half-allocated stays behind
    throw;
  }
  V.capacity = P;
  lib.volAllocs = std::move(o);
  lib.volBytes = b;
  lib.used += b;
  lib.vol = V;
  return lib.vol;
}

const BdptBuffers& EnsureBdpt(int cap) {
  Lib& lib = L();
  if (lib.bdpt.vert && (int)lib.bdpt.cap == cap) return lib.bdpt;
  Check(cudaStreamSynchronize(lib.stream), "sync");
  FreeAll(lib.bdptAllocs);
  lib.used -= lib.bdptBytes;
  lib.bdptBytes = 0;
  uint64_t per = 2ull * cap * kBVertBytes + (uint64_t)cap * (3 * sizeof(float4) + 4) + 3 * sizeof(float4) + 20;
  // at most 2^24 samples a wave: a sorted connection packs its sample slot in 24 bits
  uint32_t nw = (uint32_t)std::min<uint64_t>(std::min<uint64_t>(lib.maxPaths, 1u << 24),
                                             std::max<uint64_t>(1024, lib.bdptScratch / per));
  BdptBuffers V{};
  auto& o = lib.bdptAllocs;
  uint64_t& b = lib.bdptBytes;
  V.vert = reinterpret_cast<BVert*>(DevAlloc<uint8_t>(2ull * cap * nw * kBVertBytes, o, b));
  V.walkA = DevAlloc<float4>(nw, o, b);
  V.walkB = DevAlloc<float4>(nw, o, b);
  V.fix = DevAlloc<float4>(nw, o, b);
  V.nCam = DevAlloc<uint32_t>(nw, o, b);
  V.nLight = DevAlloc<uint32_t>(nw, o, b);
  V.shCap = (uint32_t)std::min<uint64_t>(0xffffffffu, (uint64_t)nw * cap);
  V.shO = DevAlloc<float4>(V.shCap, o, b);
  V.shD = DevAlloc<float4>(V.shCap, o, b);
  V.shC = DevAlloc<float4>(V.shCap, o, b);
  V.order = DevAlloc<uint32_t>(nw, o, b);
  V.keyStart = DevAlloc<uint32_t>((size_t)(cap + 1) * (cap + 1) + 1, o, b);
  V.keyFill = DevAlloc<uint32_t>((size_t)(cap + 1) * (cap + 1), o, b);
  V.itemStart = DevAlloc<uint32_t>((size_t)(cap + 1) * (cap + 1) + 1, o, b);
  V.rng1 = DevAlloc<uint2>(nw, o, b);
  V.items = DevAlloc<uint32_t>((size_t)nw * cap, o, b);
  V.bucket = DevAlloc<uint32_t>(3 * kBdptBuckets + 1, o, b);
  V.cap = (uint32_t)cap;
  V.nw = nw;
  lib.bdpt = V;
  lib.used += b;
  return lib.bdpt;
}

// Zeroes the wave counters; keeps the device-error word and, with keepMaxCam,
// the longest-camera-subpath word.
void ResetCounters(const PathBuffers& B, bool keepMaxCam, cudaStream_t st) {
  size_t head = keepMaxCam ? (size_t)kMiscBase : (size_t)kMiscBase + 1;
  Check(cudaMemsetAsync(B.counters, 0, head * sizeof(uint32_t), st), "cudaMemsetAsync");
  Check(cudaMemsetAsync(B.counters + kMiscBase + 2, 0, (kCounterWords - kMiscBase - 2) * sizeof(uint32_t), st),
        "cudaMemsetAsync");
}

// One subpath bounce loop: extend + walk per depth until the queue empties.
uint64_t BdptWalks(const DevScene& S, const TraceTune& tu, uint32_t count, bool light, int cap, ProfSink& ps) {
  Lib& lib = L();
  const PathBuffers& B = lib.paths;
  const BdptBuffers& V = lib.bdpt;
  int grid = std::max(1, std::min(lib.sms * 8, (int)((count + 127) / 128)));
  int tgrid = std::max(1, std::min(lib.sms * tu.blocksPerSm, (int)((count + 127) / 128)));
  int iters = S.maxDepth >= 0 ? std::min(cap, S.maxDepth + 1) : cap;
  uint64_t launches = 0;
  for (int d = 0; d < iters; d++) {
    cudaEvent_t a = nullptr;
    ps.Begin(1, a);
    Check(LaunchExtend(S, B, d, tgrid, lib.stream, nullptr, tu.refillBusy, tu.leafFrac8), "extend");
    ps.End(1, a);
    ps.Begin(2, a);
    Check(LaunchBdptWalk(S, B, V, d, light, grid, lib.stream), "bdpt walk");
    ps.End(2, a);
    launches += 2;
    if (S.maxDepth < 0 && (d % 8) == 7) {
      uint32_t next = 0;
      Check(cudaMemcpyAsync(&next, B.counters + d + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, lib.stream), "copy");
      Check(cudaStreamSynchronize(lib.stream), "sync");
      if (next == 0) break;
    }
  }
  return launches;
}

// The bdpt stages for `w.count` (<= the scratch's wave size) pixel samples:
// film (splats and valid samples) and / or per-sample camera-side radiance `out`.
uint64_t RunBdptWave(const DevScene& S, const TraceTune& tu, const WaveParams& w, const FilmView& film, float* out,
                     ProfSink& ps) {
  Lib& lib = L();
  const int cap = BdptCap(S);
  const BdptBuffers& V = EnsureBdpt(cap);
  const PathBuffers& B = lib.paths;
  const uint32_t count = w.count;
  uint64_t launches = 0;
  cudaEvent_t a = nullptr;
  ResetCounters(B, false, lib.stream);
  ps.Begin(0, a);
  Check(LaunchBdptCamera(S, B, V, w, lib.stream), "bdpt camera");
  ps.End(0, a);
  launches += 1 + BdptWalks(S, tu, count, false, cap, ps);
  ResetCounters(B, true, lib.stream);
  ps.Begin(0, a);
  Check(LaunchBdptLight(S, B, V, count, lib.stream), "bdpt light");
  ps.End(0, a);
  launches += 1 + BdptWalks(S, tu, count, true, cap, ps);
  Check(cudaMemsetAsync(V.keyFill, 0, (size_t)(cap + 1) * (cap + 1) * sizeof(uint32_t), lib.stream), "cudaMemsetAsync");
  Check(cudaMemsetAsync(V.bucket, 0, kBdptBuckets * sizeof(uint32_t), lib.stream), "cudaMemsetAsync");
  Check(LaunchBdptLightFix(S, V, count, lib.stream), "bdpt light fix-up");
  uint32_t maxCam = 0;
  Check(cudaMemcpyAsync(&maxCam, B.counters + kMiscBase, sizeof(uint32_t), cudaMemcpyDeviceToHost, lib.stream), "copy");
  Check(cudaStreamSynchronize(lib.stream), "sync");
  launches += 3;
  int grid = lib.sms * 8;
  int tgrid = std::max(1, std::min(lib.sms * tu.blocksPerSm, (int)((count + 127) / 128)));
  for (int t = 1; t <= (int)maxCam && t <= cap; t++) {
    ps.Begin(2, a);
    if (t >= 2)
      Check(LaunchBdptConnectSplit(S, B, V, count, t, grid, lib.stream), "bdpt connect");
    else
      Check(LaunchBdptRound1(S, B, V, count, film.accum != nullptr, grid, lib.stream), "bdpt connect");
    ps.End(2, a);
    ps.Begin(3, a);
    Check(LaunchBdptShadow(S, B, V, t, film.accum, tgrid, lib.stream, tu.refillBusy, tu.leafFrac8), "bdpt shadow");
    ps.End(3, a);
    launches += t >= 2 ? 9 : 6;
  }
  ps.Begin(4, a);
  Check(LaunchBdptAccumulate(B, film, count, out, lib.stream), "bdpt accumulate");
  ps.End(4, a);
  return launches + 1;
}

// Launches the bounce loop for `count` generated paths. Returns kernels launched.
uint64_t LaunchBounces(const DevScene& S, const TraceTune& tu, uint32_t count, ProfSink& ps,
                       unsigned long long* trav = nullptr, const GuideDev* G = nullptr) {
  Lib& lib = L();
  uint64_t launches = 0;
  int grid = std::max(1, std::min(lib.sms * 8, (int)((count + 127) / 128)));
  int tgrid = std::max(1, std::min(lib.sms * tu.blocksPerSm, (int)((count + 127) / 128)));
  int iters = S.maxDepth >= 0 ? std::max(1, S.maxDepth) : kMaxBounce;
  if (iters > kMaxBounce) iters = kMaxBounce;
  if (S.isAO) {  // ao.cpp:22-36: first hit, one visibility ray
    cudaEvent_t a = nullptr;
    ps.Begin(1, a);
    Check(LaunchExtend(S, lib.paths, 0, tgrid, lib.stream, trav, tu.refillBusy, tu.leafFrac8), "extend");
    ps.End(1, a);
    ps.Begin(2, a);
    Check(LaunchShadeAO(S, lib.paths, grid, lib.stream), "ao");
    ps.End(2, a);
    ps.Begin(3, a);
    Check(LaunchShadow(S, lib.paths, 0, tgrid, lib.stream, trav, tu.refillBusy, tu.leafFrac8), "shadow");
    ps.End(3, a);
    return 3;
  }
  for (int d = 0; d < iters; d++) {
    cudaEvent_t a = nullptr;
    ps.Begin(1, a);
    Check(LaunchExtend(S, lib.paths, d, tgrid, lib.stream, trav, tu.refillBusy, tu.leafFrac8), "extend");
    ps.End(1, a);
    if (G) {
      ps.Begin(6, a);
      Check(LaunchGuideInfer(S, lib.paths, *G, d, count, lib.stream), "guide inference");
      ps.End(6, a);
      launches++;
    }
    ps.Begin(2, a);
    Check(LaunchShade(S, lib.paths, d, grid, lib.stream, G, false, tu.shadeBlock), "shade");
    ps.End(2, a);
    ps.Begin(3, a);
    Check(LaunchShadow(S, lib.paths, d, tgrid, lib.stream, trav, tu.refillBusy, tu.leafFrac8), "shadow");
    ps.End(3, a);
    launches += 2 + kShadeClasses;
    if (S.maxDepth < 0 && (d % 8) == 7) {
      // unbounded depth: stop once the next queue is empty
      Check(cudaMemcpyAsync(lib.hCounters, lib.paths.counters, (d + 2) * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                            lib.stream),
            "counter readback");
      Check(cudaStreamSynchronize(lib.stream), "sync");
      if (lib.hCounters[d + 1] == 0) break;
    }
  }
  return launches;
}

// Graph replay applies to fixed-depth `path` jobs without per-kernel profiling
// or traversal counting (those record events / host readbacks per launch).
bool GraphEligible(const rad_job* j) {
  const DevScene& S = j->scene->dev;
  return !S.isVol && S.maxDepth >= 0 &&
         !(j->flags & (RAD_JOB_PROFILE_KERNELS | RAD_JOB_COUNT_TRAVERSAL | RAD_JOB_GUIDE));
}

GuideNet& EnsureGuide(rad_scene* sc) {
  if (!sc->guide) {
    try {
      sc->guide = GuideCreate(sc->guideCfg, sc->worldLo, sc->worldHi);
    } catch (const std::runtime_error& e) {
      throw Error{RAD_ERR_CUDA, e.what()};
    }
    L().used += sc->guide->bytes;
  }
  return *sc->guide;
}

void EnsureGuideBuffers(Lib& lib, uint32_t recCap) {
  if (!lib.guideMix) {
    Check(cudaMalloc(&lib.guideMix, (size_t)lib.maxPaths * kGMixF4 * sizeof(float4)), "guide mixtures");
    lib.guideBytes += (uint64_t)lib.maxPaths * kGMixF4 * sizeof(float4);
  }
  if (lib.guideRecCap < recCap) {
    if (lib.guideRec) {
      cudaFree(lib.guideRec);
      lib.guideBytes -= (uint64_t)lib.guideRecCap * kGRecF4 * sizeof(float4);
    }
    lib.guideRec = nullptr;
    lib.guideRecCap = 0;
    Check(cudaMalloc(&lib.guideRec, (size_t)recCap * kGRecF4 * sizeof(float4)), "guide records");
    lib.guideRecCap = recCap;
    lib.guideBytes += (uint64_t)recCap * kGRecF4 * sizeof(float4);
  }
  lib.paths.guideRec = lib.guideRec;
}

// Training steps after a guided training wave: record weights, then
// cfg.stepsPerWave Adam steps, each on every stepsPerWave-th record.
// Adam steps on the wave's records: stepsPerWave per sample the wave holds, each
// on a strided batch (every S-th record), so steps and batch sizes per training
// sample do not depend on how many samples share a wave.
void GuideTrainWave(GuideNet& net, const GuideDev& G, ProfSink& ps, rad_job* j, uint32_t samples) {
  Lib& lib = L();
  cudaEvent_t a = nullptr;
  ps.Begin(7, a);
  Check(LaunchGuideFinalize(lib.paths, G, lib.stream), "guide finalize");
  uint32_t S = net.cfg.stepsPerWave * std::max(1u, samples);
  uint32_t maxBatch = (G.recCap + S - 1) / S;
  for (uint32_t s = 0; s < S; s++) {
    Check(LaunchGuideTrain(G, G.rec, G.ctl, 0, G.recCap, S, s, net.cfg.weightClamp, net.g, net.g + net.nTable,
                           reinterpret_cast<float*>(net.ctl + 2), maxBatch, lib.paths.counters + kMiscBase + 1,
                           lib.stream),
          "guide train");
    net.step++;
    Check(LaunchGuideAdam(net.p, net.m, net.v, net.g, net.ph, net.nParams, net.cfg.lr, net.nTable, net.cfg.lrMlp,
                          net.cfg.beta1, net.cfg.beta2, net.cfg.eps, 1.f, net.step, G.ctl, G.recCap, S, s,
                          net.cfg.lazyTable != 0, lib.stream),
          "guide adam");
  }
  ps.End(7, a);
  j->stats.kernel_launches += 1 + 2 * S;
  j->stats.guide_train_steps += S;
}

// A guided wave: the bounce loop with the guide inference stage, then (while
// the job is in its training fraction) the training steps on its records.
uint32_t WaveSamples(rad_job* j);

void RunWaveGuided(rad_job* j) {
  Lib& lib = L();
  const DevScene& S = j->scene->dev;
  GuideNet& net = EnsureGuide(j->scene);
  EnsureGuideBuffers(lib, net.cfg.recCap);
  uint32_t W = (uint32_t)S.cam.width, H = (uint32_t)S.cam.height;
  uint64_t npix = (uint64_t)W * H;
  ProfSink ps{j};
  FilmView film{j->accum, (int32_t)W, (int32_t)H, j->dStats};
  bool train = j->nextSample < j->trainSamples;
  // a small frame's wave holds several consecutive samples, as plain waves do; a training wave holds
  // at most 4 (the guide learns between waves, so the samples it shades stay close to its current
  // state), stops at the end of the training fraction, and its Adam steps scale with its samples
  uint32_t k = std::min(WaveSamples(j), j->spp - j->nextSample);
  if (train) k = std::min(std::min(k, 4u), j->trainSamples - j->nextSample);
  for (uint64_t p0 = 0; p0 < npix; p0 += lib.maxPaths) {
    uint32_t count = (uint32_t)std::min<uint64_t>(lib.maxPaths, npix - p0) * k;
    uint32_t smp = j->first + j->nextSample;
    WaveParams w{(uint32_t)p0, count, smp, j->seed, nullptr, nullptr, nullptr, k};
    GuideDev G = GuideView(net);
    G.mix = lib.guideMix;
    G.rec = lib.guideRec;
    G.recCap = net.cfg.recCap;
    G.train = train ? 1u : 0u;
    G.trainSalt = GuideHash32(smp * 0x9e3779b9u + j->seed * 0x85ebca6bu + (uint32_t)p0);
    G.recTotal = j->dStats + 8;
    if (train) Check(cudaMemsetAsync(net.ctl, 0, 4 * sizeof(uint32_t), lib.stream), "guide control reset");
    cudaEvent_t a = nullptr;
    ps.Begin(0, a);
    Check(LaunchGenerate(S, lib.paths, w, lib.stream), "generate");
    ps.End(0, a);
    uint64_t launches = 1 + LaunchBounces(S, j->scene->tune, count, ps, nullptr, &G);
    ps.Begin(4, a);
    Check(LaunchAccumulate(lib.paths, film, count, lib.stream, nullptr, k), "accumulate");
    ps.End(4, a);
    launches++;
    j->stats.kernel_launches += launches;
    if (train) GuideTrainWave(net, G, ps, j, k);
  }
  j->nextSample += k;
  j->launched += npix * k;
}

// Runs the job's next sample over its pixels as replays of one captured graph
// per chunk (generate, bounces, accumulate); the accumulate stage advances the
// sample index held in the chunk's device WaveCtx.
// Samples per wave of a job: a frame that fills less than half of the path
// slots gets several consecutive samples per wave (up to its spp), so small
// jobs run in few full waves instead of many nearly empty ones.
uint32_t WaveSamples(rad_job* j) {
  if (j->spw == 0) {
    const DevScene& S = j->scene->dev;
    uint64_t npix = (uint64_t)S.cam.width * S.cam.height;
    uint64_t cap = L().maxPaths;
    j->spw = (npix == 0 || npix * 2 > cap) ? 1u : (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(j->spp, cap / npix));
  }
  return j->spw;
}

void RunWaveGraph(rad_job* j) {
  Lib& lib = L();
  const DevScene& S = j->scene->dev;
  uint32_t W = (uint32_t)S.cam.width, H = (uint32_t)S.cam.height;
  uint64_t npix = (uint64_t)W * H;
  const uint32_t spw = WaveSamples(j);
  size_t nChunks = (size_t)((npix + lib.maxPaths - 1) / lib.maxPaths);
  auto uploadCtx = [&]() {
    std::vector<WaveCtx> host(nChunks);
    for (auto& c : host) {
      c = WaveCtx{};
      c.film = j->accum;
      c.stats = j->dStats;
      c.sample = j->first + j->nextSample;
      c.seed = j->seed;
    }
    // stream-ordered: an earlier wave of this job may still be reading the context
    Check(cudaMemcpyAsync(j->ctx, host.data(), nChunks * sizeof(WaveCtx), cudaMemcpyHostToDevice, lib.stream),
          "ctx upload");
  };
  if (j->ctxStale && !j->graphs.empty()) {
    uploadCtx();
    j->ctxStale = false;
  }
  if (j->graphs.empty()) {
    Check(cudaMalloc(&j->ctx, nChunks * sizeof(WaveCtx)), "cudaMalloc");
    uploadCtx();
    j->ctxStale = false;
    ProfSink none{nullptr};
    FilmView film{j->accum, (int32_t)W, (int32_t)H, j->dStats};
    for (size_t c = 0; c < nChunks; c++) {
      uint64_t p0 = (uint64_t)c * lib.maxPaths;
      uint32_t count = (uint32_t)std::min<uint64_t>(lib.maxPaths, npix - p0) * spw;
      WaveParams w{(uint32_t)p0, count, 0, 0, nullptr, nullptr, j->ctx + c, spw};
      cudaGraph_t g = nullptr;
      Check(cudaStreamBeginCapture(lib.stream, cudaStreamCaptureModeThreadLocal), "begin capture");
      cudaError_t e1 = LaunchGenerate(S, lib.paths, w, lib.stream);
      uint64_t k = 1 + LaunchBounces(S, j->scene->tune, count, none);
      cudaError_t e2 = LaunchAccumulate(lib.paths, film, count, lib.stream, j->ctx + c, spw);
      cudaError_t e3 = cudaStreamEndCapture(lib.stream, &g);
      Check(e1, "generate capture");
      Check(e2, "accumulate capture");
      Check(e3, "end capture");
      cudaGraphExec_t ex = nullptr;
      cudaError_t e4 = cudaGraphInstantiate(&ex, g, 0);
      cudaGraphDestroy(g);
      Check(e4, "graph instantiate");
      j->graphs.push_back(ex);
      j->graphKernels.push_back(k + 1);
    }
  }
  for (size_t c = 0; c < j->graphs.size(); c++) {
    Check(cudaGraphLaunch(j->graphs[c], lib.stream), "graph launch");
    j->stats.kernel_launches += j->graphKernels[c];
  }
  j->nextSample += spw;
  j->launched += npix * spw;
}

// particle_tracer jobs: the next batch of light paths (ParticleTracer::Render,
// particle_tracer.cpp:39-83; one "sample" = one light path for the whole film),
// as a wavefront: starts, then per bounce closest hit, bounce and the round's
// camera-connection visibility rays.
void RunWaveParticle(rad_job* j) {
  Lib& lib = L();
  const DevScene& S = j->scene->dev;
  const TraceTune& tu = j->scene->tune;
  const PathBuffers& B = lib.paths;
  uint64_t npix = (uint64_t)S.cam.width * S.cam.height;
  const uint32_t k = std::min<uint32_t>(lib.maxPaths, j->spp - j->nextSample);
  const float scale = (float)npix / (float)j->spp;
  ParticleParams pp{(uint64_t)j->first + j->nextSample, k, j->seed, scale};
  BdptBuffers sh{};  // the visibility rays of a round live in the path state's shadow records
  sh.shO = B.shO;
  sh.shD = B.shD;
  sh.shC = B.shC;
  sh.shCap = B.capacity;
  ProfSink ps{j};
  cudaEvent_t a = nullptr;
  int grid = std::max(1, std::min(lib.sms * 8, (int)((k + 127) / 128)));
  int tgrid = std::max(1, std::min(lib.sms * tu.blocksPerSm, (int)((k + 127) / 128)));
  ResetCounters(B, false, lib.stream);
  ps.Begin(0, a);
  Check(LaunchParticleStart(S, B, pp, j->dStats, lib.stream), "particle start");
  ps.End(0, a);
  ps.Begin(3, a);
  Check(LaunchBdptShadow(S, B, sh, 1, j->accum, tgrid, lib.stream, tu.refillBusy, tu.leafFrac8), "particle splats");
  ps.End(3, a);
  uint64_t launches = 2;
  // bounce d tests depth d + 1 against max_depth before it does anything
  const int iters = S.maxDepth >= 0 ? std::min(kMaxLightBounces, std::max(0, S.maxDepth - 1)) : kMaxLightBounces;
  for (int d = 0; d < iters; d++) {
    ps.Begin(1, a);
    Check(LaunchExtend(S, B, d, tgrid, lib.stream, nullptr, tu.refillBusy, tu.leafFrac8), "extend");
    ps.End(1, a);
    ps.Begin(2, a);
    Check(LaunchParticleBounce(S, B, d, scale, grid, lib.stream), "particle bounce");
    ps.End(2, a);
    ps.Begin(3, a);
    Check(LaunchBdptShadow(S, B, sh, d + 2, j->accum, tgrid, lib.stream, tu.refillBusy, tu.leafFrac8),
          "particle splats");
    ps.End(3, a);
    launches += 3;
    if (S.maxDepth < 0 && (d % 8) == 7) {
      uint32_t next = 0;
      Check(cudaMemcpyAsync(&next, B.counters + d + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, lib.stream), "copy");
      Check(cudaStreamSynchronize(lib.stream), "sync");
      if (next == 0) break;
    }
  }
  j->stats.kernel_launches += launches;
  j->nextSample += k;
  j->launched += k;
}

// bdpt jobs (BDPT::Render, bdpt.cpp:261-305): the wavefront stages over the
// job's pixels, as many consecutive samples per wave as the scratch holds.
void RunWaveBdpt(rad_job* j) {
  const DevScene& S = j->scene->dev;
  const uint64_t npix = (uint64_t)S.cam.width * S.cam.height;
  const uint32_t nw = EnsureBdpt(BdptCap(S)).nw;
  const uint32_t k = npix * 2 > nw ? 1u : (uint32_t)std::min<uint64_t>(j->spp - j->nextSample, nw / npix);
  FilmView film{j->accum, S.cam.width, S.cam.height, j->dStats};
  ProfSink ps{j};
  const uint64_t chunk = nw / k;
  for (uint64_t p0 = 0; p0 < npix; p0 += chunk) {
    uint32_t count = (uint32_t)std::min<uint64_t>(chunk, npix - p0) * k;
    WaveParams w{(uint32_t)p0, count, j->first + j->nextSample, j->seed, nullptr, nullptr, nullptr, k};
    j->stats.kernel_launches += RunBdptWave(S, j->scene->tune, w, film, nullptr, ps);
  }
  j->nextSample += k;
  j->launched += npix * k;
}

// Jobs whose waves can share launches with other jobs' (mixed waves): plain
// `path` jobs of bounded depth, without guiding, profiling or traversal counts.
bool Mixable(const rad_job* j) {
  const DevScene& S = j->scene->dev;
  return !S.isVol && !S.isAO && !S.isParticle && !S.isBdpt && S.maxDepth >= 0 &&
         !(j->flags & (RAD_JOB_GUIDE | RAD_JOB_PROFILE_KERNELS | RAD_JOB_COUNT_TRAVERSAL));
}

// One wave holding paths of several jobs (of any scenes). With a deadline
// allowance set (earliest deadline first) or a slowdown estimate (highest
// slowdown first), js comes in that order and each job in turn takes what it
// can use of half the slots still free. Otherwise the path slots are
// split between the jobs in proportion to (remaining samples)^shareExp --
// exponent 0, equal shares (processor sharing: every job's slowdown is about
// the same); exponent 1, shares in proportion to the work left (jobs running
// together finish together: latencies even out across job sizes) -- and a
// share a job cannot use goes to the others. A job whose share covers its frame takes whole
// samples (as many consecutive ones as fit); otherwise it takes the next pixel
// chunk of its current sample, so each pixel still receives its samples in
// order and the film is the same as when the job runs alone. Every stage is one
// launch over all jobs' paths; each path finds its scene, film, pixels and
// stream through the wave's job table.
void RunMixedWave(const std::vector<rad_job*>& js) {
  Lib& lib = L();
  const uint64_t P = lib.maxPaths;
  const size_t m = js.size();
  std::vector<uint64_t> need(m), give(m, 0);
  for (size_t i = 0; i < m; i++) {
    const DevScene& S = js[i]->scene->dev;
    const uint64_t npix = (uint64_t)S.cam.width * S.cam.height;
    need[i] = (uint64_t)(js[i]->spp - js[i]->nextSample) * npix - js[i]->mixCursor;
  }
  uint64_t left = P;
  if (lib.edfNsPerSample > 0 || lib.slowNsPerSample > 0) {
    // earliest deadline / highest slowdown first (js is in that order): each job in turn takes what it can use of half
    // the slots still free (the last one all of them), so a job that missed its deadline -- and stays
    // first until it ends -- cannot hold every slot while later, nearer-deadline jobs wait
    for (size_t i = 0; i < m && left > 0; i++) {
      const uint64_t cap = i + 1 == m ? left : std::max<uint64_t>(left / 2, std::min<uint64_t>(left, 65536));
      give[i] = std::min(need[i], cap);
      left -= give[i];
    }
  } else if (lib.shareExp != 0.f && m > 1) {
    std::vector<double> w(m);
    double sum = 0;
    for (size_t i = 0; i < m; i++) sum += (w[i] = std::pow((double)std::max<uint64_t>(need[i], 1), lib.shareExp));
    for (size_t i = 0; i < m; i++) {
      uint64_t g = std::min<uint64_t>(need[i], std::max<uint64_t>(1, (uint64_t)((double)P * w[i] / sum)));
      g = std::min(g, left);
      give[i] = g;
      left -= g;
    }
  }
  for (int pass = 0; pass < 3 && left > 0; pass++) {
    size_t open = 0;
    for (size_t i = 0; i < m; i++) open += give[i] < need[i] ? 1 : 0;
    if (open == 0) break;
    const uint64_t share = std::max<uint64_t>(1, left / open);
    for (size_t i = 0; i < m && left > 0; i++) {
      if (give[i] >= need[i]) continue;
      uint64_t g = std::min(std::min(share, need[i] - give[i]), left);
      give[i] += g;
      left -= g;
    }
  }
  MixJob* tab = lib.mixHost + (size_t)lib.mixSlot * kMaxMix;
  MixJob* dtab = lib.mixDev + (size_t)lib.mixSlot * kMaxMix;
  lib.mixSlot = (lib.mixSlot + 1) % kMixRing;
  uint32_t n = 0, pathBegin = 0, totalPix = 0;
  int maxDepth = 1;
  for (size_t i = 0; i < m; i++) {
    if (give[i] == 0) continue;
    rad_job* j = js[i];
    const DevScene& S = j->scene->dev;
    const uint32_t npix = (uint32_t)S.cam.width * (uint32_t)S.cam.height;
    MixJob& J = tab[n++];
    J = MixJob{};
    J.S = S;
    J.film = j->accum;
    J.stats = j->dStats;
    J.seed = j->seed;
    J.sample = j->first + j->nextSample;
    if (j->mixCursor == 0 && give[i] >= npix) {
      J.pixelBegin = 0;
      J.npc = npix;
      J.spw = (uint32_t)std::min<uint64_t>(give[i] / npix, j->spp - j->nextSample);
      j->nextSample += J.spw;
    } else {
      J.pixelBegin = j->mixCursor;
      J.npc = (uint32_t)std::min<uint64_t>(give[i], npix - j->mixCursor);
      J.spw = 1;
      j->mixCursor += J.npc;
      if (j->mixCursor == npix) {
        j->mixCursor = 0;
        j->nextSample++;
      }
    }
    J.count = J.npc * J.spw;
    J.pathBegin = pathBegin;
    pathBegin += J.count;
    totalPix += J.npc;
    j->launched += J.count;
    j->ctxStale = true;  // its graph waves, if any, must re-read the sample index
    maxDepth = std::max(maxDepth, S.maxDepth);
  }
  if (n == 0) return;
  Check(cudaMemcpyAsync(dtab, tab, n * sizeof(MixJob), cudaMemcpyHostToDevice, lib.stream), "job table");
  PathBuffers B = lib.paths;
  B.mix = dtab;
  const uint32_t count = pathBegin;
  const TraceTune& tu = js[0]->scene->tune;
  const DevScene& S0 = tab[0].S;  // not read by the mixed kernels; launch argument only
  int grid = std::max(1, std::min(lib.sms * 8, (int)((count + 127) / 128)));
  int tgrid = std::max(1, std::min(lib.sms * tu.blocksPerSm, (int)((count + 127) / 128)));
  const int iters = std::min(maxDepth, kMaxBounce);
  Check(LaunchGenerateMix(B, count, n, lib.stream), "generate");
  for (int d = 0; d < iters; d++) {
    Check(LaunchExtend(S0, B, d, tgrid, lib.stream, nullptr, tu.refillBusy, tu.leafFrac8, true), "extend");
    Check(LaunchShade(S0, B, d, grid, lib.stream, nullptr, true, tu.shadeBlock), "shade");
    Check(LaunchShadow(S0, B, d, tgrid, lib.stream, nullptr, tu.refillBusy, tu.leafFrac8, true), "shadow");
  }
  Check(LaunchAccumulateMix(B, totalPix, count, n, lib.stream), "accumulate");
  const uint64_t launches = 2 + (uint64_t)iters * (2 + kShadeClasses);
  for (size_t i = 0; i < m; i++)
    if (give[i] > 0) {
      js[i]->stats.kernel_launches += launches;
      if (n > 1) js[i]->stats.mixed_waves++;
    }
}

// Runs wave(s) for the job's next sample index over all its pixels.
void RunWave(rad_job* j) {
  if (j->scene->dev.isParticle) {
    RunWaveParticle(j);
    return;
  }
  if (j->scene->dev.isBdpt) {
    RunWaveBdpt(j);
    return;
  }
  const uint32_t spw = WaveSamples(j);
  if (GraphEligible(j) && j->spp - j->nextSample >= spw) {
    RunWaveGraph(j);
    return;
  }
  if ((j->flags & RAD_JOB_GUIDE) && !j->scene->dev.isVol) {
    RunWaveGuided(j);
    return;
  }
  Lib& lib = L();
  const DevScene& S = j->scene->dev;
  uint32_t W = (uint32_t)S.cam.width, H = (uint32_t)S.cam.height;
  uint64_t npix = (uint64_t)W * H;
  ProfSink ps{j};
  FilmView film{j->accum, (int32_t)W, (int32_t)H, j->dStats};
  const uint32_t k = std::min(spw, j->spp - j->nextSample);  // samples in this wave
  for (uint64_t p0 = 0; p0 < npix; p0 += lib.maxPaths) {
    uint32_t count = (uint32_t)std::min<uint64_t>(lib.maxPaths, npix - p0) * k;
    WaveParams w{(uint32_t)p0, count, j->first + j->nextSample, j->seed, nullptr, nullptr, nullptr, k};
    cudaEvent_t a = nullptr;
    ps.Begin(0, a);
    Check(LaunchGenerate(S, lib.paths, w, lib.stream), "generate");
    ps.End(0, a);
    uint64_t launches = 1;
    if (S.isVol) {
      ps.Begin(5, a);
      uint32_t mode = ((j->flags & RAD_JOB_VOL_BRICKS) ? kVolBricks : 0u) | ((j->flags & RAD_JOB_VOL_FP16) ? kVolHalf : 0u) |
                      ((j->flags & RAD_JOB_VOL_REAL_DEPTH) ? kVolRealDepth : 0u);
      uint32_t* err = lib.paths.counters + kMiscBase + 1;
      if (j->flags & RAD_JOB_VOL_PERSISTENT) {
        Check(LaunchVolPath(S, lib.paths, w, err, lib.stream, mode), "vol_path");
        launches++;
      } else {
        Check(LaunchVolWavefront(S, lib.paths, EnsureVolWave(), w, err, lib.stream, mode, j->scene->tune,
                                 lib.hVolWord, &launches),
              "vol_path wavefront");
      }
      ps.End(5, a);
    } else {
      launches += LaunchBounces(S, j->scene->tune, count, ps,
                                (j->flags & RAD_JOB_COUNT_TRAVERSAL) ? j->dStats + 4 : nullptr);
    }
    ps.Begin(4, a);
    Check(LaunchAccumulate(lib.paths, film, count, lib.stream, nullptr, k), "accumulate");
    ps.End(4, a);
    launches++;
    j->stats.kernel_launches += launches;
  }
  j->nextSample += k;
  j->launched += npix * k;
}

void FinishJob(rad_job* j, int status, const std::string& err) {
  Lib& lib = L();
  if (j->accum) {
    // film memory stays until rad_job_destroy (the user reads it after wait)
  }
  {
    std::lock_guard<std::mutex> g(j->m);
    j->status = status;
    j->err = err;
    j->state = kDone;
    j->tEnd = NowMs();
  }
  j->cv.notify_all();
  (void)lib;
}

void CompleteJob(rad_job* j) {
  // called after evEnd completed
  float ms = 0;
  if (j->evStart && j->evEnd) cudaEventElapsedTime(&ms, j->evStart, j->evEnd);
  j->stats.gpu_ms = ms;
  j->stats.rays_closest = j->hStats[0];
  j->stats.rays_shadow = j->hStats[1];
  j->stats.invalid_samples = j->hStats[2];
  j->stats.samples = j->hStats[3];
  j->stats.trav_nodes_closest = j->hStats[4];
  j->stats.trav_prims_closest = j->hStats[5];
  j->stats.trav_nodes_shadow = j->hStats[6];
  j->stats.trav_prims_shadow = j->hStats[7];
  j->stats.guide_records = j->hStats[8];
  double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  uint64_t cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (size_t k = 0; k < j->profEv.size(); k++) {
    float e = 0;
    cudaEventElapsedTime(&e, j->profEv[k].first, j->profEv[k].second);
    acc[j->profKind[k]] += e;
    cnt[j->profKind[k]]++;
    L().evPool.push_back(j->profEv[k].first);
    L().evPool.push_back(j->profEv[k].second);
  }
  j->profEv.clear();
  j->profKind.clear();
  j->stats.ms_generate = acc[0];
  j->stats.ms_extend = acc[1];
  j->stats.ms_shade = acc[2];
  j->stats.ms_shadow = acc[3];
  j->stats.ms_accumulate = acc[4];
  j->stats.ms_volpath = acc[5];
  j->stats.ms_guide_infer = acc[6];
  j->stats.ms_guide_train = acc[7];
  j->stats.n_extend = cnt[1];
  j->stats.n_shade = cnt[2];
  j->stats.n_shadow = cnt[3];
  uint32_t errWord = 0;
  cudaMemcpy(&errWord, L().paths.counters + kMiscBase + 1, 4, cudaMemcpyDeviceToHost);
  if (errWord) cudaMemset(L().paths.counters + kMiscBase + 1, 0, 4);
  j->stats.wall_ms = NowMs() - j->tStart;
  j->stats.queue_ms = j->tStart - j->tSubmit;
  if (errWord) {
    FinishJob(j, RAD_ERR_DEVICE_CHECK, "device-side check fired (traversal stack or iteration bound), code " +
                                           std::to_string(errWord));
    return;
  }
  FinishJob(j, j->cancel ? RAD_ERR_CANCELLED : RAD_OK, j->cancel ? "job cancelled" : "");
}

bool AdmitFilm(rad_job* j) {
  Lib& lib = L();
  uint64_t need = j->filmBytes;
  uint64_t cur = lib.used.load();
  if (cur + need > lib.budget) return false;
  lib.used += need;
  return true;
}

void FreeSpareGraphs(JobSpare& sp) {
  for (cudaGraphExec_t g : sp.graphs) cudaGraphExecDestroy(g);
  if (sp.ctx) cudaFree(sp.ctx);
  sp.graphs.clear();
  sp.graphKernels.clear();
  sp.ctx = nullptr;
}

void FreeSpare(rad_scene* sc) {
  JobSpare& sp = sc->spare;
  if (!sp.valid) return;
  Lib& lib = L();
  lib.used -= sp.bytes;
  lib.spareBytes -= sp.bytes;
  lib.spareScenes.erase(std::find(lib.spareScenes.begin(), lib.spareScenes.end(), sc));
  FreeSpareGraphs(sp);
  if (sp.accum) cudaFree(sp.accum);
  if (sp.dStats) cudaFree(sp.dStats);
  if (sp.hStats) cudaFreeHost(sp.hStats);
  if (sp.resolve) cudaFree(sp.resolve);
  if (sp.evStart) cudaEventDestroy(sp.evStart);
  if (sp.evEnd) cudaEventDestroy(sp.evEnd);
  sp = JobSpare{};
}

// Frees every parked film (caller holds gpuMu). Admission calls this before it
// refuses a scene or a job, so parked films never keep work out.
void ReleaseSpares() {
  Lib& lib = L();
  while (!lib.spareScenes.empty()) FreeSpare(lib.spareScenes.back());
}

void AllocJobFilm(rad_job* j) {
  const DevScene& S = j->scene->dev;
  size_t npix = (size_t)S.cam.width * S.cam.height;
  JobSpare& sp = j->scene->spare;
  if (sp.valid) {  // take over the previous job's buffers (same scene: same film size)
    j->accum = sp.accum;
    j->dStats = sp.dStats;
    j->hStats = sp.hStats;
    j->resolve = sp.resolve;
    j->evStart = sp.evStart;
    j->evEnd = sp.evEnd;
    if (!sp.graphs.empty() && GraphEligible(j) && sp.spw == WaveSamples(j) && sp.tuneEpoch == j->scene->tuneEpoch) {
      j->ctx = sp.ctx;
      j->graphs = std::move(sp.graphs);
      j->graphKernels = std::move(sp.graphKernels);
      j->ctxStale = true;
      sp.ctx = nullptr;
    }
    FreeSpareGraphs(sp);
    // the job's own admission counted its film: drop the spare's count
    Lib& lib = L();
    lib.used -= sp.bytes;
    lib.spareBytes -= sp.bytes;
    lib.spareScenes.erase(std::find(lib.spareScenes.begin(), lib.spareScenes.end(), j->scene));
    sp = JobSpare{};
    std::memset(j->hStats, 0, kJobStatWords * sizeof(unsigned long long));
    Check(cudaMemsetAsync(j->accum, 0, npix * sizeof(float4), L().stream), "memset film");
    Check(cudaMemsetAsync(j->dStats, 0, kJobStatWords * sizeof(unsigned long long), L().stream), "memset stats");
    return;
  }
  Check(cudaMalloc(&j->accum, npix * sizeof(float4)), "film");
  Check(cudaMalloc(&j->dStats, kJobStatWords * sizeof(unsigned long long)), "stats");
  Check(cudaMallocHost(&j->hStats, kJobStatWords * sizeof(unsigned long long)), "stats host");
  std::memset(j->hStats, 0, kJobStatWords * sizeof(unsigned long long));
  Check(cudaMemsetAsync(j->accum, 0, npix * sizeof(float4), L().stream), "memset film");
  Check(cudaMemsetAsync(j->dStats, 0, kJobStatWords * sizeof(unsigned long long), L().stream), "memset stats");
  Check(cudaEventCreate(&j->evStart), "event");
  Check(cudaEventCreate(&j->evEnd), "event");
}

// Runs a job to completion on the calling thread (RAD_JOB_SYNC or worker).
void StartJob(rad_job* j) {
  AllocJobFilm(j);
  j->tStart = NowMs();
  Check(cudaEventRecord(j->evStart, L().stream), "event record");
  j->state = kRunning;
}

void EndJobLaunch(rad_job* j) {
  Check(cudaMemcpyAsync(j->hStats, j->dStats, kJobStatWords * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                        L().stream),
        "stats readback");
  Check(cudaEventRecord(j->evEnd, L().stream), "event record");
  j->state = kCompleting;
}

// The worker keeps at most kMaxWavesInFlight waves queued on the stream ahead
// of the GPU. Bounding the run-ahead keeps scheduling decisions late: a job
// that arrives (or is cancelled) meanwhile waits at most this many waves,
// instead of behind every wave already enqueued.

void WorkerMain() {
  Lib& lib = L();
  cudaSetDevice(lib.device);
  std::vector<rad_job*> completing;
  std::deque<cudaEvent_t> inflight;  // one event per queued wave
  auto release = [&](cudaEvent_t e) {
    std::lock_guard<std::mutex> g(lib.gpuMu);
    lib.evPool.push_back(e);
  };
  for (;;) {
    while (!inflight.empty() && cudaEventQuery(inflight.front()) == cudaSuccess) {
      release(inflight.front());
      inflight.pop_front();
    }
    while (inflight.size() >= kMaxWavesInFlight) {
      cudaEventSynchronize(inflight.front());
      release(inflight.front());
      inflight.pop_front();
    }
    rad_job* j = nullptr;
    std::vector<rad_job*> group;  // jobs of the next mixed wave
    bool reclaim = false;  // a pending job waits for memory that parked films hold
    {
      std::unique_lock<std::mutex> lk(lib.qmu);
      // admission: films that fit the budget join the running set
      for (auto it = lib.pending.begin(); it != lib.pending.end();) {
        rad_job* p = *it;
        if (p->cancel) {
          it = lib.pending.erase(it);
          FinishJob(p, RAD_ERR_CANCELLED, "job cancelled before admission");
          continue;
        }
        if (AdmitFilm(p)) {
          lib.running.push_back(p);
          p->state = kRunning;
          it = lib.pending.erase(it);
          continue;
        }
        if (lib.spareBytes.load() > 0) {
          reclaim = true;
          ++it;
          continue;
        }
        if (lib.running.empty() && completing.empty()) {
          // nothing running can free memory: this job can never be admitted
          it = lib.pending.erase(it);
          FinishJob(p, RAD_ERR_ADMISSION, "job film exceeds the device budget");
          continue;
        }
        ++it;
      }
      if (lib.running.empty() && completing.empty() && !reclaim) {
        if (lib.stop) break;
        lib.qcv.wait(lk);
        continue;
      }
      if (!lib.running.empty()) {
        // Plain `path` jobs share mixed waves once two of them run (or one has
        // a sample left half done by one); the other jobs keep waves of their
        // own. Between those and the mix group (counted by its least-served
        // member), least attained service decides: the fewest samples
        // launched goes next, ties to the earlier job.
        std::vector<rad_job*> mixable;
        if (lib.mixJobs)
          for (rad_job* c : lib.running)
            if (Mixable(c) && !c->cancel && c->nextSample < c->spp) mixable.push_back(c);
        const bool useGroup = mixable.size() >= 2 || (mixable.size() == 1 && mixable[0]->mixCursor != 0);
        uint64_t best = UINT64_MAX;
        for (rad_job* c : lib.running) {
          if (useGroup && std::find(mixable.begin(), mixable.end(), c) != mixable.end()) continue;
          if (c->launched.load() < best) {
            best = c->launched.load();
            j = c;
          }
        }
        if (useGroup) {
          std::stable_sort(mixable.begin(), mixable.end(),
                           [](rad_job* a, rad_job* b) { return a->launched.load() < b->launched.load(); });
          const bool groupFirst = !j || mixable[0]->launched.load() <= best;
          if (lib.slowNsPerSample > 0) {
            // highest slowdown so far first: age over the job's expected time alone
            const double now = NowMs(), k = lib.slowNsPerSample * 1e-6;
            auto slow = [&](rad_job* x) { return (now - x->tSubmit) / ((double)x->total * k + 20.0); };
            std::stable_sort(mixable.begin(), mixable.end(), [&](rad_job* a, rad_job* b) { return slow(a) > slow(b); });
          } else if (lib.edfNsPerSample > 0) {
            std::stable_sort(mixable.begin(), mixable.end(),
                             [](rad_job* a, rad_job* b) { return a->deadline < b->deadline; });
          }
          if (groupFirst) {
            if (mixable.size() > (size_t)kMaxMix) mixable.resize(kMaxMix);
            group = mixable;
            j = nullptr;
          }
        }
      }
    }
    if (reclaim) {
      std::lock_guard<std::mutex> g(lib.gpuMu);
      ReleaseSpares();
      continue;  // admission again, with the parked films' memory free
    }
    if (!group.empty()) {
      std::lock_guard<std::mutex> g(lib.gpuMu);
      try {
        for (rad_job* c : group)
          if (!c->accum) StartJob(c);
        RunMixedWave(group);
        cudaEvent_t e = GetEvent();
        Check(cudaEventRecord(e, lib.stream), "event record");
        inflight.push_back(e);
        for (rad_job* c : group) {
          if (c->nextSample >= c->spp && c->mixCursor == 0) {
            EndJobLaunch(c);
            std::lock_guard<std::mutex> lk(lib.qmu);
            lib.running.erase(std::find(lib.running.begin(), lib.running.end(), c));
            completing.push_back(c);
          }
        }
      } catch (const Error& e) {
        std::lock_guard<std::mutex> lk(lib.qmu);
        for (rad_job* c : group) {
          auto it = std::find(lib.running.begin(), lib.running.end(), c);
          if (it != lib.running.end()) {
            lib.running.erase(it);
            FinishJob(c, e.code, e.msg);
          }
        }
      }
    }
    if (j) {
      std::lock_guard<std::mutex> g(lib.gpuMu);
      try {
        if (!j->accum) StartJob(j);
        if (!j->cancel && j->nextSample < j->spp) {
          RunWave(j);
          cudaEvent_t e = GetEvent();
          Check(cudaEventRecord(e, lib.stream), "event record");
          inflight.push_back(e);
        }
        if (j->cancel || j->nextSample >= j->spp) {
          EndJobLaunch(j);
          std::lock_guard<std::mutex> lk(lib.qmu);
          lib.running.erase(std::find(lib.running.begin(), lib.running.end(), j));
          completing.push_back(j);
        }
      } catch (const Error& e) {
        std::lock_guard<std::mutex> lk(lib.qmu);
        auto it = std::find(lib.running.begin(), lib.running.end(), j);
        if (it != lib.running.end()) lib.running.erase(it);
        FinishJob(j, e.code, e.msg);
      }
    }
    // retire finished jobs
    for (auto it = completing.begin(); it != completing.end();) {
      rad_job* c = *it;
      cudaError_t q = cudaEventQuery(c->evEnd);
      if (q == cudaSuccess) {
        std::lock_guard<std::mutex> g(lib.gpuMu);
        CompleteJob(c);
        it = completing.erase(it);
      } else if (q == cudaErrorNotReady) {
        ++it;
      } else {
        FinishJob(c, RAD_ERR_CUDA, cudaGetErrorString(q));
        it = completing.erase(it);
      }
    }
    if (!j && group.empty() && !completing.empty()) std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
  for (cudaEvent_t e : inflight) {
    cudaEventSynchronize(e);
    release(e);
  }
}

uint64_t SceneUpload(const HostScene& hs, rad_scene* sc) {
  DevScene& D = sc->dev;
  auto& o = sc->allocs;
  uint64_t b = 0;
  auto up = [&](auto* dst, const auto& v) {
    if (!v.empty()) Check(cudaMemcpy(dst, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice), "upload");
  };
  Bvh8Node* nodes = DevAlloc<Bvh8Node>(hs.nodes.size(), o, b);
  PrimRec* prims = DevAlloc<PrimRec>(hs.prims.size(), o, b);
  uint32_t* pinfo = DevAlloc<uint32_t>(hs.primInfo.size(), o, b);
  ShapeRec* shapes = DevAlloc<ShapeRec>(hs.shapes.size(), o, b);
  MatRec* mats = DevAlloc<MatRec>(hs.mats.size(), o, b);
  LightRec* lights = DevAlloc<LightRec>(hs.lights.size(), o, b);
  MediumRec* media = DevAlloc<MediumRec>(hs.media.size(), o, b);
  float* pos = DevAlloc<float>(hs.pos.size(), o, b);
  float* nrm = DevAlloc<float>(hs.nrm.size(), o, b);
  float* uv = DevAlloc<float>(hs.uv.size(), o, b);
  uint32_t* idx = DevAlloc<uint32_t>(hs.idx.size(), o, b);
  float* cdf = DevAlloc<float>(hs.cdf.size(), o, b);
  float* vol = DevAlloc<float>(hs.volume.size(), o, b);
  uint16_t* volHalf = DevAlloc<uint16_t>(hs.volume.size(), o, b);
  float* bricks = DevAlloc<float>(hs.brickMaj.size(), o, b);
  uint8_t* scls = DevAlloc<uint8_t>(hs.shapeClass.size(), o, b);
  TexRec* tex = DevAlloc<TexRec>(hs.tex.size(), o, b);
  float* texels = DevAlloc<float>(hs.texels.size(), o, b);
  TexBind* tbind = DevAlloc<TexBind>(hs.texBind.size(), o, b);
  float* ldist = DevAlloc<float>(hs.lightDist.size(), o, b);
  up(nodes, hs.nodes);
  up(prims, hs.prims);
  up(pinfo, hs.primInfo);
  up(shapes, hs.shapes);
  up(mats, hs.mats);
  up(lights, hs.lights);
  up(media, hs.media);
  up(pos, hs.pos);
  up(nrm, hs.nrm);
  up(uv, hs.uv);
  up(idx, hs.idx);
  up(cdf, hs.cdf);
  up(vol, hs.volume);
  up(bricks, hs.brickMaj);
  if (!hs.volume.empty()) {
    Check(LaunchFloatToHalf(vol, reinterpret_cast<__half*>(volHalf), hs.volume.size(), 0), "fp16 grid");
    Check(cudaDeviceSynchronize(), "sync");
  }
  up(scls, hs.shapeClass);
  up(tex, hs.tex);
  up(texels, hs.texels);
  up(tbind, hs.texBind);
  up(ldist, hs.lightDist);
  D.nodes = nodes;
  D.prims = prims;
  D.primInfo = pinfo;
  D.shapes = shapes;
  D.mats = mats;
  D.lights = lights;
  D.media = media;
  D.pos = pos;
  D.nrm = nrm;
  D.uv = uv;
  D.idx = idx;
  D.cdf = cdf;
  D.volume = vol;
  D.volumeHalf = volHalf;
  D.brickMaj = bricks;
  D.shapeClass = scls;
  D.tex = tex;
  D.texels = texels;
  D.texBind = tbind;
  D.lightDist = ldist;
  D.nTex = (uint32_t)hs.tex.size();
  D.needDiff = hs.needDiff ? 1u : 0u;
  D.nNodes = (uint32_t)hs.nodes.size();
  D.nPrims = (uint32_t)hs.prims.size();
  D.nShapes = (uint32_t)hs.shapes.size();
  D.nLights = (uint32_t)hs.lights.size();
  D.nMedia = (uint32_t)hs.media.size();
  D.nMats = (uint32_t)hs.mats.size();
  D.envLight = hs.envLight;
  D.globalMedium = hs.globalMedium;
  D.lightPdf = hs.lightPdf;
  D.maxDepth = hs.maxDepth;
  D.rrDepth = hs.rrDepth;
  D.isVol = hs.isVol ? 1 : 0;
  D.isAO = hs.isAO ? 1 : 0;
  D.isParticle = hs.isParticle ? 1 : 0;
  D.isBdpt = hs.isBdpt ? 1 : 0;
  D.bdptMis = hs.bdptMis ? 1 : 0;
  D.cam = hs.cam;
  return b;
}

std::string ReadFile(const std::string& path) {
  std::ifstream in(path, std::ios::binary);
  if (!in) throw IoError("cannot open " + path);
  std::stringstream ss;
  ss << in.rdbuf();
  return ss.str();
}

template <typename T>
struct DevBuf {
  T* p = nullptr;
  explicit DevBuf(size_t n) {
    if (n) Check(cudaMalloc(&p, n * sizeof(T)), "cudaMalloc");
  }
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

}  // namespace

namespace rad {
// Accessors for other translation units of the C ABI.
const DevScene* SceneDevice(const rad_scene* scene) { return &scene->dev; }
const TraceTune* SceneTune(const rad_scene* scene) { return &scene->tune; }
int SceneDeviceIndex() { return L().device; }
int ReportError(int code, const char* msg) { return Fail(code, msg); }
}  // namespace rad

// ============================================================================
extern "C" {

int rad_init(const char* config_json) {
  return Guard([&] {
    std::lock_guard<std::mutex> g(g_initMu);
    InitLocked(config_json);
  });
}

int rad_shutdown(void) {
  return Guard([&] {
    std::lock_guard<std::mutex> g(g_initMu);
    Lib& lib = L();
    if (!lib.inited) return;
    {
      std::lock_guard<std::mutex> lk(lib.qmu);
      lib.stop = true;
    }
    lib.qcv.notify_all();
    if (lib.worker.joinable()) lib.worker.join();
    cudaStreamSynchronize(lib.stream);
    FreeAll(lib.pathAllocs);
    lib.used -= lib.pathBytes;
    lib.pathBytes = 0;
    if (lib.guideMix) cudaFree(lib.guideMix);
    if (lib.guideRec) cudaFree(lib.guideRec);
    lib.guideMix = nullptr;
    lib.guideRec = nullptr;
    lib.guideRecCap = 0;
    lib.guideBytes = 0;
    FreeAll(lib.bdptAllocs);
    lib.used -= lib.bdptBytes;
    lib.bdptBytes = 0;
    lib.bdpt = BdptBuffers{};
    FreeAll(lib.volAllocs);
    lib.used -= lib.volBytes;
    lib.volBytes = 0;
    lib.vol = VolWave{};
    if (lib.hVolWord) cudaFreeHost(lib.hVolWord);
    lib.hVolWord = nullptr;
    if (lib.hCounters) cudaFreeHost(lib.hCounters);
    lib.hCounters = nullptr;
    if (lib.mixHost) cudaFreeHost(lib.mixHost);
    lib.mixHost = nullptr;
    lib.mixDev = nullptr;
    for (cudaEvent_t e : lib.evPool) cudaEventDestroy(e);
    lib.evPool.clear();
    cudaStreamDestroy(lib.stream);
    lib.stream = nullptr;
    lib.inited = false;
  });
}

int rad_last_error(char* buf, size_t size) {
  if (!buf || size == 0) return RAD_ERR_INVALID_ARG;
  std::snprintf(buf, size, "%s", t_err.c_str());
  return RAD_OK;
}

int rad_version(int32_t* major, int32_t* minor) {
  if (major) *major = 0;
  if (minor) *minor = 1;
  return RAD_OK;
}

int rad_device_usage(uint64_t* used_bytes, uint64_t* budget_bytes) {
  Lib& lib = L();
  if (used_bytes) *used_bytes = lib.used.load();
  if (budget_bytes) *budget_bytes = lib.budget;
  return RAD_OK;
}

int rad_scene_load_json(const char* json_text, const char* base_dir, rad_scene** out) {
  if (!json_text || !out) return Fail(RAD_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  return Guard([&] {
    EnsureInit();
    HostScene hs;
    BuildHostScene(json_text, base_dir ? base_dir : "", hs);
    Lib& lib = L();
    rad_scene* sc = new rad_scene();
    try {
      std::lock_guard<std::mutex> g(lib.gpuMu);
      sc->bytes = SceneUpload(hs, sc);
    } catch (...) {
      FreeAll(sc->allocs);
      delete sc;
      throw;
    }
    if (lib.used.load() + sc->bytes > lib.budget && lib.spareBytes.load() > 0) {
      std::lock_guard<std::mutex> g(lib.gpuMu);
      ReleaseSpares();
    }
    if (lib.used.load() + sc->bytes > lib.budget) {
      FreeAll(sc->allocs);
      delete sc;
      throw Error{RAD_ERR_ADMISSION, "scene does not fit the device budget"};
    }
    lib.used += sc->bytes;
    rad_scene_info& in = sc->info;
    in.width = hs.cam.width;
    in.height = hs.cam.height;
    in.spp = hs.spp;
    in.seed = hs.seed;
    in.max_depth = hs.maxDepth;
    in.rr_depth = hs.rrDepth;
    in.is_vol_path = hs.isVol ? 1 : 0;
    in.n_shapes = (int32_t)hs.shapes.size();
    in.n_lights = (int32_t)hs.lights.size();
    in.n_media = (int32_t)hs.media.size();
    in.n_materials = (int32_t)hs.mats.size();
    in.n_prims = hs.nPrims;
    in.n_bvh_nodes = hs.nodes.size();
    in.device_bytes = sc->bytes;
    for (int a = 0; a < 3; a++) {
      // guide position normalisation box: world bounds, widened by 0.1 % per side
      float e = std::max(hs.worldHi[a] - hs.worldLo[a], 1e-3f);
      sc->worldLo[a] = hs.worldLo[a] - 1e-3f * e;
      sc->worldHi[a] = hs.worldHi[a] + 1e-3f * e;
    }
    *out = sc;
  });
}

int rad_scene_load_file(const char* path, rad_scene** out) {
  if (!path || !out) return Fail(RAD_ERR_INVALID_ARG, "null argument");
  std::string text;
  int st = Guard([&] { text = ReadFile(path); });
  if (st != RAD_OK) return st;
  std::string p(path);
  size_t slash = p.find_last_of('/');
  std::string dir = slash == std::string::npos ? std::string(".") : p.substr(0, slash);
  return rad_scene_load_json(text.c_str(), dir.c_str(), out);
}

int rad_scene_destroy(rad_scene* scene) {
  if (!scene) return RAD_OK;
  if (scene->jobs.load() > 0) return Fail(RAD_ERR_INVALID_ARG, "scene still has live jobs");
  return Guard([&] {
    Lib& lib = L();
    std::lock_guard<std::mutex> g(lib.gpuMu);
    cudaStreamSynchronize(lib.stream);
    FreeSpare(scene);
    FreeAll(scene->allocs);
    lib.used -= scene->bytes;
    if (scene->guide) {
      lib.used -= scene->guide->bytes;
      GuideDestroy(scene->guide);
    }
    delete scene;
  });
}

int rad_scene_info_get(const rad_scene* scene, rad_scene_info* info) {
  if (!scene || !info) return Fail(RAD_ERR_INVALID_ARG, "null argument");
  *info = scene->info;
  return RAD_OK;
}

int rad_scene_footprint(const rad_scene* scene, uint64_t* bytes) {
  if (!scene || !bytes) return Fail(RAD_ERR_INVALID_ARG, "null argument");
  *bytes = scene->bytes;
  return RAD_OK;
}

int rad_job_submit(rad_scene* scene, const rad_job_desc* desc, rad_job** out) {
  if (!scene || !out) return Fail(RAD_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  return Guard([&] {
    EnsureInit();
    Lib& lib = L();
    rad_job* j = new rad_job();
    j->scene = scene;
    j->spp = desc && desc->spp ? desc->spp : (uint32_t)scene->info.spp;
    j->seed = desc && desc->seed != UINT32_MAX ? desc->seed : scene->info.seed;
    j->first = desc ? desc->first_sample : 0;
    j->flags = desc ? desc->flags : 0;
    if (j->flags & RAD_JOB_GUIDE)
      j->trainSamples = (uint32_t)std::ceil((double)scene->guideCfg.trainFraction * (double)j->spp);
    uint64_t npix = (uint64_t)scene->info.width * scene->info.height;
    j->total = scene->dev.isParticle ? j->spp : npix * j->spp;  // particle_tracer: spp = light paths
    j->filmBytes = npix * sizeof(float4) + 64;
    j->tSubmit = NowMs();
    j->deadline = j->tSubmit + (double)j->total * lib.edfNsPerSample * 1e-6;
    scene->jobs++;
    *out = j;
    if (j->flags & RAD_JOB_SYNC) {
      if (j->filmBytes + lib.used.load() > lib.budget && lib.spareBytes.load() > 0) {
        std::lock_guard<std::mutex> g(lib.gpuMu);
        ReleaseSpares();
      }
      if (j->filmBytes + lib.used.load() > lib.budget) {
        FinishJob(j, RAD_ERR_ADMISSION, "job film exceeds the device budget");
        return;
      }
      lib.used += j->filmBytes;
      std::lock_guard<std::mutex> g(lib.gpuMu);
      try {
        StartJob(j);
        while (j->nextSample < j->spp && !j->cancel) RunWave(j);
        EndJobLaunch(j);
        Check(cudaEventSynchronize(j->evEnd), "sync");
        CompleteJob(j);
      } catch (const Error& e) {
        FinishJob(j, e.code, e.msg);
      }
      return;
    }
    {
      std::lock_guard<std::mutex> lk(lib.qmu);
      lib.pending.push_back(j);
    }
    lib.qcv.notify_all();
  });
}

int rad_job_wait(rad_job* job, int64_t timeout_ms) {
  if (!job) return Fail(RAD_ERR_INVALID_ARG, "null job");
  std::unique_lock<std::mutex> lk(job->m);
  auto done = [&] { return job->state == kDone; };
  if (timeout_ms < 0) {
    job->cv.wait(lk, done);
  } else if (!job->cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), done)) {
    return Fail(RAD_ERR_TIMEOUT, "job not finished within the timeout");
  }
  if (job->status != RAD_OK) return Fail(job->status, job->err);
  return RAD_OK;
}

int rad_job_cancel(rad_job* job) {
  if (!job) return Fail(RAD_ERR_INVALID_ARG, "null job");
  {
    std::lock_guard<std::mutex> lk(L().qmu);
    job->cancel = true;
  }
  L().qcv.notify_all();
  return RAD_OK;
}

int rad_job_progress(rad_job* job, uint64_t* done, uint64_t* total) {
  if (!job) return Fail(RAD_ERR_INVALID_ARG, "null job");
  bool finished;
  {
    std::lock_guard<std::mutex> lk(job->m);
    finished = job->state == kDone;
  }
  if (done) *done = finished && job->status == RAD_OK ? job->total : job->launched.load();
  if (total) *total = job->total;
  return RAD_OK;
}

int rad_job_film(rad_job* job, float* rgb, int32_t width, int32_t height) {
  if (!job || !rgb) return Fail(RAD_ERR_INVALID_ARG, "null argument");
  {
    std::lock_guard<std::mutex> lk(job->m);
    if (job->state != kDone) return Fail(RAD_ERR_NOT_READY, "job is still running");
    if (job->status != RAD_OK && job->status != RAD_ERR_CANCELLED) return Fail(job->status, job->err);
  }
  const DevScene& S = job->scene->dev;
  if (width != S.cam.width || height != S.cam.height) return Fail(RAD_ERR_INVALID_ARG, "film size mismatch");
  if (!job->accum) return Fail(RAD_ERR_NOT_READY, "job has no film");
  return Guard([&] {
    Lib& lib = L();
    std::lock_guard<std::mutex> g(lib.gpuMu);
    size_t n = (size_t)width * height * 3;
    if (!job->resolve) Check(cudaMalloc(&job->resolve, n * sizeof(float)), "cudaMalloc");
    // sample_renderer.cpp:109-114; a particle film already carries pixels / light paths
    float scale = S.isParticle ? 1.0f : 1.0f / (float)job->spp;
    Check(LaunchResolveFilm(FilmView{job->accum, width, height, nullptr}, scale, job->resolve, lib.stream), "resolve");
    Check(cudaMemcpyAsync(rgb, job->resolve, n * sizeof(float), cudaMemcpyDeviceToHost, lib.stream), "film copy");
    Check(cudaStreamSynchronize(lib.stream), "sync");
  });
}

int rad_job_stats(rad_job* job, rad_stats* stats) {
  if (!job || !stats) return Fail(RAD_ERR_INVALID_ARG, "null argument");
  std::lock_guard<std::mutex> lk(job->m);
  *stats = job->stats;
  return RAD_OK;
}

int rad_job_destroy(rad_job* job) {
  if (!job) return RAD_OK;
  rad_job_cancel(job);
  rad_job_wait(job, -1);
  return Guard([&] {
    Lib& lib = L();
    std::lock_guard<std::mutex> g(lib.gpuMu);
    cudaStreamSynchronize(lib.stream);
    JobSpare& sp = job->scene->spare;
    if (job->accum && job->dStats && job->hStats && job->evStart && job->evEnd) {  // keep for the scene's next job
      FreeSpare(job->scene);
      // the film stays counted in lib.used while it is parked
      sp.bytes = job->filmBytes;
      lib.spareBytes += sp.bytes;
      lib.spareScenes.push_back(job->scene);
      sp.valid = true;
      sp.accum = job->accum;
      sp.dStats = job->dStats;
      sp.hStats = job->hStats;
      sp.resolve = job->resolve;
      sp.evStart = job->evStart;
      sp.evEnd = job->evEnd;
      sp.ctx = job->ctx;
      sp.graphs = std::move(job->graphs);
      sp.graphKernels = std::move(job->graphKernels);
      sp.spw = job->spw;
      sp.tuneEpoch = job->scene->tuneEpoch;
    } else {
      if (job->accum) lib.used -= job->filmBytes;
      if (job->accum) cudaFree(job->accum);
      if (job->dStats) cudaFree(job->dStats);
      if (job->hStats) cudaFreeHost(job->hStats);
      if (job->resolve) cudaFree(job->resolve);
      for (cudaGraphExec_t g : job->graphs) cudaGraphExecDestroy(g);
      if (job->ctx) cudaFree(job->ctx);
      if (job->evStart) cudaEventDestroy(job->evStart);
      if (job->evEnd) cudaEventDestroy(job->evEnd);
    }
    job->scene->jobs--;
    delete job;
  });
}

int rad_trace_batch_device(rad_scene* scene, const float* d_rays, int64_t n, float* d_hits, int32_t any_hit) {
  if (!scene || (n > 0 && (!d_rays || !d_hits)) || n < 0) return Fail(RAD_ERR_INVALID_ARG, "bad argument");
  return Guard([&] {
    Lib& lib = L();
    Check(LaunchTrace(scene->dev, d_rays, n, d_hits, any_hit, lib.paths.counters + kMiscBase + 1, lib.stream),
          "trace");
  });
}

int rad_trace_batch(rad_scene* scene, const float* rays, int64_t n, float* hits, int32_t any_hit) {
  if (!scene || (n > 0 && (!rays || !hits)) || n < 0) return Fail(RAD_ERR_INVALID_ARG, "bad argument");
  if (n == 0) return RAD_OK;
  return Guard([&] {
    Lib& lib = L();
    std::lock_guard<std::mutex> g(lib.gpuMu);
    DevBuf<float> dr(8 * n), dh(5 * n);
    Check(cudaMemcpyAsync(dr.p, rays, 8 * n * sizeof(float), cudaMemcpyHostToDevice, lib.stream), "copy");
    uint32_t zero = 0;
    Check(cudaMemcpyAsync(lib.paths.counters + kMiscBase + 1, &zero, 4, cudaMemcpyHostToDevice, lib.stream), "copy");
    Check(LaunchTrace(scene->dev, dr.p, n, dh.p, any_hit, lib.paths.counters + kMiscBase + 1, lib.stream), "trace");
    Check(cudaMemcpyAsync(hits, dh.p, 5 * n * sizeof(float), cudaMemcpyDeviceToHost, lib.stream), "copy");
    uint32_t err = 0;
    Check(cudaMemcpyAsync(&err, lib.paths.counters + kMiscBase + 1, 4, cudaMemcpyDeviceToHost, lib.stream), "copy");
    Check(cudaStreamSynchronize(lib.stream), "sync");
    if (err) throw Error{RAD_ERR_DEVICE_CHECK, "traversal stack bound exceeded"};
  });
}

int rad_bsdf_eval_batch(const char* bsdf_json, const float* wi, const float* wo, int64_t n, float* f, float* pdf) {
  if (!bsdf_json || n < 0 || (n > 0 && (!wi || !wo || !f || !pdf))) return Fail(RAD_ERR_INVALID_ARG, "bad argument");
  return Guard([&] {
    EnsureInit();
    std::vector<MatRec> mats;
    BuildMaterialRecords(JsonReader::Parse(bsdf_json), mats);
    if (n == 0) return;
    Lib& lib = L();
    std::lock_guard<std::mutex> g(lib.gpuMu);
    DevBuf<MatRec> dm(mats.size());
    DevBuf<float> dwi(3 * n), dwo(3 * n), df(3 * n), dp(n);
    Check(cudaMemcpyAsync(dm.p, mats.data(), mats.size() * sizeof(MatRec), cudaMemcpyHostToDevice, lib.stream), "copy");
    Check(cudaMemcpyAsync(dwi.p, wi, 12 * n, cudaMemcpyHostToDevice, lib.stream), "copy");
    Check(cudaMemcpyAsync(dwo.p, wo, 12 * n, cudaMemcpyHostToDevice, lib.stream), "copy");
    Check(LaunchBsdfEval(dm.p, dwi.p, dwo.p, n, df.p, dp.p, lib.stream), "bsdf eval");
    Check(cudaMemcpyAsync(f, df.p, 12 * n, cudaMemcpyDeviceToHost, lib.stream), "copy");
    Check(cudaMemcpyAsync(pdf, dp.p, 4 * n, cudaMemcpyDeviceToHost, lib.stream), "copy");
    Check(cudaStreamSynchronize(lib.stream), "sync");
  });
}

int rad_bsdf_sample_batch(const char* bsdf_json, const float* wi, const float* u, int64_t n, float* wo, float* pdf,
                          float* f, float* eta, uint32_t* type) {
  if (!bsdf_json || n < 0 || (n > 0 && (!wi || !u || !wo || !pdf || !f || !eta || !type)))
    return Fail(RAD_ERR_INVALID_ARG, "bad argument");
  return Guard([&] {
    EnsureInit();
    std::vector<MatRec> mats;
    BuildMaterialRecords(JsonReader::Parse(bsdf_json), mats);
    if (n == 0) return;
    Lib& lib = L();
    std::lock_guard<std::mutex> g(lib.gpuMu);
    DevBuf<MatRec> dm(mats.size());
    DevBuf<float> dwi(3 * n), du(3 * n), dwo(3 * n), dp(n), df(3 * n), de(n);
    DevBuf<uint32_t> dt(n);
    Check(cudaMemcpyAsync(dm.p, mats.data(), mats.size() * sizeof(MatRec), cudaMemcpyHostToDevice, lib.stream), "copy");
    Check(cudaMemcpyAsync(dwi.p, wi, 12 * n, cudaMemcpyHostToDevice, lib.stream), "copy");
    Check(cudaMemcpyAsync(du.p, u, 12 * n, cudaMemcpyHostToDevice, lib.stream), "copy");
    Check(LaunchBsdfSample(dm.p, dwi.p, du.p, n, dwo.p, dp.p, df.p, de.p, dt.p, lib.stream), "bsdf sample");
    Check(cudaMemcpyAsync(wo, dwo.p, 12 * n, cudaMemcpyDeviceToHost, lib.stream), "copy");
    Check(cudaMemcpyAsync(pdf, dp.p, 4 * n, cudaMemcpyDeviceToHost, lib.stream), "copy");
    Check(cudaMemcpyAsync(f, df.p, 12 * n, cudaMemcpyDeviceToHost, lib.stream), "copy");
    Check(cudaMemcpyAsync(eta, de.p, 4 * n, cudaMemcpyDeviceToHost, lib.stream), "copy");
    Check(cudaMemcpyAsync(type, dt.p, 4 * n, cudaMemcpyDeviceToHost, lib.stream), "copy");
    Check(cudaStreamSynchronize(lib.stream), "sync");
  });
}

int rad_camera_rays(rad_scene* scene, const uint32_t* pixels, int64_t n, uint32_t sample, uint32_t seed,
                    float* rays) {
  if (!scene || n < 0 || (n > 0 && (!pixels || !rays))) return Fail(RAD_ERR_INVALID_ARG, "bad argument");
  if (n == 0) return RAD_OK;
  uint64_t npix = (uint64_t)scene->info.width * scene->info.height;
  for (int64_t i = 0; i < n; i++)
    if (pixels[i] >= npix) return Fail(RAD_ERR_INVALID_ARG, "pixel index out of range");
  return Guard([&] {
    Lib& lib = L();
    std::lock_guard<std::mutex> g(lib.gpuMu);
    DevBuf<uint32_t> dp(n);
    DevBuf<float> dr(8 * n);
    Check(cudaMemcpyAsync(dp.p, pixels, 4 * n, cudaMemcpyHostToDevice, lib.stream), "copy");
    Check(LaunchCameraRays(scene->dev, dp.p, n, sample, seed, dr.p, lib.stream), "camera");
    Check(cudaMemcpyAsync(rays, dr.p, 32 * n, cudaMemcpyDeviceToHost, lib.stream), "copy");
    Check(cudaStreamSynchronize(lib.stream), "sync");
  });
}

int rad_scene_texture_eval(rad_scene* scene, uint32_t texture, const float* uv, const float* duv, int64_t n,
                           float* out) {
  if (!scene || n < 0 || (n > 0 && (!uv || !duv || !out))) return Fail(RAD_ERR_INVALID_ARG, "bad argument");
  if (texture >= scene->dev.nTex) return Fail(RAD_ERR_INVALID_ARG, "texture index out of range");
  if (n == 0) return RAD_OK;
  return Guard([&] {
    Lib& lib = L();
    std::lock_guard<std::mutex> g(lib.gpuMu);
    DevBuf<float> du(2 * n), dd(4 * n), dout(3 * n);
    Check(cudaMemcpyAsync(du.p, uv, 8 * n, cudaMemcpyHostToDevice, lib.stream), "copy");
    Check(cudaMemcpyAsync(dd.p, duv, 16 * n, cudaMemcpyHostToDevice, lib.stream), "copy");
    Check(LaunchTexEval(scene->dev, texture, du.p, dd.p, n, dout.p, lib.stream), "texture eval");
    Check(cudaMemcpyAsync(out, dout.p, 12 * n, cudaMemcpyDeviceToHost, lib.stream), "copy");
    Check(cudaStreamSynchronize(lib.stream), "sync");
  });
}

int rad_render_samples(rad_scene* scene, const uint32_t* pixels, const uint32_t* samples, int64_t n, uint32_t seed,
                       float* radiance) {
  if (!scene || n < 0 || (n > 0 && (!pixels || !samples || !radiance))) return Fail(RAD_ERR_INVALID_ARG, "bad argument");
  if (scene->dev.isParticle)
    return Fail(RAD_ERR_UNSUPPORTED, "particle_tracer splats light paths: it has no per-pixel samples");
  if (n == 0) return RAD_OK;
  uint64_t npix = (uint64_t)scene->info.width * scene->info.height;
  for (int64_t i = 0; i < n; i++)
    if (pixels[i] >= npix) return Fail(RAD_ERR_INVALID_ARG, "pixel index out of range");
  return Guard([&] {
    Lib& lib = L();
    std::lock_guard<std::mutex> g(lib.gpuMu);
    DevBuf<uint32_t> dp(n), ds(n);
    DevBuf<float> dout(3 * n);
    Check(cudaMemcpyAsync(dp.p, pixels, 4 * n, cudaMemcpyHostToDevice, lib.stream), "copy");
    Check(cudaMemcpyAsync(ds.p, samples, 4 * n, cudaMemcpyHostToDevice, lib.stream), "copy");
    uint32_t zero = 0;
    Check(cudaMemcpyAsync(lib.paths.counters + kMiscBase + 1, &zero, 4, cudaMemcpyHostToDevice, lib.stream), "copy");
    const int64_t step = scene->dev.isBdpt ? (int64_t)EnsureBdpt(BdptCap(scene->dev)).nw : (int64_t)lib.maxPaths;
    for (int64_t b = 0; b < n; b += step) {
      uint32_t count = (uint32_t)std::min<int64_t>(step, n - b);
      WaveParams w{0, count, 0, seed, dp.p + b, ds.p + b};
      ProfSink ps{nullptr};
      if (scene->dev.isBdpt) {
        RunBdptWave(scene->dev, scene->tune, w, FilmView{}, dout.p + 3 * b, ps);
        continue;
      }
      Check(LaunchGenerate(scene->dev, lib.paths, w, lib.stream), "generate");
      if (scene->dev.isVol) {
        Check(LaunchVolWavefront(scene->dev, lib.paths, EnsureVolWave(), w, lib.paths.counters + kMiscBase + 1,
                                 lib.stream, 0u, scene->tune, lib.hVolWord, nullptr),
              "vol_path wavefront");
      } else {
        LaunchBounces(scene->dev, scene->tune, count, ps);
      }
      Check(LaunchGatherRadiance(lib.paths, count, dout.p + 3 * b, lib.stream), "gather");
    }
    Check(cudaMemcpyAsync(radiance, dout.p, 12 * n, cudaMemcpyDeviceToHost, lib.stream), "copy");
    uint32_t err = 0;
    Check(cudaMemcpyAsync(&err, lib.paths.counters + kMiscBase + 1, 4, cudaMemcpyDeviceToHost, lib.stream), "copy");
    Check(cudaStreamSynchronize(lib.stream), "sync");
    if (err) throw Error{RAD_ERR_DEVICE_CHECK, "device-side bound exceeded, code " + std::to_string(err)};
  });
}

// ---- learned path guiding ----------------------------------------------------
int rad_guide_enable(rad_scene* scene, const char* config_json) {
  if (!scene) return Fail(RAD_ERR_INVALID_ARG, "null scene");
  return Guard([&] {
    EnsureInit();
    GuideConfig cfg;
    try {
      GuideParseConfig(config_json, cfg);
    } catch (const std::runtime_error& e) {
      throw Error{RAD_ERR_INVALID_ARG, e.what()};
    }
    Lib& lib = L();
    std::lock_guard<std::mutex> g(lib.gpuMu);
    if (scene->jobs.load() > 0) throw Error{RAD_ERR_INVALID_ARG, "scene has live jobs"};
    cudaStreamSynchronize(lib.stream);
    if (scene->guide) {
      lib.used -= scene->guide->bytes;
      GuideDestroy(scene->guide);
      scene->guide = nullptr;
    }
    scene->guideCfg = cfg;
    EnsureGuide(scene);
  });
}

int rad_guide_checkpoint(rad_scene* scene, void* buf, size_t size, size_t* needed) {
  if (!scene) return Fail(RAD_ERR_INVALID_ARG, "null scene");
  return Guard([&] {
    Lib& lib = L();
    std::lock_guard<std::mutex> g(lib.gpuMu);
    if (!scene->guide) throw Error{RAD_ERR_NOT_READY, "scene has no guide network"};
    size_t n = GuideCheckpointBytes(*scene->guide);
    if (needed) *needed = n;
    if (!buf) return;
    if (size < n) throw Error{RAD_ERR_INVALID_ARG, "checkpoint buffer too small"};
    cudaStreamSynchronize(lib.stream);
    try {
      GuideCheckpoint(*scene->guide, buf, lib.stream);
    } catch (const std::runtime_error& e) {
      throw Error{RAD_ERR_CUDA, e.what()};
    }
  });
}

int rad_guide_load(rad_scene* scene, const void* buf, size_t size) {
  if (!scene || !buf) return Fail(RAD_ERR_INVALID_ARG, "null argument");
  return Guard([&] {
    EnsureInit();
    Lib& lib = L();
    std::lock_guard<std::mutex> g(lib.gpuMu);
    if (scene->jobs.load() > 0) throw Error{RAD_ERR_INVALID_ARG, "scene has live jobs"};
    cudaStreamSynchronize(lib.stream);
    GuideNet* n = nullptr;
    try {
      n = GuideFromCheckpoint(buf, size, scene->guideCfg, lib.stream);
    } catch (const std::runtime_error& e) {
      throw Error{RAD_ERR_INVALID_ARG, e.what()};
    }
    if (scene->guide) {
      lib.used -= scene->guide->bytes;
      GuideDestroy(scene->guide);
    }
    scene->guide = n;
    scene->guideCfg = n->cfg;
    lib.used += n->bytes;
  });
}

int rad_guide_forward(rad_scene* scene, const float* queries, int64_t n, float* raw, float* mix) {
  if (!scene || n < 0 || (n > 0 && !queries)) return Fail(RAD_ERR_INVALID_ARG, "bad argument");
  if (n == 0) return RAD_OK;
  if (n > (int64_t)UINT32_MAX) return Fail(RAD_ERR_INVALID_ARG, "too many queries");
  return Guard([&] {
    EnsureInit();
    Lib& lib = L();
    std::lock_guard<std::mutex> g(lib.gpuMu);
    GuideNet& net = EnsureGuide(scene);
    DevBuf<float> dq(9 * n), draw(raw ? (size_t)kGOut * n : 0);
    DevBuf<float4> dmix(mix ? (size_t)kGMixF4 * n : 0);
    Check(cudaMemcpyAsync(dq.p, queries, 36 * n, cudaMemcpyHostToDevice, lib.stream), "copy");
    GuideDev G = GuideView(net);
    uint32_t* err = lib.paths.counters + kMiscBase + 1;
    Check(cudaMemsetAsync(err, 0, sizeof(uint32_t), lib.stream), "memset");
    Check(LaunchGuideQuery(G, dq.p, (uint32_t)n, draw.p, dmix.p, err, lib.stream), "guide query");
    if (raw) Check(cudaMemcpyAsync(raw, draw.p, sizeof(float) * kGOut * n, cudaMemcpyDeviceToHost, lib.stream), "copy");
    if (mix)
      Check(cudaMemcpyAsync(mix, dmix.p, sizeof(float4) * kGMixF4 * n, cudaMemcpyDeviceToHost, lib.stream), "copy");
    uint32_t errWord = 0;
    Check(cudaMemcpyAsync(&errWord, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, lib.stream), "copy");
    Check(cudaStreamSynchronize(lib.stream), "sync");
    if (errWord) throw Error{RAD_ERR_DEVICE_CHECK, "guide network: a tensor-core wait gave up"};
  });
}

int rad_guide_mix_eval(const float* mix, const float* dirs, const float* u, int64_t n, float* pdf, float* out_dirs) {
  if (!mix || !pdf || n < 0 || (!dirs && !u) || (dirs && u) || (u && !out_dirs))
    return Fail(RAD_ERR_INVALID_ARG, "bad argument");
  if (n == 0) return RAD_OK;
  return Guard([&] {
    EnsureInit();
    Lib& lib = L();
    std::lock_guard<std::mutex> g(lib.gpuMu);
    DevBuf<float4> dm((size_t)kGMixF4 * n);
    DevBuf<float> dd(dirs ? 3 * n : 0), du(u ? 3 * n : 0), dp(n), dout(u ? 3 * n : 0);
    Check(cudaMemcpyAsync(dm.p, mix, sizeof(float4) * kGMixF4 * n, cudaMemcpyHostToDevice, lib.stream), "copy");
    if (dirs) Check(cudaMemcpyAsync(dd.p, dirs, 12 * n, cudaMemcpyHostToDevice, lib.stream), "copy");
    if (u) Check(cudaMemcpyAsync(du.p, u, 12 * n, cudaMemcpyHostToDevice, lib.stream), "copy");
    Check(LaunchGuideMixEval(dm.p, dd.p, du.p, (uint32_t)n, dp.p, dout.p, lib.stream), "mixture eval");
    Check(cudaMemcpyAsync(pdf, dp.p, 4 * n, cudaMemcpyDeviceToHost, lib.stream), "copy");
    if (u) Check(cudaMemcpyAsync(out_dirs, dout.p, 12 * n, cudaMemcpyDeviceToHost, lib.stream), "copy");
    Check(cudaStreamSynchronize(lib.stream), "sync");
  });
}

int rad_guide_grad(rad_scene* scene, const float* records, int64_t n, float* grad, float* loss) {
  if (!scene || n < 0 || (n > 0 && !records) || !grad) return Fail(RAD_ERR_INVALID_ARG, "bad argument");
  if (n > (int64_t)(1u << 26)) return Fail(RAD_ERR_INVALID_ARG, "too many records");
  return Guard([&] {
    EnsureInit();
    Lib& lib = L();
    std::lock_guard<std::mutex> g(lib.gpuMu);
    GuideNet& net = EnsureGuide(scene);
    // repack (P, b | N, - | wo, - | wi, w) rows into the kGRecF4 record layout
    std::vector<float4> host((size_t)std::max<int64_t>(n, 1) * kGRecF4);
    for (int64_t i = 0; i < n; i++)
      for (int k = 0; k < 4; k++) {
        const float* s = records + 16 * i + 4 * k;
        host[(size_t)i * kGRecF4 + k] = make_float4(s[0], s[1], s[2], s[3]);
      }
    DevBuf<float4> drec(host.size());
    DevBuf<float> dloss(1);
    Check(cudaMemcpyAsync(drec.p, host.data(), host.size() * sizeof(float4), cudaMemcpyHostToDevice, lib.stream),
          "copy");
    Check(cudaMemsetAsync(dloss.p, 0, 4, lib.stream), "memset");
    cudaStreamSynchronize(lib.stream);
    Check(cudaMemsetAsync(net.g, 0, net.nParams * sizeof(float), lib.stream), "memset");
    GuideDev G = GuideView(net);
    uint32_t* err = lib.paths.counters + kMiscBase + 1;
    Check(cudaMemsetAsync(err, 0, sizeof(uint32_t), lib.stream), "memset");
    if (n > 0)
      Check(LaunchGuideTrain(G, drec.p, nullptr, (uint32_t)n, (uint32_t)n, 1, 0, INFINITY, net.g, net.g + net.nTable,
                             dloss.p, (uint32_t)n, err, lib.stream),
            "guide gradient");
    Check(cudaMemcpyAsync(grad, net.g, net.nParams * sizeof(float), cudaMemcpyDeviceToHost, lib.stream), "copy");
    float l = 0.f;
    uint32_t errWord = 0;
    Check(cudaMemcpyAsync(&l, dloss.p, 4, cudaMemcpyDeviceToHost, lib.stream), "copy");
    Check(cudaMemcpyAsync(&errWord, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, lib.stream), "copy");
    Check(cudaMemsetAsync(net.g, 0, net.nParams * sizeof(float), lib.stream), "memset");
    Check(cudaStreamSynchronize(lib.stream), "sync");
    if (errWord) throw Error{RAD_ERR_DEVICE_CHECK, "guide network: a tensor-core wait gave up"};
    if (loss) *loss = l;
  });
}

int rad_guide_info(rad_scene* scene, rad_guide_info_t* info) {
  if (!scene || !info) return Fail(RAD_ERR_INVALID_ARG, "null argument");
  return Guard([&] {
    Lib& lib = L();
    std::lock_guard<std::mutex> g(lib.gpuMu);
    if (!scene->guide) throw Error{RAD_ERR_NOT_READY, "scene has no guide network"};
    const GuideNet& n = *scene->guide;
    *info = rad_guide_info_t{};
    info->n_params = n.nParams;
    info->n_table = n.nTable;
    info->log2_table = n.cfg.log2T;
    info->levels = kGLevels;
    for (int l = 0; l < kGLevels; l++) info->level_res[l] = n.res[l];
    for (int a = 0; a < 3; a++) {
      info->lo[a] = n.lo[a];
      info->hi[a] = n.hi[a];
    }
    info->adam_steps = n.step;
    info->device_bytes = n.bytes;
  });
}

// ---- autotuner ----------------------------------------------------------------
// Times full waves (generate + the bounce loop, sample 0 of the first pixel
// chunk, so every candidate traces the same paths) for each candidate launch
// configuration and keeps the fastest in the scene.
int rad_autotune(rad_scene* scene, const char* config_json, rad_tune_result* out) {
  if (!scene) return Fail(RAD_ERR_INVALID_ARG, "null scene");
  if (scene->dev.isParticle || scene->dev.isBdpt)
    return Fail(RAD_ERR_UNSUPPORTED, "the autotuner covers the `path` and `vol_path` kernels");
  return Guard([&] {
    EnsureInit();
    int reps = 2;
    const bool vol = scene->dev.isVol != 0;
    std::vector<int> leaf = {2, 3, 4, 5, 6}, refill = {16, 20, 24, 28, 32}, perSm = {4, 6, 8}, shade = {64, 128, 256};
    std::vector<int> chunk = {TraceTune{}.volChunk};
    if (vol) {
      // vol_path's part kernels: the lane top-up threshold, blocks per SM (at
      // most their occupancy, 4) and the chunk of steps; the leaf vote and shade
      // block do not apply
      const TraceTune def;
      leaf = {def.leafFrac8};
      shade = {def.shadeBlock};
      refill = {8, 12, 16, 20, 24, 28, 32};
      perSm = {2, 3, 4};
      chunk = {4, 8, 16, 32, 64};
    }
    if (config_json && *config_json) {
      JValue c = JsonReader::Parse(config_json);
      if (const JValue* v = c.get("reps")) reps = std::max(1, (int)v->n);
      auto list = [&](const char* k, std::vector<int>& dst, int lo, int hi) {
        if (const JValue* v = c.get(k)) {
          if (!v->isArr() || v->a.empty()) throw Error{RAD_ERR_INVALID_ARG, std::string(k) + " must be a list"};
          dst.clear();
          for (const JValue& e : v->a) {
            int x = (int)e.n;
            if (x < lo || x > hi) throw Error{RAD_ERR_INVALID_ARG, std::string(k) + " value out of range"};
            dst.push_back(x);
          }
        }
      };
      list("leaf_frac8", leaf, 1, 8);
      list("refill_busy", refill, 1, 32);
      list("blocks_per_sm", perSm, 1, 8);
      list("shade_block", shade, 64, 256);
      if (vol) list("vol_chunk", chunk, 1, 1 << 20);
      for (int v : shade)
        if (v != 64 && v != 128 && v != 256) throw Error{RAD_ERR_INVALID_ARG, "shade_block values are 64, 128 or 256"};
    }
    Lib& lib = L();
    std::lock_guard<std::mutex> g(lib.gpuMu);
    const DevScene& S = scene->dev;
    uint64_t npix = (uint64_t)S.cam.width * S.cam.height;
    uint32_t count = (uint32_t)std::min<uint64_t>(npix, lib.maxPaths);
    cudaEvent_t a = GetEvent(), b = GetEvent();
    ProfSink none{nullptr};
    auto wave = [&](const TraceTune& tu) {
      WaveParams w{0, count, 0, scene->info.seed, nullptr, nullptr};
      Check(LaunchGenerate(S, lib.paths, w, lib.stream), "generate");
      if (vol)
        Check(LaunchVolWavefront(S, lib.paths, EnsureVolWave(), w, lib.paths.counters + kMiscBase + 1, lib.stream, 0u,
                                 tu, lib.hVolWord, nullptr),
              "vol_path wavefront");
      else
        LaunchBounces(S, tu, count, none);
    };
    std::vector<std::pair<TraceTune, float>> timed;
    auto time = [&](const TraceTune& tu) -> float {
      for (const auto& t : timed)
        if (t.first.refillBusy == tu.refillBusy && t.first.blocksPerSm == tu.blocksPerSm &&
            t.first.leafFrac8 == tu.leafFrac8 && t.first.shadeBlock == tu.shadeBlock &&
            t.first.volChunk == tu.volChunk)
          return t.second;
      wave(tu);  // warm-up
      Check(cudaEventRecord(a, lib.stream), "event");
      for (int k = 0; k < reps; k++) wave(tu);
      Check(cudaEventRecord(b, lib.stream), "event");
      Check(cudaEventSynchronize(b), "sync");
      float ms = 0.f;
      cudaEventElapsedTime(&ms, a, b);
      ms /= (float)reps;
      timed.push_back({tu, ms});
      return ms;
    };
    // coordinate descent from the defaults: each axis in turn, the others held at
    // the best values found so far
    // (vol_path: the defaults' 8 blocks per SM run as each part kernel's occupancy, outside the list)
    const float volDefaultMs = vol ? time(TraceTune{}) : 0.f;
    TraceTune best;
    if (std::find(leaf.begin(), leaf.end(), best.leafFrac8) == leaf.end()) best.leafFrac8 = leaf[0];
    if (std::find(refill.begin(), refill.end(), best.refillBusy) == refill.end()) best.refillBusy = refill[0];
    if (std::find(perSm.begin(), perSm.end(), best.blocksPerSm) == perSm.end()) best.blocksPerSm = perSm[0];
    if (std::find(shade.begin(), shade.end(), best.shadeBlock) == shade.end()) best.shadeBlock = shade[0];
    if (std::find(chunk.begin(), chunk.end(), best.volChunk) == chunk.end()) best.volChunk = chunk[0];
    float bestMs = time(best);
    auto axis = [&](const std::vector<int>& vals, int32_t TraceTune::*field) {
      for (int v : vals) {
        TraceTune tu = best;
        tu.*field = v;
        float ms = time(tu);
        if (ms < bestMs) {
          bestMs = ms;
          best = tu;
        }
      }
    };
    axis(leaf, &TraceTune::leafFrac8);
    axis(refill, &TraceTune::refillBusy);
    axis(perSm, &TraceTune::blocksPerSm);
    axis(shade, &TraceTune::shadeBlock);
    axis(chunk, &TraceTune::volChunk);
    rad_tune_result res{};
    res.vol_chunk = best.volChunk;
    res.shade_block = best.shadeBlock;
    res.refill_busy = best.refillBusy;
    res.blocks_per_sm = best.blocksPerSm;
    res.leaf_frac8 = best.leafFrac8;
    res.best_ms = bestMs;
    res.candidates = (int32_t)timed.size();
    const TraceTune def;
    res.default_ms = volDefaultMs;
    for (const auto& t : timed)
      if (!vol && t.first.refillBusy == def.refillBusy && t.first.blocksPerSm == def.blocksPerSm &&
          t.first.leafFrac8 == def.leafFrac8 && t.first.shadeBlock == def.shadeBlock &&
          t.first.volChunk == def.volChunk)
        res.default_ms = t.second;
    lib.evPool.push_back(a);
    lib.evPool.push_back(b);
    uint32_t errWord = 0;
    Check(cudaMemcpy(&errWord, lib.paths.counters + kMiscBase + 1, 4, cudaMemcpyDeviceToHost), "copy");
    if (errWord) {
      cudaMemset(lib.paths.counters + kMiscBase + 1, 0, 4);
      throw Error{RAD_ERR_DEVICE_CHECK, "device-side check fired while tuning"};
    }
    scene->tune = best;
    scene->tuneEpoch++;
    if (out) *out = res;
  });
}

}  // extern "C"
