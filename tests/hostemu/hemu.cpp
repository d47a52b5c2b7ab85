// Host-emulation harness (test infrastructure, never part of the product).
//
// Compiles the renderer's device code -- the BVH8 traversal (dtrace.cuh), the
// scene, BSDF and light functions (dscene.cuh, dbsdf.cuh, dlight.cuh) and the
// wavefront kernels of k_path.cu and k_vol.cu -- for the host with
// RAD_HOST_EMULATION (dmath.cuh: each kernel runs as a loop over its grid, one
// thread at a time, each thread the only active lane of its warp). Scenes are
// compiled by the product's own host code (host_scene.cpp, host_bvh.cpp) into
// the same records the GPU reads. Transcendentals are the host libm's, as in
// the oracle, so every difference between these results and the oracle's is a
// difference in the algorithm, not in sinf / expf rounding.
#define RAD_HOST_EMULATION 1
#include <algorithm>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>

#include "host_json.h"
#include "host_scene.h"

// Ulp nudges: with a nonzero seed, each result of the eleven transcendental
// functions the device code calls (those whose bit in the mask is set) is
// moved, from a seeded stream, with probability 1/2 by 1 .. max_ulps ulps
// (uniform) up or down (1/2 each), else left as it is. A sample whose
// radiance changes under such nudges depends on the last-ulp rounding of some
// transcendental -- the only place the GPU (CUDA's math library, whose
// single-precision functions are within a few ulp) and the oracle (the host
// libm) differ. Targeted mode instead moves exactly one call (by its index
// among the calls of a render) by a given number of ulps.
namespace hemu {
inline uint64_t g_nudge = 0;
inline uint32_t g_mask = 0x7ffu;
inline uint32_t g_maxUlps = 2;
inline uint64_t g_calls = 0;      // transcendental calls of the current render
inline int64_t g_target = -1;     // targeted mode: the call to move
inline int32_t g_targetUlps = 0;  // and by how many ulps (signed)
inline float Nudge(float y, uint32_t fn) {
  const uint64_t call = g_calls++;
  if (!std::isfinite(y)) return y;
  if (g_target >= 0) {
    if ((int64_t)call != g_target) return y;
    const float dir = g_targetUlps > 0 ? INFINITY : -INFINITY;
    for (int32_t i = 0; i < std::abs(g_targetUlps); i++) y = std::nextafter(y, dir);
    return y;
  }
  if (g_nudge == 0 || !((g_mask >> fn) & 1u)) return y;
  uint64_t z = (g_nudge += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  if (z >> 63) return y;
  const float dir = ((z >> 62) & 1u) ? INFINITY : -INFINITY;
  uint32_t k = 1u + (uint32_t)((z & 0xffffffffu) % g_maxUlps);
  for (uint32_t i = 0; i < k; i++) y = std::nextafter(y, dir);
  return y;
}
}  // namespace hemu
#define sinf(x) hemu::Nudge(::sinf(x), 0)
#define cosf(x) hemu::Nudge(::cosf(x), 1)
#define tanf(x) hemu::Nudge(::tanf(x), 2)
#define expf(x) hemu::Nudge(::expf(x), 3)
#define logf(x) hemu::Nudge(::logf(x), 4)
#define log2f(x) hemu::Nudge(::log2f(x), 5)
#define powf(x, y) hemu::Nudge(::powf(x, y), 6)
#define atan2f(y, x) hemu::Nudge(::atan2f(y, x), 7)
#define acosf(x) hemu::Nudge(::acosf(x), 8)
#define asinf(x) hemu::Nudge(::asinf(x), 9)
#define erff(x) hemu::Nudge(::erff(x), 10)

#include "k_path.cu"
#include "k_vol.cu"

namespace {

using namespace rad;

thread_local std::string g_err;

struct HemuScene {
  HostScene hs;
  DevScene S{};
  std::vector<uint16_t> volHalf;  // fp16 copy of the grid (unused by the fp32 estimators)
};

// DevScene over the host vectors, field by field as the runtime's upload fills it.
void Bind(HemuScene& h) {
  HostScene& hs = h.hs;
  DevScene& D = h.S;
  D = DevScene{};
  D.nodes = hs.nodes.data();
  D.prims = hs.prims.data();
  D.primInfo = hs.primInfo.data();
  D.shapes = hs.shapes.data();
  D.mats = hs.mats.data();
  D.lights = hs.lights.data();
  D.media = hs.media.data();
  D.pos = hs.pos.data();
  D.nrm = hs.nrm.empty() ? nullptr : hs.nrm.data();
  D.uv = hs.uv.empty() ? nullptr : hs.uv.data();
  D.idx = hs.idx.data();
  D.cdf = hs.cdf.data();
  D.volume = hs.volume.data();
  h.volHalf.assign(hs.volume.size(), 0);
  D.volumeHalf = h.volHalf.data();
  D.brickMaj = hs.brickMaj.data();
  D.shapeClass = hs.shapeClass.data();
  D.tex = hs.tex.data();
  D.texels = hs.texels.data();
  D.texBind = hs.texBind.data();
  D.lightDist = hs.lightDist.data();
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
}

// Runs `kernel` over a grid of `blocks` x `block` threads, one thread at a time.
template <class F>
void Grid(uint32_t blocks, uint32_t block, F kernel) {
  gridDim = HemuDim3{blocks, 1u, 1u};
  blockDim = HemuDim3{block, 1u, 1u};
  for (uint32_t b = 0; b < blocks; b++)
    for (uint32_t t = 0; t < block; t++) {
      blockIdx = HemuDim3{b, 0u, 0u};
      threadIdx = HemuDim3{t, 0u, 0u};
      kernel();
    }
}

// Path state for n paths in host memory, laid out as the runtime's buffers.
struct HostPaths {
  std::vector<float4> rayO, rayD, thr, L, prev, shO, shD, shC;
  std::vector<uint2> rng;
  std::vector<uint32_t> pixel, q0, q1, classQ, counters;
  std::vector<HitRec> hit;
  PathBuffers B{};
  explicit HostPaths(uint32_t n) {
    for (auto* v : {&rayO, &rayD, &thr, &L, &prev, &shO, &shD, &shC}) v->assign(n, float4{0, 0, 0, 0});
    rng.assign(n, uint2{0, 0});
    pixel.assign(n, 0);
    q0.assign(n, 0);
    q1.assign(n, 0);
    classQ.assign((size_t)kShadeClasses * n, 0);
    counters.assign(kCounterWords, 0);
    hit.assign(n, HitRec{});
    B.rayO = rayO.data();
    B.rayD = rayD.data();
    B.thr = thr.data();
    B.L = L.data();
    B.prev = prev.data();
    B.rng = rng.data();
    B.pixel = pixel.data();
    B.hit = hit.data();
    B.q[0] = q0.data();
    B.q[1] = q1.data();
    B.shO = shO.data();
    B.shD = shD.data();
    B.shC = shC.data();
    B.classQ = classQ.data();
    B.counters = counters.data();
    B.capacity = n;
    B.guideRec = nullptr;
  }
};

// vol_path as the per-event wavefront: the rounds of part kernels of
// LaunchVolWavefront, each over a grid of two one-lane warps, until every path
// has ended.
constexpr uint32_t kHemuVolWavefront = 256u;
template <bool BRICKS>
void VolWavefront(const DevScene& S, PathBuffers& B, uint32_t n, uint32_t* err, uint32_t mode, int chunk) {
  std::vector<VolPathState> states(n);
  std::vector<uint32_t> q((size_t)2 * kVolActs * n, 0u), cnt(kVolCountWords, 0u);
  VolWave V{states.data(), q.data(), cnt.data(), n};
  for (uint32_t r = 0; cnt[kVolEndedWord] < n; r++) {
    if (r > 65536) throw std::runtime_error("vol_path wavefront: paths left after 65536 rounds");
    const uint32_t cur = r & 1u;
    if (r == 0)
      Grid(1, 2, [&] { KVolEvent<kActTop, true, BRICKS, false>(S, B, V, n, cur, err, mode, 16, chunk); });
    else
      Grid(1, 2, [&] { KVolEvent<kActTop, false, BRICKS, false>(S, B, V, n, cur, err, mode, 16, chunk); });
    Grid(1, 2, [&] { KVolEvent<kActScatter, false, BRICKS, false>(S, B, V, n, cur, err, mode, 16, chunk); });
    Grid(1, 2, [&] { KVolEvent<kActSurface, false, BRICKS, false>(S, B, V, n, cur, err, mode, 16, chunk); });
    Grid(1, 2, [&] { KVolEvent<kActNee, false, BRICKS, false>(S, B, V, n, cur, err, mode, 16, chunk); });
    Grid(1, 2, [&] { KVolEvent<kActScatterEnd, false, BRICKS, false>(S, B, V, n, cur, err, mode, 16, chunk); });
    Grid(1, 2, [&] { KVolEvent<kActSurfaceEnd, false, BRICKS, false>(S, B, V, n, cur, err, mode, 16, chunk); });
    Grid(1, 32, [&] { KVolRoundEnd(V, cur); });
  }
}

// The wave of rad_render_samples: generate, then the bounce loop (extend, the
// shade classes, shadow) or the vol_path kernel, with the kernels' own code.
// Traversal refills a lane as soon as it is idle (a warp of one lane), which
// changes only the order rays are taken in, not any ray's result.
void RenderSamples(const DevScene& S, const uint32_t* pix, const uint32_t* smp, uint32_t n, uint32_t seed,
                   uint32_t volMode, float* out) {
  HostPaths P(n);
  PathBuffers& B = P.B;
  WaveParams w{0, n, 0, seed, pix, smp, nullptr, 0};
  uint32_t gen = std::max<uint32_t>(n, (uint32_t)kCounterWords);
  Grid((gen + kBlock - 1) / kBlock, kBlock, [&] { KGenerate(S, B, w); });
  uint32_t* err = B.counters + kMiscBase + 1;
  GuideDev none{};
  if (S.isVol && (volMode & kHemuVolWavefront)) {
    if (volMode & kVolHalf) throw std::runtime_error("the fp16 grid is not emulated");
    // a short chunk, so that paths often continue their part in a later round
    if (volMode & kVolBricks)
      VolWavefront<true>(S, B, n, err, volMode & ~kHemuVolWavefront, 3);
    else
      VolWavefront<false>(S, B, n, err, volMode & ~kHemuVolWavefront, 3);
  } else if (S.isVol) {
    switch (volMode & (kVolBricks | kVolHalf)) {
      case 0: Grid(1, 1, [&] { KVolPath<false, false>(S, B, n, err, volMode); }); break;
      case kVolBricks: Grid(1, 1, [&] { KVolPath<true, false>(S, B, n, err, volMode); }); break;
      default: throw std::runtime_error("the fp16 grid is not emulated");
    }
  } else if (S.isAO) {
    Grid(1, 1, [&] { KExtend<false, false>(S, B, 0, nullptr, 1, 4); });
    Grid(1, 1, [&] { KShadeAO(S, B); });
    Grid(1, 1, [&] { KShadow<false, false>(S, B, 0, nullptr, 1, 4); });
  } else {
    int iters = S.maxDepth >= 0 ? std::max(1, S.maxDepth) : kMaxBounce;
    if (iters > kMaxBounce) iters = kMaxBounce;
    for (int d = 0; d < iters && B.counters[d] != 0; d++) {
      Grid(1, 1, [&] { KExtend<false, false>(S, B, d, nullptr, 1, 4); });
      Grid(1, 1, [&] { KShadeClass<SC_EMIT, false, false>(S, B, none, d); });
      Grid(1, 1, [&] { KShadeClass<SC_GLASS, false, false>(S, B, none, d); });
      Grid(1, 1, [&] { KShadeClass<SC_DIFFUSE, false, false>(S, B, none, d); });
      Grid(1, 1, [&] { KShadeClass<SC_METAL, false, false>(S, B, none, d); });
      Grid(1, 1, [&] { KShadeClass<SC_DISNEY, false, false>(S, B, none, d); });
      Grid(1, 1, [&] { KShadeClass<SC_GENERIC, false, false>(S, B, none, d); });
      Grid(1, 1, [&] { KShadow<false, false>(S, B, d, nullptr, 1, 4); });
    }
  }
  if (*err) throw std::runtime_error("device-side check fired, code " + std::to_string(*err));
  for (uint32_t i = 0; i < n; i++) {
    out[3 * i] = B.L[i].x;
    out[3 * i + 1] = B.L[i].y;
    out[3 * i + 2] = B.L[i].z;
  }
}

template <class F>
int Guarded(F f) {
  try {
    f();
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

template <class F>
void Parallel(int64_t n, int threads, F f) {
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  std::vector<std::thread> pool;
  int64_t chunk = (n + threads - 1) / threads;
  for (int t = 0; t < threads; t++) {
    int64_t a = t * chunk, b = std::min<int64_t>(n, a + chunk);
    if (a >= b) break;
    pool.emplace_back([=] {
      for (int64_t i = a; i < b; i++) f(i);
    });
  }
  for (auto& th : pool) th.join();
}

}  // namespace

extern "C" {

const char* hemu_last_error() { return g_err.c_str(); }

// 0 = exact host libm results (the default); else the seed of the ulp nudges.
void hemu_set_nudge(uint64_t seed) { hemu::g_nudge = seed; }
// Which functions are nudged (bit i: sinf, cosf, tanf, expf, logf, log2f,
// powf, atan2f, acosf, asinf, erff) and by at most how many ulps.
void hemu_set_nudge_config(uint32_t mask, uint32_t max_ulps) {
  hemu::g_mask = mask;
  hemu::g_maxUlps = max_ulps < 1u ? 1u : max_ulps;
}
// Targeted mode: only call number `index` of each render moves, by `ulps`
// (signed); index < 0 leaves targeted mode.
void hemu_set_nudge_target(int64_t index, int32_t ulps) {
  hemu::g_target = index;
  hemu::g_targetUlps = ulps;
}
// Transcendental calls made by the last hemu_render_samples.
uint64_t hemu_last_calls() { return hemu::g_calls; }

void* hemu_scene_load(const char* json, const char* base_dir) {
  auto h = std::make_unique<HemuScene>();
  if (Guarded([&] { BuildHostScene(json, base_dir ? base_dir : "", h->hs); }) != 0) return nullptr;
  Bind(*h);
  return h.release();
}

void hemu_scene_free(void* s) { delete static_cast<HemuScene*>(s); }

// Perspective::SampleRay for pixel samples (KCamera's arithmetic): n x 8 floats.
int hemu_camera_rays(void* s, const uint32_t* pix, int64_t n, uint32_t sample, uint32_t seed, float* out) {
  const DevScene& S = static_cast<HemuScene*>(s)->S;
  return Guarded([&] {
    for (int64_t i = 0; i < n; i++) {
      uint32_t p = pix[i];
      uint32_t x = p % (uint32_t)S.cam.width, y = p / (uint32_t)S.cam.width;
      Pcg32 rng = PcgForSample(p, sample, seed);
      float jx = Next1D(rng);
      float jy = Next1D(rng);
      V3 O, D;
      float tmin, tmax;
      CameraRay(S.cam, (float)x + jx, (float)y + jy, O, D, tmin, tmax);
      float* o = out + 8 * i;
      o[0] = O.x, o[1] = O.y, o[2] = O.z, o[3] = tmin, o[4] = D.x, o[5] = D.y, o[6] = D.z, o[7] = tmax;
    }
  });
}

// BVH8 closest / any hit (KTrace's arithmetic): n x 5 words as rad_trace_batch.
int hemu_trace(void* s, const float* rays, int64_t n, float* hits, int any_hit, int threads) {
  const DevScene& S = static_cast<HemuScene*>(s)->S;
  uint32_t errWord = 0;
  int rc = Guarded([&] {
    Parallel(n, threads, [&](int64_t i) {
      const float* q = rays + 8 * i;
      RayPre r = MakeRayPre(V3{q[0], q[1], q[2]}, V3{q[4], q[5], q[6]}, q[3]);
      TraceHit h;
      uint32_t err = 0;
      float* o = hits + 5 * i;
      if (any_hit) {
        bool occ = TraceBvh8<true>(S, r, q[7], h, &err);
        o[0] = o[1] = o[2] = 0.f;
        o[3] = __uint_as_float(occ ? 1u : 0u);
        o[4] = __uint_as_float(0u);
      } else {
        bool hit = TraceBvh8<false>(S, r, q[7], h, &err);
        o[0] = hit ? h.t : kInf;
        o[1] = hit ? h.u : 0.f;
        o[2] = hit ? h.v : 0.f;
        o[3] = __uint_as_float(hit ? h.prim : kNoPrim);
        o[4] = __uint_as_float(hit ? h.front : 0u);
      }
      if (err) __atomic_fetch_or(&errWord, err, __ATOMIC_RELAXED);
    });
  });
  if (rc == 0 && errWord) {
    g_err = "traversal stack overflow";
    return 1;
  }
  return rc;
}

// Bsdf::Eval + Pdf (KBsdfEval's arithmetic) for one BSDF given as reference JSON.
int hemu_bsdf_eval(const char* json, const float* wi, const float* wo, int64_t n, float* f, float* pdf) {
  return Guarded([&] {
    std::vector<MatRec> mats;
    BuildMaterialRecords(JsonReader::Parse(json), mats);
    for (int64_t i = 0; i < n; i++) {
      V3 v;
      float p;
      BsdfEvalPdf(mats.data(), 0, ld3(wi + 3 * i), ld3(wo + 3 * i), v, p);
      f[3 * i] = v.x, f[3 * i + 1] = v.y, f[3 * i + 2] = v.z;
      pdf[i] = p;
    }
  });
}

// Bsdf::Sample (KBsdfSample's arithmetic).
int hemu_bsdf_sample(const char* json, const float* wi, const float* u, int64_t n, float* wo, float* pdf, float* f,
                     float* eta, uint32_t* type) {
  return Guarded([&] {
    std::vector<MatRec> mats;
    BuildMaterialRecords(JsonReader::Parse(json), mats);
    for (int64_t i = 0; i < n; i++) {
      BsdfSampleRes r = BsdfSample(mats.data(), 0, ld3(wi + 3 * i), u[3 * i], V2{u[3 * i + 1], u[3 * i + 2]});
      wo[3 * i] = r.wo.x, wo[3 * i + 1] = r.wo.y, wo[3 * i + 2] = r.wo.z;
      pdf[i] = r.pdf;
      f[3 * i] = r.f.x, f[3 * i + 1] = r.f.y, f[3 * i + 2] = r.f.z;
      eta[i] = r.eta;
      type[i] = r.type;
    }
  });
}

// A mixed wave of n jobs (the serving loop's RunMixedWave): job k renders every
// pixel of scene k at samples [sample0, sample0 + spw) with seed seeds[k], all
// jobs' paths in the same launches of the MIX kernels (generate, extend, shade
// classes, shadow). out[k]: job k's per-path radiance, path s * npix + j being
// pixel j, sample sample0 + s.
int hemu_render_mixed(void** scenes, int n, uint32_t spw, uint32_t sample0, const uint32_t* seeds, float** out) {
  return Guarded([&] {
    if (n < 1 || n > kMaxMix) throw std::runtime_error("1 to kMaxMix jobs");
    std::vector<MixJob> tab((size_t)n);
    uint32_t total = 0;
    int iters = 1;
    for (int k = 0; k < n; k++) {
      const DevScene& S = static_cast<HemuScene*>(scenes[k])->S;
      if (S.isVol || S.isAO || S.isParticle || S.isBdpt || S.maxDepth < 0)
        throw std::runtime_error("mixed waves hold plain path jobs of bounded depth");
      const uint32_t npix = (uint32_t)S.cam.width * (uint32_t)S.cam.height;
      MixJob J{};
      J.S = S;
      J.pixelBegin = 0;
      J.npc = npix;
      J.spw = spw;
      J.sample = sample0;
      J.seed = seeds[k];
      J.count = npix * spw;
      J.pathBegin = total;
      total += J.count;
      tab[(size_t)k] = J;
      iters = std::max(iters, S.maxDepth);
    }
    iters = std::min(iters, kMaxBounce);
    HostPaths P(total);
    std::vector<uint8_t> job(total, 0);
    PathBuffers& B = P.B;
    B.job = job.data();
    B.mix = tab.data();
    const DevScene& S0 = tab[0].S;
    uint32_t gen = std::max<uint32_t>(total, (uint32_t)kCounterWords);
    Grid((gen + kBlock - 1) / kBlock, kBlock, [&] { KGenerateMix(B, total, (uint32_t)n); });
    GuideDev none{};
    for (int d = 0; d < iters && B.counters[d] != 0; d++) {
      Grid(1, 1, [&] { KExtend<false, true>(S0, B, d, nullptr, 1, 4); });
      Grid(1, 1, [&] { KShadeClass<SC_EMIT, false, true>(S0, B, none, d); });
      Grid(1, 1, [&] { KShadeClass<SC_GLASS, false, true>(S0, B, none, d); });
      Grid(1, 1, [&] { KShadeClass<SC_DIFFUSE, false, true>(S0, B, none, d); });
      Grid(1, 1, [&] { KShadeClass<SC_METAL, false, true>(S0, B, none, d); });
      Grid(1, 1, [&] { KShadeClass<SC_DISNEY, false, true>(S0, B, none, d); });
      Grid(1, 1, [&] { KShadeClass<SC_GENERIC, false, true>(S0, B, none, d); });
      Grid(1, 1, [&] { KShadow<false, true>(S0, B, d, nullptr, 1, 4); });
    }
    if (B.counters[kMiscBase + 1]) throw std::runtime_error("device-side check fired");
    for (int k = 0; k < n; k++)
      for (uint32_t i = 0; i < tab[(size_t)k].count; i++) {
        const float4 l = B.L[tab[(size_t)k].pathBegin + i];
        out[k][3 * i] = l.x;
        out[k][3 * i + 1] = l.y;
        out[k][3 * i + 2] = l.z;
      }
  });
}

// Li of (pixel, sample) pairs through the emulated kernels (rad_render_samples).
// vol_mode: the vol_path estimator bits (0 = the reference's algorithm).
int hemu_render_samples(void* s, const uint32_t* pix, const uint32_t* smp, int64_t n, uint32_t seed,
                        uint32_t vol_mode, float* out) {
  const DevScene& S = static_cast<HemuScene*>(s)->S;
  hemu::g_calls = 0;
  return Guarded([&] {
    if (S.isParticle || S.isBdpt) throw std::runtime_error("renderer has no emulated per-sample wave");
    const uint64_t npix = (uint64_t)S.cam.width * S.cam.height;
    for (int64_t i = 0; i < n; i++)
      if (pix[i] >= npix) throw std::runtime_error("pixel index out of range");
    RenderSamples(S, pix, smp, (uint32_t)n, seed, vol_mode, out);
  });
}

}  // extern "C"
