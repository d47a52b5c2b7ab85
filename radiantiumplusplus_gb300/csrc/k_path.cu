// Wavefront `path` integrator (Path::Li, rad.offline/src/renderer/path.cpp:131-236)
// split into stages over per-bounce path queues:
//   generate   -- camera ray per pixel sample (perspective.cpp:73-82), PCG stream
//   extend     -- closest hit for every queued path (BVH8, embree.cpp:87-111)
//   shade      -- one kernel per shade class (the extend stage sorts hits into
//                 per-class queues): emitter MIS, NEE light sample + BSDF
//                 eval/pdf (emits a shadow record), BSDF sample, Russian
//                 roulette, next ray; survivors are appended to the next queue
//                 with warp-aggregated atomics
//   shadow     -- occlusion of the NEE rays (scene.cpp:53-63); unoccluded
//                 contributions are added to the path's radiance
//   accumulate -- film += radiance with the reference's invalid-sample drop
//                 (sample_renderer.cpp:93-114)
// Every stage is a grid-stride kernel over a device-side count, so a whole wave
// is a fixed launch sequence that a CUDA graph can capture.
#include "dbsdf.cuh"
#include "dscene.cuh"
#include "kernels.h"

namespace rad {

constexpr int kBlock = 128;

#ifndef RAD_HOST_EMULATION
static int g_gridBlocks = 0;
int PathGridBlocks() {
  if (g_gridBlocks == 0) {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    g_gridBlocks = sms * 8;
  }
  return g_gridBlocks;
}
#endif

RD float MisWeight(float a, float b) {  // path.cpp:231-236
  a *= a;
  b *= b;
  float w = a / (a + b);
  return isfinite(w) ? w : 0.f;
}

// Warp-aggregated append: one atomic per warp; returns the slot for this lane.
__device__ __forceinline__ uint32_t WarpAppend(uint32_t* counter, bool pred) {
  uint32_t mask = __ballot_sync(0xffffffffu, pred);
  uint32_t lane = threadIdx.x & 31u;
  uint32_t base = 0;
  if (mask) {
    int leader = __ffs(mask) - 1;
    if ((int)lane == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
  }
  return base + __popc(mask & ((1u << lane) - 1u));
}

// Camera ray, PCG stream and path state of path slot i (pixel `pix`, sample `smp`).
__device__ __forceinline__ void GeneratePath(const DevScene& S, const PathBuffers& B, uint32_t i, uint32_t pix,
                                             uint32_t smp, uint32_t seed) {
  uint32_t x = pix % (uint32_t)S.cam.width, y = pix / (uint32_t)S.cam.width;
  Pcg32 rng = PcgForSample(pix, smp, seed);
  float jx = Next1D(rng);
  float jy = Next1D(rng);
  V3 O, D;
  float tmin, tmax;
  CameraRay(S.cam, (float)x + jx, (float)y + jy, O, D, tmin, tmax);
  B.rayO[i] = make_float4(O.x, O.y, O.z, tmin);
  B.rayD[i] = make_float4(D.x, D.y, D.z, tmax);
  B.thr[i] = make_float4(1.f, 1.f, 1.f, 1.f);
  B.L[i] = make_float4(0.f, 0.f, 0.f, 1.f);
  // the first shading point has no previous vertex: the slot carries the screen
  // position, from which textured materials rebuild the camera ray differentials
  B.prev[i] = make_float4((float)x + jx, (float)y + jy, 0.f, __uint_as_float(1u));
  B.rng[i] = make_uint2((uint32_t)rng.state, (uint32_t)(rng.state >> 32));
  B.pixel[i] = pix;
  B.q[0][i] = i;
}

__global__ void __launch_bounds__(kBlock) KGenerate(DevScene S, PathBuffers B, WaveParams w) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  // reset this wave's counters (all but the sticky device-error word)
  for (uint32_t k = i; k < (uint32_t)kCounterWords; k += gridDim.x * blockDim.x) {
    if (k != (uint32_t)(kMiscBase + 1)) B.counters[k] = k == 0 ? w.count : 0u;
  }
  if (i >= w.count) return;
  const uint32_t spw = w.spw > 1u ? w.spw : 1u;
  const uint32_t npc = w.count / spw;  // pixels per sample of this wave
  const uint32_t j = spw > 1u ? i % npc : i, s = spw > 1u ? i / npc : 0u;
  uint32_t pix = w.pixelList ? w.pixelList[i] : w.pixelBegin + j;
  if (pix >= (uint32_t)S.cam.width * (uint32_t)S.cam.height) {
    // a caller's device-side pixel list the host could not check: report, and
    // trace pixel 0 instead so no film write leaves the film
    atomicOr(B.counters + kMiscBase + 1, kErrPixelRange);
    pix = 0;
  }
  uint32_t smp = w.sampleList ? w.sampleList[i] : (w.ctx ? w.ctx->sample : w.sample) + s;
  uint32_t seed = w.ctx ? w.ctx->seed : w.seed;
  GeneratePath(S, B, i, pix, smp, seed);
}

// Job of path slot i in a mixed wave (jobs hold ascending, contiguous slot ranges).
__device__ __forceinline__ uint32_t MixJobOf(const MixJob* mix, uint32_t nJobs, uint32_t i) {
  uint32_t k = 0;
  while (k + 1u < nJobs && i >= mix[k + 1u].pathBegin) k++;
  return k;
}

// Mixed wave: every job's paths, each with its own scene, pixels, samples and seed.
__global__ void __launch_bounds__(kBlock) KGenerateMix(PathBuffers B, uint32_t total, uint32_t nJobs) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  for (uint32_t k = i; k < (uint32_t)kCounterWords; k += gridDim.x * blockDim.x) {
    if (k != (uint32_t)(kMiscBase + 1)) B.counters[k] = k == 0 ? total : 0u;
  }
  if (i >= total) return;
  const uint32_t k = MixJobOf(B.mix, nJobs, i);
  const MixJob& J = B.mix[k];
  const uint32_t local = i - J.pathBegin;
  B.job[i] = (uint8_t)k;
  GeneratePath(J.S, B, i, J.pixelBegin + local % J.npc, J.sample + local / J.npc, J.seed);
}

// Adds per-warp sums of traversal counters into 64-bit totals (counting variants only).
__device__ __forceinline__ void FlushTravCounts(unsigned long long* out, uint32_t nodes, uint32_t prims) {
  for (int o = 16; o > 0; o >>= 1) {
    nodes += __shfl_down_sync(0xffffffffu, nodes, o);
    prims += __shfl_down_sync(0xffffffffu, prims, o);
  }
  if ((threadIdx.x & 31u) == 0) {
    atomicAdd(out, (unsigned long long)nodes);
    atomicAdd(out + 1, (unsigned long long)prims);
  }
}

// Persistent ray fetch: a warp keeps tracing one BVH8 node per lane per step
// while at least `refillBusy` of its lanes are still busy; then the lanes whose
// rays finished write their results and every idle lane takes the next ray of
// the queue from a per-bounce counter (one atomic per warp). Lanes of a warp thus
// stay busy although ray traversal lengths vary widely (one ray per thread left
// ~9 of 32 lanes active per instruction).
// The scene of a path: the wave's one scene, or in a mixed wave that of its job jb.
template <bool MIX>
__device__ __forceinline__ const DevScene& SceneOf(const DevScene& S0, const PathBuffers& B, uint32_t jb) {
  if constexpr (MIX) {
    return B.mix[jb].S;
  } else {
    return S0;
  }
}

// MIX: a mixed wave; each lane's ray belongs to the job B.job[p] of B.mix, whose
// scene it traces (the default instantiation reads the one scene S0).
template <bool COUNT, bool MIX>
__global__ void __launch_bounds__(kBlock, 8)
    KExtend(DevScene S0, PathBuffers B, int depth, unsigned long long* trav, int refillBusy, int leafFrac8) {
  const uint32_t count = B.counters[depth];
  // Blocks past one thread per queued ray leave at once: late bounces hold few
  // rays, and every warp's first fetch is an atomic on the one queue counter.
  if (blockIdx.x * blockDim.x >= count) return;
  const uint32_t* qin = B.q[depth & 1];
  uint32_t* fetch = B.counters + kFetchBase + 2 * depth;
  uint32_t* err = B.counters + kMiscBase + 1;
  uint32_t* classCnt = B.counters + kClassBase + depth * kShadeClasses;
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t nN = 0, nP = 0;
  bool live = false, done = false, drained = false;
  uint32_t p = 0, jb = 0;
  RayPre r;
  TraceHit h;
  TravState st;
  uint2 stack[kTraceStack];
  for (;;) {
    // ---- idle lanes take the next rays of the queue
    uint32_t need = __ballot_sync(0xffffffffu, !live);
    if (need && !drained) {
      int leader = __ffs(need) - 1;
      uint32_t base = 0;
      if ((int)lane == leader) base = atomicAdd(fetch, (uint32_t)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (base + (uint32_t)__popc(need) >= count) drained = true;
      if (!live) {
        uint32_t i = base + __popc(need & ((1u << lane) - 1u));
        if (i < count) {
          p = qin[i];
          if (MIX) jb = B.job[p];
          float4 o = B.rayO[p], d = B.rayD[p];
          r = MakeRayPre(V3{o.x, o.y, o.z}, V3{d.x, d.y, d.z}, o.w);
          TraceInit(d.w, h, st);
          live = true;
          done = SceneOf<MIX>(S0, B, jb).nNodes == 0;
        }
      }
    }
    if (__ballot_sync(0xffffffffu, live) == 0u) break;
    // ---- trace until too few lanes are busy (all of them once the queue is drained)
    const int minBusy = drained ? 1 : refillBusy;
    for (;;) {
      // leaf phase once at least leafFrac8 / 8 of the busy lanes hold pending
      // leaves (the others wait), else a node phase for the lanes without
      const bool busy = live && !done, pend = busy && st.leafMask != 0u;
      const int nb = __popc(__ballot_sync(0xffffffffu, busy));
      if (nb < minBusy || nb == 0) break;
      const bool leafPhase = 8 * __popc(__ballot_sync(0xffffffffu, pend)) >= leafFrac8 * nb;
      if (busy && pend == leafPhase)
        done = TravStep<false, COUNT>(SceneOf<MIX>(S0, B, jb), r, h, stack, st, err, &nN, &nP) != kTravContinue;
    }
    // ---- finished lanes: hit record and shade-class append
    const bool fin = live && done;
    uint32_t cls = 0xffu;
    if (fin) {
      const DevScene& S = SceneOf<MIX>(S0, B, jb);
      const bool lastDepth = S.maxDepth >= 0 && depth + 1 >= S.maxDepth;
      HitRec hr;
      hr.t = h.t;
      hr.u = h.u;
      hr.v = h.v;
      hr.prim = h.prim;
      hr.shape = h.shape;
      hr.front = h.front;
      hr.pad[0] = hr.pad[1] = 0;
      B.hit[p] = hr;
      cls = (h.prim == kNoPrim || lastDepth) ? SC_EMIT : (uint32_t)S.shapeClass[h.shape];
      live = false;
    }
    // group lanes by shade class; one atomic per class present in the warp
    uint32_t grp = __match_any_sync(0xffffffffu, cls);
    int leader = __ffs(grp) - 1;
    uint32_t slot = 0;
    if (cls != 0xffu && (int)lane == leader) slot = atomicAdd(classCnt + cls, (uint32_t)__popc(grp));
    slot = __shfl_sync(0xffffffffu, slot, leader);
    if (cls != 0xffu) {
      slot += __popc(grp & ((1u << lane) - 1u));
      B.classQ[(size_t)cls * B.capacity + slot] = p;
    }
  }
  if (COUNT) FlushTravCounts(trav, nN, nP);
}

// Guided scattering at a non-emitter hit (one-sample MIS between the guide
// mixture and the BSDF, dguide.cuh): draws the selection, samples the chosen
// strategy, weights by f cos / p_mix, applies Russian roulette as Path::Li does
// (path.cpp:213-219), writes the next ray and, on training paths, appends a
// training record (linked to this vertex's shadow record so the shadow stage
// can add the NEE radiance it owes the record). Returns whether the path continues.
template <int K>
__device__ __forceinline__ bool GuidedScatter(const DevScene& S, const PathBuffers& B, const GuideDev& G, int depth,
                                              uint32_t p, const SurfInt& si, V3 D, const MatRec* mats, uint32_t bsdf,
                                              const float4* gmix, float gc, V3 thr, float eta, Pcg32& rng,
                                              bool shadow, float4& shC, const TexCtx* tc) {
  float us = Next1D(rng);
  float xl = Next1D(rng);
  V2 xd = Next2D(rng);
  V3 f, wiW;
  float pm, bpdf, etaS = 1.f;
  bool delta = false, discrete = false, ok;
  if (us < gc) {
    wiW = GuideMixSamplePacked(gmix, xl, xd);
    V3 wl = ToLocal(si.sh, wiW);
    ClassEvalPdf<K>(mats, bsdf, si.Wi, wl, f, bpdf, tc);
    pm = gc * GuideMixPdfPacked(gmix, wiW) + (1.f - gc) * bpdf;
    ok = pm > 0.f && !is_zero(f);
  } else {
    BsdfSampleRes bs = ClassSample<K>(mats, bsdf, si.Wi, xl, xd, tc);
    f = bs.f;
    bpdf = bs.pdf;
    etaS = bs.eta;
    delta = (bs.type & BT_DELTA) != 0u;
    // delta lobes and mask pass-through are point masses the guide never draws
    discrete = (bs.type & (BT_DELTA | BT_NULL)) != 0u;
    wiW = ToWorld(si.sh, bs.wo);
    pm = discrete ? (1.f - gc) * bs.pdf : gc * GuideMixPdfPacked(gmix, wiW) + (1.f - gc) * bs.pdf;
    ok = bs.pdf > 0.f && pm > 0.f;
  }
  if (!ok) return false;
  V3 thr0 = thr;
  thr = cmul(thr, f) / pm;
  eta *= etaS;
  if (depth >= S.rrDepth) {
    float rr = fminr(max_comp(thr) * Sqr(eta), 0.95f);
    if (Next1D(rng) > rr) return false;
    thr = thr * Rcp(rr);
  }
  V3 no = OffsetP(si.P, si.N, wiW);
  B.rayO[p] = make_float4(no.x, no.y, no.z, 0.f);
  B.rayD[p] = make_float4(wiW.x, wiW.y, wiW.z, kFloatMax);
  B.thr[p] = make_float4(thr.x, thr.y, thr.z, eta);
  B.prev[p] = make_float4(si.P.x, si.P.y, si.P.z, __uint_as_float(delta ? 1u : 0u));
  B.rng[p] = make_uint2((uint32_t)rng.state, (uint32_t)(rng.state >> 32));
  float4 L4 = B.L[p];
  B.L[p] = make_float4(L4.x, L4.y, L4.z, pm);
  if (G.train && !discrete && (uint32_t)depth < G.trainDepth &&
      (G.trainShift == 0u || (GuideHash32(p ^ G.trainSalt) >> (32u - G.trainShift)) == 0u)) {
    uint32_t slot = atomicAdd(G.ctl, 1u);
    if (slot < G.recCap) {
      float4* r = G.rec + (size_t)slot * kGRecF4;
      r[0] = make_float4(si.P.x, si.P.y, si.P.z, bpdf);
      r[1] = make_float4(si.sh.N.x, si.sh.N.y, si.sh.N.z, __uint_as_float(p));
      r[2] = make_float4(-D.x, -D.y, -D.z, pm);
      r[3] = make_float4(wiW.x, wiW.y, wiW.z, 0.f);
      r[4] = make_float4(L4.x, L4.y, L4.z, 0.f);
      r[5] = make_float4(thr0.x, thr0.y, thr0.z, 0.f);
      if (shadow) shC.w = __uint_as_float(slot + 1u);
    }
  }
  return true;
}

// Path::Li for one bounce, for the paths of shade class K (path.cpp:141-225).
// SC_EMIT: misses, emitter hits, shapes without a BSDF and the last bounce --
// emitter MIS only, then the path ends. Other classes: hits on a non-emitter
// shape with a BSDF of that class -- NEE, BSDF sample, Russian roulette.
constexpr int kShadeMaxBlock = 256;  // the tuner's largest shade block

template <int K, bool GUIDED, bool MIX>
__global__ void __launch_bounds__(kShadeMaxBlock) KShadeClass(DevScene S0, PathBuffers B, GuideDev G, int depth) {
  uint32_t count = B.counters[kClassBase + depth * kShadeClasses + K];
  const uint32_t* qin = B.classQ + (size_t)K * B.capacity;
  uint32_t* qout = B.q[(depth + 1) & 1];
  uint32_t* cntOut = B.counters + depth + 1;
  uint32_t* cntSh = B.counters + kShadowBase + depth;
  uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t base = blockIdx.x * blockDim.x; base < count; base += stride) {
    uint32_t i = base + threadIdx.x;
    bool active = i < count;
    bool keep = false, shadow = false;
    uint32_t p = 0;
    float4 shO = make_float4(0, 0, 0, 0), shD = shO, shC = shO;
    if (active) {
      p = qin[i];
      const DevScene& S = SceneOf<MIX>(S0, B, MIX ? B.job[p] : 0u);
      HitRec h = B.hit[p];
      float4 ro = B.rayO[p], rd = B.rayD[p];
      V3 O{ro.x, ro.y, ro.z}, D{rd.x, rd.y, rd.z};
      float4 thr4 = B.thr[p];
      V3 thr{thr4.x, thr4.y, thr4.z};
      if constexpr (K == SC_EMIT) {
        float4 L4 = B.L[p];
        int hitLight = h.prim != kNoPrim ? S.shapes[h.shape].light : S.envLight;
        if (hitLight >= 0) {
          bool anyHit = h.prim != kNoPrim;
          SurfInt si;
          if (anyHit) {
            TraceHit th{h.t, h.u, h.v, h.prim, h.shape, h.front};
            si = ComputeSI(S, O, D, th);
          } else {
            si.T = kInf;
            si.P = v3s(0.f);
            si.N = v3s(0.f);
            si.shape = -1;
            si.sh.S = si.sh.T = si.sh.N = v3s(0.f);
            si.Wi = -D;  // scene.cpp:45-47: world-space -D on a miss
          }
          V2 uvL{0.f, 0.f};  // a bitmap area light reads its radiance at the hit's uv
          if (anyHit && S.lights[hitLight].tex && S.lights[hitLight].kind == LIGHT_AREA) {
            TraceHit th{h.t, h.u, h.v, h.prim, h.shape, h.front};
            uvL = ComputeUV(S, th, si).uv;
          }
          float4 pv = B.prev[p];
          bool specular = __float_as_uint(pv.w) & 1u;
          float weight;
          if (specular) {
            weight = 1.f;
          } else {
            // SurfaceInteraction::ToDsr (interaction.cpp:68-74)
            V3 prevP{pv.x, pv.y, pv.z};
            V3 rel = si.P - prevP;
            float dist = norm(rel);
            V3 dir = anyHit ? rel / dist : -si.Wi;
            weight = MisWeight(L4.w, PdfLightDirection(S, hitLight, prevP, dir, si.sh.N, dist, uvL));
          }
          V3 li = EvalLightAt(S, hitLight, &si, uvL);
          V3 L = V3{L4.x, L4.y, L4.z} + cmul(thr, li) * weight;
          B.L[p] = make_float4(L.x, L.y, L.z, L4.w);
        }
      } else {
        float eta = thr4.w;
        uint2 rs = B.rng[p];
        Pcg32 rng;
        rng.state = ((uint64_t)rs.y << 32) | rs.x;
        TraceHit th{h.t, h.u, h.v, h.prim, h.shape, h.front};
        SurfInt si = ComputeSI(S, O, D, th);
        uint32_t bsdf = (uint32_t)S.shapes[h.shape].bsdf;
        const MatRec* mats = S.mats;
        // textured materials are all in the generic class: uv (and, on camera
        // rays, uv derivatives) for their lookups
        TexCtx tcx;
        const TexCtx* tc = nullptr;
        if constexpr (K == SC_GENERIC) {
          if (S.nTex) {
            SurfUV su = ComputeUV(S, th, si);
            tcx = TexCtx{S.tex, S.texels, S.texBind, su.uv, V2{0.f, 0.f}, V2{0.f, 0.f}};
            if (depth == 0 && S.needDiff) {
              float4 pv = B.prev[p];
              CameraUVDerivs(S.cam, pv.x, pv.y, O, si, su, tcx.duvdx, tcx.duvdy);
            }
            tc = &tcx;
          }
        }
        const float4* gmix = nullptr;
        float gc = 0.f;
        if constexpr (GUIDED) {
          gmix = G.mix + (size_t)p * kGMixF4;
          // a BSDF with only delta lobes gives the guide nothing to propose
          gc = (mats[bsdf].flags & BT_NODELTA) ? gmix[10].x : 0.f;
        }
        if (mats[bsdf].flags & BT_NODELTA) {
          float xl = Next1D(rng);
          V2 xd = Next2D(rng);
          V3 li;
          DirSample dsr = SampleLightDirection(S, si.P, xl, xd, li);
          if (dsr.Pdf > 0.f) {
            V3 wo = ToLocal(si.sh, dsr.Dir);
            V3 f;
            float bsdfPdf;
            ClassEvalPdf<K>(mats, bsdf, si.Wi, wo, f, bsdfPdf, tc);
            if constexpr (GUIDED) bsdfPdf = gc * GuideMixPdfPacked(gmix, dsr.Dir) + (1.f - gc) * bsdfPdf;
            // Scene::IsOcclude (scene.cpp:53-63)
            V3 so = OffsetP(si.P, si.N, dsr.P - si.P);
            V3 sd = dsr.P - so;
            float sdist = norm(sd);
            if (!(sdist < kShadowEps)) {
              sd = sd / sdist;
              float weight = dsr.IsDelta ? 1.f : MisWeight(dsr.Pdf, bsdfPdf);
              V3 c = cmul(cmul(thr, f), li) * weight / dsr.Pdf;
              shadow = true;
              shO = make_float4(so.x, so.y, so.z, sdist * (1.f - kShadowEps));
              shD = make_float4(sd.x, sd.y, sd.z, __uint_as_float(p));
              shC = make_float4(c.x, c.y, c.z, 0.f);
            }
          }
        }
        if constexpr (GUIDED) {
          keep = GuidedScatter<K>(S, B, G, depth, p, si, D, mats, bsdf, gmix, gc, thr, eta, rng, shadow, shC, tc);
        } else {
        float xl = Next1D(rng);
        V2 xd = Next2D(rng);
        BsdfSampleRes bs = ClassSample<K>(mats, bsdf, si.Wi, xl, xd, tc);
        if (bs.pdf > 0.f) {
          thr = cmul(thr, bs.f) / bs.pdf;
          eta *= bs.eta;
          bool survive = true;
          if (depth >= S.rrDepth) {
            float rr = fminr(max_comp(thr) * Sqr(eta), 0.95f);
            if (Next1D(rng) > rr) {
              survive = false;
            } else {
              thr = thr * Rcp(rr);
            }
          }
          if (survive) {
            keep = true;
            V3 nd = ToWorld(si.sh, bs.wo);
            V3 no = OffsetP(si.P, si.N, nd);
            bool specular = (bs.type & BT_DELTA) != 0u;
            B.rayO[p] = make_float4(no.x, no.y, no.z, 0.f);
            B.rayD[p] = make_float4(nd.x, nd.y, nd.z, kFloatMax);
            B.thr[p] = make_float4(thr.x, thr.y, thr.z, eta);
            B.prev[p] = make_float4(si.P.x, si.P.y, si.P.z, __uint_as_float(specular ? 1u : 0u));
            B.rng[p] = make_uint2((uint32_t)rng.state, (uint32_t)(rng.state >> 32));
            float4 L4 = B.L[p];
            B.L[p] = make_float4(L4.x, L4.y, L4.z, bs.pdf);
          }
        }
        }
      }
    }
    if constexpr (K != SC_EMIT) {
      uint32_t slot = WarpAppend(cntOut, keep);
      if (keep) qout[slot] = p;
      uint32_t sslot = WarpAppend(cntSh, shadow);
      if (shadow) {
        B.shO[sslot] = shO;
        B.shD[sslot] = shD;
        B.shC[sslot] = shC;
      }
    }
  }
}

// AO::Li (ao.cpp:22-36) after the first hit: a cosine-weighted direction and a
// visibility ray of unbounded length; the shadow stage adds cos / pi / pdf when
// nothing blocks it. Misses contribute 0.
__global__ void __launch_bounds__(kBlock) KShadeAO(DevScene S, PathBuffers B) {
  uint32_t count = B.counters[0];
  uint32_t* cntSh = B.counters + kShadowBase;
  uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t base = blockIdx.x * blockDim.x; base < count; base += stride) {
    uint32_t i = base + threadIdx.x;
    bool shadow = false;
    float4 shO = make_float4(0, 0, 0, 0), shD = shO, shC = shO;
    if (i < count) {
      uint32_t p = B.q[0][i];
      HitRec h = B.hit[p];
      if (h.prim != kNoPrim) {
        float4 ro = B.rayO[p], rd = B.rayD[p];
        TraceHit th{h.t, h.u, h.v, h.prim, h.shape, h.front};
        SurfInt si = ComputeSI(S, V3{ro.x, ro.y, ro.z}, V3{rd.x, rd.y, rd.z}, th);
        uint2 rs = B.rng[p];
        Pcg32 rng;
        rng.state = ((uint64_t)rs.y << 32) | rs.x;
        V3 wo = SquareToCosineHemisphere(Next2D(rng));
        float pdf = SquareToCosineHemispherePdf(wo);
        if (wo.z > 0.f) {
          V3 d = ToWorld(si.sh, wo);
          V3 o = OffsetP(si.P, si.N, d);
          float l = wo.z / kPi / pdf;
          shadow = true;
          shO = make_float4(o.x, o.y, o.z, kFloatMax);
          shD = make_float4(d.x, d.y, d.z, __uint_as_float(p));
          shC = make_float4(l, l, l, 0.f);
        }
      }
    }
    uint32_t sslot = WarpAppend(cntSh, shadow);
    if (shadow) {
      B.shO[sslot] = shO;
      B.shD[sslot] = shD;
      B.shC[sslot] = shC;
    }
  }
}

template <bool COUNT, bool MIX>
__global__ void __launch_bounds__(kBlock, 8)
    KShadow(DevScene S0, PathBuffers B, int depth, unsigned long long* trav, int refillBusy, int leafFrac8) {
  const uint32_t count = B.counters[kShadowBase + depth];
  if (blockIdx.x * blockDim.x >= count) return;  // as KExtend
  uint32_t* fetch = B.counters + kFetchBase + 2 * depth + 1;
  uint32_t* err = B.counters + kMiscBase + 1;
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t nN = 0, nP = 0;
  bool live = false, done = false, drained = false, occ = false;
  uint32_t i = 0, jb = 0;
  RayPre r;
  TraceHit h;
  TravState st;
  uint2 stack[kTraceStack];
  for (;;) {
    uint32_t need = __ballot_sync(0xffffffffu, !live);
    if (need && !drained) {
      int leader = __ffs(need) - 1;
      uint32_t base = 0;
      if ((int)lane == leader) base = atomicAdd(fetch, (uint32_t)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (base + (uint32_t)__popc(need) >= count) drained = true;
      if (!live) {
        uint32_t k = base + __popc(need & ((1u << lane) - 1u));
        if (k < count) {
          i = k;
          float4 o = B.shO[i], d = B.shD[i];
          if (MIX) jb = B.job[__float_as_uint(d.w)];
          r = MakeRayPre(V3{o.x, o.y, o.z}, V3{d.x, d.y, d.z}, 0.f);
          TraceInit(o.w, h, st);
          live = true;
          done = SceneOf<MIX>(S0, B, jb).nNodes == 0;
          occ = false;
        }
      }
    }
    if (__ballot_sync(0xffffffffu, live) == 0u) break;
    const int minBusy = drained ? 1 : refillBusy;
    for (;;) {
      const bool busy = live && !done, pend = busy && st.leafMask != 0u;
      const int nb = __popc(__ballot_sync(0xffffffffu, busy));
      if (nb < minBusy || nb == 0) break;
      const bool leafPhase = 8 * __popc(__ballot_sync(0xffffffffu, pend)) >= leafFrac8 * nb;
      if (busy && pend == leafPhase) {
        int res = TravStep<true, COUNT>(SceneOf<MIX>(S0, B, jb), r, h, stack, st, err, &nN, &nP);
        if (res != kTravContinue) {
          done = true;
          occ = res == kTravDone && h.prim != kNoPrim;
        }
      }
    }
    if (live && done) {
      if (!occ) {
        uint32_t p = __float_as_uint(B.shD[i].w);
        float4 c = B.shC[i];
        float4 l = B.L[p];
        B.L[p] = make_float4(l.x + c.x, l.y + c.y, l.z + c.z, l.w);
        uint32_t rec = __float_as_uint(c.w);  // guide training record + 1, or 0
        if (rec) {
          float4* r4 = B.guideRec + (size_t)(rec - 1u) * kGRecF4 + 4;
          float4 lb = *r4;
          *r4 = make_float4(lb.x + c.x, lb.y + c.y, lb.z + c.z, lb.w);
        }
      }
      live = false;
    }
  }
  if (COUNT) FlushTravCounts(trav + 2, nN, nP);
}

// sample_renderer.cpp:101-105: drop NaN in any channel, Inf / negative in the
// first channel only (spectrum.h:28-29), the sample still counts in 1/spp.
// One thread per pixel of the wave; with spw samples per wave it adds them in
// sample order, so the film is the same as after spw one-sample waves.
__global__ void __launch_bounds__(256)
    KAccumulate(PathBuffers B, FilmView film, uint32_t count, WaveCtx* ctx, uint32_t spw) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (ctx) {
    film.accum = ctx->film;
    film.stats = ctx->stats;
    if (i == 0) ctx->sample += spw;  // generate of this wave has completed: advance for the next replay
  }
  if (i == 0 && film.stats) {
    unsigned long long cl = 0, sh = 0;
    for (int k = 0; k <= kMaxBounce; k++) {
      cl += B.counters[k];
      sh += B.counters[kShadowBase + k];
    }
    cl += B.counters[kMiscBase + 2];
    sh += B.counters[kMiscBase + 3];
    film.stats[0] += cl;
    film.stats[1] += sh;
    film.stats[3] += count;
  }
  const uint32_t npc = count / spw;
  uint32_t nbad = 0;
  if (i < npc) {
    uint32_t pix = B.pixel[i];
    float4 a = film.accum[pix];
    for (uint32_t s = 0; s < spw; s++) {
      float4 l = B.L[(size_t)s * npc + i];
      bool bad = isnan(l.x) || isnan(l.y) || isnan(l.z) || isinf(l.x) || l.x < 0.f;
      if (!bad) {
        a.x += l.x;
        a.y += l.y;
        a.z += l.z;
      } else {
        nbad++;
      }
      a.w += 1.f;
    }
    film.accum[pix] = a;
  }
  for (int o = 16; o > 0; o >>= 1) nbad += __shfl_down_sync(0xffffffffu, nbad, o);
  if (nbad && (threadIdx.x & 31u) == 0 && film.stats) atomicAdd(film.stats + 2, (unsigned long long)nbad);
}

// Mixed wave: one thread per (job, pixel) of the wave adds that pixel's spw
// samples, in sample order, into its job's film, with KAccumulate's
// invalid-sample rule. Samples and invalid samples are counted per job; the
// wave's rays are apportioned to its jobs by their shares of its paths.
__global__ void __launch_bounds__(256)
    KAccumulateMix(PathBuffers B, uint32_t totalPix, uint32_t total, uint32_t nJobs) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0) {
    unsigned long long cl = 0, sh = 0;
    for (int k = 0; k <= kMaxBounce; k++) {
      cl += B.counters[k];
      sh += B.counters[kShadowBase + k];
    }
    for (uint32_t k = 0; k < nJobs; k++) {
      unsigned long long* st = B.mix[k].stats;
      const unsigned long long c = B.mix[k].count;
      if (!st) continue;
      st[0] += cl * c / total;
      st[1] += sh * c / total;
      st[3] += c;
    }
  }
  if (t >= totalPix) return;
  uint32_t k = 0, base = 0;
  while (k + 1u < nJobs && t >= base + B.mix[k].npc) {
    base += B.mix[k].npc;
    k++;
  }
  const MixJob& J = B.mix[k];
  const uint32_t j = t - base;
  float4* px = J.film + (J.pixelBegin + j);
  float4 a = *px;
  uint32_t nbad = 0;
  for (uint32_t s = 0; s < J.spw; s++) {
    float4 l = B.L[J.pathBegin + s * J.npc + j];
    bool bad = isnan(l.x) || isnan(l.y) || isnan(l.z) || isinf(l.x) || l.x < 0.f;
    if (!bad) {
      a.x += l.x;
      a.y += l.y;
      a.z += l.z;
    } else {
      nbad++;
    }
    a.w += 1.f;
  }
  *px = a;
  if (nbad && J.stats) atomicAdd(J.stats + 2, (unsigned long long)nbad);
}

__global__ void KGatherRadiance(PathBuffers B, uint32_t count, float* out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  float4 l = B.L[i];
  out[3 * i] = l.x;
  out[3 * i + 1] = l.y;
  out[3 * i + 2] = l.z;
}

__global__ void KResolveFilm(FilmView film, float scale, float* out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)(film.width * film.height)) return;
  float4 a = film.accum[i];
  out[3 * i] = a.x * scale;
  out[3 * i + 1] = a.y * scale;
  out[3 * i + 2] = a.z * scale;
}

#ifndef RAD_HOST_EMULATION
// ---- launchers (a host harness runs the kernels above as loops over their grids)
cudaError_t LaunchGenerate(const DevScene& S, const PathBuffers& B, const WaveParams& w, cudaStream_t st) {
  uint32_t n = w.count > (uint32_t)kCounterWords ? w.count : (uint32_t)kCounterWords;
  KGenerate<<<(n + kBlock - 1) / kBlock, kBlock, 0, st>>>(S, B, w);
  return cudaGetLastError();
}
cudaError_t LaunchExtend(const DevScene& S, const PathBuffers& B, int depth, int grid, cudaStream_t st,
                         unsigned long long* trav, int refillBusy, int leafFrac8, bool mix) {
  if (mix)
    KExtend<false, true><<<grid, kBlock, 0, st>>>(S, B, depth, nullptr, refillBusy, leafFrac8);
  else if (trav)
    KExtend<true, false><<<grid, kBlock, 0, st>>>(S, B, depth, trav, refillBusy, leafFrac8);
  else
    KExtend<false, false><<<grid, kBlock, 0, st>>>(S, B, depth, nullptr, refillBusy, leafFrac8);
  return cudaGetLastError();
}
cudaError_t LaunchShade(const DevScene& S, const PathBuffers& B, int depth, int grid, cudaStream_t st,
                        const GuideDev* G, bool mix, int block) {
  GuideDev none{};
  if (block != 64 && block != 256) block = kBlock;
  grid = std::max(1, grid * kBlock / block);
  if (mix) {  // mixed waves hold plain jobs only
    KShadeClass<SC_EMIT, false, true><<<grid, block, 0, st>>>(S, B, none, depth);
    KShadeClass<SC_GLASS, false, true><<<grid, block, 0, st>>>(S, B, none, depth);
    KShadeClass<SC_DIFFUSE, false, true><<<grid, block, 0, st>>>(S, B, none, depth);
    KShadeClass<SC_METAL, false, true><<<grid, block, 0, st>>>(S, B, none, depth);
    KShadeClass<SC_DISNEY, false, true><<<grid, block, 0, st>>>(S, B, none, depth);
    KShadeClass<SC_GENERIC, false, true><<<grid, block, 0, st>>>(S, B, none, depth);
    return cudaGetLastError();
  }
  KShadeClass<SC_EMIT, false, false><<<grid, block, 0, st>>>(S, B, none, depth);
  KShadeClass<SC_GLASS, false, false><<<grid, block, 0, st>>>(S, B, none, depth);
  if (G) {
    KShadeClass<SC_DIFFUSE, true, false><<<grid, block, 0, st>>>(S, B, *G, depth);
    KShadeClass<SC_METAL, true, false><<<grid, block, 0, st>>>(S, B, *G, depth);
    KShadeClass<SC_DISNEY, true, false><<<grid, block, 0, st>>>(S, B, *G, depth);
    KShadeClass<SC_GENERIC, true, false><<<grid, block, 0, st>>>(S, B, *G, depth);
  } else {
    KShadeClass<SC_DIFFUSE, false, false><<<grid, block, 0, st>>>(S, B, none, depth);
    KShadeClass<SC_METAL, false, false><<<grid, block, 0, st>>>(S, B, none, depth);
    KShadeClass<SC_DISNEY, false, false><<<grid, block, 0, st>>>(S, B, none, depth);
    KShadeClass<SC_GENERIC, false, false><<<grid, block, 0, st>>>(S, B, none, depth);
  }
  return cudaGetLastError();
}
cudaError_t LaunchShadeAO(const DevScene& S, const PathBuffers& B, int grid, cudaStream_t st) {
  KShadeAO<<<grid, kBlock, 0, st>>>(S, B);
  return cudaGetLastError();
}
cudaError_t LaunchShadow(const DevScene& S, const PathBuffers& B, int depth, int grid, cudaStream_t st,
                         unsigned long long* trav, int refillBusy, int leafFrac8, bool mix) {
  if (mix)
    KShadow<false, true><<<grid, kBlock, 0, st>>>(S, B, depth, nullptr, refillBusy, leafFrac8);
  else if (trav)
    KShadow<true, false><<<grid, kBlock, 0, st>>>(S, B, depth, trav, refillBusy, leafFrac8);
  else
    KShadow<false, false><<<grid, kBlock, 0, st>>>(S, B, depth, nullptr, refillBusy, leafFrac8);
  return cudaGetLastError();
}
cudaError_t LaunchAccumulate(const PathBuffers& B, const FilmView& film, uint32_t count, cudaStream_t st,
                             WaveCtx* ctx, uint32_t spw) {
  if (count == 0) return cudaSuccess;
  if (spw < 1u) spw = 1u;
  uint32_t npc = count / spw;
  KAccumulate<<<(npc + 255) / 256, 256, 0, st>>>(B, film, count, ctx, spw);
  return cudaGetLastError();
}
cudaError_t LaunchGenerateMix(const PathBuffers& B, uint32_t total, uint32_t nJobs, cudaStream_t st) {
  uint32_t n = total > (uint32_t)kCounterWords ? total : (uint32_t)kCounterWords;
  KGenerateMix<<<(n + kBlock - 1) / kBlock, kBlock, 0, st>>>(B, total, nJobs);
  return cudaGetLastError();
}
cudaError_t LaunchAccumulateMix(const PathBuffers& B, uint32_t totalPixels, uint32_t total, uint32_t nJobs,
                                cudaStream_t st) {
  if (totalPixels == 0) return cudaSuccess;
  KAccumulateMix<<<(totalPixels + 255) / 256, 256, 0, st>>>(B, totalPixels, total, nJobs);
  return cudaGetLastError();
}
cudaError_t LaunchGatherRadiance(const PathBuffers& B, uint32_t count, float* out, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  KGatherRadiance<<<(count + 255) / 256, 256, 0, st>>>(B, count, out);
  return cudaGetLastError();
}
cudaError_t LaunchResolveFilm(const FilmView& film, float scale, float* out, cudaStream_t st) {
  uint32_t n = (uint32_t)(film.width * film.height);
  if (n == 0) return cudaSuccess;
  KResolveFilm<<<(n + 255) / 256, 256, 0, st>>>(film, scale, out);
  return cudaGetLastError();
}

#endif  // RAD_HOST_EMULATION

}  // namespace rad
