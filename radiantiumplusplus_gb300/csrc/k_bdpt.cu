// Renderer "bdpt" as a wavefront over one wave of pixel samples (the per-sample
// steps are in dbdpt.cuh):
//   camera subpaths: KBdptCamera, then per bounce the BVH8 closest-hit kernel
//     (KExtend) and KBdptWalk;
//   light subpaths: KBdptLight, the same bounce loop, KBdptLightFix;
//   connections, one round per camera vertex index t, over the samples ordered
//     by subpath lengths: round 1 (t = 1, splats) one thread per connection,
//     each starting from the sample's stream advanced past the draws of the
//     connections before it; rounds t >= 2 the s <= 1 connections per sample
//     (s = 1 draws the round's random numbers) and the s >= 2 ones one per
//     thread. Every connection queues its visibility ray; KBdptShadow traces
//     them with the persistent any-hit traversal and adds the unoccluded
//     contributions (atomics: a sample has several) to the sample or, for
//     t = 1, to the film pixel they land on;
//   KBdptAccumulate adds each valid sample into the film.
#include <algorithm>

#include "dbdpt.cuh"
#include "kernels.h"

namespace rad {

static_assert(sizeof(BVert) == kBVertBytes, "BVert size");

constexpr int kBdptBlock = 128;

RD VPath CamPath(const BdptBuffers& V, uint32_t p) { return VPath{V.vert + p, V.nw}; }
RD VPath LightPathOf(const BdptBuffers& V, uint32_t p) { return VPath{V.vert + (size_t)V.cap * V.nw + p, V.nw}; }

RD void StoreWalk(const BdptBuffers& V, uint32_t p, const WalkState& w) {
  V.walkA[p] = make_float4(w.thr.x, w.thr.y, w.thr.z, w.eta);
  V.walkB[p] = make_float4(w.pdfFwd, w.rr, __uint_as_float((uint32_t)w.n), 0.f);
}
RD WalkState LoadWalk(const BdptBuffers& V, uint32_t p) {
  float4 a = V.walkA[p], b = V.walkB[p];
  WalkState w;
  w.thr = V3{a.x, a.y, a.z};
  w.eta = a.w;
  w.pdfFwd = b.x;
  w.rr = b.y;
  w.n = (int)__float_as_uint(b.z);
  return w;
}
RD void StoreRng(const PathBuffers& B, uint32_t p, const Pcg32& rng) {
  B.rng[p] = make_uint2((uint32_t)rng.state, (uint32_t)(rng.state >> 32));
}
RD Pcg32 LoadRng(const PathBuffers& B, uint32_t p) {
  uint2 s = B.rng[p];
  Pcg32 r;
  r.state = (uint64_t)s.x | ((uint64_t)s.y << 32);
  return r;
}

// Warp-aggregated append of p to queue q (all lanes of the warp call it).
__device__ __forceinline__ void Enqueue(uint32_t* q, uint32_t* cnt, uint32_t p, bool push) {
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t m = __ballot_sync(0xffffffffu, push);
  if (!m) return;
  int leader = __ffs(m) - 1;
  uint32_t base = 0;
  if ((int)lane == leader) base = atomicAdd(cnt, (uint32_t)__popc(m));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (push) q[base + __popc(m & ((1u << lane) - 1u))] = p;
}

__global__ void __launch_bounds__(kBdptBlock) KBdptCamera(DevScene S, PathBuffers B, BdptBuffers V, WaveParams w) {
  const uint32_t spw = w.spw > 1u ? w.spw : 1u;
  const uint32_t npc = w.count / spw;
  uint32_t* maxCam = B.counters + kMiscBase;
  for (uint32_t base = blockIdx.x * blockDim.x; base < w.count; base += gridDim.x * blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    bool push = false;
    if (i < w.count) {
      const uint32_t j = spw > 1u ? i % npc : i, s = spw > 1u ? i / npc : 0u;
      uint32_t pix = w.pixelList ? w.pixelList[i] : w.pixelBegin + j;
      uint32_t smp = w.sampleList ? w.sampleList[i] : w.sample + s;
      Pcg32 rng = PcgForSample(pix, smp, w.seed);
      WalkState ws;
      V3 O, D;
      float tmin, tmax;
      CameraPathStart(S, rng, pix, CamPath(V, i), ws, O, D, tmin, tmax);
      push = WalkContinue(S, rng, ws, 0);
      B.rayO[i] = make_float4(O.x, O.y, O.z, tmin);
      B.rayD[i] = make_float4(D.x, D.y, D.z, tmax);
      StoreWalk(V, i, ws);
      StoreRng(B, i, rng);
      B.pixel[i] = pix;
      B.L[i] = make_float4(0.f, 0.f, 0.f, 0.f);
      V.nCam[i] = (uint32_t)ws.n;
      V.nLight[i] = 0u;
      if (!push) atomicMax(maxCam, (uint32_t)ws.n);
    }
    Enqueue(B.q[0], B.counters, i, push);
  }
}

__global__ void __launch_bounds__(kBdptBlock) KBdptLight(DevScene S, PathBuffers B, BdptBuffers V, uint32_t count) {
  for (uint32_t base = blockIdx.x * blockDim.x; base < count; base += gridDim.x * blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    bool push = false;
    if (i < count) {
      Pcg32 rng = LoadRng(B, i);
      WalkState ws;
      V3 O, D;
      LightFix fix{};
      if (LightPathStart(S, rng, LightPathOf(V, i), ws, O, D, fix)) {
        push = WalkContinue(S, rng, ws, 0);
        B.rayO[i] = make_float4(O.x, O.y, O.z, 0.f);
        B.rayD[i] = make_float4(D.x, D.y, D.z, kFloatMax);
        StoreWalk(V, i, ws);
        V.fix[i] = make_float4(fix.D.x, fix.D.y, fix.D.z, fix.pdfPos);
      }
      StoreRng(B, i, rng);
      V.nLight[i] = (uint32_t)ws.n;
    }
    Enqueue(B.q[0], B.counters, i, push);
  }
}

template <bool LIGHT>
__global__ void __launch_bounds__(kBdptBlock) KBdptWalk(DevScene S, PathBuffers B, BdptBuffers V, int depth) {
  uint32_t start[kShadeClasses + 1];  // the hits class by class (neighbours sample the same kind of BSDF)
  ClassQueueStarts(B, depth, start);
  const uint32_t count = start[kShadeClasses];
  uint32_t* maxCam = B.counters + kMiscBase;
  for (uint32_t base = blockIdx.x * blockDim.x; base < count; base += gridDim.x * blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    bool push = false;
    uint32_t p = 0;
    if (i < count) {
      p = ClassQueueEntry(B, start, i);
      Pcg32 rng = LoadRng(B, p);
      WalkState ws = LoadWalk(V, p);
      float4 o4 = B.rayO[p], d4 = B.rayD[p];
      V3 O{o4.x, o4.y, o4.z}, D{d4.x, d4.y, d4.z};
      HitRec hr = B.hit[p];
      TraceHit h{hr.t, hr.u, hr.v, hr.prim, hr.shape, hr.front};
      VPath path = LIGHT ? LightPathOf(V, p) : CamPath(V, p);
      bool go = WalkStep(S, rng, path, (int)V.cap, ws, depth, LIGHT, hr.prim != kNoPrim, h, O, D);
      if (go) go = WalkContinue(S, rng, ws, depth + 1);
      if (go) {
        B.rayO[p] = make_float4(O.x, O.y, O.z, 0.f);
        B.rayD[p] = make_float4(D.x, D.y, D.z, kFloatMax);
      }
      StoreWalk(V, p, ws);
      StoreRng(B, p, rng);
      if (LIGHT) {
        V.nLight[p] = (uint32_t)ws.n;
      } else {
        V.nCam[p] = (uint32_t)ws.n;
        if (!go) atomicMax(maxCam, (uint32_t)ws.n);
      }
      push = go;
    }
    Enqueue(B.q[(depth + 1) & 1], B.counters + depth + 1, p, push);
  }
}

RD uint32_t SortKey(const BdptBuffers& V, uint32_t p) { return V.nCam[p] * (V.cap + 1u) + V.nLight[p]; }

__global__ void __launch_bounds__(kBdptBlock) KBdptLightFix(DevScene S, BdptBuffers V, uint32_t count) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    uint32_t n = V.nLight[i];
    atomicAdd(V.keyFill + SortKey(V, i), 1u);
    if (n == 0u) continue;
    float4 f = V.fix[i];
    LightPathFinish(S, LightPathOf(V, i), (int)n, LightFix{V3{f.x, f.y, f.z}, f.w});
  }
}

// Exclusive scan of the key counts (at most 65^2 keys: one thread suffices),
// which become the scatter cursors.
__global__ void KBdptKeyScan(BdptBuffers V) {
  const uint32_t nk = (V.cap + 1u) * (V.cap + 1u);
  uint32_t acc = 0, items = 0;
  for (uint32_t k = 0; k < nk; k++) {
    uint32_t c = V.keyFill[k], nl = k % (V.cap + 1u);
    V.keyStart[k] = acc;
    V.itemStart[k] = items;
    V.keyFill[k] = acc;
    acc += c;
    items += nl > 1u ? c * (nl - 1u) : 0u;
  }
  V.keyStart[nk] = acc;
  V.itemStart[nk] = items;
}

__global__ void __launch_bounds__(kBdptBlock) KBdptKeyScatter(BdptBuffers V, uint32_t count) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
    V.order[atomicAdd(V.keyFill + SortKey(V, i), 1u)] = i;
}

// Queues the visibility ray of connection `o` of sample p (round t).
__device__ __forceinline__ void EmitConnection(const DevScene& S, const BdptBuffers& V, uint32_t* nsh, uint32_t* err,
                                               uint32_t p, const ConnOut& o, bool splats) {
  uint32_t tag = p;
  if (o.splat) {
    if (!splats) return;
    int x = (int)o.pixel.x, y = (int)o.pixel.y;
    if (x < 0 || y < 0 || x >= S.cam.width || y >= S.cam.height) return;
    tag = 0x80000000u | (uint32_t)(y * S.cam.width + x);
  }
  V3 ro, rd;
  float tmax;
  if (!ShadowRay(o.P, o.N, o.target, ro, rd, tmax)) return;
  uint32_t slot = atomicAdd(nsh, 1u);
  if (slot >= V.shCap) {
    atomicOr(err, 8u);  // more visibility rays than the round's buffer holds
    return;
  }
  V.shO[slot] = make_float4(ro.x, ro.y, ro.z, tmax);
  V.shD[slot] = make_float4(rd.x, rd.y, rd.z, __uint_as_float(tag));
  V.shC[slot] = make_float4(o.c.x, o.c.y, o.c.z, 0.f);
}

// Round t >= 2, the s = 0 and s = 1 connections of each sample of the suffix
// (the only ones of the round that draw random numbers: s = 1's light sample),
// in the order of V.items (by the camera vertex's shade class).
__global__ void __launch_bounds__(kBdptBlock) KBdptConnectHead(DevScene S, PathBuffers B, BdptBuffers V, uint32_t count,
                                                              int t) {
  uint32_t* nsh = B.counters + kShadowBase + (t - 1);
  uint32_t* err = B.counters + kMiscBase + 1;
  const uint32_t first = V.keyStart[(uint32_t)t * (V.cap + 1u)];
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < count - first; j += gridDim.x * blockDim.x) {
    const uint32_t p = V.items[j] & 0xffffffu;
    const int nl = (int)V.nLight[p];
    Pcg32 rng = LoadRng(B, p);
    VPath cam = CamPath(V, p), lig = LightPathOf(V, p);
    float4 L4 = B.L[p];
    V3 acc{L4.x, L4.y, L4.z};
    for (int s = 0; s <= nl && s <= 1; ++s) {
      ConnOut o;
      if (!ConnectBdpt(S, rng, lig, cam, s, t, o)) continue;
      if (!o.vis)
        acc = acc + o.c;
      else
        EmitConnection(S, V, nsh, err, p, o, true);
    }
    B.L[p] = make_float4(acc.x, acc.y, acc.z, 0.f);
    StoreRng(B, p, rng);
  }
}

// The s >= 2 connections of round t, item g (counted over the samples with
// at least t camera vertices): a binary search over the per-key item starts
// (samples of one key have the same light subpath length nl, hence nl - 1
// such connections) gives the sample and s.
RD void RoundItem(const BdptBuffers& V, uint32_t k0, uint32_t g, uint32_t& p, int& s) {
  const uint32_t c1 = V.cap + 1u, nk = c1 * c1;
  uint32_t lo = k0, hi = nk;  // the last key with itemStart <= g
  while (hi - lo > 1u) {
    uint32_t mid = (lo + hi) >> 1;
    if (V.itemStart[mid] <= g) lo = mid; else hi = mid;
  }
  const uint32_t nl = lo % c1, local = g - V.itemStart[lo];
  p = V.order[V.keyStart[lo] + local / (nl - 1u)];
  s = 2 + (int)(local % (nl - 1u));
}
RD uint32_t VClass(const DevScene& S, const BVert& v) { return v.type == BV_SURFACE ? S.shapeClass[v.id] : 0u; }
// Bucket of connection (p, s) of round t: the shade classes of its camera and light vertices.
RD uint32_t ItemBucket(const DevScene& S, const BdptBuffers& V, uint32_t p, int s, int t) {
  return VClass(S, CamPath(V, p)[t - 1]) * (uint32_t)kShadeClasses + VClass(S, LightPathOf(V, p)[s - 1]);
}

// Round t's work items counted per bucket (pass 0) or scattered into V.items
// bucket by bucket (pass 1), with warp-aggregated atomics. head: the samples
// with at least t camera vertices (their s <= 1 connections), bucketed by the
// camera vertex's shade class; else the s >= 2 connections, bucketed by both
// vertices' classes.
__global__ void __launch_bounds__(kBdptBlock) KBdptItemSort(DevScene S, BdptBuffers V, int t, int pass, int head,
                                                           uint32_t count) {
  const uint32_t c1 = V.cap + 1u, nk = c1 * c1;
  const uint32_t k0 = (uint32_t)t * c1;
  const uint32_t g0 = head ? V.keyStart[k0] : V.itemStart[k0];
  const uint32_t n = head ? count - g0 : V.itemStart[nk] - g0;
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t* cnt = V.bucket + (pass == 0 ? 0 : 2 * kBdptBuckets);
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    const uint32_t j = base + threadIdx.x;
    const bool ok = j < n;
    uint32_t p = 0, key = 0xffffffffu;
    int s = 0;
    if (ok && head) {
      p = V.order[g0 + j];
      key = VClass(S, CamPath(V, p)[t - 1]);
    } else if (ok) {
      RoundItem(V, k0, g0 + j, p, s);
      key = ItemBucket(S, V, p, s, t);
    }
    const uint32_t grp = __match_any_sync(0xffffffffu, key);
    const int leader = __ffs(grp) - 1;
    uint32_t slot = 0;
    if (ok && (int)lane == leader) slot = atomicAdd(cnt + key, (uint32_t)__popc(grp));
    slot = __shfl_sync(0xffffffffu, slot, leader);
    if (ok && pass == 1) V.items[slot + __popc(grp & ((1u << lane) - 1u))] = p | ((uint32_t)s << 24);
  }
}
// Bucket starts (exclusive scan of the counts, copied into the scatter cursors);
// zeroes the counts for the next round.
__global__ void KBdptItemScan(BdptBuffers V) {
  uint32_t acc = 0;
  for (int b = 0; b < kBdptBuckets; b++) {
    uint32_t c = V.bucket[b];
    V.bucket[kBdptBuckets + b] = acc;
    V.bucket[2 * kBdptBuckets + b] = acc;
    V.bucket[b] = 0;
    acc += c;
  }
  V.bucket[3 * kBdptBuckets] = acc;
}

// Round t's s >= 2 connections, one per thread in bucket order (t >= 2: no
// random numbers; t = 1: each starts from the sample's stream advanced past the
// draws of the connections before it).
__global__ void __launch_bounds__(kBdptBlock) KBdptConnectTail(DevScene S, PathBuffers B, BdptBuffers V, int t) {
  uint32_t* nsh = B.counters + kShadowBase + (t - 1);
  uint32_t* err = B.counters + kMiscBase + 1;
  const uint32_t c1 = V.cap + 1u, nk = c1 * c1;
  const uint32_t n = V.itemStart[nk] - V.itemStart[(uint32_t)t * c1];
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const uint32_t it = V.items[j];
    const uint32_t p = it & 0xffffffu;
    const int s = (int)(it >> 24);
    VPath lig = LightPathOf(V, p);
    Pcg32 rng;
    rng.state = 0;  // rounds t >= 2: these connections draw no random numbers
    if (t == 1) {
      uint2 st = V.rng1[p];
      rng.state = (uint64_t)st.x | ((uint64_t)st.y << 32);
      PcgAdvance(rng, Round1Draws(S, lig, s));
    }
    ConnOut o;
    if (ConnectBdpt(S, rng, lig, CamPath(V, p), s, t, o)) EmitConnection(S, V, nsh, err, p, o, true);
  }
}

// Round t = 1, per sample: keep the stream's state for the connections and
// advance the sample's stream past all of them.
__global__ void __launch_bounds__(kBdptBlock) KBdptRound1Head(DevScene S, PathBuffers B, BdptBuffers V, uint32_t count) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < count; p += gridDim.x * blockDim.x) {
    const int nl = (int)V.nLight[p];
    uint2 st = B.rng[p];
    V.rng1[p] = st;
    Pcg32 rng = LoadRng(B, p);
    PcgAdvance(rng, Round1Draws(S, LightPathOf(V, p), nl + 1));
    StoreRng(B, p, rng);
  }
}

// Persistent any-hit traversal of round t's visibility rays (the warp-refill
// scheme of KShadow).
__global__ void __launch_bounds__(kBdptBlock, 8)
    KBdptShadow(DevScene S, PathBuffers B, BdptBuffers V, int t, float4* film, int refillBusy, int leafFrac8) {
  const uint32_t count = min(B.counters[kShadowBase + (t - 1)], V.shCap);
  if (blockIdx.x * blockDim.x >= count) return;  // blocks past one thread per ray leave at once
  uint32_t* fetch = B.counters + kFetchBase + 2 * (t - 1) + 1;
  uint32_t* err = B.counters + kMiscBase + 1;
  const uint32_t lane = threadIdx.x & 31u;
  bool live = false, done = false, drained = false, occ = false;
  uint32_t i = 0;
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
          float4 o = V.shO[i], d = V.shD[i];
          r = MakeRayPre(V3{o.x, o.y, o.z}, V3{d.x, d.y, d.z}, 0.f);
          TraceInit(o.w, h, st);
          live = true;
          done = S.nNodes == 0;
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
        int res = TravStep<true, false>(S, r, h, stack, st, err, nullptr, nullptr);
        if (res != kTravContinue) {
          done = true;
          occ = res == kTravDone && h.prim != kNoPrim;
        }
      }
    }
    if (live && done) {
      if (!occ) {
        uint32_t tag = __float_as_uint(V.shD[i].w);
        float4 c = V.shC[i];
        float4* dst = (tag & 0x80000000u) ? (film ? film + (tag & 0x7fffffffu) : nullptr) : B.L + tag;
        if (dst) {
          atomicAdd(&dst->x, c.x);
          atomicAdd(&dst->y, c.y);
          atomicAdd(&dst->z, c.z);
        }
      }
      live = false;
    }
  }
}

// sample_renderer.cpp:101-105 (bdpt.cpp:283-287): NaN in any channel, Inf /
// negative in the first drop the sample, which still counts in 1 / spp.
__global__ void __launch_bounds__(256) KBdptAccumulate(PathBuffers B, FilmView film, uint32_t count, float* out) {
  uint32_t nbad = 0;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) {
    float4 l = B.L[i];
    if (out) {
      out[3 * (size_t)i] = l.x;
      out[3 * (size_t)i + 1] = l.y;
      out[3 * (size_t)i + 2] = l.z;
    }
    if (film.accum) {
      bool bad = isnan(l.x) || isnan(l.y) || isnan(l.z) || isinf(l.x) || l.x < 0.f;
      if (bad) {
        nbad = 1;
      } else if (l.x != 0.f || l.y != 0.f || l.z != 0.f) {
        float4* a = film.accum + B.pixel[i];
        atomicAdd(&a->x, l.x);
        atomicAdd(&a->y, l.y);
        atomicAdd(&a->z, l.z);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) nbad += __shfl_down_sync(0xffffffffu, nbad, o);
  if (film.stats) {
    if (nbad && (threadIdx.x & 31u) == 0) atomicAdd(film.stats + 2, (unsigned long long)nbad);
    if (i == 0) atomicAdd(film.stats + 3, (unsigned long long)count);
  }
}

static int GridFor(uint32_t n, int maxGrid) {
  return std::max(1, std::min(maxGrid, (int)((n + kBdptBlock - 1) / kBdptBlock)));
}

cudaError_t LaunchBdptCamera(const DevScene& S, const PathBuffers& B, const BdptBuffers& V, const WaveParams& w,
                             cudaStream_t st) {
  if (w.count == 0) return cudaSuccess;
  KBdptCamera<<<GridFor(w.count, 1 << 16), kBdptBlock, 0, st>>>(S, B, V, w);
  return cudaGetLastError();
}
cudaError_t LaunchBdptLight(const DevScene& S, const PathBuffers& B, const BdptBuffers& V, uint32_t count,
                            cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  KBdptLight<<<GridFor(count, 1 << 16), kBdptBlock, 0, st>>>(S, B, V, count);
  return cudaGetLastError();
}
cudaError_t LaunchBdptWalk(const DevScene& S, const PathBuffers& B, const BdptBuffers& V, int depth, bool light,
                           int grid, cudaStream_t st) {
  if (light)
    KBdptWalk<true><<<grid, kBdptBlock, 0, st>>>(S, B, V, depth);
  else
    KBdptWalk<false><<<grid, kBdptBlock, 0, st>>>(S, B, V, depth);
  return cudaGetLastError();
}
cudaError_t LaunchBdptLightFix(const DevScene& S, const BdptBuffers& V, uint32_t count, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  KBdptLightFix<<<GridFor(count, 1 << 16), kBdptBlock, 0, st>>>(S, V, count);
  KBdptKeyScan<<<1, 1, 0, st>>>(V);
  KBdptKeyScatter<<<GridFor(count, 1 << 16), kBdptBlock, 0, st>>>(V, count);
  return cudaGetLastError();
}
// The s >= 2 connections of round t: sorted into buckets, then one per thread.
static void LaunchSort(const DevScene& S, const BdptBuffers& V, int t, bool head, uint32_t count, int grid,
                       cudaStream_t st) {
  KBdptItemSort<<<grid, kBdptBlock, 0, st>>>(S, V, t, 0, head ? 1 : 0, count);
  KBdptItemScan<<<1, 1, 0, st>>>(V);
  KBdptItemSort<<<grid, kBdptBlock, 0, st>>>(S, V, t, 1, head ? 1 : 0, count);
}
static void LaunchTail(const DevScene& S, const PathBuffers& B, const BdptBuffers& V, int t, int grid,
                       cudaStream_t st) {
  LaunchSort(S, V, t, false, 0, grid, st);
  KBdptConnectTail<<<grid, kBdptBlock, 0, st>>>(S, B, V, t);
}
cudaError_t LaunchBdptConnectSplit(const DevScene& S, const PathBuffers& B, const BdptBuffers& V, uint32_t count,
                                   int t, int grid, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  LaunchSort(S, V, t, true, count, grid, st);
  KBdptConnectHead<<<GridFor(count, grid), kBdptBlock, 0, st>>>(S, B, V, count, t);
  LaunchTail(S, B, V, t, grid, st);
  return cudaGetLastError();
}
cudaError_t LaunchBdptRound1(const DevScene& S, const PathBuffers& B, const BdptBuffers& V, uint32_t count,
                             bool splats, int grid, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  KBdptRound1Head<<<GridFor(count, grid), kBdptBlock, 0, st>>>(S, B, V, count);
  if (splats) LaunchTail(S, B, V, 1, grid, st);
  return cudaGetLastError();
}
cudaError_t LaunchBdptShadow(const DevScene& S, const PathBuffers& B, const BdptBuffers& V, int t, float4* film,
                             int grid, cudaStream_t st, int refillBusy, int leafFrac8) {
  KBdptShadow<<<grid, kBdptBlock, 0, st>>>(S, B, V, t, film, refillBusy, leafFrac8);
  return cudaGetLastError();
}
cudaError_t LaunchBdptAccumulate(const PathBuffers& B, const FilmView& film, uint32_t count, float* out,
                                 cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  KBdptAccumulate<<<(count + 255) / 256, 256, 0, st>>>(B, film, count, out);
  return cudaGetLastError();
}

}  // namespace rad
