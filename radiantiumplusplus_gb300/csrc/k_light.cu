// Renderer "particle_tracer" (dlight.cuh) as a wavefront: the light paths'
// starts, then per bounce the BVH8 closest-hit kernel and KParticleBounce; the
// camera connections of each round go through the any-hit kernel of bdpt
// (KBdptShadow), which splats the unoccluded ones into the job's film with
// float atomics (the film resolves with scale 1).
#include "dlight.cuh"
#include "kernels.h"

namespace rad {

// Warp-aggregated append of p to queue q (all lanes of the warp call it).
__device__ __forceinline__ void ParticleEnqueue(uint32_t* q, uint32_t* cnt, uint32_t p, bool push) {
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t m = __ballot_sync(0xffffffffu, push);
  if (!m) return;
  int leader = __ffs(m) - 1;
  uint32_t base = 0;
  if ((int)lane == leader) base = atomicAdd(cnt, (uint32_t)__popc(m));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (push) q[base + __popc(m & ((1u << lane) - 1u))] = p;
}

// Light paths [pp.first, pp.first + count) of the wave, one per slot: the
// emitter's camera connection into visibility round 0, the emitted ray into
// queue 0.
__global__ void __launch_bounds__(128) KParticleStart(DevScene S, PathBuffers B, ParticleParams pp, unsigned long long* stats) {
  uint32_t* nsh = B.counters + kShadowBase;
  if (stats && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(stats + 3, (unsigned long long)pp.count);
  for (uint32_t base = blockIdx.x * blockDim.x; base < pp.count; base += gridDim.x * blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    bool push = false;
    if (i < pp.count) {
      Pcg32 rng;
      CamSplat em;
      bool hasEm;
      V3 O, D, thr;
      push = ParticleStart(S, pp.first + i, pp.seed, pp.sampleScale, rng, em, hasEm, O, D, thr);
      if (hasEm) {
        uint32_t slot = atomicAdd(nsh, 1u);
        B.shO[slot] = make_float4(em.o.x, em.o.y, em.o.z, em.tmax);
        B.shD[slot] = make_float4(em.d.x, em.d.y, em.d.z, __uint_as_float(0x80000000u | em.pixel));
        B.shC[slot] = make_float4(em.c.x, em.c.y, em.c.z, 0.f);
      }
      if (push) {
        B.rayO[i] = make_float4(O.x, O.y, O.z, 0.f);
        B.rayD[i] = make_float4(D.x, D.y, D.z, kFloatMax);
        B.thr[i] = make_float4(thr.x, thr.y, thr.z, 1.f);
        B.rng[i] = make_uint2((uint32_t)rng.state, (uint32_t)(rng.state >> 32));
      }
    }
    ParticleEnqueue(B.q[0], B.counters, i, push);
  }
}

// Bounce d of the queued light paths (after the closest-hit kernel, taken class
// by class from its shade-class queues): camera connection into visibility
// round d + 1, next ray into the next queue.
__global__ void __launch_bounds__(128) KParticleBounce(DevScene S, PathBuffers B, int d, float sampleScale) {
  uint32_t start[kShadeClasses + 1];
  ClassQueueStarts(B, d, start);
  const uint32_t count = start[kShadeClasses];
  uint32_t* nsh = B.counters + kShadowBase + d + 1;
  for (uint32_t base = blockIdx.x * blockDim.x; base < count; base += gridDim.x * blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    bool push = false;
    uint32_t p = 0;
    if (i < count) {
      p = ClassQueueEntry(B, start, i);
      uint2 rs = B.rng[p];
      Pcg32 rng;
      rng.state = (uint64_t)rs.x | ((uint64_t)rs.y << 32);
      float4 o4 = B.rayO[p], d4 = B.rayD[p], t4 = B.thr[p];
      V3 O{o4.x, o4.y, o4.z}, D{d4.x, d4.y, d4.z}, thr{t4.x, t4.y, t4.z};
      float eta = t4.w;
      HitRec hr = B.hit[p];
      TraceHit h{hr.t, hr.u, hr.v, hr.prim, hr.shape, hr.front};
      CamSplat cs;
      bool hasCs;
      push = ParticleBounce(S, rng, d, hr.prim != kNoPrim, h, O, D, thr, eta, sampleScale, cs, hasCs);
      if (hasCs) {
        uint32_t slot = atomicAdd(nsh, 1u);
        B.shO[slot] = make_float4(cs.o.x, cs.o.y, cs.o.z, cs.tmax);
        B.shD[slot] = make_float4(cs.d.x, cs.d.y, cs.d.z, __uint_as_float(0x80000000u | cs.pixel));
        B.shC[slot] = make_float4(cs.c.x, cs.c.y, cs.c.z, 0.f);
      }
      if (push) {
        B.rayO[p] = make_float4(O.x, O.y, O.z, 0.f);
        B.rayD[p] = make_float4(D.x, D.y, D.z, kFloatMax);
        B.thr[p] = make_float4(thr.x, thr.y, thr.z, eta);
        B.rng[p] = make_uint2((uint32_t)rng.state, (uint32_t)(rng.state >> 32));
      }
    }
    ParticleEnqueue(B.q[(d + 1) & 1], B.counters + d + 1, p, push);
  }
}

cudaError_t LaunchParticleStart(const DevScene& S, const PathBuffers& B, const ParticleParams& pp,
                                unsigned long long* stats, cudaStream_t st) {
  if (pp.count == 0) return cudaSuccess;
  uint32_t blocks = (pp.count + 127) / 128;
  KParticleStart<<<blocks < 65536u ? blocks : 65536u, 128, 0, st>>>(S, B, pp, stats);
  return cudaGetLastError();
}
cudaError_t LaunchParticleBounce(const DevScene& S, const PathBuffers& B, int d, float sampleScale, int grid,
                                 cudaStream_t st) {
  KParticleBounce<<<grid, 128, 0, st>>>(S, B, d, sampleScale);
  return cudaGetLastError();
}

}  // namespace rad
