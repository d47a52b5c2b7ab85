// Renderers that splat into the film: "particle_tracer" (dlight.cuh), one
// thread per light path, film resolved with scale 1; and "bdpt" (dbdpt.cuh),
// one thread per pixel sample, its camera-side radiance and its t = 1 splats
// added into the film, resolved with 1 / spp. Splats are atomic adds.
#include "dbdpt.cuh"
#include "kernels.h"

namespace rad {

__global__ void __launch_bounds__(128) KParticle(DevScene S, FilmView film, ParticleParams pp, uint32_t* err) {
  ParticleFilm pf{film.accum, film.width, film.height};
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < pp.count;
       i += (uint64_t)gridDim.x * blockDim.x)
    ParticlePath(S, pf, pp.first + i, pp.seed, pp.sampleScale, err);
}

cudaError_t LaunchParticle(const DevScene& S, const FilmView& film, const ParticleParams& pp, uint32_t* err, int grid,
                           cudaStream_t st) {
  if (pp.count == 0) return cudaSuccess;
  KParticle<<<grid, 128, 0, st>>>(S, film, pp, err);
  return cudaGetLastError();
}

// Pixel samples of a wave (the path-index mapping of the generate stage). With
// `out`, each sample's camera-side radiance is written there; with a film, the
// valid ones (sample_renderer.cpp:101-105 test) and every t = 1 splat are added.
__global__ void __launch_bounds__(128) KBdpt(DevScene S, FilmView film, WaveParams w, float* out, uint32_t* err) {
  const uint32_t spw = w.spw > 1u ? w.spw : 1u;
  const uint32_t npc = w.count / spw;
  ParticleFilm pf{film.accum, film.width, film.height};
  uint32_t nbad = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < w.count; i += gridDim.x * blockDim.x) {
    const uint32_t j = spw > 1u ? i % npc : i, s = spw > 1u ? i / npc : 0u;
    uint32_t pix = w.pixelList ? w.pixelList[i] : w.pixelBegin + j;
    uint32_t smp = w.sampleList ? w.sampleList[i] : w.sample + s;
    V3 l = BdptSample(S, film.accum ? &pf : nullptr, pix, smp, w.seed, err);
    if (out) {
      out[3 * (size_t)i] = l.x;
      out[3 * (size_t)i + 1] = l.y;
      out[3 * (size_t)i + 2] = l.z;
    }
    if (film.accum) {
      bool bad = isnan(l.x) || isnan(l.y) || isnan(l.z) || isinf(l.x) || l.x < 0.f;
      if (bad) {
        nbad++;
      } else if (!IsBlack(l)) {
        float4* a = film.accum + pix;
        atomicAdd(&a->x, l.x);
        atomicAdd(&a->y, l.y);
        atomicAdd(&a->z, l.z);
      }
    }
  }
  if (film.stats) {
    if (nbad) atomicAdd(film.stats + 2, (unsigned long long)nbad);
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(film.stats + 3, (unsigned long long)w.count);
  }
}

cudaError_t LaunchBdpt(const DevScene& S, const FilmView& film, const WaveParams& w, float* out, uint32_t* err,
                       int grid, cudaStream_t st) {
  if (w.count == 0) return cudaSuccess;
  KBdpt<<<grid, 128, 0, st>>>(S, film, w, out, err);
  return cudaGetLastError();
}

}  // namespace rad
