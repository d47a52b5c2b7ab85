// Renderer "particle_tracer" (dlight.cuh): one thread follows one light path;
// splats are atomic adds into the job's float4 film, whose resolve then uses
// scale 1.
#include "dlight.cuh"
#include "kernels.h"

namespace rad {

__global__ void __launch_bounds__(128) KParticle(DevScene S, FilmView film, ParticleParams pp, uint32_t* err) {
  ParticleFilm pf{film.accum, film.width, film.height};
  if (film.stats && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(film.stats + 3, (unsigned long long)pp.count);
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

}  // namespace rad
