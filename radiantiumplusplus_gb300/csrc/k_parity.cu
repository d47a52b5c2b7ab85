// Batch kernels behind the parity entry points: BSDF eval/pdf/sample on
// (wi, wo, params) batches (Bsdf::Eval/Pdf/Sample, bsdf.h:103-142), closest /
// any hit on ray batches (Accel, accel.h:10-30) and camera rays
// (Perspective::SampleRay, perspective.cpp:73-82). One thread per record.
#include "dbsdf.cuh"
#include "dscene.cuh"
#include "kernels.h"

namespace rad {

__global__ void KBsdfEval(const MatRec* mats, const float* wi, const float* wo, int64_t n, float* f, float* pdf) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  V3 a = ld3(wi + 3 * i), o = ld3(wo + 3 * i);
  V3 v;
  float p;
  BsdfEvalPdf(mats, 0, a, o, v, p);
  f[3 * i] = v.x;
  f[3 * i + 1] = v.y;
  f[3 * i + 2] = v.z;
  pdf[i] = p;
}

__global__ void KBsdfSample(const MatRec* mats, const float* wi, const float* u, int64_t n, float* wo, float* pdf,
                            float* f, float* eta, uint32_t* type) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  V3 a = ld3(wi + 3 * i);
  BsdfSampleRes r = BsdfSample(mats, 0, a, u[3 * i], V2{u[3 * i + 1], u[3 * i + 2]});
  wo[3 * i] = r.wo.x;
  wo[3 * i + 1] = r.wo.y;
  wo[3 * i + 2] = r.wo.z;
  pdf[i] = r.pdf;
  f[3 * i] = r.f.x;
  f[3 * i + 1] = r.f.y;
  f[3 * i + 2] = r.f.z;
  eta[i] = r.eta;
  type[i] = r.type;
}

__global__ void __launch_bounds__(128) KTrace(DevScene S, const float* rays, int64_t n, float* hits, int anyHit,
                                              uint32_t* err) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4* r4 = reinterpret_cast<const float4*>(rays) + 2 * i;
  float4 o = r4[0], d = r4[1];
  RayPre r = MakeRayPre(V3{o.x, o.y, o.z}, V3{d.x, d.y, d.z}, o.w);
  TraceHit h;
  float* out = hits + 5 * i;
  if (anyHit) {
    bool occ = TraceBvh8<true>(S, r, d.w, h, err);
    out[0] = 0.f;
    out[1] = 0.f;
    out[2] = 0.f;
    out[3] = __uint_as_float(occ ? 1u : 0u);
    out[4] = __uint_as_float(0u);
  } else {
    bool hit = TraceBvh8<false>(S, r, d.w, h, err);
    out[0] = hit ? h.t : kInf;
    out[1] = hit ? h.u : 0.f;
    out[2] = hit ? h.v : 0.f;
    out[3] = __uint_as_float(hit ? h.prim : kNoPrim);
    out[4] = __uint_as_float(hit ? h.front : 0u);
  }
}

__global__ void KCamera(DevScene S, const uint32_t* pix, int64_t n, uint32_t sample, uint32_t seed, float* out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t p = pix[i];
  uint32_t x = p % (uint32_t)S.cam.width, y = p / (uint32_t)S.cam.width;
  Pcg32 rng = PcgForSample(p, sample, seed);
  float jx = Next1D(rng);
  float jy = Next1D(rng);
  V3 O, D;
  float tmin, tmax;
  CameraRay(S.cam, (float)x + jx, (float)y + jy, O, D, tmin, tmax);
  float* o = out + 8 * i;
  o[0] = O.x;
  o[1] = O.y;
  o[2] = O.z;
  o[3] = tmin;
  o[4] = D.x;
  o[5] = D.y;
  o[6] = D.z;
  o[7] = tmax;
}

// Texture<T>::Eval at given uv and uv derivatives (texture.h:57-62).
__global__ void KTexEval(DevScene S, uint32_t tex, const float* uv, const float* duv, int64_t n, float* out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  TexCtx x{S.tex, S.texels, S.texBind, V2{uv[2 * i], uv[2 * i + 1]}, V2{duv[4 * i], duv[4 * i + 1]},
           V2{duv[4 * i + 2], duv[4 * i + 3]}};
  TexVal v = TexEval(x, tex, x.uv);
  out[3 * i] = v.c[0];
  out[3 * i + 1] = v.c[1];
  out[3 * i + 2] = v.c[2];
}

static unsigned Blocks(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

cudaError_t LaunchTexEval(const DevScene& S, uint32_t tex, const float* uv, const float* duv, int64_t n, float* out,
                          cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  KTexEval<<<Blocks(n, 128), 128, 0, st>>>(S, tex, uv, duv, n, out);
  return cudaGetLastError();
}

cudaError_t LaunchBsdfEval(const MatRec* mats, const float* wi, const float* wo, int64_t n, float* f, float* pdf,
                           cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  KBsdfEval<<<Blocks(n, 128), 128, 0, st>>>(mats, wi, wo, n, f, pdf);
  return cudaGetLastError();
}
cudaError_t LaunchBsdfSample(const MatRec* mats, const float* wi, const float* u, int64_t n, float* wo, float* pdf,
                             float* f, float* eta, uint32_t* type, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  KBsdfSample<<<Blocks(n, 128), 128, 0, st>>>(mats, wi, u, n, wo, pdf, f, eta, type);
  return cudaGetLastError();
}
cudaError_t LaunchTrace(const DevScene& S, const float* rays, int64_t n, float* hits, int anyHit, uint32_t* err,
                        cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  KTrace<<<Blocks(n, 128), 128, 0, st>>>(S, rays, n, hits, anyHit, err);
  return cudaGetLastError();
}
cudaError_t LaunchCameraRays(const DevScene& S, const uint32_t* pix, int64_t n, uint32_t sample, uint32_t seed,
                             float* out, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  KCamera<<<Blocks(n, 128), 128, 0, st>>>(S, pix, n, sample, seed, out);
  return cudaGetLastError();
}

}  // namespace rad
