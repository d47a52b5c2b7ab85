// Guide network kernels (see dguide.cuh for the method):
//   KGuideInferTc  -- per bounce: hash-grid encode + MLP for every hit of a
//                     guided shade class, mixture parameters per path slot
//   KGuideQueryTc  -- the same network on caller-given queries (parity hook)
//   KGuideFinalize -- training weight of each recorded vertex from the path's
//                     final radiance
//   KGuideTrain    -- forward + backward of the loss over a batch of records:
//                     MLP weight gradients and hash-table gradients
//   KGuideAdam     -- Adam step, refreshes the fp16 copies
// Inference runs the MLP on the fifth-generation tensor cores (tcgen05: M = 128
// tiles, operands in shared memory, fp32 accumulator in TMEM; dtc.cuh).
// Training runs on them too: 128-record tiles, the forward as in inference,
// then per layer dIn = G W (M = 128 records) and dW = G^T In (M = the layer's
// outputs padded to 128, K = records) with dW accumulated in TMEM over the
// CTA's tiles.
#include <algorithm>

#include "dguide.cuh"
#include "dscene.cuh"
#include "dtc.cuh"
#include "kernels.h"

namespace rad {

namespace {

__device__ __forceinline__ uint32_t Pack2(__half lo, __half hi) {
  return (uint32_t)__half_as_ushort(lo) | ((uint32_t)__half_as_ushort(hi) << 16);
}
__device__ __forceinline__ uint32_t PackF2(float lo, float hi) {
  return Pack2(__float2half_rn(lo), __float2half_rn(hi));
}

__device__ __forceinline__ void GuidePosToUnit(const GuideDev& G, V3 P, float u[3]) {
  u[0] = clampr((P.x - G.lo[0]) * G.inv[0], 0.f, 1.f);
  u[1] = clampr((P.y - G.lo[1]) * G.inv[1], 0.f, 1.f);
  u[2] = clampr((P.z - G.lo[2]) * G.inv[2], 0.f, 1.f);
}

// Hash-grid features of levels [l0, l1) into row[2l], row[2l + 1] (fp16).
__device__ __forceinline__ void GuideEncodeLevels(const GuideDev& G, const float u[3], int l0, int l1, __half* row) {
  for (int l = l0; l < l1; l++) {
    uint32_t res = G.res[l];
    uint32_t cx, cy, cz;
    float tx, ty, tz;
    GuideCell(u[0], res, cx, tx);
    GuideCell(u[1], res, cy, ty);
    GuideCell(u[2], res, cz, tz);
    const __half2* tab = reinterpret_cast<const __half2*>(G.table) + ((size_t)l << G.log2T);
    float f0 = 0.f, f1 = 0.f;
#pragma unroll
    for (int c = 0; c < 8; c++) {
      uint32_t bx = c & 1u, by = (c >> 1) & 1u, bz = (c >> 2) & 1u;
      float w = (bx ? tx : 1.f - tx) * (by ? ty : 1.f - ty) * (bz ? tz : 1.f - tz);
      uint32_t idx = GuideGridIndex(cx + bx, cy + by, cz + bz, res, G.log2T);
      float2 v = __half22float2(tab[idx]);
      f0 += w * v.x;
      f1 += w * v.y;
    }
    *reinterpret_cast<uint32_t*>(row + 2 * l) = PackF2(f0, f1);
  }
}

__device__ __forceinline__ void GuideEncodeTail(V3 N, V3 wo, __half* row) {
  *reinterpret_cast<uint32_t*>(row + 32) = PackF2(N.x, N.y);
  *reinterpret_cast<uint32_t*>(row + 34) = PackF2(N.z, wo.x);
  *reinterpret_cast<uint32_t*>(row + 36) = PackF2(wo.y, wo.z);
  *reinterpret_cast<uint32_t*>(row + 38) = PackF2(1.f, 0.f);
  for (int k = 40; k < kGIn; k += 2) *reinterpret_cast<uint32_t*>(row + k) = 0u;
}

__device__ __forceinline__ void StoreMix(const float* o, const GuideDev& G, float4* mx) {
  GuideMix m;
  GuideMixFromRaw(o, G.logKMax, G.cMax, m);
  for (int k = 0; k < kGLobes; k++) mx[k] = make_float4(m.mu[k].x, m.mu[k].y, m.mu[k].z, m.kappa[k]);
  mx[8] = make_float4(m.pi[0], m.pi[1], m.pi[2], m.pi[3]);
  mx[9] = make_float4(m.pi[4], m.pi[5], m.pi[6], m.pi[7]);
  mx[10] = make_float4(m.c, 0.f, 0.f, 0.f);
}

// ---- the MLP on the fifth-generation tensor cores (tcgen05, accumulator in TMEM)
// One tile = 128 queries (a CTA of 4 warps, one query per thread): every layer
// is one M = 128 MMA chain over K in steps of 16, issued by one thread, with
// the activations and the four weight matrices in shared memory in the K-major
// core-matrix layout (dtc.cuh) and the fp32 accumulator in 64 TMEM columns. The
// epilogue (ReLU, fp16) reads each thread's row back with tcgen05.ld and writes
// the next layer's operand. Every wait is bounded: on a timeout the kernel sets
// kErrGuideTc, waits (bounded) for its outstanding MMA, frees its TMEM and ends.
constexpr int kTcRows = 128;
constexpr uint32_t kTcW0 = 0;                                // 64 x 48
constexpr uint32_t kTcW1 = kTcW0 + kGHid * kGIn * 2;         // 64 x 64
constexpr uint32_t kTcW2 = kTcW1 + kGHid * kGHid * 2;        // 64 x 64
constexpr uint32_t kTcW3 = kTcW2 + kGHid * kGHid * 2;        // 48 x 64
constexpr uint32_t kTcAct = kTcW3 + kGOut * kGHid * 2;       // 128 x 64 activations
constexpr uint32_t kTcMisc = kTcAct + kTcRows * kGHid * 2;   // mbarrier, TMEM address
constexpr int kTcSmem = (int)kTcMisc + 16;
constexpr uint32_t kTcCols = 64;                             // TMEM columns (fp32 accumulator, N <= 64)
constexpr uint32_t kTcWaitLimit = 1u << 22;
static_assert(kTcW1 % 16 == 0 && kTcW2 % 16 == 0 && kTcW3 % 16 == 0 && kTcAct % 16 == 0 && kTcMisc % 16 == 0,
              "descriptor addresses are 16-byte aligned");

__device__ __forceinline__ void TcLoadWeights(const __half* gw, unsigned char* sm) {
  for (int i = threadIdx.x; i < kGHid * kGIn; i += blockDim.x) {
    int n = i / kGIn, k = i % kGIn;
    *reinterpret_cast<__half*>(sm + kTcW0 + TcOffset(n, k, kGIn)) = gw[kGW0 + i];
  }
  for (int i = threadIdx.x; i < kGHid * kGHid; i += blockDim.x) {
    int n = i / kGHid, k = i % kGHid;
    *reinterpret_cast<__half*>(sm + kTcW1 + TcOffset(n, k, kGHid)) = gw[kGW1 + i];
    *reinterpret_cast<__half*>(sm + kTcW2 + TcOffset(n, k, kGHid)) = gw[kGW2 + i];
  }
  for (int i = threadIdx.x; i < kGOut * kGHid; i += blockDim.x) {
    int n = i / kGHid, k = i % kGHid;
    *reinterpret_cast<__half*>(sm + kTcW3 + TcOffset(n, k, kGHid)) = gw[kGW3 + i];
  }
}

// The 48 network inputs of one query (32 grid features, N, wo, 1, zeros) as 24 fp16 pairs.
__device__ __forceinline__ void TcEncodeRow(const GuideDev& G, V3 P, V3 N, V3 wo, uint32_t (&v)[24]) {
  __half row[kGIn];
  float u[3];
  GuidePosToUnit(G, P, u);
  GuideEncodeLevels(G, u, 0, kGLevels, row);
  GuideEncodeTail(N, wo, row);
#pragma unroll
  for (int i = 0; i < 24; i++) v[i] = *reinterpret_cast<const uint32_t*>(row + 2 * i);
}

// Writes this thread's 48-input row into the layer-0 operand (K = 48).
__device__ __forceinline__ void TcStoreInputs(unsigned char* sm, uint32_t r, const uint32_t (&v)[24]) {
#pragma unroll
  for (int c = 0; c < kGIn / 8; c++)
    *reinterpret_cast<uint4*>(sm + kTcAct + TcOffset(r, 8 * c, kGIn)) =
        make_uint4(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]);
}

// One layer: D = act x W^T into TMEM (thread 0 issues), then every thread waits.
// Returns false if the wait gave up (the caller stops).
__device__ __forceinline__ bool TcLayer(unsigned char* sm, uint32_t tmem, uint64_t* mbar, uint32_t& phase,
                                        uint32_t wOff, int K, int N, int* fail) {
  if (threadIdx.x == 0) {
    TcFenceAfter();
    const uint32_t a0 = SmemAddr(sm + kTcAct), b0 = SmemAddr(sm + wOff);
    const uint32_t idesc = TcIdescF16(kTcRows, (uint32_t)N);
    for (int s = 0; s < K / 16; s++)
      TcMma(tmem, TcSmemDesc(a0 + 256u * s, 128u, 16u * K), TcSmemDesc(b0 + 256u * s, 128u, 16u * K), idesc, s > 0);
    TcCommit(mbar);
  }
  const bool ok = MbarWait(mbar, phase, kTcWaitLimit);
  if (!ok) atomicOr(fail, 1);
  __syncthreads();
  if (*fail) return false;
  phase ^= 1u;
  TcFenceAfter();
  return true;
}

// ReLU of this thread's 64 accumulator columns, as the next layer's fp16 operand (K = 64).
__device__ __forceinline__ void TcReluToAct(unsigned char* sm, uint32_t tmemRow, uint32_t r) {
#pragma unroll
  for (int c0 = 0; c0 < kGHid; c0 += 16) {
    float v[16];
    TcLoad16(tmemRow + c0, v);
#pragma unroll
    for (int q = 0; q < 2; q++) {
      uint4 w;
      w.x = PackF2(fmaxf(v[8 * q + 0], 0.f), fmaxf(v[8 * q + 1], 0.f));
      w.y = PackF2(fmaxf(v[8 * q + 2], 0.f), fmaxf(v[8 * q + 3], 0.f));
      w.z = PackF2(fmaxf(v[8 * q + 4], 0.f), fmaxf(v[8 * q + 5], 0.f));
      w.w = PackF2(fmaxf(v[8 * q + 6], 0.f), fmaxf(v[8 * q + 7], 0.f));
      *reinterpret_cast<uint4*>(sm + kTcAct + TcOffset(r, c0 + 8 * q, kGHid)) = w;
    }
  }
}

// The four layers of the tile; o receives this thread's 48 outputs. Returns false on a wait timeout.
__device__ __forceinline__ bool TcMlpTile(unsigned char* sm, uint32_t tmem, uint64_t* mbar, uint32_t& phase,
                                          int* fail, float (&o)[kGOut]) {
  const uint32_t r = threadIdx.x;
  const uint32_t tmemRow = tmem + ((32u * (threadIdx.x >> 5)) << 16);
  FenceProxyAsync();
  TcFenceBefore();
  __syncthreads();
  const uint32_t wOff[3] = {kTcW0, kTcW1, kTcW2};
  for (int l = 0; l < 3; l++) {
    if (!TcLayer(sm, tmem, mbar, phase, wOff[l], l == 0 ? kGIn : kGHid, kGHid, fail)) return false;
    TcReluToAct(sm, tmemRow, r);
    FenceProxyAsync();
    TcFenceBefore();
    __syncthreads();
  }
  if (!TcLayer(sm, tmem, mbar, phase, kTcW3, kGHid, kGOut, fail)) return false;
#pragma unroll
  for (int c0 = 0; c0 < kGOut; c0 += 16) {
    float v[16];
    TcLoad16(tmemRow + c0, v);
#pragma unroll
    for (int i = 0; i < 16; i++) o[c0 + i] = v[i];
  }
  TcFenceBefore();
  __syncthreads();  // every TMEM read done before the next tile's MMA
  return true;
}

// Set-up shared by the tcgen05 kernels: weights, mbarrier, TMEM columns.
__device__ __forceinline__ uint32_t TcSetup(const GuideDev& G, unsigned char* sm, uint64_t*& mbar, int*& fail) {
  mbar = reinterpret_cast<uint64_t*>(sm + kTcMisc);
  uint32_t* slot = reinterpret_cast<uint32_t*>(sm + kTcMisc + 8);
  fail = reinterpret_cast<int*>(sm + kTcMisc + 12);
  if (threadIdx.x == 0) {
    MbarInit(mbar, 1);
    *fail = 0;
  }
  if (threadIdx.x < 32) TcAlloc(slot, kTcCols);
  TcLoadWeights(G.weights, sm);
  FenceProxyAsync();
  TcFenceBefore();
  __syncthreads();
  TcFenceAfter();
  return *slot;
}

// After the tile loop: on a timeout, one more bounded wait for the MMA still
// outstanding; then the TMEM columns are freed.
__device__ __forceinline__ void TcTeardown(uint32_t tmem, uint64_t* mbar, uint32_t phase, int* fail, uint32_t* err) {
  if (*fail) {
    MbarWait(mbar, phase, kTcWaitLimit);
    if (threadIdx.x == 0) atomicOr(err, kErrGuideTc);
  }
  TcFenceBefore();
  __syncthreads();
  TcFenceAfter();
  if (threadIdx.x < 32) TcDealloc(tmem, kTcCols);
}

}  // namespace

// Per bounce, the guide network for every hit of a guided shade class (all
// but emitters and rough_glass: near-delta transmission gains little from a
// smooth directional guide): 128 queries per tile, one per thread, the MLP on
// tcgen05.
__global__ void __launch_bounds__(kTcRows, 1)
    KGuideInferTc(DevScene S, PathBuffers B, GuideDev G, int depth) {
  extern __shared__ __align__(1024) unsigned char smtc[];
  const uint32_t* cnt = B.counters + kClassBase + depth * kShadeClasses;
  const uint32_t n1 = cnt[SC_DIFFUSE], n2 = cnt[SC_METAL], n4 = cnt[SC_DISNEY], n5 = cnt[SC_GENERIC];
  const uint32_t total = n1 + n2 + n4 + n5;
  // CTAs without a tile leave before the weight load and the TMEM allocation
  // (late bounces hold few queries)
  if (blockIdx.x * kTcRows >= total) return;
  uint64_t* mbar;
  int* fail;
  const uint32_t tmem = TcSetup(G, smtc, mbar, fail);
  uint32_t phase = 0;
  for (uint32_t base = blockIdx.x * kTcRows; base < total; base += gridDim.x * kTcRows) {
    const uint32_t q = base + threadIdx.x;
    const bool valid = q < total;
    uint32_t p = 0;
    uint32_t v[24];
#pragma unroll
    for (int i = 0; i < 24; i++) v[i] = 0u;
    if (valid) {
      uint32_t j = q, cls;
      if (j < n1) {
        cls = SC_DIFFUSE;
      } else if ((j -= n1) < n2) {
        cls = SC_METAL;
      } else if ((j -= n2) < n4) {
        cls = SC_DISNEY;
      } else {
        j -= n4;
        cls = SC_GENERIC;
      }
      p = B.classQ[(size_t)cls * B.capacity + j];
      HitRec h = B.hit[p];
      float4 ro = B.rayO[p], rd = B.rayD[p];
      V3 O{ro.x, ro.y, ro.z}, D{rd.x, rd.y, rd.z};
      TraceHit th{h.t, h.u, h.v, h.prim, h.shape, h.front};
      SurfInt si = ComputeSI(S, O, D, th);
      TcEncodeRow(G, si.P, si.sh.N, -D, v);
    }
    TcStoreInputs(smtc, threadIdx.x, v);
    float o[kGOut];
    if (!TcMlpTile(smtc, tmem, mbar, phase, fail, o)) break;
    if (valid) StoreMix(o, G, G.mix + (size_t)p * kGMixF4);
  }
  TcTeardown(tmem, mbar, phase, fail, B.counters + kMiscBase + 1);
}

// The same network on caller-given queries (the parity hook runs the inference code):
// queries n x 9 (P, N, wo); raw n x kGOut (optional); mix n x kGMixF4 float4 (optional).
__global__ void __launch_bounds__(kTcRows, 1)
    KGuideQueryTc(GuideDev G, const float* queries, uint32_t n, float* raw, float4* mix, uint32_t* err) {
  extern __shared__ __align__(1024) unsigned char smtc[];
  if (blockIdx.x * kTcRows >= n) return;  // as KGuideInferTc
  uint64_t* mbar;
  int* fail;
  const uint32_t tmem = TcSetup(G, smtc, mbar, fail);
  uint32_t phase = 0;
  for (uint32_t base = blockIdx.x * kTcRows; base < n; base += gridDim.x * kTcRows) {
    const uint32_t q = base + threadIdx.x;
    const bool valid = q < n;
    uint32_t v[24];
#pragma unroll
    for (int i = 0; i < 24; i++) v[i] = 0u;
    if (valid) {
      const float* x = queries + (size_t)q * 9;
      TcEncodeRow(G, V3{x[0], x[1], x[2]}, V3{x[3], x[4], x[5]}, V3{x[6], x[7], x[8]}, v);
    }
    TcStoreInputs(smtc, threadIdx.x, v);
    float o[kGOut];
    if (!TcMlpTile(smtc, tmem, mbar, phase, fail, o)) break;
    if (valid) {
      if (raw)
        for (int k = 0; k < kGOut; k++) raw[(size_t)q * kGOut + k] = k < kGOutUsed ? o[k] : 0.f;
      if (mix) StoreMix(o, G, mix + (size_t)q * kGMixF4);
    }
  }
  TcTeardown(tmem, mbar, phase, fail, err);
}

// Mixture pdf at given directions, and samples from u (n x 3) of packed mixtures.
__global__ void KGuideMixEval(const float4* mix, const float* dirs, const float* u, uint32_t n, float* pdf,
                              float* outDirs) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4* mx = mix + (size_t)i * kGMixF4;
  if (dirs) pdf[i] = GuideMixPdfPacked(mx, V3{dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]});
  if (u) {
    V3 w = GuideMixSamplePacked(mx, u[3 * i], V2{u[3 * i + 1], u[3 * i + 2]});
    outDirs[3 * i] = w.x;
    outDirs[3 * i + 1] = w.y;
    outDirs[3 * i + 2] = w.z;
    pdf[i] = GuideMixPdfPacked(mx, w);
  }
}

// Training weight of each record: lum((L_final - L_before) / T_before).
__global__ void KGuideFinalize(PathBuffers B, GuideDev G) {
  uint32_t count = min(G.ctl[0], G.recCap);
  float sum = 0.f;
  for (uint32_t base = blockIdx.x * blockDim.x; base < count; base += gridDim.x * blockDim.x) {
    uint32_t i = base + threadIdx.x;
    float w = 0.f;
    if (i < count) {
      float4* r = G.rec + (size_t)i * kGRecF4;
      uint32_t p = __float_as_uint(r[1].w);
      float4 lf = B.L[p], lb = r[4], tb = r[5];
      float dx = tb.x > 0.f ? (lf.x - lb.x) / tb.x : 0.f;
      float dy = tb.y > 0.f ? (lf.y - lb.y) / tb.y : 0.f;
      float dz = tb.z > 0.f ? (lf.z - lb.z) / tb.z : 0.f;
      w = Luminance(V3{dx, dy, dz});
      if (!(w > 0.f) || !isfinite(w)) w = 0.f;
      r[3].w = w;
      sum += w;
    }
  }
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
  if ((threadIdx.x & 31u) == 0 && sum > 0.f) atomicAdd(reinterpret_cast<float*>(G.ctl + 1), sum);
  if (blockIdx.x == 0 && threadIdx.x == 0 && G.recTotal) *G.recTotal += count;
}

struct GuideTrainArgs {
  GuideDev G;
  const float4* rec;     // records (kGRecF4 float4 each; r0..r3 are read)
  const uint32_t* ctl;   // when set: count = min(ctl[0], cap), mean weight = ctl[1] / count
  uint32_t count, cap;   // explicit count when ctl is null
  uint32_t steps, step;  // this batch = records j * steps + step
  float wClamp;          // normalised weights are clamped to this
  float* gradTable;      // fp32, [level][entry][feature]
  float* gradW;          // fp32, kGWCount
  float* lossOut;        // fp32 loss sum (optional)
  uint32_t* err;         // device error word
};

// ---- training on the fifth-generation tensor cores
// One tile = 128 records (one per thread of a 4-warp CTA). Forward: the four
// layers as in inference; each thread keeps its ReLU masks and also writes its
// layer inputs transposed (feature-major, K = 128 records) for the weight
// gradients. Backward, layer l = 3..0, one commit each:
//   dW_l += G_l^T In_l  (M = out features padded to 128, N = in features,
//                        K = the tile's 128 records; accumulated in TMEM over
//                        all of the CTA's tiles)
//   dIn  = G_l W_l      (M = 128 records, N = in features, K = out features)
// where G_l is the output gradient of layer l (fp16), kept both record-major
// (A of dIn) and feature-major (A of dW; rows beyond the layer's outputs hold
// stale values that only reach accumulator rows that are never read). The
// masked dIn is the next G; layer 0's dIn (the 32 grid features) is scattered
// into the hash-table gradients. After the last tile the CTA adds its dW rows
// to the global gradient. Every wait is bounded (kErrGuideTc, TMEM freed).
constexpr uint32_t kTrWt0 = kTcW3 + kGOut * kGHid * 2;       // W0^T: N = 48 inputs, K = 64
constexpr uint32_t kTrWt1 = kTrWt0 + kGIn * kGHid * 2;       // W1^T: 64 x 64
constexpr uint32_t kTrWt2 = kTrWt1 + kGHid * kGHid * 2;      // W2^T: 64 x 64
constexpr uint32_t kTrWt3 = kTrWt2 + kGHid * kGHid * 2;      // W3^T: N = 64, K = 48
constexpr uint32_t kTrAct = kTrWt3 + kGHid * kGOut * 2;      // 128 x 64 activations (A of the forward)
constexpr uint32_t kTrT0 = kTrAct + kTcRows * kGHid * 2;     // X^T: 48 x 128
constexpr uint32_t kTrT1 = kTrT0 + kGIn * kTcRows * 2;       // H1^T: 64 x 128
constexpr uint32_t kTrT2 = kTrT1 + kGHid * kTcRows * 2;
constexpr uint32_t kTrT3 = kTrT2 + kGHid * kTcRows * 2;
constexpr uint32_t kTrGf = kTrT3 + kGHid * kTcRows * 2;      // G record-major: 128 x 64
constexpr uint32_t kTrGt = kTrGf + kTcRows * kGHid * 2;      // G feature-major: 128 (padded) x 128
constexpr uint32_t kTrMisc = kTrGt + kTcRows * kTcRows * 2;  // mbarrier, TMEM address, fail flag
constexpr int kTrainSmem = (int)kTrMisc + 16;
constexpr uint32_t kTrCols = 512;                            // TMEM: scratch 0..63, dW3, dW2, dW1, dW0
static_assert(kTrWt0 % 16 == 0 && kTrAct % 16 == 0 && kTrT0 % 16 == 0 && kTrGf % 16 == 0 && kTrGt % 16 == 0 &&
                  kTrMisc % 16 == 0,
              "descriptor addresses are 16-byte aligned");
static_assert(kTrainSmem <= 227 * 1024, "training tile fits in shared memory");
// TMEM column of dW_l: dW0 256..303, dW1 192.., dW2 128.., dW3 64..; 0..63 scratch
__device__ __forceinline__ uint32_t TrDW(int l) { return 256u - 64u * (uint32_t)l; }

// D[d] (+)= A x B^T over K, both operands K-major with K halves per row (thread 0).
__device__ __forceinline__ void TcChain(uint32_t d, uint32_t aAddr, uint32_t bAddr, int K, uint32_t idesc, bool acc) {
  for (int s = 0; s < K / 16; s++)
    TcMma(d, TcSmemDesc(aAddr + 256u * s, 128u, 16u * K), TcSmemDesc(bAddr + 256u * s, 128u, 16u * K), idesc,
          acc || s > 0);
}

// Shared-memory operands written by the threads become visible to the tensor
// cores; thread 0 issues `issue` and commits; every thread waits (bounded).
template <class F>
__device__ __forceinline__ bool TcRun(uint64_t* mbar, uint32_t& phase, int* fail, F issue) {
  FenceProxyAsync();
  TcFenceBefore();
  __syncthreads();
  if (threadIdx.x == 0) {
    TcFenceAfter();
    issue();
    TcCommit(mbar);
  }
  const bool ok = MbarWait(mbar, phase, kTcWaitLimit);
  if (!ok) atomicOr(fail, 1);
  __syncthreads();
  if (*fail) return false;
  phase ^= 1u;
  TcFenceAfter();
  return true;
}

__device__ __forceinline__ void StoreHalfT(unsigned char* sm, uint32_t base, uint32_t feature, uint32_t r, float v) {
  *reinterpret_cast<__half*>(sm + base + TcOffset(feature, r, kTcRows)) = __float2half_rn(v);
}

// This thread's row of the 64-column scratch accumulator after a forward layer:
// ReLU, fp16, into the next layer's operand (record-major) and into In^T; the
// ReLU mask is returned (bit k: activation k > 0).
__device__ __forceinline__ uint64_t TrReluOut(unsigned char* sm, uint32_t tmemRow, uint32_t r, uint32_t tBase) {
  uint64_t mask = 0;
#pragma unroll
  for (int c0 = 0; c0 < kGHid; c0 += 16) {
    float v[16];
    TcLoad16(tmemRow + c0, v);
#pragma unroll
    for (int i = 0; i < 16; i++) {
      v[i] = fmaxf(v[i], 0.f);
      if (v[i] > 0.f) mask |= 1ull << (c0 + i);
    }
#pragma unroll
    for (int q = 0; q < 2; q++) {
      uint4 w;
      w.x = PackF2(v[8 * q + 0], v[8 * q + 1]);
      w.y = PackF2(v[8 * q + 2], v[8 * q + 3]);
      w.z = PackF2(v[8 * q + 4], v[8 * q + 5]);
      w.w = PackF2(v[8 * q + 6], v[8 * q + 7]);
      *reinterpret_cast<uint4*>(sm + kTrAct + TcOffset(r, c0 + 8 * q, kGHid)) = w;
    }
#pragma unroll
    for (int i = 0; i < 16; i++) StoreHalfT(sm, tBase, (uint32_t)(c0 + i), r, v[i]);
  }
  return mask;
}

// This thread's row of dIn (scratch columns, 64 wide) masked by the ReLU mask
// of the layer input, as the next output gradient (fp16, both layouts).
__device__ __forceinline__ void TrMaskedGrad(unsigned char* sm, uint32_t tmemRow, uint32_t r, uint64_t mask) {
#pragma unroll
  for (int c0 = 0; c0 < kGHid; c0 += 16) {
    float v[16];
    TcLoad16(tmemRow + c0, v);
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = ((mask >> (c0 + i)) & 1ull) ? v[i] : 0.f;
#pragma unroll
    for (int q = 0; q < 2; q++) {
      uint4 w;
      w.x = PackF2(v[8 * q + 0], v[8 * q + 1]);
      w.y = PackF2(v[8 * q + 2], v[8 * q + 3]);
      w.z = PackF2(v[8 * q + 4], v[8 * q + 5]);
      w.w = PackF2(v[8 * q + 6], v[8 * q + 7]);
      *reinterpret_cast<uint4*>(sm + kTrGf + TcOffset(r, c0 + 8 * q, kGHid)) = w;
    }
#pragma unroll
    for (int i = 0; i < 16; i++) StoreHalfT(sm, kTrGt, (uint32_t)(c0 + i), r, v[i]);
  }
}

__global__ void __launch_bounds__(kTcRows, 1) KGuideTrainTc(GuideTrainArgs a) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const GuideDev& G = a.G;
  const uint32_t r = threadIdx.x;
  const uint32_t count = a.ctl ? min(a.ctl[0], a.cap) : a.count;
  const uint32_t batch = count > a.step ? (count - a.step + a.steps - 1) / a.steps : 0u;
  // CTAs without a tile leave before the weight loads and the TMEM allocation
  if (blockIdx.x * kTcRows >= batch) return;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + kTrMisc);
  uint32_t* slot = reinterpret_cast<uint32_t*>(sm + kTrMisc + 8);
  int* fail = reinterpret_cast<int*>(sm + kTrMisc + 12);
  if (r == 0) {
    MbarInit(mbar, 1);
    *fail = 0;
  }
  if (r < 32) TcAlloc(slot, kTrCols);
  // forward weights [out][in] and transposed [in][out], K-major
  TcLoadWeights(G.weights, sm);
  const __half* gw = G.weights;
  for (int i = (int)r; i < kGIn * kGHid; i += blockDim.x) {
    int n = i / kGHid, k = i % kGHid;  // n: input, k: output
    *reinterpret_cast<__half*>(sm + kTrWt0 + TcOffset(n, k, kGHid)) = gw[kGW0 + k * kGIn + n];
  }
  for (int i = (int)r; i < kGHid * kGHid; i += blockDim.x) {
    int n = i / kGHid, k = i % kGHid;
    *reinterpret_cast<__half*>(sm + kTrWt1 + TcOffset(n, k, kGHid)) = gw[kGW1 + k * kGHid + n];
    *reinterpret_cast<__half*>(sm + kTrWt2 + TcOffset(n, k, kGHid)) = gw[kGW2 + k * kGHid + n];
  }
  for (int i = (int)r; i < kGHid * kGOut; i += blockDim.x) {
    int n = i / kGOut, k = i % kGOut;
    *reinterpret_cast<__half*>(sm + kTrWt3 + TcOffset(n, k, kGOut)) = gw[kGW3 + k * kGHid + n];
  }
  FenceProxyAsync();
  TcFenceBefore();
  __syncthreads();
  TcFenceAfter();
  const uint32_t tmem = *slot;
  const uint32_t tmemRow = tmem + ((32u * (r >> 5)) << 16);
  uint32_t phase = 0;

  float norm = 1.f;
  if (a.ctl) {
    float s = __uint_as_float(a.ctl[1]);
    norm = (s > 0.f && count > 0) ? (float)count / s : 0.f;
  }
  const uint32_t idH = TcIdescF16(kTcRows, kGHid), idO = TcIdescF16(kTcRows, kGOut);
  float lossSum = 0.f;
  uint32_t tiles = 0;
  bool ok = true;
  for (uint32_t tb = blockIdx.x * kTcRows; tb < batch && ok; tb += gridDim.x * kTcRows, tiles++) {
    // ---- encode: this thread's record into the layer-0 operand and X^T
    const uint32_t j = tb + r;
    const bool valid = j < batch;
    uint32_t v[24];
#pragma unroll
    for (int i = 0; i < 24; i++) v[i] = 0u;
    V3 wi{0.f, 0.f, 0.f};
    float pb = 0.f, w = 0.f;
    float4 r0 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) {
      const float4* rc = a.rec + (size_t)(j * a.steps + a.step) * kGRecF4;
      r0 = rc[0];
      const float4 r1 = rc[1], r2 = rc[2], r3 = rc[3];
      TcEncodeRow(G, V3{r0.x, r0.y, r0.z}, V3{r1.x, r1.y, r1.z}, V3{r2.x, r2.y, r2.z}, v);
      wi = V3{r3.x, r3.y, r3.z};
      pb = r0.w;
      w = fminf(r3.w * norm, a.wClamp);
      if (!(w > 0.f)) w = 0.f;
    }
#pragma unroll
    for (int c = 0; c < kGIn / 8; c++)
      *reinterpret_cast<uint4*>(sm + kTrAct + TcOffset(r, 8 * c, kGIn)) =
          make_uint4(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]);
#pragma unroll
    for (int i = 0; i < 24; i++) {
      *reinterpret_cast<uint16_t*>(sm + kTrT0 + TcOffset(2 * i, r, kTcRows)) = (uint16_t)(v[i] & 0xffffu);
      *reinterpret_cast<uint16_t*>(sm + kTrT0 + TcOffset(2 * i + 1, r, kTcRows)) = (uint16_t)(v[i] >> 16);
    }
    // ---- forward
    uint64_t mask[3];
    const uint32_t fw[3] = {kTcW0, kTcW1, kTcW2}, tOut[3] = {kTrT1, kTrT2, kTrT3};
    for (int l = 0; l < 3 && ok; l++) {
      const int K = l == 0 ? kGIn : kGHid;
      ok = TcRun(mbar, phase, fail, [&] { TcChain(tmem, SmemAddr(sm + kTrAct), SmemAddr(sm + fw[l]), K, idH, false); });
      if (ok) mask[l] = TrReluOut(sm, tmemRow, r, tOut[l]);
    }
    if (!ok) break;
    ok = TcRun(mbar, phase, fail, [&] { TcChain(tmem, SmemAddr(sm + kTrAct), SmemAddr(sm + kTcW3), kGHid, idO, false); });
    if (!ok) break;
    // ---- loss gradient at the outputs: G_3 in both layouts
    {
      float o[kGOut], dO[kGOut];
#pragma unroll
      for (int c0 = 0; c0 < kGOut; c0 += 16) {
        float t[16];
        TcLoad16(tmemRow + c0, t);
#pragma unroll
        for (int i = 0; i < 16; i++) o[c0 + i] = c0 + i < kGOutUsed ? t[i] : 0.f;
      }
      if (w > 0.f) {
        lossSum += GuideLossGrad(o, wi, pb, w, G.logKMax, G.cMax, dO);
      } else {
        for (int k = 0; k < kGOut; k++) dO[k] = 0.f;
      }
#pragma unroll
      for (int c = 0; c < kGOut / 8; c++)
        *reinterpret_cast<uint4*>(sm + kTrGf + TcOffset(r, 8 * c, kGOut)) =
            make_uint4(PackF2(dO[8 * c], dO[8 * c + 1]), PackF2(dO[8 * c + 2], dO[8 * c + 3]),
                       PackF2(dO[8 * c + 4], dO[8 * c + 5]), PackF2(dO[8 * c + 6], dO[8 * c + 7]));
      for (int k = 0; k < kGOut; k++) StoreHalfT(sm, kTrGt, (uint32_t)k, r, dO[k]);
    }
    // ---- backward: dW_l += G^T In_l and dIn = G W_l, layers 3, 2, 1
    const bool acc = tiles > 0;
    const uint32_t tIn[4] = {kTrT0, kTrT1, kTrT2, kTrT3}, wt[4] = {kTrWt0, kTrWt1, kTrWt2, kTrWt3};
    for (int l = 3; l >= 1 && ok; l--) {
      const int K = l == 3 ? kGOut : kGHid;
      ok = TcRun(mbar, phase, fail, [&] {
        TcChain(tmem + TrDW(l), SmemAddr(sm + kTrGt), SmemAddr(sm + tIn[l]), kTcRows, idH, acc);
        TcChain(tmem, SmemAddr(sm + kTrGf), SmemAddr(sm + wt[l]), K, idH, false);
      });
      if (ok) TrMaskedGrad(sm, tmemRow, r, mask[l - 1]);
    }
    if (!ok) break;
    // ---- layer 0: dW0 += G^T X, dX = G W0 (N = 48; the 32 grid features are used)
    ok = TcRun(mbar, phase, fail, [&] {
      TcChain(tmem + TrDW(0), SmemAddr(sm + kTrGt), SmemAddr(sm + kTrT0), kTcRows, idO, acc);
      TcChain(tmem, SmemAddr(sm + kTrGf), SmemAddr(sm + kTrWt0), kGHid, idO, false);
    });
    if (!ok) break;
    float dx[32];
    TcLoad16(tmemRow, *reinterpret_cast<float(*)[16]>(dx));
    TcLoad16(tmemRow + 16, *reinterpret_cast<float(*)[16]>(dx + 16));
    TcFenceBefore();  // the next tile's MMAs are issued after every thread's reads
    // ---- hash-table gradients (scatter)
    if (valid && w > 0.f) {
      float u[3];
      GuidePosToUnit(G, V3{r0.x, r0.y, r0.z}, u);
      for (int l = 0; l < kGLevels; l++) {
        const float g0 = dx[2 * l], g1 = dx[2 * l + 1];
        if (g0 == 0.f && g1 == 0.f) continue;
        const uint32_t res = G.res[l];
        uint32_t cx, cy, cz;
        float tx, ty, tz;
        GuideCell(u[0], res, cx, tx);
        GuideCell(u[1], res, cy, ty);
        GuideCell(u[2], res, cz, tz);
        float2* gt = reinterpret_cast<float2*>(a.gradTable) + ((size_t)l << G.log2T);
        for (int c = 0; c < 8; c++) {
          const uint32_t bx = c & 1u, by = (c >> 1) & 1u, bz = (c >> 2) & 1u;
          const float cw = (bx ? tx : 1.f - tx) * (by ? ty : 1.f - ty) * (bz ? tz : 1.f - tz);
          const uint32_t idx = GuideGridIndex(cx + bx, cy + by, cz + bz, res, G.log2T);
          atomicAdd(gt + idx, make_float2(cw * g0, cw * g1));
        }
      }
    }
  }
  // ---- this CTA's weight gradients: row r of dW_l (out feature r) in TMEM lane r
  if (ok && tiles > 0 && r < (uint32_t)kGHid) {
    const int outs[4] = {kGHid, kGHid, kGHid, kGOut}, ins[4] = {kGIn, kGHid, kGHid, kGHid};
    const int base[4] = {kGW0, kGW1, kGW2, kGW3};
    for (int l = 0; l < 4; l++) {
      for (int c0 = 0; c0 < ins[l]; c0 += 16) {
        float t[16];
        TcLoad16(tmemRow + TrDW(l) + (uint32_t)c0, t);
        if ((int)r < outs[l])
          for (int i = 0; i < 16; i++)
            if (t[i] != 0.f) atomicAdd(a.gradW + base[l] + (int)r * ins[l] + c0 + i, t[i]);
      }
    }
  }
  if (a.lossOut) {
    for (int o = 16; o > 0; o >>= 1) lossSum += __shfl_down_sync(0xffffffffu, lossSum, o);
    if ((r & 31u) == 0 && lossSum != 0.f) atomicAdd(a.lossOut, lossSum);
  }
  // teardown: on a timeout, one more bounded wait for the MMA still outstanding
  if (*fail) {
    MbarWait(mbar, phase, kTcWaitLimit);
    if (r == 0) atomicOr(a.err, kErrGuideTc);
  }
  TcFenceBefore();
  __syncthreads();
  TcFenceAfter();
  if (r < 32) TcDealloc(tmem, kTrCols);
}

struct GuideAdamArgs {
  float* p;
  float* m;
  float* v;
  float* g;
  __half* ph;
  uint64_t n;
  float lr, b1, b2, eps, gscale, bc1, bc2;
  uint64_t split;  // parameters [split, n) use lr2
  float lr2;
  uint64_t lazySplit;  // parameters below it without a gradient are left untouched (split, or 0)
  const uint32_t* ctl;  // when set: gscale = 1 / (records of batch `step`), no update for an empty batch
  uint32_t cap, steps, step;
};

// Hash-table entries ([0, lazySplit), the table when the lazy update is on)
// without a gradient in the batch keep their parameters and moments (the lazy
// update of sparse embedding tables): a batch touches a few percent of the
// table, so the step reads the gradient of every entry but the moments and
// parameters of the touched ones only. The MLP's parameters take every step.
__global__ void KGuideAdam(GuideAdamArgs a) {
  if (a.ctl) {
    uint32_t count = min(a.ctl[0], a.cap);
    uint32_t batch = count > a.step ? (count - a.step + a.steps - 1) / a.steps : 0u;
    if (batch == 0) return;
    a.gscale = 1.f / (float)batch;
  }
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (uint64_t)gridDim.x * blockDim.x) {
    const float graw = a.g[i];
    if (graw == 0.f && i < a.lazySplit) continue;
    float gi = graw * a.gscale;
    if (!isfinite(gi)) gi = 0.f;
    float m = a.b1 * a.m[i] + (1.f - a.b1) * gi;
    float v = a.b2 * a.v[i] + (1.f - a.b2) * gi * gi;
    float lr = i < a.split ? a.lr : a.lr2;
    float p = a.p[i] - lr * (m / a.bc1) / (sqrtf(v / a.bc2) + a.eps);
    a.m[i] = m;
    a.v[i] = v;
    a.p[i] = p;
    a.g[i] = 0.f;
    a.ph[i] = __float2half_rn(p);
  }
}

__global__ void KFloatToHalf(const float* src, __half* dst, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    dst[i] = __float2half_rn(src[i]);
}

// ---------------------------------------------------------------- launchers
static int GuideGrid(int perSm) { return PathGridBlocks() / 8 * perSm; }

cudaError_t GuideKernelsInit() {
  cudaError_t e = cudaFuncSetAttribute(KGuideInferTc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(KGuideQueryTc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(KGuideTrainTc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrainSmem);
}

cudaError_t LaunchGuideInfer(const DevScene& S, const PathBuffers& B, const GuideDev& G, int depth, uint32_t maxCount,
                             cudaStream_t st) {
  // tcgen05 tiles of 128 queries; at most 4 CTAs per SM (4 x 64 TMEM columns of 512)
  int blocks = (int)std::min<uint32_t>((maxCount + kTcRows - 1) / kTcRows, (uint32_t)GuideGrid(4));
  if (blocks < 1) blocks = 1;
  KGuideInferTc<<<blocks, kTcRows, kTcSmem, st>>>(S, B, G, depth);
  return cudaGetLastError();
}

cudaError_t LaunchGuideQuery(const GuideDev& G, const float* queries, uint32_t n, float* raw, float4* mix,
                             uint32_t* err, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  int blocks = (int)std::min<uint32_t>((n + kTcRows - 1) / kTcRows, (uint32_t)GuideGrid(4));
  KGuideQueryTc<<<blocks, kTcRows, kTcSmem, st>>>(G, queries, n, raw, mix, err);
  return cudaGetLastError();
}

cudaError_t LaunchGuideMixEval(const float4* mix, const float* dirs, const float* u, uint32_t n, float* pdf,
                               float* outDirs, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  KGuideMixEval<<<(n + 127) / 128, 128, 0, st>>>(mix, dirs, u, n, pdf, outDirs);
  return cudaGetLastError();
}

cudaError_t LaunchGuideFinalize(const PathBuffers& B, const GuideDev& G, cudaStream_t st) {
  KGuideFinalize<<<GuideGrid(4), 256, 0, st>>>(B, G);
  return cudaGetLastError();
}

cudaError_t LaunchGuideTrain(const GuideDev& G, const float4* rec, const uint32_t* ctl, uint32_t count, uint32_t cap,
                             uint32_t steps, uint32_t step, float wClamp, float* gradTable, float* gradW,
                             float* lossOut, uint32_t maxBatch, uint32_t* err, cudaStream_t st) {
  GuideTrainArgs a{G, rec, ctl, count, cap, steps, step, wClamp, gradTable, gradW, lossOut, err};
  // one CTA per SM (its shared memory and 512 TMEM columns)
  int blocks = (int)std::min<uint32_t>((maxBatch + kTcRows - 1) / kTcRows, (uint32_t)GuideGrid(1));
  if (blocks < 1) blocks = 1;
  KGuideTrainTc<<<blocks, kTcRows, kTrainSmem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t LaunchGuideAdam(float* p, float* m, float* v, float* g, __half* ph, uint64_t n, float lr, uint64_t split,
                            float lr2, float b1, float b2, float eps, float gscale, uint32_t t, const uint32_t* ctl,
                            uint32_t cap, uint32_t steps, uint32_t step, bool lazyTable, cudaStream_t st) {
  GuideAdamArgs a{p,     m,   v,   g,   ph,  n,   lr,   b1,   b2,  eps, gscale, 1.f - powf(b1, (float)t),
                  1.f - powf(b2, (float)t), split, lr2, lazyTable ? split : 0u, ctl, cap, steps, step};
  KGuideAdam<<<GuideGrid(8), 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t LaunchFloatToHalf(const float* src, __half* dst, uint64_t n, cudaStream_t st) {
  KFloatToHalf<<<GuideGrid(8), 256, 0, st>>>(src, dst, n);
  return cudaGetLastError();
}

}  // namespace rad
