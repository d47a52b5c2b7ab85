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
// Training's products (forward, dIn = G W and dW = G^T In over 64-record tiles)
// run on mma.sync m16n8k16 (fp16 operands, fp32 accumulation), one warp per 16
// or 32 rows, with the weights in shared memory padded for conflict-free
// fragment loads.
#include <algorithm>

#include "dguide.cuh"
#include "dscene.cuh"
#include "dtc.cuh"
#include "kernels.h"

namespace rad {

namespace {

constexpr int kLd48 = 56;    // smem row stride (halves) of a 48-wide operand
constexpr int kLd64 = 72;    // ... of a 64-wide operand
constexpr int kActLd = 88;   // activation row: 88 halves = 44 floats of output
// forward weights in shared memory, [out][in] with padded rows
constexpr int kSW0 = 0;
constexpr int kSW1 = kSW0 + kGHid * kLd48;
constexpr int kSW2 = kSW1 + kGHid * kLd64;
constexpr int kSW3 = kSW2 + kGHid * kLd64;
constexpr int kSWEnd = kSW3 + kGOut * kLd64;  // 16256 halves

enum { kRelu = 0, kMask = 1, kF32 = 2 };

__device__ __forceinline__ void Mma16816(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t Ld32(const __half* p) { return *reinterpret_cast<const uint32_t*>(p); }
__device__ __forceinline__ uint32_t Pack2(__half lo, __half hi) {
  return (uint32_t)__half_as_ushort(lo) | ((uint32_t)__half_as_ushort(hi) << 16);
}
__device__ __forceinline__ uint32_t PackF2(float lo, float hi) {
  return Pack2(__float2half_rn(lo), __float2half_rn(hi));
}

// D[r][n] = sum_k A[r][k] Bm[n][k] over the warp's MT x 16 rows. A and the
// output may alias (each 16-row tile is read completely before it is written).
// Epilogues: kRelu -> fp16 max(0, x); kMask -> fp16 x where mask[r][n] > 0;
// kF32 -> fp32, columns below `ldo` only.
template <int K, int N, int MT, int MODE>
__device__ __forceinline__ void WarpGemm(const __half* A, int lda, const __half* Bm, int ldb, void* out, int ldo,
                                         const __half* mask, int ldm) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int mt = 0; mt < MT; mt++) {
    float acc[N / 8][4];
#pragma unroll
    for (int i = 0; i < N / 8; i++) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.f;
#pragma unroll
    for (int kk = 0; kk < K; kk += 16) {
      const __half* ap = A + (mt * 16 + g) * lda + kk + 2 * t;
      uint32_t a[4] = {Ld32(ap), Ld32(ap + 8 * lda), Ld32(ap + 8), Ld32(ap + 8 * lda + 8)};
#pragma unroll
      for (int nt = 0; nt < N / 8; nt++) {
        const __half* bp = Bm + (nt * 8 + g) * ldb + kk + 2 * t;
        uint32_t b[2] = {Ld32(bp), Ld32(bp + 8)};
        Mma16816(acc[nt], a, b);
      }
    }
    __syncwarp();
#pragma unroll
    for (int nt = 0; nt < N / 8; nt++) {
      const int r0 = mt * 16 + g, c = nt * 8 + 2 * t;
      if constexpr (MODE == kF32) {
        if (c < ldo) {
          float* o = static_cast<float*>(out);
          o[r0 * ldo + c] = acc[nt][0];
          o[r0 * ldo + c + 1] = acc[nt][1];
          o[(r0 + 8) * ldo + c] = acc[nt][2];
          o[(r0 + 8) * ldo + c + 1] = acc[nt][3];
        }
      } else {
        float v0 = acc[nt][0], v1 = acc[nt][1], v2 = acc[nt][2], v3 = acc[nt][3];
        if constexpr (MODE == kRelu) {
          v0 = fmaxf(v0, 0.f);
          v1 = fmaxf(v1, 0.f);
          v2 = fmaxf(v2, 0.f);
          v3 = fmaxf(v3, 0.f);
        } else {
          if (!(__half2float(mask[r0 * ldm + c]) > 0.f)) v0 = 0.f;
          if (!(__half2float(mask[r0 * ldm + c + 1]) > 0.f)) v1 = 0.f;
          if (!(__half2float(mask[(r0 + 8) * ldm + c]) > 0.f)) v2 = 0.f;
          if (!(__half2float(mask[(r0 + 8) * ldm + c + 1]) > 0.f)) v3 = 0.f;
        }
        __half* o = static_cast<__half*>(out);
        *reinterpret_cast<uint32_t*>(o + r0 * ldo + c) = PackF2(v0, v1);
        *reinterpret_cast<uint32_t*>(o + (r0 + 8) * ldo + c) = PackF2(v2, v3);
      }
    }
    __syncwarp();
  }
}

// dW[n][k] += sum_r G[r][n] In[r][k] for n in [n0, n0 + 16), k < KIN, r < 64
// (a 64-record tile). The warp owns those 16 rows of dW.
template <int KIN>
__device__ __forceinline__ void WarpGradW(const __half* G, int ldg, const __half* In, int ldi, float* dW, int n0) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  float acc[KIN / 8][4];
#pragma unroll
  for (int i = 0; i < KIN / 8; i++) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.f;
#pragma unroll
  for (int rr = 0; rr < 64; rr += 16) {
    const __half* gp = G + (rr + 2 * t) * ldg + n0 + g;
    uint32_t a[4] = {Pack2(gp[0], gp[ldg]), Pack2(gp[8], gp[ldg + 8]), Pack2(gp[8 * ldg], gp[9 * ldg]),
                     Pack2(gp[8 * ldg + 8], gp[9 * ldg + 8])};
#pragma unroll
    for (int kt = 0; kt < KIN / 8; kt++) {
      const __half* bp = In + (rr + 2 * t) * ldi + kt * 8 + g;
      uint32_t b[2] = {Pack2(bp[0], bp[ldi]), Pack2(bp[8 * ldi], bp[9 * ldi])};
      Mma16816(acc[kt], a, b);
    }
  }
#pragma unroll
  for (int kt = 0; kt < KIN / 8; kt++) {
    const int c = kt * 8 + 2 * t;
    dW[(n0 + g) * KIN + c] += acc[kt][0];
    dW[(n0 + g) * KIN + c + 1] += acc[kt][1];
    dW[(n0 + g + 8) * KIN + c] += acc[kt][2];
    dW[(n0 + g + 8) * KIN + c + 1] += acc[kt][3];
  }
}

__device__ void LoadFwdWeights(const __half* gw, __half* s) {
  const __half z = __float2half_rn(0.f);
  for (int i = threadIdx.x; i < kGHid * kLd48; i += blockDim.x) {
    int n = i / kLd48, k = i % kLd48;
    s[kSW0 + i] = k < kGIn ? gw[kGW0 + n * kGIn + k] : z;
  }
  for (int i = threadIdx.x; i < kGHid * kLd64; i += blockDim.x) {
    int n = i / kLd64, k = i % kLd64;
    s[kSW1 + i] = k < kGHid ? gw[kGW1 + n * kGHid + k] : z;
    s[kSW2 + i] = k < kGHid ? gw[kGW2 + n * kGHid + k] : z;
  }
  for (int i = threadIdx.x; i < kGOut * kLd64; i += blockDim.x) {
    int n = i / kLd64, k = i % kLd64;
    s[kSW3 + i] = k < kGHid ? gw[kGW3 + n * kGHid + k] : z;
  }
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
  uint64_t* mbar;
  int* fail;
  const uint32_t tmem = TcSetup(G, smtc, mbar, fail);
  uint32_t phase = 0;
  const uint32_t* cnt = B.counters + kClassBase + depth * kShadeClasses;
  const uint32_t n1 = cnt[SC_DIFFUSE], n2 = cnt[SC_METAL], n4 = cnt[SC_DISNEY], n5 = cnt[SC_GENERIC];
  const uint32_t total = n1 + n2 + n4 + n5;
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

namespace {
constexpr int kTRec = 64;  // records per tile (4 warps x 16 rows)
constexpr int kTB0 = kSWEnd;                 // W0^T [48][72]
constexpr int kTB1 = kTB0 + kGIn * kLd64;    // W1^T [64][72]
constexpr int kTB2 = kTB1 + kGHid * kLd64;   // W2^T [64][72]
constexpr int kTB3 = kTB2 + kGHid * kLd64;   // W3^T [64][56]
constexpr int kTX = kTB3 + kGHid * kLd48;    // X  [64][56]
constexpr int kTH1 = kTX + kTRec * kLd48;    // H1 [64][72]
constexpr int kTH2 = kTH1 + kTRec * kLd64;
constexpr int kTH3 = kTH2 + kTRec * kLd64;
constexpr int kTG0 = kTH3 + kTRec * kLd64;   // gradient ping [64][88] (or fp32 [64][44])
constexpr int kTG1 = kTG0 + kTRec * kActLd;  // gradient pong
constexpr int kTHalves = kTG1 + kTRec * kActLd;
constexpr int kTrainSmem = kTHalves * 2 + kGWCount * 4 + kTRec * 5 * 4;
}  // namespace

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
};

__global__ void __launch_bounds__(128, 1) KGuideTrain(GuideTrainArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __half* sh = reinterpret_cast<__half*>(smraw);
  float* dW = reinterpret_cast<float*>(smraw + kTHalves * 2);
  float* sRec = dW + kGWCount;  // per record: wi xyz, p_bsdf, weight
  const GuideDev& G = a.G;
  const int tid = threadIdx.x, warp = tid >> 5;
  // weights: forward [out][in] and transposed [in][out] copies
  LoadFwdWeights(G.weights, sh);
  const __half z = __float2half_rn(0.f);
  const __half* gw = G.weights;
  for (int i = tid; i < kGIn * kLd64; i += blockDim.x) {
    int k = i / kLd64, n = i % kLd64;
    sh[kTB0 + i] = n < kGHid ? gw[kGW0 + n * kGIn + k] : z;
  }
  for (int i = tid; i < kGHid * kLd64; i += blockDim.x) {
    int k = i / kLd64, n = i % kLd64;
    sh[kTB1 + i] = n < kGHid ? gw[kGW1 + n * kGHid + k] : z;
    sh[kTB2 + i] = n < kGHid ? gw[kGW2 + n * kGHid + k] : z;
  }
  for (int i = tid; i < kGHid * kLd48; i += blockDim.x) {
    int k = i / kLd48, n = i % kLd48;
    sh[kTB3 + i] = n < kGOut ? gw[kGW3 + n * kGHid + k] : z;
  }
  for (int i = tid; i < kGWCount; i += blockDim.x) dW[i] = 0.f;
  uint32_t count = a.ctl ? min(a.ctl[0], a.cap) : a.count;
  float norm = 1.f;
  if (a.ctl) {
    float s = __uint_as_float(a.ctl[1]);
    norm = (s > 0.f && count > 0) ? (float)count / s : 0.f;
  }
  uint32_t batch = count > a.step ? (count - a.step + a.steps - 1) / a.steps : 0u;
  __syncthreads();
  __half* X = sh + kTX;
  __half* H1 = sh + kTH1;
  __half* H2 = sh + kTH2;
  __half* H3 = sh + kTH3;
  __half* G0 = sh + kTG0;
  __half* G1 = sh + kTG1;
  float lossSum = 0.f;
  for (uint32_t tb = blockIdx.x * kTRec; tb < batch; tb += gridDim.x * kTRec) {
    // ---- encode (two threads per record, eight levels each)
    {
      const int r = tid & 63, half = tid >> 6;
      const uint32_t j = tb + r;
      const bool valid = j < batch;
      __half* row = X + r * kLd48;
      if (valid) {
        const float4* rc = a.rec + (size_t)(j * a.steps + a.step) * kGRecF4;
        float4 r0 = rc[0], r1 = rc[1], r2 = rc[2], r3 = rc[3];
        float u[3];
        GuidePosToUnit(G, V3{r0.x, r0.y, r0.z}, u);
        GuideEncodeLevels(G, u, half * 8, half * 8 + 8, row);
        if (half == 0) {
          GuideEncodeTail(V3{r1.x, r1.y, r1.z}, V3{r2.x, r2.y, r2.z}, row);
          float w = fminf(r3.w * norm, a.wClamp);
          sRec[r * 5 + 0] = r3.x;
          sRec[r * 5 + 1] = r3.y;
          sRec[r * 5 + 2] = r3.z;
          sRec[r * 5 + 3] = r0.w;
          sRec[r * 5 + 4] = (w > 0.f) ? w : 0.f;
        }
      } else {
        for (int k = half * 24; k < half * 24 + 24; k += 2) *reinterpret_cast<uint32_t*>(row + k) = 0u;
        if (half == 0)
          for (int k = 0; k < 5; k++) sRec[r * 5 + k] = 0.f;
      }
    }
    __syncthreads();
    // ---- forward, warp w owns rows [16w, 16w + 16)
    {
      const int r0 = warp * 16;
      WarpGemm<kGIn, kGHid, 1, kRelu>(X + r0 * kLd48, kLd48, sh + kSW0, kLd48, H1 + r0 * kLd64, kLd64, nullptr, 0);
      WarpGemm<kGHid, kGHid, 1, kRelu>(H1 + r0 * kLd64, kLd64, sh + kSW1, kLd64, H2 + r0 * kLd64, kLd64, nullptr, 0);
      WarpGemm<kGHid, kGHid, 1, kRelu>(H2 + r0 * kLd64, kLd64, sh + kSW2, kLd64, H3 + r0 * kLd64, kLd64, nullptr, 0);
      WarpGemm<kGHid, kGOut, 1, kF32>(H3 + r0 * kLd64, kLd64, sh + kSW3, kLd64,
                                      reinterpret_cast<float*>(G0) + r0 * (kActLd / 2), kActLd / 2, nullptr, 0);
    }
    __syncthreads();
    // ---- loss gradient at the outputs (one thread per record)
    if (tid < kTRec) {
      const float* o = reinterpret_cast<const float*>(G0) + tid * (kActLd / 2);
      float dO[kGOut];
      float w = sRec[tid * 5 + 4];
      float loss = 0.f;
      if (w > 0.f) {
        float oo[kGOut];
        for (int k = 0; k < kGOut; k++) oo[k] = k < kGOutUsed ? o[k] : 0.f;
        loss = GuideLossGrad(oo, V3{sRec[tid * 5], sRec[tid * 5 + 1], sRec[tid * 5 + 2]}, sRec[tid * 5 + 3], w,
                             G.logKMax, G.cMax, dO);
      } else {
        for (int k = 0; k < kGOut; k++) dO[k] = 0.f;
      }
      lossSum += loss;
      __half* gr = G1 + tid * kActLd;
      for (int k = 0; k < kGOut; k += 2) *reinterpret_cast<uint32_t*>(gr + k) = PackF2(dO[k], dO[k + 1]);
    }
    __syncthreads();
    // ---- layer 3: dW3 += dO^T H3, dH3 = (dO W3) * [H3 > 0]
    {
      const int r0 = warp * 16;
      if (warp < 3) WarpGradW<kGHid>(G1, kActLd, H3, kLd64, dW + kGW3, warp * 16);
      WarpGemm<kGOut, kGHid, 1, kMask>(G1 + r0 * kActLd, kActLd, sh + kTB3, kLd48, G0 + r0 * kActLd, kActLd,
                                       H3 + r0 * kLd64, kLd64);
    }
    __syncthreads();
    {
      const int r0 = warp * 16;
      WarpGradW<kGHid>(G0, kActLd, H2, kLd64, dW + kGW2, warp * 16);
      WarpGemm<kGHid, kGHid, 1, kMask>(G0 + r0 * kActLd, kActLd, sh + kTB2, kLd64, G1 + r0 * kActLd, kActLd,
                                       H2 + r0 * kLd64, kLd64);
    }
    __syncthreads();
    {
      const int r0 = warp * 16;
      WarpGradW<kGHid>(G1, kActLd, H1, kLd64, dW + kGW1, warp * 16);
      WarpGemm<kGHid, kGHid, 1, kMask>(G1 + r0 * kActLd, kActLd, sh + kTB1, kLd64, G0 + r0 * kActLd, kActLd,
                                       H1 + r0 * kLd64, kLd64);
    }
    __syncthreads();
    {
      const int r0 = warp * 16;
      WarpGradW<kGIn>(G0, kActLd, X, kLd48, dW + kGW0, warp * 16);
      // input gradient of the 32 grid features, fp32
      WarpGemm<kGHid, 32, 1, kF32>(G0 + r0 * kActLd, kActLd, sh + kTB0, kLd64,
                                   reinterpret_cast<float*>(G1) + r0 * (kActLd / 2), kActLd / 2, nullptr, 0);
    }
    __syncthreads();
    // ---- hash-table gradients (scatter)
    {
      const int r = tid & 63, half = tid >> 6;
      const uint32_t j = tb + r;
      if (j < batch && sRec[r * 5 + 4] > 0.f) {
        const float4* rc = a.rec + (size_t)(j * a.steps + a.step) * kGRecF4;
        float4 r0 = rc[0];
        float u[3];
        GuidePosToUnit(G, V3{r0.x, r0.y, r0.z}, u);
        const float* dx = reinterpret_cast<const float*>(G1) + r * (kActLd / 2);
        for (int l = half * 8; l < half * 8 + 8; l++) {
          float g0 = dx[2 * l], g1 = dx[2 * l + 1];
          if (g0 == 0.f && g1 == 0.f) continue;
          uint32_t res = G.res[l];
          uint32_t cx, cy, cz;
          float tx, ty, tz;
          GuideCell(u[0], res, cx, tx);
          GuideCell(u[1], res, cy, ty);
          GuideCell(u[2], res, cz, tz);
          float2* gt = reinterpret_cast<float2*>(a.gradTable) + ((size_t)l << G.log2T);
          for (int c = 0; c < 8; c++) {
            uint32_t bx = c & 1u, by = (c >> 1) & 1u, bz = (c >> 2) & 1u;
            float w = (bx ? tx : 1.f - tx) * (by ? ty : 1.f - ty) * (bz ? tz : 1.f - tz);
            uint32_t idx = GuideGridIndex(cx + bx, cy + by, cz + bz, res, G.log2T);
            atomicAdd(gt + idx, make_float2(w * g0, w * g1));
          }
        }
      }
    }
    __syncthreads();
  }
  for (int i = tid; i < kGWCount; i += blockDim.x)
    if (dW[i] != 0.f) atomicAdd(a.gradW + i, dW[i]);
  if (a.lossOut && tid < kTRec) {  // the loss threads are warps 0 and 1
    for (int o = 16; o > 0; o >>= 1) lossSum += __shfl_down_sync(0xffffffffu, lossSum, o);
    if ((tid & 31) == 0 && lossSum != 0.f) atomicAdd(a.lossOut, lossSum);
  }
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
  const uint32_t* ctl;  // when set: gscale = 1 / (records of batch `step`), no update for an empty batch
  uint32_t cap, steps, step;
};

// Hash-table entries ([0, split)) without a gradient in the batch keep their
// parameters and moments (the lazy update of sparse embedding tables): a batch
// touches a few percent of the table, so the step reads the gradient of every
// entry but the moments and parameters of the touched ones only. The MLP's
// parameters ([split, n)) take every step.
__global__ void KGuideAdam(GuideAdamArgs a) {
  if (a.ctl) {
    uint32_t count = min(a.ctl[0], a.cap);
    uint32_t batch = count > a.step ? (count - a.step + a.steps - 1) / a.steps : 0u;
    if (batch == 0) return;
    a.gscale = 1.f / (float)batch;
  }
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (uint64_t)gridDim.x * blockDim.x) {
    const float graw = a.g[i];
    if (graw == 0.f && i < a.split) continue;
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
  return cudaFuncSetAttribute(KGuideTrain, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrainSmem);
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
                             float* lossOut, uint32_t maxBatch, cudaStream_t st) {
  GuideTrainArgs a{G, rec, ctl, count, cap, steps, step, wClamp, gradTable, gradW, lossOut};
  int blocks = (int)std::min<uint32_t>((maxBatch + kTRec - 1) / kTRec, (uint32_t)GuideGrid(1));
  if (blocks < 1) blocks = 1;
  KGuideTrain<<<blocks, 128, kTrainSmem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t LaunchGuideAdam(float* p, float* m, float* v, float* g, __half* ph, uint64_t n, float lr, uint64_t split,
                            float lr2, float b1, float b2, float eps, float gscale, uint32_t t, const uint32_t* ctl,
                            uint32_t cap, uint32_t steps, uint32_t step, cudaStream_t st) {
  GuideAdamArgs a{p,     m,   v,   g,   ph,  n,   lr,   b1,   b2,  eps, gscale, 1.f - powf(b1, (float)t),
                  1.f - powf(b2, (float)t), split, lr2, ctl, cap, steps, step};
  KGuideAdam<<<GuideGrid(8), 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t LaunchFloatToHalf(const float* src, __half* dst, uint64_t n, cudaStream_t st) {
  KFloatToHalf<<<GuideGrid(8), 256, 0, st>>>(src, dst, n);
  return cudaGetLastError();
}

}  // namespace rad
