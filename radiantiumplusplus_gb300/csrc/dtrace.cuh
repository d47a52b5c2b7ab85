// BVH8 traversal replacing Embree's rtcIntersect1 / rtcOccluded1
// (rad.offline/src/accel/embree.cpp:79-111). One thread per ray; nodes are
// fetched as five 128-bit loads, primitives as three. Hit acceptance is the
// same as the CPU oracle's: t in (tmin, best), and on an exact tie the lower
// global primitive id wins, so the closest hit is independent of traversal
// order. Triangle test: watertight (Woop, Benthin, Wald, JCGT 2013).
#pragma once
#include "dmath.cuh"

namespace rad {

constexpr uint32_t kNoPrim = 0xffffffffu;
constexpr int kTraceStack = 48;

struct RayPre {
  V3 O, D;
  float tmin;
  // watertight shear
  int kx, ky, kz;
  float Sx, Sy, Sz;
  // box test
  V3 inv;
  uint32_t oct;
};

RD RayPre MakeRayPre(V3 O, V3 D, float tmin) {
  RayPre r;
  r.O = O;
  r.D = D;
  r.tmin = tmin;
  float ax = fabsf(D.x), ay = fabsf(D.y), az = fabsf(D.z);
  int kz = 0;
  if (ay > ax) kz = 1;
  if (az > fmaxr(ax, ay)) kz = 2;
  int kx = kz + 1 == 3 ? 0 : kz + 1;
  int ky = kx + 1 == 3 ? 0 : kx + 1;
  if (comp(D, kz) < 0.f) {
    int t = kx;
    kx = ky;
    ky = t;
  }
  r.kx = kx;
  r.ky = ky;
  r.kz = kz;
  float dz = comp(D, kz);
  r.Sx = comp(D, kx) / dz;
  r.Sy = comp(D, ky) / dz;
  r.Sz = 1.0f / dz;
  // zero direction components become +-1e-20 for the box test only (no NaN slabs)
  float dx = fabsf(D.x) < 1e-20f ? copysignf(1e-20f, D.x) : D.x;
  float dy = fabsf(D.y) < 1e-20f ? copysignf(1e-20f, D.y) : D.y;
  float dzz = fabsf(D.z) < 1e-20f ? copysignf(1e-20f, D.z) : D.z;
  r.inv = V3{1.f / dx, 1.f / dy, 1.f / dzz};
  r.oct = (r.inv.x < 0.f ? 1u : 0u) | (r.inv.y < 0.f ? 2u : 0u) | (r.inv.z < 0.f ? 4u : 0u);
  return r;
}

// Watertight triangle test; returns t and Embree barycentrics (u weights v1,
// v weights v2); det > 0 is the front face (counter-clockwise seen from the ray).
RD bool TriTest(const RayPre& r, V3 v0, V3 v1, V3 v2, float& t, float& u, float& v, bool& front) {
  V3 A = v0 - r.O, B = v1 - r.O, C = v2 - r.O;
  float Akz = comp(A, r.kz), Bkz = comp(B, r.kz), Ckz = comp(C, r.kz);
  float Ax = comp(A, r.kx) - r.Sx * Akz, Ay = comp(A, r.ky) - r.Sy * Akz;
  float Bx = comp(B, r.kx) - r.Sx * Bkz, By = comp(B, r.ky) - r.Sy * Bkz;
  float Cx = comp(C, r.kx) - r.Sx * Ckz, Cy = comp(C, r.ky) - r.Sy * Ckz;
  float U = Cx * By - Cy * Bx;
  float V = Ax * Cy - Ay * Cx;
  float W = Bx * Ay - By * Ax;
  if (U == 0.f || V == 0.f || W == 0.f) {
    U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
    V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
    W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
  }
  if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return false;
  float det = U + V + W;
  if (det == 0.f) return false;
  float Az = r.Sz * Akz, Bz = r.Sz * Bkz, Cz = r.Sz * Ckz;
  float T = U * Az + V * Bz + W * Cz;
  t = T / det;
  u = V / det;
  v = W / det;
  front = det > 0.f;
  return true;
}

// rectangle.cpp:34-46 in the shape's object space (float32 world->object rows).
RD bool RectTest(const RayPre& r, const float4 m0, const float4 m1, const float4 m2, float& t, float& u, float& v,
                 bool& front, V3& nrmOut) {
  V3 O{((m0.x * r.O.x + m0.y * r.O.y) + m0.z * r.O.z) + m0.w, ((m1.x * r.O.x + m1.y * r.O.y) + m1.z * r.O.z) + m1.w,
       ((m2.x * r.O.x + m2.y * r.O.y) + m2.z * r.O.z) + m2.w};
  V3 D{(m0.x * r.D.x + m0.y * r.D.y) + m0.z * r.D.z, (m1.x * r.D.x + m1.y * r.D.y) + m1.z * r.D.z,
       (m2.x * r.D.x + m2.y * r.D.y) + m2.z * r.D.z};
  t = -O.z / D.z;
  V3 local = D * t + O;
  if (!(fabsf(local.x) <= 1.f && fabsf(local.y) <= 1.f)) return false;
  u = local.x;
  v = local.y;
  (void)nrmOut;
  front = D.z < 0.f;  // object-space normal is +z
  return true;
}

// sphere.cpp:40-54 with SolveQuadratic (math_ext.h:79-97).
RD bool SphereTest(const RayPre& r, float4 cr, float tfar, float& t, bool& front) {
  V3 c{cr.x, cr.y, cr.z};
  V3 o = r.O - c;
  float a = sqnorm(r.D);
  float b = 2.f * dot(o, r.D);
  float cc = sqnorm(o) - Sqr(cr.w);
  bool linearCase = a == 0.f;
  bool validLinear = linearCase && b != 0.f;
  float x0 = -cc / b, x1 = -cc / b;
  float discrim = b * b - 4.f * a * cc;
  bool validQuadratic = !linearCase && (discrim >= 0.f);
  if (validQuadratic) {
    float rootDiscrim = sqrtf(discrim);
    float temp = -0.5f * (b + copysignf(rootDiscrim, b));
    float x0p = temp / a;
    float x1p = cc / temp;
    float x0m = fminr(x0p, x1p);
    float x1m = fmaxr(x0p, x1p);
    x0 = linearCase ? x0 : x0m;
    x1 = linearCase ? x0 : x1m;
  }
  bool found = validLinear || validQuadratic;
  bool outBounds = !(x0 <= tfar && x1 >= r.tmin);
  bool inBounds = x0 < r.tmin && x1 > tfar;
  if (!(found && !outBounds && !inBounds)) return false;
  t = x0 < 0.f ? x1 : x0;
  V3 n = normalized((r.D * t + r.O) - c);
  front = dot(r.D, n) < 0.f;
  return true;
}

RD bool AcceptHit(float t, uint32_t prim, float tmin, float best, uint32_t bestPrim) {
  if (!(t > tmin)) return false;
  if (t < best) return true;
  return t == best && bestPrim != kNoPrim && prim < bestPrim;
}

struct TraceHit {
  float t, u, v;
  uint32_t prim, shape, front;
};

// Tests leaf-order primitive `lp`; updates `h` (closest) and returns true on an accepted hit.
RD bool TestPrim(const DevScene& S, const RayPre& r, uint32_t lp, bool analytic, TraceHit& h, bool anyMode) {
  const float4* pr = reinterpret_cast<const float4*>(S.prims) + 3 * (size_t)lp;
  float t, u = 0.f, v = 0.f;
  bool front;
  uint32_t gid, shape;
  if (!analytic) {
    float4 a = __ldg(pr), b = __ldg(pr + 1), c = __ldg(pr + 2);
    if (!TriTest(r, V3{a.x, a.y, a.z}, V3{b.x, b.y, b.z}, V3{c.x, c.y, c.z}, t, u, v, front)) return false;
    gid = __float_as_uint(a.w);
    shape = __float_as_uint(b.w);
  } else {
    uint2 info = __ldg(reinterpret_cast<const uint2*>(S.primInfo) + lp);
    gid = info.x;
    shape = info.y & 0x0fffffffu;
    uint32_t kind = info.y >> 28;
    if (kind == SHAPE_RECT) {
      V3 n;
      if (!RectTest(r, __ldg(pr), __ldg(pr + 1), __ldg(pr + 2), t, u, v, front, n)) return false;
    } else {
      if (!SphereTest(r, __ldg(pr), anyMode ? h.t : h.t, t, front)) return false;
    }
  }
  if (!AcceptHit(t, gid, r.tmin, h.t, h.prim)) return false;
  h.t = t;
  h.u = u;
  h.v = v;
  h.prim = gid;
  h.shape = shape;
  h.front = front ? 1u : 0u;
  return true;
}

RD uint32_t ByteOf(uint32_t w, uint32_t i) { return (w >> (8u * i)) & 0xffu; }
// Moves bit s of an 8-bit mask to bit s ^ oct (the octant's near-to-far order).
RD uint32_t XorPerm8(uint32_t x, uint32_t oct) {
  if (oct & 1u) x = ((x & 0x55u) << 1) | ((x >> 1) & 0x55u);
  if (oct & 2u) x = ((x & 0x33u) << 2) | ((x >> 2) & 0x33u);
  if (oct & 4u) x = ((x & 0x0fu) << 4) | ((x >> 4) & 0x0fu);
  return x;
}
// Byte i of w as a float, exactly: the byte becomes the low mantissa bits of
// 2^23 (one byte permute), and 2^23 is subtracted (one add) -- no conversion unit.
#if defined(RAD_HOST_EMULATION)
RD float ByteAsFloat(uint32_t w, uint32_t i) { return (float)ByteOf(w, i); }
#else
RD float ByteAsFloat(uint32_t w, uint32_t i) {
  return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u | i)) - 8388608.0f;
}
#endif

// Resumable traversal state: the node to visit next and the stack depth (the
// stack itself lives with the caller).
struct TravState {
  uint32_t node;
  int sp;
  uint32_t leafMask;         // leaf slots of the last visited node still to test
  uint32_t meta0, meta1;     // that node's meta bytes
  uint32_t primBase;
  bool last;                 // no node left after those leaves
};
constexpr int kTravContinue = 0, kTravDone = 1, kTravOverflow = 2;

// One node visit of the BVH8 traversal: tests the node's 8 child boxes, tests
// the primitives of the leaf children it hits, then picks the next node (the
// nearest internal child hit, else the stack top). Returns kTravDone when the
// ray is finished (or, for ANY, occluded), kTravOverflow if the stack would
// overflow (sets *err), else kTravContinue.
template <bool ANY, bool COUNT>
RD int TravStep(const DevScene& S, const RayPre& r, TraceHit& h, uint2* stack, TravState& st, uint32_t* err,
                uint32_t* nNodes, uint32_t* nPrims) {
  if (st.leafMask) {
    // one pending leaf of the last visited node (its primitives, 1..3)
    uint32_t s = __ffs(st.leafMask) - 1;
    st.leafMask &= st.leafMask - 1;
    uint32_t meta = ByteOf(s < 4 ? st.meta0 : st.meta1, s & 3u);
    uint32_t cnt = (meta >> 5) & 3u, off = meta & 31u;
    bool analytic = (meta >> 7) & 1u;
    for (uint32_t k = 0; k < cnt; k++) {
      if (COUNT) (*nPrims)++;
      if (TestPrim(S, r, st.primBase + off + k, analytic, h, ANY) && ANY) return kTravDone;
    }
    return (st.leafMask == 0u && st.last) ? kTravDone : kTravContinue;
  }
  const uint32_t nodeIdx = st.node;
  if (COUNT) (*nNodes)++;
  const uint4* np = reinterpret_cast<const uint4*>(S.nodes) + 5 * (size_t)nodeIdx;
  uint4 q0 = __ldg(np), q1 = __ldg(np + 1), q2 = __ldg(np + 2), q3 = __ldg(np + 3), q4 = __ldg(np + 4);
  float px = __uint_as_float(q0.x), py = __uint_as_float(q0.y), pz = __uint_as_float(q0.z);
  uint32_t ex = q0.w & 0xffu, ey = (q0.w >> 8) & 0xffu, ez = (q0.w >> 16) & 0xffu;
  uint32_t imask = q0.w >> 24;
  float ax = __uint_as_float(ex << 23) * r.inv.x, bx = (px - r.O.x) * r.inv.x;
  float ay = __uint_as_float(ey << 23) * r.inv.y, by = (py - r.O.y) * r.inv.y;
  float az = __uint_as_float(ez << 23) * r.inv.z, bz = (pz - r.O.z) * r.inv.z;
  // near/far quantised planes per axis by ray direction
  uint32_t nx0 = r.inv.x >= 0.f ? q2.x : q3.z, nx1 = r.inv.x >= 0.f ? q2.y : q3.w;
  uint32_t fx0 = r.inv.x >= 0.f ? q3.z : q2.x, fx1 = r.inv.x >= 0.f ? q3.w : q2.y;
  uint32_t ny0 = r.inv.y >= 0.f ? q2.z : q4.x, ny1 = r.inv.y >= 0.f ? q2.w : q4.y;
  uint32_t fy0 = r.inv.y >= 0.f ? q4.x : q2.z, fy1 = r.inv.y >= 0.f ? q4.y : q2.w;
  uint32_t nz0 = r.inv.z >= 0.f ? q3.x : q4.z, nz1 = r.inv.z >= 0.f ? q3.y : q4.w;
  uint32_t fz0 = r.inv.z >= 0.f ? q4.z : q3.x, fz1 = r.inv.z >= 0.f ? q4.w : q3.y;
  uint32_t childBase = q1.x, primBase = q1.y;
  float tcur = h.t;
  // all eight child boxes, one bit each in slot order (an empty slot holds an
  // inverted box, lo 255 / hi 0 on every axis, which no ray passes)
  uint32_t hits = 0;
#pragma unroll
  for (uint32_t s = 0; s < 8; s++) {
    uint32_t w = s < 4 ? 0u : 1u, i = s & 3u;
    float tnx = fmaf(ByteAsFloat(w ? nx1 : nx0, i), ax, bx);
    float tfx = fmaf(ByteAsFloat(w ? fx1 : fx0, i), ax, bx);
    float tny = fmaf(ByteAsFloat(w ? ny1 : ny0, i), ay, by);
    float tfy = fmaf(ByteAsFloat(w ? fy1 : fy0, i), ay, by);
    float tnz = fmaf(ByteAsFloat(w ? nz1 : nz0, i), az, bz);
    float tfz = fmaf(ByteAsFloat(w ? fz1 : fz0, i), az, bz);
    float tn = fmaxf(Max3(tnx, tny, tnz), r.tmin);
    float tf = fminf(Min3(tfx, tfy, tfz), tcur) * 1.00000024f;
    if (tn <= tf) hits |= 1u << s;
  }
  const uint32_t leafHits = hits & ~imask;              // bit slot
  uint32_t hitInternal = XorPerm8(hits & imask, r.oct);  // bit (slot ^ oct)
  // ---- leaves of this node: tested in the following steps, before the next
  // node visit (so the order of node visits and primitive tests is unchanged;
  // the next node below was chosen from the child boxes alone)
  st.leafMask = leafHits;
  st.meta0 = q1.z;
  st.meta1 = q1.w;
  st.primBase = primBase;
  // ---- next node
  if (hitInternal) {
    uint32_t b = __ffs(hitInternal) - 1;
    hitInternal &= hitInternal - 1;
    uint32_t s = b ^ r.oct;
    uint32_t child = childBase + __popc(imask & ((1u << s) - 1u));
    if (hitInternal) {
      if (st.sp >= kTraceStack) {
        if (err) atomicOr(err, 1u);
        return kTravOverflow;
      }
      stack[st.sp++] = make_uint2(childBase, (imask << 8) | hitInternal);
    }
    st.node = child;
    return kTravContinue;
  }
  if (st.sp == 0) {
    st.last = true;
    return st.leafMask ? kTravContinue : kTravDone;
  }
  uint2 g = stack[st.sp - 1];
  uint32_t m = g.y & 0xffu, im = g.y >> 8;
  uint32_t b = __ffs(m) - 1;
  m &= m - 1;
  uint32_t s = b ^ r.oct;
  st.node = g.x + __popc(im & ((1u << s) - 1u));
  if (m)
    stack[st.sp - 1].y = (im << 8) | m;
  else
    st.sp--;
  return kTravContinue;
}

RD void TraceInit(float tmax, TraceHit& h, TravState& st) {
  h.t = tmax;
  h.prim = kNoPrim;
  h.u = h.v = 0.f;
  h.shape = 0;
  h.front = 0;
  st.node = 0;
  st.sp = 0;
  st.leafMask = 0;
  st.last = false;
}

// Closest hit (ANY = false) or occlusion (ANY = true). Returns false and sets
// *err if the traversal stack would overflow (never silently truncates).
// COUNT = true also returns the number of nodes visited and primitives tested
// (for the roofline's algorithmic-bytes figure); the default build counts nothing.
template <bool ANY, bool COUNT = false>
RD bool TraceBvh8(const DevScene& S, const RayPre& r, float tmax, TraceHit& h, uint32_t* err,
                  uint32_t* nNodes = nullptr, uint32_t* nPrims = nullptr) {
  TravState st;
  TraceInit(tmax, h, st);
  if (S.nNodes == 0) return false;
  uint2 stack[kTraceStack];
  int res;
  while ((res = TravStep<ANY, COUNT>(S, r, h, stack, st, err, nNodes, nPrims)) == kTravContinue) {
  }
  if (res == kTravOverflow) return false;
  return h.prim != kNoPrim;
}

}  // namespace rad
