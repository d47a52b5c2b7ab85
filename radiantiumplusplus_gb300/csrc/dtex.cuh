// Device textures: constant, bitmap (nearest / bilinear / trilinear /
// anisotropic EWA over the mip chain, bitmap.cpp:66-261) and chessboard
// (chessboard.cpp:36-58), and the per-lookup resolution of textured BSDF
// parameters into a material record. FP32 in the reference's expression order.
#pragma once
#include "dmath.cuh"

namespace rad {

// What a texture lookup reads: the scene's texture tables and the surface
// point's uv with its screen-space derivatives (zero without ray differentials).
struct TexCtx {
  const TexRec* tex;
  const float* texels;
  const TexBind* binds;
  V2 uv, duvdx, duvdy;
};

// MipMap::Wrap (bitmap.cpp:149-157)
RD float TexWrap(float v, uint32_t wrap) {
  return wrap ? clampr(v - floorf(v), 0.f, 1.f) : clampr(v, 0.f, 1.f);
}
RD uint32_t LevelDim(uint32_t d, uint32_t l) { return (d >> l) > 1u ? (d >> l) : 1u; }

struct TexVal {
  float c[3];
};

RD TexVal Texel(const TexCtx& x, const TexRec& t, uint32_t level, uint32_t W, uint32_t px, uint32_t py) {
  const float* p = x.texels + t.levelOffset[level] + ((size_t)py * W + px) * t.channels;
  TexVal v;
  v.c[0] = p[0];
  v.c[1] = t.channels == 3u ? p[1] : 0.f;
  v.c[2] = t.channels == 3u ? p[2] : 0.f;
  return v;
}

// Continuous texel coordinate of a wrapped uv (bitmap.cpp:181-187, 190-197).
// A uv that is NaN, which the reference converts to an unsigned index with
// undefined result, reads texel 0 here.
RD void TexCoord(float u01, uint32_t n, float& f, uint32_t& p) {
  f = u01 * (float)(n - 1u);
  p = f >= 0.f ? (uint32_t)f : 0u;
  if (p > n - 1u) p = n - 1u;
}

// FilterNearest (bitmap.cpp:179-188)
RD TexVal TexNearest(const TexCtx& x, const TexRec& t, uint32_t level, V2 uv) {
  uint32_t W = LevelDim(t.width, level), H = LevelDim(t.height, level);
  float fu, fv;
  uint32_t pu, pv;
  TexCoord(TexWrap(uv.x, t.wrap), W, fu, pu);
  TexCoord(TexWrap(uv.y, t.wrap), H, fv, pv);
  return Texel(x, t, level, W, pu, pv);
}

// FilterBilinear (bitmap.cpp:190-214). The neighbour index is pu +/- 1 in
// unsigned arithmetic clamped to the last texel, so at pu = 0 the "left"
// neighbour is the last column, as in the reference.
RD TexVal TexBilinear(const TexCtx& x, const TexRec& t, uint32_t level, V2 uv) {
  uint32_t W = LevelDim(t.width, level), H = LevelDim(t.height, level);
  float fu, fv;
  uint32_t pu, pv;
  TexCoord(TexWrap(uv.x, t.wrap), W, fu, pu);
  TexCoord(TexWrap(uv.y, t.wrap), H, fv, pv);
  int32_t dpu = (fu > (float)pu + 0.5f) ? 1 : -1;
  int32_t dpv = (fv > (float)pv + 0.5f) ? 1 : -1;
  uint32_t apu = pu + (uint32_t)dpu, apv = pv + (uint32_t)dpv;
  apu = apu < W - 1u ? apu : W - 1u;
  apv = apv < H - 1u ? apv : H - 1u;
  float du = fminr(fabsf(fu - (float)pu - 0.5f), 1.f);
  float dv = fminr(fabsf(fv - (float)pv - 0.5f), 1.f);
  TexVal a = Texel(x, t, level, W, pu, pv), b = Texel(x, t, level, W, apu, pv);
  TexVal c = Texel(x, t, level, W, pu, apv), d = Texel(x, t, level, W, apu, apv);
  TexVal r;
  for (int k = 0; k < 3; k++)
    r.c[k] = (a.c[k] * (1.f - du) + b.c[k] * du) * (1.f - dv) + (c.c[k] * (1.f - du) + d.c[k] * du) * dv;
  return r;
}

RD TexVal TexLerp(TexVal lo, TexVal hi, float w) {
  TexVal r;
  for (int k = 0; k < 3; k++) r.c[k] = lo.c[k] * (1.f - w) + (hi.c[k] * w);
  return r;
}

// EvalEWA (bitmap.cpp:222-258). The loop visits the texels of `level` inside the
// ellipse but reads them through EvalNearest, i.e. from level 0, as the
// reference does. The texel box is capped at 4096 x 4096 (reached only for
// non-finite derivatives; the reference has no bound).
RD TexVal TexEWA(const TexCtx& x, const TexRec& t, uint32_t level, V2 uv, V2 dst0_, V2 dst1_) {
  uint32_t W = LevelDim(t.width, level), H = LevelDim(t.height, level);
  V2 st{uv.x * (float)W, uv.y * (float)H};
  V2 dst0{dst0_.x * (float)W, dst0_.y * (float)H};
  V2 dst1{dst1_.x * (float)W, dst1_.y * (float)H};
  float A = dst0.y * dst0.y + dst1.y * dst1.y + 1.f;
  float B = -2.f * (dst0.x * dst0.y + dst1.x * dst1.y);
  float C = dst0.x * dst0.x + dst1.x * dst1.x + 1.f;
  float invF = 1.f / (A * C - B * B * 0.25f);
  A *= invF;
  B *= invF;
  C *= invF;
  float det = -B * B + 4.f * A * C;
  float invDet = 1.f / det;
  float uSqrt = sqrtf(det * C), vSqrt = sqrtf(det * A);
  float fs0 = ceilf(st.x - 2.f * invDet * uSqrt), fs1 = floorf(st.x + 2.f * invDet * uSqrt);
  float ft0 = ceilf(st.y - 2.f * invDet * vSqrt), ft1 = floorf(st.y + 2.f * invDet * vSqrt);
  TexVal sum{{0.f, 0.f, 0.f}};
  float sumWts = 0.f;
  if (fs0 >= -1e9f && fs1 <= 1e9f && ft0 >= -1e9f && ft1 <= 1e9f) {
    int s0 = (int)fs0, s1 = (int)fs1, t0 = (int)ft0, t1 = (int)ft1;
    if (s1 - s0 > 4095) s1 = s0 + 4095;
    if (t1 - t0 > 4095) t1 = t0 + 4095;
    V2 invR{1.f / (float)W, 1.f / (float)H};
    const float e2 = expf(-2.f);
    for (int it = t0; it <= t1; ++it) {
      float tt = (float)it - st.y;
      for (int is = s0; is <= s1; ++is) {
        float ss = (float)is - st.x;
        float r2 = A * ss * ss + B * ss * tt + C * tt * tt;
        if (r2 < 1.f) {
          float weight = expf(-2.f * r2) - e2;
          TexVal v = TexNearest(x, t, 0u, V2{(float)is * invR.x, (float)it * invR.y});
          for (int k = 0; k < 3; k++) sum.c[k] = sum.c[k] + v.c[k] * weight;
          sumWts += weight;
        }
      }
    }
  }
  TexVal r;
  for (int k = 0; k < 3; k++) r.c[k] = sum.c[k] / sumWts;
  return r;
}

RD float SqNorm2(V2 a) { return a.x * a.x + a.y * a.y; }

// MipMap::EvalTrilinear (bitmap.cpp:78-101); EvalIsotropic always filters bilinearly.
RD TexVal TexTrilinear(const TexCtx& x, const TexRec& t, V2 uv) {
  float a = SqNorm2(x.duvdx), b = SqNorm2(x.duvdy);
  float width = sqrtf(fmaxr(a, b));
  float level = (float)(t.levels - 1u) + log2f(fmaxr(width, 1e-8f));
  if (level < 0.f) return TexBilinear(x, t, 0u, uv);
  if (level >= (float)(t.levels - 1u)) return TexBilinear(x, t, t.levels - 1u, uv);
  uint32_t down = (uint32_t)floorf(level);
  float weight = level - (float)down;
  return TexLerp(TexBilinear(x, t, down, uv), TexBilinear(x, t, down + 1u, uv), weight);
}

// MipMap::EvalAnisotropic (bitmap.cpp:106-145)
RD TexVal TexAniso(const TexCtx& x, const TexRec& t, V2 uv) {
  float a = SqNorm2(x.duvdx), b = SqNorm2(x.duvdy);
  float big = sqrtf(fmaxr(a, b));
  float small = sqrtf(fminr(a, b));
  V2 bigduv = a < b ? x.duvdy : x.duvdx;
  V2 smallduv = a < b ? x.duvdx : x.duvdy;
  if ((small * t.aniso < big) && (small > 0.f)) {
    float scale = big / (small * t.aniso);
    smallduv = V2{smallduv.x * scale, smallduv.y * scale};
    small *= scale;
  }
  if (small == 0.f) return TexBilinear(x, t, 0u, uv);
  float level = (float)(t.levels - 1u) + log2f(fmaxr(small, 1e-8f));
  if (level < 0.f) return TexEWA(x, t, 0u, uv, bigduv, smallduv);
  if (level >= (float)(t.levels - 1u)) return TexBilinear(x, t, t.levels - 1u, uv);
  uint32_t down = (uint32_t)floorf(level);
  float weight = level - (float)down;
  TexVal low = TexEWA(x, t, down, uv, bigduv, smallduv);
  TexVal high{{0.f, 0.f, 0.f}};
  if (weight != 0.f) high = TexEWA(x, t, down + 1u, uv, bigduv, smallduv);
  return TexLerp(low, high, weight);
}

// Texture<T>::Eval (texture.h:57-62) through chessboard chains.
RD TexVal TexEval(const TexCtx& x, uint32_t id, V2 uv) {
  for (int lvl = 0; lvl <= kMaxTexNest; lvl++) {
    const TexRec& t = x.tex[id];
    if (t.kind == TEX_CONST) return TexVal{{t.value[0], t.value[1], t.value[2]}};
    if (t.kind == TEX_BITMAP) {
      switch (t.filter) {
        case TF_NEAREST: return TexNearest(x, t, 0u, uv);
        case TF_TRILINEAR: return TexTrilinear(x, t, uv);
        case TF_ANISO: return TexAniso(x, t, uv);
        default: return TexBilinear(x, t, 0u, uv);
      }
    }
    // chessboard.cpp:36-58
    V3 tp = Affine4(t.toUV, V3{uv.x, uv.y, 0.f});
    V2 tuv{tp.x, tp.y};
    V2 ab{tuv.x - floorf(tuv.x), tuv.y - floorf(tuv.y)};
    bool isRight = ab.x > 0.5f, isUp = ab.y > 0.5f;
    if (isRight == isUp) {
      if (t.remap) uv = V2{(tuv.x - 0.5f) * 2.f, (tuv.y - 0.5f) * 2.f};
      id = t.childA;
    } else {
      if (t.remap) uv = V2{tuv.x * 2.f, tuv.y * 2.f};
      id = t.childB;
    }
  }
  return TexVal{{0.f, 0.f, 0.f}};  // deeper than the host allows
}

// The record with its textured parameters looked up at the context's uv
// (records without textured parameters are returned as they are).
RD const MatRec& TexturedMat(const MatRec& m, const TexCtx* x, MatRec& tmp) {
  if (m.texCount == 0u || x == nullptr) return m;
  tmp = m;
  for (uint32_t k = 0; k < m.texCount; k++) {
    TexBind b = x->binds[m.texFirst + k];
    TexVal v = TexEval(*x, b.tex, x->uv);
    for (uint32_t c = 0; c < b.channels; c++) tmp.p[b.slot + c] = b.clamp01 ? clampr(v.c[c], 0.f, 1.f) : v.c[c];
  }
  return tmp;
}

}  // namespace rad
