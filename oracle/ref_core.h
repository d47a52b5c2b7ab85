// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the RadiantiumPlusPlus `path` / `vol_path` hot path
// (module/rad.offline). Only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg may load or run anything under oracle/. The product library
// (radiantiumplusplus_gb300/) never includes, links or calls this code.
//
// Parity status: the reference cannot be compiled here (Embree 3, oneTBB,
// Eigen, spdlog, nlohmann-json are absent) and ships no tests, fixtures or
// golden images, so this restatement is "parity unpinned" against the
// reference's own outputs. It is pinned instead by analytic known-answer tests
// (tests/test_oracle_*.py): Fresnel closed forms, microfacet normalisation,
// BSDF sample/pdf consistency, white-furnace energy bounds, and by the
// committed golden fixtures under tests/golden/ generated from it.
//
// Arithmetic is scalar FP32 (the reference builds with RAD_FLOAT_32_WEIGHT,
// module/rad.offline/CMakeLists.txt:4,76-82), compiled with
// -ffp-contract=off so that every fused multiply-add is the explicit
// std::fma the reference writes as Math::Fmadd (rad.core math_base.h:68).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace orc {

using Float = float;

// ---------------------------------------------------------------------------
// Small fixed-size vectors. Reductions are evaluated left to right, as the
// reference's Eigen fixed-size-3 expressions unroll: dot = (x*x' + y*y') + z*z'.
// ---------------------------------------------------------------------------
struct V2 {
  Float x = 0, y = 0;
  V2() = default;
  V2(Float a, Float b) : x(a), y(b) {}
  Float operator[](int i) const { return i == 0 ? x : y; }
  Float& operator[](int i) { return i == 0 ? x : y; }
};

struct V3 {
  Float x = 0, y = 0, z = 0;
  V3() = default;
  V3(Float a, Float b, Float c) : x(a), y(b), z(c) {}
  explicit V3(Float a) : x(a), y(a), z(a) {}
  Float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  Float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};

inline V3 operator+(const V3& a, const V3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(const V3& a, const V3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(const V3& a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(const V3& a, Float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(Float s, const V3& a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator/(const V3& a, Float s) { return {a.x / s, a.y / s, a.z / s}; }
inline V3 cmul(const V3& a, const V3& b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 cdiv(const V3& a, const V3& b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline Float dot(const V3& a, const V3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline V3 cross(const V3& a, const V3& b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline Float sqnorm(const V3& a) { return dot(a, a); }
inline Float norm(const V3& a) { return std::sqrt(sqnorm(a)); }
// Eigen normalized(): zero vector is returned unchanged, otherwise v / sqrt(|v|^2).
inline V3 normalized(const V3& a) {
  Float n = sqnorm(a);
  if (n > 0) {
    Float s = std::sqrt(n);
    return {a.x / s, a.y / s, a.z / s};
  }
  return a;
}
inline bool is_zero(const V3& a) { return a.x == 0 && a.y == 0 && a.z == 0; }
inline Float max_comp(const V3& a) {
  // Eigen maxCoeff reduction: (a < b) ? b : a, left to right.
  Float m = a.x;
  m = (m < a.y) ? a.y : m;
  m = (m < a.z) ? a.z : m;
  return m;
}
inline Float min_comp(const V3& a) {
  Float m = a.x;
  m = (a.y < m) ? a.y : m;
  m = (a.z < m) ? a.z : m;
  return m;
}
inline V3 vmin(const V3& a, const V3& b) {  // std::min per component
  return {(b.x < a.x) ? b.x : a.x, (b.y < a.y) ? b.y : a.y, (b.z < a.z) ? b.z : a.z};
}
inline V3 vmax(const V3& a, const V3& b) {  // std::max per component
  return {(a.x < b.x) ? b.x : a.x, (a.y < b.y) ? b.y : a.y, (a.z < b.z) ? b.z : a.z};
}

using Spectrum = V3;

// ---------------------------------------------------------------------------
// Scalar helpers: rad.core/include/rad/core/math_base.h:36-105 and
// rad.offline/include/rad/offline/math_ext.h:8-142.
// ---------------------------------------------------------------------------
constexpr Float PI = static_cast<Float>(3.1415926535897932);
constexpr Float Float32Epsilon = 0x1p-24f;
constexpr Float RayEpsilon = Float32Epsilon * Float(1500);     // math_ext.h:12
constexpr Float ShadowEpsilon = RayEpsilon * Float(10);        // math_ext.h:16
constexpr Float OneMinusEpsilon = 0x1.fffffep-1f;              // math_ext.h:18

inline Float Sqr(Float v) { return v * v; }
inline Float Sign(Float v) { return v >= 0 ? Float(1) : Float(-1); }
inline Float MulSign(Float a, Float b) { return b >= 0 ? a : -a; }
inline V3 MulSign(const V3& a, Float b) { return b >= 0 ? a : -a; }
inline Float Rcp(Float v) { return Float(1) / v; }
inline Float Rsqrt(Float v) { return Rcp(std::sqrt(v)); }
inline Float Fmadd(Float a, Float b, Float c) { return std::fma(a, b, c); }
inline V3 Fmadd(const V3& a, const V3& b, const V3& c) {
  return {Fmadd(a.x, b.x, c.x), Fmadd(a.y, b.y, c.y), Fmadd(a.z, b.z, c.z)};
}
inline Float SafeSqrt(Float v) { return std::sqrt(v > 0 ? v : Float(0)); }
inline Float AbsDot(const V3& a, const V3& b) { return std::abs(dot(a, b)); }
inline Float Lerp(Float a, Float b, Float t) { return Fmadd(b, t, Fmadd(-a, t, a)); }
inline Float Radian(Float deg) { return deg * (PI / Float(180)); }
inline Float Luminance(const V3& c) {  // spectrum.h:38-40
  return (c.x * Float(0.212671)) + (c.y * Float(0.715160)) + (c.z * Float(0.072169));
}

// math_ext.h:48-61
inline std::pair<V3, V3> CoordinateSystem(const V3& n) {
  Float sign = Sign(n.z);
  Float a = -1 / (sign + n.z);
  Float b = n.x * n.y * a;
  V3 X(MulSign(Sqr(n.x) * a, n.z) + 1.0f, MulSign(b, n.z), MulSign(n.x, -n.z));
  V3 Y(b, sign + Sqr(n.y) * a, -n.y);
  return {X, Y};
}

// math_ext.h:79-97
inline void SolveQuadratic(Float a, Float b, Float c, bool& found, Float& x0, Float& x1) {
  bool linearCase = a == 0.0f;
  bool validLinear = linearCase && b != 0.0f;
  x0 = -c / b;
  x1 = -c / b;
  Float discrim = b * b - Float(4) * a * c;
  bool validQuadratic = !linearCase && (discrim >= 0.0f);
  if (validQuadratic) {
    Float rootDiscrim = std::sqrt(discrim);
    Float temp = Float(-0.5) * (b + std::copysign(rootDiscrim, b));
    Float x0p = temp / a;
    Float x1p = c / temp;
    Float x0m = std::min(x0p, x1p);
    Float x1m = std::max(x0p, x1p);
    x0 = linearCase ? x0 : x0m;
    x1 = linearCase ? x0 : x1m;
  }
  found = validLinear || validQuadratic;
}

// math_ext.h:101-104
inline Float UnitAngleZ(const V3& v) {
  Float temp = std::asin(Float(0.5) * norm(V3(v.x, v.y, v.z - MulSign(Float(1), v.z)))) * 2;
  return v.z >= 0 ? temp : PI - temp;
}

// ---------------------------------------------------------------------------
// Frame: rad.offline/src/frame.cpp:9-72
// ---------------------------------------------------------------------------
struct Frame {
  V3 S, T, N;
  Frame() = default;
  explicit Frame(const V3& n) {
    auto st = CoordinateSystem(n);
    S = st.first;
    T = st.second;
    N = n;
  }
  Frame(const V3& s, const V3& t, const V3& n) : S(s), T(t), N(n) {}
  // frame.cpp:19-21: N * v.z + (T * v.y + (S * v.x))
  V3 ToWorld(const V3& v) const { return N * v.z + (T * v.y + (S * v.x)); }
  V3 ToLocal(const V3& v) const { return V3(dot(v, S), dot(v, T), dot(v, N)); }

  static Float CosTheta(const V3& v) { return v.z; }
  static Float AbsCosTheta(const V3& v) { return std::abs(v.z); }
  static Float Sin2Theta(const V3& v) { return Fmadd(v.x, v.x, Sqr(v.y)); }
  static bool IsSameHemisphere(const V3& x, const V3& y) { return CosTheta(x) * CosTheta(y) > 0; }
  // frame.cpp:48-56. The reference clamps with cwiseMin(-1).cwiseMax(1), which
  // yields (1, 1) for every vector away from the pole; kept as written.
  static void SinCosPhi(const V3& v, Float& sinPhi, Float& cosPhi) {
    Float sin2Theta = Sin2Theta(v);
    Float invSinTheta = Rsqrt(Sin2Theta(v));
    Float rx = v.x * invSinTheta, ry = v.y * invSinTheta;
    if (std::abs(sin2Theta) <= 4 * Float32Epsilon) {
      rx = 1;
      ry = 0;
    } else {
      rx = (Float(-1) < rx) ? Float(-1) : rx;  // std::min(rx, -1)
      ry = (Float(-1) < ry) ? Float(-1) : ry;
      rx = (rx < Float(1)) ? Float(1) : rx;    // std::max(rx, 1)
      ry = (ry < Float(1)) ? Float(1) : ry;
    }
    sinPhi = ry;
    cosPhi = rx;
  }
};

// ---------------------------------------------------------------------------
// 4x4 affine/projective transform: rad.offline/src/transform.cpp:5-95.
// Matrix-vector products are row dots evaluated ((m0 v0 + m1 v1) + m2 v2) + m3 v3.
// The inverse is computed in double and rounded to float.
// ---------------------------------------------------------------------------
struct M4 {
  Float m[4][4];
  static M4 Identity() {
    M4 r{};
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 4; j++) r.m[i][j] = (i == j) ? 1.f : 0.f;
    return r;
  }
  M4 operator*(const M4& b) const {
    M4 r{};
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 4; j++) {
        Float s = m[i][0] * b.m[0][j];
        s = s + m[i][1] * b.m[1][j];
        s = s + m[i][2] * b.m[2][j];
        s = s + m[i][3] * b.m[3][j];
        r.m[i][j] = s;
      }
    return r;
  }
};

bool InvertM4(const M4& a, M4& out);

struct Transform {
  M4 ToWorld = M4::Identity();
  M4 ToLocal = M4::Identity();
  Transform() = default;
  explicit Transform(const M4& toWorld) : ToWorld(toWorld) {
    if (!InvertM4(toWorld, ToLocal)) throw std::runtime_error("matrix is not invertible");
  }
  static V3 Affine(const M4& M, const V3& v) {
    Float r[4];
    for (int i = 0; i < 4; i++) r[i] = ((M.m[i][0] * v.x + M.m[i][1] * v.y) + M.m[i][2] * v.z) + M.m[i][3];
    return V3(r[0] / r[3], r[1] / r[3], r[2] / r[3]);
  }
  static V3 Linear(const M4& M, const V3& v) {
    return V3((M.m[0][0] * v.x + M.m[0][1] * v.y) + M.m[0][2] * v.z,
              (M.m[1][0] * v.x + M.m[1][1] * v.y) + M.m[1][2] * v.z,
              (M.m[2][0] * v.x + M.m[2][1] * v.y) + M.m[2][2] * v.z);
  }
  V3 ApplyAffineToWorld(const V3& v) const { return Affine(ToWorld, v); }
  V3 ApplyAffineToLocal(const V3& v) const { return Affine(ToLocal, v); }
  V3 ApplyLinearToWorld(const V3& v) const { return Linear(ToWorld, v); }
  V3 ApplyLinearToLocal(const V3& v) const { return Linear(ToLocal, v); }
  // transform.cpp:63-65: ToLocal.linear().transpose() * v
  V3 ApplyNormalToWorld(const V3& v) const {
    const M4& M = ToLocal;
    return V3((M.m[0][0] * v.x + M.m[1][0] * v.y) + M.m[2][0] * v.z,
              (M.m[0][1] * v.x + M.m[1][1] * v.y) + M.m[2][1] * v.z,
              (M.m[0][2] * v.x + M.m[1][2] * v.y) + M.m[2][2] * v.z);
  }
  V3 TranslationToWorld() const { return V3(ToWorld.m[0][3], ToWorld.m[1][3], ToWorld.m[2][3]); }
  bool IsIdentity() const {
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 4; j++)
        if (ToWorld.m[i][j] != ((i == j) ? 1.f : 0.f)) return false;
    return true;
  }
  bool HasNonUniformScale() const {  // transform.cpp:39-44
    Float la2 = sqnorm(ApplyLinearToWorld(V3(1, 0, 0)));
    Float lb2 = sqnorm(ApplyLinearToWorld(V3(0, 1, 0)));
    Float lc2 = sqnorm(ApplyLinearToWorld(V3(0, 0, 1)));
    return std::abs(la2 - lb2) > 0.0001f || std::abs(la2 - lc2) > 0.0001f;
  }
};

// ---------------------------------------------------------------------------
// Minimal JSON DOM (the reference parses scenes with nlohmann-json).
// ---------------------------------------------------------------------------
struct Json {
  enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
  bool b = false;
  double num = 0;
  std::string str;
  std::vector<Json> arr;
  std::vector<std::pair<std::string, Json>> obj;

  const Json* find(const std::string& k) const {
    if (kind != Object) return nullptr;
    for (auto& kv : obj)
      if (kv.first == k) return &kv.second;
    return nullptr;
  }
  bool has(const std::string& k) const { return find(k) != nullptr; }
  bool is_number() const { return kind == Number; }
  bool is_array() const { return kind == Array; }
  bool is_object() const { return kind == Object; }
  static Json parse(const std::string& text);
  static Json Num(double v) {
    Json j;
    j.kind = Number;
    j.num = v;
    return j;
  }
};

// ConfigNode helpers: rad.core/include/rad/core/config_node.h:10-170
Float JNum(const Json& j);
V3 JVec3(const Json& j);
Float ReadF(const Json* cfg, const std::string& k, Float def);
int ReadI(const Json* cfg, const std::string& k, int def);
bool ReadB(const Json* cfg, const std::string& k, bool def);
std::string ReadS(const Json* cfg, const std::string& k, const std::string& def);
V3 ReadV3(const Json* cfg, const std::string& k, const V3& def);
M4 JsonAsTransform(const Json& node);  // config_node_ext.cpp:52-71

// ---------------------------------------------------------------------------
// PCG32 per-sample stream (the sampler shared by the GPU path and this oracle;
// the reference's `independent` sampler draws from std::mt19937 per TBB tile,
// independent.cpp:13-52, so image parity with it is statistical only).
// ---------------------------------------------------------------------------
inline uint64_t SplitMix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ULL;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}
struct Pcg32 {
  static constexpr uint64_t kMul = 6364136223846793005ULL;
  static constexpr uint64_t kInc = 1442695040888963407ULL;
  uint64_t state = 0;
  static Pcg32 ForSample(uint32_t pixel, uint32_t sample, uint32_t seed) {
    Pcg32 r;
    uint64_t init = SplitMix64(SplitMix64(seed) ^ ((uint64_t(pixel) << 32) | uint64_t(sample)));
    r.state = 0;
    r.NextU32();
    r.state += init;
    r.NextU32();
    return r;
  }
  uint32_t NextU32() {
    uint64_t old = state;
    state = old * kMul + kInc;
    uint32_t xs = uint32_t(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = uint32_t(old >> 59u);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
  }
  Float Next1D() { return Float(NextU32() >> 8) * 0x1p-24f; }
  V2 Next2D() {
    Float a = Next1D();
    Float b = Next1D();
    return V2(a, b);
  }
};

}  // namespace orc
