// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_core.h).
#include "ref_scene.h"

#include <algorithm>
#include <cstdio>
#include <deque>
#include <fstream>
#include <sstream>

namespace orc {

// =============================================================== JSON
namespace {
struct JParser {
  const std::string& s;
  size_t i = 0;
  explicit JParser(const std::string& t) : s(t) {}
  void ws() {
    while (i < s.size() && (s[i] == ' ' || s[i] == '\n' || s[i] == '\r' || s[i] == '\t')) i++;
  }
  [[noreturn]] void fail(const char* m) {
    throw std::runtime_error(std::string("json: ") + m + " at offset " + std::to_string(i));
  }
  Json value() {
    ws();
    if (i >= s.size()) fail("unexpected end");
    char c = s[i];
    Json j;
    if (c == '{') {
      j.kind = Json::Object;
      i++;
      ws();
      if (i < s.size() && s[i] == '}') { i++; return j; }
      for (;;) {
        ws();
        if (i >= s.size() || s[i] != '"') fail("expected key");
        std::string k = str();
        ws();
        if (i >= s.size() || s[i] != ':') fail("expected ':'");
        i++;
        Json v = value();
        j.obj.emplace_back(std::move(k), std::move(v));
        ws();
        if (i < s.size() && s[i] == ',') { i++; continue; }
        if (i < s.size() && s[i] == '}') { i++; break; }
        fail("expected ',' or '}'");
      }
    } else if (c == '[') {
      j.kind = Json::Array;
      i++;
      ws();
      if (i < s.size() && s[i] == ']') { i++; return j; }
      for (;;) {
        j.arr.push_back(value());
        ws();
        if (i < s.size() && s[i] == ',') { i++; continue; }
        if (i < s.size() && s[i] == ']') { i++; break; }
        fail("expected ',' or ']'");
      }
    } else if (c == '"') {
      j.kind = Json::String;
      j.str = str();
    } else if (s.compare(i, 4, "true") == 0) {
      j.kind = Json::Bool; j.b = true; i += 4;
    } else if (s.compare(i, 5, "false") == 0) {
      j.kind = Json::Bool; j.b = false; i += 5;
    } else if (s.compare(i, 4, "null") == 0) {
      i += 4;
    } else {
      j.kind = Json::Number;
      const char* b = s.c_str() + i;
      char* e = nullptr;
      j.num = std::strtod(b, &e);
      if (e == b) fail("bad number");
      i += size_t(e - b);
    }
    return j;
  }
  std::string str() {
    std::string out;
    i++;  // opening quote
    while (i < s.size() && s[i] != '"') {
      if (s[i] == '\\' && i + 1 < s.size()) {
        char e = s[i + 1];
        out.push_back(e == 'n' ? '\n' : e == 't' ? '\t' : e);
        i += 2;
      } else {
        out.push_back(s[i++]);
      }
    }
    if (i >= s.size()) fail("unterminated string");
    i++;
    return out;
  }
};
}  // namespace

Json Json::parse(const std::string& text) {
  JParser p(text);
  Json j = p.value();
  p.ws();
  if (p.i != text.size()) p.fail("trailing data");
  return j;
}

Float JNum(const Json& j) {
  if (!j.is_number()) throw std::runtime_error("node type is not number");
  return (Float)j.num;
}
V3 JVec3(const Json& j) {  // config_node.h:12-33: array of 3 or a broadcast number
  if (j.is_number()) return V3((Float)j.num);
  if (!j.is_array() || j.arr.size() != 3) throw std::runtime_error("node array size must be 3");
  return V3(JNum(j.arr[0]), JNum(j.arr[1]), JNum(j.arr[2]));
}
Float ReadF(const Json* c, const std::string& k, Float d) {
  const Json* j = c ? c->find(k) : nullptr;
  return j ? JNum(*j) : d;
}
int ReadI(const Json* c, const std::string& k, int d) {
  const Json* j = c ? c->find(k) : nullptr;
  return j ? (int)JNum(*j) : d;
}
bool ReadB(const Json* c, const std::string& k, bool d) {
  const Json* j = c ? c->find(k) : nullptr;
  if (!j) return d;
  if (j->kind != Json::Bool) throw std::runtime_error("node type is not bool");
  return j->b;
}
std::string ReadS(const Json* c, const std::string& k, const std::string& d) {
  const Json* j = c ? c->find(k) : nullptr;
  if (!j) return d;
  if (j->kind != Json::String) throw std::runtime_error("node type is not string");
  return j->str;
}
V3 ReadV3(const Json* c, const std::string& k, const V3& d) {
  const Json* j = c ? c->find(k) : nullptr;
  return j ? JVec3(*j) : d;
}

// Inverse via cofactors in double, rounded to float.
bool InvertM4(const M4& a, M4& out) {
  double m[16], inv[16];
  for (int i = 0; i < 16; i++) m[i] = a.m[i / 4][i % 4];
  inv[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] + m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
  inv[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] - m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
  inv[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] + m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
  inv[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] - m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
  inv[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] - m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
  inv[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] + m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
  inv[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] - m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
  inv[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] + m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
  inv[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] + m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
  inv[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] - m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
  inv[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] + m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
  inv[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] - m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
  inv[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] - m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
  inv[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] + m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
  inv[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] - m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
  inv[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] + m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
  double det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
  if (det == 0 || !std::isfinite(det)) return false;
  for (int i = 0; i < 16; i++) out.m[i / 4][i % 4] = (Float)(inv[i] / det);
  return true;
}

// config_node_ext.cpp:7-27: Rodrigues rotation of `angle` degrees about `axis`
// (the axis is used as given), or a 9-number matrix, or an (x,y,z,w) quaternion.
static void JsonAsRotate(const Json& n, Float R[3][3]) {
  if (n.is_object()) {
    V3 axis = ReadV3(&n, "axis", V3(0, 1, 0));
    Float ang = Radian(ReadF(&n, "angle", 0));
    Float s = std::sin(ang), c = std::cos(ang);
    V3 sa = axis * s;
    V3 c1 = axis * (Float(1) - c);
    Float tmp;
    tmp = c1.x * axis.y; R[0][1] = tmp - sa.z; R[1][0] = tmp + sa.z;
    tmp = c1.x * axis.z; R[0][2] = tmp + sa.y; R[2][0] = tmp - sa.y;
    tmp = c1.y * axis.z; R[1][2] = tmp - sa.x; R[2][1] = tmp + sa.x;
    R[0][0] = c1.x * axis.x + c;
    R[1][1] = c1.y * axis.y + c;
    R[2][2] = c1.z * axis.z + c;
  } else if (n.is_array() && n.arr.size() == 9) {
    for (int k = 0; k < 9; k++) R[k / 3][k % 3] = JNum(n.arr[k]);
  } else if (n.is_array() && n.arr.size() == 4) {
    Float x = JNum(n.arr[0]), y = JNum(n.arr[1]), z = JNum(n.arr[2]), w = JNum(n.arr[3]);
    Float tx = 2 * x, ty = 2 * y, tz = 2 * z;
    Float twx = tx * w, twy = ty * w, twz = tz * w, txx = tx * x, txy = ty * x, txz = tz * x;
    Float tyy = ty * y, tyz = tz * y, tzz = tz * z;
    R[0][0] = 1 - (tyy + tzz); R[0][1] = txy - twz; R[0][2] = txz + twy;
    R[1][0] = txy + twz; R[1][1] = 1 - (txx + tzz); R[1][2] = tyz - twx;
    R[2][0] = txz - twy; R[2][1] = tyz + twx; R[2][2] = 1 - (txx + tyy);
  } else {
    throw std::runtime_error("rotate node must be array or object");
  }
}

// config_node_ext.cpp:52-71: 16-number row-major matrix, or translate * rotate * scale.
M4 JsonAsTransform(const Json& node) {
  M4 r = M4::Identity();
  if (node.is_array()) {
    if (node.arr.size() != 16) throw std::runtime_error("node array size must be 16");
    for (int k = 0; k < 16; k++) r.m[k / 4][k % 4] = JNum(node.arr[k]);
    return r;
  }
  if (!node.is_object()) throw std::runtime_error("transform node must be mat4 or object");
  V3 t = ReadV3(&node, "translate", V3(0, 0, 0));
  V3 s = ReadV3(&node, "scale", V3(1, 1, 1));
  Float R[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  if (const Json* rn = node.find("rotate")) JsonAsRotate(*rn, R);
  for (int i = 0; i < 3; i++) {
    for (int j = 0; j < 3; j++) r.m[i][j] = R[i][j] * s[j];
    r.m[i][3] = t[i];
  }
  return r;
}

// ======================================================= distribution
void Discrete1D::Build(const std::vector<Float>& data) {
  pmf = data;
  cdf.resize(data.size());
  double s = 0;
  for (size_t i = 0; i < data.size(); i++) {
    s += (double)data[i];
    cdf[i] = (Float)s;
  }
  sum = Float(s);
  normalization = Float(1.0 / s);
}
size_t Discrete1D::Sample(Float xi) const {
  Float value = xi * sum;
  return size_t(std::lower_bound(cdf.begin(), cdf.end(), value) - cdf.begin());
}
std::pair<size_t, Float> Discrete1D::SampleReuse(Float xi) const {
  size_t index = Sample(xi);
  Float p = pmf[index] * normalization;
  Float c = index == 0 ? 0 : cdf[index - 1] * normalization;
  return {index, (xi - c) / p};
}

// =============================================================== shapes
// mesh_base.cpp:84-110, rectangle.cpp:204-214, sphere.cpp:251-259
PositionSample Shape::SamplePosition(const V2& xi) const {
  PositionSample psr;
  if (kind == Mesh) {
    V2 txi = xi;
    auto ir = dist.SampleReuse(txi.y);
    txi.y = ir.second;
    uint32_t face = uint32_t(ir.first) * 3;
    uint32_t f0 = idx[face], f1 = idx[face + 1], f2 = idx[face + 2];
    V3 p0 = pos[f0], p1 = pos[f1], p2 = pos[f2];
    V3 e0 = p1 - p0, e1 = p2 - p0;
    V2 b = SquareToUniformTriangle(txi);
    psr.P = e0 * b.x + (e1 * b.y + p0);
    psr.Pdf = dist.normalization;
    psr.IsDelta = false;
    if (!hasUV) {
      psr.UV = b;
    } else {
      V2 uv0 = uv[f0], uv1 = uv[f1], uv2 = uv[f2];
      Float b0 = 1 - b.x - b.y;
      psr.UV = V2(uv0.x * b0 + (uv1.x * b.x + (uv2.x * b.y)), uv0.y * b0 + (uv1.y * b.x + (uv2.y * b.y)));
    }
    if (nrm.empty()) {
      psr.N = normalized(cross(e0, e1));
    } else {
      V3 n0 = nrm[f0], n1 = nrm[f1], n2 = nrm[f2];
      psr.N = normalized(n0 * (1 - b.x - b.y) + (n1 * b.x + (n2 * b.y)));
    }
  } else if (kind == Rect) {
    V2 s(xi.x * 2 - 1, xi.y * 2 - 1);
    psr.P = toWorld.ApplyAffineToWorld(V3(s.x, s.y, 0));
    psr.N = frame.N;
    psr.Pdf = 1 / surfaceArea;
    psr.UV = xi;
    psr.IsDelta = false;
  } else {
    V3 local = SquareToUniformSphere(xi);
    psr.P = Fmadd(local, V3(radius), center);
    psr.N = local;
    psr.IsDelta = radius == 0;
    psr.Pdf = 1 / surfaceArea;
  }
  return psr;
}
Float Shape::PdfPosition() const { return kind == Mesh ? dist.normalization : 1 / surfaceArea; }

// shape.cpp:7-19 and the sphere override sphere.cpp:265-320
DirectionSample Shape::SampleDirection(const V3& refP, const V2& xi) const {
  DirectionSample dsr;
  if (kind != Sphere) {
    PositionSample psr = SamplePosition(xi);
    static_cast<PositionSample&>(dsr) = psr;
    dsr.Dir = dsr.P - refP;
    Float distanceSquared = sqnorm(dsr.Dir);
    dsr.Dist = std::sqrt(distanceSquared);
    dsr.Dir = dsr.Dir / dsr.Dist;
    Float dp = std::abs(dot(dsr.Dir, dsr.N));
    Float x = distanceSquared / dp;
    dsr.Pdf *= std::isfinite(x) ? x : 0;
    return dsr;
  }
  V3 dcv = center - refP;
  Float dc2 = sqnorm(dcv);
  Float radiusAdj = radius * (Float(1) - RayEpsilon);
  bool isOut = dc2 > Sqr(radiusAdj);
  if (isOut) {
    Float invDc = Rsqrt(dc2);
    Float sinThetaMax = radius * invDc;
    Float sinThetaMax2 = Sqr(sinThetaMax);
    Float invSinThetaMax = Rcp(sinThetaMax);
    Float cosThetaMax = SafeSqrt(1.f - sinThetaMax2);
    Float sinTheta2 = sinThetaMax2 > Float(0.00068523262)
                          ? Float(1) - Sqr(Fmadd(cosThetaMax - Float(1), xi.x, Float(1)))
                          : sinThetaMax2 * xi.x;
    Float cosTheta = SafeSqrt(Float(1) - sinTheta2);
    Float cosAlpha = sinTheta2 * invSinThetaMax + cosTheta * SafeSqrt(Fmadd(-sinTheta2, Sqr(invSinThetaMax), Float(1)));
    Float sinAlpha = SafeSqrt(Fmadd(-cosAlpha, cosAlpha, Float(1)));
    Float ph = xi.y * (Float(2) * PI);
    Float sinPhi = std::sin(ph), cosPhi = std::cos(ph);
    V3 d = Frame(dcv * -invDc).ToWorld(V3(cosPhi * sinAlpha, sinPhi * sinAlpha, cosAlpha));
    dsr.P = Fmadd(d, V3(radius), center);
    dsr.N = d;
    dsr.Dir = dsr.P - refP;
    Float dist2 = sqnorm(dsr.Dir);
    dsr.Dist = std::sqrt(dist2);
    dsr.Dir = dsr.Dir / dsr.Dist;
    dsr.Pdf = SquareToUniformConePdf(cosThetaMax);
  } else {
    V3 d = SquareToUniformSphere(xi);
    dsr.P = Fmadd(d, V3(radius), center);
    dsr.N = d;
    dsr.Dir = dsr.P - refP;
    Float dist2 = sqnorm(dsr.Dir);
    dsr.Dist = std::sqrt(dist2);
    dsr.Dir = dsr.Dir / dsr.Dist;
    dsr.Pdf = (1 / surfaceArea) * dist2 / AbsDot(dsr.Dir, dsr.N);
  }
  dsr.IsDelta = radius == 0;
  return dsr;
}

// shape.cpp:21-25 and sphere.cpp:322-328
Float Shape::PdfDirection(const V3& refP, const DirectionSample& dsr) const {
  if (kind == Sphere) {
    Float sinAlpha = radius * Rcp(norm(center - refP));
    Float cosAlpha = SafeSqrt(Float(1) - sinAlpha * sinAlpha);
    return sinAlpha < OneMinusEpsilon ? SquareToUniformConePdf(cosAlpha)
                                      : (1 / surfaceArea) * Sqr(dsr.Dist) / AbsDot(dsr.Dir, dsr.N);
  }
  Float pdf = PdfPosition();
  Float dp = std::abs(dot(dsr.Dir, dsr.N));
  pdf *= dp == 0 ? 0 : Sqr(dsr.Dist) / dp;
  return pdf;
}

// ================================================================ media
// grid.cpp:41-75 (trilinear with the half-texel neighbour rule) and :88-103
Spectrum Medium::EvalGrid(const V3& p) const {
  auto wrap = [&](Float v) {
    if (repeatWrap) return std::clamp(v - std::floor(v), Float(0), Float(1));
    return std::clamp(v, Float(0), Float(1));
  };
  V3 wp(wrap(p.x), wrap(p.y), wrap(p.z));
  V3 fp(wp.x * (Float(nx) - 1), wp.y * (Float(ny) - 1), wp.z * (Float(nz) - 1));
  int ix = (int)fp.x, iy = (int)fp.y, iz = (int)fp.z;
  int dpu = (fp.x > (ix + Float(0.5))) ? 1 : -1;
  int dpv = (fp.y > (iy + Float(0.5))) ? 1 : -1;
  int dpw = (fp.z > (iz + Float(0.5))) ? 1 : -1;
  int apu = std::clamp(ix + dpu, 0, nx - 1);
  int apv = std::clamp(iy + dpv, 0, ny - 1);
  int apw = std::clamp(iz + dpw, 0, nz - 1);
  Float du = std::min(std::abs(fp.x - ix - Float(0.5)), Float(1));
  Float dv = std::min(std::abs(fp.y - iy - Float(0.5)), Float(1));
  Float dw = std::min(std::abs(fp.z - iz - Float(0.5)), Float(1));
  auto rd = [&](int u, int v, int w) {
    size_t start = (((size_t)w * (size_t)ny + (size_t)v) * (size_t)nx + (size_t)u) * (size_t)channels;
    if (channels == 1) return V3(grid[start]);
    return V3(grid[start], grid[start + 1], grid[start + 2]);
  };
  V3 c000 = rd(ix, iy, iz), c100 = rd(apu, iy, iz), c010 = rd(ix, apv, iz), c001 = rd(ix, iy, apw);
  V3 c110 = rd(apu, apv, iz), c011 = rd(ix, apv, apw), c101 = rd(apu, iy, apw), c111 = rd(apu, apv, apw);
  V3 a = Fmadd(c000, V3(1 - du), c100 * du);
  V3 b = Fmadd(c010, V3(1 - du), c110 * du);
  V3 e = Fmadd(a, V3(1 - dv), b * dv);
  V3 f = Fmadd(c001, V3(1 - du), c101 * du);
  V3 g2 = Fmadd(c011, V3(1 - du), c111 * du);
  V3 h = Fmadd(f, V3(1 - dv), g2 * dv);
  return Fmadd(e, V3(1 - dw), h * dw);
}

// heterogeneous.cpp:64-76 (slab test) / homogeneous.cpp:23-25 (infinite)
void Medium::IntersectAABB(const Ray& ray, bool& active, Float& mint, Float& maxt) const {
  if (kind == Homogeneous) {
    active = true;
    mint = 0.f;
    maxt = std::numeric_limits<Float>::infinity();
    return;
  }
  bool contains = ray.O.x >= bbMin.x && ray.O.y >= bbMin.y && ray.O.z >= bbMin.z && ray.O.x <= bbMax.x &&
                  ray.O.y <= bbMax.y && ray.O.z <= bbMax.z;
  active = !is_zero(ray.D) || contains;
  V3 rcp(1 / ray.D.x, 1 / ray.D.y, 1 / ray.D.z);
  V3 t1 = cmul(bbMin - ray.O, rcp);
  V3 t2 = cmul(bbMax - ray.O, rcp);
  V3 t1p = vmin(t1, t2);
  V3 t2p = vmax(t1, t2);
  mint = max_comp(t1p);
  maxt = min_comp(t2p);
  active = active && maxt >= mint;
}

Spectrum Medium::Majorant() const {
  if (kind == Homogeneous) return sigmaT * scale;  // homogeneous.cpp:27-29
  return V3(maxDensity);                         // heterogeneous.cpp:38-40
}

void Medium::Coefficients(const V3& P, Spectrum& sS, Spectrum& sN, Spectrum& sT) const {
  if (kind == Homogeneous) {  // homogeneous.cpp:31-36
    sT = sigmaT * scale;
    sS = cmul(sT, albedoConst);
    sN = V3(0);
    return;
  }
  // heterogeneous.cpp:42-62
  V3 local = toWorld.ApplyAffineToLocal(P);
  Spectrum e = gridSigma ? EvalGrid(local) : sigmaT;
  sT = e * scale;
  sS = cmul(sT, albedoConst);
  sN = V3(maxDensity) - sT;
}

// ================================================================ camera
// perspective.cpp:73-82
Ray Camera::SampleRay(const V2& screen) const {
  V2 t(screen.x * (1 / Float(width)), screen.y * (1 / Float(height)));
  V3 ndc(t.x, t.y, 0);
  V3 nearP = cameraToClip.ApplyAffineToLocal(ndc);
  V3 dir = normalized(nearP);
  Float invZ = Rcp(dir.z);
  Ray r;
  r.O = cameraToWorld.ApplyAffineToWorld(V3(0, 0, 0));
  r.D = normalized(cameraToWorld.ApplyLinearToWorld(dir));
  r.MinT = nearZ * invZ;
  r.MaxT = farZ * invZ;
  return r;
}

Ray Camera::SampleRayDifferential(const V2& screen, RayDiff& diff) const {
  V2 t(screen.x * (1 / Float(width)), screen.y * (1 / Float(height)));
  V3 ndc(t.x, t.y, 0);
  V3 nearP = cameraToClip.ApplyAffineToLocal(ndc);
  Ray r = SampleRay(screen);
  diff.has = true;
  diff.Ox = diff.Oy = r.O;
  diff.Dx = cameraToWorld.ApplyLinearToWorld(normalized(nearP + dx));
  diff.Dy = cameraToWorld.ApplyLinearToWorld(normalized(nearP + dy));
  return r;
}

Float Camera::SampleDirection(const V3& ref, DirectionSample& dsr) const {
  V3 refP = cameraToWorld.ApplyAffineToLocal(ref);
  dsr = DirectionSample();
  dsr.Pdf = 0;
  if (refP.z < nearZ || refP.z > farZ) return 0;
  V3 ndcPos = cameraToClip.ApplyAffineToWorld(refP);
  if (ndcPos.x < 0 || ndcPos.x >= 1 || ndcPos.y < 0 || ndcPos.y >= 1) return 0;
  dsr.UV = V2(ndcPos.x * Float(width), ndcPos.y * Float(height));
  Float dist = norm(refP);
  Float invDist = Rcp(dist);
  V3 dir = refP * invDist;
  dsr.P = cameraToWorld.ApplyAffineToWorld(V3(0, 0, 0));
  dsr.Dir = (dsr.P - ref) * invDist;
  dsr.Dist = dist;
  dsr.N = cameraToWorld.ApplyLinearToWorld(V3(0, 0, 1));
  dsr.Pdf = 1;
  return Importance(dir) * invDist * invDist;
}

Float Camera::Importance(const V3& d) const {
  Float cosTheta = d.z;
  if (cosTheta <= 0) return 0;
  Float invCosTheta = Rcp(cosTheta);
  V2 p(d.x * invCosTheta, d.y * invCosTheta);
  if (!(rectMin.x <= p.x && rectMin.y <= p.y && p.x <= rectMax.x && p.y <= rectMax.y)) return 0;
  return normalization * invCosTheta * invCosTheta * invCosTheta;
}

Float Camera::PdfWe(const V3& worldDir) const { return Importance(cameraToWorld.ApplyLinearToLocal(worldDir)); }

void SurfaceInteraction::ComputeDifferentials(const RayDiff& ray) {
  if (!(ray.has && dUVdX.x == 0 && dUVdX.y == 0 && dUVdY.x == 0 && dUVdY.y == 0)) return;
  Float d = dot(N, P);
  Float tx = (d - dot(N, ray.Ox)) / dot(N, ray.Dx);
  Float ty = (d - dot(N, ray.Oy)) / dot(N, ray.Dy);
  V3 dpdx = (ray.Dx * tx + ray.Ox) - P;
  V3 dpdy = (ray.Dy * ty + ray.Oy) - P;
  Float a00 = dot(dPdU, dPdU), a01 = dot(dPdU, dPdV), a11 = dot(dPdV, dPdV),
        invDet = Rcp(Fmadd(a00, a11, -(a01 * a01)));
  Float b0x = dot(dPdU, dpdx), b1x = dot(dPdV, dpdx), b0y = dot(dPdU, dpdy), b1y = dot(dPdV, dpdy);
  invDet = std::isfinite(invDet) ? invDet : 0;
  dUVdX = V2(Fmadd(a11, b0x, -(a01 * b1x)) * invDet, Fmadd(a00, b1x, -(a01 * b0x)) * invDet);
  dUVdY = V2(Fmadd(a11, b0y, -(a01 * b1y)) * invDet, Fmadd(a00, b1y, -(a01 * b0y)) * invDet);
}

// math_ext.h:65-75
static M4 LookAtLeftHand(const V3& origin, const V3& target, const V3& up) {
  V3 dir = normalized(target - origin);
  V3 left = normalized(cross(normalized(up), dir));
  V3 realUp = normalized(cross(dir, left));
  M4 r = M4::Identity();
  for (int i = 0; i < 3; i++) {
    r.m[i][0] = left[i];
    r.m[i][1] = realUp[i];
    r.m[i][2] = dir[i];
    r.m[i][3] = origin[i];
  }
  return r;
}

static Camera MakeCamera(const Json& cfg) {
  if (ReadS(&cfg, "type", "") != "perspective") throw std::runtime_error("cannot find factory: camera");
  Camera c;
  c.nearZ = ReadF(&cfg, "near", Float(0.001));
  c.farZ = ReadF(&cfg, "far", Float(100));
  Float fov = ReadF(&cfg, "fov", 30);
  if (const Json* r = cfg.find("resolution")) {
    c.width = (int)JNum(r->arr.at(0));
    c.height = (int)JNum(r->arr.at(1));
  }
  M4 toWorld;
  if (const Json* tw = cfg.find("to_world")) {
    toWorld = JsonAsTransform(*tw);
  } else {
    toWorld = LookAtLeftHand(ReadV3(&cfg, "origin", V3(0, 0, -1)), ReadV3(&cfg, "target", V3(0, 0, 0)),
                             ReadV3(&cfg, "up", V3(0, 1, 0)));
  }
  c.cameraToWorld = Transform(toWorld);
  Float aspect = c.width / static_cast<Float>(c.height);
  Float recip = 1 / (c.farZ - c.nearZ);
  Float cot = 1 / std::tan(Radian(fov / 2));
  M4 persp{}, scale{}, translate = M4::Identity();
  persp.m[0][0] = cot;
  persp.m[1][1] = cot;
  persp.m[2][2] = c.farZ * recip;
  persp.m[2][3] = -c.nearZ * c.farZ * recip;
  persp.m[3][2] = 1;
  scale.m[0][0] = -Float(0.5);
  scale.m[1][1] = -Float(0.5) * aspect;
  scale.m[2][2] = 1;
  scale.m[3][3] = 1;
  translate.m[0][3] = -1;
  translate.m[1][3] = -1 / aspect;
  c.cameraToClip = Transform(scale * translate * persp);
  V3 o = c.cameraToClip.ApplyAffineToLocal(V3(0, 0, 0));
  c.dx = c.cameraToClip.ApplyAffineToLocal(V3(Float(1) / c.width, 0, 0)) - o;
  c.dy = c.cameraToClip.ApplyAffineToLocal(V3(0, Float(1) / c.height, 0)) - o;
  V3 pMin = c.cameraToClip.ApplyAffineToLocal(V3(0, 0, 0));
  V3 pMax = c.cameraToClip.ApplyAffineToLocal(V3(1, 1, 0));
  V2 a(pMin.x / pMin.z, pMin.y / pMin.z), b(pMax.x / pMax.z, pMax.y / pMax.z);
  c.rectMin = V2(std::min(a.x, b.x), std::min(a.y, b.y));  // BoundingBox2::extend
  c.rectMax = V2(std::max(a.x, b.x), std::max(a.y, b.y));
  c.normalization = 1 / ((c.rectMax.x - c.rectMin.x) * (c.rectMax.y - c.rectMin.y));
  return c;
}

// ============================================================ OBJ / vol
// wavefront_obj_reader.cpp: v / vt / vn / f (triangles; v, v/vt, v/vt/vn, v//vn),
// o / g objects; unique (v, vn, vt) triples become vertices (ToModel :408-452).
struct ObjModel {
  std::vector<V3> pos, nrm;
  std::vector<V2> uv;
  std::vector<uint32_t> idx;
};
struct ObjFile {
  std::vector<V3> p, n;
  std::vector<V2> t;
  struct Face { int v[3], vt[3], vn[3]; };
  std::vector<Face> faces;
  std::vector<std::pair<std::string, std::vector<size_t>>> objects;
};

static ObjFile ReadObj(const std::string& path) {
  std::ifstream in(path);
  if (!in) throw std::runtime_error("cannot open " + path);
  ObjFile f;
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream ss(line);
    std::string cmd;
    if (!(ss >> cmd) || cmd[0] == '#') continue;
    if (cmd == "v") {
      V3 v; ss >> v.x >> v.y >> v.z; f.p.push_back(v);
    } else if (cmd == "vn") {
      V3 v; ss >> v.x >> v.y >> v.z; f.n.push_back(v);
    } else if (cmd == "vt") {
      V2 v; ss >> v.x >> v.y; f.t.push_back(v);
    } else if (cmd == "f") {
      ObjFile::Face face{};
      for (int k = 0; k < 3; k++) {
        std::string tok;
        ss >> tok;
        int a = 0, b = 0, c = 0;
        size_t s1 = tok.find('/');
        if (s1 == std::string::npos) {
          a = std::stoi(tok);
        } else {
          a = std::stoi(tok.substr(0, s1));
          size_t s2 = tok.find('/', s1 + 1);
          if (s2 == std::string::npos) {
            b = std::stoi(tok.substr(s1 + 1));
          } else {
            if (s2 > s1 + 1) b = std::stoi(tok.substr(s1 + 1, s2 - s1 - 1));
            c = std::stoi(tok.substr(s2 + 1));
          }
        }
        face.v[k] = a; face.vt[k] = b; face.vn[k] = c;
      }
      if (!f.objects.empty()) f.objects.back().second.push_back(f.faces.size());
      f.faces.push_back(face);
    } else if (cmd == "o" || cmd == "g") {
      std::string name;
      std::getline(ss, name);
      size_t b = name.find_first_not_of(" \t");
      name = b == std::string::npos ? "" : name.substr(b);
      while (!name.empty() && (name.back() == ' ' || name.back() == '\r')) name.pop_back();
      f.objects.push_back({name, {}});
    }
  }
  return f;
}

static ObjModel ToModel(const ObjFile& f, const std::vector<size_t>* faceList) {
  auto cvt = [](int i, size_t count) { return i >= 0 ? size_t(i - 1) : count + i; };
  ObjModel m;
  std::map<std::tuple<int, int, int>, uint32_t> unique;
  size_t nf = faceList ? faceList->size() : f.faces.size();
  for (size_t q = 0; q < nf; q++) {
    const auto& face = f.faces[faceList ? (*faceList)[q] : q];
    for (int k = 0; k < 3; k++) {
      auto key = std::make_tuple(face.v[k], face.vn[k], face.vt[k]);
      auto it = unique.find(key);
      uint32_t index;
      if (it == unique.end()) {
        index = (uint32_t)m.pos.size();
        unique.emplace(key, index);
        m.pos.push_back(f.p[cvt(face.v[k], f.p.size())]);
        if (face.vn[k] != 0) m.nrm.push_back(f.n[cvt(face.vn[k], f.n.size())]);
        if (face.vt[k] != 0) m.uv.push_back(f.t[cvt(face.vt[k], f.t.size())]);
      } else {
        index = it->second;
      }
      m.idx.push_back(index);
    }
  }
  return m;
}

// volume_reader.cpp:65-124 (Mitsuba .vol version 3, fp32, 1 or 3 channels)
static void ReadVol(const std::string& path, Medium& md) {
  std::ifstream in(path, std::ios::binary);
  if (!in) throw std::runtime_error("cannot open " + path);
  char hdr[4];
  in.read(hdr, 4);
  if (hdr[0] != 'V' || hdr[1] != 'O' || hdr[2] != 'L' || hdr[3] != 3) throw std::runtime_error("not a VOL v3 file");
  int32_t type, sx, sy, sz, ch;
  in.read((char*)&type, 4);
  if (type != 1) throw std::runtime_error("vol must be Float32");
  in.read((char*)&sx, 4);
  in.read((char*)&sy, 4);
  in.read((char*)&sz, 4);
  in.read((char*)&ch, 4);
  if (ch != 1 && ch != 3) throw std::runtime_error("vol must have 1 or 3 channels");
  float dims[6];
  in.read((char*)dims, 24);
  md.nx = sx; md.ny = sy; md.nz = sz; md.channels = ch;
  md.grid.resize(size_t(sx) * sy * sz * ch);
  in.read((char*)md.grid.data(), md.grid.size() * 4);
  if (!in) throw std::runtime_error("vol truncated");
  float mx = -std::numeric_limits<float>::infinity();
  for (float v : md.grid) mx = std::max(mx, v);
  md.gridMax = mx;
}

// ================================================================ build
namespace {
struct Assets {
  std::map<std::string, ObjFile> objs;
  std::map<std::string, Medium> vols;  // only grid fields used
};
struct Entity {
  const Json* cfg;
  M4 toWorld;
};
}  // namespace

static std::string JoinPath(const std::string& base, const std::string& loc) {
  if (loc.empty() || loc[0] == '/' || base.empty()) return loc;
  return base + "/" + loc;
}

static Medium MakeMedium(const Json& cfg, const M4& toWorld, const Assets& assets) {
  Medium md;
  const Json* ph = cfg.find("phase");
  if (!ph) throw std::runtime_error("medium must have phase function");  // medium.cpp:8-17
  std::string pt = ReadS(ph, "type", "");
  if (pt == "hg_phase") {
    md.hg = true;
    md.g = ReadF(ph, "g", Float(0.8));
    if (md.g <= -1 || md.g >= 1) throw std::runtime_error("param g must lie in the interval (-1, 1)");
  } else if (pt == "isotropic_phase") {
    md.hg = false;
  } else {
    throw std::runtime_error("cannot find factory: " + pt);
  }
  std::string type = ReadS(&cfg, "type", "");
  md.scale = ReadF(&cfg, "scale", 1);
  auto readVolConst = [&](const char* k, const V3& def, bool allowGrid, bool& isGrid) -> V3 {
    isGrid = false;
    const Json* j = cfg.find(k);
    if (!j) return def;
    if (j->is_number() || j->is_array()) return JVec3(*j);
    if (!allowGrid || ReadS(j, "type", "") != "volume_grid") throw std::runtime_error(std::string("unsupported volume for ") + k);
    auto it = assets.vols.find(ReadS(j, "asset_name", ""));
    if (it == assets.vols.end()) throw std::runtime_error("unknown volume asset");
    md.grid = it->second.grid;
    md.nx = it->second.nx; md.ny = it->second.ny; md.nz = it->second.nz;
    md.channels = it->second.channels;
    md.gridMax = it->second.gridMax;
    md.repeatWrap = ReadS(j, "wrap", "clamp") == "repeat";
    isGrid = true;
    return V3(0);
  };
  bool isGrid = false;
  if (type == "homogeneous") {  // homogeneous.cpp:14-22
    md.kind = Medium::Homogeneous;
    md.sigmaT = ReadV3(&cfg, "sigma_t", V3(1));
    md.albedoConst = readVolConst("albedo", V3(0.75f), false, isGrid);
  } else if (type == "heterogeneous") {  // heterogeneous.cpp:17-36
    md.kind = Medium::Heterogeneous;
    md.sigmaT = readVolConst("sigma_t", V3(1), true, md.gridSigma);
    md.albedoConst = readVolConst("albedo", V3(0.75f), false, isGrid);
    M4 affine = M4::Identity();  // S(2) * T(-0.5): [0,1]^3 -> [-1,1]^3
    for (int i = 0; i < 3; i++) {
      affine.m[i][i] = 2;
      affine.m[i][3] = -1;
    }
    md.toWorld = Transform(toWorld * affine);
    // transform.cpp:67-77: ApplyBoxToWorld of [0,1]^3
    V3 lo(std::numeric_limits<Float>::infinity()), hi(-std::numeric_limits<Float>::infinity());
    for (int c = 0; c < 8; c++) {
      V3 p = md.toWorld.ApplyAffineToWorld(V3(Float(c & 1), Float((c >> 1) & 1), Float((c >> 2) & 1)));
      lo = vmin(lo, p);
      hi = vmax(hi, p);
    }
    md.bbMin = lo;
    md.bbMax = hi;
    Float mv = md.gridSigma ? md.gridMax : max_comp(md.sigmaT);  // Volume::GetMaxValue
    md.maxDensity = mv * md.scale;
  } else {
    throw std::runtime_error("cannot find factory: " + type);
  }
  return md;
}

std::unique_ptr<Scene> Scene::FromJson(const std::string& text, const std::string& baseDir) {
  Json root = Json::parse(text);
  auto sc = std::make_unique<Scene>();
  Scene& S = *sc;
  // assets (build_context.cpp:23-34 -> asset.cpp:17-38)
  Assets assets;
  if (const Json* an = root.find("assets")) {
    for (const Json& a : an->arr) {
      std::string type = ReadS(&a, "type", ""), name = ReadS(&a, "name", ""), loc = ReadS(&a, "location", "");
      if (type == "model_obj") {
        assets.objs.emplace(name, ReadObj(JoinPath(baseDir, loc)));
      } else if (type == "volume_data_mitsuba_vol") {
        Medium md;
        ReadVol(JoinPath(baseDir, loc), md);
        assets.vols.emplace(name, std::move(md));
      } else if (type == "image_default" || type == "image_hdr" || type == "image_exr") {
        S.images[name] = LoadImageAsset(a, type, JoinPath(baseDir, loc));
      } else {
        throw std::runtime_error("cannot find factory: " + type);
      }
    }
  }
  TexEnv env{&S.images, &S.textures};
  const Json* cam = root.find("camera");
  if (!cam) throw std::runtime_error("no child: camera");
  S.camera = MakeCamera(*cam);
  const Json* smp = root.find("sampler");
  if (smp) {
    if (ReadS(smp, "type", "") != "independent") throw std::runtime_error("cannot find factory: sampler");
    S.spp = ReadI(smp, "sample_count", 16);
    S.seed = (uint32_t)ReadI(smp, "seed", 0);
  }
  if (const Json* gm = root.find("global_medium")) {
    S.media.push_back(MakeMedium(*gm, M4::Identity(), assets));
    S.globalMedium = 0;
  }
  std::map<std::string, int> bsdfVars;
  if (const Json* bv = root.find("bsdf_vars")) {
    for (const Json& v : bv->arr) {
      std::string name = ReadS(&v, "name", "");
      const Json* def = v.find("bsdf");
      if (!def) throw std::runtime_error("no child: bsdf");
      if (bsdfVars.count(name)) throw std::runtime_error("duplicate bsdf var name: " + name);
      S.bsdfs.push_back(MakeBsdf(def, &env));
      bsdfVars[name] = (int)S.bsdfs.size() - 1;
    }
  }
  const Json* sceneNode = root.find("scene");
  if (!sceneNode) throw std::runtime_error("no child: scene");
  std::deque<Entity> q;
  for (const Json& e : sceneNode->arr) {
    Entity en{&e, M4::Identity()};
    if (const Json* tw = e.find("to_world")) en.toWorld = JsonAsTransform(*tw);
    q.push_back(en);
  }
  while (!q.empty()) {
    Entity en = q.front();
    q.pop_front();
    const Json& e = *en.cfg;
    if (const Json* ch = e.find("children")) {
      for (const Json& c : ch->arr) {
        Entity ce{&c, en.toWorld};
        if (const Json* tw = c.find("to_world")) ce.toWorld = JsonAsTransform(*tw) * en.toWorld;
        q.push_back(ce);
      }
    }
    int shapeIdx = -1, lightIdx = -1, bsdfIdx = -1;
    if (const Json* sn = e.find("shape")) {
      std::string type = ReadS(sn, "type", "");
      Shape sh;
      if (type == "rectangle") {  // rectangle.cpp:164-178
        sh.kind = Shape::Rect;
        M4 tw = en.toWorld;
        if (ReadB(sn, "is_flip_normal", false)) {
          M4 flip = M4::Identity();
          flip.m[2][2] = -1;
          tw = tw * flip;
        }
        sh.toWorld = Transform(tw);
        V3 dpdu = sh.toWorld.ApplyLinearToWorld(V3(2, 0, 0));
        V3 dpdv = sh.toWorld.ApplyLinearToWorld(V3(0, 2, 0));
        V3 n = normalized(sh.toWorld.ApplyNormalToWorld(V3(0, 0, 1)));
        sh.frame = Frame(dpdu, dpdv, n);
        sh.surfaceArea = norm(cross(dpdu, dpdv));
        sh.primCount = 1;
      } else if (type == "sphere") {  // sphere.cpp:173-189
        sh.kind = Shape::Sphere;
        V3 lc = ReadV3(sn, "center", V3(0));
        Float lr = ReadF(sn, "radius", 1);
        Transform t(en.toWorld);
        if (t.HasNonUniformScale()) throw std::runtime_error("Sphere does not support non uniform transformations");
        if (sn->has("rotate_uv")) throw std::runtime_error("rotate_uv is not supported");
        sh.center = t.ApplyAffineToWorld(lc);
        sh.radius = norm(t.ApplyLinearToWorld(V3(0, 0, lr)));
        M4 ts = M4::Identity();
        for (int i = 0; i < 3; i++) {
          ts.m[i][i] = sh.radius;
          ts.m[i][3] = sh.center[i];
        }
        sh.toWorld = Transform(ts * en.toWorld);
        sh.surfaceArea = 4 * PI * Sqr(sh.radius);
        sh.primCount = 1;
      } else if (type == "mesh" || type == "cube") {
        sh.kind = Shape::Mesh;
        Transform t(en.toWorld);
        bool ident = t.IsIdentity();
        ObjModel m;
        if (type == "cube") {  // cube.cpp:15-115 (UVs left zero, see below)
          static const float P[24][3] = {{1, -1, -1}, {1, -1, 1}, {-1, -1, 1}, {-1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                         {-1, 1, 1}, {1, 1, 1}, {1, -1, -1}, {1, 1, -1}, {1, 1, 1}, {1, -1, 1},
                                         {1, -1, 1}, {1, 1, 1}, {-1, 1, 1}, {-1, -1, 1}, {-1, -1, 1}, {-1, 1, 1},
                                         {-1, 1, -1}, {-1, -1, -1}, {1, 1, -1}, {1, -1, -1}, {-1, -1, -1}, {-1, 1, -1}};
          static const float N[6][3] = {{0, -1, 0}, {0, 1, 0}, {1, 0, 0}, {0, 0, 1}, {-1, 0, 0}, {0, 0, -1}};
          static const int T[12][3] = {{0, 1, 2}, {3, 0, 2}, {4, 5, 6}, {7, 4, 6}, {8, 9, 10}, {11, 8, 10},
                                       {12, 13, 14}, {15, 12, 14}, {16, 17, 18}, {19, 16, 18}, {20, 21, 22}, {23, 20, 22}};
          for (int i = 0; i < 24; i++) {
            m.pos.push_back(V3(P[i][0], P[i][1], P[i][2]));
            m.nrm.push_back(V3(N[i / 4][0], N[i / 4][1], N[i / 4][2]));
            m.uv.push_back(V2(0, 0));
          }
          for (int i = 0; i < 12; i++)
            for (int j = 0; j < 3; j++) m.idx.push_back((uint32_t)T[i][j]);
          ident = false;  // cube.cpp always transforms
        } else {  // mesh.cpp:14-52
          std::string an = ReadS(sn, "asset_name", "");
          auto it = assets.objs.find(an);
          if (it == assets.objs.end()) throw std::runtime_error("unknown model asset: " + an);
          if (const Json* sm = sn->find("sub_model")) {
            const std::vector<size_t>* fl = nullptr;
            for (auto& o : it->second.objects)
              if (o.first == sm->str) { fl = &o.second; break; }
            if (!fl) throw std::runtime_error("no model name: " + sm->str);
            m = ToModel(it->second, fl);
          } else {
            m = ToModel(it->second, nullptr);
          }
        }
        if (ident) {
          sh.pos = m.pos;
          sh.nrm = m.nrm;
        } else {
          for (auto& p : m.pos) sh.pos.push_back(t.ApplyAffineToWorld(p));
          for (auto& n : m.nrm) sh.nrm.push_back(t.ApplyNormalToWorld(n));
        }
        sh.uv = m.uv;
        sh.hasUV = !m.uv.empty();
        sh.idx = m.idx;
        sh.primCount = (uint32_t)(m.idx.size() / 3);
        // mesh_base.cpp:120-131: area distribution
        std::vector<Float> area;
        for (uint32_t i = 0; i < sh.primCount; i++) {
          V3 p0 = sh.pos[sh.idx[i * 3]], p1 = sh.pos[sh.idx[i * 3 + 1]], p2 = sh.pos[sh.idx[i * 3 + 2]];
          area.push_back(norm(cross(p1 - p0, p2 - p0)) * Float(0.5));
        }
        sh.dist.Build(area);
        sh.surfaceArea = sh.dist.sum;
      } else {
        throw std::runtime_error("cannot find factory: " + type);
      }
      S.shapes.push_back(std::move(sh));
      shapeIdx = (int)S.shapes.size() - 1;
    }
    if (const Json* ln = e.find("light")) {
      std::string type = ReadS(ln, "type", "");
      Light L;
      L.toWorld = Transform(en.toWorld);
      auto color = [&](const char* k, V3 def) {
        const Json* j = ln->find(k);
        if (!j) return def;
        if (j->is_number() || j->is_array()) return JVec3(*j);
        throw std::runtime_error("textured lights are not supported");
      };
      if (type == "area") {  // area.cpp:20-41
        L.kind = Light::Area;
        const Json* rj = ln->find("radiance");
        if (rj && rj->is_object()) {
          L.map = MakeTexture(*rj, 3, &env);
          uint32_t width = L.map->width, height = L.map->height;
          if (ReadS(rj, "type", "") == "chessboard") {
            // chessboard.cpp:30-31: width = height = 1, so _isUniform: the shape is sampled and the texture
            // read at each point's uv (area.cpp:45-58)
            L.uniformMap = true;
          } else if (width == 1 && height == 1) {  // _isUniform: the map is one constant
            L.radiance = L.map->Eval(TexSi{V2(0, 0), V2(), V2()});
            L.map = nullptr;
          } else {
            std::vector<Float> luminance(width * height);
            for (uint32_t y = 0; y < height; y++) {
              Float v = y / (Float)height;
              uint32_t start = y * width;
              for (uint32_t x = 0; x < width; x++) {
                Float u = x / (Float)width;
                luminance[start + x] = Luminance(L.map->Eval(TexSi{V2(u, v), V2(), V2()}));
              }
            }
            L.dist.Build(luminance.data(), width, height);
            L.uniformMap = false;
          }
        } else {
          L.radiance = color("radiance", V3(1));
        }
      } else if (type == "skybox") {  // skybox.cpp:24-50
        L.kind = Light::Skybox;
        const Json* rj = ln->find("radiance");
        if (rj && rj->is_object()) {
          L.map = MakeTexture(*rj, 3, &env);
          uint32_t width = L.map->width, height = L.map->height;
          L.uniformMap = width == 1 && height == 1;
          if (!L.uniformMap) {
            std::vector<Float> luminance(width * height);
            for (uint32_t y = 0; y < height; y++) {
              Float sinTheta = std::sin((y + Float(0.5)) / height * PI);
              Float v = y / (Float)height;
              uint32_t start = y * width;
              for (uint32_t x = 0; x < width; x++) {
                Float u = x / (Float)width;
                TexSi si{V2(u, v), V2(), V2()};
                V3 color = L.map->Eval(si);
                Float lum = Luminance(color);
                lum *= sinTheta;
                luminance[start + x] = lum;
              }
            }
            L.dist.Build(luminance.data(), width, height);
          }
        } else {
          L.radiance = color("radiance", V3(1));
        }
      } else if (type == "point") {  // point.cpp:19-26
        L.kind = Light::Point;
        L.worldPos = L.toWorld.ApplyAffineToWorld(ReadV3(ln, "position", V3(0, 0, 0)));
        L.radiance = ReadV3(ln, "intensity", V3(1, 1, 1));
      } else if (type == "projection") {  // projection.cpp:19-45
        L.kind = Light::Projection;
        const Json* ij = ln->find("irradiance");
        Float aspect = 1 / (Float)1;  // Width / Height of the irradiance texture (1 x 1 when constant)
        if (ij && ij->is_object()) {
          L.map = MakeTexture(*ij, 3, &env);
          aspect = L.map->width / (Float)L.map->height;
        } else {
          L.radiance = color("irradiance", V3(1));
        }
        L.scale = ReadV3(ln, "scale", V3(1, 1, 1));
        Float fov = ReadF(ln, "fov", Float(90));
        Float farZ = 10000;
        Float nearZ = Float(0.0001);
        Float recip = 1 / (farZ - nearZ);
        Float cot = 1 / std::tan(Radian(fov / 2));
        M4 persp{}, scale{}, translate = M4::Identity();
        persp.m[0][0] = cot;
        persp.m[1][1] = cot;
        persp.m[2][2] = farZ * recip;
        persp.m[2][3] = -nearZ * farZ * recip;
        persp.m[3][2] = 1;
        scale.m[0][0] = -Float(0.5);
        scale.m[1][1] = -Float(0.5) * aspect;
        scale.m[2][2] = 1;
        scale.m[3][3] = 1;
        translate.m[0][3] = -1;
        translate.m[1][3] = -1 / aspect;
        L.toClip = Transform(scale * translate * persp);
        V3 pMin = L.toClip.ApplyAffineToLocal(V3(0, 0, 0)), pMax = L.toClip.ApplyAffineToLocal(V3(1, 1, 0));
        Float ax = pMin.x / pMin.z, ay = pMin.y / pMin.z, bx = pMax.x / pMax.z, by = pMax.y / pMax.z;
        L.cameraArea = 1 / ((bx - ax) * (by - ay));  // BoundingBox2(min, max).volume()
      } else if (type == "directional") {
        L.kind = Light::Directional;
        L.radiance = color("irradiance", V3(1));
        L.direction = normalized(L.toWorld.ApplyLinearToWorld(ReadV3(ln, "direction", V3(0, -1, 0))));
      } else {
        throw std::runtime_error("cannot find factory: " + type);
      }
      S.lights.push_back(L);
      lightIdx = (int)S.lights.size() - 1;
    }
    if (const Json* bn = e.find("bsdf")) {
      if (const Json* ref = bn->find("ref")) {
        auto it = bsdfVars.find(ref->str);
        if (it == bsdfVars.end()) throw std::runtime_error("unknown bsdf var: " + ref->str);
        bsdfIdx = it->second;
      } else {
        S.bsdfs.push_back(MakeBsdf(bn, &env));
        bsdfIdx = (int)S.bsdfs.size() - 1;
      }
    }
    int inMed = -1, outMed = -1;
    bool outUseGlobal = true;
    if (const Json* im = e.find("in_medium")) {
      S.media.push_back(MakeMedium(*im, en.toWorld, assets));
      inMed = (int)S.media.size() - 1;
    }
    if (const Json* om = e.find("out_medium")) {
      if (const Json* ig = om->find("is_global")) {
        outUseGlobal = ig->b;
      } else {
        S.media.push_back(MakeMedium(*om, en.toWorld, assets));
        outMed = (int)S.media.size() - 1;
      }
    }
    // build_context.cpp:243-246: emitters without a BSDF get a default diffuse
    if (lightIdx >= 0 && shapeIdx >= 0 && bsdfIdx < 0) {
      Json def;
      def.kind = Json::Object;
      Json t;
      t.kind = Json::String;
      t.str = "diffuse";
      def.obj.push_back({"type", t});
      S.bsdfs.push_back(MakeBsdf(&def, &env));
      bsdfIdx = (int)S.bsdfs.size() - 1;
    }
    if (shapeIdx >= 0) {
      Shape& sh = S.shapes[shapeIdx];
      sh.light = lightIdx;
      sh.bsdf = bsdfIdx;
      if (outMed < 0 && outUseGlobal && S.globalMedium >= 0) outMed = S.globalMedium;
      sh.inMedium = inMed;
      sh.outMedium = outMed;
    }
    if (lightIdx >= 0) {
      S.lights[lightIdx].shape = shapeIdx;
      // only the rectangle has EvalParamSurface (shape.cpp:27-29)
      const Light& AL = S.lights[lightIdx];
      if (AL.kind == Light::Area && AL.map && !AL.uniformMap && (shapeIdx < 0 || S.shapes[shapeIdx].kind != Shape::Rect))
        throw std::runtime_error("no impl EvalParamSurface(): a textured area light needs a rectangle");
      // sphere.cpp:250-320 leaves the sample's uv unset: a chessboard would be read at an undefined uv
      if (AL.kind == Light::Area && AL.map && AL.uniformMap && shapeIdx >= 0 && S.shapes[shapeIdx].kind == Shape::Sphere)
        throw std::runtime_error("area: a chessboard radiance on a sphere is not supported");
    }
  }
  // renderer (path.cpp:26-29, vol_path.cpp:22-25)
  const Json* rn = root.find("renderer");
  if (!rn) throw std::runtime_error("no child: renderer");
  S.renderer = ReadS(rn, "type", "");
  if (S.renderer != "path" && S.renderer != "vol_path" && S.renderer != "ao" && S.renderer != "particle_tracer" &&
      S.renderer != "bdpt")
    throw std::runtime_error("cannot find factory: " + S.renderer);
  S.maxDepth = ReadI(rn, "max_depth", -1);
  // path.cpp, particle_tracer.cpp: 3; vol_path.cpp, bdpt.cpp: 5
  S.rrDepth = ReadI(rn, "rr_depth", S.renderer == "vol_path" || S.renderer == "bdpt" ? 5 : 3);
  if (S.renderer == "bdpt") {
    if (const Json* um = rn->find("use_mis")) S.useMis = um->b;
    for (const Light& L : S.lights)
      if (L.kind == Light::Directional) throw std::runtime_error("bdpt: the directional light is not supported");
  }
  if (const Json* an = root.find("accel")) {
    std::string at = ReadS(an, "type", "");
    if (at != "embree" && at != "gpu_bvh8") throw std::runtime_error("cannot find factory: " + at);
  }
  // primitives + BVH (replaces embree.cpp:18-43)
  uint32_t off = 0;
  for (uint32_t s = 0; s < S.shapes.size(); s++) {
    S.shapes[s].primOffset = off;
    for (uint32_t k = 0; k < S.shapes[s].primCount; k++) S.prims.push_back({s, k});
    off += S.shapes[s].primCount;
  }
  S.BuildBvh();
  // scene.cpp:11-36: uniform light selection, last env light wins
  S.lightPdf = Rcp(Float(S.lights.size()));
  V3 c((S.worldLo.x + S.worldHi.x) / 2, (S.worldLo.y + S.worldHi.y) / 2, (S.worldLo.z + S.worldHi.z) / 2);
  Float r = norm(c - S.worldHi);
  r = std::max(RayEpsilon, r * (1 + ShadowEpsilon));  // skybox.cpp:139-144
  for (size_t i = 0; i < S.lights.size(); i++) {
    if (S.lights[i].IsEnv()) S.envLight = (int)i;
    S.lights[i].worldCenter = c;
    S.lights[i].worldRadius = r;
  }
  return sc;
}

// ================================================================ BVH2
static void PrimBounds(const Scene& S, const PrimRef& p, V3& lo, V3& hi) {
  const Shape& sh = S.shapes[p.shape];
  lo = V3(std::numeric_limits<Float>::infinity());
  hi = V3(-std::numeric_limits<Float>::infinity());
  if (sh.kind == Shape::Mesh) {
    for (int k = 0; k < 3; k++) {
      V3 v = sh.pos[sh.idx[p.local * 3 + k]];
      lo = vmin(lo, v);
      hi = vmax(hi, v);
    }
  } else if (sh.kind == Shape::Rect) {  // rectangle.cpp:48-64
    const V3 cs[4] = {V3(-1, -1, 0), V3(1, -1, 0), V3(1, 1, 0), V3(-1, 1, 0)};
    for (auto& c : cs) {
      V3 v = sh.toWorld.ApplyAffineToWorld(c);
      lo = vmin(lo, v);
      hi = vmax(hi, v);
    }
  } else {  // sphere.cpp:56-69
    lo = sh.center - V3(sh.radius);
    hi = sh.center + V3(sh.radius);
  }
}

// The box the BVH tests for a primitive. Analytic primitives: the rectangle
// test runs on the float world->object rows, whose plane differs from the one
// through the corners by rounding, and a grazing ray turns that into a hit
// point outside the corner box (the sphere's roots likewise). Their boxes grow
// by 1e-5 of their largest coordinate so traversal never culls a primitive its
// own test would hit. World bounds and centroids use the unpadded box.
static void PadAnalytic(const Scene& S, const PrimRef& p, V3& lo, V3& hi) {
  if (S.shapes[p.shape].kind == Shape::Mesh) return;
  Float m = 0;
  for (int a = 0; a < 3; a++) m = std::max(m, std::max(std::abs(lo[a]), std::abs(hi[a])));
  V3 pad(m * 1e-5f);
  lo = lo - pad;
  hi = hi + pad;
}

void Scene::BuildBvh() {
  size_t n = prims.size();
  std::vector<V3> lo(n), hi(n), ce(n);
  worldLo = V3(std::numeric_limits<Float>::infinity());
  worldHi = V3(-std::numeric_limits<Float>::infinity());
  for (size_t i = 0; i < n; i++) {
    PrimBounds(*this, prims[i], lo[i], hi[i]);
    ce[i] = (lo[i] + hi[i]) * 0.5f;
    worldLo = vmin(worldLo, lo[i]);
    worldHi = vmax(worldHi, hi[i]);
    PadAnalytic(*this, prims[i], lo[i], hi[i]);
  }
  order.resize(n);
  for (size_t i = 0; i < n; i++) order[i] = (uint32_t)i;
  nodes.clear();
  nodes.reserve(2 * n + 1);
  if (n == 0) return;
  struct Task { uint32_t node, b, e; };
  std::vector<Task> stack;
  nodes.push_back(BvhNode{});
  stack.push_back({0, 0, (uint32_t)n});
  const int kBins = 16;
  while (!stack.empty()) {
    Task t = stack.back();
    stack.pop_back();
    V3 blo(std::numeric_limits<Float>::infinity()), bhi(-std::numeric_limits<Float>::infinity());
    V3 clo = blo, chi = bhi;
    for (uint32_t i = t.b; i < t.e; i++) {
      blo = vmin(blo, lo[order[i]]);
      bhi = vmax(bhi, hi[order[i]]);
      clo = vmin(clo, ce[order[i]]);
      chi = vmax(chi, ce[order[i]]);
    }
    nodes[t.node].lo = blo;
    nodes[t.node].hi = bhi;
    uint32_t cnt = t.e - t.b;
    auto area = [](const V3& a, const V3& b) {
      V3 d = b - a;
      return d.x * d.y + d.y * d.z + d.z * d.x;
    };
    int bestAxis = -1, bestSplit = -1;
    Float bestCost = std::numeric_limits<Float>::infinity();
    if (cnt > 2) {
      for (int ax = 0; ax < 3; ax++) {
        Float ext = chi[ax] - clo[ax];
        if (!(ext > 0)) continue;
        V3 bl[kBins], bh[kBins];
        int bc[kBins] = {0};
        for (int k = 0; k < kBins; k++) {
          bl[k] = V3(std::numeric_limits<Float>::infinity());
          bh[k] = V3(-std::numeric_limits<Float>::infinity());
        }
        for (uint32_t i = t.b; i < t.e; i++) {
          int k = std::min(kBins - 1, (int)((ce[order[i]][ax] - clo[ax]) / ext * kBins));
          bc[k]++;
          bl[k] = vmin(bl[k], lo[order[i]]);
          bh[k] = vmax(bh[k], hi[order[i]]);
        }
        Float rightArea[kBins];
        int rightCnt[kBins];
        V3 rl(std::numeric_limits<Float>::infinity()), rh(-std::numeric_limits<Float>::infinity());
        int rc = 0;
        for (int k = kBins - 1; k > 0; k--) {
          rl = vmin(rl, bl[k]);
          rh = vmax(rh, bh[k]);
          rc += bc[k];
          rightArea[k] = rc ? area(rl, rh) : 0;
          rightCnt[k] = rc;
        }
        V3 ll(std::numeric_limits<Float>::infinity()), lh(-std::numeric_limits<Float>::infinity());
        int lc = 0;
        for (int k = 0; k < kBins - 1; k++) {
          ll = vmin(ll, bl[k]);
          lh = vmax(lh, bh[k]);
          lc += bc[k];
          if (lc == 0 || rightCnt[k + 1] == 0) continue;
          Float cost = area(ll, lh) * lc + rightArea[k + 1] * rightCnt[k + 1];
          if (cost < bestCost) {
            bestCost = cost;
            bestAxis = ax;
            bestSplit = k;
          }
        }
      }
    }
    Float leafCost = area(blo, bhi) * cnt;
    bool makeLeaf = cnt <= 2 || (cnt <= 4 && bestCost >= leafCost) || bestAxis < 0;
    if (makeLeaf && cnt > 8 && bestAxis < 0) {
      // degenerate centroids: split in the middle of the list
      uint32_t mid = t.b + cnt / 2;
      uint32_t l = (uint32_t)nodes.size();
      nodes.push_back(BvhNode{});
      nodes.push_back(BvhNode{});
      nodes[t.node].left = l;
      stack.push_back({l, t.b, mid});
      stack.push_back({l + 1, mid, t.e});
      continue;
    }
    if (makeLeaf) {
      nodes[t.node].first = t.b;
      nodes[t.node].count = cnt;
      continue;
    }
    Float ext = chi[bestAxis] - clo[bestAxis];
    auto mid = std::partition(order.begin() + t.b, order.begin() + t.e, [&](uint32_t p) {
      int k = std::min(kBins - 1, (int)((ce[p][bestAxis] - clo[bestAxis]) / ext * kBins));
      return k <= bestSplit;
    });
    uint32_t m = uint32_t(mid - order.begin());
    uint32_t l = (uint32_t)nodes.size();
    nodes.push_back(BvhNode{});
    nodes.push_back(BvhNode{});
    nodes[t.node].left = l;
    stack.push_back({l, t.b, m});
    stack.push_back({l + 1, m, t.e});
  }
}

// Watertight ray/triangle test (Woop, Benthin, Wald, JCGT 2(1), 2013), with
// the double-precision recomputation of zero edge functions. Returns t, Embree
// barycentrics (u weights v1, v weights v2) and det > 0 for front faces.
static bool TriWatertight(const V3& O, const V3& D, const V3& v0, const V3& v1, const V3& v2, Float& t, Float& u,
                          Float& v, bool& front) {
  int kz = 0;
  Float ax = std::abs(D.x), ay = std::abs(D.y), az = std::abs(D.z);
  if (ay > ax) kz = 1;
  if (az > std::max(ax, ay)) kz = 2;
  int kx = kz + 1 == 3 ? 0 : kz + 1;
  int ky = kx + 1 == 3 ? 0 : kx + 1;
  if (D[kz] < 0) std::swap(kx, ky);
  Float Sx = D[kx] / D[kz], Sy = D[ky] / D[kz], Sz = 1.0f / D[kz];
  V3 A = v0 - O, B = v1 - O, C = v2 - O;
  Float Ax = A[kx] - Sx * A[kz], Ay = A[ky] - Sy * A[kz];
  Float Bx = B[kx] - Sx * B[kz], By = B[ky] - Sy * B[kz];
  Float Cx = C[kx] - Sx * C[kz], Cy = C[ky] - Sy * C[kz];
  Float U = Cx * By - Cy * Bx;
  Float V = Ax * Cy - Ay * Cx;
  Float W = Bx * Ay - By * Ax;
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    U = (Float)((double)Cx * (double)By - (double)Cy * (double)Bx);
    V = (Float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
    W = (Float)((double)Bx * (double)Ay - (double)By * (double)Ax);
  }
  if ((U < 0 || V < 0 || W < 0) && (U > 0 || V > 0 || W > 0)) return false;
  Float det = U + V + W;
  if (det == 0) return false;
  Float Az = Sz * A[kz], Bz = Sz * B[kz], Cz = Sz * C[kz];
  Float T = U * Az + V * Bz + W * Cz;
  t = T / det;
  u = V / det;
  v = W / det;
  front = det > 0;
  return true;
}

// Hit acceptance shared by every primitive type: t in (MinT, best), and on an
// exact tie the lower global primitive id wins, so the closest hit does not
// depend on the traversal order.
static inline bool Accept(Float t, uint32_t prim, Float tmin, const Hit& best) {
  if (!(t > tmin)) return false;
  if (t < best.t) return true;
  return t == best.t && best.prim != 0xffffffffu && prim < best.prim;
}

bool Scene::IntersectPrim(uint32_t gp, const Ray& ray, Hit& hit) const {
  const PrimRef& pr = prims[gp];
  const Shape& sh = shapes[pr.shape];
  Float t, u = 0, v = 0;
  bool front;
  if (sh.kind == Shape::Mesh) {
    const uint32_t* f = &sh.idx[pr.local * 3];
    if (!TriWatertight(ray.O, ray.D, sh.pos[f[0]], sh.pos[f[1]], sh.pos[f[2]], t, u, v, front)) return false;
  } else if (sh.kind == Shape::Rect) {  // rectangle.cpp:34-46
    V3 O = Transform::Affine(sh.toWorld.ToLocal, ray.O);
    V3 D = Transform::Linear(sh.toWorld.ToLocal, ray.D);
    t = -O.z / D.z;
    V3 local = D * t + O;
    if (!(std::abs(local.x) <= 1 && std::abs(local.y) <= 1)) return false;
    u = local.x;
    v = local.y;
    front = D.z < 0;  // object-space normal is +z
  } else {  // sphere.cpp:40-54
    V3 o = ray.O - sh.center;
    Float a = sqnorm(ray.D);
    Float b = 2 * dot(o, ray.D);
    Float c = sqnorm(o) - Sqr(sh.radius);
    bool found;
    Float nearT, farT;
    SolveQuadratic(a, b, c, found, nearT, farT);
    bool outBounds = !(nearT <= hit.t && farT >= ray.MinT);
    bool inBounds = nearT < ray.MinT && farT > hit.t;
    if (!(found && !outBounds && !inBounds)) return false;
    t = nearT < 0 ? farT : nearT;
    V3 n = normalized((ray.D * t + ray.O) - sh.center);
    front = dot(ray.D, n) < 0;
  }
  if (!Accept(t, gp, ray.MinT, hit)) return false;
  hit.t = t;
  hit.u = u;
  hit.v = v;
  hit.prim = gp;
  hit.front = front ? 1u : 0u;
  return true;
}

static inline bool BoxHit(const BvhNode& n, const V3& O, const V3& inv, Float tmin, Float tmax, Float& tnear) {
  Float t0 = tmin, t1 = tmax;
  for (int a = 0; a < 3; a++) {
    Float tn = (n.lo[a] - O[a]) * inv[a];
    Float tf = (n.hi[a] - O[a]) * inv[a];
    if (tn > tf) std::swap(tn, tf);
    tf *= 1 + 2 * 3.5762786865234375e-07f;  // robust traversal margin (Ize 2013)
    t0 = tn > t0 ? tn : t0;
    t1 = tf < t1 ? tf : t1;
  }
  tnear = t0;
  return t0 <= t1;
}

Hit Scene::Intersect(const Ray& ray) const {
  Hit h;
  h.t = ray.MaxT;
  if (nodes.empty()) return Hit{};
  V3 inv(1 / ray.D.x, 1 / ray.D.y, 1 / ray.D.z);
  uint32_t stack[128];
  int sp = 0;
  stack[sp++] = 0;
  // Nodes are pruned against the best distance widened by the same margin as
  // the slabs: a node holding a primitive at exactly the best t (an exact tie,
  // which the lower primitive id wins) is still visited, so the result does not
  // depend on the order nodes are visited in.
  const Float margin = 1 + 2 * 3.5762786865234375e-07f;
  while (sp) {
    const BvhNode& n = nodes[stack[--sp]];
    Float tn;
    if (!BoxHit(n, ray.O, inv, ray.MinT, h.t * margin, tn)) continue;
    if (n.count) {
      for (uint32_t i = 0; i < n.count; i++) IntersectPrim(order[n.first + i], ray, h);
    } else {
      Float ta, tb;
      bool ha = BoxHit(nodes[n.left], ray.O, inv, ray.MinT, h.t * margin, ta);
      bool hb = BoxHit(nodes[n.left + 1], ray.O, inv, ray.MinT, h.t * margin, tb);
      if (ha && hb) {
        if (ta <= tb) {
          stack[sp++] = n.left + 1;
          stack[sp++] = n.left;
        } else {
          stack[sp++] = n.left;
          stack[sp++] = n.left + 1;
        }
      } else if (ha) {
        stack[sp++] = n.left;
      } else if (hb) {
        stack[sp++] = n.left + 1;
      }
    }
  }
  if (!h.valid()) return Hit{};
  return h;
}

bool Scene::Occluded(const Ray& ray) const {
  if (nodes.empty()) return false;
  V3 inv(1 / ray.D.x, 1 / ray.D.y, 1 / ray.D.z);
  uint32_t stack[128];
  int sp = 0;
  stack[sp++] = 0;
  Hit h;
  h.t = ray.MaxT;
  while (sp) {
    const BvhNode& n = nodes[stack[--sp]];
    Float tn;
    if (!BoxHit(n, ray.O, inv, ray.MinT, ray.MaxT, tn)) continue;
    if (n.count) {
      for (uint32_t i = 0; i < n.count; i++) {
        Hit tmp;
        tmp.t = ray.MaxT;
        if (IntersectPrim(order[n.first + i], ray, tmp)) return true;
      }
    } else {
      stack[sp++] = n.left;
      stack[sp++] = n.left + 1;
    }
  }
  return false;
}

// scene.cpp:42-51 + HitShapeRecord::ComputeSurfaceInteraction (interaction.cpp:121-127)
bool Scene::RayIntersect(const Ray& ray, SurfaceInteraction& si) const {
  Hit h = Intersect(ray);
  si = SurfaceInteraction{};
  if (!h.valid()) {
    si.Wi = -ray.D;
    return false;
  }
  const PrimRef& pr = prims[h.prim];
  const Shape& sh = shapes[pr.shape];
  si.T = h.t;
  si.shape = (int)pr.shape;
  bool dPdUZeroCheck = true;
  if (sh.kind == Shape::Mesh) {  // mesh_base.cpp:38-82
    uint32_t face = pr.local * 3;
    uint32_t f0 = sh.idx[face], f1 = sh.idx[face + 1], f2 = sh.idx[face + 2];
    V3 p0 = sh.pos[f0], p1 = sh.pos[f1], p2 = sh.pos[f2];
    V3 bary(1.f - h.u - h.v, h.u, h.v);
    V3 dp0 = p1 - p0, dp1 = p2 - p0;
    si.P = p0 * bary.x + (p1 * bary.y + (p2 * bary.z));
    si.N = normalized(cross(dp0, dp1));
    if (!sh.hasUV) {
      si.UV = V2(h.u, h.v);
      auto st = CoordinateSystem(si.N);
      si.dPdU = st.first;
      si.dPdV = st.second;
    } else {
      V2 uv0 = sh.uv[f0], uv1 = sh.uv[f1], uv2 = sh.uv[f2];
      si.UV = V2(uv0.x * bary.x + (uv1.x * bary.y + (uv2.x * bary.z)),
                 uv0.y * bary.x + (uv1.y * bary.y + (uv2.y * bary.z)));
      V2 duv0(uv1.x - uv0.x, uv1.y - uv0.y), duv1(uv2.x - uv0.x, uv2.y - uv0.y);
      Float det = duv0.x * duv1.y - (duv0.y * duv1.x);
      Float invDet = det == 0 ? 0 : Rcp(det);
      if (invDet == 0) {
        si.dPdU = V3(0);
        si.dPdV = V3(0);
      } else {
        si.dPdU = (duv1.y * dp0 - (duv0.y * dp1)) * invDet;
        si.dPdV = (-duv1.x * dp0 + (duv0.x * dp1)) * invDet;
      }
    }
    if (sh.nrm.empty()) {
      si.Shading.N = si.N;
    } else {
      V3 n0 = sh.nrm[f0], n1 = sh.nrm[f1], n2 = sh.nrm[f2];
      V3 shN = n0 * bary.x + (n1 * bary.y + (n2 * bary.z));
      Float il = Rsqrt(sqnorm(shN));
      shN = shN * il;
      si.Shading.N = shN;
    }
  } else if (sh.kind == Shape::Rect) {  // rectangle.cpp:186-199
    V3 p = ray.At(h.t);
    si.P = sh.frame.N * dot(sh.toWorld.TranslationToWorld() - p, sh.frame.N) + p;
    si.N = sh.frame.N;
    si.Shading.N = sh.frame.N;
    si.dPdU = sh.frame.S;
    si.dPdV = sh.frame.T;
    si.UV = V2(h.u * Float(0.5) + Float(0.5), h.v * Float(0.5) + Float(0.5));
  } else {  // sphere.cpp:215-249
    V3 gn = normalized((ray.D * h.t + ray.O) - sh.center);
    si.Shading.N = gn;
    si.P = Fmadd(gn, V3(sh.radius), sh.center);
    V3 local = sh.toWorld.ApplyAffineToLocal(si.P);
    Float rd2 = Sqr(local.x) + Sqr(local.y);
    Float theta = UnitAngleZ(local);
    Float phi = std::atan2(local.y, local.x);
    if (phi < 0) phi += 2 * PI;
    si.UV = V2(phi / (2 * PI), theta / PI);
    si.dPdU = V3(-local.y, local.x, 0.f);
    Float rd = std::sqrt(rd2);
    Float invRd = Rcp(rd);
    Float cosPhi = local.x * invRd, sinPhi = local.y * invRd;
    si.dPdV = V3(local.z * cosPhi, local.z * sinPhi, -rd);
    if (rd == 0) si.dPdV = V3(1, 0, 0);
    si.dPdU = sh.toWorld.ApplyLinearToWorld(si.dPdU * (2 * PI));
    si.dPdV = sh.toWorld.ApplyLinearToWorld(si.dPdV * PI);
    si.N = si.Shading.N;
  }
  (void)dPdUZeroCheck;
  // interaction.cpp:45-53
  if (is_zero(si.dPdU)) {
    si.Shading.S = CoordinateSystem(si.Shading.N).first;
  } else {
    si.Shading.S = normalized(si.Shading.N * (-dot(si.Shading.N, si.dPdU)) + si.dPdU);
  }
  si.Shading.T = cross(si.Shading.N, si.Shading.S);
  si.Wi = si.ToLocal(-ray.D);
  return true;
}

bool Scene::IsOcclude(const V3& refP, const V3& refN, const V3& p) const {
  V3 o = OffsetP(refP, refN, p - refP);
  V3 d = p - o;
  Float dist = norm(d);
  if (dist < ShadowEpsilon) return true;
  d = d / dist;
  Ray r;
  r.O = o;
  r.D = d;
  r.MinT = 0;
  r.MaxT = dist * (1 - ShadowEpsilon);
  return Occluded(r);
}

void Scene::SampleLight(Float xi, int& index, Float& pdf) const {  // scene.cpp:65-77
  if (lights.size() < 2) {
    if (lights.size() == 1) {
      index = 0;
      pdf = 1;
    } else {
      index = -1;
      pdf = 0;
    }
    return;
  }
  uint32_t lightCount = (uint32_t)lights.size();
  Float li = xi * lightCount;
  index = (int)std::min(uint32_t(li), lightCount - 1);
  pdf = lightPdf;
}

int Scene::LightOf(const SurfaceInteraction& si) const {
  if (si.shape < 0) return envLight;
  return shapes[si.shape].light;
}

// area.cpp:42-45, skybox.cpp:53-63 (constant map)
// distribution.cpp:55-68
void Continuous1D::Build(const Float* f, size_t size) {
  pdf.assign(f, f + size);
  cdf.resize(size + 1);
  cdf[0] = 0;
  size_t count = pdf.size();
  for (size_t i = 1; i < count + 1; ++i) cdf[i] = cdf[i - 1] + pdf[i - 1] / count;
  sum = cdf[count];
  for (size_t i = 1; i < count + 1; i++) cdf[i] /= sum;
  normalization = Float(1.0 / sum);
}
// distribution.cpp:84-97
std::tuple<size_t, Float, Float> Continuous1D::Sample(Float xi) const {
  auto iter = std::lower_bound(cdf.begin(), cdf.end(), xi);
  size_t index = std::distance(cdf.begin(), iter);
  index = std::clamp(index - 1, size_t(0), cdf.size() - 2);
  Float du = xi - cdf[index];
  if ((cdf[index + 1] - cdf[index]) > 0) du /= (cdf[index + 1] - cdf[index]);
  Float p = pdf[index] * normalization;
  Float c = (index + du) / Count();
  return {index, c, p};
}
// distribution.cpp:103-129
void Continuous2D::Build(const Float* data, size_t nu, size_t nv) {
  conditional.resize(nv);
  for (size_t v = 0; v < nv; v++) conditional[v].Build(data + v * nu, nu);
  std::vector<Float> m(nv);
  for (size_t v = 0; v < nv; v++) m[v] = conditional[v].sum;
  marginal.Build(m.data(), m.size());
}
std::tuple<size_t, size_t, Float> Continuous2D::Sample(const V2& xi) const {
  auto [vj, d1, pdf1] = marginal.Sample(xi.y);
  auto [vi, d0, pdf0] = conditional[vj].Sample(xi.x);
  (void)d0;
  (void)d1;
  return {vi, vj, pdf0 * pdf1};
}
Float Continuous2D::Pdf(const V2& uv) const {
  size_t iu = std::clamp(size_t(uv.x * conditional[0].Count()), size_t(0), conditional[0].Count() - 1);
  size_t iv = std::clamp(size_t(uv.y * marginal.Count()), size_t(0), marginal.Count() - 1);
  return conditional[iv].pdf[iu] / marginal.sum;
}

Spectrum Scene::AreaRadiance(const Light& L, const V2& uv) const {
  return L.map ? L.map->Eval(TexSi{uv, V2(), V2()}) : L.radiance;
}

// Rectangle::EvalParamSurface (rectangle.cpp:236-250): position, normal and the
// norm of dPdU x dPdV (the unit frame axes) at uv
static void RectParam(const Shape& sh, const V2& uv, V3& P, V3& N, Float& dA) {
  V2 tmp(uv.x * 2 - 1, uv.y * 2 - 1);
  P = sh.toWorld.ApplyAffineToWorld(V3(tmp.x, tmp.y, 0));
  N = sh.frame.N;
  dA = norm(cross(sh.frame.S, sh.frame.T));
}

std::pair<PositionSample, Float> Scene::LightSamplePosition(int l, const V2& xi) const {
  const Light& L = lights[l];
  const Shape& sh = shapes[L.shape];
  if (!L.map || L.uniformMap) {
    PositionSample psr = sh.SamplePosition(xi);
    return {psr, psr.Pdf > 0 ? psr.Pdf : 0};
  }
  auto [iu, iv, pdf] = L.dist.Sample(xi);
  if (pdf <= 0) return {PositionSample(), Float(0)};
  Float y = iv / (Float)L.map->height;
  Float x = iu / (Float)L.map->width;
  PositionSample psr;
  Float dA;
  psr.UV = V2(x, y);
  RectParam(sh, psr.UV, psr.P, psr.N, dA);
  pdf /= dA;
  psr.Pdf = pdf;
  psr.IsDelta = false;
  return {psr, psr.Pdf > 0 ? psr.Pdf : 0};
}

// area.cpp:42-45, skybox.cpp:53-63
Spectrum Scene::EvalLight(int l, const SurfaceInteraction& si) const {
  const Light& L = lights[l];
  if (L.kind == Light::Area) {
    if (dot(si.ToWorld(si.Wi), si.N) < 0) return Spectrum(0);
    return L.map ? L.map->Eval(TexSi{si.UV, si.dUVdX, si.dUVdY}) : L.radiance;
  }
  if (L.kind == Light::Skybox) {
    if (!L.map) return L.radiance;
    V3 v = L.toWorld.ApplyLinearToLocal(-si.Wi);
    Float phi = std::atan2(v.x, -v.z);
    phi = (phi < 0) ? (phi + 2 * PI) : phi;
    Float theta = std::acos(std::clamp(v.y, Float(-1), Float(1)));
    TexSi tsi{V2(phi / (2 * PI), theta / PI), si.dUVdX, si.dUVdY};
    return L.map->Eval(tsi);
  }
  return Spectrum(0);
}

// scene.cpp:87-96 with area.cpp:47-75, skybox.cpp:65-86, point.cpp:33-49,
// projection.cpp:52-74 and the directional extension
std::pair<DirectionSample, Spectrum> Scene::SampleLightDirection(const V3& refP, Float xiL, const V2& xi) const {
  int index;
  Float pdf;
  SampleLight(xiL, index, pdf);
  if (index < 0) return {DirectionSample(), Spectrum(0)};
  auto r = SampleOneLightDirection(index, refP, xi);
  r.first.Pdf *= pdf;
  return r;
}

// Light::SampleDirection of light l.
std::pair<DirectionSample, Spectrum> Scene::SampleOneLightDirection(int index, const V3& refP, const V2& xi) const {
  DirectionSample dsr;
  Spectrum li(0);
  const Light& L = lights[index];
  if (L.kind == Light::Area && L.map && !L.uniformMap) {  // area.cpp:59-72: SurfaceInteraction::ToDsr leaves Pdf 0
    auto [iu, iv, pdf] = L.dist.Sample(xi);
    if (pdf <= 0) return {DirectionSample(), Spectrum(0)};
    V2 uv(iu / (Float)L.map->width, iv / (Float)L.map->height);
    Float dA;
    RectParam(shapes[L.shape], uv, dsr.P, dsr.N, dA);
    dsr.UV = uv;
    dsr.Pdf = 0;
    dsr.IsDelta = false;
    V3 rel = dsr.P - refP;
    dsr.Dist = norm(rel);
    dsr.Dir = rel / dsr.Dist;
    li = dot(-dsr.Dir, dsr.N) >= 0 ? L.map->Eval(TexSi{uv, V2(), V2()}) : Spectrum(0);
  } else if (L.kind == Light::Area) {
    dsr = shapes[L.shape].SampleDirection(refP, xi);
    li = dot(-dsr.Dir, dsr.N) >= 0 ? AreaRadiance(L, dsr.UV) : Spectrum(0);  // a chessboard at the sample's uv
  } else if (L.kind == Light::Skybox) {  // skybox.cpp:65-106
    Float radius = std::max(L.worldRadius, norm(refP - L.worldCenter));
    Float dist = 2 * radius;
    if (L.uniformMap) {
      V3 dir = normalized(SquareToUniformSphere(xi));
      Float phi = std::atan2(dir.x, -dir.z);
      phi = (phi < 0) ? (phi + 2 * PI) : phi;
      Float theta = std::acos(std::clamp(dir.y, Float(-1), Float(1)));
      V2 uv(phi / (2 * PI), theta / PI);
      V3 worldDir = L.toWorld.ApplyLinearToWorld(dir);
      dsr.P = worldDir * dist + refP;
      dsr.N = -worldDir;
      dsr.Pdf = SquareToUniformSpherePdf();
      dsr.Dir = worldDir;
      dsr.Dist = dist;
      dsr.IsDelta = false;
      li = L.map ? L.map->Eval(TexSi{uv, V2(), V2()}) : L.radiance;
    } else {
      // SampleLightDir (skybox.cpp:213-233)
      auto [iu, iv, pdf0] = L.dist.Sample(xi);
      Float pdfDir = pdf0;
      bool ok = pdfDir > 0;
      Float y = iv / (Float)L.map->height;
      Float x = iu / (Float)L.map->width;
      V2 uv(x, y);
      Float theta = y * PI;
      Float phi = x * 2 * PI;
      Float sinTheta = std::sin(theta);
      if (ok && sinTheta == 0) ok = false;
      if (!ok) {
        dsr.Pdf = 0;
        return {dsr, Spectrum(0)};
      }
      pdfDir /= (2 * PI * PI * sinTheta);
      V3 sph(std::cos(phi) * sinTheta, std::sin(phi) * sinTheta, std::cos(theta));  // SphericalCoordinates
      V3 dir(sph.y, sph.z, -sph.x);
      V3 worldDir = L.toWorld.ApplyLinearToWorld(dir);
      dsr.P = worldDir * dist + refP;
      dsr.N = -worldDir;
      dsr.Pdf = pdfDir;
      dsr.Dir = worldDir;
      dsr.Dist = dist;
      dsr.IsDelta = false;
      li = L.map->Eval(TexSi{uv, V2(), V2()});
    }
  } else if (L.kind == Light::Point) {  // point.cpp:33-49
    dsr.P = L.worldPos;
    dsr.N = V3(0);
    dsr.Pdf = 1;
    dsr.IsDelta = true;
    dsr.Dir = dsr.P - refP;
    Float dist2 = sqnorm(dsr.Dir);
    dsr.Dist = std::sqrt(dist2);
    Float invDist = Rcp(dsr.Dist);
    dsr.Dir = dsr.Dir * invDist;
    li = L.radiance * Sqr(invDist);
  } else if (L.kind == Light::Projection) {  // projection.cpp:52-74
    V3 local = L.toWorld.ApplyAffineToLocal(refP);
    V3 c = L.toClip.ApplyAffineToWorld(local);
    bool inRange = c.x >= 0 && c.x <= 1 && c.y >= 0 && c.y <= 1 && local.z > 0;
    if (inRange) {
      dsr.P = V3(L.toWorld.ToWorld.m[0][3], L.toWorld.ToWorld.m[1][3], L.toWorld.ToWorld.m[2][3]);
      dsr.N = normalized(L.toWorld.ApplyLinearToWorld(V3(0, 0, 1)));
      dsr.Pdf = 1;
      dsr.IsDelta = true;
      dsr.Dir = dsr.P - refP;
      Float squaredNorm = sqnorm(dsr.Dir);
      dsr.Dist = std::sqrt(squaredNorm);
      dsr.Dir = dsr.Dir * Rcp(dsr.Dist);
      dsr.UV = V2(c.x, c.y);
      Spectrum irr = L.map ? L.map->Eval(TexSi{dsr.UV, V2(), V2()}) : L.radiance;
      li = cmul(irr, L.scale) * PI / (Sqr(local.z) * dot(-dsr.Dir, dsr.N));
    }
  } else {
    Float radius = std::max(L.worldRadius, norm(refP - L.worldCenter));
    Float dist = 2 * radius;
    V3 worldDir = -L.direction;
    dsr.P = worldDir * dist + refP;
    dsr.N = L.direction;
    dsr.Pdf = 1;
    dsr.Dir = worldDir;
    dsr.Dist = dist;
    dsr.IsDelta = true;
    li = L.radiance;
  }
  return {dsr, li};
}

// Skybox::PdfDirection (skybox.cpp:108-127)
static Float SkyPdfDirection(const Light& L, const V3& dir) {
  if (L.uniformMap) return SquareToUniformSpherePdf();
  V3 v = L.toWorld.ApplyAffineToLocal(dir);
  Float theta = std::acos(std::clamp(v.y, Float(-1), Float(1)));
  Float sinTheta = std::sin(theta);
  if (sinTheta == 0) return 0;
  Float phi = std::atan2(v.x, -v.z);
  phi = (phi < 0) ? (phi + 2 * PI) : phi;
  V2 uv(phi / (2 * PI), theta / PI);
  Float pdf = L.dist.Pdf(uv);
  return pdf / (2 * PI * PI * sinTheta);
}

// scene.cpp:98-103 with area.cpp:77-91, skybox.cpp:88-106
Float Scene::PdfLightDirection(int l, const V3& refP, const DirectionSample& dsr) const {
  const Light& L = lights[l];
  Float p = 0;
  if (L.kind == Light::Area && L.map && !L.uniformMap) {  // area.cpp:81-90
    Float pdf = L.dist.Pdf(dsr.UV);
    if (pdf > 0) {
      V3 P, N;
      Float dA;
      RectParam(shapes[L.shape], dsr.UV, P, N, dA);
      Float dp = dot(dsr.Dir, dsr.N);
      p = pdf * Sqr(dsr.Dist) / (dA * -dp);
    }
  } else if (L.kind == Light::Area) {
    p = dot(-dsr.Dir, dsr.N) >= 0 ? shapes[L.shape].PdfDirection(refP, dsr) : 0;
  } else if (L.kind == Light::Skybox) {
    p = SkyPdfDirection(L, dsr.Dir);
  }
  return p * lightPdf;
}

}  // namespace orc

namespace orc {

// SquareToUniformDiskConcentric (warp.cpp:80-95)
static V2 SquareToUniformDiskConcentric(const V2& xi2) {
  Float x = Fmadd(2, xi2.x, -1), y = Fmadd(2, xi2.y, -1);
  bool quadrant = std::abs(x) < std::abs(y);
  Float r = quadrant ? y : x, rp = quadrant ? x : y;
  Float phi0 = Float(0.25) * PI * rp / r;
  if (quadrant) phi0 = Float(0.5) * PI - phi0;
  if (x == 0 && y == 0) phi0 = 0;
  return V2(r * std::cos(phi0), r * std::sin(phi0));
}

// Light::SampleRay
bool Scene::LightSampleRay(int l, const V2& xi2, const V2& xi3, Ray& ray, Spectrum& li) const {
  const Light& L = lights[l];
  ray = Ray();
  ray.MinT = 0;
  ray.MaxT = std::numeric_limits<Float>::max();
  if (L.kind == Light::Area) {  // area.cpp:120-128
    auto pp = LightSamplePosition(l, xi2);
    const PositionSample& psr = pp.first;
    Float pdf = pp.second;
    V3 local = SquareToCosineHemisphere(xi3);
    Frame fr(psr.N);  // SurfaceInteraction(psr)
    V3 d = fr.ToWorld(local);
    ray = SpawnRay(psr.P, psr.N, d);
    Spectrum eval = AreaRadiance(L, psr.UV);  // Eval(si) with no incident direction: dot(0, N) >= 0
    li = eval * PI / pdf;
    return true;
  }
  if (L.kind == Light::Point) {  // point.cpp:67-71
    ray.O = L.worldPos;
    ray.D = SquareToUniformSphere(xi3);
    li = L.radiance * 4 * PI;
    return true;
  }
  if (L.kind == Light::Projection) {  // projection.cpp:93-104
    V2 uv = xi3;
    V3 nearP = L.toClip.ApplyAffineToLocal(V3(uv.x, uv.y, 0));
    V3 nearDir = normalized(nearP);
    ray.O = V3(L.toWorld.ToWorld.m[0][3], L.toWorld.ToWorld.m[1][3], L.toWorld.ToWorld.m[2][3]);
    ray.D = L.toWorld.ApplyLinearToWorld(nearDir);
    Spectrum irr = L.map ? L.map->Eval(TexSi{uv, V2(), V2()}) : L.radiance;
    li = irr * PI * L.cameraArea;  // SampleRay leaves out the light's scale
    return true;
  }
  Float R = L.worldRadius;
  V2 offset = SquareToUniformDiskConcentric(xi2);
  if (L.kind == Light::Skybox) {  // skybox.cpp:135-163
    Float pdfDir;
    V2 uv;
    if (L.uniformMap) {
      pdfDir = SquareToUniformSpherePdf();
      uv = xi3;
    } else {
      auto [iu, iv, pdf0] = L.dist.Sample(xi3);
      pdfDir = pdf0;
      if (pdf0 <= 0) return false;
      Float vy = iv / (Float)L.map->height, vx = iu / (Float)L.map->width;
      uv = V2(vx, vy);
      Float sinTheta = std::sin(vy * PI);
      if (sinTheta == 0) return false;
      pdfDir /= (2 * PI * PI * sinTheta);
    }
    if (pdfDir <= 0) return false;
    Float theta = uv.y * PI, phi = uv.x * PI * 2;
    V3 sph(std::cos(phi) * std::sin(theta), std::sin(phi) * std::sin(theta), std::cos(theta));
    V3 d(sph.y, sph.z, -sph.x);
    V3 worldD = L.toWorld.ApplyAffineToWorld(-d);
    V3 perp = Frame(d).ToWorld(V3(offset.x, offset.y, 0));
    ray.O = L.worldCenter + (perp - worldD) * R;
    ray.D = worldD;
    Spectrum c = L.map ? L.map->Eval(TexSi{uv, V2(), V2()}) : L.radiance;
    li = c * PI * Sqr(R) / pdfDir;
    return true;
  }
  // directional (extension): parallel rays through a disk covering the world sphere
  V3 perp = Frame(L.direction).ToWorld(V3(offset.x, offset.y, 0));
  ray.O = L.worldCenter + (perp - L.direction) * R;
  ray.D = L.direction;
  li = L.radiance * PI * Sqr(R);
  return true;
}

// SampleLe of each light. The directional extension has none: scenes pairing it
// with bdpt are rejected when loaded.
Scene::LeSample Scene::LightSampleLe(int l, const V2& xi2, const V2& xi3) const {
  const Light& L = lights[l];
  LeSample r;
  r.ray.MinT = 0;
  r.ray.MaxT = std::numeric_limits<Float>::max();
  if (L.kind == Light::Area) {  // area.cpp:130-140
    auto pp = LightSamplePosition(l, xi2);
    r.psr = pp.first;
    r.pdfPos = pp.second;
    V3 local = SquareToCosineHemisphere(xi3);
    r.pdfDir = SquareToCosineHemispherePdf(local);
    Frame fr(r.psr.N);  // SurfaceInteraction(psr)
    r.ray = SpawnRay(r.psr.P, r.psr.N, fr.ToWorld(local));
    r.le = AreaRadiance(L, r.psr.UV);  // Eval(si) with no incident direction: dot(0, N) >= 0
  } else if (L.kind == Light::Point) {  // point.cpp:75-85
    r.psr.P = L.worldPos;
    r.psr.N = V3(0);
    r.psr.UV = V2(0, 0);
    r.psr.Pdf = 1;
    r.psr.IsDelta = true;
    r.pdfPos = 1;
    V3 local = SquareToUniformSphere(xi3);
    r.pdfDir = SquareToUniformSpherePdf();
    Frame fr(r.psr.N);
    r.ray = SpawnRay(r.psr.P, r.psr.N, fr.ToWorld(local));
    r.le = L.radiance;
  } else if (L.kind == Light::Projection) {  // projection.cpp:107-120
    r.psr.P = V3(L.toWorld.ToWorld.m[0][3], L.toWorld.ToWorld.m[1][3], L.toWorld.ToWorld.m[2][3]);
    r.psr.N = normalized(L.toWorld.ApplyLinearToWorld(V3(0, 0, 1)));
    r.psr.UV = V2(Float(0.5), Float(0.5));
    r.psr.Pdf = 1;
    r.psr.IsDelta = true;
    r.pdfPos = 1;
    V3 nearP = L.toClip.ApplyAffineToLocal(V3(xi3.x, xi3.y, 0));
    V3 nearDir = normalized(nearP);
    r.ray.O = r.psr.P;
    r.ray.D = L.toWorld.ApplyLinearToWorld(nearDir);
    r.le = L.map ? L.map->Eval(TexSi{xi3, V2(), V2()}) : L.radiance;  // the irradiance without the light's scale
    r.pdfDir = 1 / (L.cameraArea * PI);
  } else if (L.kind == Light::Skybox) {  // skybox.cpp:170-204
    Float R = L.worldRadius;
    V2 offset = SquareToUniformDiskConcentric(xi2);
    Float pdfDir;
    V2 uv;
    if (L.uniformMap) {
      pdfDir = SquareToUniformSpherePdf();
      uv = xi3;
    } else {
      auto [iu, iv, pdf0] = L.dist.Sample(xi3);
      pdfDir = pdf0;
      if (pdf0 <= 0) return LeSample();
      Float vy = iv / (Float)L.map->height, vx = iu / (Float)L.map->width;
      uv = V2(vx, vy);
      Float sinTheta = std::sin(vy * PI);
      if (sinTheta == 0) return LeSample();
      pdfDir /= (2 * PI * PI * sinTheta);
    }
    if (pdfDir <= 0) return LeSample();
    Float theta = uv.y * PI, phi = uv.x * PI * 2;
    V3 sph(std::cos(phi) * std::sin(theta), std::sin(phi) * std::sin(theta), std::cos(theta));
    V3 d(sph.y, sph.z, -sph.x);
    V3 worldD = L.toWorld.ApplyAffineToWorld(-d);
    V3 perp = Frame(d).ToWorld(V3(offset.x, offset.y, 0));
    r.ray.O = L.worldCenter + (perp - worldD) * R;
    r.ray.D = worldD;
    r.le = L.map ? L.map->Eval(TexSi{uv, V2(), V2()}) : L.radiance;
    r.pdfPos = 1 / (PI * Sqr(R));
    r.pdfDir = pdfDir;
    r.psr.P = r.ray.O;
    r.psr.N = r.ray.D;
    r.psr.UV = uv;
    r.psr.Pdf = r.pdfPos;
    r.psr.IsDelta = false;
  } else {
    throw std::runtime_error("bdpt: the directional light is not supported");
  }
  return r;
}

std::pair<Float, Float> Scene::LightPdfLe(int l, const PositionSample& psr, const V3& dir) const {
  const Light& L = lights[l];
  if (L.kind == Light::Area) {  // area.cpp:142-147
    Frame fr(psr.N);
    Float pdfPos = shapes[L.shape].PdfPosition();
    Float pdfDir = SquareToCosineHemispherePdf(fr.ToLocal(dir));
    return {pdfPos, std::abs(pdfDir)};
  }
  if (L.kind == Light::Point) return {Float(0), std::abs(SquareToUniformSpherePdf())};  // point.cpp:87-91
  if (L.kind == Light::Projection) {  // projection.cpp:122-133
    V3 refP = L.toWorld.ApplyAffineToLocal(psr.P);
    V3 ndcPos = L.toClip.ApplyAffineToWorld(refP);
    Float pdfDir;
    if (ndcPos.x < 0 || ndcPos.x >= 1 || ndcPos.y < 0 || ndcPos.y >= 1 || ndcPos.z <= 0)
      pdfDir = 0;
    else
      pdfDir = 1 / (L.cameraArea * PI);
    return {Float(0), std::abs(pdfDir)};
  }
  if (L.kind == Light::Skybox) {  // skybox.cpp:206-212
    return {1 / (PI * Sqr(L.worldRadius)), SkyPdfDirection(L, dir)};
  }
  throw std::runtime_error("bdpt: the directional light is not supported");
}

}  // namespace orc
