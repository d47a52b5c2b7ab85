// Host scene compilation (see host_scene.h). Float arithmetic here follows the
// reference's FP32 expression order (compiled with -ffp-contract=off) so that
// transformed geometry is bit-identical to what the reference's scene build
// produces from the same JSON.
#include "host_scene.h"

#include "host_image.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>
#include <fstream>
#include <map>
#include <sstream>
#include <tuple>

namespace rad {

namespace {

constexpr float kPiF = static_cast<float>(3.1415926535897932);

struct F3 {
  float x = 0, y = 0, z = 0;
  F3() = default;
  F3(float a, float b, float c) : x(a), y(b), z(c) {}
  float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
F3 operator+(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
F3 operator-(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
F3 operator*(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
float Dot(F3 a, F3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
F3 Cross(F3 a, F3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
float Norm(F3 a) { return std::sqrt(Dot(a, a)); }
F3 Normalize(F3 a) {
  float n = Dot(a, a);
  if (n > 0) {
    float s = std::sqrt(n);
    return {a.x / s, a.y / s, a.z / s};
  }
  return a;
}
F3 Min3(F3 a, F3 b) { return {(b.x < a.x) ? b.x : a.x, (b.y < a.y) ? b.y : a.y, (b.z < a.z) ? b.z : a.z}; }
F3 Max3(F3 a, F3 b) { return {(a.x < b.x) ? b.x : a.x, (a.y < b.y) ? b.y : a.y, (a.z < b.z) ? b.z : a.z}; }

// ---- ConfigNode-style readers (rad.core/include/rad/core/config_node.h:10-170)
float Num(const JValue& v, const char* what) {
  if (!v.isNum()) throw ConfigError(std::string("node type is not number: ") + what);
  return (float)v.n;
}
F3 Vec3(const JValue& v, const char* what) {
  if (v.isNum()) return F3((float)v.n, (float)v.n, (float)v.n);
  if (!v.isArr() || v.a.size() != 3) throw ConfigError(std::string("node array size must be 3: ") + what);
  return F3(Num(v.a[0], what), Num(v.a[1], what), Num(v.a[2], what));
}
float RF(const JValue* c, const char* k, float d) {
  const JValue* v = c ? c->get(k) : nullptr;
  return v ? Num(*v, k) : d;
}
int RI(const JValue* c, const char* k, int d) {
  const JValue* v = c ? c->get(k) : nullptr;
  return v ? (int)Num(*v, k) : d;
}
bool RB(const JValue* c, const char* k, bool d) {
  const JValue* v = c ? c->get(k) : nullptr;
  if (!v) return d;
  if (v->type != JValue::kBool) throw ConfigError(std::string("node type is not bool: ") + k);
  return v->b;
}
std::string RS(const JValue* c, const char* k, const std::string& d) {
  const JValue* v = c ? c->get(k) : nullptr;
  if (!v) return d;
  if (!v->isStr()) throw ConfigError(std::string("node type is not string: ") + k);
  return v->s;
}
F3 RV(const JValue* c, const char* k, F3 d) {
  const JValue* v = c ? c->get(k) : nullptr;
  return v ? Vec3(*v, k) : d;
}
std::string TypeOf(const JValue& v) {
  const JValue* t = v.get("type");
  if (!t || !t->isStr()) throw ConfigError("no child: type");
  return t->s;
}

// ---- transforms (transform.cpp:51-95)
struct Xf {
  M4f w, l;  // to world, to local
  explicit Xf(const M4f& toWorld) : w(toWorld) {
    if (!InvertM4f(toWorld, l)) throw ConfigError("matrix is not invertible");
  }
  static F3 Aff(const M4f& M, F3 v) {
    float r[4];
    for (int i = 0; i < 4; i++) r[i] = ((M.m[i][0] * v.x + M.m[i][1] * v.y) + M.m[i][2] * v.z) + M.m[i][3];
    return F3(r[0] / r[3], r[1] / r[3], r[2] / r[3]);
  }
  static F3 Lin(const M4f& M, F3 v) {
    return F3((M.m[0][0] * v.x + M.m[0][1] * v.y) + M.m[0][2] * v.z, (M.m[1][0] * v.x + M.m[1][1] * v.y) + M.m[1][2] * v.z,
              (M.m[2][0] * v.x + M.m[2][1] * v.y) + M.m[2][2] * v.z);
  }
  F3 AffW(F3 v) const { return Aff(w, v); }
  F3 LinW(F3 v) const { return Lin(w, v); }
  F3 NrmW(F3 v) const {
    const M4f& M = l;
    return F3((M.m[0][0] * v.x + M.m[1][0] * v.y) + M.m[2][0] * v.z, (M.m[0][1] * v.x + M.m[1][1] * v.y) + M.m[2][1] * v.z,
              (M.m[0][2] * v.x + M.m[1][2] * v.y) + M.m[2][2] * v.z);
  }
  bool Identity() const {
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 4; j++)
        if (w.m[i][j] != (i == j ? 1.f : 0.f)) return false;
    return true;
  }
  bool NonUniformScale() const {
    float a = Dot(LinW(F3(1, 0, 0)), LinW(F3(1, 0, 0)));
    float b = Dot(LinW(F3(0, 1, 0)), LinW(F3(0, 1, 0)));
    float c = Dot(LinW(F3(0, 0, 1)), LinW(F3(0, 0, 1)));
    return std::abs(a - b) > 0.0001f || std::abs(a - c) > 0.0001f;
  }
};

void RowsOf(const M4f& M, float* out12) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 4; j++) out12[i * 4 + j] = M.m[i][j];
}

// config_node_ext.cpp:7-27
void Rotation(const JValue& n, float R[3][3]) {
  if (n.isObj()) {
    F3 axis = RV(&n, "axis", F3(0, 1, 0));
    float ang = RF(&n, "angle", 0) * (kPiF / 180.f);
    float s = std::sin(ang), c = std::cos(ang);
    F3 sa = axis * s, c1 = axis * (1.f - c);
    float t;
    t = c1.x * axis.y; R[0][1] = t - sa.z; R[1][0] = t + sa.z;
    t = c1.x * axis.z; R[0][2] = t + sa.y; R[2][0] = t - sa.y;
    t = c1.y * axis.z; R[1][2] = t - sa.x; R[2][1] = t + sa.x;
    R[0][0] = c1.x * axis.x + c;
    R[1][1] = c1.y * axis.y + c;
    R[2][2] = c1.z * axis.z + c;
  } else if (n.isArr() && n.a.size() == 9) {
    for (int k = 0; k < 9; k++) R[k / 3][k % 3] = Num(n.a[k], "rotate");
  } else if (n.isArr() && n.a.size() == 4) {
    float x = Num(n.a[0], "q"), y = Num(n.a[1], "q"), z = Num(n.a[2], "q"), w = Num(n.a[3], "q");
    float tx = 2 * x, ty = 2 * y, tz = 2 * z;
    float twx = tx * w, twy = ty * w, twz = tz * w, txx = tx * x, txy = ty * x, txz = tz * x;
    float tyy = ty * y, tyz = tz * y, tzz = tz * z;
    R[0][0] = 1 - (tyy + tzz); R[0][1] = txy - twz; R[0][2] = txz + twy;
    R[1][0] = txy + twz; R[1][1] = 1 - (txx + tzz); R[1][2] = tyz - twx;
    R[2][0] = txz - twy; R[2][1] = tyz + twx; R[2][2] = 1 - (txx + tyy);
  } else {
    throw ConfigError("rotate array must be mat3 or quaternion");
  }
}

// config_node_ext.cpp:52-71
M4f Transform(const JValue& n) {
  M4f r = M4f::Identity();
  if (n.isArr()) {
    if (n.a.size() != 16) throw ConfigError("node array size must be 16");
    for (int k = 0; k < 16; k++) r.m[k / 4][k % 4] = Num(n.a[k], "to_world");
    return r;
  }
  if (!n.isObj()) throw ConfigError("transform node must be mat4 or object");
  F3 t = RV(&n, "translate", F3(0, 0, 0));
  F3 s = RV(&n, "scale", F3(1, 1, 1));
  float R[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  if (const JValue* rn = n.get("rotate")) Rotation(*rn, R);
  for (int i = 0; i < 3; i++) {
    for (int j = 0; j < 3; j++) r.m[i][j] = R[i][j] * s[j];
    r.m[i][3] = t[i];
  }
  return r;
}

// ---- assets: OBJ (wavefront_obj_reader.cpp) and Mitsuba .vol (volume_reader.cpp:65-124)
struct ObjData {
  std::vector<F3> p, n;
  std::vector<std::pair<float, float>> t;
  struct Face {
    int v[3], vt[3], vn[3];
  };
  std::vector<Face> faces;
  std::vector<std::pair<std::string, std::vector<size_t>>> objects;
};

ObjData LoadObj(const std::string& path) {
  std::ifstream in(path, std::ios::binary);
  if (!in) throw IoError("cannot open model " + path);
  std::stringstream ss;
  ss << in.rdbuf();
  const std::string text = ss.str();
  ObjData d;
  size_t i = 0, n = text.size();
  int lineNo = 0;
  auto skipSpaces = [&](size_t& k) {
    while (k < n && (text[k] == ' ' || text[k] == '\t')) k++;
  };
  while (i < n) {
    size_t e = text.find('\n', i);
    if (e == std::string::npos) e = n;
    lineNo++;
    size_t k = i;
    skipSpaces(k);
    size_t c0 = k;
    while (k < e && text[k] != ' ' && text[k] != '\t' && text[k] != '\r') k++;
    std::string cmd = text.substr(c0, k - c0);
    const char* p = text.c_str() + k;
    char* endp = nullptr;
    auto num = [&]() {
      float v = std::strtof(p, &endp);
      if (endp == p) throw IoError(path + ":" + std::to_string(lineNo) + ": bad number");
      p = endp;
      return v;
    };
    if (cmd == "v") {
      float a = num(), b = num(), c = num();
      d.p.emplace_back(a, b, c);
    } else if (cmd == "vn") {
      float a = num(), b = num(), c = num();
      d.n.emplace_back(a, b, c);
    } else if (cmd == "vt") {
      float a = num(), b = num();
      d.t.emplace_back(a, b);
    } else if (cmd == "f") {
      ObjData::Face f{};
      size_t q = k;
      for (int v = 0; v < 3; v++) {
        skipSpaces(q);
        size_t t0 = q;
        while (q < e && text[q] != ' ' && text[q] != '\t' && text[q] != '\r') q++;
        std::string tok = text.substr(t0, q - t0);
        if (tok.empty()) throw IoError(path + ":" + std::to_string(lineNo) + ": can't parse face");
        int a = 0, b = 0, cc = 0;
        size_t s1 = tok.find('/');
        if (s1 == std::string::npos) {
          a = std::atoi(tok.c_str());
        } else {
          a = std::atoi(tok.substr(0, s1).c_str());
          size_t s2 = tok.find('/', s1 + 1);
          if (s2 == std::string::npos) {
            b = std::atoi(tok.substr(s1 + 1).c_str());
          } else {
            if (s2 > s1 + 1) b = std::atoi(tok.substr(s1 + 1, s2 - s1 - 1).c_str());
            cc = std::atoi(tok.substr(s2 + 1).c_str());
          }
        }
        f.v[v] = a;
        f.vt[v] = b;
        f.vn[v] = cc;
      }
      if (!d.objects.empty()) d.objects.back().second.push_back(d.faces.size());
      d.faces.push_back(f);
    } else if (cmd == "o" || cmd == "g") {
      size_t q = k;
      skipSpaces(q);
      size_t q2 = e;
      while (q2 > q && (text[q2 - 1] == ' ' || text[q2 - 1] == '\r' || text[q2 - 1] == '\t')) q2--;
      d.objects.push_back({text.substr(q, q2 - q), {}});
    }
    i = e + 1;
  }
  return d;
}

struct ModelData {
  std::vector<F3> pos, nrm;
  std::vector<std::pair<float, float>> uv;
  std::vector<uint32_t> idx;
};

// wavefront_obj_reader.cpp:408-452: unique (v, vn, vt) triples become vertices
ModelData ToModel(const ObjData& f, const std::vector<size_t>* list) {
  auto cvt = [](int i, size_t count) { return i >= 0 ? size_t(i - 1) : count + (size_t)(long long)i; };
  ModelData m;
  std::map<std::tuple<int, int, int>, uint32_t> unique;
  size_t nf = list ? list->size() : f.faces.size();
  for (size_t q = 0; q < nf; q++) {
    const auto& face = f.faces[list ? (*list)[q] : q];
    for (int k = 0; k < 3; k++) {
      auto key = std::make_tuple(face.v[k], face.vn[k], face.vt[k]);
      auto it = unique.find(key);
      uint32_t index;
      if (it == unique.end()) {
        index = (uint32_t)m.pos.size();
        unique.emplace(key, index);
        size_t pi = cvt(face.v[k], f.p.size());
        if (pi >= f.p.size()) throw IoError("face vertex index out of range");
        m.pos.push_back(f.p[pi]);
        if (face.vn[k] != 0) {
          size_t ni = cvt(face.vn[k], f.n.size());
          if (ni >= f.n.size()) throw IoError("face normal index out of range");
          m.nrm.push_back(f.n[ni]);
        }
        if (face.vt[k] != 0) {
          size_t ti = cvt(face.vt[k], f.t.size());
          if (ti >= f.t.size()) throw IoError("face uv index out of range");
          m.uv.push_back(f.t[ti]);
        }
      } else {
        index = it->second;
      }
      m.idx.push_back(index);
    }
  }
  if (!m.nrm.empty() && m.nrm.size() != m.pos.size()) throw IoError("model mixes faces with and without normals");
  if (!m.uv.empty() && m.uv.size() != m.pos.size()) throw IoError("model mixes faces with and without uvs");
  return m;
}

struct VolData {
  std::vector<float> data;
  int nx = 0, ny = 0, nz = 0, ch = 1;
  float max = 0;
};

VolData LoadVol(const std::string& path) {
  std::ifstream in(path, std::ios::binary);
  if (!in) throw IoError("cannot open volume " + path);
  char hdr[4];
  in.read(hdr, 4);
  if (!in || hdr[0] != 'V' || hdr[1] != 'O' || hdr[2] != 'L') throw IoError("not a mitsuba vol file: " + path);
  if (hdr[3] != 3) throw IoError("only version 3 mitsuba vol files are supported");
  int32_t type, sx, sy, sz, ch;
  in.read((char*)&type, 4);
  if (type != 1) throw IoError("mitsuba vol must be Float32");
  in.read((char*)&sx, 4);
  in.read((char*)&sy, 4);
  in.read((char*)&sz, 4);
  in.read((char*)&ch, 4);
  if (ch != 1 && ch != 3) throw IoError("mitsuba vol must have 1 or 3 channels");
  if (sx <= 0 || sy <= 0 || sz <= 0) throw IoError("bad vol size");
  float dims[6];
  in.read((char*)dims, 24);
  VolData v;
  v.nx = sx;
  v.ny = sy;
  v.nz = sz;
  v.ch = ch;
  v.data.resize((size_t)sx * sy * sz * ch);
  in.read((char*)v.data.data(), (std::streamsize)(v.data.size() * 4));
  if (!in) throw IoError("vol file truncated: " + path);
  float mx = -INFINITY;
  for (float x : v.data) mx = std::max(mx, x);
  v.max = mx;
  return v;
}

std::string Join(const std::string& base, const std::string& loc) {
  if (loc.empty() || loc[0] == '/' || base.empty()) return loc;
  return base + "/" + loc;
}

// ---- image assets (rad.core asset/image_stb.cpp:12-104, image_hdr.cpp:12-57,
// image_exr.cpp:12-95): decoded (host_image.cpp) and converted to float texels.
struct ImageAsset {
  int width = 0, height = 0, channels = 0;  // channels: 1 (mono) or 3 (rgb)
  std::vector<float> px;                    // texel (x, y) at (y * width + x) * channels
  std::string type;
};

std::string ReadAll(const std::string& path) {
  std::ifstream in(path, std::ios::binary);
  if (!in) throw IoError("cannot open " + path);
  std::stringstream ss;
  ss << in.rdbuf();
  return ss.str();
}

// Color24f::ToLinear (color.h:41-46)
float SrgbToLinear(float v) { return v <= 0.04045f ? v * (1.0f / 12.92f) : std::pow((v + 0.055f) * (1.0f / 1.055f), 2.4f); }

ImageAsset LoadImageAsset(const JValue& a, const std::string& type, const std::string& path) {
  ImageAsset im;
  im.type = type;
  std::string bytes = ReadAll(path);
  try {
    if (type == "image_default") {
      int ch = RI(&a, "channel", 3);
      bool flip = RB(&a, "is_flip_y", true);
      bool lin = RB(&a, "is_to_linear", ch == 3);
      if (ch != 1 && ch != 3) throw ConfigError("channel must be 1 or 3");
      img::Ldr l = img::LoadLdr(bytes, ch, flip);
      im.width = l.width;
      im.height = l.height;
      im.channels = ch;
      im.px.resize(l.px.size());
      for (size_t i = 0; i < l.px.size(); i++) {
        float v = (float)l.px[i] / 255.f;  // color /= 255 (image_stb.cpp:59-69, :84-85)
        im.px[i] = (ch == 3 && lin) ? SrgbToLinear(v) : v;
      }
    } else {
      img::Hdr h = type == "image_hdr" ? img::LoadHdr(bytes, RB(&a, "is_flip_y", false)) : img::LoadExr(bytes);
      im.width = h.width;
      im.height = h.height;
      im.channels = 3;
      im.px = std::move(h.px);
    }
  } catch (const std::runtime_error& e) {
    if (dynamic_cast<const ConfigError*>(&e)) throw;
    throw IoError(std::string(e.what()) + ": " + path);
  }
  return im;
}

// ---- textures (texture.h:47-90, config_node_ext.h:17-45, bitmap.cpp, chessboard.cpp)
struct TexEnv {
  HostScene* hs = nullptr;  // null: records built without a scene (no textures)
  const std::map<std::string, ImageAsset>* images = nullptr;
};

// MipMap::FilterBilinear (bitmap.cpp:200-214) on an explicit level
void MipBilinear(const float* img, uint32_t W, uint32_t H, int C, uint32_t pu, uint32_t pv, float fu, float fv,
                 float* out) {
  int32_t dpu = (fu > pu + 0.5f) ? 1 : -1;
  int32_t dpv = (fv > pv + 0.5f) ? 1 : -1;
  uint32_t apu = std::min(pu + (uint32_t)dpu, W - 1), apv = std::min(pv + (uint32_t)dpv, H - 1);
  float du = std::min(std::abs(fu - pu - 0.5f), 1.f);
  float dv = std::min(std::abs(fv - pv - 0.5f), 1.f);
  for (int c = 0; c < C; c++) {
    float a = img[((size_t)pv * W + pu) * C + c], b = img[((size_t)pv * W + apu) * C + c];
    float d = img[((size_t)apv * W + pu) * C + c], e = img[((size_t)apv * W + apu) * C + c];
    out[c] = (a * (1 - du) + b * du) * (1 - dv) + (d * (1 - du) + e * du) * dv;
  }
}

// MipMap construction (bitmap.cpp:27-64): each coarser texel averages four
// bilinear lookups at the integer texel corners of the finer level.
void BuildMips(TexRec& t, std::vector<float> level0, int maxLevel, std::vector<float>& pool) {
  uint32_t W = t.width, H = t.height;
  int C = (int)t.channels;
  if (maxLevel != 0 && ((W % 2 != 0) || (H % 2 != 0))) maxLevel = 0;  // bitmap.cpp:30-33
  uint32_t real = maxLevel < 0 ? 1 + (uint32_t)std::log2((double)std::max(W, H)) : (uint32_t)maxLevel;
  real = std::max(real, 1u);
  if (real > (uint32_t)kMaxMipLevels) throw ConfigError("bitmap: more than 16 mip levels");
  t.levels = real;
  std::vector<float> last = std::move(level0);
  uint32_t lw = W, lh = H;
  for (uint32_t a = 0; a < real; a++) {
    if (a > 0) {
      uint32_t nw = std::max(1u, lw / 2), nh = std::max(1u, lh / 2);
      std::vector<float> next((size_t)nw * nh * C);
      auto corner = [&](uint32_t u, uint32_t v, float* o) {
        uint32_t pu = t.wrap ? u % lw : std::min(u, lw - 1);
        uint32_t pv = t.wrap ? v % lh : std::min(v, lh - 1);
        MipBilinear(last.data(), lw, lh, C, pu, pv, pu + 1.f, pv + 1.f, o);
      };
      for (uint32_t j = 0; j < nh; j++)
        for (uint32_t i = 0; i < nw; i++) {
          float a0[3], a1[3], a2[3], a3[3];
          corner(i * 2, j * 2, a0);
          corner(i * 2 + 1, j * 2, a1);
          corner(i * 2, j * 2 + 1, a2);
          corner(i * 2 + 1, j * 2 + 1, a3);
          for (int c = 0; c < C; c++) next[((size_t)j * nw + i) * C + c] = (a0[c] + a1[c] + a2[c] + a3[c]) * 0.25f;
        }
      last = std::move(next);
      lw = nw;
      lh = nh;
    }
    if (pool.size() + last.size() > 0xffffffffull) throw ConfigError("texture pool exceeds 2^32 texels");
    t.levelOffset[a] = (uint32_t)pool.size();
    pool.insert(pool.end(), last.begin(), last.end());
  }
}

// ConfigNodeReadTexture for a texture node (a number / array is a constant).
uint32_t AddTexture(const JValue& v, int channels, TexEnv& env) {
  HostScene& hs = *env.hs;
  TexRec t;
  std::memset(&t, 0, sizeof(t));
  t.channels = (uint32_t)channels;
  uint32_t index = (uint32_t)hs.tex.size();
  hs.tex.push_back(t);
  if (v.isNum() || v.isArr()) {
    t.kind = TEX_CONST;
    if (channels == 3) {
      F3 c = Vec3(v, "texture");
      t.value[0] = c.x;
      t.value[1] = c.y;
      t.value[2] = c.z;
    } else {
      t.value[0] = Num(v, "texture");
    }
  } else {
    std::string type = TypeOf(v);
    if (type == "bitmap") {  // bitmap.cpp:273-316
      t.kind = TEX_BITMAP;
      const JValue* an = v.get("asset_name");
      if (!an || !an->isStr()) throw ConfigError("no child: asset_name");
      auto it = env.images->find(an->s);
      if (it == env.images->end()) throw ConfigError("unknown asset: " + an->s);
      const ImageAsset& im = it->second;
      if (im.channels != channels) {
        if (im.type != "image_default") throw ConfigError(im.type + " does not support single channel");
        throw ConfigError(std::string("loaded image ") + an->s + (im.channels == 1 ? " is mono" : " is rgb"));
      }
      std::string f = RS(&v, "filter", "bilinear");
      t.filter = f == "nearest" ? TF_NEAREST : f == "trilinear" ? TF_TRILINEAR : f == "anisotropic" ? TF_ANISO : TF_BILINEAR;
      t.wrap = RS(&v, "wrap", "clamp") == "repeat" ? 1u : 0u;
      bool mip = t.filter == TF_TRILINEAR || t.filter == TF_ANISO;
      int maxLevel = RI(&v, "max_level", mip ? -1 : 0);
      t.aniso = RF(&v, "anisotropic_level", t.filter == TF_ANISO ? 8.f : 0.f);
      if (!mip && maxLevel < 0) maxLevel = 0;
      t.width = (uint32_t)im.width;
      t.height = (uint32_t)im.height;
      BuildMips(t, im.px, maxLevel, hs.texels);
      if (mip) hs.needDiff = true;
    } else if (type == "chessboard") {  // chessboard.cpp:18-32
      t.kind = TEX_CHESS;
      M4f toUV = M4f::Identity();
      if (const JValue* n = v.get("to_uv")) toUV = Transform(*n);
      Xf check(toUV);  // Transform(toUV) inverts the matrix
      for (int i = 0; i < 16; i++) t.toUV[i] = toUV.m[i / 4][i % 4];
      const JValue* a = v.get("color_a");
      const JValue* b = v.get("color_b");
      JValue da, db;
      da.type = db.type = JValue::kNum;
      da.n = 0.4f;
      db.n = 0.2f;
      t.childA = AddTexture(a ? *a : da, channels, env);
      t.childB = AddTexture(b ? *b : db, channels, env);
      t.remap = RB(&v, "remap", false) ? 1u : 0u;
    } else {
      throw FactoryError("cannot find factory: " + type);
    }
  }
  hs.tex[index] = t;
  return index;
}

// Texture::Read averaged over the texels as Plastic's constructor does
// (plastic.cpp:29-42): constant -> its value, bitmap -> level 0, chessboard ->
// Read() returns 0 (chessboard.cpp:60-62).
double MeanLuminance(const HostScene& hs, uint32_t id) {
  const TexRec& t = hs.tex[id];
  auto lum = [](const float* c) { return (c[0] * 0.212671f) + (c[1] * 0.715160f) + (c[2] * 0.072169f); };
  if (t.kind == TEX_CONST) return (double)lum(t.value) / 1.0;
  if (t.kind == TEX_CHESS) return 0.0;
  double sum = 0;
  const float* p = hs.texels.data() + t.levelOffset[0];
  for (uint32_t y = 0; y < t.height; y++)
    for (uint32_t x = 0; x < t.width; x++) sum += lum(p + ((size_t)y * t.width + x) * 3);
  return sum / (double)(t.height * t.width);
}

// ContinuousDistribution1D (distribution.cpp:55-68) appended to `pool` as
// pdf[n], cdf[n + 1], normalization; returns the unnormalised sum.
float AppendDist1D(const float* f, size_t n, std::vector<float>& pool) {
  std::vector<float> cdf(n + 1);
  cdf[0] = 0;
  for (size_t i = 1; i < n + 1; ++i) cdf[i] = cdf[i - 1] + f[i - 1] / (float)n;
  float sum = cdf[n];
  for (size_t i = 1; i < n + 1; i++) cdf[i] /= sum;
  pool.insert(pool.end(), f, f + n);
  pool.insert(pool.end(), cdf.begin(), cdf.end());
  pool.push_back((float)(1.0 / sum));
  return sum;
}

// Skybox luminance grid and ContinuousDistribution2D (skybox.cpp:27-47,
// distribution.cpp:103-118): the map read at texel corners (x / W, y / H),
// luminance weighted by sin of the row's centre latitude.
// Luminance distribution of a bitmap light over its texel corners: weighted by
// sin(theta) of the row for a skybox (skybox.cpp:28-48), unweighted for an
// area light (area.cpp:25-40).
void BuildEnvDistribution(HostScene& hs, uint32_t tex, uint32_t W, uint32_t H, LightRec& L, bool sinWeight = true) {
  std::vector<float> lum((size_t)W * H);
  for (uint32_t y = 0; y < H; y++) {
    float sinTheta = std::sin((y + 0.5f) / H * kPiF);
    float v = y / (float)H;
    for (uint32_t x = 0; x < W; x++) {
      float u = x / (float)W;
      float c[3];
      HostTexEval(hs, tex, u, v, c);
      float l = (c[0] * 0.212671f) + (c[1] * 0.715160f) + (c[2] * 0.072169f);
      lum[(size_t)y * W + x] = sinWeight ? l * sinTheta : l;
    }
  }
  if (hs.lightDist.size() + lum.size() * 2 + 4 * H + 8 > 0xffffffffull) throw ConfigError("environment map too large");
  L.dist = (uint32_t)hs.lightDist.size();
  L.distW = W;
  L.distH = H;
  std::vector<float> marginal(H);
  for (uint32_t y = 0; y < H; y++) marginal[y] = AppendDist1D(lum.data() + (size_t)y * W, W, hs.lightDist);
  float msum = AppendDist1D(marginal.data(), H, hs.lightDist);
  hs.lightDist.push_back(msum);
}

// ---- BSDF records
// Parameter reader for one BSDF record: constants go into p[], textured
// parameters become TexBind entries (their p[] slots are filled per lookup).
struct MatParams {
  MatRec& m;
  TexEnv* env;
  std::vector<TexBind> binds;
  uint32_t Tex(const JValue& v, int channels) {
    if (!env || !env->hs) throw FactoryError("textured parameters need a scene");
    return AddTexture(v, channels, *env);
  }
  void Bind(int slot, int channels, uint32_t tex, bool clamp01 = false) {
    TexBind b;
    b.slot = (uint16_t)slot;
    b.channels = (uint8_t)channels;
    b.clamp01 = clamp01 ? 1 : 0;
    b.tex = tex;
    binds.push_back(b);
  }
  // returns the texture index of a textured parameter, or -1
  int64_t Color(const JValue* c, const char* k, F3 def, int slot) {
    const JValue* v = c ? c->get(k) : nullptr;
    F3 x = def;
    if (v && !(v->isNum() || v->isArr())) {
      uint32_t t = Tex(*v, 3);
      Bind(slot, 3, t);
      return t;
    }
    if (v) x = Vec3(*v, k);
    m.p[slot] = x.x;
    m.p[slot + 1] = x.y;
    m.p[slot + 2] = x.z;
    return -1;
  }
  int64_t Mono(const JValue* c, const char* k, float def, int slot, bool clamp01 = false) {
    const JValue* v = c ? c->get(k) : nullptr;
    if (v && !v->isNum()) {
      uint32_t t = Tex(*v, 1);
      Bind(slot, 1, t, clamp01);
      return t;
    }
    float x = v ? (float)v->n : def;
    if (clamp01) x = x < 0.f ? 0.f : (1.f < x ? 1.f : x);
    m.p[slot] = x;
    return -1;
  }
  // microfacet distribution (rough_metal.cpp:30-45, rough_glass.cpp:35-50)
  void Dist(const JValue* c) {
    std::string dist = RS(c, "distribution", "ggx");
    m.p[11] = dist == "beckmann" ? 0.f : 1.f;  // unknown names fall back to GGX
    if (c && c->has("alpha")) {
      int64_t t = Mono(c, "alpha", 0.1f, 9);
      if (t >= 0) Bind(10, 1, (uint32_t)t);
      else m.p[10] = m.p[9];
    } else {
      Mono(c, "alpha_u", 0.1f, 9);
      Mono(c, "alpha_v", 0.1f, 10);
    }
    m.p[12] = RB(c, "sample_visible", true) ? 1.f : 0.f;
  }
};
bool DisneyHas(const JValue* c, const char* k) {  // disney.cpp:459-471
  const JValue* v = c ? c->get(k) : nullptr;
  if (!v) return false;
  if (v->isNum()) return (float)v->n != 0.f;
  return true;
}

// fresnel.cpp:79-84 (the polynomial fits of the internal diffuse reflectance).
float DiffuseReflectance(float eta) {
  float invEta = 1.f / eta;
  if (eta < 1.f) return std::fma(0.0636f, invEta, std::fma(eta, std::fma(eta, -1.4399f, 0.7099f), 0.6681f));
  const float c[6] = {0.919317f, -3.4793f, 6.75335f, -7.80989f, 4.98554f, -1.36881f};
  float acc = c[5];
  for (int i = 4; i >= 0; i--) acc = std::fma(invEta, acc, c[i]);
  return acc;
}
float LuminanceF(F3 c) { return (c.x * 0.212671f) + (c.y * 0.715160f) + (c.z * 0.072169f); }  // color.h:33
// Wrapper levels (two_side, mask) above the leaves of material i.
int WrapDepth(const std::vector<MatRec>& v, uint32_t i) {
  const MatRec& m = v[i];
  if (m.kind == MAT_TWO_SIDE) return 1 + std::max(WrapDepth(v, m.ref0), WrapDepth(v, m.ref1));
  if (m.kind == MAT_MASK) return 1 + WrapDepth(v, m.ref0);
  return 0;
}

uint32_t AddMaterial(const JValue* c, std::vector<MatRec>& out, TexEnv* env) {
  MatRec m;
  std::memset(&m, 0, sizeof(m));
  std::string type = c ? TypeOf(*c) : std::string("diffuse");
  uint32_t index = (uint32_t)out.size();
  out.push_back(m);
  MatParams P{m, env, {}};
  if (type == "diffuse") {  // diffuse.cpp:40-43
    m.kind = MAT_DIFFUSE;
    m.flags = BT_DIFFUSE | BT_REFLECTION;
    P.Color(c, "reflectance", F3(0.5f, 0.5f, 0.5f), 0);
  } else if (type == "rough_metal") {  // rough_metal.cpp:24-43
    m.kind = MAT_ROUGH_METAL;
    m.flags = BT_GLOSSY | BT_REFLECTION;
    P.Color(c, "reflectance", F3(1, 1, 1), 0);
    P.Color(c, "eta", F3(0.1999899f, 0.9220823f, 1.0998751f), 3);
    P.Color(c, "k", F3(3.9046354f, 2.4476316f, 2.1376500f), 6);
    P.Dist(c);
  } else if (type == "rough_glass") {  // rough_glass.cpp:24-47
    m.kind = MAT_ROUGH_GLASS;
    m.flags = BT_GLOSSY | BT_REFLECTION | BT_TRANSMISSION;
    P.Color(c, "reflectance", F3(1, 1, 1), 0);
    P.Color(c, "transmittance", F3(1, 1, 1), 3);
    float intIor = RF(c, "int_ior", 1.5046f);
    float extIor = RF(c, "ext_ior", 1.000277f);
    m.p[6] = intIor / extIor;
    m.p[7] = extIor / intIor;
    P.Dist(c);
  } else if (type == "disney") {  // disney.cpp:62-111
    m.kind = MAT_DISNEY;
    P.Color(c, "base_color", F3(0.5f, 0.5f, 0.5f), 0);
    P.Mono(c, "roughness", 0.5f, 3);
    const char* keys[] = {"anisotropic", "spec_trans", "sheen", "sheen_tint", "flatness", "spec_tint", "metallic",
                          "clearcoat"};
    const uint32_t fl[] = {DF_ANISO, DF_SPECTRANS, DF_SHEEN, DF_SHEENTINT, DF_FLATNESS, DF_SPECTINT, DF_METALLIC,
                           DF_CLEARCOAT};
    const int slot[] = {4, 5, 6, 7, 8, 9, 10, 11};
    for (int k = 0; k < 8; k++) {
      if (DisneyHas(c, keys[k])) m.dflags |= fl[k];
      P.Mono(c, keys[k], 0.f, slot[k]);
    }
    P.Mono(c, "clearcoat_gloss", 0.f, 12);
    m.p[14] = RF(c, "main_specular_sampling_rate", 1.f);
    m.p[15] = RF(c, "clearcoat_sampling_rate", 1.f);
    m.aux = RF(c, "diffuse_reflectance_sampling_rate", 1.f);
    bool hasST = (m.dflags & DF_SPECTRANS) != 0;
    bool hasEta = c && c->has("eta"), hasSpec = c && c->has("specular");
    if (hasEta && hasSpec) throw ConfigError("eta cannot set with specular at same time");
    float eta;
    if (hasEta) {
      eta = RF(c, "eta", 1.5f);
      if (hasST && eta == 1.f) eta = 1.001f;
    } else {
      float specular = RF(c, "specular", 0.5f);
      if (hasST && specular == 0.f) specular = 0.001f;
      eta = 2.f * (1.f / (1.f - std::sqrt(0.08f * specular))) - 1.f;
    }
    m.p[13] = eta;
    m.flags = BT_DIFFUSE | BT_REFLECTION;
    if (m.dflags & DF_CLEARCOAT) m.flags |= BT_GLOSSY;
    if (hasST) m.flags |= BT_TRANSMISSION;
  } else if (type == "perfect_mirror") {  // perfect_mirror.cpp:19-25
    m.kind = MAT_PERFECT_MIRROR;
    m.flags = BT_DELTA | BT_REFLECTION;
    P.Color(c, "reflectance", F3(1, 1, 1), 0);
    P.Color(c, "eta", F3(0, 0, 0), 3);
    P.Color(c, "k", F3(1, 1, 1), 6);
  } else if (type == "perfect_glass") {  // perfect_glass.cpp:19-26
    m.kind = MAT_PERFECT_GLASS;
    m.flags = BT_DELTA | BT_REFLECTION | BT_TRANSMISSION;
    P.Color(c, "reflectance", F3(1, 1, 1), 0);
    P.Color(c, "transmittance", F3(1, 1, 1), 3);
    m.p[6] = RF(c, "int_ior", 1.5046f) / RF(c, "ext_ior", 1.000277f);
  } else if (type == "plastic" || type == "rough_plastic") {  // plastic.cpp:18-44, rough_plastic.cpp:20-56
    bool rough = type == "rough_plastic";
    m.kind = rough ? MAT_ROUGH_PLASTIC : MAT_PLASTIC;
    m.flags = BT_DIFFUSE | BT_REFLECTION | BT_DELTA;
    float eta = RF(c, "int_ior", 1.49f) / RF(c, "ext_ior", 1.000277f);
    int64_t td = P.Color(c, "diffuse", F3(0.5f, 0.5f, 0.5f), 0);
    int64_t ts = P.Color(c, "specular", F3(1, 1, 1), 3);
    m.p[6] = eta;
    m.p[7] = 1.f / (eta * eta);
    m.p[8] = DiffuseReflectance(1.f / eta);
    // mean luminance over each texture's texels, accumulated in double
    double diffMean = td >= 0 ? MeanLuminance(*env->hs, (uint32_t)td) : (double)LuminanceF(F3(m.p[0], m.p[1], m.p[2])) / 1.0;
    double specMean = ts >= 0 ? MeanLuminance(*env->hs, (uint32_t)ts) : (double)LuminanceF(F3(m.p[3], m.p[4], m.p[5])) / 1.0;
    m.p[13] = (float)(specMean / (diffMean + specMean));
    m.p[14] = RB(c, "no_linear", false) ? 1.f : 0.f;
    if (rough) {
      std::string dist = RS(c, "distribution", "ggx");
      m.p[11] = dist == "beckmann" ? 0.f : 1.f;  // unknown names fall back to GGX (rough_plastic.cpp:31-38)
      int64_t t = P.Mono(c, "alpha", 0.1f, 9);
      if (t >= 0) P.Bind(10, 1, (uint32_t)t);
      else m.p[10] = m.p[9];
      m.p[12] = RB(c, "sample_visible", true) ? 1.f : 0.f;
    }
  } else if (type == "mask") {  // mask.cpp:12-21
    m.kind = MAT_MASK;
    P.Mono(c, "opacity", 0.5f, 0, true);  // EvalOpacity clamps (mask.cpp:66-68)
    if (!c->has("nested")) throw ConfigError("mask needs a nested bsdf");
    m.ref0 = AddMaterial(c->get("nested"), out, env);
    m.flags = out[m.ref0].flags;
  } else if (type == "two_side") {  // two_side.cpp:18-62
    m.kind = MAT_TWO_SIDE;
    if (c->has("two_side")) {
      m.ref0 = m.ref1 = AddMaterial(c->get("two_side"), out, env);
    } else {
      if (!c->has("out_side") || !c->has("in_side")) throw ConfigError("config must contains out_side and in_side");
      m.ref0 = AddMaterial(c->get("out_side"), out, env);
      m.ref1 = AddMaterial(c->get("in_side"), out, env);
    }
    m.flags = out[m.ref0].flags | out[m.ref1].flags;
  } else {
    throw FactoryError("cannot find factory: " + type);
  }
  if (!P.binds.empty()) {
    m.texFirst = (uint32_t)env->hs->texBind.size();
    m.texCount = (uint32_t)P.binds.size();
    env->hs->texBind.insert(env->hs->texBind.end(), P.binds.begin(), P.binds.end());
  }
  out[index] = m;
  if (WrapDepth(out, index) > kMaxBsdfNest) throw ConfigError("two_side / mask BSDFs nest more than 4 levels deep");
  return index;
}
// true when material i or a material it wraps has textured parameters
bool HasTextures(const std::vector<MatRec>& v, uint32_t i) {
  const MatRec& m = v[i];
  if (m.texCount) return true;
  if (m.kind == MAT_TWO_SIDE) return HasTextures(v, m.ref0) || HasTextures(v, m.ref1);
  if (m.kind == MAT_MASK) return HasTextures(v, m.ref0);
  return false;
}

// ---- camera (perspective.cpp:15-70, math_ext.h:65-75)
M4f LookAt(F3 origin, F3 target, F3 up) {
  F3 dir = Normalize(target - origin);
  F3 left = Normalize(Cross(Normalize(up), dir));
  F3 realUp = Normalize(Cross(dir, left));
  M4f r = M4f::Identity();
  for (int i = 0; i < 3; i++) {
    r.m[i][0] = left[i];
    r.m[i][1] = realUp[i];
    r.m[i][2] = dir[i];
    r.m[i][3] = origin[i];
  }
  return r;
}

CameraRec MakeCamera(const JValue& c) {
  if (TypeOf(c) != "perspective") throw FactoryError("cannot find factory: " + TypeOf(c));
  CameraRec cam{};
  cam.nearZ = RF(&c, "near", 0.001f);
  cam.farZ = RF(&c, "far", 100.f);
  float fov = RF(&c, "fov", 30.f);
  cam.width = 1280;
  cam.height = 720;
  if (const JValue* r = c.get("resolution")) {
    if (!r->isArr() || r->a.size() != 2) throw ConfigError("resolution must be [w, h]");
    cam.width = (int)Num(r->a[0], "resolution");
    cam.height = (int)Num(r->a[1], "resolution");
  }
  if (cam.width <= 0 || cam.height <= 0) throw ConfigError("resolution must be positive");
  M4f toWorld = c.has("to_world") ? Transform(*c.get("to_world"))
                                  : LookAt(RV(&c, "origin", F3(0, 0, -1)), RV(&c, "target", F3(0, 0, 0)),
                                           RV(&c, "up", F3(0, 1, 0)));
  Xf camToWorld(toWorld);
  float aspect = cam.width / static_cast<float>(cam.height);
  float recip = 1 / (cam.farZ - cam.nearZ);
  float cot = 1 / std::tan((fov / 2) * (kPiF / 180.f));
  M4f persp{}, scale{}, translate = M4f::Identity();
  std::memset(&persp, 0, sizeof(persp));
  std::memset(&scale, 0, sizeof(scale));
  persp.m[0][0] = cot;
  persp.m[1][1] = cot;
  persp.m[2][2] = cam.farZ * recip;
  persp.m[2][3] = -cam.nearZ * cam.farZ * recip;
  persp.m[3][2] = 1;
  scale.m[0][0] = -0.5f;
  scale.m[1][1] = -0.5f * aspect;
  scale.m[2][2] = 1;
  scale.m[3][3] = 1;
  translate.m[0][3] = -1;
  translate.m[1][3] = -1 / aspect;
  Xf toClip(scale * translate * persp);
  for (int i = 0; i < 16; i++) {
    cam.clipToCamera[i] = toClip.l.m[i / 4][i % 4];
    cam.camToWorld[i] = camToWorld.w.m[i / 4][i % 4];
  }
  F3 o = Xf::Aff(toClip.l, F3(0, 0, 0));
  F3 dx = Xf::Aff(toClip.l, F3(1.f / cam.width, 0, 0)) - o;
  F3 dy = Xf::Aff(toClip.l, F3(0, 1.f / cam.height, 0)) - o;
  cam.dx[0] = dx.x;
  cam.dx[1] = dx.y;
  cam.dx[2] = dx.z;
  cam.dy[0] = dy.x;
  cam.dy[1] = dy.y;
  cam.dy[2] = dy.z;
  for (int i = 0; i < 16; i++) {
    cam.worldToCam[i] = camToWorld.l.m[i / 4][i % 4];
    cam.camToClip[i] = toClip.w.m[i / 4][i % 4];
  }
  F3 pMin = Xf::Aff(toClip.l, F3(0, 0, 0)), pMax = Xf::Aff(toClip.l, F3(1, 1, 0));
  float ax = pMin.x / pMin.z, ay = pMin.y / pMin.z, bx = pMax.x / pMax.z, by = pMax.y / pMax.z;
  cam.rect[0] = std::min(ax, bx);
  cam.rect[1] = std::min(ay, by);
  cam.rect[2] = std::max(ax, bx);
  cam.rect[3] = std::max(ay, by);
  cam.normalization = 1 / ((cam.rect[2] - cam.rect[0]) * (cam.rect[3] - cam.rect[1]));
  return cam;
}

struct Entity {
  const JValue* cfg;
  M4f toWorld;
};

}  // namespace

M4f M4f::Identity() {
  M4f r;
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) r.m[i][j] = (i == j) ? 1.f : 0.f;
  return r;
}
M4f M4f::operator*(const M4f& b) const {
  M4f r;
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) {
      float s = m[i][0] * b.m[0][j];
      s = s + m[i][1] * b.m[1][j];
      s = s + m[i][2] * b.m[2][j];
      s = s + m[i][3] * b.m[3][j];
      r.m[i][j] = s;
    }
  return r;
}

// General 4x4 inverse by cofactors in double precision, rounded to float.
bool InvertM4f(const M4f& a, M4f& out) {
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
  for (int i = 0; i < 16; i++) out.m[i / 4][i % 4] = (float)(inv[i] / det);
  return true;
}

void BuildMaterialRecords(const JValue& bsdf, std::vector<MatRec>& out) {
  out.clear();
  AddMaterial(&bsdf, out, nullptr);
}

static MediumRec MakeMedium(const JValue& c, const M4f& toWorld, const std::map<std::string, VolData>& vols,
                            HostScene& hs) {
  MediumRec md;
  std::memset(&md, 0, sizeof(md));
  const JValue* ph = c.get("phase");
  if (!ph) throw ConfigError("medium must have phase function");  // medium.cpp:8-17
  std::string pt = TypeOf(*ph);
  if (pt == "hg_phase") {  // henyey_greenstein.cpp:13-17
    md.hg = 1;
    md.g = RF(ph, "g", 0.8f);
    if (md.g <= -1 || md.g >= 1) throw ConfigError("param g must lie in the interval (-1, 1)");
  } else if (pt == "isotropic_phase") {
    md.hg = 0;
  } else {
    throw FactoryError("cannot find factory: " + pt);
  }
  std::string type = TypeOf(c);
  md.scale = RF(&c, "scale", 1.f);
  auto constOnly = [&](const char* k, F3 def) -> F3 {
    const JValue* v = c.get(k);
    if (!v) return def;
    if (v->isNum() || v->isArr()) return Vec3(*v, k);
    throw FactoryError(std::string("only constant volumes are supported for ") + k);
  };
  F3 alb = constOnly("albedo", F3(0.75f, 0.75f, 0.75f));
  md.albedo[0] = alb.x;
  md.albedo[1] = alb.y;
  md.albedo[2] = alb.z;
  if (type == "homogeneous") {  // homogeneous.cpp:14-22
    md.kind = MED_HOMOGENEOUS;
    F3 st = RV(&c, "sigma_t", F3(1, 1, 1));
    md.sigmaT[0] = st.x;
    md.sigmaT[1] = st.y;
    md.sigmaT[2] = st.z;
    return md;
  }
  if (type != "heterogeneous") throw FactoryError("cannot find factory: " + type);
  md.kind = MED_HETEROGENEOUS;  // heterogeneous.cpp:17-36
  float maxValue;
  const JValue* sv = c.get("sigma_t");
  if (!sv || sv->isNum() || sv->isArr()) {
    F3 st = sv ? Vec3(*sv, "sigma_t") : F3(1, 1, 1);
    md.sigmaT[0] = st.x;
    md.sigmaT[1] = st.y;
    md.sigmaT[2] = st.z;
    maxValue = std::max(std::max(st.x, st.y), st.z);
  } else {
    if (TypeOf(*sv) != "volume_grid") throw FactoryError("cannot find factory: " + TypeOf(*sv));
    auto it = vols.find(RS(sv, "asset_name", ""));
    if (it == vols.end()) throw ConfigError("unknown volume asset: " + RS(sv, "asset_name", ""));
    md.gridSigma = 1;
    md.repeatWrap = RS(sv, "wrap", "clamp") == "repeat" ? 1 : 0;
    md.nx = it->second.nx;
    md.ny = it->second.ny;
    md.nz = it->second.nz;
    md.channels = it->second.ch;
    md.gridOffset = hs.volume.size();
    hs.volume.insert(hs.volume.end(), it->second.data.begin(), it->second.data.end());
    maxValue = it->second.max;
    if (!md.repeatWrap) {
      // 16^3-brick majorants over voxel coordinates f = local * (n - 1). A point in
      // cell [i, i + 1) interpolates voxels i - 1 .. i + 1 (the neighbour rule of
      // grid.cpp:41-75), so a brick's bound is the maximum over its voxels dilated by one.
      const int n[3] = {md.nx, md.ny, md.nz}, ch = md.channels;
      int nb[3];
      for (int a = 0; a < 3; a++) nb[a] = std::max(1, (n[a] - 1 + 15) / 16);
      md.brickOffset = (uint32_t)hs.brickMaj.size();
      md.hasBricks = 1;
      const std::vector<float>& g = it->second.data;
      for (int bz = 0; bz < nb[2]; bz++)
        for (int by = 0; by < nb[1]; by++)
          for (int bx = 0; bx < nb[0]; bx++) {
            float m = 0.f;
            int z0 = std::max(0, 16 * bz - 1), z1 = std::min(n[2] - 1, 16 * bz + 16);
            int y0 = std::max(0, 16 * by - 1), y1 = std::min(n[1] - 1, 16 * by + 16);
            int x0 = std::max(0, 16 * bx - 1), x1 = std::min(n[0] - 1, 16 * bx + 16);
            for (int z = z0; z <= z1; z++)
              for (int y = y0; y <= y1; y++)
                for (int x = x0; x <= x1; x++)
                  for (int c = 0; c < ch; c++)
                    m = std::max(m, g[(((size_t)z * n[1] + y) * n[0] + x) * ch + c]);
            hs.brickMaj.push_back(m * md.scale);
          }
    }
  }
  M4f affine = M4f::Identity();
  for (int i = 0; i < 3; i++) {
    affine.m[i][i] = 2;
    affine.m[i][3] = -1;
  }
  Xf x(toWorld * affine);
  RowsOf(x.l, md.toLocal);
  F3 lo(INFINITY, INFINITY, INFINITY), hi(-INFINITY, -INFINITY, -INFINITY);
  for (int k = 0; k < 8; k++) {
    F3 p = x.AffW(F3(float(k & 1), float((k >> 1) & 1), float((k >> 2) & 1)));
    lo = Min3(lo, p);
    hi = Max3(hi, p);
  }
  md.bbMin[0] = lo.x; md.bbMin[1] = lo.y; md.bbMin[2] = lo.z;
  md.bbMax[0] = hi.x; md.bbMax[1] = hi.y; md.bbMax[2] = hi.z;
  md.maxDensity = maxValue * md.scale;
  return md;
}

void BuildHostScene(const std::string& json, const std::string& baseDir, HostScene& hs) {
  JValue root = JsonReader::Parse(json);
  if (!root.isObj()) throw ConfigError("scene root must be an object");
  std::map<std::string, ObjData> objs;
  std::map<std::string, VolData> vols;
  std::map<std::string, ImageAsset> images;
  TexEnv env{&hs, &images};
  if (const JValue* an = root.get("assets")) {  // asset.cpp:17-38
    if (!an->isArr()) throw ConfigError("assets must be an array");
    for (const JValue& a : an->a) {
      std::string type = TypeOf(a), name = RS(&a, "name", ""), loc = RS(&a, "location", "");
      if (type == "model_obj") {
        objs[name] = LoadObj(Join(baseDir, loc));
      } else if (type == "volume_data_mitsuba_vol") {
        vols[name] = LoadVol(Join(baseDir, loc));
      } else if (type == "image_default" || type == "image_hdr" || type == "image_exr") {
        images[name] = LoadImageAsset(a, type, Join(baseDir, loc));
      } else {
        throw FactoryError("cannot find factory: " + type);
      }
    }
  }
  const JValue* cam = root.get("camera");
  if (!cam) throw ConfigError("no child: camera");
  hs.cam = MakeCamera(*cam);
  if (const JValue* s = root.get("sampler")) {
    if (TypeOf(*s) != "independent") throw FactoryError("cannot find factory: " + TypeOf(*s));
    hs.spp = RI(s, "sample_count", 16);
    hs.seed = (uint32_t)RI(s, "seed", 0);
  }
  if (hs.spp < 0) throw ConfigError("sample_count must be non-negative");
  if (const JValue* gm = root.get("global_medium")) {
    hs.media.push_back(MakeMedium(*gm, M4f::Identity(), vols, hs));
    hs.globalMedium = 0;
  }
  std::map<std::string, uint32_t> bsdfVars;
  if (const JValue* bv = root.get("bsdf_vars")) {
    for (const JValue& v : bv->a) {
      std::string name = RS(&v, "name", "");
      const JValue* def = v.get("bsdf");
      if (!def) throw ConfigError("no child: bsdf");
      if (bsdfVars.count(name)) throw ConfigError("duplicate bsdf var name: " + name);
      bsdfVars[name] = AddMaterial(def, hs.mats, &env);
    }
  }
  const JValue* sceneNode = root.get("scene");
  if (!sceneNode || !sceneNode->isArr()) throw ConfigError("no child: scene");
  std::deque<Entity> q;
  for (const JValue& e : sceneNode->a) {
    Entity en{&e, M4f::Identity()};
    if (const JValue* tw = e.get("to_world")) en.toWorld = Transform(*tw);
    q.push_back(en);
  }
  while (!q.empty()) {  // build_context.cpp:137-288 (BFS over entities)
    Entity en = q.front();
    q.pop_front();
    const JValue& e = *en.cfg;
    if (const JValue* ch = e.get("children")) {
      for (const JValue& c : ch->a) {
        Entity ce{&c, en.toWorld};
        if (const JValue* tw = c.get("to_world")) ce.toWorld = Transform(*tw) * en.toWorld;
        q.push_back(ce);
      }
    }
    int shapeIdx = -1, lightIdx = -1, bsdfIdx = -1;
    if (const JValue* sn = e.get("shape")) {
      std::string type = TypeOf(*sn);
      ShapeRec sh;
      std::memset(&sh, 0, sizeof(sh));
      sh.bsdf = sh.light = sh.inMedium = sh.outMedium = -1;
      if (type == "rectangle") {  // rectangle.cpp:164-178
        sh.kind = SHAPE_RECT;
        M4f tw = en.toWorld;
        if (RB(sn, "is_flip_normal", false)) {
          M4f flip = M4f::Identity();
          flip.m[2][2] = -1;
          tw = tw * flip;
        }
        Xf x(tw);
        F3 dpdu = x.LinW(F3(2, 0, 0)), dpdv = x.LinW(F3(0, 2, 0));
        F3 n = Normalize(x.NrmW(F3(0, 0, 1)));
        RowsOf(x.w, sh.m);
        float fr[12] = {dpdu.x, dpdu.y, dpdu.z, dpdv.x, dpdv.y, dpdv.z, n.x, n.y, n.z, x.w.m[0][3], x.w.m[1][3], x.w.m[2][3]};
        for (int k = 0; k < 12; k++) sh.m[12 + k] = fr[k];
        sh.surfaceArea = Norm(Cross(dpdu, dpdv));
        sh.primCount = 1;
        hs.rectIndexOfShape.push_back((uint32_t)hs.shapes.size());
        float rows[12];
        RowsOf(x.l, rows);
        hs.rectToObject.insert(hs.rectToObject.end(), rows, rows + 12);
      } else if (type == "sphere") {  // sphere.cpp:173-189
        sh.kind = SHAPE_SPHERE;
        F3 lc = RV(sn, "center", F3(0, 0, 0));
        float lr = RF(sn, "radius", 1.f);
        Xf t(en.toWorld);
        if (t.NonUniformScale()) throw ConfigError("Sphere does not support non uniform transformations");
        if (sn->has("rotate_uv")) throw FactoryError("rotate_uv is not supported");
        F3 c = t.AffW(lc);
        float r = Norm(t.LinW(F3(0, 0, lr)));
        M4f ts = M4f::Identity();
        for (int i = 0; i < 3; i++) {
          ts.m[i][i] = r;
          ts.m[i][3] = c[i];
        }
        Xf st(ts * en.toWorld);
        sh.m[0] = c.x;
        sh.m[1] = c.y;
        sh.m[2] = c.z;
        sh.m[3] = r;
        RowsOf(st.l, sh.m + 4);
        RowsOf(st.w, sh.m + 16);
        sh.surfaceArea = 4 * kPiF * (r * r);
        sh.primCount = 1;
      } else if (type == "mesh" || type == "cube") {
        sh.kind = SHAPE_MESH;
        Xf t(en.toWorld);
        bool ident = t.Identity();
        ModelData m;
        if (type == "cube") {  // cube.cpp:15-115; its UVs are never written, taken as zero
          static const float P[24][3] = {{1, -1, -1}, {1, -1, 1}, {-1, -1, 1}, {-1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                         {-1, 1, 1}, {1, 1, 1}, {1, -1, -1}, {1, 1, -1}, {1, 1, 1}, {1, -1, 1},
                                         {1, -1, 1}, {1, 1, 1}, {-1, 1, 1}, {-1, -1, 1}, {-1, -1, 1}, {-1, 1, 1},
                                         {-1, 1, -1}, {-1, -1, -1}, {1, 1, -1}, {1, -1, -1}, {-1, -1, -1}, {-1, 1, -1}};
          static const float N[6][3] = {{0, -1, 0}, {0, 1, 0}, {1, 0, 0}, {0, 0, 1}, {-1, 0, 0}, {0, 0, -1}};
          static const int T[12][3] = {{0, 1, 2}, {3, 0, 2}, {4, 5, 6}, {7, 4, 6}, {8, 9, 10}, {11, 8, 10},
                                       {12, 13, 14}, {15, 12, 14}, {16, 17, 18}, {19, 16, 18}, {20, 21, 22}, {23, 20, 22}};
          for (int i = 0; i < 24; i++) {
            m.pos.emplace_back(P[i][0], P[i][1], P[i][2]);
            m.nrm.emplace_back(N[i / 4][0], N[i / 4][1], N[i / 4][2]);
            m.uv.emplace_back(0.f, 0.f);
          }
          for (int i = 0; i < 12; i++)
            for (int j = 0; j < 3; j++) m.idx.push_back((uint32_t)T[i][j]);
          ident = false;
        } else {  // mesh.cpp:14-52
          std::string an = RS(sn, "asset_name", "");
          auto it = objs.find(an);
          if (it == objs.end()) throw ConfigError("unknown model asset: " + an);
          if (const JValue* smn = sn->get("sub_model")) {
            const std::vector<size_t>* fl = nullptr;
            for (auto& o : it->second.objects)
              if (o.first == smn->s) {
                fl = &o.second;
                break;
              }
            if (!fl) throw ConfigError("no model name: " + smn->s);
            m = ToModel(it->second, fl);
          } else {
            m = ToModel(it->second, nullptr);
          }
        }
        if (m.idx.empty()) throw ConfigError("mesh has no triangles");
        uint32_t vbase = (uint32_t)(hs.pos.size() / 3);
        sh.triOffset = (uint32_t)(hs.idx.size() / 3);
        sh.hasNormals = m.nrm.empty() ? 0 : 1;
        sh.hasUV = m.uv.empty() ? 0 : 1;
        for (size_t k = 0; k < m.pos.size(); k++) {
          F3 p = ident ? m.pos[k] : t.AffW(m.pos[k]);
          hs.pos.push_back(p.x);
          hs.pos.push_back(p.y);
          hs.pos.push_back(p.z);
          F3 nn = sh.hasNormals ? (ident ? m.nrm[k] : t.NrmW(m.nrm[k])) : F3(0, 0, 0);
          hs.nrm.push_back(nn.x);
          hs.nrm.push_back(nn.y);
          hs.nrm.push_back(nn.z);
          hs.uv.push_back(sh.hasUV ? m.uv[k].first : 0.f);
          hs.uv.push_back(sh.hasUV ? m.uv[k].second : 0.f);
        }
        for (uint32_t v : m.idx) hs.idx.push_back(vbase + v);
        sh.primCount = (uint32_t)(m.idx.size() / 3);
        // mesh_base.cpp:120-131 + distribution.cpp:19-31: triangle area CDF
        sh.cdfOffset = (uint32_t)(hs.cdf.size() / 2);
        double sum = 0;
        for (uint32_t i = 0; i < sh.primCount; i++) {
          const float* p0 = &hs.pos[3 * hs.idx[3 * (sh.triOffset + i)]];
          const float* p1 = &hs.pos[3 * hs.idx[3 * (sh.triOffset + i) + 1]];
          const float* p2 = &hs.pos[3 * hs.idx[3 * (sh.triOffset + i) + 2]];
          F3 a(p0[0], p0[1], p0[2]), b(p1[0], p1[1], p1[2]), cc(p2[0], p2[1], p2[2]);
          float area = Norm(Cross(b - a, cc - a)) * 0.5f;
          sum += (double)area;
          hs.cdf.push_back((float)sum);
          hs.cdf.push_back(area);
        }
        sh.cdfSum = (float)sum;
        sh.cdfNorm = (float)(1.0 / sum);
        sh.surfaceArea = sh.cdfSum;
      } else {
        throw FactoryError("cannot find factory: " + type);
      }
      hs.shapes.push_back(sh);
      shapeIdx = (int)hs.shapes.size() - 1;
    }
    if (const JValue* ln = e.get("light")) {
      std::string type = TypeOf(*ln);
      LightRec L;
      std::memset(&L, 0, sizeof(L));
      Xf t(en.toWorld);
      auto col = [&](const char* k, F3 def) {
        const JValue* v = ln->get(k);
        if (!v) return def;
        if (v->isNum() || v->isArr()) return Vec3(*v, k);
        throw FactoryError("textured lights are not supported");
      };
      F3 rad;
      if (type == "area") {  // area.cpp:20-40
        L.kind = LIGHT_AREA;
        const JValue* rn = ln->get("radiance");
        if (rn && rn->isObj()) {
          uint32_t tid = AddTexture(*rn, 3, env);
          const TexRec& tr = hs.tex[tid];
          uint32_t W = tr.kind == TEX_BITMAP ? tr.width : 1u, H = tr.kind == TEX_BITMAP ? tr.height : 1u;
          if (tr.kind == TEX_CHESS) {
            // a chessboard is 1 x 1 (chessboard.cpp:30-31): _isUniform, so the light samples its shape and
            // reads the texture at each point's uv (area.cpp:45-58); no distribution (distW 0)
            L.tex = tid + 1;
          } else if (W == 1 && H == 1) {  // _isUniform: one constant
            float c[3];
            HostTexEval(hs, tid, 0.f, 0.f, c);
            rad = F3(c[0], c[1], c[2]);
          } else {
            L.tex = tid + 1;
            BuildEnvDistribution(hs, tid, W, H, L, false);
          }
        } else {
          rad = col("radiance", F3(1, 1, 1));
        }
      } else if (type == "skybox") {  // skybox.cpp:24-50
        L.kind = LIGHT_SKYBOX;
        const JValue* rn = ln->get("radiance");
        if (rn && rn->isObj()) {
          uint32_t tid = AddTexture(*rn, 3, env);
          L.tex = tid + 1;
          const TexRec& tr = hs.tex[tid];
          uint32_t W = tr.kind == TEX_BITMAP ? tr.width : 1u, H = tr.kind == TEX_BITMAP ? tr.height : 1u;
          if (!(W == 1 && H == 1)) BuildEnvDistribution(hs, tid, W, H, L);
        } else {
          rad = col("radiance", F3(1, 1, 1));
        }
        RowsOf(t.w, L.lin);
        for (int i = 0; i < 16; i++) L.m[i] = t.l.m[i / 4][i % 4];
      } else if (type == "point") {  // point.cpp:19-26
        L.kind = LIGHT_POINT;
        F3 p = t.AffW(RV(ln, "position", F3(0, 0, 0)));
        L.dir[0] = p.x;
        L.dir[1] = p.y;
        L.dir[2] = p.z;
        rad = RV(ln, "intensity", F3(1, 1, 1));
      } else if (type == "projection") {  // projection.cpp:19-45 (constant irradiance: a 1x1 texture)
        L.kind = LIGHT_PROJECTION;
        F3 sc = RV(ln, "scale", F3(1, 1, 1));
        F3 irr(1, 1, 1);
        float aspect = 1 / (float)1;  // Width / Height of the irradiance texture (1 x 1 when constant)
        const JValue* in = ln->get("irradiance");
        if (in && in->isObj()) {  // a texture: looked up per sample; radiance holds the scale
          uint32_t tid = AddTexture(*in, 3, env);
          L.tex = tid + 1;
          const TexRec& tr = hs.tex[tid];
          uint32_t W = tr.kind == TEX_BITMAP ? tr.width : 1u, H = tr.kind == TEX_BITMAP ? tr.height : 1u;
          aspect = W / (float)H;
          rad = sc;
        } else {
          irr = col("irradiance", F3(1, 1, 1));
          rad = F3(irr.x * sc.x, irr.y * sc.y, irr.z * sc.z);  // irradiance.cwiseProduct(scale)
        }
        float fov = RF(ln, "fov", 90.f);
        float farZ = 10000, nearZ = 0.0001f;
        M4f persp{}, scale{}, translate = M4f::Identity();
        std::memset(&persp, 0, sizeof(persp));
        std::memset(&scale, 0, sizeof(scale));
        float recip = 1 / (farZ - nearZ);
        float cot = 1 / std::tan((fov / 2) * (kPiF / 180.f));
        persp.m[0][0] = cot;
        persp.m[1][1] = cot;
        persp.m[2][2] = farZ * recip;
        persp.m[2][3] = -nearZ * farZ * recip;
        persp.m[3][2] = 1;
        scale.m[0][0] = -0.5f;
        scale.m[1][1] = -0.5f * aspect;
        scale.m[2][2] = 1;
        scale.m[3][3] = 1;
        translate.m[0][3] = -1;
        translate.m[1][3] = -1 / aspect;
        M4f toClip = scale * translate * persp;
        Xf clip(toClip);
        for (int i = 0; i < 16; i++) {
          L.m[i] = t.l.m[i / 4][i % 4];
          L.m[16 + i] = toClip.m[i / 4][i % 4];
          L.m2[i] = clip.l.m[i / 4][i % 4];
        }
        RowsOf(t.w, L.m2 + 16);
        F3 pMin = Xf::Aff(clip.l, F3(0, 0, 0)), pMax = Xf::Aff(clip.l, F3(1, 1, 0));
        float ax = pMin.x / pMin.z, ay = pMin.y / pMin.z, bx = pMax.x / pMax.z, by = pMax.y / pMax.z;
        L.m2[28] = 1 / ((std::max(ax, bx) - std::min(ax, bx)) * (std::max(ay, by) - std::min(ay, by)));
        L.m2[29] = irr.x;
        L.m2[30] = irr.y;
        L.m2[31] = irr.z;
        L.dir[0] = t.w.m[0][3];  // TranslationToWorld
        L.dir[1] = t.w.m[1][3];
        L.dir[2] = t.w.m[2][3];
        F3 n = Normalize(t.LinW(F3(0, 0, 1)));
        L.lin[0] = n.x;
        L.lin[1] = n.y;
        L.lin[2] = n.z;
      } else if (type == "directional") {  // extension: no reference factory
        L.kind = LIGHT_DIRECTIONAL;
        rad = col("irradiance", F3(1, 1, 1));
        F3 d = Normalize(t.LinW(RV(ln, "direction", F3(0, -1, 0))));
        L.dir[0] = d.x;
        L.dir[1] = d.y;
        L.dir[2] = d.z;
      } else {
        throw FactoryError("cannot find factory: " + type);
      }
      L.radiance[0] = rad.x;
      L.radiance[1] = rad.y;
      L.radiance[2] = rad.z;
      L.shape = -1;
      hs.lights.push_back(L);
      lightIdx = (int)hs.lights.size() - 1;
    }
    if (const JValue* bn = e.get("bsdf")) {
      if (const JValue* ref = bn->get("ref")) {
        auto it = bsdfVars.find(ref->s);
        if (it == bsdfVars.end()) throw ConfigError("unknown bsdf var: " + ref->s);
        bsdfIdx = (int)it->second;
      } else {
        bsdfIdx = (int)AddMaterial(bn, hs.mats, &env);
      }
    }
    int inMed = -1, outMed = -1;
    bool outUseGlobal = true;
    if (const JValue* im = e.get("in_medium")) {
      hs.media.push_back(MakeMedium(*im, en.toWorld, vols, hs));
      inMed = (int)hs.media.size() - 1;
    }
    if (const JValue* om = e.get("out_medium")) {
      if (const JValue* ig = om->get("is_global")) {
        if (ig->type != JValue::kBool) throw ConfigError("node type is not bool: is_global");
        outUseGlobal = ig->b;
      } else {
        hs.media.push_back(MakeMedium(*om, en.toWorld, vols, hs));
        outMed = (int)hs.media.size() - 1;
      }
    }
    if (lightIdx >= 0 && shapeIdx >= 0 && bsdfIdx < 0) bsdfIdx = (int)AddMaterial(nullptr, hs.mats, &env);  // :243-246
    if (shapeIdx >= 0) {
      ShapeRec& sh = hs.shapes[shapeIdx];
      sh.light = lightIdx;
      sh.bsdf = bsdfIdx;
      if (outMed < 0 && outUseGlobal && hs.globalMedium >= 0) outMed = hs.globalMedium;
      sh.inMedium = inMed;
      sh.outMedium = outMed;
    }
    if (lightIdx >= 0) {
      hs.lights[lightIdx].shape = shapeIdx;
      if (hs.lights[lightIdx].kind == LIGHT_AREA && shapeIdx < 0) throw ConfigError("area light needs a shape");
      // only the rectangle has EvalParamSurface (shape.cpp:27-29)
      const LightRec& AL = hs.lights[lightIdx];
      if (AL.kind == LIGHT_AREA && AL.distW && hs.shapes[shapeIdx].kind != SHAPE_RECT)
        throw ConfigError("no impl EvalParamSurface(): a textured area light needs a rectangle");
      // Sphere::SamplePosition / SampleDirection leave the sample's uv unset (sphere.cpp:250-320), so the
      // reference would read a chessboard radiance at an undefined uv
      if (AL.kind == LIGHT_AREA && AL.tex && !AL.distW && hs.shapes[shapeIdx].kind == SHAPE_SPHERE)
        throw ConfigError("area: a chessboard radiance on a sphere is not supported (its samples carry no uv)");
    }
  }
  const JValue* rn = root.get("renderer");
  if (!rn) throw ConfigError("no child: renderer");
  std::string rt = TypeOf(*rn);
  if (rt != "path" && rt != "vol_path" && rt != "ao" && rt != "particle_tracer" && rt != "bdpt")
    throw FactoryError("cannot find factory: " + rt);
  hs.isVol = rt == "vol_path";
  hs.isAO = rt == "ao";
  hs.isParticle = rt == "particle_tracer";  // max_depth -1, rr_depth 3 (particle_tracer.cpp:24-25)
  hs.isBdpt = rt == "bdpt";                 // max_depth -1, rr_depth 5, use_mis true (bdpt.cpp:223-227)
  hs.maxDepth = RI(rn, "max_depth", -1);
  hs.rrDepth = RI(rn, "rr_depth", hs.isVol || hs.isBdpt ? 5 : 3);
  if (hs.isBdpt) {
    hs.bdptMis = RB(rn, "use_mis", true);
    for (const LightRec& L : hs.lights)
      if (L.kind == LIGHT_DIRECTIONAL) throw ConfigError("bdpt: the directional light is not supported");
  }
  if (const JValue* an = root.get("accel")) {
    std::string at = TypeOf(*an);
    if (at != "embree" && at != "gpu_bvh8") throw FactoryError("cannot find factory: " + at);
  }
  uint32_t off = 0;
  for (auto& sh : hs.shapes) {
    sh.primOffset = off;
    off += sh.primCount;
  }
  hs.nPrims = off;
  for (const auto& sh : hs.shapes) {
    uint8_t cls = SC_EMIT;
    if (sh.light < 0 && sh.bsdf >= 0) {
      const MatRec& m = hs.mats[sh.bsdf];
      uint32_t kind = m.kind;
      if (kind == MAT_TWO_SIDE) {
        uint32_t a = hs.mats[m.ref0].kind, b = hs.mats[m.ref1].kind;
        kind = (a == b && a != MAT_TWO_SIDE) ? a : MAT_NONE;
      }
      // textured materials are shaded by the generic class, which evaluates textures
      if (HasTextures(hs.mats, (uint32_t)sh.bsdf)) kind = MAT_NONE;
      cls = (kind >= MAT_DIFFUSE && kind <= MAT_DISNEY) ? (uint8_t)kind : (uint8_t)SC_GENERIC;
    }
    hs.shapeClass.push_back(cls);
  }
  BuildBvh8(hs);
  // scene.cpp:11-36 and skybox.cpp:139-144
  hs.lightPdf = 1.f / float(hs.lights.size());
  F3 lo(hs.worldLo[0], hs.worldLo[1], hs.worldLo[2]), hi(hs.worldHi[0], hs.worldHi[1], hs.worldHi[2]);
  F3 c((lo.x + hi.x) / 2, (lo.y + hi.y) / 2, (lo.z + hi.z) / 2);
  float r = Norm(c - hi);
  const float rayEps = 5.9604644775390625e-08f * 1500.f;
  r = std::max(rayEps, r * (1 + rayEps * 10.f));
  for (size_t i = 0; i < hs.lights.size(); i++) {
    if (hs.lights[i].kind == LIGHT_SKYBOX) hs.envLight = (int)i;
    hs.lights[i].world[0] = c.x;
    hs.lights[i].world[1] = c.y;
    hs.lights[i].world[2] = c.z;
    hs.lights[i].world[3] = r;
  }
}

}  // namespace rad
