// Host scene compilation: the reference's JSON scene (BuildContext::SetFromJson
// and Build, rad.offline/src/build/build_context.cpp:47-321) into the flat
// device records of records.h, plus the SAH BVH8 over all primitives.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "host_json.h"
#include "records.h"

namespace rad {

// Unknown factory name (the reference throws RadArgumentException "cannot find
// factory", rad.core/src/factory.cpp:13-19); mapped to RAD_ERR_UNKNOWN_FACTORY.
struct FactoryError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct IoError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

struct M4f {
  float m[4][4];
  static M4f Identity();
  M4f operator*(const M4f& b) const;
};
bool InvertM4f(const M4f& a, M4f& out);

struct HostScene {
  CameraRec cam{};
  int spp = 16;
  uint32_t seed = 0;
  bool isVol = false;
  bool isAO = false;  // renderer "ao"
  bool isParticle = false;  // renderer "particle_tracer"
  bool isBdpt = false, bdptMis = true;  // renderer "bdpt" and its use_mis
  int maxDepth = -1, rrDepth = 3;
  std::vector<MatRec> mats;
  std::vector<ShapeRec> shapes;
  std::vector<LightRec> lights;
  std::vector<MediumRec> media;
  std::vector<float> volume;
  std::vector<float> brickMaj;  // 16^3-brick majorants of the grid media
  std::vector<float> pos, nrm, uv;
  std::vector<uint32_t> idx;
  std::vector<float> cdf;
  std::vector<float> rectToObject;  // per rect shape: 12 floats (world -> object rows)
  std::vector<uint32_t> rectIndexOfShape;
  std::vector<uint8_t> shapeClass;  // see records.h SC_*
  std::vector<TexRec> tex;          // textures, in creation order
  std::vector<float> texels;        // mip chains of the bitmap textures
  std::vector<TexBind> texBind;     // textured BSDF parameters
  bool needDiff = false;            // a trilinear / anisotropic bitmap is in use
  std::vector<float> lightDist;     // 2D luminance distributions of textured skyboxes
  int envLight = -1, globalMedium = -1;
  float lightPdf = 0.f;
  uint64_t nPrims = 0;
  float worldLo[3], worldHi[3];
  // BVH8
  std::vector<Bvh8Node> nodes;
  std::vector<PrimRec> prims;
  std::vector<uint32_t> primInfo;  // 2 words per leaf-order primitive
};

// Texture `tex` of the scene at (u, v) with zero uv derivatives (host_texeval.cpp).
void HostTexEval(const HostScene& hs, uint32_t tex, float u, float v, float out[3]);

// Parses `json` (scene text) resolving asset locations against `baseDir`.
void BuildHostScene(const std::string& json, const std::string& baseDir, HostScene& out);
// One BSDF given as reference JSON -> records (root at index 0).
void BuildMaterialRecords(const JValue& bsdf, std::vector<MatRec>& out);
// Builds the BVH8 (binned SAH BVH2 -> greedy 8-wide collapse -> 8-bit
// quantised child boxes, octant-ordered slots) over the scene's primitives.
void BuildBvh8(HostScene& hs);

}  // namespace rad
