// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_core.h).
// Scene restatement: shapes (rad.offline/src/shape/*.cpp), lights
// (src/light/{area,skybox}.cpp), media (src/medium*.cpp, src/volume/grid.cpp),
// camera (src/camera/perspective.cpp), scene (src/scene.cpp) and the JSON
// builder (src/build/build_context.cpp:47-321). Intersection replaces Embree
// (src/accel/embree.cpp) with a binned-SAH BVH2 and the watertight
// ray/triangle test of Woop, Benthin and Wald (JCGT 2013).
#pragma once
#include <tuple>

#include "ref_bsdf.h"
#include "ref_texture.h"

namespace orc {

struct Ray {
  V3 O, D;
  Float MinT = 0, MaxT = std::numeric_limits<Float>::max();
  V3 At(Float t) const { return D * t + O; }  // ray.h:16
};

// Closest-hit record. `prim` is the global primitive id: the shape's prefix
// offset (shapes in scene-build order) plus the primitive index inside the
// shape, i.e. Embree's (geomID, primID) flattened. u, v follow Embree: the hit
// is (1-u-v)*v0 + u*v1 + v*v2 for triangles and the local (x, y) for quads.
struct Hit {
  Float t = std::numeric_limits<Float>::infinity();
  Float u = 0, v = 0;
  uint32_t prim = 0xffffffffu;
  uint32_t front = 0;
  bool valid() const { return prim != 0xffffffffu; }
};

struct PositionSample {  // sample_result.h:7-13
  V3 P, N;
  V2 UV;
  Float Pdf = 0;
  bool IsDelta = false;
};
struct DirectionSample : PositionSample {  // sample_result.h:15-18
  V3 Dir;
  Float Dist = 0;
};

// RayDifferential (ray.h:35-57): a camera ray's pixel-offset rays
struct RayDiff {
  bool has = false;
  V3 Ox, Oy, Dx, Dy;
};

struct SurfaceInteraction {  // interaction.h:44-110
  Float T = std::numeric_limits<Float>::infinity();
  V3 P, N;
  int shape = -1;
  Frame Shading;
  V2 UV;
  V3 dPdU, dPdV;
  V2 dUVdX, dUVdY;
  V3 Wi;
  // SurfaceInteraction::BSDF(ray) (interaction.cpp:83-109): uv derivatives from
  // a ray's differentials, when it has them.
  void ComputeDifferentials(const RayDiff& rd);
  TexSi Tex() const { return TexSi{UV, dUVdX, dUVdY}; }
  bool IsValid() const { return T != std::numeric_limits<Float>::infinity(); }
  V3 ToWorld(const V3& v) const { return Shading.ToWorld(v); }
  V3 ToLocal(const V3& v) const { return Shading.ToLocal(v); }
};

// interaction.cpp:10-26
inline V3 OffsetP(const V3& P, const V3& N, const V3& d) {
  Float m = std::max(std::max(std::abs(P.x), std::abs(P.y)), std::abs(P.z));
  Float mag = (1 + m) * RayEpsilon;
  mag = MulSign(mag, dot(N, d));
  return Fmadd(V3(mag), N, P);
}
inline Ray SpawnRay(const V3& P, const V3& N, const V3& d) {
  Ray r;
  r.O = OffsetP(P, N, d);
  r.D = d;
  r.MinT = 0;
  r.MaxT = std::numeric_limits<Float>::max();
  return r;
}

// distribution.cpp:19-53
struct Discrete1D {
  std::vector<Float> pmf, cdf;
  Float sum = 0, normalization = 0;
  void Build(const std::vector<Float>& data);
  size_t Sample(Float xi) const;
  std::pair<size_t, Float> SampleReuse(Float xi) const;
};

// distribution.cpp:55-129
struct Continuous1D {
  std::vector<Float> pdf, cdf;
  Float sum = 0, normalization = 0;
  void Build(const Float* f, size_t n);
  size_t Count() const { return pdf.size(); }
  // (index, cdf, pdf) of the sample
  std::tuple<size_t, Float, Float> Sample(Float xi) const;
};
struct Continuous2D {
  std::vector<Continuous1D> conditional;
  Continuous1D marginal;
  void Build(const Float* data, size_t nu, size_t nv);
  // (index u, index v, pdf)
  std::tuple<size_t, size_t, Float> Sample(const V2& xi) const;
  Float Pdf(const V2& uv) const;
};

struct Shape {
  enum Kind { Mesh, Rect, Sphere } kind = Mesh;
  int bsdf = -1, light = -1, inMedium = -1, outMedium = -1;
  bool ownsBsdf = false;
  Float surfaceArea = 0;
  uint32_t primOffset = 0, primCount = 0;
  // mesh (mesh_base.h:40-54)
  std::vector<V3> pos, nrm;
  std::vector<V2> uv;
  bool hasUV = false;
  std::vector<uint32_t> idx;
  Discrete1D dist;
  // rectangle (rectangle.cpp:164-183) and sphere (sphere.cpp:173-193)
  Transform toWorld;
  Frame frame;
  V3 center;
  Float radius = 1;

  PositionSample SamplePosition(const V2& xi) const;
  Float PdfPosition() const;
  DirectionSample SampleDirection(const V3& refP, const V2& xi) const;
  Float PdfDirection(const V3& refP, const DirectionSample& dsr) const;
};

struct Light {
  enum Kind { Area, Skybox, Directional, Point, Projection } kind = Area;
  int shape = -1;
  Spectrum radiance;  // area radiance, skybox constant radiance, directional irradiance,
                      // point intensity, projection irradiance (constant texture)
  Transform toWorld;
  V3 direction;  // directional: world direction the light travels
  V3 worldPos;   // point: world position (point.cpp:22-23)
  Spectrum scale;      // projection: irradiance scale
  Transform toClip;    // projection: light space -> [0,1]^2 image plane (projection.cpp:27-41)
  std::shared_ptr<Texture> map;  // skybox / area: radiance texture (null: constant radiance)
  bool uniformMap = true;        // skybox: 1 x 1 map, uniform sphere sampling
  Continuous2D dist;             // skybox / area: luminance distribution of a bitmap map
  Float cameraArea = 0;          // projection: 1 / area of the image rectangle (projection.cpp:41-44)
  V3 worldCenter;
  Float worldRadius = 0;
  bool IsEnv() const { return kind == Skybox; }
  bool IsDelta() const { return kind == Directional || kind == Point || kind == Projection; }
};

struct Medium {
  enum Kind { Homogeneous, Heterogeneous } kind = Homogeneous;
  // phase function (henyey_greenstein.cpp / isotropic.cpp)
  bool hg = true;
  Float g = 0.8f;
  // homogeneous.cpp:14-41
  Spectrum sigmaT = V3(1), albedoConst = V3(0.75f);
  Float scale = 1;
  // heterogeneous.cpp:15-79
  std::vector<float> grid;  // channel-1 or channel-3 fp32, x fastest
  int nx = 0, ny = 0, nz = 0, channels = 1;
  bool gridSigma = false, repeatWrap = false;
  Float gridMax = 0, maxDensity = 0;
  Transform toWorld;
  V3 bbMin, bbMax;

  Spectrum EvalGrid(const V3& p) const;
  void IntersectAABB(const Ray& ray, bool& active, Float& mint, Float& maxt) const;
  Spectrum Majorant() const;
  void Coefficients(const V3& P, Spectrum& sigmaS, Spectrum& sigmaN, Spectrum& sigmaT) const;
};

struct MediumInteraction {  // interaction.h:112-124
  Float T = std::numeric_limits<Float>::infinity();
  V3 P;
  Frame Shading;
  V3 Wi;
  Float MinT = 0;
  Spectrum SigmaS, SigmaN, SigmaT, CombinedExtinction;
  bool IsValid() const { return T != std::numeric_limits<Float>::infinity(); }
};

struct Camera {  // perspective.cpp:15-70
  int width = 1280, height = 720;
  Float nearZ = 0.001f, farZ = 100;
  Transform cameraToWorld, cameraToClip;
  V3 dx, dy;  // perspective.cpp:56-59
  V2 rectMin, rectMax;  // _imageRect (perspective.cpp:61-65)
  Float normalization = 0;
  Ray SampleRay(const V2& screen) const;
  // Perspective::SampleDirection + Importance (perspective.cpp:101-137): dsr.UV is the pixel position,
  // dsr.Pdf 0 outside the frustum; returns the importance
  Float SampleDirection(const V3& ref, DirectionSample& dsr) const;
  Ray SampleRayDifferential(const V2& screen, RayDiff& diff) const;  // perspective.cpp:84-97
  Float Importance(const V3& d) const;      // perspective.cpp:124-139, d in camera space
  Float PdfWe(const V3& worldDir) const;    // perspective.cpp:141-146: the direction density
};

struct BvhNode {
  V3 lo, hi;
  uint32_t left = 0, first = 0, count = 0;  // leaf iff count > 0
};

struct PrimRef {
  uint32_t shape, local;
};

struct Scene {
  std::vector<std::unique_ptr<Bsdf>> bsdfs;
  std::map<std::string, ImageAsset> images;  // image assets by name
  std::vector<const Texture*> textures;      // every texture, in creation order
  std::vector<Shape> shapes;
  std::vector<Light> lights;
  std::vector<Medium> media;
  int globalMedium = -1;
  int envLight = -1;
  Float lightPdf = 0;
  Camera camera;
  std::string renderer = "path";
  int maxDepth = -1, rrDepth = 3;
  bool useMis = true;  // bdpt.cpp:226 (use_mis)
  int spp = 16;
  uint32_t seed = 0;
  std::vector<PrimRef> prims;
  std::vector<BvhNode> nodes;
  std::vector<uint32_t> order;
  V3 worldLo, worldHi;

  static std::unique_ptr<Scene> FromJson(const std::string& text, const std::string& baseDir);
  void BuildBvh();
  // Accel::RayIntersectPreliminary / RayIntersect (accel.h:10-30)
  Hit Intersect(const Ray& ray) const;
  bool Occluded(const Ray& ray) const;
  bool IntersectPrim(uint32_t prim, const Ray& ray, Hit& hit) const;
  // scene.cpp:42-51 + interaction.cpp:121-127
  bool RayIntersect(const Ray& ray, SurfaceInteraction& si) const;
  bool IsOcclude(const V3& refP, const V3& refN, const V3& p) const;  // scene.cpp:53-63
  // scene.cpp:65-103
  void SampleLight(Float xi, int& index, Float& pdf) const;
  int LightOf(const SurfaceInteraction& si) const;  // scene.cpp:105-113, -1 if none
  std::pair<DirectionSample, Spectrum> SampleLightDirection(const V3& refP, Float xiL, const V2& xi) const;
  std::pair<DirectionSample, Spectrum> SampleOneLightDirection(int light, const V3& refP, const V2& xi) const;
  // Light::SampleRay (area.cpp:120-128, skybox.cpp:135-163, point.cpp:67-71, projection.cpp:93-104);
  // false when the light emits nothing for this sample
  bool LightSampleRay(int light, const V2& xi2, const V2& xi3, Ray& ray, Spectrum& li) const;
  Float PdfLightDirection(int light, const V3& refP, const DirectionSample& dsr) const;
  // Light::SampleLe (area.cpp:130-140, point.cpp:75-85, projection.cpp:107-120, skybox.cpp:170-204): an
  // emitted ray, its radiance, the emitting position and the position / direction densities (0 when the
  // light cannot emit this sample)
  struct LeSample {
    Ray ray;
    Spectrum le = Spectrum(0);
    PositionSample psr;
    Float pdfPos = 0, pdfDir = 0;
  };
  LeSample LightSampleLe(int light, const V2& xi2, const V2& xi3) const;
  // Light::PdfLe (area.cpp:142-147, point.cpp:87-91, projection.cpp:122-133, skybox.cpp:206-212)
  std::pair<Float, Float> LightPdfLe(int light, const PositionSample& psr, const V3& dir) const;
  Spectrum EvalLight(int light, const SurfaceInteraction& si) const;
  // DiffuseArea::SamplePosition (area.cpp:93-115): (position sample, density); a textured light samples its
  // luminance distribution at texel corners of the rectangle (Rectangle::EvalParamSurface, rectangle.cpp:236-250)
  std::pair<PositionSample, Float> LightSamplePosition(int light, const V2& xi) const;
  // the area light's radiance texture at uv (constant radiance without one)
  Spectrum AreaRadiance(const Light& L, const V2& uv) const;
  uint64_t PrimCount() const { return prims.size(); }
};

}  // namespace orc
