// Device-resident scene and path-state layouts shared by the host builder and
// the sm_103a kernels. Plain PODs, fixed sizes (static_assert'ed), all float
// data in FP32 as the reference computes (RAD_FLOAT_32_WEIGHT,
// rad.offline/CMakeLists.txt:4,76-82).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define RAD_HD __host__ __device__
#else
#define RAD_HD
#endif

namespace rad {

// ---------------------------------------------------------------- BSDFs
enum MatKind : uint32_t { MAT_NONE = 0, MAT_DIFFUSE = 1, MAT_ROUGH_METAL = 2, MAT_ROUGH_GLASS = 3, MAT_DISNEY = 4,
                          MAT_TWO_SIDE = 5, MAT_PERFECT_MIRROR = 6, MAT_PERFECT_GLASS = 7, MAT_PLASTIC = 8,
                          MAT_ROUGH_PLASTIC = 9, MAT_MASK = 10 };

// BsdfType bits (rad.offline/include/rad/offline/render/bsdf.h:32-50)
enum : uint32_t { BT_DIFFUSE = 1, BT_GLOSSY = 2, BT_DELTA = 4, BT_REFLECTION = 8, BT_TRANSMISSION = 16,
                  BT_NULL = 32, BT_NODELTA = 3 };

// Disney "present" flags (disney.cpp:459-471)
enum : uint32_t { DF_ANISO = 1, DF_SPECTRANS = 2, DF_SHEEN = 4, DF_SHEENTINT = 8, DF_FLATNESS = 16,
                  DF_SPECTINT = 32, DF_METALLIC = 64, DF_CLEARCOAT = 128 };

// One BSDF instance: 96 bytes. p[] layout per kind:
//  diffuse:     p0..2 reflectance
//  rough_metal: p0..2 R, p3..5 eta, p6..8 k, p9 alphaX, p10 alphaY, p11 ggx(1)/beckmann(0), p12 sampleVisible
//  rough_glass: p0..2 R, p3..5 T, p6 eta, p7 invEta, p9 alphaX, p10 alphaY, p11 ggx, p12 sampleVisible
//  disney:      p0..2 baseColor, p3 roughness, p4 anisotropic, p5 specTrans, p6 sheen, p7 sheenTint,
//               p8 flatness, p9 specTint, p10 metallic, p11 clearcoat, p12 clearcoatGloss, p13 eta,
//               p14 specularSample, p15 clearcoatSample; aux = diffuseReflectSample
//  perfect_mirror: p0..2 reflectance, p3..5 eta, p6..8 k
//  perfect_glass:  p0..2 R, p3..5 T, p6 eta
//  plastic, rough_plastic: p0..2 diffuse, p3..5 specular, p6 eta, p7 1/eta^2, p8 internal diffuse
//               Fresnel reflectance, p9..12 microfacet (rough_plastic), p13 specular sampling
//               weight, p14 no_linear
//  two_side:    ref0 outside material index, ref1 inside material index
//  mask:        p0 opacity clamped to [0, 1], ref0 nested material index
struct alignas(16) MatRec {
  uint32_t kind;
  uint32_t flags;      // BsdfType bits of the instance
  uint32_t dflags;     // Disney present flags
  uint32_t ref0, ref1; // two_side / mask children
  float aux;           // disney: diffuse_reflectance_sampling_rate
  uint32_t texFirst;   // textured parameters: first TexBind of this record
  uint32_t texCount;   //   and their number (0: all parameters constant)
  float p[16];
};
static_assert(sizeof(MatRec) == 96, "MatRec must stay 96 bytes");
// Deepest chain of wrapper BSDFs (two_side, mask) above a leaf BSDF.
constexpr int kMaxBsdfNest = 4;

// ---------------------------------------------------------------- textures
// Texture records (texture.h:47-90, bitmap.cpp:24-344, chessboard.cpp:15-63).
// A constant texture holds its value; a bitmap holds its mip chain in the texel
// pool (level l: max(1, w >> l) x max(1, h >> l) texels of `channels` floats, rows
// of increasing y, from levelOffset[l]); a chessboard holds its uv transform and
// the two textures it picks between.
enum TexKind : uint32_t { TEX_CONST = 0, TEX_BITMAP = 1, TEX_CHESS = 2 };
enum TexFilter : uint32_t { TF_NEAREST = 0, TF_BILINEAR = 1, TF_TRILINEAR = 2, TF_ANISO = 3 };
constexpr int kMaxMipLevels = 16;
constexpr int kMaxTexNest = 8;  // deepest chessboard chain above a leaf texture
struct alignas(16) TexRec {
  uint32_t kind, channels, filter, wrap;  // wrap: 0 clamp, 1 repeat
  uint32_t width, height, levels, remap;
  float value[3];
  float aniso;                            // anisotropic_level
  uint32_t childA, childB, pad[2];
  union {
    uint32_t levelOffset[kMaxMipLevels];  // bitmap: first float of each level
    float toUV[16];                       // chessboard: uv transform, row-major 4x4
  };
};
static_assert(sizeof(TexRec) == 128, "TexRec size");
// One textured BSDF parameter: p[slot .. slot+channels) comes from texture `tex`.
struct TexBind {
  uint16_t slot;
  uint8_t channels;
  uint8_t clamp01;  // mask opacity is clamped to [0, 1] after the lookup (mask.cpp:66-68)
  uint32_t tex;
};
static_assert(sizeof(TexBind) == 8, "TexBind size");

// ---------------------------------------------------------------- shapes
enum ShapeKind : uint32_t { SHAPE_MESH = 0, SHAPE_RECT = 1, SHAPE_SPHERE = 2 };

// One shape: 208 bytes.
struct alignas(16) ShapeRec {
  uint32_t kind;
  int32_t bsdf, light, inMedium, outMedium;
  uint32_t primOffset, primCount;  // global primitive id range
  uint32_t triOffset;              // mesh: first triangle in the global index array
  uint32_t hasNormals, hasUV;
  uint32_t cdfOffset;              // mesh: area CDF offset (emitters)
  float surfaceArea;
  float cdfSum, cdfNorm;           // DiscreteDistribution1D sum / normalization
  uint32_t pad0[2];
  // rect: toWorld rows (3x4), frame S/T/N; sphere: center, radius, toLocal rows (3x4), toWorld linear (3x3)
  float m[36];
};
static_assert(sizeof(ShapeRec) == 208, "ShapeRec size");

// ---------------------------------------------------------------- lights
enum LightKind : uint32_t { LIGHT_AREA = 0, LIGHT_SKYBOX = 1, LIGHT_DIRECTIONAL = 2, LIGHT_POINT = 3,
                            LIGHT_PROJECTION = 4 };
struct alignas(16) LightRec {
  uint32_t kind;
  int32_t shape;
  uint32_t tex;        // skybox: radiance texture + 1 (0: constant radiance)
  uint32_t dist;       // skybox with a bitmap: first float of its 2D luminance distribution
  float radiance[4];   // rgb: area radiance, sky radiance, directional irradiance, point intensity,
                       // projection irradiance x scale
  float dir[4];        // directional: world direction the light travels; point / projection: world position
  float world[4];      // world bounding sphere center xyz, radius w (skybox.cpp:139-144)
  float lin[12];       // skybox toWorld linear part, rows of 4; projection: world-space normal (lin[0..2])
  float m[32];         // projection: world -> light 4x4 (m[0..15]), light -> clip 4x4 (m[16..31]);
                       // skybox: world -> light 4x4 (m[0..15])
  uint32_t distW, distH;  // skybox with a bitmap: distribution size (texels); 0: uniform sphere sampling
  uint32_t pad2[2];
  float m2[32];        // projection: clip -> light 4x4 (m2[0..15]), light -> world linear rows of 4 (m2[16..27]),
                       // 1 / image-rectangle area (m2[28]; projection.cpp:41-44), irradiance without the
                       // scale (m2[29..31]: SampleRay / SampleLe, projection.cpp:93-120)
};
static_assert(sizeof(LightRec) == 384, "LightRec size");

// bdpt: vertices of one subpath at most (camera or light vertex included)
constexpr int kMaxBdptVertices = 64;
// particle_tracer: bounces of one light path at most (max_depth -1 is capped like camera paths)
constexpr int kMaxLightBounces = 256;

// ---------------------------------------------------------------- media
enum MediumKind : uint32_t { MED_HOMOGENEOUS = 0, MED_HETEROGENEOUS = 1 };
struct alignas(16) MediumRec {
  uint32_t kind;
  uint32_t hg;            // 1 = henyey-greenstein, 0 = isotropic
  uint32_t gridSigma;     // sigma_t from a grid
  uint32_t repeatWrap;
  float g, scale, maxDensity, pad0;
  float sigmaT[4], albedo[4];
  float bbMin[4], bbMax[4];
  float toLocal[12];      // heterogeneous: world -> [0,1]^3 grid space, rows of 4
  int32_t nx, ny, nz, channels;
  uint64_t gridOffset;    // element offset of the grid in the volume pools (fp32 and fp16 copies)
  uint32_t brickOffset;   // first 16^3-brick majorant in the brick pool
  uint32_t hasBricks;     // 1: brick majorants exist (clamped grids)
};
static_assert(sizeof(MediumRec) == 176, "MediumRec size");

// ---------------------------------------------------------------- camera
struct alignas(16) CameraRec {
  float clipToCamera[16];  // cameraToClip.ToLocal (perspective.cpp:79)
  float camToWorld[16];    // cameraToWorld.ToWorld
  float nearZ, farZ;
  int32_t width, height;
  float dx[4], dy[4];      // camera-space offsets of one pixel step (perspective.cpp:56-59)
  float worldToCam[16];    // cameraToWorld.ToLocal
  float camToClip[16];     // cameraToClip.ToWorld
  float rect[4];           // image-plane rectangle at z = 1 (min x, min y, max x, max y), perspective.cpp:61-65
  float normalization;     // 1 / its area
  float pad[3];
};

// ---------------------------------------------------------------- BVH8
// 80-byte 8-wide node with 8-bit quantised child boxes (5 x uint4):
//  q0 = (px, py, pz, ex | ey<<8 | ez<<16 | imask<<24)
//  q1 = (childBase, primBase, meta[0..3], meta[4..7])
//  q2 = (qlo.x[0..7], qlo.y[0..7]); q3 = (qlo.z[0..7], qhi.x[0..7]); q4 = (qhi.y[0..7], qhi.z[0..7])
// Child slot s is internal when imask bit s is set (node = childBase + number
// of internal slots below s). Otherwise meta[s] = 0 marks an empty slot, else
// bit 7 = analytic primitives, bits 6..5 = primitive count (1..3), bits 4..0 =
// offset from primBase. Slots are assigned by ray octant at build time so that
// visiting slot (b ^ octant) for b = 0..7 is close to front-to-back.
struct alignas(16) Bvh8Node {
  uint32_t w[20];
};
static_assert(sizeof(Bvh8Node) == 80, "Bvh8Node must be 80 bytes");

// Leaf-order primitive record, 48 bytes (3 x float4):
//  triangle: (v0, prim id bits) (v1, shape id bits) (v2, 0)
//  rectangle: rows of the float32 world->object matrix (rectangle.cpp:34-46)
//  sphere:   (center, radius) (-, -, -, -) (-, -, -, -)
// primInfo (uint2, leaf order): (global prim id, shape id | kind << 28).
struct alignas(16) PrimRec {
  float v[12];
};
static_assert(sizeof(PrimRec) == 48, "PrimRec must be 48 bytes");

// ---------------------------------------------------------------- scene
// Shade classes: the extend stage sorts hits into one queue per class so that
// each shade kernel runs one BSDF's code. 0 = miss / emitter / no BSDF (emission
// only), 1..4 = MatKind of the (possibly two-sided) leaf BSDF, 5 = anything else.
enum : uint32_t { SC_EMIT = 0, SC_DIFFUSE = 1, SC_METAL = 2, SC_GLASS = 3, SC_DISNEY = 4, SC_GENERIC = 5 };
constexpr int kShadeClasses = 6;

struct DevScene {
  const Bvh8Node* nodes;
  const PrimRec* prims;
  const uint32_t* primInfo;   // 2 words per leaf-order primitive
  const ShapeRec* shapes;
  const MatRec* mats;
  const LightRec* lights;
  const MediumRec* media;
  const float* pos;            // global vertex positions, 3 floats each
  const float* nrm;            // global vertex normals (or null)
  const float* uv;             // global vertex uvs (or null)
  const uint32_t* idx;         // global triangle indices, 3 per triangle
  const float* cdf;            // emitter-mesh area CDF / PMF (2 floats per triangle)
  const float* volume;         // density grids
  const uint16_t* volumeHalf;  // fp16 copy of the density grids (bit patterns)
  const float* brickMaj;       // per-medium 16^3-brick majorants (scale applied)
  const uint8_t* shapeClass;   // shade class per shape
  const TexRec* tex;           // textures
  const float* texels;         // texel pool
  const TexBind* texBind;      // textured BSDF parameters
  const float* lightDist;      // 2D luminance distributions of textured skyboxes
  uint32_t nNodes, nPrims, nShapes, nLights;
  uint32_t nMedia, nMats;
  uint32_t nTex, needDiff;     // needDiff: a trilinear / anisotropic texture reads ray differentials
  int32_t envLight, globalMedium;
  float lightPdf;
  int32_t maxDepth, rrDepth, isVol;
  int32_t isAO;                // renderer "ao" (ao.cpp): one hit, one cosine-sampled visibility ray
  int32_t isParticle;          // renderer "particle_tracer": light paths splatted into the film
  int32_t isBdpt, bdptMis;     // renderer "bdpt"; its use_mis flag
  CameraRec cam;
};

// Hit record written by the extend kernel, 32 bytes.
struct alignas(16) HitRec {
  float t, u, v;
  uint32_t prim;   // global prim id, 0xffffffff = miss
  uint32_t shape;
  uint32_t front;
  uint32_t pad[2];
};

}  // namespace rad
