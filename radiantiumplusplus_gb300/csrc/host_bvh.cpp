// BVH8 construction, replacing Embree's RTC_BUILD_QUALITY_HIGH build
// (rad.offline/src/accel/embree.cpp:18-43):
//  1. binned SAH binary BVH (32 bins, leaves of at most 3 primitives of one
//     kind), built in parallel over large subtrees;
//  2. greedy collapse into 8-wide nodes (repeatedly open the child with the
//     largest surface area, as in Ylitie et al., "Efficient Incoherent Ray
//     Traversal on GPUs Through Compressed Wide BVHs", HPG 2017);
//  3. child slots assigned by ray octant (greedy on centroid offsets) so a ray
//     visits slot (b ^ octant) for b = 0..7 roughly front to back;
//  4. child boxes quantised to 8 bits per plane against a power-of-two grid,
//     rounded outwards.
// Primitives are laid out in leaf order as 48-byte records (records.h).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>

#include "host_scene.h"

namespace rad {

namespace {

struct Box {
  float lo[3], hi[3];
  void Reset() {
    for (int k = 0; k < 3; k++) {
      lo[k] = INFINITY;
      hi[k] = -INFINITY;
    }
  }
  void Grow(const Box& b) {
    for (int k = 0; k < 3; k++) {
      lo[k] = (b.lo[k] < lo[k]) ? b.lo[k] : lo[k];
      hi[k] = (hi[k] < b.hi[k]) ? b.hi[k] : hi[k];
    }
  }
  void GrowP(const float* p) {
    for (int k = 0; k < 3; k++) {
      lo[k] = (p[k] < lo[k]) ? p[k] : lo[k];
      hi[k] = (hi[k] < p[k]) ? p[k] : hi[k];
    }
  }
  float Area() const {
    float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    if (!(dx >= 0)) return 0.f;
    return dx * dy + dy * dz + dz * dx;
  }
};

struct BNode {
  Box b;
  uint32_t left = 0;             // internal: children left, left + 1
  uint32_t first = 0, count = 0; // leaf: range in the permutation
};

struct Builder {
  const std::vector<Box>& pb;
  const std::vector<float>& cen;  // 3 per prim
  const std::vector<uint8_t>& kind;
  std::vector<uint32_t>& perm;
  std::vector<BNode>& nodes;
  std::atomic<uint32_t> next{1};

  Builder(const std::vector<Box>& b, const std::vector<float>& c, const std::vector<uint8_t>& k,
          std::vector<uint32_t>& p, std::vector<BNode>& n)
      : pb(b), cen(c), kind(k), perm(p), nodes(n) {}

  void MakeLeaf(uint32_t ni, uint32_t b, uint32_t e) {
    nodes[ni].first = b;
    nodes[ni].count = e - b;
  }
  bool MixedKind(uint32_t b, uint32_t e) const {
    for (uint32_t i = b + 1; i < e; i++)
      if (kind[perm[i]] != kind[perm[b]]) return true;
    return false;
  }
  void Split(uint32_t ni, uint32_t b, uint32_t m, uint32_t e, int depth) {
    uint32_t l = next.fetch_add(2);
    nodes[ni].left = l;
    nodes[ni].count = 0;
    if (e - b > 65536 && depth < 5) {
      std::thread t([&, l, b, m, depth]() { Build(l, b, m, depth + 1); });
      Build(l + 1, m, e, depth + 1);
      t.join();
    } else {
      Build(l, b, m, depth + 1);
      Build(l + 1, m, e, depth + 1);
    }
  }

  void Build(uint32_t ni, uint32_t b, uint32_t e, int depth) {
    Box bb, cb;
    bb.Reset();
    cb.Reset();
    for (uint32_t i = b; i < e; i++) {
      bb.Grow(pb[perm[i]]);
      cb.GrowP(&cen[3 * (size_t)perm[i]]);
    }
    nodes[ni].b = bb;
    uint32_t n = e - b;
    if (n == 1 || (n == 2 && !MixedKind(b, e))) {
      MakeLeaf(ni, b, e);
      return;
    }
    constexpr int kBins = 32;
    int bestAxis = -1, bestSplit = -1;
    float bestCost = INFINITY;
    for (int ax = 0; ax < 3; ax++) {
      float ext = cb.hi[ax] - cb.lo[ax];
      if (!(ext > 0)) continue;
      float scale = kBins / ext;
      Box bins[kBins];
      uint32_t cnt[kBins] = {0};
      for (int k = 0; k < kBins; k++) bins[k].Reset();
      for (uint32_t i = b; i < e; i++) {
        uint32_t p = perm[i];
        int k = std::min(kBins - 1, (int)((cen[3 * (size_t)p + ax] - cb.lo[ax]) * scale));
        cnt[k]++;
        bins[k].Grow(pb[p]);
      }
      float rArea[kBins];
      uint32_t rCnt[kBins];
      Box acc;
      acc.Reset();
      uint32_t c = 0;
      for (int k = kBins - 1; k > 0; k--) {
        acc.Grow(bins[k]);
        c += cnt[k];
        rArea[k] = acc.Area();
        rCnt[k] = c;
      }
      acc.Reset();
      c = 0;
      for (int k = 0; k < kBins - 1; k++) {
        acc.Grow(bins[k]);
        c += cnt[k];
        if (c == 0 || rCnt[k + 1] == 0) continue;
        float cost = acc.Area() * c + rArea[k + 1] * rCnt[k + 1];
        if (cost < bestCost) {
          bestCost = cost;
          bestAxis = ax;
          bestSplit = k;
        }
      }
    }
    bool mixed = n <= 3 && MixedKind(b, e);
    float leafCost = bb.Area() * n * 1.2f;  // intersection vs traversal cost
    if (n <= 3 && !mixed && (bestAxis < 0 || leafCost <= bestCost)) {
      MakeLeaf(ni, b, e);
      return;
    }
    uint32_t m;
    if (mixed) {  // leaves hold one kind of primitive: split triangles from analytic ones
      m = (uint32_t)(std::stable_partition(perm.begin() + b, perm.begin() + e,
                                           [&](uint32_t p) { return kind[p] == 0; }) -
                     perm.begin());
    } else if (bestAxis < 0) {  // identical centroids: split the list
      m = b + n / 2;
    } else {
      float ext = cb.hi[bestAxis] - cb.lo[bestAxis];
      float scale = kBins / ext;
      m = (uint32_t)(std::partition(perm.begin() + b, perm.begin() + e,
                                    [&](uint32_t p) {
                                      int k = std::min(kBins - 1,
                                                       (int)((cen[3 * (size_t)p + bestAxis] - cb.lo[bestAxis]) * scale));
                                      return k <= bestSplit;
                                    }) -
                     perm.begin());
      if (m == b || m == e) m = b + n / 2;
    }
    Split(ni, b, m, e, depth);
  }
};

}  // namespace

void BuildBvh8(HostScene& hs) {
  const size_t n = hs.nPrims;
  std::vector<Box> pb(n);
  std::vector<float> cen(3 * n);
  std::vector<uint8_t> kind(n);
  std::vector<uint32_t> shapeOf(n), localOf(n);
  Box world;
  world.Reset();
  // Primitive bounds: triangles by vertices, rectangles by their four corners
  // (rectangle.cpp:48-64), spheres by center +- radius (sphere.cpp:56-69).
  std::vector<int> rectSlot(hs.shapes.size(), -1);
  for (size_t r = 0; r < hs.rectIndexOfShape.size(); r++) rectSlot[hs.rectIndexOfShape[r]] = (int)r;
  for (size_t s = 0; s < hs.shapes.size(); s++) {
    const ShapeRec& sh = hs.shapes[s];
    for (uint32_t k = 0; k < sh.primCount; k++) {
      uint32_t g = sh.primOffset + k;
      shapeOf[g] = (uint32_t)s;
      localOf[g] = k;
      Box b;
      b.Reset();
      if (sh.kind == SHAPE_MESH) {
        kind[g] = 0;
        for (int v = 0; v < 3; v++) b.GrowP(&hs.pos[3 * (size_t)hs.idx[3 * (size_t)(sh.triOffset + k) + v]]);
      } else if (sh.kind == SHAPE_RECT) {
        kind[g] = 1;
        const float* m = sh.m;
        const float cs[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
        for (auto& c : cs) {
          float p[3];
          for (int i = 0; i < 3; i++) p[i] = ((m[i * 4] * c[0] + m[i * 4 + 1] * c[1]) + m[i * 4 + 2] * 0.f) + m[i * 4 + 3];
          b.GrowP(p);
        }
      } else {
        kind[g] = 1;
        for (int i = 0; i < 3; i++) {
          b.lo[i] = sh.m[i] - sh.m[3];
          b.hi[i] = sh.m[i] + sh.m[3];
        }
      }
      for (int i = 0; i < 3; i++) cen[3 * g + i] = (b.lo[i] + b.hi[i]) * 0.5f;
      world.Grow(b);
      if (sh.kind != SHAPE_MESH) {
        // Analytic primitives: the rectangle test runs on the float
        // world->object rows, whose plane differs from the one through the
        // corners by rounding, and a grazing ray turns that into a hit point
        // outside the corner box (the sphere's roots likewise). The boxes the
        // BVH tests grow by 1e-5 of their largest coordinate so traversal never
        // culls a primitive its own test would hit; world bounds and centroids
        // keep the unpadded box.
        float m = 0.f;
        for (int i = 0; i < 3; i++) m = std::max(m, std::max(std::fabs(b.lo[i]), std::fabs(b.hi[i])));
        for (int i = 0; i < 3; i++) {
          b.lo[i] -= m * 1e-5f;
          b.hi[i] += m * 1e-5f;
        }
      }
      pb[g] = b;
    }
  }
  for (int i = 0; i < 3; i++) {
    hs.worldLo[i] = world.lo[i];
    hs.worldHi[i] = world.hi[i];
  }
  hs.nodes.clear();
  hs.prims.clear();
  hs.primInfo.clear();
  if (n == 0) return;

  std::vector<uint32_t> perm(n);
  for (size_t i = 0; i < n; i++) perm[i] = (uint32_t)i;
  std::vector<BNode> bn(2 * n + 1);
  Builder bld(pb, cen, kind, perm, bn);
  bld.Build(0, 0, (uint32_t)n, 0);

  // ---- collapse to 8-wide, breadth first; internal children of a node are contiguous
  struct Task {
    uint32_t bnode, wide;
  };
  std::vector<Task> queue;
  queue.push_back({0, 0});
  hs.nodes.push_back(Bvh8Node{});
  hs.prims.reserve(n);
  hs.primInfo.reserve(2 * n);
  for (size_t qi = 0; qi < queue.size(); qi++) {
    Task t = queue[qi];
    std::vector<uint32_t> ch;
    if (bn[t.bnode].count > 0) {
      ch.push_back(t.bnode);  // root is a leaf: one leaf child
    } else {
      ch.push_back(bn[t.bnode].left);
      ch.push_back(bn[t.bnode].left + 1);
    }
    while (ch.size() < 8) {
      int best = -1;
      float bestA = -1;
      for (size_t c = 0; c < ch.size(); c++) {
        if (bn[ch[c]].count > 0) continue;
        float a = bn[ch[c]].b.Area();
        if (a > bestA) {
          bestA = a;
          best = (int)c;
        }
      }
      if (best < 0) break;
      uint32_t l = bn[ch[best]].left;
      ch[best] = l;
      ch.push_back(l + 1);
    }
    // node box
    Box nb;
    nb.Reset();
    for (uint32_t c : ch) nb.Grow(bn[c].b);
    // octant slot assignment
    int slotOf[8];
    for (int s = 0; s < 8; s++) slotOf[s] = -1;
    {
      float nc[3];
      for (int i = 0; i < 3; i++) nc[i] = (nb.lo[i] + nb.hi[i]) * 0.5f;
      bool used[8] = {false};
      std::vector<bool> done(ch.size(), false);
      for (size_t round = 0; round < ch.size(); round++) {
        float bc = INFINITY;
        int bi = -1, bs = -1;
        for (size_t c = 0; c < ch.size(); c++) {
          if (done[c]) continue;
          float cc[3];
          for (int i = 0; i < 3; i++) cc[i] = (bn[ch[c]].b.lo[i] + bn[ch[c]].b.hi[i]) * 0.5f - nc[i];
          for (int s = 0; s < 8; s++) {
            if (used[s]) continue;
            float d = (s & 1 ? -cc[0] : cc[0]) + (s & 2 ? -cc[1] : cc[1]) + (s & 4 ? -cc[2] : cc[2]);
            if (d < bc) {
              bc = d;
              bi = (int)c;
              bs = s;
            }
          }
        }
        done[bi] = true;
        used[bs] = true;
        slotOf[bs] = bi;
      }
    }
    // quantisation grid
    int ex[3];
    for (int i = 0; i < 3; i++) {
      double extent = (double)nb.hi[i] - (double)nb.lo[i];
      double floorExt = std::max(std::abs((double)nb.lo[i]), std::abs((double)nb.hi[i])) * 1e-6 + 1e-30;
      if (extent < floorExt) extent = floorExt;
      int e = (int)std::ceil(std::log2(extent / 255.0));
      while (extent / std::ldexp(1.0, e) > 255.0) e++;
      while (e > -126 && extent / std::ldexp(1.0, e - 1) <= 255.0) e--;
      e = std::min(std::max(e, -126), 127);
      ex[i] = e;
    }
    float p[3] = {nb.lo[0], nb.lo[1], nb.lo[2]};
    uint32_t imask = 0;
    // empty slots: an inverted box (lo 255, hi 0 on every axis) that no ray passes,
    // so traversal tests all eight slots without checking which are in use
    uint8_t meta[8] = {0}, qlo[3][8], qhi[3][8];
    std::memset(qlo, 255, sizeof(qlo));
    std::memset(qhi, 0, sizeof(qhi));
    uint32_t childBase = (uint32_t)hs.nodes.size();
    uint32_t primBase = (uint32_t)hs.prims.size();
    // internal children first (contiguous, in slot order), then leaf primitives (in slot order)
    for (int s = 0; s < 8; s++) {
      if (slotOf[s] < 0) continue;
      uint32_t c = ch[slotOf[s]];
      const Box& cb = bn[c].b;
      for (int i = 0; i < 3; i++) {
        double sc = std::ldexp(1.0, ex[i]);
        double lo = std::floor(((double)cb.lo[i] - (double)p[i]) / sc);
        double hi = std::ceil(((double)cb.hi[i] - (double)p[i]) / sc);
        lo = std::min(std::max(lo, 0.0), 255.0);
        hi = std::min(std::max(hi, 0.0), 255.0);
        if (hi <= lo) hi = std::min(lo + 1.0, 255.0);
        if (hi <= lo) lo = hi - 1.0;
        qlo[i][s] = (uint8_t)lo;
        qhi[i][s] = (uint8_t)hi;
      }
      if (bn[c].count == 0) {
        imask |= 1u << s;
        uint32_t wi = (uint32_t)hs.nodes.size();
        hs.nodes.push_back(Bvh8Node{});
        queue.push_back({c, wi});
      }
    }
    for (int s = 0; s < 8; s++) {
      if (slotOf[s] < 0) continue;
      uint32_t c = ch[slotOf[s]];
      if (bn[c].count == 0) continue;
      uint32_t off = (uint32_t)hs.prims.size() - primBase;
      uint32_t cnt = bn[c].count;
      bool analytic = kind[perm[bn[c].first]] != 0;
      meta[s] = (uint8_t)((analytic ? 0x80u : 0u) | (cnt << 5) | off);
      for (uint32_t k = 0; k < cnt; k++) {
        uint32_t g = perm[bn[c].first + k];
        const ShapeRec& sh = hs.shapes[shapeOf[g]];
        PrimRec pr;
        std::memset(&pr, 0, sizeof(pr));
        if (sh.kind == SHAPE_MESH) {
          for (int v = 0; v < 3; v++) {
            const float* vp = &hs.pos[3 * (size_t)hs.idx[3 * (size_t)(sh.triOffset + localOf[g]) + v]];
            pr.v[4 * v] = vp[0];
            pr.v[4 * v + 1] = vp[1];
            pr.v[4 * v + 2] = vp[2];
          }
          std::memcpy(&pr.v[3], &g, 4);
          uint32_t sid = shapeOf[g];
          std::memcpy(&pr.v[7], &sid, 4);
        } else if (sh.kind == SHAPE_RECT) {
          std::memcpy(pr.v, &hs.rectToObject[12 * (size_t)rectSlot[shapeOf[g]]], 48);
        } else {
          pr.v[0] = sh.m[0];
          pr.v[1] = sh.m[1];
          pr.v[2] = sh.m[2];
          pr.v[3] = sh.m[3];
        }
        hs.prims.push_back(pr);
        hs.primInfo.push_back(g);
        hs.primInfo.push_back(shapeOf[g] | ((uint32_t)sh.kind << 28));
      }
    }
    Bvh8Node& nd = hs.nodes[t.wide];  // vector may have grown
    std::memcpy(&nd.w[0], &p[0], 4);
    std::memcpy(&nd.w[1], &p[1], 4);
    std::memcpy(&nd.w[2], &p[2], 4);
    nd.w[3] = (uint32_t)(ex[0] + 127) | ((uint32_t)(ex[1] + 127) << 8) | ((uint32_t)(ex[2] + 127) << 16) | (imask << 24);
    nd.w[4] = childBase;
    nd.w[5] = primBase;
    nd.w[6] = meta[0] | (meta[1] << 8) | (meta[2] << 16) | ((uint32_t)meta[3] << 24);
    nd.w[7] = meta[4] | (meta[5] << 8) | (meta[6] << 16) | ((uint32_t)meta[7] << 24);
    auto pack = [](const uint8_t* q, int from) {
      return (uint32_t)q[from] | ((uint32_t)q[from + 1] << 8) | ((uint32_t)q[from + 2] << 16) | ((uint32_t)q[from + 3] << 24);
    };
    nd.w[8] = pack(qlo[0], 0);
    nd.w[9] = pack(qlo[0], 4);
    nd.w[10] = pack(qlo[1], 0);
    nd.w[11] = pack(qlo[1], 4);
    nd.w[12] = pack(qlo[2], 0);
    nd.w[13] = pack(qlo[2], 4);
    nd.w[14] = pack(qhi[0], 0);
    nd.w[15] = pack(qhi[0], 4);
    nd.w[16] = pack(qhi[1], 0);
    nd.w[17] = pack(qhi[1], 4);
    nd.w[18] = pack(qhi[2], 0);
    nd.w[19] = pack(qhi[2], 4);
  }
}

}  // namespace rad
