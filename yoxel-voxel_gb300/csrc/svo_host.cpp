// svo_host.cpp - host-side SVO scene data: seeded generators, the .vox
// reader/writer, pool validation and the breadth-first device re-layout.
//
// Reference counterparts (znah/yoxel-voxel):
//   SVOData::Load                     cell/svodata.h:31-50
//   VoxNode / EmptyNode / FullNode    reaction/report/main.tex:36-56
//   surface voxel + normal rule       scene_gen.py:32-66
//   DynamicSVO::BuildRange (GROW)     ore/src/main.cpp:121-129 (source absent;
//                                     restated as a top-down region build)
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "yv_internal.h"

namespace yv {

static std::mutex g_err_mu;
static std::string g_last_error;
void set_last_error(const std::string& s) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_last_error = s;
}
const char* last_error_cstr() {
  static thread_local std::string copy;
  std::lock_guard<std::mutex> lk(g_err_mu);
  copy = g_last_error;
  return copy.c_str();
}

uint64_t hash64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

int hardware_threads() {
  unsigned n = std::thread::hardware_concurrency();
  if (n == 0) n = 1;
  if (n > 64) n = 64;
  return (int)n;
}

// ---------------------------------------------------------------------------
// Camera (RendererBase::InitRayDir, cell/renderer_base.h:50-61).  Host code is
// compiled with -ffp-contract=off: one rounding per written operation.
// ---------------------------------------------------------------------------
static void normalize3(float* v) {
  float len = std::sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
  v[0] = v[0] / len;
  v[1] = v[1] / len;
  v[2] = v[2] / len;
}

void init_ray_dir(const float dir[3], const float up[3], float fov_deg,
                  int width, int height, float dir0[3], float du[3],
                  float dv[3]) {
  float vfwd[3] = {dir[0], dir[1], dir[2]};
  normalize3(vfwd);
  float vright[3] = {vfwd[1] * up[2] - vfwd[2] * up[1],
                     vfwd[2] * up[0] - vfwd[0] * up[2],
                     vfwd[0] * up[1] - vfwd[1] * up[0]};
  normalize3(vright);
  float vup[3] = {vright[1] * vfwd[2] - vright[2] * vfwd[1],
                  vright[2] * vfwd[0] - vright[0] * vfwd[2],
                  vright[0] * vfwd[1] - vright[1] * vfwd[0]};
  float half = fov_deg / 2.0f;
  float rad = half * (float)(3.14159265358979323846 / 180.0);
  float da = std::tan(rad) / (float)width;
  for (int i = 0; i < 3; ++i) {
    du[i] = (2.0f * vright[i]) * da;
    dv[i] = (-2.0f * vup[i]) * da;
  }
  for (int i = 0; i < 3; ++i) {
    float a = (du[i] * (float)width) / 2.0f;
    float b = (dv[i] * (float)height) / 2.0f;
    dir0[i] = (vfwd[i] - a) - b;
  }
}

void adjust_dir(float d[3]) {
  const float eps = 1e-5f;
  for (int i = 0; i < 3; ++i)
    if (std::fabs(d[i]) < eps) d[i] = std::copysign(eps, d[i]);
}

// ---------------------------------------------------------------------------
// Top-down region builder.
//
// A node exists for a cube region iff the region holds at least one surface
// voxel (inside the solid, with a 6-neighbour outside; neighbours outside the
// grid count as outside).  A region without surface voxels is uniformly
// inside (FullNode) or outside (EmptyNode).  Sources give an exact voxel
// membership test plus conservative region tests; children that all come
// back EMPTY (FULL) collapse to EMPTY (FULL), so the result is canonical
// whatever the region tests prove early.
// ---------------------------------------------------------------------------
enum { CLS_MIXED = 0, CLS_EMPTY = 1, CLS_FULL = 2 };

template <class Src>
struct Builder {
  const Src& src;
  int G;
  std::vector<yv_vox_node> nodes;
  std::vector<yv_leaf_attr> attrs;
  std::vector<std::vector<int>> cand;  // candidate primitives per level

  Builder(const Src& s, int g) : src(s), G(g) {}

  bool surface(int x, int y, int z, const std::vector<int>& c) const {
    static const int nb[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0},
                                 {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
    for (int k = 0; k < 6; ++k) {
      int nx = x + nb[k][0], ny = y + nb[k][1], nz = z + nb[k][2];
      if (nx < 0 || ny < 0 || nz < 0 || nx >= G || ny >= G || nz >= G)
        return true;
      if (!src.inside(nx, ny, nz, c)) return true;
    }
    return false;
  }

  // Returns YV_EMPTY_NODE, YV_FULL_NODE or a local node index.
  uint32_t build(int x0, int y0, int z0, int s, int lvl) {
    if ((int)cand.size() <= lvl + 1) cand.resize((size_t)lvl + 2);
    const std::vector<int>& cin = cand[(size_t)lvl];
    std::vector<int>& cout = cand[(size_t)lvl + 1];
    int cls = src.classify(x0, y0, z0, s, cin, cout);
    if (cls == CLS_EMPTY) return YV_EMPTY_NODE;
    if (cls == CLS_FULL) return YV_FULL_NODE;
    yv_vox_node n;
    std::memset(&n, 0, sizeof(n));
    int n_empty = 0, n_full = 0;
    if (s == 2) {
      const std::vector<int>& c = cout;
      for (int ch = 0; ch < 8; ++ch) {
        int x = x0 + (ch & 1), y = y0 + ((ch >> 1) & 1), z = z0 + ((ch >> 2) & 1);
        if (!src.inside(x, y, z, c)) {
          n.child[ch] = YV_EMPTY_NODE;
          ++n_empty;
        } else if (surface(x, y, z, c)) {
          n.child[ch] = (uint32_t)attrs.size();
          n.flags |= 1u << ch;
          attrs.push_back(src.attr(x, y, z, c));
        } else {
          n.child[ch] = YV_FULL_NODE;
          ++n_full;
        }
      }
    } else {
      int h = s / 2;
      uint32_t w[8];
      for (int ch = 0; ch < 8; ++ch) {
        w[ch] = build(x0 + (ch & 1) * h, y0 + ((ch >> 1) & 1) * h,
                      z0 + ((ch >> 2) & 1) * h, h, lvl + 1);
        if (w[ch] == YV_EMPTY_NODE) ++n_empty;
        if (w[ch] == YV_FULL_NODE) ++n_full;
        n.child[ch] = w[ch];
      }
    }
    if (n_empty == 8) return YV_EMPTY_NODE;
    if (n_full == 8) return YV_FULL_NODE;
    for (int ch = 0; ch < 8; ++ch)
      if (!((n.flags >> ch) & 1u) && (n.child[ch] & 0x80000000u))
        n.flags |= 1u << (8 + ch);
    nodes.push_back(n);
    return (uint32_t)(nodes.size() - 1);
  }
};

// Canonical breadth-first numbering of nodes and leaves.
static void canonicalize(const std::vector<yv_vox_node>& in_nodes,
                         const std::vector<yv_leaf_attr>& in_attrs,
                         uint32_t root, yv_svo_host* out) {
  out->nodes.clear();
  out->attrs.clear();
  if (root & 0x80000000u) {
    out->root = root;
    return;
  }
  out->nodes.reserve(in_nodes.size());
  out->attrs.reserve(in_attrs.size());
  std::vector<uint32_t> order;
  order.reserve(in_nodes.size());
  order.push_back(root);
  for (size_t i = 0; i < order.size(); ++i) {
    const yv_vox_node& n = in_nodes[order[i]];
    for (int ch = 0; ch < 8; ++ch)
      if (!((n.flags >> ch) & 1u) && !(n.child[ch] & 0x80000000u))
        order.push_back(n.child[ch]);
  }
  // positions in `order` are the new ids (tree: each node reached once)
  uint32_t next_node = 1;
  for (size_t i = 0; i < order.size(); ++i) {
    yv_vox_node n = in_nodes[order[i]];
    for (int ch = 0; ch < 8; ++ch) {
      if ((n.flags >> ch) & 1u) {
        out->attrs.push_back(in_attrs[n.child[ch]]);
        n.child[ch] = (uint32_t)(out->attrs.size() - 1);
      } else if (!(n.child[ch] & 0x80000000u)) {
        n.child[ch] = next_node++;
      }
    }
    out->nodes.push_back(n);
  }
  out->root = 0;
}

// Builds the 64 level-2 subtrees on worker threads, then the two top levels.
template <class Src>
static void build_tree(const Src& src, int depth, yv_svo_host* out) {
  const int G = 1 << depth;
  out->depth = depth;
  if (depth < 3) {
    Builder<Src> b(src, G);
    b.cand.resize((size_t)depth + 2);
    src.all_candidates(b.cand[0]);
    uint32_t r = b.build(0, 0, 0, G, 0);
    canonicalize(b.nodes, b.attrs, r, out);
    return;
  }
  const int q = G / 4;
  struct Sub {
    std::vector<yv_vox_node> nodes;
    std::vector<yv_leaf_attr> attrs;
    uint32_t word;
  };
  std::vector<Sub> subs(64);
  std::vector<int> all;
  src.all_candidates(all);
  int nth = std::min(hardware_threads(), 64);
  std::vector<std::thread> th;
  std::atomic_int next{0};
  for (int t = 0; t < nth; ++t)
    th.emplace_back([&]() {
      for (;;) {
        int i = next.fetch_add(1);
        if (i >= 64) break;
        // subtree i = level-1 child (i>>3), level-2 child (i&7)
        int c1 = i >> 3, c2 = i & 7;
        int x0 = (c1 & 1) * 2 * q + (c2 & 1) * q;
        int y0 = ((c1 >> 1) & 1) * 2 * q + ((c2 >> 1) & 1) * q;
        int z0 = ((c1 >> 2) & 1) * 2 * q + ((c2 >> 2) & 1) * q;
        Builder<Src> b(src, G);
        b.cand.resize((size_t)depth + 2);
        b.cand[0] = all;
        subs[(size_t)i].word = b.build(x0, y0, z0, q, 0);
        subs[(size_t)i].nodes.swap(b.nodes);
        subs[(size_t)i].attrs.swap(b.attrs);
      }
    });
  for (auto& t : th) t.join();
  // merge subtree arrays with offsets
  std::vector<yv_vox_node> nodes;
  std::vector<yv_leaf_attr> attrs;
  size_t tot_n = 0, tot_a = 0;
  for (auto& s : subs) {
    tot_n += s.nodes.size();
    tot_a += s.attrs.size();
  }
  nodes.reserve(tot_n + 9);
  attrs.reserve(tot_a);
  std::vector<uint32_t> sub_word(64);
  for (int i = 0; i < 64; ++i) {
    Sub& s = subs[(size_t)i];
    uint32_t noff = (uint32_t)nodes.size(), aoff = (uint32_t)attrs.size();
    for (auto n : s.nodes) {
      for (int ch = 0; ch < 8; ++ch) {
        if ((n.flags >> ch) & 1u)
          n.child[ch] += aoff;
        else if (!(n.child[ch] & 0x80000000u))
          n.child[ch] += noff;
      }
      nodes.push_back(n);
    }
    attrs.insert(attrs.end(), s.attrs.begin(), s.attrs.end());
    sub_word[(size_t)i] =
        (s.word & 0x80000000u) ? s.word : s.word + noff;
    std::vector<yv_vox_node>().swap(s.nodes);
    std::vector<yv_leaf_attr>().swap(s.attrs);
  }
  auto combine = [&](const uint32_t* w) -> uint32_t {
    int ne = 0, nf = 0;
    yv_vox_node n;
    std::memset(&n, 0, sizeof(n));
    for (int ch = 0; ch < 8; ++ch) {
      n.child[ch] = w[ch];
      if (w[ch] == YV_EMPTY_NODE) ++ne;
      if (w[ch] == YV_FULL_NODE) ++nf;
      if (w[ch] & 0x80000000u) n.flags |= 1u << (8 + ch);
    }
    if (ne == 8) return YV_EMPTY_NODE;
    if (nf == 8) return YV_FULL_NODE;
    nodes.push_back(n);
    return (uint32_t)(nodes.size() - 1);
  };
  uint32_t l1[8];
  for (int c1 = 0; c1 < 8; ++c1) l1[c1] = combine(&sub_word[(size_t)c1 * 8]);
  uint32_t root = combine(l1);
  canonicalize(nodes, attrs, root, out);
}

static int8_t quant_n(double v) {
  double q = std::floor(127.0 * v + 0.5);
  if (q > 127.0) q = 127.0;
  if (q < -127.0) q = -127.0;
  return (int8_t)(int)q;
}

static void normal_attr(yv_leaf_attr* a, double nx, double ny, double nz) {
  double len = std::sqrt(nx * nx + ny * ny + nz * nz);
  if (len > 0) {
    nx /= len;
    ny /= len;
    nz /= len;
  } else {
    nx = ny = nz = 0;
  }
  a->nx = quant_n(nx);
  a->ny = quant_n(ny);
  a->nz = quant_n(nz);
  a->nw = 0;
}

// ---------------------------------------------------------------------------
// Sphere-union source (the cfg "200 spheres in 256^3" scene family).
// ---------------------------------------------------------------------------
struct SphereSrc {
  int G;
  std::vector<double> cx, cy, cz, r2;
  std::vector<uint8_t> rgb;

  void all_candidates(std::vector<int>& c) const {
    c.resize(cx.size());
    for (size_t i = 0; i < cx.size(); ++i) c[i] = (int)i;
  }
  static double box_d2(double c, double lo, double hi) {
    double d = c < lo ? lo - c : (c > hi ? c - hi : 0.0);
    return d * d;
  }
  static double far_d2(double c, double lo, double hi) {
    double a = c - lo, b = hi - c;
    double d = std::fabs(a) > std::fabs(b) ? a : b;
    return d * d;
  }
  int classify(int x0, int y0, int z0, int s, const std::vector<int>& in,
               std::vector<int>& out) const {
    // voxel centres of the region and of the region grown by one voxel
    double lo[3] = {x0 + 0.5, y0 + 0.5, z0 + 0.5};
    double hi[3] = {x0 + s - 0.5, y0 + s - 0.5, z0 + s - 0.5};
    out.clear();
    bool any_in = false;
    for (int i : in) {
      double c[3] = {cx[(size_t)i], cy[(size_t)i], cz[(size_t)i]};
      double r = r2[(size_t)i];
      double m = 1e-9 * (r + 1.0);
      double de = 0, dr = 0;
      for (int k = 0; k < 3; ++k) {
        de += box_d2(c[k], lo[k] - 1.0, hi[k] + 1.0);
        dr += box_d2(c[k], lo[k], hi[k]);
      }
      if (de <= r + m) out.push_back(i);
      if (dr <= r + m) any_in = true;
    }
    if (!any_in) return CLS_EMPTY;
    if (x0 >= 1 && y0 >= 1 && z0 >= 1 && x0 + s <= G - 1 && y0 + s <= G - 1 &&
        z0 + s <= G - 1) {
      for (int i : out) {
        double c[3] = {cx[(size_t)i], cy[(size_t)i], cz[(size_t)i]};
        double f = 0;
        for (int k = 0; k < 3; ++k) f += far_d2(c[k], lo[k] - 1.0, hi[k] + 1.0);
        if (f < r2[(size_t)i] - 1e-9 * (r2[(size_t)i] + 1.0)) return CLS_FULL;
      }
    }
    return CLS_MIXED;
  }
  int first(int x, int y, int z, const std::vector<int>& c) const {
    double px = x + 0.5, py = y + 0.5, pz = z + 0.5;
    for (int i : c) {
      double dx = px - cx[(size_t)i], dy = py - cy[(size_t)i], dz = pz - cz[(size_t)i];
      if (dx * dx + dy * dy + dz * dz <= r2[(size_t)i]) return i;
    }
    return -1;
  }
  bool inside(int x, int y, int z, const std::vector<int>& c) const {
    return first(x, y, z, c) >= 0;
  }
  yv_leaf_attr attr(int x, int y, int z, const std::vector<int>& c) const {
    int i = first(x, y, z, c);
    yv_leaf_attr a;
    std::memset(&a, 0, sizeof(a));
    a.r = rgb[(size_t)i * 3];
    a.g = rgb[(size_t)i * 3 + 1];
    a.b = rgb[(size_t)i * 3 + 2];
    a.a = 255;
    normal_attr(&a, x + 0.5 - cx[(size_t)i], y + 0.5 - cy[(size_t)i],
                z + 0.5 - cz[(size_t)i]);
    return a;
  }
};

// ---------------------------------------------------------------------------
// Terrain source: value-noise heightfield + floating cubes.
// ---------------------------------------------------------------------------
struct TerrainSrc {
  int G = 0, depth = 0;
  std::vector<int16_t> h;                      // column height (solid z <= h)
  std::vector<std::vector<int16_t>> hmin, hmax;  // per level (block 2^k)
  std::vector<int> c0x, c0y, c0z, cs;          // cubes
  std::vector<uint8_t> crgb;

  int H(int x, int y) const { return h[(size_t)y * (size_t)G + (size_t)x]; }

  void all_candidates(std::vector<int>& c) const {
    c.resize(cs.size());
    for (size_t i = 0; i < cs.size(); ++i) c[i] = (int)i;
  }
  // min/max height of the aligned block containing (x0, y0) at size s
  int block_min(int lvl, int bx, int by) const {
    int n = G >> lvl;
    if (bx < 0 || by < 0 || bx >= n || by >= n) return -1;
    return hmin[(size_t)lvl][(size_t)by * (size_t)n + (size_t)bx];
  }
  int classify(int x0, int y0, int z0, int s, const std::vector<int>& in,
               std::vector<int>& out) const {
    int lvl = 0;
    while ((1 << lvl) < s) ++lvl;
    int n = G >> lvl, bx = x0 >> lvl, by = y0 >> lvl;
    int hmx = hmax[(size_t)lvl][(size_t)by * (size_t)n + (size_t)bx];
    out.clear();
    bool cube_in = false;
    for (int i : in) {
      int a0 = c0x[(size_t)i], b0 = c0y[(size_t)i], e0 = c0z[(size_t)i], w = cs[(size_t)i];
      // cube [a0, a0+w) vs region grown by one voxel
      if (a0 + w <= x0 - 1 || a0 >= x0 + s + 1 || b0 + w <= y0 - 1 ||
          b0 >= y0 + s + 1 || e0 + w <= z0 - 1 || e0 >= z0 + s + 1)
        continue;
      out.push_back(i);
      if (!(a0 + w <= x0 || a0 >= x0 + s || b0 + w <= y0 || b0 >= y0 + s ||
            e0 + w <= z0 || e0 >= z0 + s))
        cube_in = true;
    }
    if (z0 > hmx && !cube_in) return CLS_EMPTY;
    if (x0 >= 1 && y0 >= 1 && z0 >= 1 && x0 + s <= G - 1 && y0 + s <= G - 1) {
      int mn = 1 << 30;
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx)
          mn = std::min(mn, block_min(lvl, bx + dx, by + dy));
      if (mn >= z0 + s) return CLS_FULL;
    }
    return CLS_MIXED;
  }
  int cube_of(int x, int y, int z, const std::vector<int>& c) const {
    for (int i : c) {
      int a0 = c0x[(size_t)i], b0 = c0y[(size_t)i], e0 = c0z[(size_t)i], w = cs[(size_t)i];
      if (x >= a0 && x < a0 + w && y >= b0 && y < b0 + w && z >= e0 && z < e0 + w)
        return i;
    }
    return -1;
  }
  bool inside(int x, int y, int z, const std::vector<int>& c) const {
    if (z <= H(x, y)) return true;
    return cube_of(x, y, z, c) >= 0;
  }
  bool in_grid_inside(int x, int y, int z, const std::vector<int>& c) const {
    if (x < 0 || y < 0 || z < 0 || x >= G || y >= G || z >= G) return false;
    return inside(x, y, z, c);
  }
  yv_leaf_attr attr(int x, int y, int z, const std::vector<int>& c) const {
    yv_leaf_attr a;
    std::memset(&a, 0, sizeof(a));
    a.a = 255;
    if (z > H(x, y)) {
      int i = cube_of(x, y, z, c);
      a.r = crgb[(size_t)i * 3];
      a.g = crgb[(size_t)i * 3 + 1];
      a.b = crgb[(size_t)i * 3 + 2];
      double hw = cs[(size_t)i] * 0.5;
      double nx = x + 0.5 - (c0x[(size_t)i] + hw), ny = y + 0.5 - (c0y[(size_t)i] + hw),
             nz = z + 0.5 - (c0z[(size_t)i] + hw);
      if (nx == 0 && ny == 0 && nz == 0) nz = 1;
      normal_attr(&a, nx, ny, nz);
      return a;
    }
    // height-banded palette with per-voxel hash noise
    double t = (double)z / (double)G;
    double lowc[3] = {70, 130, 55}, midc[3] = {150, 115, 75}, hic[3] = {225, 225, 230};
    double col[3];
    for (int k = 0; k < 3; ++k) {
      double u = (t - 0.35) / 0.3;
      u = u < 0 ? 0 : (u > 1 ? 1 : u);
      double v = (t - 0.62) / 0.1;
      v = v < 0 ? 0 : (v > 1 ? 1 : v);
      col[k] = lowc[k] + (midc[k] - lowc[k]) * u;
      col[k] = col[k] + (hic[k] - col[k]) * v;
    }
    uint64_t hh = hash64(((uint64_t)(uint32_t)x << 42) ^ ((uint64_t)(uint32_t)y << 21) ^ (uint64_t)(uint32_t)z);
    int jit = (int)(hh & 31) - 16;
    a.r = (uint8_t)std::max(0, std::min(255, (int)col[0] + jit));
    a.g = (uint8_t)std::max(0, std::min(255, (int)col[1] + jit));
    a.b = (uint8_t)std::max(0, std::min(255, (int)col[2] + jit));
    if (!in_grid_inside(x, y, z + 1, c)) {
      int xm = std::max(0, x - 1), xp = std::min(G - 1, x + 1);
      int ym = std::max(0, y - 1), yp = std::min(G - 1, y + 1);
      double gx = (H(xp, y) - H(xm, y)) * 0.5, gy = (H(x, yp) - H(x, ym)) * 0.5;
      normal_attr(&a, -gx, -gy, 1.0);
    } else {
      double n[3] = {0, 0, 0};
      static const int nb[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0},
                                   {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
      for (int k = 0; k < 6; ++k)
        if (!in_grid_inside(x + nb[k][0], y + nb[k][1], z + nb[k][2], c))
          for (int j = 0; j < 3; ++j) n[j] += nb[k][j];
      if (n[0] == 0 && n[1] == 0 && n[2] == 0) n[2] = 1;
      normal_attr(&a, n[0], n[1], n[2]);
    }
    return a;
  }
};

static double lattice2(uint64_t seed, int oct, int64_t ix, int64_t iy) {
  uint64_t k = seed * 0x9E3779B97F4A7C15ull + (uint64_t)oct * 0xC2B2AE3D27D4EB4Full +
               (uint64_t)ix * 0x165667B19E3779F9ull + (uint64_t)iy * 0x27D4EB2F165667C5ull;
  return (double)(hash64(k) >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

static double value_noise2(uint64_t seed, int oct, double u, double v) {
  double fu = std::floor(u), fv = std::floor(v);
  int64_t iu = (int64_t)fu, iv = (int64_t)fv;
  double su = u - fu, sv = v - fv;
  su = su * su * (3.0 - 2.0 * su);
  sv = sv * sv * (3.0 - 2.0 * sv);
  double a = lattice2(seed, oct, iu, iv), b = lattice2(seed, oct, iu + 1, iv);
  double c = lattice2(seed, oct, iu, iv + 1), d = lattice2(seed, oct, iu + 1, iv + 1);
  double ab = a + (b - a) * su, cd = c + (d - c) * su;
  return ab + (cd - ab) * sv;
}

}  // namespace yv

using namespace yv;

// ---------------------------------------------------------------------------
// C ABI: host containers and generators
// ---------------------------------------------------------------------------
extern "C" {

yv_status yv_svo_gen_spheres(yv_svo_host** out, int depth, int n_spheres,
                             float rmin, float rmax, uint64_t seed) {
  if (!out || depth < 1 || depth > 12 || n_spheres < 0 || !(rmin >= 0) ||
      !(rmax >= rmin))
    return YV_ERR_INVALID_ARG;
  *out = nullptr;
  try {
    SphereSrc src;
    src.G = 1 << depth;
    SplitMix64 rng(seed);
    for (int i = 0; i < n_spheres; ++i) {
      double cx = rng.u01() * src.G, cy = rng.u01() * src.G, cz = rng.u01() * src.G;
      double r = (double)rmin + rng.u01() * ((double)rmax - (double)rmin);
      src.cx.push_back(cx);
      src.cy.push_back(cy);
      src.cz.push_back(cz);
      src.r2.push_back(r * r);
      uint64_t c = rng.next();
      src.rgb.push_back((uint8_t)(c & 255));
      src.rgb.push_back((uint8_t)((c >> 8) & 255));
      src.rgb.push_back((uint8_t)((c >> 16) & 255));
    }
    yv_svo_host* h = new yv_svo_host();
    build_tree(src, depth, h);
    *out = h;
    return YV_OK;
  } catch (const std::bad_alloc&) {
    return YV_ERR_OUT_OF_MEMORY;
  } catch (...) {
    return YV_ERR_INVALID_ARG;
  }
}

yv_status yv_svo_gen_terrain(yv_svo_host** out, int depth, int n_cubes,
                             int cube_min, int cube_max, uint64_t seed) {
  if (!out || depth < 2 || depth > 12 || n_cubes < 0 || cube_min < 1 ||
      cube_max < cube_min || cube_max > (1 << depth))
    return YV_ERR_INVALID_ARG;
  *out = nullptr;
  try {
    TerrainSrc src;
    src.depth = depth;
    src.G = 1 << depth;
    const int G = src.G;
    src.h.assign((size_t)G * (size_t)G, 0);
    // height = G*(0.5 + 0.3*n), n = normalised 6-octave value noise whose
    // base lattice spacing is G/8 voxels (256 voxels at 2048^3)
    int nth = hardware_threads();
    std::vector<std::thread> th;
    for (int t = 0; t < nth; ++t)
      th.emplace_back([&, t]() {
        for (int y = t; y < G; y += nth)
          for (int x = 0; x < G; ++x) {
            double sum = 0, wsum = 0, w = 1.0;
            for (int o = 0; o < 6; ++o) {
              double f = (double)(1 << o) * 8.0 / (double)G;
              sum += w * value_noise2(seed, o, (x + 0.5) * f, (y + 0.5) * f);
              wsum += w;
              w *= 0.5;
            }
            double hv = (double)G * (0.5 + 0.3 * (sum / wsum));
            int hi = (int)std::floor(hv);
            hi = std::max(0, std::min(G - 1, hi));
            src.h[(size_t)y * (size_t)G + (size_t)x] = (int16_t)hi;
          }
      });
    for (auto& t : th) t.join();
    // min/max pyramids
    src.hmin.resize((size_t)depth + 1);
    src.hmax.resize((size_t)depth + 1);
    src.hmin[0] = src.h;
    src.hmax[0] = src.h;
    for (int l = 1; l <= depth; ++l) {
      int n = G >> l, pn = G >> (l - 1);
      src.hmin[(size_t)l].resize((size_t)n * (size_t)n);
      src.hmax[(size_t)l].resize((size_t)n * (size_t)n);
      for (int y = 0; y < n; ++y)
        for (int x = 0; x < n; ++x) {
          int mn = 1 << 30, mx = -(1 << 30);
          for (int k = 0; k < 4; ++k) {
            size_t idx = (size_t)(2 * y + (k >> 1)) * (size_t)pn + (size_t)(2 * x + (k & 1));
            mn = std::min(mn, (int)src.hmin[(size_t)l - 1][idx]);
            mx = std::max(mx, (int)src.hmax[(size_t)l - 1][idx]);
          }
          src.hmin[(size_t)l][(size_t)y * (size_t)n + (size_t)x] = (int16_t)mn;
          src.hmax[(size_t)l][(size_t)y * (size_t)n + (size_t)x] = (int16_t)mx;
        }
    }
    SplitMix64 rng(seed ^ 0xC0BE5ull);
    for (int i = 0; i < n_cubes; ++i) {
      int side = cube_min + (int)(rng.next() % (uint64_t)(cube_max - cube_min + 1));
      int span = G - side + 1;
      src.c0x.push_back((int)(rng.next() % (uint64_t)span));
      src.c0y.push_back((int)(rng.next() % (uint64_t)span));
      src.c0z.push_back((int)(rng.next() % (uint64_t)span));
      src.cs.push_back(side);
      uint64_t c = rng.next();
      src.crgb.push_back((uint8_t)(c & 255));
      src.crgb.push_back((uint8_t)((c >> 8) & 255));
      src.crgb.push_back((uint8_t)((c >> 16) & 255));
    }
    yv_svo_host* h = new yv_svo_host();
    build_tree(src, depth, h);
    *out = h;
    return YV_OK;
  } catch (const std::bad_alloc&) {
    return YV_ERR_OUT_OF_MEMORY;
  } catch (...) {
    return YV_ERR_INVALID_ARG;
  }
}

yv_status yv_svo_from_arrays(yv_svo_host** out, const yv_vox_node* nodes,
                             uint32_t count, uint32_t root,
                             const yv_leaf_attr* attrs, uint32_t nattrs) {
  if (!out || (count && !nodes) || (nattrs && !attrs)) return YV_ERR_INVALID_ARG;
  *out = nullptr;
  try {
    yv_svo_host* h = new yv_svo_host();
    h->nodes.assign(nodes, nodes + count);
    h->attrs.assign(attrs, attrs + nattrs);
    h->root = root;
    DeviceLayout dl;
    std::string why;
    if (build_device_layout(nodes, count, root, nattrs, &dl, &why) == YV_OK)
      h->depth = dl.depth;
    *out = h;
    return YV_OK;
  } catch (const std::bad_alloc&) {
    return YV_ERR_OUT_OF_MEMORY;
  }
}

// Leaf VoxData of a file without an attribute section: RGB565 colour in the
// low half-word, octahedral int8x2 normal in the high half-word (the 16-bit
// colour + 16-bit normal split of reaction/report/main.tex:38,65).
static yv_leaf_attr decode_packed_voxdata(uint32_t v) {
  yv_leaf_attr a;
  std::memset(&a, 0, sizeof(a));
  uint32_t c = v & 0xFFFFu;
  a.r = (uint8_t)(((c >> 11) & 31) * 255 / 31);
  a.g = (uint8_t)(((c >> 5) & 63) * 255 / 63);
  a.b = (uint8_t)((c & 31) * 255 / 31);
  a.a = 255;
  double ox = (double)(int8_t)((v >> 16) & 0xFF) / 127.0;
  double oy = (double)(int8_t)((v >> 24) & 0xFF) / 127.0;
  double oz = 1.0 - std::fabs(ox) - std::fabs(oy);
  if (oz < 0) {
    double tx = (1.0 - std::fabs(oy)) * (ox >= 0 ? 1 : -1);
    double ty = (1.0 - std::fabs(ox)) * (oy >= 0 ? 1 : -1);
    ox = tx;
    oy = ty;
  }
  normal_attr(&a, ox, oy, oz);
  return a;
}

// The reference's packed VoxData of a host pool - in leaves and in every
// node's data (the subtree at a coarser level, reaction/report/main.tex:61)
// - decoded into attributes; leaves and node data then index them.
static void decode_packed_pool(yv_svo_host* h) {
  std::unordered_map<uint32_t, uint32_t> remap;
  auto attr_of = [&](uint32_t v) {
    auto it = remap.find(v);
    if (it != remap.end()) return it->second;
    const uint32_t idx = (uint32_t)h->attrs.size();
    remap.emplace(v, idx);
    h->attrs.push_back(decode_packed_voxdata(v));
    return idx;
  };
  for (auto& n : h->nodes)
    for (int ch = 0; ch < 8; ++ch)
      if ((n.flags >> ch) & 1u) n.child[ch] = attr_of(n.child[ch]);
  for (auto& n : h->nodes) n.data = attr_of(n.data);
  h->lod = !h->nodes.empty();
}

static void set_depth(yv_svo_host* h) {
  DeviceLayout dl;
  std::string why;
  if (build_device_layout(h->nodes.data(), (uint32_t)h->nodes.size(), h->root,
                          (uint32_t)h->attrs.size(), &dl, &why) == YV_OK)
    h->depth = dl.depth;
}

yv_status yv_svo_from_packed(yv_svo_host** out, const yv_vox_node* nodes, uint32_t count,
                             uint32_t root) {
  if (!out || (count && !nodes)) return YV_ERR_INVALID_ARG;
  *out = nullptr;
  yv_svo_host* h = nullptr;
  try {
    h = new yv_svo_host();
    h->root = root;
    h->nodes.assign(nodes, nodes + count);
    decode_packed_pool(h);
    set_depth(h);
    *out = h;
    return YV_OK;
  } catch (const std::bad_alloc&) {
    delete h;
    return YV_ERR_OUT_OF_MEMORY;
  }
}

yv_status yv_svo_load_vox(yv_svo_host** out, const char* path) {
  if (!out || !path) return YV_ERR_INVALID_ARG;
  *out = nullptr;
  FILE* f = std::fopen(path, "rb");
  if (!f) return YV_ERR_IO;
  uint32_t hdr[4];
  if (std::fread(hdr, 4, 4, f) != 4) {
    std::fclose(f);
    return YV_ERR_IO;
  }
  yv_svo_host* h = nullptr;
  try {
    h = new yv_svo_host();
    h->root = hdr[0];
    h->nodes.resize(hdr[3]);
    if (hdr[3] && std::fread(h->nodes.data(), sizeof(yv_vox_node), hdr[3], f) != hdr[3]) {
      delete h;
      std::fclose(f);
      return YV_ERR_IO;
    }
    char magic[4];
    uint32_t na = 0;
    bool has_attrs = std::fread(magic, 1, 4, f) == 4 && std::memcmp(magic, "YVAT", 4) == 0 &&
                     std::fread(&na, 4, 1, f) == 1;
    if (has_attrs) {
      h->attrs.resize(na);
      if (na && std::fread(h->attrs.data(), sizeof(yv_leaf_attr), na, f) != na) {
        delete h;
        std::fclose(f);
        return YV_ERR_IO;
      }
      char lod_magic[4];
      h->lod = std::fread(lod_magic, 1, 4, f) == 4 && std::memcmp(lod_magic, "YVLD", 4) == 0;
    } else {
      decode_packed_pool(h);
    }
    std::fclose(f);
    set_depth(h);
    *out = h;
    return YV_OK;
  } catch (const std::bad_alloc&) {
    delete h;
    std::fclose(f);
    return YV_ERR_OUT_OF_MEMORY;
  }
}

yv_status yv_svo_save_vox(const yv_svo_host* svo, const char* path) {
  if (!svo || !path) return YV_ERR_INVALID_ARG;
  FILE* f = std::fopen(path, "wb");
  if (!f) return YV_ERR_IO;
  uint32_t hdr[4] = {svo->root, 0, 0, (uint32_t)svo->nodes.size()};
  uint32_t na = (uint32_t)svo->attrs.size();
  bool ok = std::fwrite(hdr, 4, 4, f) == 4 &&
            std::fwrite(svo->nodes.data(), sizeof(yv_vox_node), svo->nodes.size(), f) ==
                svo->nodes.size() &&
            std::fwrite("YVAT", 1, 4, f) == 4 && std::fwrite(&na, 4, 1, f) == 1 &&
            std::fwrite(svo->attrs.data(), sizeof(yv_leaf_attr), na, f) == na;
  if (ok && svo->lod) ok = std::fwrite("YVLD", 1, 4, f) == 4;
  ok = (std::fclose(f) == 0) && ok;
  return ok ? YV_OK : YV_ERR_IO;
}

void yv_svo_free(yv_svo_host* svo) { delete svo; }
const char* yv_last_error(void) { return last_error_cstr(); }
uint32_t yv_svo_node_count(const yv_svo_host* s) { return s ? (uint32_t)s->nodes.size() : 0; }
uint32_t yv_svo_root(const yv_svo_host* s) { return s ? s->root : YV_EMPTY_NODE; }
const yv_vox_node* yv_svo_nodes(const yv_svo_host* s) { return s ? s->nodes.data() : nullptr; }
uint32_t yv_svo_attr_count(const yv_svo_host* s) { return s ? (uint32_t)s->attrs.size() : 0; }
const yv_leaf_attr* yv_svo_attrs(const yv_svo_host* s) { return s ? s->attrs.data() : nullptr; }
int yv_svo_depth(const yv_svo_host* s) { return s ? s->depth : 0; }
int yv_svo_has_lod(const yv_svo_host* s) { return s && s->lod ? 1 : 0; }

// Integer mean rounded half away from zero.
static int64_t mean_round(int64_t sum, int64_t n) {
  return sum >= 0 ? (2 * sum + n) / (2 * n) : -((-2 * sum + n) / (2 * n));
}

yv_status yv_svo_build_lod(yv_svo_host* s) {
  if (!s) return YV_ERR_INVALID_ARG;
  const size_t nn = s->nodes.size(), na = s->attrs.size();
  if (na + nn > 0x7FFFFFFFu) return YV_ERR_UNSUPPORTED;
  for (const auto& n : s->nodes)
    for (int ch = 0; ch < 8; ++ch) {
      const uint32_t c = n.child[ch];
      if ((n.flags >> ch) & 1u) {
        if (c >= na) return YV_ERR_BAD_POOL;
      } else if (!(c & 0x80000000u) && c >= nn) {
        return YV_ERR_BAD_POOL;
      }
    }
  // per node: sums of r, g, b, nx, ny, nz and the leaf count of its subtree,
  // post-order over an explicit stack (children before parents)
  struct Acc {
    int64_t v[6];
    int64_t n;
  };
  try {
    std::vector<Acc> acc(nn);
    std::vector<uint8_t> state(nn, 0);  // 0 new, 1 open, 2 done
    std::vector<uint32_t> stack;
    for (size_t start = 0; start < nn; ++start) {
      if (state[start]) continue;
      stack.push_back((uint32_t)start);
      while (!stack.empty()) {
        const uint32_t id = stack.back();
        const yv_vox_node& n = s->nodes[id];
        if (state[id] == 0) {
          state[id] = 1;
          for (int ch = 0; ch < 8; ++ch) {
            const uint32_t c = n.child[ch];
            if (((n.flags >> ch) & 1u) || (c & 0x80000000u)) continue;
            if (state[c] == 1) return YV_ERR_BAD_POOL;  // cycle
            if (state[c] == 0) stack.push_back(c);
          }
          continue;
        }
        stack.pop_back();
        if (state[id] == 2) continue;
        Acc a{};
        for (int ch = 0; ch < 8; ++ch) {
          const uint32_t c = n.child[ch];
          if ((n.flags >> ch) & 1u) {
            const yv_leaf_attr& l = s->attrs[c];
            a.v[0] += l.r;
            a.v[1] += l.g;
            a.v[2] += l.b;
            a.v[3] += l.nx;
            a.v[4] += l.ny;
            a.v[5] += l.nz;
            a.n += 1;
          } else if (!(c & 0x80000000u)) {
            for (int k = 0; k < 6; ++k) a.v[k] += acc[c].v[k];
            a.n += acc[c].n;
          }
        }
        acc[id] = a;
        state[id] = 2;
      }
    }
    s->attrs.reserve(na + nn);
    for (size_t id = 0; id < nn; ++id) {
      const Acc& a = acc[id];
      yv_leaf_attr l;
      std::memset(&l, 0, sizeof(l));
      if (a.n > 0) {
        l.r = (uint8_t)mean_round(a.v[0], a.n);
        l.g = (uint8_t)mean_round(a.v[1], a.n);
        l.b = (uint8_t)mean_round(a.v[2], a.n);
        l.a = 255;
        l.nx = (int8_t)mean_round(a.v[3], a.n);
        l.ny = (int8_t)mean_round(a.v[4], a.n);
        l.nz = (int8_t)mean_round(a.v[5], a.n);
      }
      s->attrs.push_back(l);
      s->nodes[id].data = (uint32_t)(na + id);
    }
    s->lod = true;
    return YV_OK;
  } catch (const std::bad_alloc&) {
    return YV_ERR_OUT_OF_MEMORY;
  }
}

yv_status yv_svo_validate(const yv_vox_node* nodes, uint32_t count,
                          uint32_t root, uint32_t nattrs) {
  DeviceLayout dl;
  std::string why;
  return build_device_layout(nodes, count, root, nattrs, &dl, &why);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Device re-layout + validation
// ---------------------------------------------------------------------------
namespace yv {

yv_status build_device_layout(const yv_vox_node* nodes, uint32_t count,
                              uint32_t root, uint32_t nattrs,
                              DeviceLayout* out, std::string* why) {
  out->words.clear();
  out->orig_id.clear();
  out->root_word = YV_DW_NULL;
  out->depth = 0;
  if (root & 0x80000000u) return YV_OK;  // null root: empty scene
  if (!nodes || root >= count) {
    *why = "root index outside the pool";
    return YV_ERR_BAD_POOL;
  }
  // iterative DFS: cycle check + height (levels of nodes)
  std::vector<uint8_t> color(count, 0);  // 0 new, 1 on stack, 2 done
  std::vector<uint8_t> height(count, 0);
  struct Frame { uint32_t id; int ch; };
  std::vector<Frame> st;
  st.push_back({root, 0});
  color[root] = 1;
  while (!st.empty()) {
    Frame& fr = st.back();
    const yv_vox_node& n = nodes[fr.id];
    if (fr.ch < 8) {
      int ch = fr.ch++;
      uint32_t w = n.child[ch];
      if ((n.flags >> ch) & 1u) {
        if (w >= nattrs || w > 0x7FFFFFFFu) {
          *why = "leaf VoxData outside the attribute array";
          return YV_ERR_BAD_POOL;
        }
        continue;
      }
      if (w & 0x80000000u) continue;
      if (w >= count) {
        *why = "child index outside the pool";
        return YV_ERR_BAD_POOL;
      }
      if (color[w] == 1) {
        *why = "cycle in the node graph";
        return YV_ERR_BAD_POOL;
      }
      if (color[w] == 0) {
        if (st.size() >= (size_t)YV_MAX_DEPTH) {
          *why = "tree deeper than 16 node levels";
          return YV_ERR_BAD_POOL;
        }
        color[w] = 1;
        st.push_back({w, 0});
      }
      continue;
    }
    int hgt = 1;
    for (int ch = 0; ch < 8; ++ch) {
      uint32_t w = n.child[ch];
      if (((n.flags >> ch) & 1u) || (w & 0x80000000u)) continue;
      hgt = std::max(hgt, 1 + (int)height[w]);
    }
    if (hgt > YV_MAX_DEPTH) {
      *why = "tree deeper than 16 node levels";
      return YV_ERR_BAD_POOL;
    }
    height[fr.id] = (uint8_t)hgt;
    color[fr.id] = 2;
    st.pop_back();
  }
  out->depth = height[root];
  // breadth-first numbering of the reachable nodes
  std::vector<uint32_t> newid(count, 0xFFFFFFFFu);
  std::vector<uint32_t> order;
  order.push_back(root);
  newid[root] = 0;
  for (size_t i = 0; i < order.size(); ++i) {
    const yv_vox_node& n = nodes[order[i]];
    for (int ch = 0; ch < 8; ++ch) {
      uint32_t w = n.child[ch];
      if (((n.flags >> ch) & 1u) || (w & 0x80000000u)) continue;
      if (newid[w] == 0xFFFFFFFFu) {
        newid[w] = (uint32_t)order.size();
        order.push_back(w);
      }
    }
  }
  if (order.size() > YV_MAX_DEVICE_NODES) {
    *why = "pool larger than 2^29 nodes";
    return YV_ERR_BAD_POOL;
  }
  out->words.resize(order.size() * 8);
  out->orig_id = order;
  for (size_t i = 0; i < order.size(); ++i) {
    const yv_vox_node& n = nodes[order[i]];
    for (int ch = 0; ch < 8; ++ch) {
      uint32_t w = n.child[ch], dw;
      if ((n.flags >> ch) & 1u)
        dw = YV_DW_LEAF | w;
      else if (w & 0x80000000u)
        dw = YV_DW_NULL;
      else
        dw = newid[w];
      out->words[i * 8 + (size_t)ch] = dw;
    }
  }
  out->root_word = 0;
  return YV_OK;
}

}  // namespace yv
