// volume_host.cpp - host-side brick volumes in the ntree layout.
//
// Reference counterparts (znah/yoxel-voxel):
//   ntree::Node Grid/Brick/Const, shrink-to-const   ntree/ntree/nodes.h:13-100
//   RangeBuilder (dense range -> tree)              ntree/ntree/ntree.h:11-63
//   CalcSceneSize(depth) = N^(depth-1) * B          ntree/ntree/gpu_nodes.h:18-21
//   BrickPool<T> (pool of fixed-size bricks)        ntree/BrickManager.h:5-80
//   child offset (z*N + y)*N + x                    ntree/ntree/nodes.h:99
//
// Layout: grid nodes of N^3 = 64 child refs (N = 4).  A ref is
//   0x80000000            empty (a Const node of density 0)
//   0x40000000 | b        brick b of the pool (last grid level only)
//   g                     grid node g
// Bricks hold a 9^3 lattice (8^3 cells plus the far-side apron that repeats
// the first lattice layer of the +x/+y/+z neighbours), so trilinear sampling
// never leaves the brick.  The reference bricks are 4^3 with no apron
// (BrickBoundary = 0, gpu_nodes.h:15-17) sampled by hardware texture
// filtering; here filtering is done in software and needs the apron.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>

#include "yv_internal.h"

struct yv_volume_host {
  int levels = 0;
  int nb = 0;  // brick cells per axis
  int S = 0;   // lattice cells per axis
  std::vector<uint32_t> grids;
  std::vector<float> density;    // nbricks * 729
  std::vector<uint8_t> albedo;   // nbricks * 729 * 3
  std::vector<int32_t> cell;     // nbricks * 3
  std::vector<int32_t> nbr_up;   // nbricks * 7: owner of the apron (+x,+y,+xy,+z,...)
  std::vector<int32_t> nbr_dn;   // nbricks * 7: bricks whose apron repeats my low faces
};

namespace yv {
namespace {

constexpr int kB = 8;      // brick cells per axis
constexpr int kL = 9;      // lattice points per axis (with apron)
constexpr int kL3 = 729;

double lattice3(uint64_t seed, int oct, int64_t ix, int64_t iy, int64_t iz) {
  uint64_t k = seed * 0x9E3779B97F4A7C15ull + (uint64_t)oct * 0xC2B2AE3D27D4EB4Full +
               (uint64_t)ix * 0x165667B19E3779F9ull + (uint64_t)iy * 0x27D4EB2F165667C5ull +
               (uint64_t)iz * 0x94D049BB133111EBull;
  return (double)(hash64(k) >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

double smooth(double t) { return t * t * (3.0 - 2.0 * t); }

// Lattice values of one noise octave over the scene, tabulated once (the
// same lattice3 values the formula would hash on every lookup).
struct LatticeTable {
  int n = 0;  // entries per axis
  std::vector<double> v;
  void build(uint64_t seed, int oct, int n_) {
    n = n_;
    v.resize((size_t)n * n * n);
    for (int z = 0; z < n; ++z)
      for (int y = 0; y < n; ++y)
        for (int x = 0; x < n; ++x)
          v[((size_t)z * n + y) * n + x] = lattice3(seed, oct, x, y, z);
  }
  double at(int64_t x, int64_t y, int64_t z) const {
    return v[((size_t)z * (size_t)n + (size_t)y) * (size_t)n + (size_t)x];
  }
  // value_noise3 from the table (x, y, z >= 0 inside the table)
  double noise(double x, double y, double z) const {
    double fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
    int64_t ix = (int64_t)fx, iy = (int64_t)fy, iz = (int64_t)fz;
    double sx = smooth(x - fx), sy = smooth(y - fy), sz = smooth(z - fz);
    double x00 = at(ix, iy, iz) + (at(ix + 1, iy, iz) - at(ix, iy, iz)) * sx;
    double x01 = at(ix, iy + 1, iz) + (at(ix + 1, iy + 1, iz) - at(ix, iy + 1, iz)) * sx;
    double x10 = at(ix, iy, iz + 1) + (at(ix + 1, iy, iz + 1) - at(ix, iy, iz + 1)) * sx;
    double x11 = at(ix, iy + 1, iz + 1) + (at(ix + 1, iy + 1, iz + 1) - at(ix, iy + 1, iz + 1)) * sx;
    double y0 = x00 + (x01 - x00) * sy, y1 = x10 + (x11 - x10) * sy;
    return y0 + (y1 - y0) * sz;
  }
  double box_max(const double* lo, const double* hi) const {
    double m = -1e30;
    for (int64_t z = (int64_t)std::floor(lo[2]); z <= (int64_t)std::floor(hi[2]) + 1; ++z)
      for (int64_t y = (int64_t)std::floor(lo[1]); y <= (int64_t)std::floor(hi[1]) + 1; ++y)
        for (int64_t x = (int64_t)std::floor(lo[0]); x <= (int64_t)std::floor(hi[0]) + 1; ++x)
          m = std::max(m, at(x, y, z));
    return m;
  }
};

struct NoiseVolume {
  uint64_t seed;
  int S;
  double offset, amplitude;
  double wsum = 1.0 + 0.5 + 0.25 + 0.125;
  LatticeTable oct[4], col[3];
  void init() {
    for (int o = 0; o < 4; ++o) oct[o].build(seed, o, 8 * (1 << o) + 2);
    for (int c = 0; c < 3; ++c) col[c].build(seed ^ (0xA1BEull + (uint64_t)c * 977), 7 + c, 6);
  }
  // density at lattice point p (integer lattice coordinates)
  double density(int x, int y, int z) const {
    double f = 8.0 / S, sum = 0.0, w = 1.0;
    for (int o = 0; o < 4; ++o) {
      double s = f * (double)(1 << o);
      sum += w * oct[o].noise(x * s, y * s, z * s);
      w *= 0.5;
    }
    double d = amplitude * (sum / wsum) - offset;
    return d < 0 ? 0 : (d > 1 ? 1 : d);
  }
  bool maybe_nonzero(int cx, int cy, int cz) const {
    double f = 8.0 / S, ub = 0.0, w = 1.0;
    for (int o = 0; o < 4; ++o) {
      double s = f * (double)(1 << o);
      double lo[3] = {cx * kB * s, cy * kB * s, cz * kB * s};
      double hi[3] = {(cx * kB + kB) * s, (cy * kB + kB) * s, (cz * kB + kB) * s};
      ub += w * oct[o].box_max(lo, hi);
      w *= 0.5;
    }
    return amplitude * (ub / wsum) - offset > 0.0;
  }
  void albedo(int x, int y, int z, uint8_t* rgb) const {
    double s = 4.0 / S;
    for (int c = 0; c < 3; ++c) {
      double n = col[c].noise(x * s, y * s, z * s);
      double v = 140.0 + 110.0 * n;
      rgb[c] = (uint8_t)std::max(0.0, std::min(255.0, std::floor(v + 0.5)));
    }
  }
};

// Builds the N=4 tree over the occupied brick cells (ncell^3 grid, bricks
// numbered in breadth-first order of the tree) and fills cell / neighbour
// tables.  `occ` maps a cell to its provisional brick id (-1 = empty).
void build_tree(yv_volume_host* v, const std::vector<int32_t>& occ,
                std::vector<int32_t>* order_out) {
  const int nb = v->nb;
  const int levels = v->levels;
  struct Item { int level, x, y, z; uint32_t slot; };
  // any-occupied pyramid: level l has nb >> (2*(levels-l)) ... computed lazily
  std::vector<std::vector<uint8_t>> any((size_t)levels + 1);
  any[(size_t)levels].resize((size_t)nb * nb * nb);
  for (size_t i = 0; i < occ.size(); ++i) any[(size_t)levels][i] = occ[i] >= 0;
  for (int l = levels - 1; l >= 0; --l) {
    int n = 1 << (2 * l), pn = 1 << (2 * (l + 1));
    any[(size_t)l].assign((size_t)n * n * n, 0);
    for (int z = 0; z < pn; ++z)
      for (int y = 0; y < pn; ++y)
        for (int x = 0; x < pn; ++x)
          if (any[(size_t)l + 1][((size_t)z * pn + y) * pn + x])
            any[(size_t)l][((size_t)(z >> 2) * n + (y >> 2)) * n + (x >> 2)] = 1;
  }
  v->grids.clear();
  std::vector<int32_t> order;  // provisional brick ids in final order
  v->grids.resize(64, 0x80000000u);
  std::vector<Item> q;
  q.push_back({0, 0, 0, 0, 0});
  for (size_t qi = 0; qi < q.size(); ++qi) {
    Item it = q[qi];
    uint32_t g = it.slot;
    int cl = it.level + 1;  // level of the children
    int n = 1 << (2 * cl);
    for (int c = 0; c < 64; ++c) {
      int x = it.x * 4 + (c & 3), y = it.y * 4 + ((c >> 2) & 3), z = it.z * 4 + (c >> 4);
      uint32_t ref = 0x80000000u;
      if (any[(size_t)cl][((size_t)z * n + y) * n + x]) {
        if (cl == levels) {
          int32_t pid = occ[((size_t)z * nb + y) * nb + x];
          ref = 0x40000000u | (uint32_t)order.size();
          order.push_back(pid);
        } else {
          uint32_t child = (uint32_t)(v->grids.size() / 64);
          v->grids.resize(v->grids.size() + 64, 0x80000000u);
          ref = child;
          q.push_back({cl, x, y, z, child});
        }
      }
      v->grids[(size_t)g * 64 + (size_t)c] = ref;
    }
  }
  *order_out = order;
}

void fill_neighbors(yv_volume_host* v) {
  const int nb = v->nb;
  const size_t n = v->cell.size() / 3;
  std::vector<int32_t> map((size_t)nb * nb * nb, -1);
  for (size_t b = 0; b < n; ++b)
    map[((size_t)v->cell[b * 3 + 2] * nb + v->cell[b * 3 + 1]) * nb + v->cell[b * 3]] = (int32_t)b;
  v->nbr_up.assign(n * 7, -1);
  v->nbr_dn.assign(n * 7, -1);
  for (size_t b = 0; b < n; ++b)
    for (int m = 1; m < 8; ++m) {
      int dx = m & 1, dy = (m >> 1) & 1, dz = (m >> 2) & 1;
      int x = v->cell[b * 3], y = v->cell[b * 3 + 1], z = v->cell[b * 3 + 2];
      int ux = x + dx, uy = y + dy, uz = z + dz;
      if (ux < nb && uy < nb && uz < nb)
        v->nbr_up[b * 7 + (size_t)(m - 1)] = map[((size_t)uz * nb + uy) * nb + ux];
      int lx = x - dx, ly = y - dy, lz = z - dz;
      if (lx >= 0 && ly >= 0 && lz >= 0)
        v->nbr_dn[b * 7 + (size_t)(m - 1)] = map[((size_t)lz * nb + ly) * nb + lx];
    }
}

}  // namespace

yv_status volume_host_from_parts(int levels, std::vector<uint32_t>&& grids,
                                 std::vector<float>&& density, std::vector<uint8_t>&& albedo,
                                 std::vector<int32_t>&& cells, yv_volume_host** out) {
  try {
    yv_volume_host* v = new yv_volume_host();
    v->levels = levels;
    v->nb = 1 << (2 * levels);
    v->S = v->nb * kB;
    v->grids = std::move(grids);
    v->density = std::move(density);
    v->albedo = std::move(albedo);
    v->cell = std::move(cells);
    fill_neighbors(v);
    *out = v;
    return YV_OK;
  } catch (const std::bad_alloc&) {
    return YV_ERR_OUT_OF_MEMORY;
  }
}

}  // namespace yv

using namespace yv;

extern "C" {

yv_status yv_volume_gen_noise(yv_volume_host** out, int levels, float offset,
                              float amplitude, uint64_t seed) {
  if (!out || levels < 1 || levels > 5 || !std::isfinite(offset) || !std::isfinite(amplitude))
    return YV_ERR_INVALID_ARG;
  *out = nullptr;
  try {
    yv_volume_host* v = new yv_volume_host();
    v->levels = levels;
    v->nb = 1 << (2 * levels);
    v->S = v->nb * kB;
    NoiseVolume nv{seed, v->S, (double)offset, (double)amplitude};
    nv.init();
    const int nb = v->nb;
    const size_t ncell = (size_t)nb * nb * nb;
    // candidate cells (bound test), then exact evaluation in parallel
    std::vector<int32_t> cand;
    for (int z = 0; z < nb; ++z)
      for (int y = 0; y < nb; ++y)
        for (int x = 0; x < nb; ++x)
          if (nv.maybe_nonzero(x, y, z)) cand.push_back((int32_t)(((size_t)z * nb + y) * nb + x));
    std::vector<float> cden(cand.size() * kL3);
    std::vector<uint8_t> calb(cand.size() * kL3 * 3);
    std::vector<uint8_t> keep(cand.size(), 0);
    std::atomic<size_t> next{0};
    std::vector<std::thread> th;
    int nth = hardware_threads();
    for (int t = 0; t < nth; ++t)
      th.emplace_back([&]() {
        for (;;) {
          size_t i = next.fetch_add(1);
          if (i >= cand.size()) break;
          int c = cand[i];
          int cx = c % nb, cy = (c / nb) % nb, cz = c / (nb * nb);
          bool nz = false;
          for (int z = 0; z < kL; ++z)
            for (int y = 0; y < kL; ++y)
              for (int x = 0; x < kL; ++x) {
                float d = (float)nv.density(cx * kB + x, cy * kB + y, cz * kB + z);
                cden[i * kL3 + (size_t)((z * kL + y) * kL + x)] = d;
                nz = nz || d > 0.f;
              }
          keep[i] = nz;
          if (nz)
            for (int k = 0; k < kL3; ++k)
              nv.albedo(cx * kB + k % kL, cy * kB + (k / kL) % kL, cz * kB + k / (kL * kL),
                        &calb[(i * kL3 + (size_t)k) * 3]);
        }
      });
    for (auto& t : th) t.join();
    std::vector<int32_t> occ(ncell, -1);
    std::vector<int32_t> prov;  // provisional id -> candidate index
    for (size_t i = 0; i < cand.size(); ++i)
      if (keep[i]) {
        occ[(size_t)cand[i]] = (int32_t)prov.size();
        prov.push_back((int32_t)i);
      }
    std::vector<int32_t> order;
    build_tree(v, occ, &order);
    const size_t n = order.size();
    v->density.resize(n * kL3);
    v->albedo.resize(n * kL3 * 3);
    v->cell.resize(n * 3);
    for (size_t b = 0; b < n; ++b) {
      size_t ci = (size_t)prov[(size_t)order[b]];
      int c = cand[ci];
      int cx = c % nb, cy = (c / nb) % nb, cz = c / (nb * nb);
      v->cell[b * 3] = cx;
      v->cell[b * 3 + 1] = cy;
      v->cell[b * 3 + 2] = cz;
      std::memcpy(&v->density[b * kL3], &cden[ci * kL3], kL3 * sizeof(float));
      std::memcpy(&v->albedo[b * kL3 * 3], &calb[ci * kL3 * 3], kL3 * 3);
    }
    fill_neighbors(v);
    *out = v;
    return YV_OK;
  } catch (const std::bad_alloc&) {
    return YV_ERR_OUT_OF_MEMORY;
  }
}

// RangeBuilder::build analogue: dense (S+1)^3 lattice -> tree + pool, bricks
// whose 9^3 lattice is all zero become empty refs (Node::Shrink).
yv_status yv_volume_from_dense(yv_volume_host** out, int levels, const float* density,
                               const uint8_t* albedo_rgb) {
  if (!out || !density || levels < 1 || levels > 4) return YV_ERR_INVALID_ARG;
  *out = nullptr;
  try {
    yv_volume_host* v = new yv_volume_host();
    v->levels = levels;
    v->nb = 1 << (2 * levels);
    v->S = v->nb * kB;
    const int nb = v->nb;
    const size_t L = (size_t)v->S + 1;
    auto at = [&](int x, int y, int z) { return ((size_t)z * L + (size_t)y) * L + (size_t)x; };
    std::vector<int32_t> occ((size_t)nb * nb * nb, -1);
    std::vector<int32_t> cells;
    for (int z = 0; z < nb; ++z)
      for (int y = 0; y < nb; ++y)
        for (int x = 0; x < nb; ++x) {
          bool nz = false;
          for (int k = 0; k < kL3 && !nz; ++k)
            nz = density[at(x * kB + k % kL, y * kB + (k / kL) % kL, z * kB + k / (kL * kL))] != 0.f;
          if (nz) {
            occ[((size_t)z * nb + y) * nb + x] = (int32_t)cells.size();
            cells.push_back((int32_t)(((size_t)z * nb + y) * nb + x));
          }
        }
    std::vector<int32_t> order;
    build_tree(v, occ, &order);
    const size_t n = order.size();
    v->density.resize(n * kL3);
    v->albedo.assign(n * kL3 * 3, 255);
    v->cell.resize(n * 3);
    for (size_t b = 0; b < n; ++b) {
      int c = cells[(size_t)order[b]];
      int cx = c % nb, cy = (c / nb) % nb, cz = c / (nb * nb);
      v->cell[b * 3] = cx;
      v->cell[b * 3 + 1] = cy;
      v->cell[b * 3 + 2] = cz;
      for (int k = 0; k < kL3; ++k) {
        size_t src = at(cx * kB + k % kL, cy * kB + (k / kL) % kL, cz * kB + k / (kL * kL));
        v->density[b * kL3 + (size_t)k] = density[src];
        if (albedo_rgb)
          for (int ch = 0; ch < 3; ++ch)
            v->albedo[(b * kL3 + (size_t)k) * 3 + (size_t)ch] = albedo_rgb[src * 3 + (size_t)ch];
      }
    }
    fill_neighbors(v);
    *out = v;
    return YV_OK;
  } catch (const std::bad_alloc&) {
    return YV_ERR_OUT_OF_MEMORY;
  }
}

void yv_volume_free(yv_volume_host* v) { delete v; }
int yv_volume_levels(const yv_volume_host* v) { return v ? v->levels : 0; }
uint32_t yv_volume_grid_count(const yv_volume_host* v) { return v ? (uint32_t)(v->grids.size() / 64) : 0; }
const uint32_t* yv_volume_grids(const yv_volume_host* v) { return v ? v->grids.data() : nullptr; }
uint32_t yv_volume_brick_count(const yv_volume_host* v) { return v ? (uint32_t)(v->cell.size() / 3) : 0; }
const float* yv_volume_density(const yv_volume_host* v) { return v ? v->density.data() : nullptr; }
const uint8_t* yv_volume_albedo(const yv_volume_host* v) { return v ? v->albedo.data() : nullptr; }
const int32_t* yv_volume_brick_cells(const yv_volume_host* v) { return v ? v->cell.data() : nullptr; }
const int32_t* yv_volume_neighbors(const yv_volume_host* v, int upper) {
  if (!v) return nullptr;
  return upper ? v->nbr_up.data() : v->nbr_dn.data();
}

}  // extern "C"
