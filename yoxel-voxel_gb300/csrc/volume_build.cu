// volume_build.cu - GPU build of the ntree brick volume from a dense lattice:
// RangeBuilder (ntree/ntree/ntree.h:11-63) over an (S+1)^3 lattice, the
// producer side of the brick path (the GPU brick-pool construction of
// reaction/voxtree/density.cu:30-284 and BrickPool::Update,
// reaction/voxtree/brickpool/BrickPool.cpp:21-62: mark, scan, pack).
//
// Same result as the host builder yv_volume_from_dense, bit for bit: brick
// cells whose 9^3 lattice (with the far-side apron) holds a nonzero density
// are occupied; an N = 4 grid tree over them, grid nodes and bricks numbered
// in breadth-first order (children c = x | y<<2 | z<<4), the root always a
// grid node; bricks copy their 9^3 lattice values and RGB (white without an
// rgb lattice); neighbour tables for the apron fold.
//
// Passes: a cell is marked from per-row cell bits (one warp per lattice row,
// coalesced loads and ballots) ORed over its 9 x 9 rows;
// one pass per level ORs 64 child flags; top-down, an exclusive scan of the
// per-node counts of occupied children expands level l's breadth-first list
// into level l+1's and gives every node its first child id (bricks are the
// last level's children); emit passes write the grid refs, pack the bricks
// (optionally straight into a device pool format) and fill the neighbours.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "dev_scan.cuh"
#include "yv_internal.h"
#include "yv_kernels.h"

namespace yv {
namespace {

constexpr int kVB = 8;  // brick cells per axis
constexpr int kVL = 9;  // lattice points per axis with the apron
constexpr int kVL3 = 729;

struct Lattice {
  const float* d;
  const uint8_t* rgb;
  uint64_t L;  // lattice points per axis (S + 1)
  int nb;      // brick cells per axis
};

__device__ __forceinline__ uint64_t lat(const Lattice& g, int x, int y, int z) {
  return ((uint64_t)z * g.L + (uint64_t)y) * g.L + (uint64_t)x;
}

// Cell and level sizes are powers of two: index splits use shifts.

// Mark, pass 1: per lattice row (y, z), one bit per brick cell cx: some
// point of x in [8 cx, 8 cx + 8] (the cell's 8 points and its far apron
// point) is nonzero.  One warp per row reads it in coalesced 32-point chunks
// (eight loads in flight); the ballot of chunk j holds the points of cells
// 4j..4j+3, and a cell's apron point is the first point of the next cell.
// R[(z L + y) NW + w], NW = max(1, nb / 32) words per row.
__global__ void mark_rows_kernel(Lattice g, uint32_t* R) {
  constexpr int kU = 8;
  const uint32_t lane = threadIdx.x & 31u;
  const uint64_t rows = g.L * g.L;
  const uint32_t NW = g.nb >= 32 ? (uint32_t)g.nb / 32u : 1u;
  const uint32_t chunks = (uint32_t)((g.L + 31) / 32);  // 4 nb / 32 + 1
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t row = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; row < rows;
       row += nwarps) {
    const float* p = g.d + row * g.L;
    uint32_t word = 0, prev = 0;  // cell bits being assembled, previous chunk's ballot
    for (uint32_t j0 = 0; j0 < chunks; j0 += kU) {
      float v[kU];
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const uint64_t x = (uint64_t)(j0 + u) * 32u + lane;
        v[u] = (j0 + u < chunks && x < g.L) ? __ldg(p + x) : 0.f;
      }
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const uint32_t j = j0 + (uint32_t)u;
        if (j >= chunks) break;
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, v[u] != 0.f);
        if (j > 0) {
          // cells 4(j-1)..4(j-1)+3: own bytes of the previous chunk, apron =
          // the first bit of the following byte (bit 0 of this chunk for
          // the last one).  Bit 8k of `own` = byte k nonzero; the four
          // bits 0, 8, 16, 24 are gathered into bits 24..27 by one multiply
          // (no carries: the partial products below bit 24 are distinct).
          uint32_t own = prev | (prev >> 4);
          own |= own >> 2;
          own |= own >> 1;
          const uint32_t ap = (prev >> 8) | ((m & 1u) << 24);
          const uint32_t c4 = (((own | ap) & 0x01010101u) * 0x01020408u) >> 24;
          const uint32_t cbase = 4u * (j - 1);  // first cell of the group
          if (cbase < (uint32_t)g.nb) {
            word |= c4 << (cbase & 31u);
            if ((cbase & 31u) == 28u || cbase + 4u >= (uint32_t)g.nb) {
              if (lane == 0) R[row * NW + (cbase >> 5)] = word;
              word = 0;
            }
          }
        }
        prev = m;
      }
    }
  }
}

// Mark, pass 1, flat form (lattice 16-byte aligned, 16 <= nb <= 256, so a
// warp's 128 points touch at most two rows): the rows
// in groups of 4 (4 L floats start on a 16-byte boundary, L = 8 nb + 1 being
// odd only shifts the rows inside a group), read as float4 by one warp per
// group, 128 points per warp load.  A lane marks the cells of its 4 points
// (own cell x >> 3, apron cell x / 8 - 1 for x a non-zero multiple of 8) in
// a 32-bit window of cells of the warp's row; one warp OR reduction per row
// the load touches (at most 2), and lane 0 merges it into the group's row
// words in shared memory.  Same R as mark_rows_kernel.
constexpr uint32_t kFlatMaxNW = 8;

__global__ void mark_rows_flat_kernel(Lattice g, uint32_t* R) {
  __shared__ uint32_t acc_all[8][4][kFlatMaxNW];
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t(*acc)[kFlatMaxNW] = acc_all[(threadIdx.x >> 5) & 7u];
  const uint32_t L = (uint32_t)g.L;
  const uint32_t nb = (uint32_t)g.nb;
  const uint32_t NW = nb >= 32 ? nb / 32u : 1u;
  const uint64_t rows = g.L * g.L;
  const uint64_t groups = (rows + 3) / 4;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const float4* d4 = reinterpret_cast<const float4*>(g.d);
  for (uint64_t grp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; grp < groups;
       grp += nwarps) {
    const uint64_t left_rows = rows - grp * 4;
    const uint32_t nrows = left_rows < 4 ? (uint32_t)left_rows : 4u;
    const uint32_t nfl = nrows * L;             // floats of the group
    const uint32_t n4 = (nfl + 3) / 4;          // float4 loads (the last may run past)
    if (lane < 4 * kFlatMaxNW) acc[lane >> 3][lane & 7u] = 0u;
    __syncwarp();
    const float4* src = d4 + grp * (uint64_t)L;  // 4 L floats = L float4
    // row and x of the warp's first point, advanced by 128 points a step
    // (L > 128: at most one row boundary per step)
    uint32_t ra = 0, xs = 0;
    for (uint32_t f0 = 0; f0 < n4; f0 += 32u) {
      const uint32_t f = f0 + lane;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (4u * f + 3u < nfl) {
        v = __ldg(src + f);
      } else if (f < n4) {
        // the group's (and the lattice's) last points: no read past them
        const float* s1 = reinterpret_cast<const float*>(src) + 4u * f;
        const uint32_t left = nfl - 4u * f;
        v.x = __ldg(s1);
        if (left > 1u) v.y = __ldg(s1 + 1);
        if (left > 2u) v.z = __ldg(s1 + 2);
      }
      // the warp's 128 points: rows ra (first point) .. ra + 1
      const int c_lo = (int)(xs >> 3) - 1;  // window: cells c_lo .. c_lo + 31
      const uint32_t rb = ra + 1;           // cells -1..30 of the next row
      const uint32_t xl = xs + 4u * lane;   // x of the lane's first point in row ra
      uint32_t wa = 0, wb = 0;
      const float e[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const uint32_t i = 4u * f + (uint32_t)k;
        if (e[k] == 0.f || i >= nfl) continue;
        uint32_t x = xl + (uint32_t)k;
        const bool next_row = x >= L;
        if (next_row) x -= L;
        const uint32_t own = x >> 3;  // x = 8 nb: no own cell
        uint32_t bits = 0;
        if (own < nb) bits |= 2u;                  // cell own
        if ((x & 7u) == 0u && x > 0u) bits |= 1u;  // apron of cell own - 1
        if (!next_row) {
          wa |= bits << (own - (uint32_t)(c_lo + 1));
        } else {
          wb |= bits << own;  // window of row rb starts at cell -1
        }
      }
      wa = __reduce_or_sync(0xFFFFFFFFu, wa);
      wb = __reduce_or_sync(0xFFFFFFFFu, wb);
      if (lane == 0) {
        // window bit b = cell base + b: row ra base c_lo, row rb base -1
        if (wa) {
          int c0 = c_lo;
          uint64_t s = wa;
          if (c0 < 0) { s >>= 1; c0 = 0; }
          s <<= (c0 & 31);
          const uint32_t w = (uint32_t)c0 >> 5;
          if (w < NW) acc[ra][w] |= (uint32_t)s;
          if (w + 1 < NW) acc[ra][w + 1] |= (uint32_t)(s >> 32);
        }
        if (wb && rb < nrows) acc[rb][0] |= wb >> 1;
      }
      xs += 128u;
      if (xs >= L) {
        xs -= L;
        ++ra;
      }
    }
    __syncwarp();
    if (lane < nrows * NW) {
      const uint32_t r = lane / NW, w = lane % NW;
      R[(grp * 4 + r) * NW + w] = acc[r][w] & (nb >= 32 ? 0xFFFFFFFFu : ((1u << nb) - 1u));
    }
    __syncwarp();
  }
}

// Mark, pass 2: a cell is occupied when its bit is set in any of the 9 x 9
// rows y in [8 cy, 8 cy + 8], z in [8 cz, 8 cz + 8].  One thread per row word
// and (cy, cz); count = occupied cells, one atomic per warp.
__global__ void mark_cells_from_rows_kernel(Lattice g, const uint32_t* R, uint8_t* occ,
                                            uint32_t* count) {
  const uint32_t NW = g.nb >= 32 ? (uint32_t)g.nb / 32u : 1u;
  const int nbs = __ffs(g.nb) - 1;
  const uint64_t total = (uint64_t)NW * g.nb * g.nb;
  uint32_t my = 0;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
       t += (uint64_t)gridDim.x * blockDim.x) {
    const int wsh = __ffs(NW) - 1;  // NW is a power of two
    const uint32_t w = (uint32_t)(t & (NW - 1u));
    const uint64_t yz = t >> wsh;
    const uint32_t cy = (uint32_t)(yz & (uint64_t)(g.nb - 1)), cz = (uint32_t)(yz >> nbs);
    uint32_t acc = 0;
    for (int dz = 0; dz < 9; ++dz)
      for (int dy = 0; dy < 9; ++dy)
        acc |= R[(((uint64_t)(8 * cz + dz)) * g.L + (8 * cy + dy)) * NW + w];
    const int nbits = g.nb >= 32 ? 32 : g.nb;
    for (int b = 0; b < nbits; ++b)
      occ[((uint64_t)cz << (2 * nbs)) + ((uint64_t)cy << nbs) + 32u * w + (uint32_t)b] =
          (uint8_t)((acc >> b) & 1u);
    my += (uint32_t)__popc(nbits == 32 ? acc : acc & ((1u << nbits) - 1u));
  }
  my = __reduce_add_sync(0xFFFFFFFFu, my);
  if ((threadIdx.x & 31u) == 0 && my) atomicAdd(count, my);
}

// Index of child c (x | y<<2 | z<<4) of node p of a level with n = 2^s
// nodes per axis, in the level below (4n per axis).
__device__ __forceinline__ uint64_t child64(uint64_t p, uint32_t n, int c) {
  const int s = __ffs(n) - 1;
  const uint64_t x = p & (n - 1u), y = (p >> s) & (n - 1u), z = p >> (2 * s);
  return (4 * x + (c & 3)) + ((4 * y + ((c >> 2) & 3)) << (s + 2)) +
         ((4 * z + (c >> 4)) << (2 * s + 4));
}

// Level l (n per axis) from level l+1 (4n per axis): OR of 64 children.
// count: occupied nodes of the level, one atomic per warp.
__global__ void fold64_kernel(const uint8_t* child, uint32_t n, uint8_t* out, uint32_t* count) {
  const uint64_t total = (uint64_t)n * n * n;
  uint32_t my = 0;
  for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < total;
       p += (uint64_t)gridDim.x * blockDim.x) {
    uint8_t a = 0;
    for (int c = 0; c < 64 && !a; ++c) a = child[child64(p, n, c)];
    out[p] = a;
    my += a;
  }
  my = __reduce_add_sync(0xFFFFFFFFu, my);
  if ((threadIdx.x & 31u) == 0 && my) atomicAdd(count, my);
}

__global__ void count64_kernel(const uint64_t* list, uint32_t m, const uint8_t* child_any,
                               uint32_t n, uint32_t* counts) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    uint32_t k = 0;
    for (int c = 0; c < 64; ++c) k += child_any[child64(list[i], n, c)] ? 1u : 0u;
    counts[i] = k;
  }
}

__global__ void expand64_kernel(const uint64_t* list, uint32_t m, const uint8_t* child_any,
                                uint32_t n, const uint32_t* offsets, uint64_t* next) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    uint32_t o = offsets[i];
    for (int c = 0; c < 64; ++c) {
      const uint64_t q = child64(list[i], n, c);
      if (child_any[q]) next[o++] = q;
    }
  }
}

// Grid refs of one level: occupied children are grid nodes (child_base +
// rank) or, at the last level, bricks (0x40000000 | rank).
__global__ void emit_grids_kernel(const uint64_t* list, uint32_t m, const uint8_t* child_any,
                                  uint32_t n, const uint32_t* offsets, uint32_t node_base,
                                  uint32_t child_base, bool bricks, uint32_t* grids) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    uint32_t next = offsets[i];
    uint32_t* g = grids + (size_t)(node_base + i) * 64;
    for (int c = 0; c < 64; ++c) {
      uint32_t ref = 0x80000000u;
      if (child_any[child64(list[i], n, c)]) {
        ref = bricks ? (0x40000000u | next) : (child_base + next);
        ++next;
      }
      g[c] = ref;
    }
  }
}

__device__ __forceinline__ uint16_t f16_saturating(float f) {
  if (f != f) return 0;  // NaN -> 0, as the host upload
  uint16_t u = __half_as_ushort(__float2half_rn(f));
  if ((u & 0x7FFFu) == 0x7C00u) u = (uint16_t)((u & 0x8000u) | 0x7BFFu);
  return u;
}

// Pack: one warp per brick, its 729 lattice values (and RGB).  format < 0:
// fp32 density + uint8 RGB (host container layout); else a device pool
// format (YV_PRECISION_*), written to d_out / a_out.
// mask (device pools, optional): the cell occupancy mask of the march (16
// words per brick, bit (y & 3) * 8 + x of word z * 2 + (y >> 2) set where
// trilinear cell (x, y, z) has a non-zero stored density corner), from a
// 729-bit non-zero map of the brick's lattice the warp gathers by ballots
// while it packs (blocks of 256 threads).
__device__ __forceinline__ uint32_t lattice_row9(const uint32_t* bits, int off) {
  const int w = off >> 5, sh = off & 31;
  uint32_t v = bits[w] >> sh;
  if (sh > 23) v |= bits[w + 1] << (32 - sh);
  return v & 0x1FFu;
}

// bits (device pools, optional, zeroed before): the brick bitmap, bit
// (ci & 31) of word ci >> 5 set for the cell ci = (cz nb + cy) nb + cx of
// every brick.
__global__ void pack_bricks_kernel(Lattice g, const uint64_t* cells, uint32_t nbricks, int format,
                                   float* dens, uint8_t* rgb, void* d_out, void* a_out,
                                   int32_t* cell_xyz, int32_t* map, uint32_t* mask,
                                   uint32_t* bits) {
  __shared__ uint32_t nzbits[8][24];
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t* nz = nzbits[(threadIdx.x >> 5) & 7u];
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nbs = __ffs(g.nb) - 1;
  const bool half = format == YV_PRECISION_F16 || format == YV_PRECISION_F16_PACKED;
  for (uint32_t b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < nbricks; b += nwarps) {
    const uint64_t c = cells[b];
    const int cx = (int)(c & (uint64_t)(g.nb - 1)), cy = (int)((c >> nbs) & (uint64_t)(g.nb - 1)),
              cz = (int)(c >> (2 * nbs));
    if (lane == 0) {
      cell_xyz[3 * (size_t)b] = cx;
      cell_xyz[3 * (size_t)b + 1] = cy;
      cell_xyz[3 * (size_t)b + 2] = cz;
      map[c] = (int32_t)b;
      if (bits) {
        const uint64_t ci = ((uint64_t)cz * (uint64_t)g.nb + (uint64_t)cy) * (uint64_t)g.nb +
                            (uint64_t)cx;
        atomicOr(bits + (ci >> 5), 1u << (uint32_t)(ci & 31u));
      }
    }
    // lattice point k = lane + 32 q; the loads of 8 points are issued before
    // any is used
    for (int q0 = 0; q0 < (kVL3 + 31) / 32; q0 += 8) {
      float pv[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int k = (int)lane + 32 * (q0 + u);
        pv[u] = k < kVL3 ? __ldg(g.d + lat(g, cx * kVB + k % kVL, cy * kVB + (k / kVL) % kVL,
                                            cz * kVB + k / (kVL * kVL)))
                         : 0.f;
      }
      if (mask) {
        // after all 8 loads are issued: the non-zero points as stored (the
        // fp16 formats round small values to 0), one ballot per 32
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const bool nzv = half ? (f16_saturating(pv[u]) & 0x7FFFu) != 0 : pv[u] != 0.f;
          const uint32_t bits = __ballot_sync(0xFFFFFFFFu, nzv);
          if (lane == 0 && q0 + u < 24) nz[q0 + u] = bits;
        }
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int k = (int)lane + 32 * (q0 + u);
        if (k >= kVL3) break;
        const uint64_t src = lat(g, cx * kVB + k % kVL, cy * kVB + (k / kVL) % kVL,
                                 cz * kVB + k / (kVL * kVL));
        const float v = pv[u];
        uint8_t r = 255, gg = 255, bb = 255;
        if (g.rgb) {
          r = g.rgb[3 * src];
          gg = g.rgb[3 * src + 1];
          bb = g.rgb[3 * src + 2];
        }
        const size_t o = (size_t)b * kVL3 + (size_t)k;
        if (format < 0) {
          dens[o] = v;
          rgb[3 * o] = r;
          rgb[3 * o + 1] = gg;
          rgb[3 * o + 2] = bb;
        } else if (format == YV_PRECISION_F16) {
          static_cast<uint16_t*>(d_out)[o] = f16_saturating(v);
          static_cast<uchar4*>(a_out)[o] = make_uchar4(r, gg, bb, 255);
        } else if (format == YV_PRECISION_F32) {
          static_cast<float*>(d_out)[o] = v;
          float* a = static_cast<float*>(a_out) + 3 * o;
          a[0] = __fmul_rn((float)r, 1.0f / 255.0f);
          a[1] = __fmul_rn((float)gg, 1.0f / 255.0f);
          a[2] = __fmul_rn((float)bb, 1.0f / 255.0f);
        } else if (format == YV_PRECISION_F32_PACKED) {
          static_cast<float4*>(a_out)[o] =
              make_float4(__fmul_rn((float)r, 1.0f / 255.0f), __fmul_rn((float)gg, 1.0f / 255.0f),
                          __fmul_rn((float)bb, 1.0f / 255.0f), v);
        } else {
          static_cast<uint2*>(a_out)[o] =
              make_uint2((uint32_t)f16_saturating(v) | ((uint32_t)r << 16) | ((uint32_t)gg << 24),
                         (uint32_t)bb);
        }
      }
    }
    if (mask) {
      if (lane == 0) nz[23] = 0u;  // beyond the 729 points
      __syncwarp();
      if (lane < 16u) {
        const int z = (int)(lane >> 1), y0 = (int)(lane & 1u) * 4;
        uint32_t word = 0;
        for (int yy = 0; yy < 4; ++yy) {
          uint32_t rows = 0;
          for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy) {
              const uint32_t r9 = lattice_row9(nz, (z + dz) * 81 + (y0 + yy + dy) * 9);
              rows |= r9 | (r9 >> 1);  // cell x holds point x or x + 1
            }
          word |= (rows & 0xFFu) << (8 * yy);
        }
        mask[(size_t)b * 16u + lane] = word;
      }
      __syncwarp();
    }
  }
}

// Apron neighbour tables (index m-1 for the offset m = dx | dy<<1 | dz<<2).
__global__ void neighbors_kernel(const int32_t* cell_xyz, const int32_t* map, uint32_t nbricks,
                                 int nb, int32_t* up, int32_t* dn) {
  for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < nbricks;
       b += gridDim.x * blockDim.x) {
    const int x = cell_xyz[3 * (size_t)b], y = cell_xyz[3 * (size_t)b + 1],
              z = cell_xyz[3 * (size_t)b + 2];
    for (int m = 1; m < 8; ++m) {
      const int dx = m & 1, dy = (m >> 1) & 1, dz = (m >> 2) & 1;
      const int ux = x + dx, uy = y + dy, uz = z + dz;
      up[7 * (size_t)b + m - 1] =
          (ux < nb && uy < nb && uz < nb) ? map[((size_t)uz * nb + uy) * nb + ux] : -1;
      const int lx = x - dx, ly = y - dy, lz = z - dz;
      dn[7 * (size_t)b + m - 1] =
          (lx >= 0 && ly >= 0 && lz >= 0) ? map[((size_t)lz * nb + ly) * nb + lx] : -1;
    }
  }
}

yv_status vbuild_fail(cudaError_t e, const char* what) {
  set_last_error(std::string("dense volume build: ") + what + ": " + cudaGetErrorString(e));
  cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? YV_ERR_OUT_OF_MEMORY : YV_ERR_CUDA;
}

// Tree of a dense lattice on the device: grid refs (ngrids x 64) and the
// breadth-first brick cells.  Buffers come from the scratch pool.
struct VolumeTree {
  DevBuf grids, cells;  // uint32 grids[ngrids*64], uint64 cells[nbricks]
  uint32_t ngrids = 0, nbricks = 0;
};

yv_status build_volume_tree(const Lattice& g, int levels, cudaStream_t s, VolumeTree& t) {
  cudaError_t e;
  std::vector<DevBuf> any((size_t)levels + 1);
  for (int l = 0; l <= levels; ++l) {
    const uint64_t n = 1ull << (2 * l);
    if ((e = any[(size_t)l].alloc(n * n * n, s)) != cudaSuccess) return vbuild_fail(e, "alloc");
  }
  // occupied nodes per level (counted by the mark and fold passes, read
  // back once): the breadth-first lists below need no host read per level
  DevBuf dc;
  if ((e = dc.alloc((size_t)(levels + 1) * 4, s)) != cudaSuccess ||
      (e = cudaMemsetAsync(dc.p, 0, (size_t)(levels + 1) * 4, s)) != cudaSuccess)
    return vbuild_fail(e, "alloc");
  {
    const uint64_t NW = g.nb >= 32 ? (uint64_t)g.nb / 32 : 1;
    DevBuf rows;
    if ((e = rows.alloc(g.L * g.L * NW * 4, s)) != cudaSuccess) return vbuild_fail(e, "alloc");
    if (g.nb >= 16 && NW <= kFlatMaxNW && (reinterpret_cast<uintptr_t>(g.d) & 15u) == 0)
      mark_rows_flat_kernel<<<grid_for((g.L * g.L + 3) / 4 * 32), 256, 0, s>>>(
          g, rows.as<uint32_t>());
    else
      mark_rows_kernel<<<grid_for(g.L * g.L * 32), 256, 0, s>>>(g, rows.as<uint32_t>());
    mark_cells_from_rows_kernel<<<grid_for(NW * g.nb * g.nb), 256, 0, s>>>(
        g, rows.as<uint32_t>(), any[(size_t)levels].as<uint8_t>(), dc.as<uint32_t>() + levels);
  }
  for (int l = levels - 1; l >= 0; --l) {
    const uint32_t n = 1u << (2 * l);
    fold64_kernel<<<grid_for((uint64_t)n * n * n), 256, 0, s>>>(
        any[(size_t)l + 1].as<uint8_t>(), n, any[(size_t)l].as<uint8_t>(),
        dc.as<uint32_t>() + l);
  }
  std::vector<uint32_t> occ((size_t)levels + 1, 0);
  if ((e = cudaGetLastError()) != cudaSuccess ||
      (e = cudaMemcpyAsync(occ.data(), dc.p, (size_t)(levels + 1) * 4, cudaMemcpyDeviceToHost,
                           s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return vbuild_fail(e, "mark");
  // breadth-first lists: level 0 = the root (always a grid node)
  std::vector<DevBuf> list((size_t)levels + 1), offs((size_t)levels);
  std::vector<uint32_t> m((size_t)levels + 1, 0), base((size_t)levels + 1, 0);
  if ((e = list[0].alloc(8, s)) != cudaSuccess ||
      (e = cudaMemsetAsync(list[0].p, 0, 8, s)) != cudaSuccess)
    return vbuild_fail(e, "alloc");
  m[0] = 1;
  for (int l = 0; l < levels; ++l) {
    const uint32_t n = 1u << (2 * l);
    DevBuf counts;
    if ((e = counts.alloc((size_t)m[(size_t)l] * 4, s)) != cudaSuccess ||
        (e = offs[(size_t)l].alloc((size_t)m[(size_t)l] * 4, s)) != cudaSuccess)
      return vbuild_fail(e, "alloc");
    if (m[(size_t)l])
      count64_kernel<<<grid_for(m[(size_t)l]), 256, 0, s>>>(
          list[(size_t)l].as<uint64_t>(), m[(size_t)l], any[(size_t)l + 1].as<uint8_t>(), n,
          counts.as<uint32_t>());
    if ((e = cudaGetLastError()) != cudaSuccess ||
        (e = exclusive_scan(counts.as<uint32_t>(), offs[(size_t)l].as<uint32_t>(),
                            m[(size_t)l], nullptr, s)) != cudaSuccess)
      return vbuild_fail(e, "scan");
    const uint32_t total = occ[(size_t)l + 1];  // the scanned total
    base[(size_t)l + 1] = base[(size_t)l] + m[(size_t)l];
    m[(size_t)l + 1] = total;
    if ((e = list[(size_t)l + 1].alloc((size_t)(total ? total : 1) * 8, s)) != cudaSuccess)
      return vbuild_fail(e, "alloc");
    if (m[(size_t)l])
      expand64_kernel<<<grid_for(m[(size_t)l]), 256, 0, s>>>(
          list[(size_t)l].as<uint64_t>(), m[(size_t)l], any[(size_t)l + 1].as<uint8_t>(), n,
          offs[(size_t)l].as<uint32_t>(), list[(size_t)l + 1].as<uint64_t>());
    if ((e = cudaGetLastError()) != cudaSuccess) return vbuild_fail(e, "expand");
  }
  // grid nodes: levels 0..levels-1; bricks: the last list
  t.ngrids = base[(size_t)levels];
  t.nbricks = m[(size_t)levels];
  if ((e = t.grids.alloc((size_t)t.ngrids * 256, s)) != cudaSuccess)
    return vbuild_fail(e, "alloc");
  for (int l = 0; l < levels; ++l) {
    if (!m[(size_t)l]) continue;
    const bool last = l == levels - 1;
    emit_grids_kernel<<<grid_for(m[(size_t)l]), 256, 0, s>>>(
        list[(size_t)l].as<uint64_t>(), m[(size_t)l], any[(size_t)l + 1].as<uint8_t>(),
        1u << (2 * l), offs[(size_t)l].as<uint32_t>(), base[(size_t)l],
        last ? 0u : base[(size_t)l + 1], last, t.grids.as<uint32_t>());
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return vbuild_fail(e, "grids");
  // hand over the brick list
  std::swap(t.cells.p, list[(size_t)levels].p);
  t.cells.s = s;
  return YV_OK;
}

bool lattice_args(const float* density, int levels, Lattice* g, const uint8_t* rgb) {
  if (!density || levels < 1 || levels > 4) return false;
  g->d = density;
  g->rgb = rgb;
  g->nb = 1 << (2 * levels);
  g->L = (uint64_t)g->nb * kVB + 1;
  return true;
}

}  // namespace
}  // namespace yv

using namespace yv;

extern "C" {

yv_status yv_volume_build_dense(const float* density, const uint8_t* rgb, int32_t levels,
                                void* stream, yv_volume_host** out) {
  if (!out) return YV_ERR_INVALID_ARG;
  *out = nullptr;
  Lattice g;
  if (!lattice_args(density, levels, &g, rgb)) return YV_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  VolumeTree t;
  yv_status st = build_volume_tree(g, levels, s, t);
  if (st != YV_OK) return st;
  const size_t n = (size_t)t.nbricks * kVL3;
  DevBuf dens, col, cxyz, map;
  const uint64_t cells = (uint64_t)g.nb * g.nb * g.nb;
  cudaError_t e;
  if ((e = dens.alloc(n * 4, s)) != cudaSuccess || (e = col.alloc(n * 3, s)) != cudaSuccess ||
      (e = cxyz.alloc((size_t)t.nbricks * 12, s)) != cudaSuccess ||
      (e = map.alloc(cells * 4, s)) != cudaSuccess)
    return vbuild_fail(e, "alloc");
  if (t.nbricks)
    pack_bricks_kernel<<<grid_for((uint64_t)t.nbricks * 32), 256, 0, s>>>(
        g, t.cells.as<uint64_t>(), t.nbricks, -1, dens.as<float>(), col.as<uint8_t>(), nullptr,
        nullptr, cxyz.as<int32_t>(), map.as<int32_t>(), nullptr, nullptr);
  if ((e = cudaGetLastError()) != cudaSuccess) return vbuild_fail(e, "pack");
  std::vector<uint32_t> grids((size_t)t.ngrids * 64);
  std::vector<float> hd(n);
  std::vector<uint8_t> hc(n * 3);
  std::vector<int32_t> hcell((size_t)t.nbricks * 3);
  if ((e = cudaMemcpyAsync(grids.data(), t.grids.p, grids.size() * 4, cudaMemcpyDeviceToHost,
                           s)) != cudaSuccess ||
      (n && (e = cudaMemcpyAsync(hd.data(), dens.p, n * 4, cudaMemcpyDeviceToHost, s)) !=
                cudaSuccess) ||
      (n && (e = cudaMemcpyAsync(hc.data(), col.p, n * 3, cudaMemcpyDeviceToHost, s)) !=
                cudaSuccess) ||
      (t.nbricks && (e = cudaMemcpyAsync(hcell.data(), cxyz.p, hcell.size() * 4,
                                         cudaMemcpyDeviceToHost, s)) != cudaSuccess) ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return vbuild_fail(e, "download");
  return volume_host_from_parts(levels, std::move(grids), std::move(hd), std::move(hc),
                                std::move(hcell), out);
}

}  // extern "C"

namespace yv {
namespace {

// Builds the device pool from a lattice into `into` (reusing its arrays
// where they are large enough) or into a new volume (*out).
yv_status upload_dense(const float* density, const uint8_t* rgb, int32_t levels,
                       int32_t precision, cudaStream_t s, yv_volume_gpu* into,
                       yv_volume_gpu** out) {
  Lattice g;
  if (!lattice_args(density, levels, &g, rgb) || precision < YV_PRECISION_F16 ||
      precision > YV_PRECISION_F16_PACKED)
    return YV_ERR_INVALID_ARG;
  VolumeTree t;
  yv_status st = build_volume_tree(g, levels, s, t);
  if (st != YV_OK) return st;
  const size_t n = (size_t)t.nbricks * kVL3;
  const uint64_t cells = (uint64_t)g.nb * g.nb * g.nb;
  size_t dbytes = 0, abytes = 0;
  switch (precision) {
    case YV_PRECISION_F16: dbytes = n * 2; abytes = n * 4; break;
    case YV_PRECISION_F32: dbytes = n * 4; abytes = n * 12; break;
    case YV_PRECISION_F32_PACKED: abytes = n * 16; break;
    default: abytes = n * 8; break;
  }
  // the device pool (owned by the yv_volume_gpu): grids, density, albedo,
  // neighbours up / down
  const size_t bytes[5] = {(size_t)t.ngrids * 256, dbytes, abytes, (size_t)t.nbricks * 28,
                           (size_t)t.nbricks * 28};
  void* fresh[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  void** mem = fresh;
  size_t* cap = nullptr;
  yv_volume_device* desc = nullptr;
  if (into) volume_gpu_arrays(into, &mem, &cap, &desc);
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 5 && e == cudaSuccess; ++i) {
    if (!bytes[i] || (cap && cap[i] >= bytes[i])) continue;
    if (cap) {
      // grow: the old array may still be read by queued work on `s`
      e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) break;
      cudaFree(mem[i]);
      mem[i] = nullptr;
      cap[i] = 0;
    }
    e = cudaMalloc(&mem[i], bytes[i]);
    if (e == cudaSuccess && cap) cap[i] = bytes[i];
  }
  // the acceleration arrays: the cell occupancy mask (written by the pack
  // kernel), then the brick bitmap
  uint32_t *mask = nullptr, *bits = nullptr;
  if (e == cudaSuccess && t.nbricks) {
    if (into) {
      const yv_status mst = volume_gpu_accel_buffer(into, t.nbricks, levels, s, &mask, &bits);
      if (mst != YV_OK) return mst;
    } else {
      e = cudaMalloc(&mask, volume_accel_bytes(t.nbricks, levels));
      if (e == cudaSuccess && levels <= 4) bits = mask + (size_t)t.nbricks * 16u;
    }
  }
  DevBuf cxyz, map;
  if (e == cudaSuccess) e = cxyz.alloc((size_t)t.nbricks * 12, s);
  if (e == cudaSuccess) e = map.alloc(cells * 4, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(map.p, 0xFF, cells * 4, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(mem[0], t.grids.p, bytes[0], cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess && bits)
    e = cudaMemsetAsync(bits, 0, (size_t)YV_BRICK_BITS_WORDS(levels) * 4u, s);
  if (e == cudaSuccess && t.nbricks) {
    pack_bricks_kernel<<<grid_for((uint64_t)t.nbricks * 32), 256, 0, s>>>(
        g, t.cells.as<uint64_t>(), t.nbricks, precision, nullptr, nullptr, mem[1], mem[2],
        cxyz.as<int32_t>(), map.as<int32_t>(), mask, bits);
    neighbors_kernel<<<grid_for(t.nbricks), 256, 0, s>>>(
        cxyz.as<int32_t>(), map.as<int32_t>(), t.nbricks, g.nb, static_cast<int32_t*>(mem[3]),
        static_cast<int32_t*>(mem[4]));
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    if (!into) {
      for (void* p : fresh) cudaFree(p);
      cudaFree(mask);
    }
    return vbuild_fail(e, "device pool");
  }
  yv_volume_device d;
  d.grids = static_cast<const uint32_t*>(mem[0]);
  d.ngrids = t.ngrids;
  d.levels = levels;
  d.density = mem[1];
  d.albedo = mem[2];
  d.nbricks = t.nbricks;
  d.precision = precision;
  d.nbr_up = static_cast<const int32_t*>(mem[3]);
  d.nbr_dn = static_cast<const int32_t*>(mem[4]);
  d.cell_mask = mask;
  d.brick_bits = bits;
  if (into) {
    *desc = d;
    return YV_OK;
  }
  // a new volume: its buffers are complete once the stream gets here
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) {
    for (void* p : fresh) cudaFree(p);
    cudaFree(mask);
    return vbuild_fail(e, "device pool");
  }
  return volume_gpu_from_device(fresh, bytes, d, out, mask);
}

}  // namespace
}  // namespace yv

extern "C" {

yv_status yv_volume_upload_dense(const float* density, const uint8_t* rgb, int32_t levels,
                                 int32_t precision, void* stream, yv_volume_gpu** out) {
  if (!out) return YV_ERR_INVALID_ARG;
  *out = nullptr;
  return upload_dense(density, rgb, levels, precision, static_cast<cudaStream_t>(stream),
                      nullptr, out);
}

yv_status yv_volume_rebuild_dense(yv_volume_gpu* vol, const float* density, const uint8_t* rgb,
                                  int32_t levels, void* stream) {
  if (!vol) return YV_ERR_INVALID_ARG;
  yv_volume_device d;
  yv_status st = yv_volume_gpu_desc(vol, &d);
  if (st != YV_OK) return st;
  return upload_dense(density, rgb, levels, d.precision, static_cast<cudaStream_t>(stream), vol,
                      nullptr);
}

}  // extern "C"
