// svo_build.cu - GPU build of the canonical sparse voxel octree from a
// dense density grid: the iso/raw-source form of DynamicSVO::BuildRange
// (the GROW pass driven by a voxel source, ore/src/main.cpp:37-129,
// demo/Demo.cpp:82-114; the DynamicSVO source is not in the reference
// snapshot), with the surface-voxel rule of scene_gen.py:32-66 and the
// VoxNode layout of reaction/report/main.tex:36-56.
//
// Rules (identical to the host generators' canonical form):
//   voxel v of the 2^depth grid is solid iff density[v] > iso; a solid voxel
//   with a 6-neighbour outside the grid or not solid is a surface voxel (a
//   leaf); a cube region without surface voxels is EmptyNode (no solid
//   voxel) or FullNode; nodes are numbered breadth-first from the root
//   (id 0), children in child order c = x | y<<1 | z<<2, leaves in the same
//   order.  Leaf: RGB of the voxel (white without an rgb grid), A = 255,
//   normal = quantised normalize of the central difference (d(x-1) -
//   d(x+1), ...) with coordinates clamped to the grid, every step an FP32
//   round-to-nearest operation (zero for a zero or non-finite length).
//
// GB300 design, level-synchronous with no recursion and no host loop over
// regions:
//   1. one warp per 32-voxel row run packs the solid bits (ballot); one
//      thread per word and 2x2 row pair finds the surface voxels by bit
//      shifts and classifies the 16 bottom regions (2^3 voxels) it covers
//      (voxel codes empty / full / leaf, 2 bits each);
//   2. one pass per level folds 8 child classes into the parent class
//      (EMPTY if all 8 EMPTY, FULL if all 8 FULL, else a node);
//   3. top-down, the breadth-first node list of level k+1 is the
//      stable expansion of level k's list (an exclusive scan of the per-node
//      counts of node children gives every node its first child id), and the
//      same scan over leaf children numbers the attributes;
//   4. one pass per level writes the VoxNodes, one pass the leaf attributes.
// Depth <= 11 (a 2048^3 grid: 8.6 G voxels, 34 GB of float density).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "dev_scan.cuh"
#include "yv_internal.h"
#include "yv_kernels.h"

namespace yv {
namespace {

enum : uint8_t { kClsEmpty = 0, kClsFull = 1, kClsNode = 2 };
// voxel child codes of a bottom region (2 bits each)
enum : uint32_t { kVoxEmpty = 0, kVoxFull = 1, kVoxLeaf = 2 };

struct Grid {
  const float* d;
  const uint8_t* rgb;
  int G;
  float iso;
};

__device__ __forceinline__ size_t vidx(int G, int x, int y, int z) {
  return (size_t)x + (size_t)G * ((size_t)y + (size_t)G * (size_t)z);
}

__device__ __forceinline__ float dens_clamped(const Grid& g, int x, int y, int z) {
  x = x < 0 ? 0 : (x >= g.G ? g.G - 1 : x);
  y = y < 0 ? 0 : (y >= g.G ? g.G - 1 : y);
  z = z < 0 ? 0 : (z >= g.G ? g.G - 1 : z);
  return __ldg(g.d + vidx(g.G, x, y, z));
}

// Pass 1a: solid bits, one 32-voxel run of a row per warp and word (lane i
// tests x = 32 w + i, a ballot packs the run): S[(z G + y) WR + w],
// WR = max(1, G / 32) words per row (a power of two, as is G); bits beyond
// the grid are 0.  Eight words per iteration keep eight coalesced 128-byte
// loads in flight; word indices fit 32 bits (G^2 WR <= 2^28) and are split
// with shifts.
__global__ void solid_bits_kernel(Grid g, uint32_t WR, uint32_t* S) {
  constexpr int kU = 8;
  const uint32_t lane = threadIdx.x & 31u;
  const int wsh = __ffs(WR) - 1;
  const uint32_t total = (uint32_t)g.G * (uint32_t)g.G * WR;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t w0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w0 < total;
       w0 += kU * nwarps) {
    bool sol[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const uint32_t wi = w0 + (uint32_t)u * nwarps;
      const uint32_t x = ((wi & (WR - 1u)) << 5) + lane;
      sol[u] = wi < total && x < (uint32_t)g.G &&
               __ldg(g.d + (uint64_t)(wi >> wsh) * (uint64_t)g.G + x) > g.iso;
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const uint32_t wi = w0 + (uint32_t)u * nwarps;
      const uint32_t m = __ballot_sync(0xFFFFFFFFu, sol[u]);
      if (lane == 0 && wi < total) S[wi] = m;
    }
  }
}

// Pass 1a for rows of 128 voxels or more (G >= 128): one 128-voxel chunk
// per warp and iteration, each lane a 16-byte load of 4 voxels; the lanes'
// 4-bit groups are ORed into 32-bit words within groups of 8 lanes (3
// shuffles), lane 8j writing word j of the chunk.  Same bits as above.
__global__ void solid_bits_v4_kernel(Grid g, uint32_t WR, uint32_t* S) {
  constexpr int kU = 4;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t CR = WR >> 2;  // chunks per row
  const int csh = __ffs(CR) - 1;
  const uint32_t total = (uint32_t)g.G * CR * (uint32_t)g.G;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const float4* d4 = reinterpret_cast<const float4*>(g.d);
  for (uint32_t c0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c0 < total;
       c0 += kU * nwarps) {
    float4 v[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const uint32_t c = c0 + (uint32_t)u * nwarps;
      v[u] = c < total ? __ldg(d4 + (((uint64_t)(c >> csh) * g.G + ((c & (CR - 1u)) << 7)) >> 2) +
                               lane)
                       : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const uint32_t c = c0 + (uint32_t)u * nwarps;
      const uint32_t nib = (uint32_t)(v[u].x > g.iso) | ((uint32_t)(v[u].y > g.iso) << 1) |
                           ((uint32_t)(v[u].z > g.iso) << 2) | ((uint32_t)(v[u].w > g.iso) << 3);
      uint32_t word = nib << (4 * (lane & 7u));
      word |= __shfl_xor_sync(0xFFFFFFFFu, word, 1);
      word |= __shfl_xor_sync(0xFFFFFFFFu, word, 2);
      word |= __shfl_xor_sync(0xFFFFFFFFu, word, 4);
      if ((lane & 7u) == 0u && c < total)
        S[((uint64_t)(c >> csh) * WR) + ((c & (CR - 1u)) << 2) + (lane >> 3)] = word;
    }
  }
}

// Pass 1b: bottom regions (2^3 voxels) from the bits.  One thread per word
// and pair of rows in y and in z: a voxel is a surface voxel when it is
// solid and one of its 6 neighbours is not (bit shifts across the word and
// its x neighbours, the words of the adjacent rows; outside the grid = not
// solid).  Writes the class and the 2-bit voxel codes of the (up to) 16
// regions the word covers, as one 16-byte and two 16-byte vector stores when
// the word covers 16 regions.  Indices are split with shifts (WR and n are
// powers of two).
// node_count / leaf_count (either may be null): node regions and leaf
// (surface) voxels, added with one atomic per warp.
__global__ void classify_bits_kernel(const uint32_t* S, int G, uint32_t WR, uint32_t n,
                                     uint8_t* cls, uint16_t* codes, uint32_t* node_count,
                                     uint32_t* leaf_count) {
  uint32_t my_nodes = 0, my_leaves = 0;
  const uint64_t total = (uint64_t)WR * n * n;
  const int nreg = n < 16u ? (int)n : 16;
  const int wsh = __ffs(WR) - 1, nsh = __ffs(n) - 1;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
       t += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t w = (uint32_t)(t & (WR - 1u));
    const uint32_t ry = (uint32_t)((t >> wsh) & (n - 1u)), rz = (uint32_t)(t >> (wsh + nsh));
    uint32_t sol[2][2], surf[2][2];
#pragma unroll
    for (int dz = 0; dz < 2; ++dz)
#pragma unroll
      for (int dy = 0; dy < 2; ++dy) {
        const int y = 2 * (int)ry + dy, z = 2 * (int)rz + dz;
        const uint64_t row = ((uint64_t)z * G + y) * WR;
        const uint32_t W = S[row + w];
        const uint32_t wl = (W << 1) | (w > 0 ? S[row + w - 1] >> 31 : 0u);
        const uint32_t wr = (W >> 1) | (w + 1 < WR ? (S[row + w + 1] & 1u) << 31 : 0u);
        const uint32_t ym = y > 0 ? S[row - WR + w] : 0u;
        const uint32_t yp = y + 1 < G ? S[row + WR + w] : 0u;
        const uint32_t zm = z > 0 ? S[row - (uint64_t)G * WR + w] : 0u;
        const uint32_t zp = z + 1 < G ? S[row + (uint64_t)G * WR + w] : 0u;
        sol[dz][dy] = W;
        surf[dz][dy] = W & ~(wl & wr & ym & yp & zm & zp);
      }
    const uint64_t rbase = (uint64_t)16 * w + ((uint64_t)(ry + ((uint64_t)rz << nsh)) << nsh);
    // Region k holds bits 2k, 2k+1 of the four rows.  Bit-parallel over the
    // 16 regions: bit 2k of `any` = some voxel solid, of `all_full` = all 8
    // solid and not surface; only the other (node) regions need per-voxel
    // codes (empty regions code 0, full ones 0x5555).
    const uint32_t so_or = sol[0][0] | sol[0][1] | sol[1][0] | sol[1][1];
    const uint32_t fu_and = (sol[0][0] & ~surf[0][0]) & (sol[0][1] & ~surf[0][1]) &
                            (sol[1][0] & ~surf[1][0]) & (sol[1][1] & ~surf[1][1]);
    const uint32_t any = (so_or | (so_or >> 1)) & 0x55555555u;
    const uint32_t all_full = fu_and & (fu_and >> 1) & 0x55555555u;
    uint32_t cw[4] = {0u, 0u, 0u, 0u}, kw[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const uint32_t b = 1u << (2 * k);
      const uint32_t cl = !(any & b) ? kClsEmpty : ((all_full & b) ? kClsFull : kClsNode);
      cw[k >> 2] |= cl << (8 * (k & 3));
      if (cl == kClsFull) kw[k >> 1] |= 0x5555u << (16 * (k & 1));
    }
    if (nreg == 16) {
      // rbase is a multiple of 16: 16-byte aligned classes, 32-byte aligned codes
      reinterpret_cast<uint4*>(cls + rbase)[0] = make_uint4(cw[0], cw[1], cw[2], cw[3]);
      uint4* cp = reinterpret_cast<uint4*>(codes + rbase);
      cp[0] = make_uint4(kw[0], kw[1], kw[2], kw[3]);
      cp[1] = make_uint4(kw[4], kw[5], kw[6], kw[7]);
    } else {
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        if (k >= nreg) break;
        cls[rbase + k] = (uint8_t)(cw[k >> 2] >> (8 * (k & 3)));
        codes[rbase + k] = (uint16_t)(kw[k >> 1] >> (16 * (k & 1)));
      }
    }
    // per-voxel codes of the node regions (few), over the zeros just stored
    uint32_t nodes_mask = any & ~all_full;
    my_nodes += __popc(nodes_mask);
    my_leaves += __popc(surf[0][0]) + __popc(surf[0][1]) + __popc(surf[1][0]) +
                 __popc(surf[1][1]);
    while (nodes_mask) {
      const int k = (__ffs(nodes_mask) - 1) >> 1;
      nodes_mask &= nodes_mask - 1u;
      uint32_t code = 0;
#pragma unroll
      for (int ch = 0; ch < 8; ++ch) {
        const int bit = 2 * k + (ch & 1);
        const uint32_t so = (sol[ch >> 2][(ch >> 1) & 1] >> bit) & 1u;
        const uint32_t su = (surf[ch >> 2][(ch >> 1) & 1] >> bit) & 1u;
        const uint32_t c = !so ? kVoxEmpty : (su ? kVoxLeaf : kVoxFull);
        code |= c << (2 * ch);
      }
      codes[rbase + k] = (uint16_t)code;
    }
  }
  my_nodes = __reduce_add_sync(0xFFFFFFFFu, my_nodes);
  my_leaves = __reduce_add_sync(0xFFFFFFFFu, my_leaves);
  if ((threadIdx.x & 31u) == 0) {
    if (node_count && my_nodes) atomicAdd(node_count, my_nodes);
    if (leaf_count && my_leaves) atomicAdd(leaf_count, my_leaves);
  }
}

// Index of child ch of region r of a level with n = 2^s regions per axis,
// in the level below (2n per axis).
__device__ __forceinline__ uint64_t child_region(uint64_t r, uint32_t n, int ch) {
  const int s = __ffs(n) - 1;
  const uint64_t rx = r & (n - 1u), ry = (r >> s) & (n - 1u), rz = r >> (2 * s);
  return (2 * rx + (ch & 1)) + ((2 * ry + ((ch >> 1) & 1)) << (s + 1)) +
         ((2 * rz + (ch >> 2)) << (2 * s + 2));
}

// Pass 2: class of each region of level k (n per axis) from its 8 children
// at level k+1 (2n per axis).
// count (may be null): node regions of the level, one atomic per warp.
__global__ void fold_level_kernel(const uint8_t* child, uint32_t n, uint8_t* cls,
                                  uint32_t* count) {
  const uint64_t total = (uint64_t)n * n * n;
  uint32_t my_nodes = 0;
  for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < total;
       r += (uint64_t)gridDim.x * blockDim.x) {
    int n_empty = 0, n_full = 0;
#pragma unroll
    for (int ch = 0; ch < 8; ++ch) {
      const uint8_t k = child[child_region(r, n, ch)];
      n_empty += k == kClsEmpty;
      n_full += k == kClsFull;
    }
    const uint8_t c = n_empty == 8 ? kClsEmpty : (n_full == 8 ? kClsFull : kClsNode);
    cls[r] = c;
    my_nodes += c == kClsNode;
  }
  my_nodes = __reduce_add_sync(0xFFFFFFFFu, my_nodes);
  if (count && (threadIdx.x & 31u) == 0 && my_nodes) atomicAdd(count, my_nodes);
}

// Mask of node children (level < bottom) or leaf children (bottom level).
__device__ __forceinline__ uint32_t node_mask(const uint8_t* child_cls, uint64_t r, uint32_t n) {
  uint32_t mask = 0;
#pragma unroll
  for (int ch = 0; ch < 8; ++ch)
    if (child_cls[child_region(r, n, ch)] == kClsNode) mask |= 1u << ch;
  return mask;
}
__device__ __forceinline__ uint32_t leaf_mask(uint16_t code) {
  uint32_t mask = 0;
#pragma unroll
  for (int ch = 0; ch < 8; ++ch)
    if (((code >> (2 * ch)) & 3u) == kVoxLeaf) mask |= 1u << ch;
  return mask;
}

// Pass 3a: per node of a level list, the number of node children (or of
// leaf children at the bottom level).
__global__ void count_kernel(const uint64_t* list, uint32_t m, const uint8_t* child_cls,
                             const uint16_t* codes, uint32_t n, uint32_t* counts) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const uint64_t r = list[i];
    counts[i] = (uint32_t)__popc(codes ? leaf_mask(codes[r]) : node_mask(child_cls, r, n));
  }
}

// Pass 3b: the next level's list, in breadth-first order.
__global__ void expand_kernel(const uint64_t* list, uint32_t m, const uint8_t* child_cls,
                              uint32_t n, const uint32_t* offsets, uint64_t* next) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const uint64_t r = list[i];
    uint32_t o = offsets[i];
#pragma unroll
    for (int ch = 0; ch < 8; ++ch) {
      const uint64_t c = child_region(r, n, ch);
      if (child_cls[c] == kClsNode) next[o++] = c;
    }
  }
}

__device__ __forceinline__ uint32_t null_word(uint32_t cls_or_code_full) {
  return cls_or_code_full ? YV_FULL_NODE : YV_EMPTY_NODE;
}

// Pass 4a: VoxNodes of one level above the bottom.
__global__ void emit_nodes_kernel(const uint64_t* list, uint32_t m, const uint8_t* child_cls,
                                  uint32_t n, const uint32_t* offsets, uint32_t child_base,
                                  uint32_t node_base, yv_vox_node* out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const uint64_t r = list[i];
    yv_vox_node v;
    v.flags = 0;
    v.data = 0;
    uint32_t next = child_base + offsets[i];
#pragma unroll
    for (int ch = 0; ch < 8; ++ch) {
      const uint8_t k = child_cls[child_region(r, n, ch)];
      if (k == kClsNode) {
        v.child[ch] = next++;
      } else {
        v.child[ch] = null_word(k == kClsFull);
        v.flags |= 1u << (8 + ch);
      }
    }
    out[node_base + i] = v;
  }
}

__device__ __forceinline__ int8_t quant_n(float v) {
  float q = floorf(__fadd_rn(__fmul_rn(127.f, v), 0.5f));
  if (q > 127.f) q = 127.f;
  if (q < -127.f) q = -127.f;
  return (int8_t)(int)q;
}

// Pass 4b: bottom-level VoxNodes (leaf indices from the scanned offsets).
__global__ void emit_bottom_kernel(const uint64_t* list, uint32_t m, const uint16_t* codes,
                                   const uint32_t* offsets, uint32_t node_base,
                                   yv_vox_node* out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const uint32_t code = codes[list[i]];
    yv_vox_node v;
    v.flags = 0;
    v.data = 0;
    uint32_t next = offsets[i];
#pragma unroll
    for (int ch = 0; ch < 8; ++ch) {
      const uint32_t c = (code >> (2 * ch)) & 3u;
      if (c != kVoxLeaf) {
        v.child[ch] = null_word(c == kVoxFull);
        v.flags |= 1u << (8 + ch);
      } else {
        v.child[ch] = next++;
        v.flags |= 1u << ch;
      }
    }
    out[node_base + i] = v;
  }
}

// Pass 4c: leaf attributes, one thread per (bottom node, child): the 8
// lanes of a node handle neighbouring voxels, so the six density loads of
// the central differences of a warp's leaves share sectors.
__global__ void emit_leaves_kernel(Grid g, const uint64_t* list, uint32_t m,
                                   const uint16_t* codes, uint32_t n, const uint32_t* offsets,
                                   yv_leaf_attr* attrs) {
  const uint64_t total = 8ull * m;
  const int sh = __ffs(n) - 1;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
       t += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t i = (uint32_t)(t >> 3);
    const int ch = (int)(t & 7u);
    const uint64_t r = list[i];
    const uint32_t code = codes[r];
    if (((code >> (2 * ch)) & 3u) != kVoxLeaf) continue;
    uint32_t before = 0;  // leaf children before ch
#pragma unroll
    for (int q = 0; q < 8; ++q)
      before += (q < ch && ((code >> (2 * q)) & 3u) == kVoxLeaf) ? 1u : 0u;
    const int rx = (int)(r & (n - 1u)), ry = (int)((r >> sh) & (n - 1u)),
              rz = (int)(r >> (2 * sh));
    const int x = 2 * rx + (ch & 1), y = 2 * ry + ((ch >> 1) & 1), z = 2 * rz + (ch >> 2);
    yv_leaf_attr a;
    if (g.rgb) {
      const size_t o = 3 * vidx(g.G, x, y, z);
      a.r = g.rgb[o];
      a.g = g.rgb[o + 1];
      a.b = g.rgb[o + 2];
    } else {
      a.r = a.g = a.b = 255;
    }
    a.a = 255;
    const float fx = __fsub_rn(dens_clamped(g, x - 1, y, z), dens_clamped(g, x + 1, y, z));
    const float fy = __fsub_rn(dens_clamped(g, x, y - 1, z), dens_clamped(g, x, y + 1, z));
    const float fz = __fsub_rn(dens_clamped(g, x, y, z - 1), dens_clamped(g, x, y, z + 1));
    const float len2 =
        __fadd_rn(__fadd_rn(__fmul_rn(fx, fx), __fmul_rn(fy, fy)), __fmul_rn(fz, fz));
    float nx = 0.f, ny = 0.f, nz = 0.f;
    if (len2 > 0.f && len2 <= 3.402823466e38f) {
      const float len = __fsqrt_rn(len2);
      nx = __fdiv_rn(fx, len);
      ny = __fdiv_rn(fy, len);
      nz = __fdiv_rn(fz, len);
    }
    a.nx = quant_n(nx);
    a.ny = quant_n(ny);
    a.nz = quant_n(nz);
    a.nw = 0;
    attrs[offsets[i] + before] = a;
  }
}

// Renderer layout: 32-byte child-word records, identity id map, 16-byte
// shading records (RGBA8 + unit normal, the FP32 normalisation of the
// upload path).
__global__ void device_layout_kernel(const yv_vox_node* nodes, uint32_t nn, uint32_t* words,
                                     uint32_t* orig) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
    const yv_vox_node v = nodes[i];
#pragma unroll
    for (int ch = 0; ch < 8; ++ch) {
      const uint32_t w = v.child[ch];
      words[8 * (size_t)i + ch] = ((v.flags >> ch) & 1u) ? (YV_DW_LEAF | w)
                                  : (w & 0x80000000u)     ? YV_DW_NULL
                                                          : w;
    }
    orig[i] = i;
  }
}

__global__ void shading_kernel(const yv_leaf_attr* attrs, uint32_t na, uint4* rec) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < na; i += gridDim.x * blockDim.x) {
    const yv_leaf_attr a = attrs[i];
    const float nx = (float)a.nx, ny = (float)a.ny, nz = (float)a.nz;
    const float len2 =
        __fadd_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)), __fmul_rn(nz, nz));
    float u[3] = {0.f, 0.f, 0.f};
    if (len2 > 0.f) {
      const float len = __fsqrt_rn(len2);
      u[0] = __fdiv_rn(nx, len);
      u[1] = __fdiv_rn(ny, len);
      u[2] = __fdiv_rn(nz, len);
    }
    rec[i] = make_uint4((uint32_t)a.r | ((uint32_t)a.g << 8) | ((uint32_t)a.b << 16) |
                            ((uint32_t)a.a << 24),
                        __float_as_uint(u[0]), __float_as_uint(u[1]), __float_as_uint(u[2]));
  }
}

struct BuildResult {
  DevBuf nodes;  // yv_vox_node[nn]
  DevBuf attrs;  // yv_leaf_attr[na]
  uint32_t nn = 0, na = 0, root = YV_EMPTY_NODE;
};

yv_status build_fail(cudaError_t e, const char* what) {
  set_last_error(std::string("dense SVO build: ") + what + ": " + cudaGetErrorString(e));
  cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? YV_ERR_OUT_OF_MEMORY : YV_ERR_CUDA;
}

yv_status build_dense(const float* density, const uint8_t* rgb, int depth, float iso,
                      cudaStream_t s, BuildResult& res) {
  if (!density || depth < 1 || depth > 11 || std::isnan(iso)) return YV_ERR_INVALID_ARG;
  const int G = 1 << depth;
  const Grid g{density, rgb, G, iso};
  // class arrays of every level, codes of the bottom regions
  std::vector<DevBuf> cls((size_t)depth);
  DevBuf codes;
  cudaError_t e;
  for (int k = 0; k < depth; ++k) {
    const uint64_t n = 1ull << k;
    if ((e = cls[(size_t)k].alloc(n * n * n, s)) != cudaSuccess) return build_fail(e, "alloc");
  }
  const uint32_t nb = (uint32_t)(G / 2);
  const uint64_t nb3 = (uint64_t)nb * nb * nb;
  const uint32_t WR = G >= 32 ? (uint32_t)(G / 32) : 1u;
  DevBuf bits;
  if ((e = codes.alloc(nb3 * 2, s)) != cudaSuccess ||
      (e = bits.alloc((uint64_t)G * G * WR * 4, s)) != cudaSuccess)
    return build_fail(e, "alloc");
  // level sizes, counted by the classify and fold passes: hc[0] = root
  // class, hc[k] = node regions of level k (k >= 1), hc[depth] = leaves
  DevBuf dc;
  if ((e = dc.alloc((size_t)(depth + 1) * 4, s)) != cudaSuccess ||
      (e = cudaMemsetAsync(dc.p, 0, (size_t)(depth + 1) * 4, s)) != cudaSuccess)
    return build_fail(e, "alloc");
  uint32_t* dcp = dc.as<uint32_t>();
  if (G >= 128)
    solid_bits_v4_kernel<<<grid_for((uint64_t)G * G * WR * 8), 256, 0, s>>>(
        g, WR, bits.as<uint32_t>());
  else
    solid_bits_kernel<<<grid_for((uint64_t)G * G * WR * 32 / 4), 256, 0, s>>>(
        g, WR, bits.as<uint32_t>());
  classify_bits_kernel<<<grid_for((uint64_t)WR * nb * nb), 256, 0, s>>>(
      bits.as<uint32_t>(), G, WR, nb, cls[(size_t)depth - 1].as<uint8_t>(), codes.as<uint16_t>(),
      depth > 1 ? dcp + depth - 1 : nullptr, dcp + depth);
  for (int k = depth - 2; k >= 0; --k) {
    const uint32_t n = 1u << k;
    fold_level_kernel<<<grid_for((uint64_t)n * n * n), 256, 0, s>>>(
        cls[(size_t)k + 1].as<uint8_t>(), n, cls[(size_t)k].as<uint8_t>(),
        k > 0 ? dcp + k : nullptr);
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return build_fail(e, "classify");
  // read back with one sync (the root class byte into hc[0])
  if ((e = cudaMemcpyAsync(dc.p, cls[0].p, 1, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
    return build_fail(e, "level sizes");
  std::vector<uint32_t> hc((size_t)depth + 1, 0);
  if ((e = cudaGetLastError()) != cudaSuccess ||
      (e = cudaMemcpyAsync(hc.data(), dc.p, (size_t)(depth + 1) * 4, cudaMemcpyDeviceToHost,
                           s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return build_fail(e, "level sizes");
  const uint8_t root_cls = (uint8_t)(hc[0] & 0xFFu);
  if (root_cls != kClsNode) {
    res.root = root_cls == kClsFull ? YV_FULL_NODE : YV_EMPTY_NODE;
    return YV_OK;
  }
  // breadth-first lists, level by level, with no host round trip: the
  // scanned totals are the level sizes counted above
  std::vector<DevBuf> list((size_t)depth), offs((size_t)depth);
  std::vector<uint32_t> m((size_t)depth, 0), base((size_t)depth + 1, 0);
  m[0] = 1;
  for (int k = 1; k < depth; ++k) m[(size_t)k] = hc[(size_t)k];
  for (int k = 0; k < depth; ++k) {
    base[(size_t)k + 1] = base[(size_t)k] + m[(size_t)k];
    if ((uint64_t)base[(size_t)k] + m[(size_t)k] > YV_MAX_DEVICE_NODES) {
      set_last_error("dense SVO build: more than 2^29 nodes");
      return YV_ERR_UNSUPPORTED;
    }
  }
  const uint32_t n_attrs = hc[(size_t)depth];
  if ((e = list[0].alloc(8, s)) != cudaSuccess) return build_fail(e, "alloc");
  if ((e = cudaMemsetAsync(list[0].p, 0, 8, s)) != cudaSuccess) return build_fail(e, "list");
  for (int k = 0; k < depth; ++k) {
    const bool bottom = k == depth - 1;
    const uint32_t n = 1u << k;
    DevBuf counts;
    if ((e = counts.alloc((size_t)m[(size_t)k] * 4, s)) != cudaSuccess ||
        (e = offs[(size_t)k].alloc((size_t)m[(size_t)k] * 4, s)) != cudaSuccess)
      return build_fail(e, "alloc");
    if (m[(size_t)k])
      count_kernel<<<grid_for(m[(size_t)k]), 256, 0, s>>>(
        list[(size_t)k].as<uint64_t>(), m[(size_t)k],
        bottom ? nullptr : cls[(size_t)k + 1].as<uint8_t>(), bottom ? codes.as<uint16_t>() : nullptr,
        n, counts.as<uint32_t>());
    if ((e = cudaGetLastError()) != cudaSuccess ||
        (e = exclusive_scan(counts.as<uint32_t>(), offs[(size_t)k].as<uint32_t>(), m[(size_t)k],
                            nullptr, s)) != cudaSuccess)
      return build_fail(e, "scan");
    if (bottom) break;
    if ((e = list[(size_t)k + 1].alloc((size_t)m[(size_t)k + 1] * 8, s)) != cudaSuccess)
      return build_fail(e, "alloc");
    expand_kernel<<<grid_for(m[(size_t)k]), 256, 0, s>>>(
        list[(size_t)k].as<uint64_t>(), m[(size_t)k], cls[(size_t)k + 1].as<uint8_t>(), n,
        offs[(size_t)k].as<uint32_t>(), list[(size_t)k + 1].as<uint64_t>());
    if ((e = cudaGetLastError()) != cudaSuccess) return build_fail(e, "expand");
  }
  res.nn = base[(size_t)depth];
  res.na = n_attrs;
  res.root = 0;
  if ((e = res.nodes.alloc((size_t)res.nn * sizeof(yv_vox_node), s)) != cudaSuccess ||
      (e = res.attrs.alloc((size_t)res.na * sizeof(yv_leaf_attr), s)) != cudaSuccess)
    return build_fail(e, "alloc");
  for (int k = 0; k < depth - 1; ++k)
    emit_nodes_kernel<<<grid_for(m[(size_t)k]), 256, 0, s>>>(
        list[(size_t)k].as<uint64_t>(), m[(size_t)k], cls[(size_t)k + 1].as<uint8_t>(),
        1u << k, offs[(size_t)k].as<uint32_t>(), base[(size_t)k + 1], base[(size_t)k],
        res.nodes.as<yv_vox_node>());
  const int kb = depth - 1;
  emit_bottom_kernel<<<grid_for(m[(size_t)kb]), 256, 0, s>>>(
      list[(size_t)kb].as<uint64_t>(), m[(size_t)kb], codes.as<uint16_t>(),
      offs[(size_t)kb].as<uint32_t>(), base[(size_t)kb], res.nodes.as<yv_vox_node>());
  if (res.na)
    emit_leaves_kernel<<<grid_for(8ull * m[(size_t)kb]), 256, 0, s>>>(
        g, list[(size_t)kb].as<uint64_t>(), m[(size_t)kb], codes.as<uint16_t>(), 1u << kb,
        offs[(size_t)kb].as<uint32_t>(), res.attrs.as<yv_leaf_attr>());
  if ((e = cudaGetLastError()) != cudaSuccess) return build_fail(e, "emit");
  return YV_OK;
}

}  // namespace
}  // namespace yv

using namespace yv;

extern "C" {

yv_status yv_svo_build_dense(const float* density, const uint8_t* rgb, int32_t depth, float iso,
                             void* stream, yv_svo_host** out) {
  if (!out) return YV_ERR_INVALID_ARG;
  *out = nullptr;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  BuildResult res;
  yv_status st = build_dense(density, rgb, depth, iso, s, res);
  if (st != YV_OK) return st;
  std::vector<yv_vox_node> nodes(res.nn);
  std::vector<yv_leaf_attr> attrs(res.na);
  cudaError_t e = cudaSuccess;
  if (res.nn)
    e = cudaMemcpyAsync(nodes.data(), res.nodes.p, (size_t)res.nn * sizeof(yv_vox_node),
                        cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && res.na)
    e = cudaMemcpyAsync(attrs.data(), res.attrs.p, (size_t)res.na * sizeof(yv_leaf_attr),
                        cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return build_fail(e, "download");
  return yv_svo_from_arrays(out, nodes.data(), res.nn, res.root, attrs.data(), res.na);
}

yv_status yv_set_scene_dense(yv_renderer* r, const float* density, const uint8_t* rgb,
                             int32_t depth, float iso, void* stream) {
  if (!r) return YV_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  BuildResult res;
  yv_status st = build_dense(density, rgb, depth, iso, s, res);
  if (st != YV_OK) return st;
  // renderer layout, written into the renderer's (reused) scene buffers
  uint32_t *words = nullptr, *orig = nullptr;
  void* rec = nullptr;
  st = renderer_scene_buffers(r, res.nn, res.na, &words, &orig, &rec);
  if (st != YV_OK) return st;
  cudaError_t e = cudaSuccess;
  if (res.nn) {
    device_layout_kernel<<<grid_for(res.nn), 256, 0, s>>>(res.nodes.as<yv_vox_node>(), res.nn,
                                                          words, orig);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && res.na) {
    shading_kernel<<<grid_for(res.na), 256, 0, s>>>(res.attrs.as<yv_leaf_attr>(), res.na,
                                                    static_cast<uint4*>(rec));
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return build_fail(e, "device layout");
  renderer_commit_scene(r, res.nn, res.na, (res.root & 0x80000000u) ? YV_DW_NULL : 0u);
  return YV_OK;
}

}  // extern "C"
