/*
 * yv_oracle_build.c - CPU oracle for the SVO build from a dense density grid.
 *
 * TEST INFRASTRUCTURE ONLY (the checker of the CUDA builder and the timed
 * CPU baseline of the build); the product library never links or calls it.
 *
 * Restates the iso/raw-source form of DynamicSVO::BuildRange (the GROW pass
 * driven by a voxel source, ore/src/main.cpp:37-129 and
 * demo/Demo.cpp:82-114; the DynamicSVO source itself is not in the
 * reference snapshot) with the surface-voxel rule of scene_gen.py:32-66 and
 * the node layout of reaction/report/main.tex:36-56:
 *   - voxel v of the 2^depth grid is solid iff density[v] > iso;
 *   - a solid voxel with a 6-neighbour that is outside the grid or not solid
 *     is a surface voxel: a leaf (flags bit ch, child = attribute index);
 *   - a cube region without surface voxels is EmptyNode (0x80000000, no
 *     solid voxel) or FullNode (0x80000001), with the null flag bit 8+ch;
 *     a node whose 8 children are all EmptyNode (FullNode) is itself
 *     EmptyNode (FullNode);
 *   - nodes are numbered breadth-first from the root (id 0), children in
 *     child order c = x | y<<1 | z<<2; attributes in the same order;
 *   - leaf attribute: RGB of the voxel (white without an rgb grid), A = 255,
 *     normal = the central difference (d(x-1) - d(x+1), d(y-1) - d(y+1),
 *     d(z-1) - d(z+1)) in float with coordinates clamped to the grid,
 *     normalised in float (len^2 = (x*x + y*y) + z*z, sqrt, three
 *     divisions, each rounded to nearest) and quantised as
 *     floor(127 v + 0.5) in float, clamped to [-127, 127] (nw = 0); a zero
 *     or non-finite len^2 gives a zero normal.
 * Density is indexed x + G (y + G z), G = 2^depth.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "yv_oracle.h"

#define ORC_EMPTY 0x80000000u
#define ORC_FULL 0x80000001u

typedef struct {
  uint32_t flags, data, child[8];
} orc_node;

typedef struct {
  const float* d;
  const uint8_t* rgb;
  int G;
  float iso;
  orc_node* nodes;
  size_t n_nodes, cap_nodes;
  uint8_t* attrs;
  size_t n_attrs, cap_attrs;
  int oom;
} orc_build;

static float orc_dens(const orc_build* b, int x, int y, int z) {
  const int G = b->G;
  x = x < 0 ? 0 : (x >= G ? G - 1 : x);
  y = y < 0 ? 0 : (y >= G ? G - 1 : y);
  z = z < 0 ? 0 : (z >= G ? G - 1 : z);
  return b->d[(size_t)x + (size_t)G * ((size_t)y + (size_t)G * (size_t)z)];
}

static int orc_solid(const orc_build* b, int x, int y, int z) {
  const int G = b->G;
  if (x < 0 || y < 0 || z < 0 || x >= G || y >= G || z >= G) return 0;
  return b->d[(size_t)x + (size_t)G * ((size_t)y + (size_t)G * (size_t)z)] > b->iso;
}

static int orc_surface(const orc_build* b, int x, int y, int z) {
  return !orc_solid(b, x + 1, y, z) || !orc_solid(b, x - 1, y, z) ||
         !orc_solid(b, x, y + 1, z) || !orc_solid(b, x, y - 1, z) ||
         !orc_solid(b, x, y, z + 1) || !orc_solid(b, x, y, z - 1);
}

static int8_t orc_quant(float v) {
  float q = floorf(127.0f * v + 0.5f);
  if (q > 127.0f) q = 127.0f;
  if (q < -127.0f) q = -127.0f;
  return (int8_t)(int)q;
}

static void orc_leaf_attr(const orc_build* b, int x, int y, int z, uint8_t* a) {
  const int G = b->G;
  const size_t v = (size_t)x + (size_t)G * ((size_t)y + (size_t)G * (size_t)z);
  a[0] = b->rgb ? b->rgb[v * 3] : 255;
  a[1] = b->rgb ? b->rgb[v * 3 + 1] : 255;
  a[2] = b->rgb ? b->rgb[v * 3 + 2] : 255;
  a[3] = 255;
  const float fx = orc_dens(b, x - 1, y, z) - orc_dens(b, x + 1, y, z);
  const float fy = orc_dens(b, x, y - 1, z) - orc_dens(b, x, y + 1, z);
  const float fz = orc_dens(b, x, y, z - 1) - orc_dens(b, x, y, z + 1);
  const float len2 = fx * fx + fy * fy + fz * fz;
  float nx = 0.f, ny = 0.f, nz = 0.f;
  if (len2 > 0.f && len2 <= FLT_MAX) {
    const float len = sqrtf(len2);
    nx = fx / len;
    ny = fy / len;
    nz = fz / len;
  }
  a[4] = (uint8_t)orc_quant(nx);
  a[5] = (uint8_t)orc_quant(ny);
  a[6] = (uint8_t)orc_quant(nz);
  a[7] = 0;
}

static uint32_t orc_push_node(orc_build* b, const orc_node* n) {
  if (b->n_nodes == b->cap_nodes) {
    size_t c = b->cap_nodes ? 2 * b->cap_nodes : 1024;
    orc_node* p = (orc_node*)realloc(b->nodes, c * sizeof(orc_node));
    if (!p) {
      b->oom = 1;
      return ORC_EMPTY;
    }
    b->nodes = p;
    b->cap_nodes = c;
  }
  b->nodes[b->n_nodes] = *n;
  return (uint32_t)b->n_nodes++;
}

static uint32_t orc_push_attr(orc_build* b, const uint8_t* a) {
  if (b->n_attrs == b->cap_attrs) {
    size_t c = b->cap_attrs ? 2 * b->cap_attrs : 1024;
    uint8_t* p = (uint8_t*)realloc(b->attrs, c * 8);
    if (!p) {
      b->oom = 1;
      return 0;
    }
    b->attrs = p;
    b->cap_attrs = c;
  }
  memcpy(b->attrs + b->n_attrs * 8, a, 8);
  return (uint32_t)b->n_attrs++;
}

/* Post-order build of the region [x0, x0+s)^3; returns EmptyNode, FullNode
 * or the temporary index of the node. */
static uint32_t orc_build_region(orc_build* b, int x0, int y0, int z0, int s) {
  orc_node n;
  memset(&n, 0, sizeof(n));
  int n_empty = 0, n_full = 0;
  if (s == 2) {
    for (int ch = 0; ch < 8; ++ch) {
      const int x = x0 + (ch & 1), y = y0 + ((ch >> 1) & 1), z = z0 + ((ch >> 2) & 1);
      if (!orc_solid(b, x, y, z)) {
        n.child[ch] = ORC_EMPTY;
        ++n_empty;
      } else if (orc_surface(b, x, y, z)) {
        uint8_t a[8];
        orc_leaf_attr(b, x, y, z, a);
        n.child[ch] = orc_push_attr(b, a);
        n.flags |= 1u << ch;
      } else {
        n.child[ch] = ORC_FULL;
        ++n_full;
      }
    }
  } else {
    const int h = s / 2;
    for (int ch = 0; ch < 8; ++ch) {
      const uint32_t w = orc_build_region(b, x0 + (ch & 1) * h, y0 + ((ch >> 1) & 1) * h,
                                          z0 + ((ch >> 2) & 1) * h, h);
      if (w == ORC_EMPTY) ++n_empty;
      if (w == ORC_FULL) ++n_full;
      n.child[ch] = w;
    }
  }
  if (n_empty == 8) return ORC_EMPTY;
  if (n_full == 8) return ORC_FULL;
  for (int ch = 0; ch < 8; ++ch)
    if (!((n.flags >> ch) & 1u) && (n.child[ch] & 0x80000000u)) n.flags |= 1u << (8 + ch);
  return orc_push_node(b, &n);
}

int orc_svo_build_dense(const float* density, const uint8_t* rgb, int depth, float iso,
                        uint32_t* nodes, uint32_t node_cap, uint8_t* attrs,
                        uint32_t attr_cap, uint32_t* n_nodes, uint32_t* n_attrs,
                        uint32_t* root) {
  if (depth < 1 || depth > 12 || !density || !n_nodes || !n_attrs || !root) return 2;
  orc_build b;
  memset(&b, 0, sizeof(b));
  b.d = density;
  b.rgb = rgb;
  b.G = 1 << depth;
  b.iso = iso;
  const uint32_t r = orc_build_region(&b, 0, 0, 0, b.G);
  if (b.oom) {
    free(b.nodes);
    free(b.attrs);
    return 3;
  }
  *n_nodes = (uint32_t)b.n_nodes;
  *n_attrs = (uint32_t)b.n_attrs;
  if (r & 0x80000000u) {
    *root = r;
    *n_nodes = 0;
    *n_attrs = 0;
    free(b.nodes);
    free(b.attrs);
    return 0;
  }
  if (b.n_nodes > node_cap || b.n_attrs > attr_cap || !nodes || (b.n_attrs && !attrs)) {
    free(b.nodes);
    free(b.attrs);
    return 1;
  }
  /* breadth-first renumbering: queue of temporary indices */
  uint32_t* order = (uint32_t*)malloc(b.n_nodes * sizeof(uint32_t));
  if (!order) {
    free(b.nodes);
    free(b.attrs);
    return 3;
  }
  size_t head = 0, tail = 0;
  order[tail++] = r;
  while (head < tail) {
    const orc_node* n = &b.nodes[order[head++]];
    for (int ch = 0; ch < 8; ++ch)
      if (!((n->flags >> ch) & 1u) && !(n->child[ch] & 0x80000000u))
        order[tail++] = n->child[ch];
  }
  uint32_t next_node = 1, next_attr = 0;
  for (size_t i = 0; i < tail; ++i) {
    orc_node n = b.nodes[order[i]];
    for (int ch = 0; ch < 8; ++ch) {
      if ((n.flags >> ch) & 1u) {
        memcpy(attrs + (size_t)next_attr * 8, b.attrs + (size_t)n.child[ch] * 8, 8);
        n.child[ch] = next_attr++;
      } else if (!(n.child[ch] & 0x80000000u)) {
        n.child[ch] = next_node++;
      }
    }
    uint32_t* o = nodes + i * 10;
    o[0] = n.flags;
    o[1] = n.data;
    for (int ch = 0; ch < 8; ++ch) o[2 + ch] = n.child[ch];
  }
  *root = 0;
  free(order);
  free(b.nodes);
  free(b.attrs);
  return 0;
}
