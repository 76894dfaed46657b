// svo_kernels.cu - sparse-voxel-octree first-hit ray cast for sm_103a.
//
// One persistent kernel per frame: ray generation (RendererBase::InitRayDir /
// RenderRect, cell/renderer_base.h:50-61, cell/ppu_renderer.cpp:43-70),
// octree descent (RecTrace, cell/ppu_renderer.cpp:18-41, with FindFirstChild
// and GoNext of cell/spu/trace_spu.cpp:48-93), Lambert shading and an
// optional hard-shadow ray per hit, fused.
//
// Design (GB300):
//  * persistent grid (SMs x resident blocks); each warp pops 8x4 pixel tiles
//    from a global counter, so long rays never stall a whole block;
//  * node records are 32 B (one L2 sector) read with two 128-bit loads; the
//    breadth-first first `smem_nodes` records (the top tree levels, touched
//    by every ray) are staged once per block in shared memory;
//  * the recursion of RecTrace becomes a loop with a per-level node-id stack
//    in shared memory and a 3-bit-per-level child path in a register.  On a
//    pop the parent's slab values are not stored: they are recomputed by
//    replaying FindFirstChild/GoNext from the root along the path, which
//    repeats the reference's float operations and so reproduces its values
//    bit for bit (no FMA contraction: every operation is an explicit
//    round-to-nearest intrinsic);
//  * every loop is bounded: a ray that exceeds the iteration cap or the stack
//    depth stops, is reported as a miss and sets a status bit.
#include <cuda_runtime.h>

#include <cstdint>

#include "yv_internal.h"
#include "yv_kernels.h"

namespace yv {
namespace {

constexpr uint32_t kIterCap = 1u << 20;

struct Box {
  float x1, y1, z1, x2, y2, z2;
};

__device__ __forceinline__ float max3f(float a, float b, float c) {
  float m = a > b ? a : b;  // max_vec_float3 order
  return m > c ? m : c;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float m = a < b ? a : b;
  return m < c ? m : c;
}

// FindFirstChild (cell/spu/trace_spu.cpp:48-68).
__device__ __forceinline__ uint32_t ffc(Box& t) {
  const float te = max3f(t.x1, t.y1, t.z1);
  uint32_t ch = 0;
  float tm = __fmul_rn(0.5f, __fadd_rn(t.x1, t.x2));
  if (te > tm) { ch |= 1u; t.x1 = tm; } else { t.x2 = tm; }
  tm = __fmul_rn(0.5f, __fadd_rn(t.y1, t.y2));
  if (te > tm) { ch |= 2u; t.y1 = tm; } else { t.y2 = tm; }
  tm = __fmul_rn(0.5f, __fadd_rn(t.z1, t.z2));
  if (te > tm) { ch |= 4u; t.z1 = tm; } else { t.z2 = tm; }
  return ch;
}

// GoNext (cell/spu/trace_spu.cpp:70-93), argmin tie order of :75-78.
__device__ __forceinline__ bool go_next(uint32_t& ch, Box& t) {
  int e;
  if (t.x2 > t.y2)
    e = (t.y2 < t.z2) ? 1 : 2;
  else
    e = (t.x2 < t.z2) ? 0 : 2;
  const uint32_t mask = 1u << e;
  if (ch & mask) return false;
  ch ^= mask;
  if (e == 0) {
    const float dt = __fsub_rn(t.x2, t.x1);
    t.x1 = t.x2;
    t.x2 = __fadd_rn(t.x2, dt);
  } else if (e == 1) {
    const float dt = __fsub_rn(t.y2, t.y1);
    t.y1 = t.y2;
    t.y2 = __fadd_rn(t.y2, dt);
  } else {
    const float dt = __fsub_rn(t.z2, t.z1);
    t.z1 = t.z2;
    t.z2 = __fadd_rn(t.z2, dt);
  }
  return true;
}

__device__ __forceinline__ uint32_t sel_child(const uint4& a, const uint4& b,
                                              uint32_t c) {
  const uint4 v = (c & 4u) ? b : a;
  const uint32_t lo = (c & 1u) ? v.y : v.x;
  const uint32_t hi = (c & 1u) ? v.w : v.z;
  return (c & 2u) ? hi : lo;
}

__device__ __forceinline__ void fetch_node(const SvoDeviceScene& sc,
                                           const uint4* sm, uint32_t nsm,
                                           uint32_t id, uint4& a, uint4& b) {
  if (id < nsm) {
    a = sm[2 * id];
    b = sm[2 * id + 1];
  } else {
    const uint4* p = sc.nodes + 2 * (size_t)id;
    a = __ldg(p);
    b = __ldg(p + 1);
  }
}

__device__ __forceinline__ uint64_t set_path(uint64_t path, int level,
                                             uint32_t ch) {
  const int sh = 3 * level;
  return (path & ~(7ull << sh)) | ((uint64_t)ch << sh);
}

struct HitRec {
  uint32_t node;   // device node index
  uint32_t child;  // reference child index (ch ^ dirFlags)
  uint32_t leaf;   // VoxData (attribute index)
  uint32_t dir_flags;
  int level;
  float t;
  Box box;         // leaf box (t1, t2)
};

// AdjustDir + SetupTrace + RecTrace for one ray.  kCull: also skip leaves
// lying entirely behind the origin (shadow rays start inside the scene).
template <bool kCull>
__device__ bool svo_trace(const SvoDeviceScene& sc, const uint4* sm,
                          uint32_t nsm, uint32_t* stk, uint32_t stride,
                          float px, float py, float pz, float dx, float dy,
                          float dz, HitRec& hr, uint32_t& fetches,
                          uint32_t& err) {
  // SetupTrace: octant mirroring (reaction/report/voxel.tex:312-326)
  uint32_t df = 0;
  if (dx < 0.f) { px = __fsub_rn(1.f, px); dx = -dx; df |= 1u; }
  if (dy < 0.f) { py = __fsub_rn(1.f, py); dy = -dy; df |= 2u; }
  if (dz < 0.f) { pz = __fsub_rn(1.f, pz); dz = -dz; df |= 4u; }
  Box R;
  R.x1 = __fdiv_rn(__fsub_rn(0.f, px), dx);
  R.x2 = __fdiv_rn(__fsub_rn(1.f, px), dx);
  R.y1 = __fdiv_rn(__fsub_rn(0.f, py), dy);
  R.y2 = __fdiv_rn(__fsub_rn(1.f, py), dy);
  R.z1 = __fdiv_rn(__fsub_rn(0.f, pz), dz);
  R.z2 = __fdiv_rn(__fsub_rn(1.f, pz), dz);
  if (!(max3f(R.x1, R.y1, R.z1) < min3f(R.x2, R.y2, R.z2))) return false;
  uint32_t node = sc.root_word;
  // RecTrace entry test (cell/ppu_renderer.cpp:20-21)
  if ((node & (YV_DW_NULL | YV_DW_LEAF)) || min3f(R.x2, R.y2, R.z2) <= 0.f)
    return false;
  if (node >= sc.n_nodes) {
    err |= YV_DEV_ERR_POOL;
    return false;
  }
  uint4 na, nb;
  fetch_node(sc, sm, nsm, node, na, nb);
  ++fetches;
  Box t = R;
  uint32_t ch = ffc(t);
  uint64_t path = ch;
  int level = 0;
  for (uint32_t it = 0;; ++it) {
    if (it >= kIterCap) {
      err |= YV_DEV_ERR_ITER;
      return false;
    }
    const uint32_t c = ch ^ df;
    const uint32_t w = sel_child(na, nb, c);
    if (w & YV_DW_LEAF) {
      if (!kCull || min3f(t.x2, t.y2, t.z2) > 0.f) {
        hr.node = node;
        hr.child = c;
        hr.leaf = w & 0x7FFFFFFFu;
        hr.dir_flags = df;
        hr.level = level;
        hr.t = max3f(t.x1, t.y1, t.z1);
        hr.box = t;
        return true;
      }
    } else if (!(w & YV_DW_NULL) && min3f(t.x2, t.y2, t.z2) > 0.f) {
      // descend (the recursive call of cell/ppu_renderer.cpp:34)
      if (level + 1 >= YV_MAX_DEPTH) {
        err |= YV_DEV_ERR_DEPTH;
        return false;
      }
      if (w >= sc.n_nodes) {
        err |= YV_DEV_ERR_POOL;
        return false;
      }
      stk[level * stride] = node;
      ++level;
      node = w;
      fetch_node(sc, sm, nsm, node, na, nb);
      ++fetches;
      ch = ffc(t);
      path = set_path(path, level, ch);
      continue;
    }
    if (go_next(ch, t)) {
      path = set_path(path, level, ch);
      continue;
    }
    // Pop: find the deepest ancestor level whose GoNext succeeds, replaying
    // the exact slab arithmetic from the root along the recorded path.
    int best = -1;
    Box bb = R;
    uint32_t bch = 0;
    Box r = R;
    for (int lv = 0; lv < level; ++lv) {
      const uint32_t tgt = (uint32_t)(path >> (3 * lv)) & 7u;
      uint32_t cc = ffc(r);
#pragma unroll 1
      for (int k = 0; k < 3 && cc != tgt; ++k) go_next(cc, r);
      Box q = r;
      uint32_t qc = tgt;
      if (go_next(qc, q)) {
        best = lv;
        bb = q;
        bch = qc;
      }
    }
    if (best < 0) return false;
    level = best;
    node = stk[level * stride];
    fetch_node(sc, sm, nsm, node, na, nb);
    t = bb;
    ch = bch;
    path = set_path(path, level, ch);
  }
}

// Per-pixel ray direction (cell/ppu_renderer.cpp:56) + AdjustDir (eps 1e-5).
__device__ __forceinline__ void pixel_dir(const SvoFrameArgs& a, int x, int y,
                                          float& dx, float& dy, float& dz) {
  const float fx = (float)x, fy = (float)y;
  dx = __fadd_rn(__fadd_rn(a.dir0[0], __fmul_rn(a.du[0], fx)), __fmul_rn(a.dv[0], fy));
  dy = __fadd_rn(__fadd_rn(a.dir0[1], __fmul_rn(a.du[1], fx)), __fmul_rn(a.dv[1], fy));
  dz = __fadd_rn(__fadd_rn(a.dir0[2], __fmul_rn(a.du[2], fx)), __fmul_rn(a.dv[2], fy));
  const float len = __fsqrt_rn(
      __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
  dx = __fdiv_rn(dx, len);
  dy = __fdiv_rn(dy, len);
  dz = __fdiv_rn(dz, len);
  const float eps = 1e-5f;
  if (fabsf(dx) < eps) dx = copysignf(eps, dx);
  if (fabsf(dy) < eps) dy = copysignf(eps, dy);
  if (fabsf(dz) < eps) dz = copysignf(eps, dz);
}

// Lambert: ambient + diffuse*max(0, n.L) (ambient only in shadow).
__device__ __forceinline__ uint32_t shade(uint2 at, const SvoFrameArgs& a,
                                          bool shadowed) {
  const float nx = (float)(int8_t)(at.y & 0xFFu);
  const float ny = (float)(int8_t)((at.y >> 8) & 0xFFu);
  const float nz = (float)(int8_t)((at.y >> 16) & 0xFFu);
  const float len2 =
      __fadd_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)), __fmul_rn(nz, nz));
  float ndl = 0.f;
  if (len2 > 0.f) {
    const float len = __fsqrt_rn(len2);
    const float ux = __fdiv_rn(nx, len), uy = __fdiv_rn(ny, len), uz = __fdiv_rn(nz, len);
    ndl = __fadd_rn(__fadd_rn(__fmul_rn(ux, a.light[0]), __fmul_rn(uy, a.light[1])),
                    __fmul_rn(uz, a.light[2]));
  }
  const float dif = ndl > 0.f ? ndl : 0.f;
  const float inten = shadowed ? a.ambient : __fadd_rn(a.ambient, __fmul_rn(a.diffuse, dif));
  uint32_t out = 0xFF000000u;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float v = __fadd_rn(__fmul_rn((float)((at.x >> (8 * c)) & 0xFFu), inten), 0.5f);
    const uint32_t u = v >= 255.f ? 255u : __float2uint_rz(v);
    out |= u << (8 * c);
  }
  return out;
}

__global__ void __launch_bounds__(256) svo_frame_kernel(SvoDeviceScene sc,
                                                        SvoFrameArgs a,
                                                        uint32_t nsm) {
  extern __shared__ uint4 smem[];
  uint4* snodes = smem;
  uint32_t* sstack = reinterpret_cast<uint32_t*>(smem + 2 * nsm);
  for (uint32_t i = threadIdx.x; i < 2 * nsm; i += blockDim.x)
    snodes[i] = __ldg(sc.nodes + i);
  __syncthreads();

  const uint32_t lane = threadIdx.x & 31u;
  uint32_t* stk = sstack + threadIdx.x;
  const uint32_t stride = blockDim.x;
  const int tiles_x = (a.width + 7) >> 3;
  const int n_tiles = tiles_x * ((a.height + 3) >> 2);
  uint32_t err = 0;

  for (;;) {
    uint32_t tile = 0;
    if (lane == 0) tile = atomicAdd(&a.counters[0], 1u);
    tile = __shfl_sync(0xFFFFFFFFu, tile, 0);
    if (tile >= (uint32_t)n_tiles) break;
    const int x = (int)(tile % (uint32_t)tiles_x) * 8 + (int)(lane & 7u);
    const int y = (int)(tile / (uint32_t)tiles_x) * 4 + (int)(lane >> 3);
    const bool valid = x < a.width && y < a.height;
    bool hit = false, shadowed = false;
    if (valid) {
      float dx, dy, dz;
      pixel_dir(a, x, y, dx, dy, dz);
      HitRec hr;
      uint32_t f = 0, fs = 0;
      hit = svo_trace<false>(sc, snodes, nsm, stk, stride, a.pos[0], a.pos[1],
                             a.pos[2], dx, dy, dz, hr, f, err);
      uint32_t rgba = 0, hw = 0xFFFFFFFFu;
      float ht = 0.f;
      if (hit) {
        hw = (__ldg(sc.orig_id + hr.node) << 3) | hr.child;
        ht = hr.t;
        uint2 at = make_uint2(0u, 0u);
        if (hr.leaf < sc.n_attrs)
          at = __ldg(sc.attrs + hr.leaf);
        else
          err |= YV_DEV_ERR_POOL;
        if (a.shadows) {
          // hit point, moved half a leaf out through the entry face
          float o[3];
          o[0] = __fadd_rn(a.pos[0], __fmul_rn(dx, ht));
          o[1] = __fadd_rn(a.pos[1], __fmul_rn(dy, ht));
          o[2] = __fadd_rn(a.pos[2], __fmul_rn(dz, ht));
          int e = 0;
          float m = hr.box.x1;
          if (hr.box.y1 > m) { e = 1; m = hr.box.y1; }
          if (hr.box.z1 > m) { e = 2; }
          const float half = __int_as_float((127 - (hr.level + 2)) << 23);
          const float off = ((hr.dir_flags >> e) & 1u) ? half : -half;
          o[e] = __fadd_rn(o[e], off);
          HitRec hs;
          shadowed = svo_trace<true>(sc, snodes, nsm, stk, stride, o[0], o[1],
                                     o[2], a.light_ray[0], a.light_ray[1],
                                     a.light_ray[2], hs, fs, err);
        }
        rgba = shade(at, a, shadowed);
      }
      const size_t off = (size_t)y * (size_t)a.width + (size_t)x;
      if (a.rgba) a.rgba[off] = rgba;
      if (a.hit) a.hit[off] = hw;
      if (a.hit_t) a.hit_t[off] = ht;
      if (a.fetches) a.fetches[off] = f;
      if (a.shadow_fetches) a.shadow_fetches[off] = fs;
    }
    const uint32_t hm = __ballot_sync(0xFFFFFFFFu, hit);
    const uint32_t sm_ = __ballot_sync(0xFFFFFFFFu, shadowed);
    if (lane == 0 && hm) {
      atomicAdd(&a.counters[2], (uint32_t)__popc(hm));
      if (sm_) atomicAdd(&a.counters[3], (uint32_t)__popc(sm_));
    }
  }
  if (err) atomicOr(&a.counters[1], err);
}

}  // namespace

int device_sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
  if (cached[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 1;
    cached[dev] = n;
  }
  return cached[dev];
}

cudaError_t launch_svo_frame(const SvoDeviceScene& sc, const SvoFrameArgs& a,
                             const LaunchCfg& cfg, cudaStream_t stream,
                             int* launches) {
  int bt = cfg.block_threads;
  if (bt < 32 || bt > 256 || (bt & 31)) bt = 256;
  uint32_t nsm = (uint32_t)(cfg.smem_nodes < 0 ? 0 : cfg.smem_nodes);
  if (nsm > sc.n_nodes) nsm = sc.n_nodes;
  if (nsm > 4096) nsm = 4096;
  const size_t smem = (size_t)nsm * 32u + (size_t)YV_MAX_DEPTH * (size_t)bt * 4u;
  if (smem > 48u * 1024u) {
    static bool opted_in[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    if (!opted_in[dev]) {
      cudaError_t e = cudaFuncSetAttribute(
          svo_frame_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
      if (e != cudaSuccess) return e;
      opted_in[dev] = true;
    }
  }
  int per_sm = cfg.blocks_per_sm;
  if (per_sm <= 0) {
    cudaError_t e =
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, svo_frame_kernel, bt, smem);
    if (e != cudaSuccess) return e;
    if (per_sm <= 0) per_sm = 1;
  }
  const int grid = device_sm_count() * per_sm;
  cudaError_t e = cudaMemsetAsync(a.counters, 0, kSvoCounterWords * sizeof(uint32_t), stream);
  if (e != cudaSuccess) return e;
  svo_frame_kernel<<<grid, bt, smem, stream>>>(sc, a, nsm);
  if (launches) *launches = 1;
  return cudaGetLastError();
}

}  // namespace yv
