// svo_trace.cuh - device code of the sparse-voxel-octree first-hit ray cast
// for sm_103a (included by svo_kernels.cu and svo_noalloc.cu).
//
// One persistent kernel per frame: ray generation (RendererBase::InitRayDir /
// RenderRect, cell/renderer_base.h:50-61, cell/ppu_renderer.cpp:43-70),
// octree descent (RecTrace, cell/ppu_renderer.cpp:18-41, with FindFirstChild
// and GoNext of cell/spu/trace_spu.cpp:48-93), Lambert shading and an
// optional hard-shadow ray per hit, fused.
//
// Design (GB300):
//  * persistent grid (SMs x resident blocks).  Every lane runs its own small
//    state machine (primary ray -> shadow ray -> idle) one traversal step per
//    loop iteration; idle lanes of a warp are refilled together from a
//    global ray counter (one atomic per refill), so a warp never waits for
//    the slowest ray of a tile and the shadow rays of some lanes overlap the
//    primary rays of others.  Consecutive ray ids map to 8x4 pixel tiles, so
//    lanes refilled together trace neighbouring pixels;
//  * node records are 32 B (one L2 sector); a traversal step reads the one
//    32-bit child word it tests (the sector stays in L1 while the ray is in
//    the node).  Staging the breadth-first first `smem_nodes` records (the
//    top tree levels) in shared memory is a separately compiled variant the
//    launch configuration can ask for; reading every record through L1
//    measured as fast or faster, so it is off by default;
//  * the recursion of RecTrace becomes an explicit per-lane stack of
//    (node id, child, slab box) frames, so a pop restores the parent's exact
//    float values: every operation is an explicit round-to-nearest intrinsic
//    (no FMA contraction), which keeps hit ids bit-identical to the FP32
//    restatement of the reference;
//  * every loop is bounded: a ray that exceeds the step cap or the stack
//    depth stops, is reported as a miss and sets a status bit;
//  * an optional frame time budget bounds the queue itself: a warp about to
//    take new rays after the budget has elapsed (the global timer against
//    its block's start) takes none, and the frame reports a timeout.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "yv_internal.h"
#include "yv_kernels.h"

namespace yv {
namespace {

constexpr uint32_t kFetchCap = 1u << 20;
// traversal steps between two warp votes (refill / end-of-ray handling)
constexpr int kStepsPerVote = 8;

struct Box {
  float x1, y1, z1, x2, y2, z2;
};

__device__ __forceinline__ float max3f(float a, float b, float c) {
  float m = a > b ? a : b;  // max_vec_float3 order
  return m > c ? m : c;
}
// Minimum / maximum for the comparisons of the traversal (slab values are
// never NaN; +0 and -0 compare equal, so the choice between them is moot).
__device__ __forceinline__ float fmin3(float a, float b, float c) {
  return fminf(fminf(a, b), c);
}
__device__ __forceinline__ float fmax3(float a, float b, float c) {
  return fmaxf(fmaxf(a, b), c);
}

// FindFirstChild (cell/spu/trace_spu.cpp:48-68).
__device__ __forceinline__ uint32_t ffc(Box& t) {
  const float te = fmax3(t.x1, t.y1, t.z1);
  uint32_t ch = 0;
  float tm = __fmul_rn(0.5f, __fadd_rn(t.x1, t.x2));
  if (te > tm) { ch |= 1u; t.x1 = tm; } else { t.x2 = tm; }
  tm = __fmul_rn(0.5f, __fadd_rn(t.y1, t.y2));
  if (te > tm) { ch |= 2u; t.y1 = tm; } else { t.y2 = tm; }
  tm = __fmul_rn(0.5f, __fadd_rn(t.z1, t.z2));
  if (te > tm) { ch |= 4u; t.z1 = tm; } else { t.z2 = tm; }
  return ch;
}

// GoNext (cell/spu/trace_spu.cpp:70-93) in two parts: the exit axis (the
// argmin tie order of :75-78) and the move into the sibling across it.
__device__ __forceinline__ int exit_axis(const Box& t) {
  if (t.x2 > t.y2) return (t.y2 < t.z2) ? 1 : 2;
  return (t.x2 < t.z2) ? 0 : 2;
}

__device__ __forceinline__ void advance(uint32_t& ch, Box& t, int e) {
  // branch-free: the lanes of a warp cross different axes
  ch ^= 1u << e;
  const bool ex = e == 0, ey = e == 1, ez = e == 2;
  const float a1 = ex ? t.x1 : (ey ? t.y1 : t.z1);
  const float a2 = ex ? t.x2 : (ey ? t.y2 : t.z2);
  const float n2 = __fadd_rn(a2, __fsub_rn(a2, a1));
  t.x1 = ex ? a2 : t.x1;
  t.x2 = ex ? n2 : t.x2;
  t.y1 = ey ? a2 : t.y1;
  t.y2 = ey ? n2 : t.y2;
  t.z1 = ez ? a2 : t.z1;
  t.z2 = ez ? n2 : t.z2;
}

// Child word c of node id, read where it lies at every step (the node's
// sector stays in L1 while the ray is inside it, so the 8 words are not
// held in registers).  kRef = false: the library's 32-byte device records
// (top levels from shared memory).  kRef = true: the reference's 40-byte
// VoxNode {flags, data, child[8]} read in place, its leaf / null flags
// folded into the same word encoding.
// kStaged: the first nsm records are read from shared memory.
template <bool kRef, bool kStaged>
__device__ __forceinline__ uint32_t child_word(const SvoDeviceScene& sc, const uint32_t* sm,
                                               uint32_t nsm, uint32_t id, uint32_t c) {
  if (kRef) {
    const uint32_t* p = reinterpret_cast<const uint32_t*>(sc.nodes) + 10 * (size_t)id;
    const uint32_t fl = __ldg(p);
    const uint32_t cw = __ldg(p + 2 + c);
    return ((fl >> c) & 1u) ? (YV_DW_LEAF | cw) : ((cw & 0x80000000u) ? YV_DW_NULL : cw);
  }
  if (kStaged && id < nsm) return sm[8 * id + c];
  return __ldg(reinterpret_cast<const uint32_t*>(sc.nodes) + 8 * (size_t)id + c);
}

// Nanoseconds of the GPU's global timer.
__device__ __forceinline__ unsigned long long global_timer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// One stack frame: a level whose current child still has a next sibling
// along the ray - the node, the child taken and that child's slab box,
// exactly as RecTrace holds them in its activation record - and the level.
// Levels whose current child is the last one the ray crosses are never
// pushed: returning to them would only return further.
struct __align__(16) Frame {
  uint32_t idch;  // node << 3 | ch
  float x1, y1, z1;
  float x2, y2, z2;
  uint32_t level;
};

enum : uint32_t { kIdle = 0, kPrimary = 1, kShadow = 2, kDone = 3 };
enum : int { kContinue = 0, kHit = 1, kMiss = 2 };

// Traversal state of one lane.
struct Trace {
  uint32_t node, ch, df, fetches;
  uint32_t sp;  // frames held
  uint32_t lo;  // with a shared-memory ring: frames below lo are in local memory
  int level;
  Box t;
};

// Per-lane frame stack.  kRing = 0: every frame in a local-memory array.
// kRing > 0 (a power of two): the newest kRing frames in a shared-memory
// ring, one 16-byte column per lane (lane-contiguous, so a warp's stores and
// loads are conflict-free and move only the active lanes' bytes); a push
// into a full ring first moves the oldest frame to the local array.
template <int kRing>
__device__ __forceinline__ void push_frame(Frame* stk, uint4* ring, Trace& tr, const Frame& f) {
  if (kRing == 0) {
    stk[tr.sp++] = f;
    return;
  }
  if (tr.sp - tr.lo == (uint32_t)kRing) {
    const uint32_t s = tr.lo & (uint32_t)(kRing - 1);
    const uint4 q0 = ring[(2 * s) * 32], q1 = ring[(2 * s + 1) * 32];
    Frame g;
    g.idch = q0.x;
    g.x1 = __uint_as_float(q0.y); g.y1 = __uint_as_float(q0.z); g.z1 = __uint_as_float(q0.w);
    g.x2 = __uint_as_float(q1.x); g.y2 = __uint_as_float(q1.y); g.z2 = __uint_as_float(q1.z);
    g.level = q1.w;
    stk[tr.lo++] = g;
  }
  const uint32_t s = tr.sp & (uint32_t)(kRing - 1);
  ring[(2 * s) * 32] =
      make_uint4(f.idch, __float_as_uint(f.x1), __float_as_uint(f.y1), __float_as_uint(f.z1));
  ring[(2 * s + 1) * 32] =
      make_uint4(__float_as_uint(f.x2), __float_as_uint(f.y2), __float_as_uint(f.z2), f.level);
  ++tr.sp;
}

template <int kRing>
__device__ __forceinline__ Frame pop_frame(const Frame* stk, const uint4* ring, Trace& tr) {
  --tr.sp;
  if (kRing == 0) return stk[tr.sp];
  if (tr.sp < tr.lo) {
    tr.lo = tr.sp;
    return stk[tr.sp];
  }
  const uint32_t s = tr.sp & (uint32_t)(kRing - 1);
  const uint4 q0 = ring[(2 * s) * 32], q1 = ring[(2 * s + 1) * 32];
  Frame g;
  g.idch = q0.x;
  g.x1 = __uint_as_float(q0.y); g.y1 = __uint_as_float(q0.z); g.z1 = __uint_as_float(q0.w);
  g.x2 = __uint_as_float(q1.x); g.y2 = __uint_as_float(q1.y); g.z2 = __uint_as_float(q1.z);
  g.level = q1.w;
  return g;
}


// SetupTrace (reaction/report/voxel.tex:312-326) + RecTrace entry test
// (cell/ppu_renderer.cpp:20-21) + the root fetch.  False: the ray misses.
__device__ __forceinline__ bool begin_trace(const SvoDeviceScene& sc, float px, float py, float pz,
                                            float dx, float dy, float dz, Trace& tr,
                                            uint32_t& err) {
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
  tr.fetches = 0;
  if (!(fmax3(R.x1, R.y1, R.z1) < fmin3(R.x2, R.y2, R.z2))) return false;
  const uint32_t root = sc.root_word;
  if ((root & (YV_DW_NULL | YV_DW_LEAF)) || fmin3(R.x2, R.y2, R.z2) <= 0.f) return false;
  if (root >= sc.n_nodes) {
    err |= YV_DEV_ERR_POOL;
    return false;
  }
  tr.node = root;
  tr.df = df;
  tr.level = 0;
  tr.sp = 0;
  tr.lo = 0;
  tr.fetches = 1;
  tr.t = R;
  tr.ch = ffc(tr.t);
  return true;
}

// One step of RecTrace: test the current child (leaf -> hit, subtree ->
// descend), else move to the next sibling, first returning to the nearest
// pushed level when this one is exhausted (that level's next sibling exists
// by construction, so both cases share the move).
// kRef (caller-supplied VoxNode pool): child refs are range-checked, depth
// is capped at YV_MAX_DEPTH levels and a ray stops with YV_DEV_ERR_ITER after
// kFetchCap fetches.  The library's own layout is validated acyclic, in
// range and at most YV_MAX_DEPTH levels deep when it is built, so it needs
// none of these.  In both cases a push happens at level < YV_MAX_DEPTH - 1,
// so at most YV_MAX_DEPTH - 1 frames are ever held.
// kLod (library layout only): before descending into a subtree whose cube
// side 2^-(level+1) is smaller than max(t_enter, 0) * lod_coef, the ray stops
// there as at a leaf, with the subtree's level-of-detail attribute.
template <bool kRef, int kRing, bool kStaged = false, bool kLod = false>
__device__ __forceinline__ int trace_step(const SvoDeviceScene& sc, const uint32_t* sm,
                                          uint32_t nsm, Frame* stk, uint4* ring, Trace& tr,
                                          bool cull, uint32_t& leaf, uint32_t& err,
                                          float lod_coef = 0.f) {
  const uint32_t w = child_word<kRef, kStaged>(sc, sm, nsm, tr.node, tr.ch ^ tr.df);
  const bool ahead = fmin3(tr.t.x2, tr.t.y2, tr.t.z2) > 0.f;
  // exit axis of the current child and whether it is the last one along
  // the ray in this node (needed by both the descent and the sibling move)
  int e = exit_axis(tr.t);
  const bool last = (tr.ch >> e) & 1u;
  if (w & YV_DW_LEAF) {
    if (!cull || ahead) {
      leaf = w & 0x7FFFFFFFu;
      return kHit;
    }
  } else if (!(w & YV_DW_NULL) && ahead) {
    if (kLod) {
      const float side = __int_as_float((126 - tr.level) << 23);  // 2^-(level+1)
      const float te = fmaxf(fmax3(tr.t.x1, tr.t.y1, tr.t.z1), 0.f);
      if (side < __fmul_rn(te, lod_coef)) {
        leaf = __ldg(sc.node_data + w);
        return kHit;
      }
    }
    // descend: the recursive call of cell/ppu_renderer.cpp:34
    if (kRef) {
      if (tr.fetches >= kFetchCap) {
        err |= YV_DEV_ERR_ITER;
        return kMiss;
      }
      if (tr.level + 1 >= YV_MAX_DEPTH) {
        err |= YV_DEV_ERR_DEPTH;
        return kMiss;
      }
      if (w >= sc.n_nodes) {
        err |= YV_DEV_ERR_POOL;
        return kMiss;
      }
    }
    ++tr.fetches;
    if (!last) {
      Frame f;
      f.idch = (tr.node << 3) | tr.ch;
      f.x1 = tr.t.x1; f.y1 = tr.t.y1; f.z1 = tr.t.z1;
      f.x2 = tr.t.x2; f.y2 = tr.t.y2; f.z2 = tr.t.z2;
      f.level = (uint32_t)tr.level;
      push_frame<kRing>(stk, ring, tr, f);
    }
    ++tr.level;
    tr.node = w;
    tr.ch = ffc(tr.t);
    return kContinue;
  }
  if (last) {
    if (tr.sp == 0) return kMiss;
    const Frame f = pop_frame<kRing>(stk, ring, tr);
    tr.ch = f.idch & 7u;
    tr.node = f.idch >> 3;
    tr.level = (int)f.level;
    tr.t.x1 = f.x1; tr.t.y1 = f.y1; tr.t.z1 = f.z1;
    tr.t.x2 = f.x2; tr.t.y2 = f.y2; tr.t.z2 = f.z2;
    e = exit_axis(tr.t);
  }
  advance(tr.ch, tr.t, e);
  return kContinue;
}

// Per-pixel ray direction (cell/ppu_renderer.cpp:56) + AdjustDir (eps 1e-5).
__device__ __forceinline__ void pixel_dir(const SvoFrameArgs& a, int x, int y, float& dx,
                                          float& dy, float& dz) {
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

// Shading record of a leaf: x = RGBA8, y/z/w = the unit normal in FP32
// (int8 normal / its length, each a round-to-nearest operation; zero for a
// zero normal).  The library's layout stores these records (normalised once
// on the host); a caller's 8-byte yv_leaf_attr is normalised here.
__device__ __forceinline__ uint4 shading_record(uint2 at) {
  const float nx = (float)(int8_t)(at.y & 0xFFu);
  const float ny = (float)(int8_t)((at.y >> 8) & 0xFFu);
  const float nz = (float)(int8_t)((at.y >> 16) & 0xFFu);
  const float len2 =
      __fadd_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)), __fmul_rn(nz, nz));
  float ux = 0.f, uy = 0.f, uz = 0.f;
  if (len2 > 0.f) {
    const float len = __fsqrt_rn(len2);
    ux = __fdiv_rn(nx, len);
    uy = __fdiv_rn(ny, len);
    uz = __fdiv_rn(nz, len);
  }
  return make_uint4(at.x, __float_as_uint(ux), __float_as_uint(uy), __float_as_uint(uz));
}

template <bool kRef>
__device__ __forceinline__ uint4 load_shading(const SvoDeviceScene& sc, uint32_t leaf) {
  if (kRef) return shading_record(__ldg(static_cast<const uint2*>(sc.attrs) + leaf));
  return __ldg(static_cast<const uint4*>(sc.attrs) + leaf);
}

// Lambert: ambient + diffuse*max(0, n.L) (ambient only in shadow).
__device__ __forceinline__ uint32_t shade(uint4 at, const SvoFrameArgs& a, bool shadowed) {
  const float ndl = __fadd_rn(__fadd_rn(__fmul_rn(__uint_as_float(at.y), a.light[0]),
                                        __fmul_rn(__uint_as_float(at.z), a.light[1])),
                              __fmul_rn(__uint_as_float(at.w), a.light[2]));
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

// `at` is the hit leaf's shading record (zero for a miss): its normal goes to
// the optional per-pixel normal output.
__device__ __forceinline__ void write_pixel(const SvoFrameArgs& a, uint32_t off, uint32_t rgba,
                                            uint32_t hitw, float ht, uint32_t f, uint32_t fs,
                                            uint4 at = make_uint4(0u, 0u, 0u, 0u)) {
  if (a.rgba) a.rgba[off] = rgba;
  if (a.hit) a.hit[off] = hitw;
  if (a.hit_t) a.hit_t[off] = ht;
  if (a.fetches) a.fetches[off] = f;
  if (a.shadow_fetches) a.shadow_fetches[off] = fs;
  if (a.normal) {
    const size_t n = 3u * (size_t)off;  // off < 2^31: 3 off needs 64 bits
    a.normal[n] = __uint_as_float(at.y);
    a.normal[n + 1u] = __uint_as_float(at.z);
    a.normal[n + 2u] = __uint_as_float(at.w);
  }
}

// kMinBlocks: resident 256-thread blocks per SM the register allocation is
// sized for (the occupancy / register-spill trade-off is autotuned).
// kRef: the node pool is the reference VoxNode layout (hit ids are then the
// pool's own node indices); otherwise the library's device layout.
// kRing: frames of the per-lane shared-memory ring (0: local memory only);
// kStaged: the first nsm node records are copied to shared memory and read
// there (measured: reading every record through L1 is as fast or faster,
// so the default is unstaged and nsm = 0).
// Dynamic shared memory = 32 B x nsm staged nodes + 1 KB x kRing per warp.
// kLod: level-of-detail cut-off (a.lod_coef, sc.node_data; library layout).
template <int kMinBlocks, bool kRef, int kRing, bool kStaged, bool kLod = false>
__global__ void __launch_bounds__(256, kMinBlocks)
    svo_frame_kernel(SvoDeviceScene sc, SvoFrameArgs a, uint32_t nsm, uint32_t refill_min) {
  extern __shared__ uint4 smem[];
  // the block's deadline under a frame budget (held in shared memory, not
  // in a register of the traversal)
  __shared__ unsigned long long deadline;
  if (!kStaged) nsm = 0;
  for (uint32_t i = threadIdx.x; i < 2 * nsm; i += blockDim.x) smem[i] = __ldg(sc.nodes + i);
  if (threadIdx.x == 0 && a.budget_us)
    deadline = global_timer_ns() + 1000ull * (unsigned long long)a.budget_us;
  __syncthreads();
  const uint32_t* smw = reinterpret_cast<const uint32_t*>(smem);
  uint4* ring = smem + 2 * nsm + (threadIdx.x >> 5) * (2 * kRing * 32) + (threadIdx.x & 31u);

  Frame stk[YV_MAX_DEPTH];
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t lt_mask = (1u << lane) - 1u;
  const uint32_t tiles_x = (uint32_t)((a.width + 7) >> 3);
  const uint32_t n_ids = a.id_end;
  uint32_t err = 0, my_hits = 0, my_shadowed = 0;

  uint32_t mode = kIdle, off = 0;
  Trace tr;
  float dx = 0.f, dy = 0.f, dz = 0.f;
  uint32_t hitw = 0xFFFFFFFFu, fp = 0;
  float ht = 0.f;
  uint4 attr = make_uint4(0u, 0u, 0u, 0u);

  for (;;) {
    // ---- refill idle lanes from the global ray counter ----
    const uint32_t idle = __ballot_sync(0xFFFFFFFFu, mode == kIdle);
    // past the frame budget: the idle lanes take no new rays (lane 0's
    // reading of the timer decides for the warp)
    if (idle && a.budget_us &&
        __shfl_sync(0xFFFFFFFFu, global_timer_ns() > deadline ? 1 : 0, 0)) {
      if (mode == kIdle) mode = kDone;
      if (lane == 0) err |= YV_DEV_ERR_TIMEOUT;
    } else if (idle) {
      const uint32_t leader = (uint32_t)__ffs(idle) - 1u;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(&a.counters[0], (uint32_t)__popc(idle));
      base = __shfl_sync(0xFFFFFFFFu, base, (int)leader);
      if (mode == kIdle) {
        const uint32_t id = a.id_begin + base + (uint32_t)__popc(idle & lt_mask);
        if (id >= n_ids) {
          mode = kDone;
        } else {
          const uint32_t tile = id >> 5, w = id & 31u;
          const int x = (int)((tile % tiles_x) * 8u + (w & 7u));
          const int y = (int)((tile / tiles_x) * 4u + (w >> 3));
          if (x < a.width && y < a.height) {
            off = (uint32_t)y * (uint32_t)a.width + (uint32_t)x;
            pixel_dir(a, x, y, dx, dy, dz);
            if (begin_trace(sc, a.pos[0], a.pos[1], a.pos[2], dx, dy, dz, tr, err)) {
              mode = kPrimary;
            } else {
              write_pixel(a, off, 0u, 0xFFFFFFFFu, 0.f, tr.fetches, 0u);
            }
          }
        }
      }
    }
    if (__all_sync(0xFFFFFFFFu, mode == kDone)) break;

    // ---- trace until refill_min lanes (or all) are free: up to kStepsPerVote
    // steps per warp vote, the end of a ray handled once after them (a lane
    // whose ray ended idles for the rest of the group) ----
    for (;;) {
      int r = kContinue;
      uint32_t leaf = 0;
#pragma unroll
      for (int k = 0; k < kStepsPerVote; ++k)
        if ((mode == kPrimary || mode == kShadow) && r == kContinue)
          r = trace_step<kRef, kRing, kStaged, kLod>(sc, smw, nsm, stk, ring, tr,
                                                     mode == kShadow, leaf, err, a.lod_coef);
      if (r != kContinue) {
        if (mode == kShadow) {
          // end of a shadow ray
          const bool sh = r == kHit;
          my_shadowed += sh ? 1u : 0u;
          write_pixel(a, off, shade(attr, a, sh), hitw, ht, fp, tr.fetches, attr);
          mode = kIdle;
        } else if (r == kMiss) {
          write_pixel(a, off, 0u, 0xFFFFFFFFu, 0.f, tr.fetches, 0u);
          mode = kIdle;
        } else {
          ++my_hits;
          hitw = ((kRef ? tr.node : __ldg(sc.orig_id + tr.node)) << 3) | (tr.ch ^ tr.df);
          ht = max3f(tr.t.x1, tr.t.y1, tr.t.z1);
          fp = tr.fetches;
          attr = make_uint4(0u, 0u, 0u, 0u);
          if (leaf < sc.n_attrs)
            attr = load_shading<kRef>(sc, leaf);
          else
            err |= YV_DEV_ERR_POOL;
          mode = kIdle;
          if (a.shadows) {
            // shadow ray: the hit point moved half a leaf out through the entry face
            float o[3];
            o[0] = __fadd_rn(a.pos[0], __fmul_rn(dx, ht));
            o[1] = __fadd_rn(a.pos[1], __fmul_rn(dy, ht));
            o[2] = __fadd_rn(a.pos[2], __fmul_rn(dz, ht));
            int e = 0;
            float m = tr.t.x1;
            if (tr.t.y1 > m) { e = 1; m = tr.t.y1; }
            if (tr.t.z1 > m) e = 2;
            const float half = __int_as_float((127 - (tr.level + 2)) << 23);
            const float d_off = ((tr.df >> e) & 1u) ? half : -half;
            o[e] = __fadd_rn(o[e], d_off);
            if (begin_trace(sc, o[0], o[1], o[2], a.light_ray[0], a.light_ray[1],
                            a.light_ray[2], tr, err))
              mode = kShadow;
            else
              write_pixel(a, off, shade(attr, a, false), hitw, ht, fp, tr.fetches, attr);
          } else {
            write_pixel(a, off, shade(attr, a, false), hitw, ht, fp, 0u, attr);
          }
        }
      }
      const uint32_t free_lanes = __ballot_sync(0xFFFFFFFFu, mode == kIdle || mode == kDone);
      if (free_lanes == 0xFFFFFFFFu || __popc(free_lanes) >= (int)refill_min) break;
    }
  }

  // block totals of the counters, one atomic per block and counter
  __shared__ uint32_t red[3];
  if (threadIdx.x < 3) red[threadIdx.x] = 0;
  __syncthreads();
  if (my_hits) atomicAdd(&red[0], my_hits);
  if (my_shadowed) atomicAdd(&red[1], my_shadowed);
  if (err) atomicOr(&red[2], err);
  __syncthreads();
  if (threadIdx.x == 0) {
    if (red[0]) atomicAdd(&a.counters[2], red[0]);
    if (red[1]) atomicAdd(&a.counters[3], red[1]);
    if (red[2]) atomicOr(&a.counters[1], red[2]);
  }
}

}  // namespace
}  // namespace yv
