// batch_kernels.cu - batched persistent render: many scenes and cameras of
// uneven depth and resolution (SVO first-hit and brick compositing) traced in
// ONE launch from a global ray queue.
//
// Nearest reference structure: the SPU tile loop, where every SPE walks
// 16x16 tiles with a static stride (cell/spu/trace_spu.cpp:162-177); here the
// stride is replaced by a dynamic queue over the tiles of all scenes, so
// small frames no longer leave the GPU idle between per-scene launches and
// the tail of one scene overlaps the next.  Scenes are ordered by estimated
// cost (largest first) in the ray-id space.
//
// A warp pops 32 consecutive ray ids (one 8x4 tile of one scene, item
// boundaries are tile aligned); SVO lanes then run the per-lane traversal
// state machine of svo_trace.cuh, brick lanes the march of brick_march.cuh.
// Per-ray arithmetic is exactly that of the single-scene kernels, so results
// are bit-identical to per-scene launches.
#include "brick_march.cuh"
#include "svo_trace.cuh"
#include "yv_batch.h"

namespace yv {
namespace {

// Dynamic shared memory: the item table (the batch's own items only, so a
// small batch leaves more of the SM's memory to L1), then the per-lane frame
// ring of the SVO traversal, 1 KB x kBatchRing per warp.
constexpr int kBatchRing = 4;

__host__ __device__ __forceinline__ uint32_t item_table_vec4(int nitems) {
  return (uint32_t)(((size_t)nitems * sizeof(BatchItem) + 15u) / 16u);
}

// kP: the lattice format of every brick item (its march alone is compiled
// in), or -1 for a batch mixing formats (all four marches).
template <int kMinBlocks, int kP>
__global__ void __launch_bounds__(256, kMinBlocks) batch_kernel(BatchLaunch b) {
  extern __shared__ uint4 dyn_smem[];
  BatchItem* items = reinterpret_cast<BatchItem*>(dyn_smem);
  uint4* ring_smem = dyn_smem + item_table_vec4(b.nitems);
  {
    const uint32_t words = (uint32_t)(b.nitems * (int)sizeof(BatchItem) / 4);
    const uint32_t* src = reinterpret_cast<const uint32_t*>(b.items);
    uint32_t* dst = reinterpret_cast<uint32_t*>(items);
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) dst[i] = __ldg(src + i);
  }
  __syncthreads();

  Frame stk[YV_MAX_DEPTH];
  uint4* ring = ring_smem + (threadIdx.x >> 5) * (2 * kBatchRing * 32) + (threadIdx.x & 31u);
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t err = 0;
  uint32_t mode = kIdle, off = 0;
  int item = 0;
  Trace tr;
  float dx = 0.f, dy = 0.f, dz = 0.f;
  uint32_t hitw = 0xFFFFFFFFu, fp = 0;
  float ht = 0.f;
  uint4 attr = make_uint4(0u, 0u, 0u, 0u);

  for (;;) {
    const uint32_t busy = __ballot_sync(0xFFFFFFFFu, mode == kPrimary || mode == kShadow);
    if (busy == 0) {
      // Every lane is idle: the SVO state of its last ray is dead.  Saying
      // so keeps it out of the registers while a brick tile is marched.
      tr = Trace{};
      dx = dy = dz = 0.f;
      hitw = 0xFFFFFFFFu;
      fp = 0;
      ht = 0.f;
      attr = make_uint4(0u, 0u, 0u, 0u);
      // the whole warp takes the next 8x4 tile of the queue
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(&b.counters[0], 32u);
      base = __shfl_sync(0xFFFFFFFFu, base, 0);
      if (base >= b.total_ids) break;
      int k = 0;
      while (k + 1 < b.nitems && items[k + 1].id_base <= base) ++k;
      item = k;
      const BatchItem& it = items[k];
      const uint32_t tile = (base - it.id_base) >> 5;
      const int x = (int)((tile % it.tiles_x) * 8u + (lane & 7u));
      const int y = (int)((tile / it.tiles_x) * 4u + (lane >> 3));
      if (x < it.width && y < it.height) {
        off = (uint32_t)y * (uint32_t)it.width + (uint32_t)x;
        if (it.kind == kBatchSvo) {
          pixel_dir(it.fa, x, y, dx, dy, dz);
          if (begin_trace(it.svo, it.fa.pos[0], it.fa.pos[1], it.fa.pos[2], dx, dy, dz, tr,
                          err)) {
            mode = kPrimary;
          } else {
            write_pixel(it.fa, off, 0u, 0xFFFFFFFFu, 0.f, tr.fetches, 0u);
          }
        } else {
          float o[3], d[3];
          pixel_ray(it.vcam, x, y, o, d);
          NoVis nv;
          RayOut r;
          switch (kP >= 0 ? kP : it.vol.precision) {
            case 0: march<0>(it.vol, nullptr, 0u, o, d, nv, r); break;
            case 1: march<1>(it.vol, nullptr, 0u, o, d, nv, r); break;
            case 2: march<2>(it.vol, nullptr, 0u, o, d, nv, r); break;
            default: march<3>(it.vol, nullptr, 0u, o, d, nv, r); break;
          }
          if (r.bad) err |= YV_DEV_ERR_POOL;
          reinterpret_cast<float4*>(it.frgba)[off] = make_float4(r.c[0], r.c[1], r.c[2], r.a);
        }
      }
      continue;
    }

    // up to kStepsPerVote traversal steps, then the end of a ray once
    const BatchItem& it = items[item];
    int r = kContinue;
    uint32_t leaf = 0;
#pragma unroll
    for (int k = 0; k < kStepsPerVote; ++k)
      if ((mode == kPrimary || mode == kShadow) && r == kContinue)
        r = trace_step<false, kBatchRing>(it.svo, nullptr, 0u, stk, ring, tr, mode == kShadow,
                                          leaf, err);
    if (r == kContinue) continue;
    if (mode == kShadow) {
      write_pixel(it.fa, off, shade(attr, it.fa, r == kHit), hitw, ht, fp, tr.fetches, attr);
      mode = kIdle;
    } else if (r == kMiss) {
      write_pixel(it.fa, off, 0u, 0xFFFFFFFFu, 0.f, tr.fetches, 0u);
      mode = kIdle;
    } else {
      hitw = (__ldg(it.svo.orig_id + tr.node) << 3) | (tr.ch ^ tr.df);
      ht = max3f(tr.t.x1, tr.t.y1, tr.t.z1);
      fp = tr.fetches;
      attr = make_uint4(0u, 0u, 0u, 0u);
      if (leaf < it.svo.n_attrs)
        attr = load_shading<false>(it.svo, leaf);
      else
        err |= YV_DEV_ERR_POOL;
      mode = kIdle;
      if (!it.fa.shadows) {
        write_pixel(it.fa, off, shade(attr, it.fa, false), hitw, ht, fp, 0u, attr);
      } else {
        float o[3];
        o[0] = __fadd_rn(it.fa.pos[0], __fmul_rn(dx, ht));
        o[1] = __fadd_rn(it.fa.pos[1], __fmul_rn(dy, ht));
        o[2] = __fadd_rn(it.fa.pos[2], __fmul_rn(dz, ht));
        int e = 0;
        float m = tr.t.x1;
        if (tr.t.y1 > m) { e = 1; m = tr.t.y1; }
        if (tr.t.z1 > m) e = 2;
        const float half = __int_as_float((127 - (tr.level + 2)) << 23);
        const float d_off = ((tr.df >> e) & 1u) ? half : -half;
        o[e] = __fadd_rn(o[e], d_off);
        if (begin_trace(it.svo, o[0], o[1], o[2], it.fa.light_ray[0], it.fa.light_ray[1],
                        it.fa.light_ray[2], tr, err))
          mode = kShadow;
        else
          write_pixel(it.fa, off, shade(attr, it.fa, false), hitw, ht, fp, tr.fetches, attr);
      }
    }
  }
  if (err) atomicOr(&b.counters[1], err);
}

template <int kMinBlocks, int kP>
cudaError_t launch_batch_with(const BatchLaunch& b, int bt, cudaStream_t s) {
  auto kern = batch_kernel<kMinBlocks, kP>;
  const size_t smem =
      (size_t)item_table_vec4(b.nitems) * 16u + (size_t)(bt / 32) * kBatchRing * 1024u;
  static bool opted_in[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  cudaError_t e = cudaSuccess;
  if (!opted_in[dev]) {
    // room for the largest table and ring
    e = cudaFuncSetAttribute(
        kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
        (int)((size_t)item_table_vec4(kMaxBatchItems) * 16u + 8u * kBatchRing * 1024u));
    if (e != cudaSuccess) return e;
    opted_in[dev] = true;
  }
  int resident = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, kern, bt, smem);
  if (e != cudaSuccess) return e;
  if (resident <= 0) return cudaErrorInvalidConfiguration;
  e = cudaMemsetAsync(b.counters, 0, 2 * sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  kern<<<device_sm_count() * resident, bt, smem, s>>>(b);
  return cudaGetLastError();
}

template <int kP>
cudaError_t launch_by_budget(const BatchLaunch& b, int mb, int bt, cudaStream_t s) {
  if (mb <= 2) return launch_batch_with<2, kP>(b, bt, s);
  if (mb == 3) return launch_batch_with<3, kP>(b, bt, s);
  return launch_batch_with<4, kP>(b, bt, s);
}

}  // namespace

cudaError_t launch_batch(const BatchLaunch& b, const LaunchCfg& cfg, cudaStream_t s) {
  if (b.nitems <= 0) return cudaSuccess;
  int bt = cfg.block_threads;
  if (bt < 32 || bt > 256 || (bt & 31)) bt = 256;
  // register budget per blocks_per_sm: 2 (default), 3, 4
  const int mb = cfg.blocks_per_sm <= 0 ? 2 : (cfg.blocks_per_sm > 4 ? 4 : cfg.blocks_per_sm);
  switch (b.brick_precision) {
    case 0: return launch_by_budget<0>(b, mb, bt, s);
    case 1: return launch_by_budget<1>(b, mb, bt, s);
    case 2: return launch_by_budget<2>(b, mb, bt, s);
    case 3: return launch_by_budget<3>(b, mb, bt, s);
    default: return launch_by_budget<-1>(b, mb, bt, s);
  }
}

}  // namespace yv
