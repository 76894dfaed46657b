// svo_kernels.cu - launcher of the sparse-voxel-octree frame kernel
// (device code in svo_trace.cuh) for the library's device node layout.
#include <atomic>
#include <mutex>

#include "svo_trace.cuh"

namespace yv {

int device_sm_count() {
  // entry points may run on several host threads: the cache is atomic (a
  // race only repeats the same attribute query)
  static std::atomic<int> cached[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
  int n = cached[dev].load(std::memory_order_relaxed);
  if (n == 0) {
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 1;
    cached[dev].store(n, std::memory_order_relaxed);
  }
  return n;
}

// Frames of the per-lane shared-memory stack ring.
constexpr int kSvoRing = 4;

cudaError_t scratch_alloc(void** p, size_t bytes, cudaStream_t s) {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaMallocAsync(p, bytes, s);
  cudaMemPool_t pool;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!pools[dev]) {
      cudaMemPoolProps props = {};
      props.allocType = cudaMemAllocationTypePinned;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = dev;
      e = cudaMemPoolCreate(&pools[dev], &props);
      if (e != cudaSuccess) {
        pools[dev] = nullptr;
        return e;
      }
      uint64_t keep = 4ull << 30;
      cudaMemPoolSetAttribute(pools[dev], cudaMemPoolAttrReleaseThreshold, &keep);
    }
    pool = pools[dev];
  }
  return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

cudaError_t scratch_free(void* p, cudaStream_t s) { return p ? cudaFreeAsync(p, s) : cudaSuccess; }

template <int kMinBlocks, bool kStaged, bool kLod = false, bool kRef = false>
static cudaError_t launch_with(const SvoDeviceScene& sc, const SvoFrameArgs& a, int bt,
                               uint32_t nsm, uint32_t refill, int per_sm, cudaStream_t stream) {
  auto kern = svo_frame_kernel<kMinBlocks, kRef, kSvoRing, kStaged, kLod>;
  const size_t smem = (size_t)nsm * 32u + (size_t)(bt / 32) * kSvoRing * 1024u;
  if (smem > 48u * 1024u) {
    static bool opted_in[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    if (!opted_in[dev]) {
      int optin = 0;
      cudaFuncAttributes fa;
      cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
      if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, kern);
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 optin - (int)fa.sharedSizeBytes);
      if (e != cudaSuccess) return e;
      opted_in[dev] = true;
    }
  }
  int resident = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, kern, bt, smem);
  if (e != cudaSuccess) return e;
  if (resident <= 0) return cudaErrorInvalidConfiguration;
  const int grid = device_sm_count() * (per_sm > 0 && per_sm < resident ? per_sm : resident);
  e = cudaMemsetAsync(a.counters, 0, kSvoCounterWords * sizeof(uint32_t), stream);
  if (e != cudaSuccess) return e;
  kern<<<grid, bt, smem, stream>>>(sc, a, nsm, refill);
  return cudaGetLastError();
}

cudaError_t launch_svo_frame(const SvoDeviceScene& sc, const SvoFrameArgs& a,
                             const LaunchCfg& cfg, cudaStream_t stream, int* launches) {
  int bt = cfg.block_threads;
  if (bt < 32 || bt > 256 || (bt & 31)) bt = 256;
  uint32_t nsm = (uint32_t)(cfg.smem_nodes < 0 ? 0 : cfg.smem_nodes);
  if (nsm > sc.n_nodes) nsm = sc.n_nodes;
  if (nsm > 4096) nsm = 4096;
  uint32_t refill = (uint32_t)(cfg.tile_rays <= 0 ? 32 : cfg.tile_rays);
  if (refill > 32) refill = 32;
  // register budget: blocks_per_sm 2 (up to 128 regs), 3 (80), 4 (64), 5
  // (51).  0 = by the frame's size: 5 (fastest on the 2048^3 frame with
  // unstaged node reads: 0.991 ms against 1.003 at 4 and 1.105 at 3; 6
  // blocks spill), fewer while the frame holds under two 8x4-pixel tiles
  // per resident warp, down to 3 (a warp takes a tile at a time, so a small
  // frame ends on the warps that took two: the 512^2 frame 0.108 ms at 5,
  // 0.104 at 4, 0.100 at 3)
  int mb = cfg.blocks_per_sm > 5 ? 5 : cfg.blocks_per_sm;
  if (mb <= 0) {
    const uint64_t tiles = (a.id_end - a.id_begin) / 32u;
    const uint64_t warps_per_block = (uint64_t)(bt / 32);
    mb = 5;
    while (mb > 3 && tiles < 2ull * (uint64_t)device_sm_count() * (uint64_t)mb * warps_per_block)
      --mb;
  }
  cudaError_t e;
  if (sc.ref_layout) {
    // a caller VoxNode pool (an editable scene's device mirror): checked
    // traversal, the default launch shape
    e = launch_with<3, false, false, true>(sc, a, bt, 0, refill, 0, stream);
  } else if (a.lod_coef > 0.f && sc.node_data) {
    // level-of-detail frames: one instantiation, the default launch shape
    e = launch_with<5, false, true>(sc, a, bt, 0, refill, 0, stream);
  } else if (nsm == 0) {
    if (mb <= 2)
      e = launch_with<2, false>(sc, a, bt, nsm, refill, 0, stream);
    else if (mb == 3)
      e = launch_with<3, false>(sc, a, bt, nsm, refill, 0, stream);
    else if (mb == 4)
      e = launch_with<4, false>(sc, a, bt, nsm, refill, 0, stream);
    else
      e = launch_with<5, false>(sc, a, bt, nsm, refill, 0, stream);
  } else {
    if (mb <= 2)
      e = launch_with<2, true>(sc, a, bt, nsm, refill, 0, stream);
    else if (mb == 3)
      e = launch_with<3, true>(sc, a, bt, nsm, refill, 0, stream);
    else if (mb == 4)
      e = launch_with<4, true>(sc, a, bt, nsm, refill, 0, stream);
    else
      e = launch_with<5, true>(sc, a, bt, nsm, refill, 0, stream);
  }
  if (launches) *launches = 1;
  return e;
}

}  // namespace yv
