// yv_kernels.h - launch interface between the host C ABI and the CUDA
// kernels.  Host-callable functions only; no device code here.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace yv {

// Device copy of an SVO scene (layout described in yv_internal.h).
struct SvoDeviceScene {
  const uint4* nodes = nullptr;       // 2 x uint4 (8 child words) per node
  const uint32_t* orig_id = nullptr;  // device index -> caller node id
  // library layout: 16-byte shading records {RGBA8, unit normal xyz fp32};
  // caller VoxNode pools: the caller's yv_leaf_attr (8 bytes)
  const void* attrs = nullptr;
  // level-of-detail attribute index of every node (device order), or null
  const uint32_t* node_data = nullptr;
  uint32_t n_nodes = 0;
  uint32_t n_attrs = 0;
  uint32_t root_word = 0x40000000u;
  // host-side: 1 = `nodes` / `attrs` are a caller VoxNode pool (40-byte
  // records, 8-byte attributes, pool ids as root and children)
  uint32_t ref_layout = 0;
};

// One frame of the SVO renderer.
struct SvoFrameArgs {
  float pos[3];
  float dir0[3], du[3], dv[3];   // RendererBase::InitRayDir basis
  float light[3];                // shading direction (toward the light)
  float light_ray[3];            // light direction after AdjustDir
  float ambient, diffuse;
  int shadows;
  int width, height;
  float lod_coef;                // > 0: stop at subtrees smaller than t * lod_coef
  uint32_t* rgba;                // optional outputs (device)
  uint32_t* hit;
  float* hit_t;
  uint32_t* fetches;
  uint32_t* shadow_fetches;
  float* normal;                 // 3 floats per pixel
  uint32_t* counters;            // device scratch, kSvoCounterWords words
  // ray ids [id_begin, id_end) of the frame to trace (32 per 8x4-pixel
  // tile, tiles row-major); the whole frame is [0, 32 * tiles)
  uint32_t id_begin, id_end;
  // frame time budget of the persistent queue in microseconds (0: none):
  // once it has elapsed since a block started, the block's warps take no
  // new rays and the frame reports YV_DEV_ERR_TIMEOUT
  uint32_t budget_us;
};

// Ray ids of a whole width x height frame (8x4-pixel tiles of 32 ids).
inline uint32_t frame_ray_ids(int width, int height) {
  return (uint32_t)((width + 7) / 8) * (uint32_t)((height + 3) / 4) * 32u;
}

// Scratch words a frame uses: [0] tile queue, [1] status bits, [2] hits,
// [3] shadowed hits.
constexpr int kSvoCounterWords = 8;

struct LaunchCfg {
  int block_threads = 256;
  int blocks_per_sm = 0;   // 0: occupancy-derived
  int smem_nodes = 0;      // top-of-tree records staged in shared memory
  int tile_rays = 32;
};

// Enqueues one frame (counter reset + persistent kernel) on `stream`.
cudaError_t launch_svo_frame(const SvoDeviceScene& sc, const SvoFrameArgs& a,
                             const LaunchCfg& cfg, cudaStream_t stream,
                             int* launches);

// Number of SMs of the current device (cached per device).
int device_sm_count();

// Stream-ordered scratch memory from a library-owned pool on the current
// device that keeps up to 4 GiB cached across synchronisations, so calls
// repeated every step (the adjoint's gradient scratch, scene builds) do not
// go back to the driver for memory each time.  The caller's default pool is
// left as it is.
cudaError_t scratch_alloc(void** p, size_t bytes, cudaStream_t s);
cudaError_t scratch_free(void* p, cudaStream_t s);

}  // namespace yv
