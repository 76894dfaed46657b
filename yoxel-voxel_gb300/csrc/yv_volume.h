// yv_volume.h - launch interface of the brick-volume kernels (host side).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace yv {

constexpr int kMaxVolumeCams = 64;  // cameras per launch (kernel-parameter table)

// RendererBase::InitRayDir basis of one camera.
struct CamBasis {
  float pos[3];
  float dir0[3], du[3], dv[3];
};

// One volume as the march reads it.
struct VolumeView {
  // tree + pool (device pointers)
  const uint32_t* grids;
  uint32_t ngrids;
  int levels;
  int nb;                // brick cells per axis = 4^levels
  const void* density;   // precision 0: fp16, 1: fp32 (nbricks*729); 2, 3: unused
  const void* albedo;    // precision 0: uchar4, 1: fp32x3, 2: float4 (r,g,b,density),
                         // 3: uint2 {fp16 density | r<<16 | g<<24, b}
  uint32_t nbricks;
  int precision;
  // per brick 16 words: bit (y & 3) * 8 + x of word z * 2 + (y >> 2) set
  // where trilinear cell (x, y, z) has a non-zero density corner; null = none
  const uint32_t* cell_mask;
  // one bit per brick cell ((cz * nb + cy) * nb + cx), clear where the tree
  // holds no brick: an empty cell costs one load instead of a descent;
  // null = descend for every cell
  const uint32_t* brick_bits;
  // march
  float S;               // lattice cells per axis
  float cell_size;       // world size of a brick cell = 8/S
  float alpha_scale;
  float dt, inv_dt;      // world step and its inverse
};

struct VolumeArgs {
  VolumeView v;
  const int32_t* nbr_up;  // nbricks*7
  const int32_t* nbr_dn;  // nbricks*7
  // cameras
  int ncams, width, height;
  CamBasis cam[kMaxVolumeCams];
  // outputs / adjoint inputs
  float* rgba;            // ncams*h*w float4 (optional if rgba8 is set)
  uint32_t* rgba8;        // optional ncams*h*w RGBA8 (float2uint of trace.cu)
  uint32_t* samples;      // optional per-ray counters
  uint32_t* bricks_entered;
  const float* rgba_fwd;  // backward: forward output
  const float* grad_rgba; // backward: dL/d rgba
  float* grad_density;    // backward outputs (pool layout)
  float* grad_albedo;
  float4* grad_packed;    // backward scratch: (albedo rgb, density) per lattice point
  uint32_t* status;       // optional device status word
  // forward only: warp tiles [tile_begin, tile_end) of the launch (march
  // order, see tile_ids); tile_end = 0: all of them
  uint32_t tile_begin, tile_end;
};

cudaError_t launch_volume_forward(const VolumeArgs& a, cudaStream_t s);
// Warp tiles of one camera's width x height frame in the march's order:
// 16x16-pixel squares (row-major) of 8 tiles of 8x4 pixels.
uint32_t volume_tiles_per_camera(int width, int height);
cudaError_t launch_volume_backward(const VolumeArgs& a, cudaStream_t s);
// packed[i] = (albedo rgb, density) of n lattice points (fp32 layouts).
cudaError_t launch_pack_f32(const float* density, const float* albedo, uint32_t n,
                            float4* packed, cudaStream_t s);
// grad_density += packed.w, grad_albedo += packed.xyz (n lattice points).
cudaError_t launch_unpack_grads(const float4* packed, uint32_t n, float* grad_density,
                                float* grad_albedo, cudaStream_t s);
// gather=true: fold apron gradients into owners, then copy owners to aprons;
// gather=false: copy owners to aprons only (parameter sync).
cudaError_t launch_apron_fold(const VolumeArgs& a, int channels, float* g, bool gather,
                              cudaStream_t s);
int device_sm_count_vol();
// mask[b * 16 + w] for the nbricks bricks of v (cell_mask of VolumeView).
cudaError_t launch_cell_mask(const VolumeView& v, uint32_t* mask, cudaStream_t s);
// brick_bits of v's tree (ceil(nb^3 / 32) words).
cudaError_t launch_brick_bits(const VolumeView& v, uint32_t* bits, cudaStream_t s);

}  // namespace yv
