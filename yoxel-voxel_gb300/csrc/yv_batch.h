// yv_batch.h - device table of a batched persistent render (host side).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "yv_c_api.h"
#include "yv_kernels.h"
#include "yv_volume.h"

namespace yv {

constexpr int kMaxBatchItems = 64;

enum BatchKind : int32_t { kBatchSvo = 0, kBatchBrick = 1 };  // brick: any VolumeView precision

// One scene + camera of a batch.  Ray ids [id_base, id_base + 32*tiles) map
// to the item's 8x4 pixel tiles.
struct BatchItem {
  int32_t kind;
  int32_t width, height;
  uint32_t id_base;
  uint32_t tiles_x;
  uint32_t tiles;
  SvoDeviceScene svo;   // kind == kBatchSvo
  SvoFrameArgs fa;      //   camera basis, light, outputs
  VolumeView vol;       // brick kinds
  CamBasis vcam;
  float* frgba;         //   RGBA float output
};

struct BatchLaunch {
  const BatchItem* items;  // device table
  int nitems;
  uint32_t total_ids;
  uint32_t* counters;      // device scratch: [0] queue, [1] status
  int brick_precision;     // lattice format shared by every brick item, -1 if mixed
};

// Enqueues counter reset + the persistent batch kernel.
cudaError_t launch_batch(const BatchLaunch& b, const LaunchCfg& cfg, cudaStream_t s);

// Scene + frame parameters of a renderer (internal accessor of api.cpp).
struct yv_renderer_view {
  SvoDeviceScene sc;
  SvoFrameArgs fa;
  float fov_deg;
};
bool renderer_view(const yv_renderer* r, yv_renderer_view* v);

// Enqueues the renderer's frame unlit (ambient 1, diffuse 0, no shadow rays:
// rgba = the hit leaves' albedo) into `out`; counters as for any frame.
yv_status renderer_enqueue_unlit(yv_renderer* r, const yv_frame_outputs* out, cudaStream_t s);

}  // namespace yv
