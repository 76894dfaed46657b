// api_batch.cpp - C ABI of the batched persistent render: many scenes and
// cameras (SVO first-hit and brick compositing) in one launch fed by a
// global ray queue, optionally replayed from a captured CUDA graph; and the
// per-scene launches it replaces.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "yv_batch.h"
#include "yv_internal.h"

using namespace yv;

struct yv_batch {
  int device = 0;
  std::vector<BatchItem> items;  // in insertion order
  std::vector<int> order;        // launch order (largest first)
  LaunchCfg cfg;
  LaunchCfg sep_cfg;
  // device scratch: item table, queue/status counters, per-item counters
  BatchItem* d_items = nullptr;
  uint32_t* d_counters = nullptr;
  uint32_t* d_sep = nullptr;
  size_t sep_cap = 0;
  uint32_t total_ids = 0;
  bool dirty = true;
  // captured graph of the persistent launch
  cudaStream_t cap_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool graph_valid = false;
};

namespace {

yv_status fail(cudaError_t e, const char* what) {
  set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
  cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? YV_ERR_OUT_OF_MEMORY : YV_ERR_CUDA;
}

void drop_graph(yv_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  b->graph_valid = false;
}

// Lays the items out in the ray-id space, largest estimated cost first
// (brick rays weigh 4 primary SVO rays), and uploads the table.
yv_status prepare(yv_batch* b) {
  if (!b->dirty) return YV_OK;
  const int n = (int)b->items.size();
  std::vector<double> cost((size_t)n);
  for (int i = 0; i < n; ++i) {
    const BatchItem& it = b->items[(size_t)i];
    double px = (double)it.width * it.height;
    cost[(size_t)i] = it.kind == kBatchSvo ? px * (it.fa.shadows ? 2.0 : 1.0) : 4.0 * px;
  }
  b->order.resize((size_t)n);
  for (int i = 0; i < n; ++i) b->order[(size_t)i] = i;
  std::stable_sort(b->order.begin(), b->order.end(),
                   [&](int x, int y) { return cost[(size_t)x] > cost[(size_t)y]; });
  std::vector<BatchItem> table((size_t)n);
  uint64_t base = 0;
  for (int i = 0; i < n; ++i) {
    BatchItem it = b->items[(size_t)b->order[(size_t)i]];
    it.id_base = (uint32_t)base;
    base += (uint64_t)it.tiles * 32u;
    table[(size_t)i] = it;
  }
  // 32-bit ray ids with room above for the queue counter's overshoot (every
  // warp adds 32 past the end once), so the counter never wraps
  if (base > 0x7FFFFFFFull) {
    set_last_error("batch has more than 2^31 rays");
    return YV_ERR_INVALID_ARG;
  }
  b->total_ids = (uint32_t)base;
  cudaError_t e = cudaSuccess;
  if (!b->d_items) e = cudaMalloc(&b->d_items, sizeof(BatchItem) * kMaxBatchItems);
  if (e == cudaSuccess && !b->d_counters) e = cudaMalloc(&b->d_counters, 64);
  if (e == cudaSuccess && n)
    e = cudaMemcpy(b->d_items, table.data(), sizeof(BatchItem) * (size_t)n,
                   cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return fail(e, "batch table upload");
  drop_graph(b);
  b->dirty = false;
  return YV_OK;
}

BatchLaunch launch_desc(const yv_batch* b) {
  BatchLaunch l;
  l.items = b->d_items;
  l.nitems = (int)b->items.size();
  l.total_ids = b->total_ids;
  l.counters = b->d_counters;
  // the batch kernel is compiled per brick lattice format: a batch whose
  // volumes share one (or that has none) runs the kernel carrying only that
  // march
  l.brick_precision = 3;
  bool first = true;
  for (const BatchItem& it : b->items) {
    if (it.kind != kBatchBrick) continue;
    if (first) l.brick_precision = it.vol.precision;
    else if (l.brick_precision != it.vol.precision) l.brick_precision = -1;
    first = false;
  }
  return l;
}

LaunchCfg to_cfg(const yv_launch_config* c) {
  LaunchCfg d;
  d.block_threads = c->block_threads > 0 ? c->block_threads : 256;
  d.blocks_per_sm = c->blocks_per_sm > 0 ? c->blocks_per_sm : 0;
  d.smem_nodes = c->smem_nodes >= 0 ? c->smem_nodes : LaunchCfg().smem_nodes;
  d.tile_rays = c->tile_rays > 0 ? c->tile_rays : 0;
  return d;
}

}  // namespace

extern "C" {

yv_status yv_batch_create(yv_batch** out) {
  if (!out) return YV_ERR_INVALID_ARG;
  *out = nullptr;
  yv_batch* b = new (std::nothrow) yv_batch();
  if (!b) return YV_ERR_OUT_OF_MEMORY;
  cudaError_t e = cudaGetDevice(&b->device);
  if (e != cudaSuccess) {
    delete b;
    return fail(e, "cudaGetDevice");
  }
  *out = b;
  return YV_OK;
}

void yv_batch_destroy(yv_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  cudaDeviceSynchronize();
  drop_graph(b);
  if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
  cudaFree(b->d_items);
  cudaFree(b->d_counters);
  cudaFree(b->d_sep);
  delete b;
}

yv_status yv_batch_clear(yv_batch* b) {
  if (!b) return YV_ERR_INVALID_ARG;
  b->items.clear();
  b->dirty = true;
  return YV_OK;
}

yv_status yv_batch_add_svo(yv_batch* b, const yv_renderer* r, void* d_rgba) {
  if (!b || !r || !d_rgba) return YV_ERR_INVALID_ARG;
  yv_frame_outputs o;
  std::memset(&o, 0, sizeof(o));
  o.rgba = d_rgba;
  return yv_batch_add_svo_outputs(b, r, &o);
}

yv_status yv_batch_add_svo_outputs(yv_batch* b, const yv_renderer* r,
                                   const yv_frame_outputs* out) {
  if (!b || !r || !out ||
      !(out->rgba || out->hit || out->hit_t || out->fetches || out->shadow_fetches ||
        out->normal))
    return YV_ERR_INVALID_ARG;
  if ((int)b->items.size() >= kMaxBatchItems) return YV_ERR_UNSUPPORTED;
  yv_renderer_view v;
  if (!renderer_view(r, &v)) return YV_ERR_NO_SCENE;
  if (v.sc.ref_layout) {
    set_last_error("yv_batch_add_svo: a renderer bound to an editable scene cannot be batched");
    return YV_ERR_UNSUPPORTED;
  }
  BatchItem it{};
  it.kind = kBatchSvo;
  it.width = v.fa.width;
  it.height = v.fa.height;
  it.tiles_x = (uint32_t)((it.width + 7) / 8);
  it.tiles = it.tiles_x * (uint32_t)((it.height + 3) / 4);
  it.svo = v.sc;
  it.fa = v.fa;
  it.fa.rgba = static_cast<uint32_t*>(out->rgba);
  it.fa.hit = static_cast<uint32_t*>(out->hit);
  it.fa.hit_t = static_cast<float*>(out->hit_t);
  it.fa.fetches = static_cast<uint32_t*>(out->fetches);
  it.fa.shadow_fetches = static_cast<uint32_t*>(out->shadow_fetches);
  it.fa.normal = static_cast<float*>(out->normal);
  b->items.push_back(it);
  b->dirty = true;
  return YV_OK;
}

yv_status yv_batch_add_volume(yv_batch* b, const yv_volume_device* vol, const yv_camera* cam,
                              int32_t width, int32_t height, const yv_march_params* mp,
                              float* d_rgba) {
  if (!b || !vol || !cam || !mp || !d_rgba || width <= 0 || height <= 0 || !vol->grids ||
      vol->levels < 1 || vol->levels > 5 || !(mp->step_vox > 0.f) ||
      !(cam->fov_deg > 0.f && cam->fov_deg < 180.f) || vol->precision < YV_PRECISION_F16 ||
      vol->precision > YV_PRECISION_F16_PACKED || (vol->nbricks && !vol->albedo) ||
      (vol->nbricks && vol->precision < YV_PRECISION_F32_PACKED && !vol->density))
    return YV_ERR_INVALID_ARG;
  if ((int)b->items.size() >= kMaxBatchItems) return YV_ERR_UNSUPPORTED;
  BatchItem it{};
  it.kind = kBatchBrick;
  it.width = width;
  it.height = height;
  it.tiles_x = (uint32_t)((width + 7) / 8);
  it.tiles = it.tiles_x * (uint32_t)((height + 3) / 4);
  VolumeView& v = it.vol;
  v.grids = vol->grids;
  v.ngrids = vol->ngrids;
  v.levels = vol->levels;
  v.nb = 1 << (2 * vol->levels);
  v.density = vol->density;
  v.albedo = vol->albedo;
  v.nbricks = vol->nbricks;
  v.precision = vol->precision;
  v.cell_mask = vol->cell_mask;
  v.brick_bits = vol->brick_bits;
  v.S = (float)(8 * v.nb);
  v.cell_size = 8.0f / v.S;
  v.alpha_scale = mp->alpha_scale;
  v.dt = mp->step_vox / v.S;
  v.inv_dt = v.S / mp->step_vox;
  std::memcpy(it.vcam.pos, cam->pos, sizeof(it.vcam.pos));
  init_ray_dir(cam->dir, cam->up, cam->fov_deg, width, height, it.vcam.dir0, it.vcam.du,
               it.vcam.dv);
  it.frgba = d_rgba;
  b->items.push_back(it);
  b->dirty = true;
  return YV_OK;
}

yv_status yv_batch_set_launch_config(yv_batch* b, const yv_launch_config* cfg) {
  if (!b || !cfg || (cfg->block_threads > 0 && (cfg->block_threads > 256 ||
                                                (cfg->block_threads & 31))))
    return YV_ERR_INVALID_ARG;
  b->cfg = to_cfg(cfg);
  drop_graph(b);
  return YV_OK;
}

yv_status yv_batch_render(yv_batch* b, int32_t use_graph, void* stream) {
  if (!b) return YV_ERR_INVALID_ARG;
  cudaError_t e = cudaSetDevice(b->device);
  if (e != cudaSuccess) return fail(e, "cudaSetDevice");
  yv_status st = prepare(b);
  if (st != YV_OK) return st;
  if (b->items.empty()) return YV_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!use_graph) {
    e = launch_batch(launch_desc(b), b->cfg, s);
    return e == cudaSuccess ? YV_OK : fail(e, "batch launch");
  }
  if (!b->graph_valid) {
    if (!b->cap_stream) {
      e = cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking);
      if (e != cudaSuccess) return fail(e, "capture stream");
    }
    e = cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      cudaError_t le = launch_batch(launch_desc(b), b->cfg, b->cap_stream);
      e = cudaStreamEndCapture(b->cap_stream, &b->graph);
      if (le != cudaSuccess) e = le;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
    if (e != cudaSuccess) {
      drop_graph(b);
      return fail(e, "batch graph capture");
    }
    b->graph_valid = true;
  }
  e = cudaGraphLaunch(b->exec, s);
  return e == cudaSuccess ? YV_OK : fail(e, "batch graph launch");
}

yv_status yv_batch_render_separate(yv_batch* b, void* stream) {
  if (!b) return YV_ERR_INVALID_ARG;
  cudaError_t e = cudaSetDevice(b->device);
  if (e != cudaSuccess) return fail(e, "cudaSetDevice");
  const size_t n = b->items.size();
  if (b->sep_cap < n) {
    cudaFree(b->d_sep);
    b->d_sep = nullptr;
    b->sep_cap = 0;
    e = cudaMalloc(&b->d_sep, n * kSvoCounterWords * sizeof(uint32_t));
    if (e != cudaSuccess) return fail(e, "cudaMalloc(per-scene counters)");
    b->sep_cap = n;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  VolumeArgs* va = new (std::nothrow) VolumeArgs;
  if (!va) return YV_ERR_OUT_OF_MEMORY;
  for (size_t i = 0; i < n && e == cudaSuccess; ++i) {
    const BatchItem& it = b->items[i];
    if (it.kind == kBatchSvo) {
      SvoFrameArgs fa = it.fa;
      fa.counters = b->d_sep + i * kSvoCounterWords;
      e = launch_svo_frame(it.svo, fa, b->sep_cfg, s, nullptr);
    } else {
      std::memset(va, 0, sizeof(*va));
      va->v = it.vol;
      va->ncams = 1;
      va->width = it.width;
      va->height = it.height;
      va->cam[0] = it.vcam;
      va->rgba = it.frgba;
      e = launch_volume_forward(*va, s);
    }
  }
  delete va;
  return e == cudaSuccess ? YV_OK : fail(e, "per-scene launch");
}

yv_status yv_batch_info(const yv_batch* b, uint32_t* n_items, uint64_t* rays) {
  if (!b || !n_items || !rays) return YV_ERR_INVALID_ARG;
  *n_items = (uint32_t)b->items.size();
  uint64_t r = 0;
  for (const BatchItem& it : b->items) r += (uint64_t)it.width * (uint64_t)it.height;
  *rays = r;
  return YV_OK;
}

}  // extern "C"
