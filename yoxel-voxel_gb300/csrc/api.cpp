// api.cpp - C ABI of the SVO renderer: ISVORenderer (cell/svorenderer.h:5-31,
// cell/renderer_base.h:7-62) and the CUDA SVORenderer host
// (demo/SVORenderer.h:8-64, demo/SVORenderer.cpp:39-149), over the kernels of
// svo_kernels.cu.  No CUDA error aborts: every failure is a yv_status.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "yv_batch.h"
#include "yv_internal.h"
#include "yv_kernels.h"

using namespace yv;

struct yv_renderer {
  int device = 0;
  // camera (RendererBase defaults, cell/renderer_base.h:25; SVORenderer
  // view dir (1,0,0), demo/SVORenderer.cpp:9)
  float pos[3] = {0.f, 0.f, 0.f};
  float dir[3] = {1.f, 0.f, 0.f};
  float up[3] = {0.f, 0.f, 1.f};
  float fov = 70.f;
  int width = 640, height = 480;
  yv_light light;
  LaunchCfg cfg;
  // device scene
  uint32_t* d_words = nullptr;
  uint32_t* d_orig = nullptr;
  uint4* d_attrs = nullptr;  // shading records, 16 B per leaf
  uint32_t* d_node_data = nullptr;  // level-of-detail attribute per node, or null
  size_t cap_nodes = 0, cap_attrs = 0;  // allocated records of the three
  float detail = 0.f;  // SVORenderer::m_detailCoef; 0 = exact leaves
  uint32_t budget_us = 0;  // frame time budget of the plain frames; 0 = none
  // SVORenderer::SetScene(DynamicSVO*): a non-owned editable scene whose
  // device mirror (as of its last sync) is traced in place
  const yv_svo_dynamic* dyn = nullptr;
  SvoDeviceScene scene;
  bool has_scene = false;
  uint64_t scene_bytes = 0;
  // renderer-owned frame buffer (RendererBase::m_colorBuf) and scratch
  uint32_t* d_rgba = nullptr;
  size_t rgba_cap = 0;
  uint32_t* d_counters = nullptr;
  uint32_t* h_counters = nullptr;  // pinned copy of the counters (yv_render_frame)
  cudaStream_t last_stream = nullptr;
  uint64_t last_pixels = 0;
  int last_shadows = 0;
  uint32_t last_launches = 0;
  bool frame_pending = false;
};

static yv_status cuda_fail(cudaError_t e, const char* what) {
  set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
  cudaGetLastError();  // clear the non-sticky error
  return e == cudaErrorMemoryAllocation ? YV_ERR_OUT_OF_MEMORY : YV_ERR_CUDA;
}

#define YV_CUDA(call, what)                          \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

static void free_scene(yv_renderer* r) {
  cudaFree(r->d_words);
  cudaFree(r->d_orig);
  cudaFree(r->d_attrs);
  cudaFree(r->d_node_data);
  r->d_words = nullptr;
  r->d_orig = nullptr;
  r->d_attrs = nullptr;
  r->d_node_data = nullptr;
  r->cap_nodes = r->cap_attrs = 0;
  r->has_scene = false;
  r->scene = SvoDeviceScene();
  r->scene_bytes = 0;
  r->dyn = nullptr;
}

// The scene the kernels see: the renderer's own device copy, or the
// current synced state of a bound editable scene.
static SvoDeviceScene scene_of(const yv_renderer* r) {
  if (!r->dyn) return r->scene;
  const yv_vox_node* nodes = nullptr;
  const yv_leaf_attr* attrs = nullptr;
  uint32_t count = 0, root = YV_EMPTY_NODE, nattrs = 0;
  yv_svo_dynamic_device(r->dyn, &nodes, &count, &root, &attrs, &nattrs);
  SvoDeviceScene sc;
  sc.nodes = reinterpret_cast<const uint4*>(nodes);
  sc.attrs = attrs;
  sc.n_nodes = count;
  sc.n_attrs = nattrs;
  sc.root_word = (root & 0x80000000u) || !nodes ? YV_DW_NULL : root;
  sc.ref_layout = 1;
  return sc;
}

namespace yv {

// Scene buffers for a scene built on the device: waits for the renderer's
// last frame, drops the current scene and returns buffers for nn node
// records (8 child words + id each) and na shading records, reusing the
// existing allocations when they are large enough.
yv_status renderer_scene_buffers(yv_renderer* r, uint32_t nn, uint32_t na, uint32_t** words,
                                 uint32_t** orig, void** attrs) {
  YV_CUDA(cudaSetDevice(r->device), "cudaSetDevice");
  if (r->frame_pending) cudaStreamSynchronize(r->last_stream);
  r->has_scene = false;
  r->scene = SvoDeviceScene();
  r->dyn = nullptr;
  cudaFree(r->d_node_data);
  r->d_node_data = nullptr;
  const size_t want_n = nn ? nn : 1, want_a = na ? na : 1;
  if (want_n > r->cap_nodes) {
    cudaFree(r->d_words);
    cudaFree(r->d_orig);
    r->d_words = r->d_orig = nullptr;
    r->cap_nodes = 0;
    YV_CUDA(cudaMalloc(&r->d_words, want_n * 32u), "cudaMalloc(nodes)");
    YV_CUDA(cudaMalloc(&r->d_orig, want_n * 4u), "cudaMalloc(ids)");
    r->cap_nodes = want_n;
  }
  if (want_a > r->cap_attrs) {
    cudaFree(r->d_attrs);
    r->d_attrs = nullptr;
    r->cap_attrs = 0;
    YV_CUDA(cudaMalloc(&r->d_attrs, want_a * 16u), "cudaMalloc(attrs)");
    r->cap_attrs = want_a;
  }
  *words = r->d_words;
  *orig = r->d_orig;
  *attrs = r->d_attrs;
  return YV_OK;
}

// Makes the buffers filled after renderer_scene_buffers the current scene.
void renderer_commit_scene(yv_renderer* r, uint32_t nn, uint32_t na, uint32_t root_word) {
  r->scene.nodes = reinterpret_cast<const uint4*>(r->d_words);
  r->scene.orig_id = r->d_orig;
  r->scene.attrs = r->d_attrs;
  r->scene.n_nodes = nn;
  r->scene.n_attrs = na;
  r->scene.root_word = root_word;
  r->scene_bytes = (uint64_t)nn * 36u + (uint64_t)na * 16u;
  r->has_scene = true;
}

}  // namespace yv

extern "C" {

const char* yv_status_string(yv_status s) {
  switch (s) {
    case YV_OK: return "ok";
    case YV_ERR_INVALID_ARG: return "invalid argument";
    case YV_ERR_NO_SCENE: return "no scene set";
    case YV_ERR_BAD_POOL: return "malformed node or brick pool";
    case YV_ERR_ITERATION_CAP: return "ray iteration cap reached";
    case YV_ERR_TIMEOUT: return "frame time budget ran out";
    case YV_ERR_CUDA: return "CUDA runtime error";
    case YV_ERR_OUT_OF_MEMORY: return "out of memory";
    case YV_ERR_IO: return "file I/O error";
    case YV_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
  }
}

yv_status yv_renderer_create(yv_renderer** out) {
  if (!out) return YV_ERR_INVALID_ARG;
  *out = nullptr;
  yv_renderer* r = new (std::nothrow) yv_renderer();
  if (!r) return YV_ERR_OUT_OF_MEMORY;
  cudaError_t e = cudaGetDevice(&r->device);
  if (e != cudaSuccess) {
    delete r;
    return cuda_fail(e, "cudaGetDevice");
  }
  e = cudaMalloc(&r->d_counters, kSvoCounterWords * sizeof(uint32_t));
  if (e != cudaSuccess) {
    delete r;
    return cuda_fail(e, "cudaMalloc(counters)");
  }
  cudaMemset(r->d_counters, 0, kSvoCounterWords * sizeof(uint32_t));
  // default light: the configs' directional light normalize(0.3, 0.5, 0.8)
  float l[3] = {0.3f, 0.5f, 0.8f};
  float n = std::sqrt((l[0] * l[0] + l[1] * l[1]) + l[2] * l[2]);
  for (int i = 0; i < 3; ++i) r->light.dir[i] = l[i] / n;
  r->light.ambient = 0.15f;
  r->light.diffuse = 0.85f;
  r->light.shadows = 0;
  *out = r;
  return YV_OK;
}

void yv_renderer_destroy(yv_renderer* r) {
  if (!r) return;
  cudaSetDevice(r->device);
  if (r->frame_pending) cudaStreamSynchronize(r->last_stream);
  free_scene(r);
  cudaFree(r->d_rgba);
  cudaFree(r->d_counters);
  cudaFreeHost(r->h_counters);
  delete r;
}

}  // extern "C"

// lod: every node's `data` is a level-of-detail attribute index, uploaded in
// device order for the level-of-detail cut-off.
static yv_status set_scene_impl(yv_renderer* r, const yv_vox_node* nodes, uint32_t count,
                                uint32_t root, const yv_leaf_attr* attrs, uint32_t nattrs,
                                bool lod) {
  if (!r || (count && !nodes) || (nattrs && !attrs)) return YV_ERR_INVALID_ARG;
  DeviceLayout dl;
  std::string why;
  yv_status st = build_device_layout(nodes, count, root, nattrs, &dl, &why);
  if (st != YV_OK) {
    set_last_error(why);
    return st;
  }
  std::vector<uint32_t> node_data;
  if (lod) {
    node_data.resize(dl.orig_id.size());
    for (size_t i = 0; i < node_data.size(); ++i) {
      node_data[i] = nodes[dl.orig_id[i]].data;
      if (node_data[i] >= nattrs) {
        set_last_error("level-of-detail attribute of node " + std::to_string(dl.orig_id[i]) +
                       " out of range");
        return YV_ERR_BAD_POOL;
      }
    }
  }
  YV_CUDA(cudaSetDevice(r->device), "cudaSetDevice");
  if (r->frame_pending) cudaStreamSynchronize(r->last_stream);
  free_scene(r);
  const size_t nn = dl.orig_id.size();
  if (nn) {
    YV_CUDA(cudaMalloc(&r->d_words, nn * 32u), "cudaMalloc(nodes)");
    YV_CUDA(cudaMalloc(&r->d_orig, nn * 4u), "cudaMalloc(orig)");
    YV_CUDA(cudaMemcpy(r->d_words, dl.words.data(), nn * 32u, cudaMemcpyHostToDevice),
            "upload nodes");
    YV_CUDA(cudaMemcpy(r->d_orig, dl.orig_id.data(), nn * 4u, cudaMemcpyHostToDevice),
            "upload ids");
  }
  if (nattrs) {
    // Per leaf: RGBA8 + the unit normal, normalised here once with the
    // same FP32 operations the shading of every hit would repeat.
    std::vector<uint32_t> rec((size_t)nattrs * 4u);
    for (uint32_t i = 0; i < nattrs; ++i) {
      const yv_leaf_attr& at = attrs[i];
      const float nx = (float)at.nx, ny = (float)at.ny, nz = (float)at.nz;
      const float len2 = nx * nx + ny * ny + nz * nz;
      float u[3] = {0.f, 0.f, 0.f};
      if (len2 > 0.f) {
        const float len = std::sqrt(len2);
        u[0] = nx / len;
        u[1] = ny / len;
        u[2] = nz / len;
      }
      uint32_t* q = &rec[(size_t)i * 4u];
      q[0] = (uint32_t)at.r | ((uint32_t)at.g << 8) | ((uint32_t)at.b << 16) |
             ((uint32_t)at.a << 24);
      std::memcpy(q + 1, u, 12);
    }
    YV_CUDA(cudaMalloc(&r->d_attrs, (size_t)nattrs * 16u), "cudaMalloc(attrs)");
    YV_CUDA(cudaMemcpy(r->d_attrs, rec.data(), (size_t)nattrs * 16u, cudaMemcpyHostToDevice),
            "upload attrs");
  }
  r->cap_nodes = nn;
  r->cap_attrs = nattrs;
  r->scene.nodes = reinterpret_cast<const uint4*>(r->d_words);
  r->scene.orig_id = r->d_orig;
  r->scene.attrs = r->d_attrs;
  r->scene.n_nodes = (uint32_t)nn;
  r->scene.n_attrs = nattrs;
  r->scene.root_word = dl.root_word;
  r->scene_bytes = (uint64_t)nn * 36u + (uint64_t)nattrs * 16u;
  if (lod && nn) {
    YV_CUDA(cudaMalloc(&r->d_node_data, nn * 4u), "cudaMalloc(node data)");
    YV_CUDA(cudaMemcpy(r->d_node_data, node_data.data(), nn * 4u, cudaMemcpyHostToDevice),
            "upload node data");
    r->scene.node_data = r->d_node_data;
    r->scene_bytes += (uint64_t)nn * 4u;
  }
  r->has_scene = true;
  return YV_OK;
}

extern "C" {

yv_status yv_set_scene_svo(yv_renderer* r, const yv_vox_node* nodes,
                           uint32_t count, uint32_t root,
                           const yv_leaf_attr* attrs, uint32_t nattrs) {
  return set_scene_impl(r, nodes, count, root, attrs, nattrs, false);
}

yv_status yv_set_scene_svo_packed(yv_renderer* r, const yv_vox_node* nodes, uint32_t count,
                                  uint32_t root) {
  if (!r) return YV_ERR_INVALID_ARG;
  yv_svo_host* h = nullptr;
  yv_status st = yv_svo_from_packed(&h, nodes, count, root);
  if (st != YV_OK) return st;
  st = yv_set_scene_host(r, h);
  yv_svo_free(h);
  return st;
}

yv_status yv_set_scene_host(yv_renderer* r, const yv_svo_host* svo) {
  if (!r || !svo) return YV_ERR_INVALID_ARG;
  return set_scene_impl(r, yv_svo_nodes(svo), yv_svo_node_count(svo), yv_svo_root(svo),
                        yv_svo_attrs(svo), yv_svo_attr_count(svo), yv_svo_has_lod(svo) != 0);
}

yv_status yv_set_detail_coef(yv_renderer* r, float coef) {
  if (!r || !std::isfinite(coef) || coef < 0.f) return YV_ERR_INVALID_ARG;
  r->detail = coef;
  return YV_OK;
}

yv_status yv_set_frame_budget(yv_renderer* r, uint32_t microseconds) {
  if (!r) return YV_ERR_INVALID_ARG;
  r->budget_us = microseconds;
  return YV_OK;
}

yv_status yv_get_frame_budget(const yv_renderer* r, uint32_t* microseconds) {
  if (!r || !microseconds) return YV_ERR_INVALID_ARG;
  *microseconds = r->budget_us;
  return YV_OK;
}

yv_status yv_get_detail_coef(const yv_renderer* r, float* coef) {
  if (!r || !coef) return YV_ERR_INVALID_ARG;
  *coef = r->detail;
  return YV_OK;
}

yv_status yv_set_scene_dynamic(yv_renderer* r, const yv_svo_dynamic* s) {
  if (!r || !s) return YV_ERR_INVALID_ARG;
  YV_CUDA(cudaSetDevice(r->device), "cudaSetDevice");
  if (r->frame_pending) cudaStreamSynchronize(r->last_stream);
  free_scene(r);
  r->dyn = s;
  r->has_scene = true;
  return YV_OK;
}

yv_status yv_load_scene_vox(yv_renderer* r, const char* path) {
  if (!r || !path) return YV_ERR_INVALID_ARG;
  yv_svo_host* h = nullptr;
  yv_status st = yv_svo_load_vox(&h, path);
  if (st != YV_OK) return st;
  st = yv_set_scene_host(r, h);
  yv_svo_free(h);
  return st;
}

static bool finite3(const float* v) {
  return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]);
}

yv_status yv_set_view_pos(yv_renderer* r, const float pos[3]) {
  if (!r || !pos || !finite3(pos)) return YV_ERR_INVALID_ARG;
  std::memcpy(r->pos, pos, sizeof(r->pos));
  return YV_OK;
}
yv_status yv_set_view_dir(yv_renderer* r, const float dir[3]) {
  if (!r || !dir || !finite3(dir) || (dir[0] == 0 && dir[1] == 0 && dir[2] == 0))
    return YV_ERR_INVALID_ARG;
  std::memcpy(r->dir, dir, sizeof(r->dir));
  return YV_OK;
}
yv_status yv_set_view_up(yv_renderer* r, const float up[3]) {
  if (!r || !up || !finite3(up)) return YV_ERR_INVALID_ARG;
  std::memcpy(r->up, up, sizeof(r->up));
  return YV_OK;
}
yv_status yv_set_resolution(yv_renderer* r, int width, int height) {
  // the frame kernel numbers rays in 8x4-pixel tiles with 32-bit ids: the
  // padded ray count stays below 2^31
  if (!r || width <= 0 || height <= 0 ||
      (uint64_t)((width + 7) / 8) * (uint64_t)((height + 3) / 4) * 32u > 0x7FFFFFFFull) {
    set_last_error("yv_set_resolution: frame of more than 2^31 rays in 8x4 tiles");
    return YV_ERR_INVALID_ARG;
  }
  r->width = width;
  r->height = height;
  return YV_OK;
}
yv_status yv_get_resolution(const yv_renderer* r, int* width, int* height) {
  if (!r || !width || !height) return YV_ERR_INVALID_ARG;
  *width = r->width;
  *height = r->height;
  return YV_OK;
}
yv_status yv_set_fov(yv_renderer* r, float fov_deg) {
  if (!r || !(fov_deg > 0.f && fov_deg < 180.f)) return YV_ERR_INVALID_ARG;
  r->fov = fov_deg;
  return YV_OK;
}
yv_status yv_get_fov(const yv_renderer* r, float* fov_deg) {
  if (!r || !fov_deg) return YV_ERR_INVALID_ARG;
  *fov_deg = r->fov;
  return YV_OK;
}
yv_status yv_set_light(yv_renderer* r, const yv_light* light) {
  if (!r || !light || !finite3(light->dir)) return YV_ERR_INVALID_ARG;
  r->light = *light;
  return YV_OK;
}
yv_status yv_set_launch_config(yv_renderer* r, const yv_launch_config* c) {
  if (!r || !c) return YV_ERR_INVALID_ARG;
  LaunchCfg d;
  r->cfg.block_threads = c->block_threads > 0 ? c->block_threads : d.block_threads;
  r->cfg.blocks_per_sm = c->blocks_per_sm > 0 ? c->blocks_per_sm : 0;
  r->cfg.smem_nodes = c->smem_nodes >= 0 ? c->smem_nodes : d.smem_nodes;
  r->cfg.tile_rays = c->tile_rays > 0 ? c->tile_rays : d.tile_rays;
  if (r->cfg.block_threads > 256 || (r->cfg.block_threads & 31)) return YV_ERR_INVALID_ARG;
  return YV_OK;
}
yv_status yv_get_launch_config(const yv_renderer* r, yv_launch_config* c) {
  if (!r || !c) return YV_ERR_INVALID_ARG;
  c->block_threads = r->cfg.block_threads;
  c->blocks_per_sm = r->cfg.blocks_per_sm;
  c->smem_nodes = r->cfg.smem_nodes;
  c->tile_rays = r->cfg.tile_rays;
  return YV_OK;
}

yv_status yv_get_ray_basis(const yv_renderer* r, float dir0[3], float du[3], float dv[3]) {
  if (!r || !dir0 || !du || !dv) return YV_ERR_INVALID_ARG;
  init_ray_dir(r->dir, r->up, r->fov, r->width, r->height, dir0, du, dv);
  return YV_OK;
}

yv_status yv_get_device_scene_info(const yv_renderer* r, uint64_t* nodes, uint64_t* bytes) {
  if (!r || !nodes || !bytes) return YV_ERR_INVALID_ARG;
  *nodes = scene_of(r).n_nodes;
  *bytes = r->scene_bytes;
  return YV_OK;
}

// Scene and frame parameters of a renderer as the kernels take them
// (outputs and counters left null).
static void fill_frame_args(const yv_renderer* r, SvoFrameArgs& a) {
  std::memset(&a, 0, sizeof(a));
  std::memcpy(a.pos, r->pos, sizeof(a.pos));
  init_ray_dir(r->dir, r->up, r->fov, r->width, r->height, a.dir0, a.du, a.dv);
  std::memcpy(a.light, r->light.dir, sizeof(a.light));
  std::memcpy(a.light_ray, r->light.dir, sizeof(a.light_ray));
  adjust_dir(a.light_ray);
  a.ambient = r->light.ambient;
  a.diffuse = r->light.diffuse;
  a.shadows = r->light.shadows ? 1 : 0;
  a.width = r->width;
  a.height = r->height;
  a.id_begin = 0;
  a.id_end = frame_ray_ids(r->width, r->height);
  // SVORenderer::Render: rp.detailCoef = m_detailCoef * (fov / 2 in
  // radians) / width (demo/SVORenderer.cpp:104), in double, rounded once
  a.lod_coef = (r->detail > 0.f && r->scene.node_data)
                   ? (float)((double)r->detail * (double)r->fov *
                             (3.14159265358979323846 / 360.0) / (double)r->width)
                   : 0.f;
}

}  // extern "C"

namespace yv {
bool renderer_view(const yv_renderer* r, yv_renderer_view* v) {
  if (!r) return false;
  v->sc = scene_of(r);
  fill_frame_args(r, v->fa);
  v->fov_deg = r->fov;
  return r->has_scene;
}
}  // namespace yv

extern "C" {

// Pixels of the frame inside 8x4 tiles [tb, te) (row-major tiles; edge
// tiles are clipped to the frame).
static uint64_t tile_range_pixels(int width, int height, uint32_t tb, uint32_t te) {
  const uint32_t tiles_x = (uint32_t)((width + 7) / 8);
  uint64_t n = 0;
  for (uint32_t t = tb; t < te; ++t) {
    const int x0 = (int)(t % tiles_x) * 8, y0 = (int)(t / tiles_x) * 4;
    n += (uint64_t)std::min(8, width - x0) * (uint64_t)std::min(4, height - y0);
  }
  return n;
}

// `unlit`: the light is replaced by ambient 1, diffuse 0 and no shadow rays,
// so rgba carries the hit leaves' albedo.  Tiles [tb, te) of the frame
// (te = UINT32_MAX: the whole frame).
static yv_status enqueue_frame(yv_renderer* r, const yv_frame_outputs* out, cudaStream_t s,
                               bool unlit = false, uint32_t tb = 0,
                               uint32_t te = 0xFFFFFFFFu) {
  if (!r->has_scene) return YV_ERR_NO_SCENE;
  SvoFrameArgs a;
  fill_frame_args(r, a);
  const uint32_t ntiles = a.id_end / 32u;
  if (te > ntiles) te = ntiles;
  if (tb > te) tb = te;
  a.id_begin = tb * 32u;
  a.id_end = te * 32u;
  if (unlit) {
    a.ambient = 1.0f;
    a.diffuse = 0.0f;
    a.shadows = 0;
  }
  a.rgba = static_cast<uint32_t*>(out->rgba);
  a.hit = static_cast<uint32_t*>(out->hit);
  a.hit_t = static_cast<float*>(out->hit_t);
  a.fetches = static_cast<uint32_t*>(out->fetches);
  a.shadow_fetches = static_cast<uint32_t*>(out->shadow_fetches);
  a.normal = static_cast<float*>(out->normal);
  a.counters = r->d_counters;
  if (!unlit) a.budget_us = r->budget_us;
  int launches = 0;
  YV_CUDA(launch_svo_frame(scene_of(r), a, r->cfg, s, &launches), "svo frame launch");
  r->last_stream = s;
  r->last_pixels = (tb == 0 && te == ntiles) ? (uint64_t)r->width * (uint64_t)r->height
                                             : tile_range_pixels(r->width, r->height, tb, te);
  r->last_shadows = a.shadows;
  r->last_launches = (uint32_t)launches;
  r->frame_pending = true;
  return YV_OK;
}

}  // extern "C"

namespace yv {
yv_status renderer_enqueue_unlit(yv_renderer* r, const yv_frame_outputs* out, cudaStream_t s) {
  if (!r || !out) return YV_ERR_INVALID_ARG;
  YV_CUDA(cudaSetDevice(r->device), "cudaSetDevice");
  return enqueue_frame(r, out, s, true);
}
}  // namespace yv

extern "C" {

yv_status yv_render_frame_async(yv_renderer* r, const yv_frame_outputs* out, void* stream) {
  if (!r || !out) return YV_ERR_INVALID_ARG;
  YV_CUDA(cudaSetDevice(r->device), "cudaSetDevice");
  return enqueue_frame(r, out, static_cast<cudaStream_t>(stream));
}

yv_status yv_render_frame_tiles(yv_renderer* r, uint32_t tile_begin, uint32_t tile_end,
                                const yv_frame_outputs* out, void* stream) {
  if (!r || !out || tile_begin > tile_end) return YV_ERR_INVALID_ARG;
  if (!r->has_scene) return YV_ERR_NO_SCENE;
  const uint32_t ntiles = frame_ray_ids(r->width, r->height) / 32u;
  if (tile_end > ntiles) return YV_ERR_INVALID_ARG;
  YV_CUDA(cudaSetDevice(r->device), "cudaSetDevice");
  return enqueue_frame(r, out, static_cast<cudaStream_t>(stream), false, tile_begin, tile_end);
}

yv_status yv_get_tile_count(const yv_renderer* r, uint32_t* tiles_x, uint32_t* tiles_y) {
  if (!r || !tiles_x || !tiles_y) return YV_ERR_INVALID_ARG;
  *tiles_x = (uint32_t)((r->width + 7) / 8);
  *tiles_y = (uint32_t)((r->height + 3) / 4);
  return YV_OK;
}

// Frame statistics from the counter words c of the last frame.
static yv_status stats_from_counters(yv_renderer* r, const uint32_t* c, yv_frame_stats* stats) {
  r->frame_pending = false;
  stats->primary_rays = r->last_pixels;
  stats->hits = c[2];
  stats->shadow_rays = r->last_shadows ? c[2] : 0;
  stats->shadowed = c[3];
  stats->launches = r->last_launches;
  yv_status st = YV_OK;
  if (c[1] & YV_DEV_ERR_POOL) st = YV_ERR_BAD_POOL;
  else if (c[1] & (YV_DEV_ERR_ITER | YV_DEV_ERR_DEPTH)) st = YV_ERR_ITERATION_CAP;
  else if (c[1] & YV_DEV_ERR_TIMEOUT) st = YV_ERR_TIMEOUT;
  stats->status = (uint32_t)st;
  return st;
}

yv_status yv_renderer_frame_stats(yv_renderer* r, yv_frame_stats* stats) {
  if (!r || !stats) return YV_ERR_INVALID_ARG;
  std::memset(stats, 0, sizeof(*stats));
  YV_CUDA(cudaSetDevice(r->device), "cudaSetDevice");
  uint32_t c[kSvoCounterWords];
  YV_CUDA(cudaStreamSynchronize(r->last_stream), "frame sync");
  YV_CUDA(cudaMemcpy(c, r->d_counters, sizeof(c), cudaMemcpyDeviceToHost), "read counters");
  return stats_from_counters(r, c, stats);
}

yv_status yv_render_frame(yv_renderer* r, uint32_t* host_rgba, void* device_rgba, void* stream) {
  if (!r) return YV_ERR_INVALID_ARG;
  if (!r->has_scene) return YV_ERR_NO_SCENE;
  YV_CUDA(cudaSetDevice(r->device), "cudaSetDevice");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  void* dst = device_rgba;
  const size_t px = (size_t)r->width * (size_t)r->height;
  if (!dst) {
    if (r->rgba_cap < px) {
      if (r->frame_pending) cudaStreamSynchronize(r->last_stream);
      cudaFree(r->d_rgba);
      r->d_rgba = nullptr;
      r->rgba_cap = 0;
      YV_CUDA(cudaMalloc(&r->d_rgba, px * 4u), "cudaMalloc(frame)");
      r->rgba_cap = px;
    }
    dst = r->d_rgba;
  }
  yv_frame_outputs o;
  std::memset(&o, 0, sizeof(o));
  o.rgba = dst;
  yv_status st = enqueue_frame(r, &o, s);
  if (st != YV_OK) return st;
  if (host_rgba)
    YV_CUDA(cudaMemcpyAsync(host_rgba, dst, px * 4u, cudaMemcpyDeviceToHost, s), "read frame");
  // the counters come back in the same stream as the frame: one wait
  if (!r->h_counters)
    YV_CUDA(cudaMallocHost(&r->h_counters, kSvoCounterWords * sizeof(uint32_t)),
            "cudaMallocHost(counters)");
  YV_CUDA(cudaMemcpyAsync(r->h_counters, r->d_counters, kSvoCounterWords * sizeof(uint32_t),
                          cudaMemcpyDeviceToHost, s),
          "read counters");
  YV_CUDA(cudaStreamSynchronize(s), "frame sync");
  yv_frame_stats stats;
  std::memset(&stats, 0, sizeof(stats));
  return stats_from_counters(r, r->h_counters, &stats);
}

}  // extern "C"
