/* yv_svo_renderer.hpp - C++ mirror of the reference's SVO renderer
 * interface over the C ABI of yv_c_api.h.  Header-only; link with
 * libyoxel.so.
 *
 *   SVOData        cell/svodata.h:22-55     (node pool + root, .vox loader)
 *   ISVORenderer   cell/svorenderer.h:5-24  (SetScene, SetViewPos/Dir/Up,
 *                                            SetResolution, GetResolution,
 *                                            SetFOV, RenderFrame)
 *   CreateSimpleRenderer / CreateThreadedRenderer  cell/svorenderer.h:26-27
 *   LightParams, SetSSNA / SetShowNormals / SetLigth, Render(d_dstBuf),
 *   DumpTraceData   demo/SVORenderer.h:8-64 (the point-light renderer with
 *                   screen-space normals; lights start disabled as the
 *                   SVORenderer constructor leaves them)
 *
 * Semantics kept from the reference: SetScene stores a non-owning pointer
 * (RendererBase::SetScene, cell/renderer_base.h:28; the pool is copied to
 * the device when the scene is set and again if the same object is set
 * again); RenderFrame returns NULL without a scene (cell/ppu_renderer.cpp:
 * 78-79) and otherwise a pointer to a renderer-owned RGBA8 buffer valid
 * until the next SetResolution or RenderFrame (cell/renderer_base.h:22,
 * 39-43).  Both factories return the GPU renderer: the reference's simple
 * and 4-thread CPU renderers differ only in how the pixel loop is split.
 * Nothing throws; Status() reports the yv_status of the last call. */
#pragma once

#include <cstdint>
#include <cstdio>
#include <memory>
#include <string>
#include <vector>

#include "yv_c_api.h"

namespace yv {

struct point_3f {
  float x, y, z;
  point_3f(float x_ = 0.f, float y_ = 0.f, float z_ = 0.f) : x(x_), y(y_), z(z_) {}
};

struct point_2i {
  int x, y;
  point_2i(int x_ = 0, int y_ = 0) : x(x_), y(y_) {}
};

/* RGBA8 pixel, red in the low byte (Color32). */
typedef uint32_t Color32;

/* VoxNodeId of an empty tree (EmptyNode, reaction/report/main.tex:54). */
const uint32_t kEmptyNode = 0x80000000u;

/* SVOData: a node pool and its root, owned (a yv_svo_host). */
class SVOData {
 public:
  SVOData() {}
  ~SVOData() { yv_svo_free(h_); }
  SVOData(const SVOData&) = delete;
  SVOData& operator=(const SVOData&) = delete;

  /* SVOData::Load (cell/svodata.h:31-50).  On failure the previous contents
   * are kept and the status is returned. */
  yv_status Load(const char* fn) {
    yv_svo_host* h = nullptr;
    const yv_status st = yv_svo_load_vox(&h, fn);
    if (st == YV_OK) Reset(h);
    return st;
  }
  /* Scene generators of the library (seeded, deterministic). */
  yv_status Spheres(int depth, int n, float rmin, float rmax, uint64_t seed) {
    yv_svo_host* h = nullptr;
    const yv_status st = yv_svo_gen_spheres(&h, depth, n, rmin, rmax, seed);
    if (st == YV_OK) Reset(h);
    return st;
  }
  yv_status Terrain(int depth, int cubes, int cube_min, int cube_max, uint64_t seed) {
    yv_svo_host* h = nullptr;
    const yv_status st = yv_svo_gen_terrain(&h, depth, cubes, cube_min, cube_max, seed);
    if (st == YV_OK) Reset(h);
    return st;
  }
  /* A copy of caller arrays (VoxNode pool + leaf attributes). */
  yv_status Assign(const yv_vox_node* nodes, uint32_t count, uint32_t root,
                   const yv_leaf_attr* attrs, uint32_t nattrs) {
    yv_svo_host* h = nullptr;
    const yv_status st = yv_svo_from_arrays(&h, nodes, count, root, attrs, nattrs);
    if (st == YV_OK) Reset(h);
    return st;
  }
  yv_status Save(const char* fn) const {
    return h_ ? yv_svo_save_vox(h_, fn) : YV_ERR_INVALID_ARG;
  }
  /* The node `data` of reaction/report/main.tex:61: mean colour and normal
   * of every subtree, for the renderer's level-of-detail cut-off. */
  yv_status BuildLOD() { return h_ ? yv_svo_build_lod(h_) : YV_ERR_INVALID_ARG; }

  uint32_t GetRoot() const { return h_ ? yv_svo_root(h_) : kEmptyNode; }
  uint32_t Size() const { return h_ ? yv_svo_node_count(h_) : 0u; }
  const yv_vox_node& operator[](uint32_t id) const { return yv_svo_nodes(h_)[id]; }
  const yv_svo_host* Handle() const { return h_; }

 private:
  void Reset(yv_svo_host* h) {
    yv_svo_free(h_);
    h_ = h;
  }
  yv_svo_host* h_ = nullptr;
};

/* ISVORenderer (cell/svorenderer.h:5-24). */
class ISVORenderer {
 protected:
  ISVORenderer() {}

 public:
  virtual ~ISVORenderer() {}
  virtual void SetScene(SVOData* svo) = 0;
  virtual void SetViewPos(const point_3f& pos) = 0;
  virtual void SetViewDir(const point_3f& dir) = 0;
  virtual void SetViewUp(const point_3f& up) = 0;
  virtual void SetResolution(int width, int height) = 0;
  virtual point_2i GetResolution() const = 0;
  virtual void SetFOV(float fov) = 0;
  virtual const Color32* RenderFrame() = 0;
};

/* The GB300 renderer behind ISVORenderer. */
/* LightParams as demo/Demo.cpp:141-147 fills it: attenuation
 * 1 / (c.x + c.y d + c.z d^2). */
struct LightParams {
  bool enabled = false;
  point_3f pos, diffuse, specular, attenuationCoefs;
};

class GPURenderer : public ISVORenderer {
 public:
  GPURenderer() { status_ = yv_renderer_create(&r_); }
  ~GPURenderer() override { yv_renderer_destroy(r_); }
  GPURenderer(const GPURenderer&) = delete;
  GPURenderer& operator=(const GPURenderer&) = delete;

  void SetScene(SVOData* svo) override {
    scene_ = svo;
    if (!r_) return;
    status_ = svo && svo->Handle() ? yv_set_scene_host(r_, svo->Handle()) : YV_OK;
    if (status_ != YV_OK) scene_ = nullptr;
  }
  void SetViewPos(const point_3f& p) override { Vec(yv_set_view_pos, p); }
  void SetViewDir(const point_3f& p) override { Vec(yv_set_view_dir, p); }
  void SetViewUp(const point_3f& p) override { Vec(yv_set_view_up, p); }
  void SetResolution(int width, int height) override {
    if (!r_) return;
    status_ = yv_set_resolution(r_, width, height);
    if (status_ == YV_OK) buf_.assign((size_t)width * (size_t)height, 0u);
  }
  point_2i GetResolution() const override {
    int w = 0, h = 0;
    if (r_) yv_get_resolution(r_, &w, &h);
    return point_2i(w, h);
  }
  void SetFOV(float fov) override {
    if (r_) status_ = yv_set_fov(r_, fov);
  }
  /* demo/SVORenderer.h:22 */
  float GetFOV() const {
    float f = 0.f;
    if (r_) yv_get_fov(r_, &f);
    return f;
  }
  const Color32* RenderFrame() override {
    if (!r_ || !scene_ || !scene_->Handle()) {
      status_ = r_ ? YV_ERR_NO_SCENE : status_;
      return nullptr;
    }
    const point_2i res = GetResolution();
    buf_.resize((size_t)res.x * (size_t)res.y);
    status_ = yv_render_frame(r_, buf_.data(), nullptr, nullptr);
    return status_ == YV_OK ? buf_.data() : nullptr;
  }

  /* Beyond ISVORenderer: the light (the reference's SimpleShader light,
   * demo/Demo.cpp:141-147) and the status of the last call. */
  void SetLight(const point_3f& dir, float ambient, float diffuse, bool shadows) {
    if (!r_) return;
    yv_light l;
    l.dir[0] = dir.x;
    l.dir[1] = dir.y;
    l.dir[2] = dir.z;
    l.ambient = ambient;
    l.diffuse = diffuse;
    l.shadows = shadows ? 1 : 0;
    status_ = yv_set_light(r_, &l);
  }
  yv_status Status() const { return status_; }
  yv_renderer* Handle() const { return r_; }

  /* demo/SVORenderer.h:28-36: screen-space normals, normal display, the
   * point lights and a frame into a device RGBA8 buffer (async on the
   * default stream). */
  /* demo/SVORenderer.h:25-26 (0 = exact leaves, the default here). */
  void SetDetailCoef(float coef) {
    if (r_) status_ = yv_set_detail_coef(r_, coef);
  }
  float GetDetailCoef() const {
    float c = 0.f;
    if (r_) yv_get_detail_coef(r_, &c);
    return c;
  }
  /* Frame time budget of the ray queue (no reference counterpart; 0 = none):
   * a frame past it reports YV_ERR_TIMEOUT through Status(). */
  void SetFrameBudget(uint32_t microseconds) {
    if (r_) status_ = yv_set_frame_budget(r_, microseconds);
  }
  uint32_t GetFrameBudget() const {
    uint32_t us = 0;
    if (r_) yv_get_frame_budget(r_, &us);
    return us;
  }
  void SetSSNA(bool enable) { Ssna().ssna = enable ? 1 : 0; }
  bool GetSSNA() { return Ssna().ssna != 0; }
  void SetShowNormals(bool enable) { Ssna().show_normals = enable ? 1 : 0; }
  bool GetShowNormals() { return Ssna().show_normals != 0; }
  void SetLigth(int i, const LightParams& lp) {
    if (i < 0 || i >= YV_SSNA_MAX_LIGHTS) {
      status_ = YV_ERR_INVALID_ARG;
      return;
    }
    yv_point_light& l = Ssna().lights[i];
    l.enabled = lp.enabled ? 1 : 0;
    const point_3f* src[4] = {&lp.pos, &lp.diffuse, &lp.specular, &lp.attenuationCoefs};
    float* dst[4] = {l.pos, l.diffuse, l.specular, l.attenuation};
    for (int k = 0; k < 4; ++k) {
      dst[k][0] = src[k]->x;
      dst[k][1] = src[k]->y;
      dst[k][2] = src[k]->z;
    }
  }
  yv_ssna_params& SsnaParams() { return Ssna(); }
  void Render(void* d_dstBuf) {
    if (!r_) return;
    status_ = yv_render_ssna(r_, &Ssna(), d_dstBuf, nullptr, nullptr, nullptr);
  }
  /* demo/SVORenderer.cpp:158-186: <fnbase>_<w>x<h>.dist / .color /
   * .normal, one float, Color32 and 3 floats per pixel. */
  bool DumpTraceData(const std::string& fnbase) {
    if (!r_) return false;
    const point_2i res = GetResolution();
    const size_t n = (size_t)res.x * (size_t)res.y;
    std::vector<float> dist(n), normal(3 * n);
    std::vector<uint32_t> color(n);
    status_ = yv_renderer_trace_dump(r_, dist.data(), color.data(), normal.data());
    if (status_ != YV_OK) return false;
    const std::string base =
        fnbase + "_" + std::to_string(res.x) + "x" + std::to_string(res.y);
    return WriteFile(base + ".dist", dist.data(), n * 4) &&
           WriteFile(base + ".color", color.data(), n * 4) &&
           WriteFile(base + ".normal", normal.data(), n * 12);
  }

 private:
  yv_ssna_params& Ssna() {
    if (!ssna_init_) {
      if (r_) yv_ssna_defaults(r_, &ssna_);
      for (int i = 0; i < YV_SSNA_MAX_LIGHTS; ++i) ssna_.lights[i].enabled = 0;
      ssna_init_ = true;
    }
    return ssna_;
  }
  static bool WriteFile(const std::string& fn, const void* p, size_t bytes) {
    FILE* f = std::fopen(fn.c_str(), "wb");
    if (!f) return false;
    const bool ok = std::fwrite(p, 1, bytes, f) == bytes;
    return std::fclose(f) == 0 && ok;
  }
  void Vec(yv_status (*fn)(yv_renderer*, const float*), const point_3f& p) {
    if (!r_) return;
    const float v[3] = {p.x, p.y, p.z};
    status_ = fn(r_, v);
  }
  yv_renderer* r_ = nullptr;
  yv_ssna_params ssna_{};
  bool ssna_init_ = false;
  SVOData* scene_ = nullptr;
  std::vector<Color32> buf_;
  yv_status status_ = YV_OK;
};

/* cell/svorenderer.h:26-27 */
inline std::shared_ptr<ISVORenderer> CreateSimpleRenderer() {
  return std::make_shared<GPURenderer>();
}
inline std::shared_ptr<ISVORenderer> CreateThreadedRenderer() {
  return std::make_shared<GPURenderer>();
}

}  // namespace yv
