// ref_harness.cpp - C entry points over the reference's CPU renderer
// (cell/ppu_renderer.cpp with cell/renderer_base.h and cell/svodata.h,
// compiled on the host by oracle/build_ref.py) for the tests that pin the
// oracle: the scene is loaded by the reference's own SVOData::Load, the frame
// rendered by its SimpleRenderer (InitRayDir, RenderRect, RecTrace, with the
// SPU FindFirstChild / GoNext), and every pixel's hit read back with its
// node-fetch count.  Test infrastructure for oracle/_ref only.
#include "stdafx.h"
#include "renderer_base.h"
#include "svorenderer.h"

#include <mutex>

namespace {

// per-pixel fetch counts of the single-threaded renderer: AdjustDir opens a
// pixel, FindFirstChild (one per node fetch) counts into it
std::vector<uint32_t> g_pixel_fetches;
bool g_counting = false;
int (*g_counter)(void) = nullptr;  // SPU renderer: its own fetch counter
int g_last = 0;

// 32-bit SPU effective addresses are the low word of a host address inside
// one 4 GiB window (the node pool is allocated so that it does not cross one)
uintptr_t g_ea_high = 0;

// reads the reference renderer's protected camera basis
struct BasisProbe : public RendererBase {
  void basis(RayDirData& r) { InitRayDir(r); }
  const Color32* RenderFrame() { return nullptr; }
};

}  // namespace

extern "C" void yvref_pixel_begin(void) {
  if (!g_counting) return;
  if (g_counter) {
    const int now = g_counter();
    if (!g_pixel_fetches.empty()) g_pixel_fetches.back() = (uint32_t)(now - g_last);
    g_last = now;
  }
  g_pixel_fetches.push_back(0);
}

extern "C" void yvref_count_fetch(void) {
  if (g_counting && !g_counter && !g_pixel_fetches.empty()) ++g_pixel_fetches.back();
}

extern "C" void* yvref_ea_to_ptr(unsigned int ea) {
  return reinterpret_cast<void*>(g_ea_high | (uintptr_t)ea);
}

extern "C" int yvref_spu_fetch_count(void);
extern "C" int yvref_spu_render(const VoxNode* nodes, uint32_t root, const float pos[3],
                                const float dir0[3], const float du[3], const float dv[3],
                                int width, int height, uint32_t* data, float* t);

// The reference camera basis (RendererBase::InitRayDir) for a view.
extern "C" int yvref_ray_basis(const float dir[3], const float up[3], float fov, int width,
                               int height, float dir0[3], float du[3], float dv[3]) {
  BasisProbe p;
  p.SetViewDir(point_3f(dir[0], dir[1], dir[2]));
  p.SetViewUp(point_3f(up[0], up[1], up[2]));
  p.SetFOV(fov);
  p.SetResolution(width, height);
  RayDirData r;
  p.basis(r);
  const point_3f* v[3] = {&r.dir0, &r.du, &r.dv};
  float* out[3] = {dir0, du, dv};
  for (int i = 0; i < 3; ++i) {
    out[i][0] = v[i]->x;
    out[i][1] = v[i]->y;
    out[i][2] = v[i]->z;
  }
  return 0;
}

// One frame of the reference CPU renderer over a .vox file:
// CreateSimpleRenderer (threaded = 0) or CreateThreadedRenderer (threaded =
// 1; fetch counts are then not recorded).  Per pixel: the hit leaf's VoxData
// (0xFFFFFFFF for a miss), its t, and the node fetches of its RecTrace.
extern "C" int yvref_ppu_render(const char* vox_path, const float pos[3], const float dir[3],
                                const float up[3], float fov, int width, int height,
                                int threaded, uint32_t* data, float* t, uint32_t* fetches) {
  static std::mutex mu;
  std::lock_guard<std::mutex> lk(mu);
  SVOData svo;
  svo.Load(vox_path);
  shared_ptr<ISVORenderer> r = threaded ? CreateThreadedRenderer() : CreateSimpleRenderer();
  r->SetScene(&svo);
  r->SetViewPos(point_3f(pos[0], pos[1], pos[2]));
  r->SetViewDir(point_3f(dir[0], dir[1], dir[2]));
  r->SetViewUp(point_3f(up[0], up[1], up[2]));
  r->SetResolution(width, height);
  r->SetFOV(fov);
  g_pixel_fetches.clear();
  g_counter = nullptr;
  g_counting = !threaded;
  const Color32* buf = r->RenderFrame();
  g_counting = false;
  if (!buf) return 2;
  const size_t n = (size_t)width * (size_t)height;
  for (size_t i = 0; i < n; ++i) {
    data[i] = buf[i].data;
    t[i] = buf[i].t;
  }
  if (fetches && !threaded) {
    if (g_pixel_fetches.size() != n) return 3;
    std::memcpy(fetches, g_pixel_fetches.data(), n * sizeof(uint32_t));
  }
  return 0;
}

// The same frame through the reference SPU tracer (RenderBlock, RecTrace,
// FetchNode with its 2048-entry node cache), on the basis of the CPU
// renderer's InitRayDir.  nodes: count VoxNode records.
extern "C" int yvref_spu_frame(const uint32_t* nodes, uint32_t count, uint32_t root,
                               const float pos[3], const float dir[3], const float up[3],
                               float fov, int width, int height, uint32_t* data, float* t,
                               uint32_t* fetches) {
  static std::mutex mu;
  std::lock_guard<std::mutex> lk(mu);
  // a copy of the pool inside one 4 GiB window (aligned to a power of two at
  // least its size)
  const size_t bytes = (size_t)count * sizeof(VoxNode) + 64;
  size_t align = 64;
  while (align < bytes) align <<= 1;
  void* pool = nullptr;
  if (posix_memalign(&pool, align, bytes) != 0) return 7;
  std::memcpy(pool, nodes, (size_t)count * sizeof(VoxNode));
  g_ea_high = reinterpret_cast<uintptr_t>(pool) & ~(uintptr_t)0xFFFFFFFFu;
  float d0[3], du[3], dv[3];
  yvref_ray_basis(dir, up, fov, width, height, d0, du, dv);
  // pixel order of the block renderer: blocks row-major, pixels row-major
  // inside a block (out-of-frame pixels of edge blocks are traced too)
  g_pixel_fetches.clear();
  g_counter = yvref_spu_fetch_count;
  g_last = 0;
  g_counting = true;
  std::vector<uint32_t> dd((size_t)width * height);
  std::vector<float> tt((size_t)width * height);
  int st = yvref_spu_render(static_cast<const VoxNode*>(pool), root, pos, d0, du, dv, width,
                            height, dd.data(), tt.data());
  yvref_pixel_begin();  // closes the last pixel
  g_counting = false;
  g_counter = nullptr;
  free(pool);
  if (st) return st;
  std::memcpy(data, dd.data(), dd.size() * sizeof(uint32_t));
  std::memcpy(t, tt.data(), tt.size() * sizeof(float));
  if (fetches) {
    const int B = 16, bw = (width + B - 1) / B, bh = (height + B - 1) / B;
    if (g_pixel_fetches.size() != (size_t)bw * bh * B * B + 1) return 3;
    size_t i = 0;
    for (int by = 0; by < bh; ++by)
      for (int bx = 0; bx < bw; ++bx)
        for (int y = 0; y < B; ++y)
          for (int x = 0; x < B; ++x, ++i) {
            const int px = bx * B + x, py = by * B + y;
            if (px < width && py < height) fetches[(size_t)py * width + px] = g_pixel_fetches[i];
          }
  }
  return 0;
}
