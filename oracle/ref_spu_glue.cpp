// ref_spu_glue.cpp - compiles the reference's SPU tracer
// (cell/spu/trace_spu.cpp, found on the include path that
// oracle/build_ref.py sets) on the host with the stand-ins of ref_shim/,
// and exposes its FindFirstChildSPU / GoNextSPU and its block renderer
// (RenderBlock with the FetchNode node cache) to the harness.
// Test infrastructure for oracle/_ref only.
#include "trace_spu.cpp"

extern "C" int yvref_spu_find_first_child(float* t1, float* t2) {
  float4 a = {t1[0], t1[1], t1[2], 0.f}, b = {t2[0], t2[1], t2[2], 0.f};
  const int ch = FindFirstChildSPU(a, b);
  for (int i = 0; i < 3; ++i) {
    t1[i] = a[i];
    t2[i] = b[i];
  }
  return ch;
}

extern "C" int yvref_spu_go_next(int* ch, float* t1, float* t2) {
  float4 a = {t1[0], t1[1], t1[2], 0.f}, b = {t2[0], t2[1], t2[2], 0.f};
  const bool ok = GoNextSPU(*ch, a, b);
  for (int i = 0; i < 3; ++i) {
    t1[i] = a[i];
    t2[i] = b[i];
  }
  return ok ? 1 : 0;
}

extern "C" int yvref_spu_fetch_count(void) { return fetchCount; }

// One frame through the SPU block renderer: 16x16 blocks in row-major order
// (the tile loop of the SPU main with one SPE), the camera basis given.
// data / t: per pixel the hit leaf's VoxData and t (0xFFFFFFFF for a miss).
extern "C" int yvref_spu_render(const VoxNode* nodes, uint32_t root, const float pos[3],
                                const float dir0[3], const float du[3], const float dv[3],
                                int width, int height, uint32_t* data, float* t) {
  params.pos = point_3f(pos[0], pos[1], pos[2]);
  params.rdd.dir0 = point_3f(dir0[0], dir0[1], dir0[2]);
  params.rdd.du = point_3f(du[0], du[1], du[2]);
  params.rdd.dv = point_3f(dv[0], dv[1], dv[2]);
  params.viewSize = point_2i(width, height);
  params.root = root;
  params.nodes = nodes;
  for (int i = 0; i < CacheSize; ++i) cacheIds[i] = EmptyNode;
  fetchCount = missCount = 0;
  shader.viewerPos = params.pos;
  shader.lightPos = params.pos;
  for (int by = 0; by < (height + BlockSize - 1) / BlockSize; ++by)
    for (int bx = 0; bx < (width + BlockSize - 1) / BlockSize; ++bx) {
      RenderBlock(point_2i(bx * BlockSize, by * BlockSize));
      for (int y = 0; y < BlockSize; ++y)
        for (int x = 0; x < BlockSize; ++x) {
          const int px = bx * BlockSize + x, py = by * BlockSize + y;
          if (px >= width || py >= height) continue;
          const Color32& c = result[y * BlockSize + x];
          data[(size_t)py * width + px] = c.data;
          t[(size_t)py * width + px] = c.t;
        }
    }
  return 0;
}
