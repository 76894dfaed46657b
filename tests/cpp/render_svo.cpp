// Caller of the C++ ISVORenderer mirror (include/yv_svo_renderer.hpp) in the
// shape of the reference's cell/main.cpp:21-40: build a scene, set the
// camera, render one frame and write it as raw RGBA8 (uint32 per pixel).
//
// usage: render_svo host <vox path>          (no GPU: host-side API only)
//        render_svo gpu  <vox path> <out.raw> (one 64x48 frame, plus the
//                                             trace dump <out.raw>.dmp_64x48.*)
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "yv_svo_renderer.hpp"

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  const bool gpu = std::strcmp(argv[1], "gpu") == 0;
  yv::SVOData svo;
  if (svo.GetRoot() != yv::kEmptyNode || svo.Size() != 0) return 3;
  if (svo.Spheres(6, 40, 1.0f, 6.0f, 7) != YV_OK) return 4;
  if (svo.Save(argv[2]) != YV_OK) return 5;
  yv::SVOData loaded;
  if (loaded.Load(argv[2]) != YV_OK) return 6;
  if (loaded.Size() != svo.Size() || loaded.GetRoot() != svo.GetRoot()) return 7;
  if (loaded.Load("/nonexistent/path.vox") == YV_OK || loaded.Size() != svo.Size()) return 8;
  std::printf("nodes %u root %u\n", loaded.Size(), loaded.GetRoot());

  std::shared_ptr<yv::ISVORenderer> r = yv::CreateSimpleRenderer();
  yv::GPURenderer* g = static_cast<yv::GPURenderer*>(r.get());
  if (!gpu) {
    // without a device the renderer reports the CUDA error and renders NULL
    const yv::Color32* f = r->RenderFrame();
    std::printf("renderer status %d frame %s\n", (int)g->Status(), f ? "non-null" : "null");
    return f == nullptr && g->Status() != YV_OK ? 0 : 9;
  }
  if (g->Status() != YV_OK) return 10;
  r->SetResolution(64, 48);
  if (r->RenderFrame() != nullptr || g->Status() != YV_ERR_NO_SCENE) return 11;
  r->SetScene(&loaded);
  r->SetViewPos(yv::point_3f(1.1f, 0.45f, 0.72f));
  r->SetViewDir(yv::point_3f(-0.6f, 0.05f, -0.22f));
  r->SetViewUp(yv::point_3f(0.f, 0.f, 1.f));
  r->SetFOV(55.f);
  // light toward normalize(0.3, 0.5, 0.8), normalised in double precision
  const double l[3] = {0.3, 0.5, 0.8};
  const double n = std::sqrt(l[0] * l[0] + l[1] * l[1] + l[2] * l[2]);
  g->SetLight(yv::point_3f((float)(l[0] / n), (float)(l[1] / n), (float)(l[2] / n)), 0.15f,
              0.85f, true);
  const yv::point_2i res = r->GetResolution();
  if (res.x != 64 || res.y != 48) return 12;
  const yv::Color32* f = r->RenderFrame();
  if (!f) return 13;
  FILE* out = std::fopen(argv[3], "wb");
  if (!out) return 14;
  std::fwrite(f, sizeof(yv::Color32), (size_t)res.x * res.y, out);
  std::fclose(out);
  // SVORenderer::DumpTraceData: <base>_64x48.dist / .color / .normal
  g->SetSSNA(true);
  if (!g->GetSSNA() || g->GetShowNormals()) return 15;
  if (!g->DumpTraceData(std::string(argv[3]) + ".dmp")) return 16;
  std::printf("frame written\n");
  return 0;
}
