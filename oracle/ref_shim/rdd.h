// rdd.h - RayDirData, the camera basis RendererBase::InitRayDir fills
// (cell/renderer_base.h:50-61): dir0 + du x + dv y is pixel (x, y)'s ray.
#pragma once

struct RayDirData {
  point_3f dir0, du, dv;
};
