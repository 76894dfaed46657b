// shader.h - SimpleShader stand-in: the reference's shading code is not in
// its snapshot, so Shade() returns a white Color32 that carries the hit it
// was called with (the leaf's VoxData and t); the tests compare hits.
#pragma once

struct SimpleShader {
  point_3f viewerPos, lightPos;
  Color32 Shade(VoxData data, const point_3f&, float t) const {
    Color32 c(255, 255, 255, 255);
    c.data = data;
    c.t = t;
    return c;
  }
};
