// stdafx.h - precompiled-header stand-in for the reference's renderer
// sources: the standard headers they use and the point types of the `cg`
// vector library their snapshot does not ship (float 3-vectors with +, -,
// scalar *, /, ^ = cross product, normalized(), grad2rad(); int 2-vectors),
// plus Color32.  Test infrastructure for oracle/_ref only.
#pragma once
#include <math.h>

#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <memory>
#include <vector>

using std::max;
using std::min;
using std::shared_ptr;
using std::tan;  // tan(float) is the float function, as the oracle's tanf

typedef unsigned int uint;
typedef unsigned char uchar;

namespace cg {

struct point_3f {
  float x, y, z;
  point_3f() : x(0.f), y(0.f), z(0.f) {}
  point_3f(float a, float b, float c) : x(a), y(b), z(c) {}
};
inline point_3f operator+(const point_3f& a, const point_3f& b) {
  return point_3f(a.x + b.x, a.y + b.y, a.z + b.z);
}
inline point_3f operator-(const point_3f& a, const point_3f& b) {
  return point_3f(a.x - b.x, a.y - b.y, a.z - b.z);
}
inline point_3f operator-(const point_3f& a) { return point_3f(-a.x, -a.y, -a.z); }
inline point_3f operator*(const point_3f& a, float s) { return point_3f(a.x * s, a.y * s, a.z * s); }
inline point_3f operator*(float s, const point_3f& a) { return point_3f(s * a.x, s * a.y, s * a.z); }
inline point_3f operator/(const point_3f& a, float s) { return point_3f(a.x / s, a.y / s, a.z / s); }
// cross product
inline point_3f operator^(const point_3f& a, const point_3f& b) {
  return point_3f(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline point_3f normalized(const point_3f& v) {
  const float len = std::sqrt((v.x * v.x + v.y * v.y) + v.z * v.z);
  return point_3f(v.x / len, v.y / len, v.z / len);
}
inline float grad2rad(float deg) { return deg * (float)(3.14159265358979323846 / 180.0); }

struct point_2i {
  int x, y;
  point_2i() : x(0), y(0) {}
  point_2i(int a, int b) : x(a), y(b) {}
};
inline point_2i operator+(const point_2i& a, const point_2i& b) {
  return point_2i(a.x + b.x, a.y + b.y);
}
inline point_2i operator*(const point_2i& a, int s) { return point_2i(a.x * s, a.y * s); }
inline point_2i operator/(const point_2i& a, int s) { return point_2i(a.x / s, a.y / s); }

}  // namespace cg

using cg::point_2i;
using cg::point_3f;

// RGBA8 colour; `data` / `t` carry the hit the shader was called for (the
// leaf's VoxData and the hit distance), so a test can read hits out of the
// frame buffer the reference renderer returns.
struct Color32 {
  unsigned char r, g, b, a;
  uint32_t data;
  float t;
  Color32() {}
  Color32(int r_, int g_, int b_, int a_)
      : r((unsigned char)r_), g((unsigned char)g_), b((unsigned char)b_), a((unsigned char)a_),
        data(0xFFFFFFFFu), t(0.f) {}
};
