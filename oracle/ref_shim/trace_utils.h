// trace_utils.h - the traversal helpers of the reference's missing
// cpp/trace_utils.h.  SetupTrace / AdjustDir are restated (octant mirroring
// into the unit cube, eps 1e-5: cell/spu/trace_spu.c_:66-105,
// reaction/report/voxel.tex:309-326), as in the oracle.  FindFirstChild /
// GoNext of the CPU renderer run the reference's own SPU functions
// (cell/spu/trace_spu.cpp:48-93, compiled in ref_spu_glue.cpp).  Two hooks
// let the harness count node fetches per pixel: AdjustDir starts a pixel,
// every FindFirstChild of the CPU renderer follows one node fetch.
#pragma once

#define GLOBAL_FUNC

extern "C" void yvref_pixel_begin(void);
extern "C" void yvref_count_fetch(void);
extern "C" int yvref_spu_find_first_child(float* t1, float* t2);
extern "C" int yvref_spu_go_next(int* ch, float* t1, float* t2);

inline float maxCoord(const point_3f& p) {
  const float m = p.x > p.y ? p.x : p.y;
  return m > p.z ? m : p.z;
}
inline float minCoord(const point_3f& p) {
  const float m = p.x < p.y ? p.x : p.y;
  return m < p.z ? m : p.z;
}
template <class V>
inline float max_vec_float3(const V& v) {
  const float m = v[0] > v[1] ? v[0] : v[1];
  return m > v[2] ? m : v[2];
}
template <class V>
inline float min_vec_float3(const V& v) {
  const float m = v[0] < v[1] ? v[0] : v[1];
  return m < v[2] ? m : v[2];
}

inline void AdjustDir(point_3f& d) {
  yvref_pixel_begin();
  const float eps = 1e-5f;
  if (std::fabs(d.x) < eps) d.x = std::copysign(eps, d.x);
  if (std::fabs(d.y) < eps) d.y = std::copysign(eps, d.y);
  if (std::fabs(d.z) < eps) d.z = std::copysign(eps, d.z);
}

inline bool SetupTrace(const point_3f& pos, const point_3f& dir, point_3f& t1, point_3f& t2,
                       uint& dirFlags) {
  float p[3] = {pos.x, pos.y, pos.z}, d[3] = {dir.x, dir.y, dir.z}, a[3], b[3];
  dirFlags = 0;
  for (int i = 0; i < 3; ++i) {
    if (d[i] < 0.f) {
      p[i] = 1.f - p[i];
      d[i] = -d[i];
      dirFlags |= 1u << i;
    }
    a[i] = (0.f - p[i]) / d[i];
    b[i] = (1.f - p[i]) / d[i];
  }
  t1 = point_3f(a[0], a[1], a[2]);
  t2 = point_3f(b[0], b[1], b[2]);
  return maxCoord(t1) < minCoord(t2);
}

inline int FindFirstChild(point_3f& t1, point_3f& t2) {
  yvref_count_fetch();
  float a[3] = {t1.x, t1.y, t1.z}, b[3] = {t2.x, t2.y, t2.z};
  const int ch = yvref_spu_find_first_child(a, b);
  t1 = point_3f(a[0], a[1], a[2]);
  t2 = point_3f(b[0], b[1], b[2]);
  return ch;
}

inline bool GoNext(int& ch, point_3f& t1, point_3f& t2) {
  float a[3] = {t1.x, t1.y, t1.z}, b[3] = {t2.x, t2.y, t2.z};
  const int ok = yvref_spu_go_next(&ch, a, b);
  t1 = point_3f(a[0], a[1], a[2]);
  t2 = point_3f(b[0], b[1], b[2]);
  return ok != 0;
}
