// cutil_math.h stand-in for compiling reaction/trace/trace.cu (and its
// utils.h) on the host: CUDA qualifiers as nothing, the vector types and
// the float3 / float4 arithmetic the march uses (component-wise operators,
// dot, normalize, fminf / fmaxf, saturate), and texture references whose
// tex3D is a software fetch: normalized coordinates with clamp addressing;
// cudaReadModeNormalizedFloat textures (the volume) filter linearly
// (texel centres at (i + 0.5) / N, exact weights, not the hardware's
// fixed-point ones), element-type textures (the brick marks) take the
// nearest texel.  Test infrastructure for oracle/_ref only.
#pragma once
#include <math.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#define __device__
#define __host__
#define __global__
#define __constant__
#define __forceinline__ inline

using std::ceil;
using std::copysign;
using std::sqrt;

struct float2 { float x, y; };
struct float3 { float x, y, z; };
struct float4 { float x, y, z, w; };
struct int2 { int x, y; };
struct int3 { int x, y, z; };
struct uint3 { unsigned int x, y, z; };

inline float3 make_float3(float a, float b, float c) { return float3{a, b, c}; }
inline float3 make_float3(float s) { return float3{s, s, s}; }
inline float3 make_float3(const float4& v) { return float3{v.x, v.y, v.z}; }
inline float3 make_float3(const int3& v) { return float3{(float)v.x, (float)v.y, (float)v.z}; }
inline float4 make_float4(float a, float b, float c, float d) { return float4{a, b, c, d}; }
inline float4 make_float4(float s) { return float4{s, s, s, s}; }
inline int3 make_int3(const float3& v) { return int3{(int)v.x, (int)v.y, (int)v.z}; }
inline int2 make_int2(int a, int b) { return int2{a, b}; }

inline float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float3 operator*(float3 a, float3 b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float3 operator/(float3 a, float3 b) { return make_float3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline float3 operator+(float3 a, float s) { return make_float3(a.x + s, a.y + s, a.z + s); }
inline float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
inline float3 operator*(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
inline void operator+=(float3& a, float3 b) { a = a + b; }
inline float4 operator+(float4 a, float4 b) {
  return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
inline float4 operator*(float4 a, float s) { return make_float4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline void operator+=(float4& a, float4 b) { a = a + b; }

inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float dot(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline float3 normalize(float3 v) {
  const float inv = 1.0f / std::sqrt(dot(v, v));
  return v * inv;
}
inline float fminf(float a, float b) { return std::fmin(a, b); }
inline float fmaxf(float a, float b) { return std::fmax(a, b); }
inline float3 fminf(float3 a, float3 b) {
  return make_float3(std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z));
}
inline float3 fmaxf(float3 a, float3 b) {
  return make_float3(std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z));
}
inline float saturate(float v) { return v < 0.f ? 0.f : (v > 1.f ? 1.f : v); }
inline float max(float a, float b) { return a > b ? a : b; }
inline float min(float a, float b) { return a < b ? a : b; }
inline double max(float a, double b) { return (double)a > b ? (double)a : b; }

enum cudaTextureReadMode { cudaReadModeElementType = 0, cudaReadModeNormalizedFloat = 1 };

// A 3D texture reference bound to host data (x fastest).
template <class T, int dim, int mode>
struct texture {
  const T* data = nullptr;
  int nx = 0, ny = 0, nz = 0;
  T at(int x, int y, int z) const {
    x = x < 0 ? 0 : (x >= nx ? nx - 1 : x);
    y = y < 0 ? 0 : (y >= ny ? ny - 1 : y);
    z = z < 0 ? 0 : (z >= nz ? nz - 1 : z);
    return data[((size_t)z * ny + y) * nx + x];
  }
};

template <class T>
inline float tex3D(const texture<T, 3, cudaReadModeNormalizedFloat>& t, float u, float v,
                   float w) {
  const float c[3] = {u * t.nx - 0.5f, v * t.ny - 0.5f, w * t.nz - 0.5f};
  int i[3];
  float f[3];
  for (int k = 0; k < 3; ++k) {
    const float fl = std::floor(c[k]);
    i[k] = (int)fl;
    f[k] = c[k] - fl;
  }
  float r = 0.f;
  for (int j = 0; j < 8; ++j) {
    const int dx = j & 1, dy = (j >> 1) & 1, dz = j >> 2;
    const float wgt = (dx ? f[0] : 1.f - f[0]) * (dy ? f[1] : 1.f - f[1]) *
                      (dz ? f[2] : 1.f - f[2]);
    r += wgt * ((float)t.at(i[0] + dx, i[1] + dy, i[2] + dz) / 255.0f);
  }
  return r;
}

template <class T>
inline T tex3D(const texture<T, 3, cudaReadModeElementType>& t, float u, float v, float w) {
  return t.at((int)std::floor(u * t.nx), (int)std::floor(v * t.ny), (int)std::floor(w * t.nz));
}

extern uint3 threadIdx, blockIdx, blockDim;
