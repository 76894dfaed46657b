// ssna.cu - screen-space normal approximation (SSNA) and point-light Phong
// shading of a traced SVO frame: SVORenderer::Render with m_ssna
// (demo/SVORenderer.cpp:88-146), the blur kernel of InitBlur (:55-78), the
// depth-limited Gaussian blur and the depth normals prototyped in
// demo/dumps/ztools.py (limitedGaussBlur mode 2, :154-233; multipassGaussBlur,
// :252-266; calcNormals, :23-43), the LightParams of Demo.cpp:141-147 and
// DumpTraceData (:158-186).  The reference's BlurZ / ShadeSimple kernels are
// not in its snapshot; these passes restate the host code and the prototype.
//
// Passes of one frame (all on the caller's stream, no host sync):
//   0. the renderer's frame kernel, unlit: albedo (Color32), hit distance t
//      and the hit leaf's stored unit normal per pixel;
//   1. depth: z = t / |u| (u the pixel's unnormalised ray, whose forward
//      component is 1, so z is the view depth); a miss gets kFar;
//   2. blur_passes passes of the 5x5 kernel exp(-(dx^2 + dy^2)) / sum
//      (InitBlur with BlurZKernSize 5, scale 2), pass i blurring the pixels
//      with 0 < z <= 5 voxel / (pixel_angle * 3 (i + 1)); for a tap s of a
//      pixel d, with thr the edge threshold:
//        s > d + thr       -> s = d + edge_pad * thr      (a far tap)
//        d > s + thr       -> the mirrored tap m (2d - offset):
//                               d > m + thr -> weight 0
//                               else s = m (clamped as a far tap)
//      taps outside the frame are left out, the weights renormalised;
//   3. shading: the normal is the cross product of the depth-reconstructed
//      position differences along x and y, each taken on the side with the
//      smaller |dz| (calcNormals' absMin), turned toward the eye (the
//      stored normal where a pixel has no hit neighbour on an axis or the
//      cross product vanishes); colour = albedo * (ambient + sum of
//      diffuse * max(n.L, 0) * att) + sum of specular * max(R.V, 0)^e * att
//      with att = 1 / (a0 + a1 d + a2 d^2), clamped to [0, 1], *255 + 0.5.
// Every step is an FP32 round-to-nearest operation in the order written, so
// the depth and normals are reproducible on the CPU; the specular power is
// powf.
//
// Launch shape: every pass works on 32x32-pixel tiles with 256 threads, 4
// pixels a thread, and issues all of a thread's global loads before it uses
// any, so the depth-buffer passes (8 MB in, 8 MB out at 1920x1080, L2
// resident) are not bound by load latency.  The depth pass also finds the
// frame's smallest hit depth, and a blur pass whose limit lies below it
// returns without work.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>

#include "dev_scan.cuh"
#include "yv_batch.h"
#include "yv_internal.h"
#include "yv_kernels.h"

namespace yv {
namespace {

constexpr float kFar = 1e30f;
constexpr int kTX = 32, kTY = 8;       // threads of a block
constexpr int kTile = 32;              // kTile x kTile pixels per block
constexpr int kRowsPer = kTile / kTY;  // pixels (rows) per thread
constexpr int kHalo = 2;
constexpr int kSm = kTile + 2 * kHalo;  // shared tile side of the blur
constexpr int kMaxPasses = 64;         // blur passes a frame may ask for

struct BlurWeights {
  float k[25];  // [oy + 2][ox + 2]
};

struct View {
  float pos[3], dir0[3], du[3], dv[3];
  int width, height;
};

struct Shading {
  float ambient[3];
  float spec_exp;
  int nlights;
  int ssna;
  int show_normals;
  float lpos[YV_SSNA_MAX_LIGHTS][3];
  float ldif[YV_SSNA_MAX_LIGHTS][3];
  float lspec[YV_SSNA_MAX_LIGHTS][3];
  float latt[YV_SSNA_MAX_LIGHTS][3];
};

__device__ __forceinline__ void ray_u(const View& v, int x, int y, float u[3]) {
  const float fx = (float)x, fy = (float)y;
#pragma unroll
  for (int i = 0; i < 3; ++i)
    u[i] = __fadd_rn(__fadd_rn(v.dir0[i], __fmul_rn(v.du[i], fx)), __fmul_rn(v.dv[i], fy));
}

__device__ __forceinline__ float dot3(const float a[3], const float b[3]) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a[0], b[0]), __fmul_rn(a[1], b[1])),
                   __fmul_rn(a[2], b[2]));
}

// zmin: the smallest hit depth of the frame (bits of a non-negative float,
// which order like the floats), for skipping blur passes that blur nothing.
__global__ void __launch_bounds__(kTX* kTY)
    depth_kernel(const uint32_t* __restrict__ albedo, const float* __restrict__ hit_t, View v,
                 float* __restrict__ z, uint32_t* __restrict__ zmin) {
  const int x = blockIdx.x * kTile + threadIdx.x;
  const int y0 = blockIdx.y * kTile + threadIdx.y;
  uint32_t my_min = 0x7F7FFFFFu;  // FLT_MAX
  uint32_t a[kRowsPer];
  float t[kRowsPer];
#pragma unroll
  for (int r = 0; r < kRowsPer; ++r) {
    const int y = y0 + r * kTY;
    const size_t off = (size_t)y * (size_t)v.width + (size_t)x;
    a[r] = (x < v.width && y < v.height) ? __ldg(albedo + off) : 0u;
    t[r] = (x < v.width && y < v.height) ? __ldg(hit_t + off) : 0.f;
  }
#pragma unroll
  for (int r = 0; r < kRowsPer; ++r) {
    const int y = y0 + r * kTY;
    if (x >= v.width || y >= v.height) continue;
    float out = kFar;
    if (a[r] >> 24) {
      float u[3];
      ray_u(v, x, y, u);
      out = __fdiv_rn(t[r], __fsqrt_rn(dot3(u, u)));
      const uint32_t b = __float_as_uint(fmaxf(out, 0.f));
      my_min = b < my_min ? b : my_min;
    }
    z[(size_t)y * (size_t)v.width + (size_t)x] = out;
  }
  my_min = __reduce_min_sync(0xFFFFFFFFu, my_min);
  if ((threadIdx.x & 31u) == 0) atomicMin(zmin, my_min);
}

// Blurred depth of pixel (x, y) of a w x h frame; at(dx, dy) is the depth of
// the pixel at offset (dx, dy), asked only for offsets inside the frame.
// kEdge = false: the pixel is 2 or more pixels inside the frame, so every
// tap and mirrored tap is (the bounds tests drop out).
template <bool kEdge, class At>
__device__ __forceinline__ float blur_taps(At at, float d, int x, int y, int w, int h,
                                           float thr, float pad_thr, const BlurWeights& bw) {
  const float d_far = __fadd_rn(d, thr), d_pad = __fadd_rn(d, pad_thr);
  float acc = 0.f, c = 0.f;
#pragma unroll
  for (int oy = -2; oy <= 2; ++oy) {
#pragma unroll
    for (int ox = -2; ox <= 2; ++ox) {
      const int sx = x + ox, sy = y + oy;
      if (kEdge && (sx < 0 || sy < 0 || sx >= w || sy >= h)) continue;
      float s = at(ox, oy);
      float k = bw.k[(oy + 2) * 5 + ox + 2];
      if (s > d_far) {
        s = d_pad;
      } else if (d > __fadd_rn(s, thr)) {
        const int mx = x - ox, my = y - oy;
        if (kEdge && (mx < 0 || my < 0 || mx >= w || my >= h)) {
          k = 0.f;
        } else {
          const float m = at(-ox, -oy);
          if (d > __fadd_rn(m, thr)) k = 0.f;
          else s = m > d_far ? d_pad : m;
        }
      }
      acc = __fadd_rn(acc, __fmul_rn(s, k));
      c = __fadd_rn(c, k);
    }
  }
  return __fdiv_rn(acc, c);
}

template <class At>
__device__ __forceinline__ float blur_pixel(At at, int x, int y, int w, int h, float zlimit,
                                            float thr, float pad_thr, const BlurWeights& bw) {
  const float d = at(0, 0);
  if (!(d > 0.f && d <= zlimit)) return d;
  if (x >= 2 && y >= 2 && x + 2 < w && y + 2 < h)
    return blur_taps<false>(at, d, x, y, w, h, thr, pad_thr, bw);
  return blur_taps<true>(at, d, x, y, w, h, thr, pad_thr, bw);
}

// Whether a blur pass with limit zlimit can change a pixel of a frame whose
// smallest hit depth is zm.  Every blurred depth is a weighted mean of depths
// and depths moved away from the eye (edge_pad >= 0), so the buffer's
// smallest depth falls only by rounding (about 51 ulp a pass, 2e-4 relative
// over 64 passes); a pass with zlimit below zm (1 - 2^-10) blurs nothing.
// The passes that run are a prefix of the schedule: the limits decrease.
__device__ __forceinline__ bool pass_runs(float zm, float zlimit) {
  return zlimit >= __fmul_rn(zm, 1.f - 1.f / 1024.f);
}

// A pass that blurs nothing returns at once; its buffers keep their roles.
__global__ void __launch_bounds__(kTX* kTY)
    blur_kernel(const float* __restrict__ zin, float* __restrict__ zout, int w, int h,
                float zlimit, float thr, float pad_thr, BlurWeights bw,
                const uint32_t* __restrict__ zmin) {
  if (!pass_runs(__uint_as_float(__ldg(zmin)), zlimit)) return;
  __shared__ float tile[kSm][kSm];
  constexpr int kLoads = (kSm * kSm + kTX * kTY - 1) / (kTX * kTY);
  const int x0 = blockIdx.x * kTile - kHalo, y0 = blockIdx.y * kTile - kHalo;
  const int tid = threadIdx.y * kTX + threadIdx.x;
  float ld[kLoads];
#pragma unroll
  for (int j = 0; j < kLoads; ++j) {
    const int i = tid + j * kTX * kTY;
    const int gx = x0 + i % kSm, gy = y0 + i / kSm;
    ld[j] = (i < kSm * kSm && gx >= 0 && gy >= 0 && gx < w && gy < h)
                ? __ldg(zin + (size_t)gy * w + gx)
                : kFar;
  }
#pragma unroll
  for (int j = 0; j < kLoads; ++j) {
    const int i = tid + j * kTX * kTY;
    if (i < kSm * kSm) tile[i / kSm][i % kSm] = ld[j];
  }
  __syncthreads();
  const int x = blockIdx.x * kTile + threadIdx.x;
  if (x >= w) return;
  const int tx = threadIdx.x + kHalo;
#pragma unroll
  for (int r = 0; r < kRowsPer; ++r) {
    const int y = blockIdx.y * kTile + threadIdx.y + r * kTY;
    if (y >= h) break;
    const int ty = threadIdx.y + r * kTY + kHalo;
    zout[(size_t)y * w + x] =
        blur_pixel([&](int dx, int dy) { return tile[ty + dy][tx + dx]; }, x, y, w, h, zlimit,
                   thr, pad_thr, bw);
  }
}

// Tangent along one axis from the pixel's depth zc (position pc) and its
// neighbours' depths zl at -step and zh at +step (kFar: no hit or outside
// the frame); false when neither neighbour holds a hit.
__device__ __forceinline__ bool tangent(const View& v, int x, int y, int sx, int sy, float zc,
                                        const float pc[3], float zl, float zh, float t[3]) {
  const bool has_lo = zl < kFar, has_hi = zh < kFar;
  if (!has_lo && !has_hi) return false;
  const bool use_hi =
      has_hi && (!has_lo || fabsf(__fsub_rn(zh, zc)) < fabsf(__fsub_rn(zc, zl)));
  float u[3];
  if (use_hi) {
    ray_u(v, x + sx, y + sy, u);
#pragma unroll
    for (int i = 0; i < 3; ++i) t[i] = __fsub_rn(__fmul_rn(zh, u[i]), pc[i]);
  } else {
    ray_u(v, x - sx, y - sy, u);
#pragma unroll
    for (int i = 0; i < 3; ++i) t[i] = __fsub_rn(pc[i], __fmul_rn(zl, u[i]));
  }
  return true;
}

__device__ __forceinline__ uint32_t to_u8(float c) {
  c = fminf(fmaxf(c, 0.f), 1.f);
  return __float2uint_rz(__fadd_rn(__fmul_rn(c, 255.f), 0.5f));
}

// Colour of a hit pixel; n holds the stored normal on entry and the normal
// used on return.  zn = depths of the (x-1, x+1, y-1, y+1) neighbours.
// Per light, with lv = light - P, d = |lv| and u the pixel's ray:
//   n.L = (n.lv) / d,  R.V = (lv.u - 2 (n.L) (n.u) d) / (d |u|)
// (R = 2 (n.L) n - L, V = -u / |u|), one division each.
__device__ __forceinline__ uint32_t shade_pixel(uint32_t alb, float zc, const float zn[4],
                                                float n[3], const View& v, const Shading& sh,
                                                int x, int y) {
  float u[3], p[3];
  ray_u(v, x, y, u);
#pragma unroll
  for (int i = 0; i < 3; ++i) p[i] = __fmul_rn(zc, u[i]);
  if (sh.ssna) {
    float tx[3], ty[3];
    if (tangent(v, x, y, 1, 0, zc, p, zn[0], zn[1], tx) &&
        tangent(v, x, y, 0, 1, zc, p, zn[2], zn[3], ty)) {
      float c[3] = {__fsub_rn(__fmul_rn(tx[1], ty[2]), __fmul_rn(tx[2], ty[1])),
                    __fsub_rn(__fmul_rn(tx[2], ty[0]), __fmul_rn(tx[0], ty[2])),
                    __fsub_rn(__fmul_rn(tx[0], ty[1]), __fmul_rn(tx[1], ty[0]))};
      if (dot3(c, u) > 0.f) {
        c[0] = -c[0];
        c[1] = -c[1];
        c[2] = -c[2];
      }
      const float len2 = dot3(c, c);
      if (len2 > 0.f && len2 <= 3.402823466e38f) {
        const float inv = __fdiv_rn(1.f, __fsqrt_rn(len2));
#pragma unroll
        for (int i = 0; i < 3; ++i) n[i] = __fmul_rn(c[i], inv);
      }
    }
  }
  uint32_t out = 0xFF000000u;
  if (sh.show_normals) {
#pragma unroll
    for (int i = 0; i < 3; ++i) out |= to_u8(__fadd_rn(__fmul_rn(n[i], 0.5f), 0.5f)) << (8 * i);
    return out;
  }
  float a[3], col[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    a[i] = __fmul_rn((float)((alb >> (8 * i)) & 0xFFu), 1.0f / 255.0f);
    col[i] = __fmul_rn(a[i], sh.ambient[i]);
  }
  const float ulen = __fsqrt_rn(dot3(u, u));
  const float nu = dot3(n, u);
  for (int l = 0; l < sh.nlights; ++l) {
    float lv[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) lv[i] = __fsub_rn(sh.lpos[l][i], __fadd_rn(v.pos[i], p[i]));
    const float d2 = dot3(lv, lv);
    const float d = __fsqrt_rn(d2);
    if (!(d > 0.f)) continue;
    const float ndl = __fdiv_rn(dot3(n, lv), d);
    if (!(ndl > 0.f)) continue;
    const float den = __fadd_rn(__fadd_rn(sh.latt[l][0], __fmul_rn(sh.latt[l][1], d)),
                                __fmul_rn(sh.latt[l][2], d2));
    const float att = den > 0.f ? __fdiv_rn(1.f, den) : 0.f;
    const float na = __fmul_rn(ndl, att);
#pragma unroll
    for (int i = 0; i < 3; ++i)
      col[i] = __fadd_rn(col[i], __fmul_rn(a[i], __fmul_rn(na, sh.ldif[l][i])));
    const float num = __fsub_rn(dot3(lv, u), __fmul_rn(__fmul_rn(__fmul_rn(2.f, ndl), nu), d));
    const float rv = __fdiv_rn(num, __fmul_rn(d, ulen));
    if (!(rv > 0.f)) continue;
    const float sp = __fmul_rn(powf(rv, sh.spec_exp), att);
#pragma unroll
    for (int i = 0; i < 3; ++i) col[i] = __fadd_rn(col[i], __fmul_rn(sh.lspec[l][i], sp));
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) out |= to_u8(col[i]) << (8 * i);
  return out;
}

// The final depth is in za after an even number of passes that ran, zb
// after an odd number (pass_runs decides each).
struct PassLimits {
  float z[kMaxPasses];
  int n;
};

__global__ void __launch_bounds__(kTX* kTY)
    shade_kernel(const uint32_t* __restrict__ albedo, const float* __restrict__ za,
                 const float* __restrict__ zb, PassLimits pl, const uint32_t* __restrict__ zmin,
                 const float* __restrict__ stored_n, View v, Shading sh,
                 uint32_t* __restrict__ rgba, float* __restrict__ depth_out,
                 float* __restrict__ normal_out) {
  const float zm = __uint_as_float(__ldg(zmin));
  int ran = 0;
  for (int i = 0; i < pl.n; ++i) ran += pass_runs(zm, pl.z[i]) ? 1 : 0;
  const float* __restrict__ z = (ran & 1) ? zb : za;
  const int x = blockIdx.x * kTile + threadIdx.x;
  const int y0 = blockIdx.y * kTile + threadIdx.y;
  const int w = v.width, h = v.height;
  if (x >= w) return;
  // loads first: albedo, the depth cross, then the stored normals of the hits
  uint32_t a[kRowsPer];
  float zc[kRowsPer], zn[kRowsPer][4], sn[kRowsPer][3];
#pragma unroll
  for (int r = 0; r < kRowsPer; ++r) {
    const int y = y0 + r * kTY;
    const size_t off = (size_t)y * (size_t)w + (size_t)x;
    const bool in = y < h;
    a[r] = in ? __ldg(albedo + off) : 0u;
    zc[r] = in ? __ldg(z + off) : kFar;
    zn[r][0] = in && x > 0 ? __ldg(z + off - 1) : kFar;
    zn[r][1] = in && x + 1 < w ? __ldg(z + off + 1) : kFar;
    zn[r][2] = in && y > 0 ? __ldg(z + off - w) : kFar;
    zn[r][3] = in && y + 1 < h ? __ldg(z + off + w) : kFar;
  }
#pragma unroll
  for (int r = 0; r < kRowsPer; ++r) {
    const size_t off = (size_t)(y0 + r * kTY) * (size_t)w + (size_t)x;
    const bool hit = (a[r] >> 24) != 0u;
    sn[r][0] = hit ? __ldg(stored_n + 3 * off) : 0.f;
    sn[r][1] = hit ? __ldg(stored_n + 3 * off + 1) : 0.f;
    sn[r][2] = hit ? __ldg(stored_n + 3 * off + 2) : 0.f;
  }
#pragma unroll
  for (int r = 0; r < kRowsPer; ++r) {
    const int y = y0 + r * kTY;
    if (y >= h) break;
    const size_t off = (size_t)y * (size_t)w + (size_t)x;
    const bool hit = (a[r] >> 24) != 0u;
    float n[3] = {sn[r][0], sn[r][1], sn[r][2]};
    rgba[off] = hit ? shade_pixel(a[r], zc[r], zn[r], n, v, sh, x, y) : 0u;
    if (depth_out) depth_out[off] = hit ? zc[r] : 0.f;
    if (normal_out) {
      normal_out[3 * off] = n[0];
      normal_out[3 * off + 1] = n[1];
      normal_out[3 * off + 2] = n[2];
    }
  }
}

__global__ void dump_kernel(const uint32_t* __restrict__ albedo, const float* __restrict__ hit_t,
                            int w, int h, float* __restrict__ dist) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= w || y >= h) return;
  const size_t off = (size_t)y * (size_t)w + (size_t)x;
  dist[off] = (albedo[off] >> 24) ? hit_t[off] : 0.f;
}

BlurWeights blur_weights() {
  // InitBlur with BlurZKernSize 5: h = 5/2 = 2, t = scale (i - h) / h with
  // scale 2, i.e. t = i - 2; weights exp(-(tx^2 + ty^2)), normalised.
  double w[25], sum = 0.0;
  for (int y = 0; y < 5; ++y)
    for (int x = 0; x < 5; ++x) {
      const double tx = x - 2.0, ty = y - 2.0;
      w[y * 5 + x] = std::exp(-(tx * tx + ty * ty));
      sum += w[y * 5 + x];
    }
  BlurWeights b;
  for (int i = 0; i < 25; ++i) b.k[i] = (float)(w[i] / sum);
  return b;
}

yv_status ssna_fail(cudaError_t e, const char* what) {
  set_last_error(std::string("ssna: ") + what + ": " + cudaGetErrorString(e));
  cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? YV_ERR_OUT_OF_MEMORY : YV_ERR_CUDA;
}

View make_view(const yv_renderer_view& rv) {
  View v;
  std::memcpy(v.pos, rv.fa.pos, sizeof(v.pos));
  std::memcpy(v.dir0, rv.fa.dir0, sizeof(v.dir0));
  std::memcpy(v.du, rv.fa.du, sizeof(v.du));
  std::memcpy(v.dv, rv.fa.dv, sizeof(v.dv));
  v.width = rv.fa.width;
  v.height = rv.fa.height;
  return v;
}

}  // namespace
}  // namespace yv

using namespace yv;

extern "C" {

yv_status yv_ssna_defaults(const yv_renderer* r, yv_ssna_params* p) {
  if (!r || !p) return YV_ERR_INVALID_ARG;
  std::memset(p, 0, sizeof(*p));
  yv_renderer_view rv;
  std::memset(&rv, 0, sizeof(rv));
  renderer_view(r, &rv);  // the camera is set whether or not a scene is
  p->ssna = 1;
  p->blur_passes = 5;
  p->voxel_size = 1.0f / 2048.0f;
  p->edge_threshold = 4.0f / 2048.0f;
  p->edge_pad = 0.3f;
  p->ambient[0] = p->ambient[1] = p->ambient[2] = 0.1f;
  p->specular_exp = 10.0f;
  yv_point_light& l = p->lights[0];
  l.enabled = 1;
  std::memcpy(l.pos, rv.fa.pos, sizeof(l.pos));
  l.diffuse[0] = l.diffuse[1] = l.diffuse[2] = 0.7f;
  l.specular[0] = l.specular[1] = l.specular[2] = 0.3f;
  l.attenuation[0] = 1.0f;
  l.attenuation[1] = 0.0f;
  l.attenuation[2] = 0.5f;
  return YV_OK;
}

yv_status yv_render_ssna(yv_renderer* r, const yv_ssna_params* p, void* device_rgba,
                         void* device_depth, void* device_normals, void* stream) {
  if (!r || !p || !device_rgba) return YV_ERR_INVALID_ARG;
  if (p->blur_passes < 0 || p->blur_passes > 64 || !(p->voxel_size > 0.f) ||
      !(p->edge_threshold >= 0.f) || !(p->edge_pad >= 0.f) || std::isnan(p->specular_exp))
    return YV_ERR_INVALID_ARG;
  yv_renderer_view rv;
  if (!renderer_view(r, &rv)) return YV_ERR_NO_SCENE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const View v = make_view(rv);
  const size_t px = (size_t)v.width * (size_t)v.height;
  const int passes = p->ssna ? p->blur_passes : 0;
  DevBuf alb, ht, nrm, za, zb, zmin;
  cudaError_t e;
  if ((e = alb.alloc(px * 4, s)) != cudaSuccess || (e = ht.alloc(px * 4, s)) != cudaSuccess ||
      (e = nrm.alloc(px * 12, s)) != cudaSuccess || (e = za.alloc(px * 4, s)) != cudaSuccess ||
      (e = zb.alloc(passes > 0 ? px * 4 : 16, s)) != cudaSuccess ||
      (e = zmin.alloc(4, s)) != cudaSuccess ||
      (e = cudaMemsetAsync(zmin.p, 0x7F, 4, s)) != cudaSuccess)  // 3.4e38: above every depth
    return ssna_fail(e, "scratch");
  yv_frame_outputs fo;
  std::memset(&fo, 0, sizeof(fo));
  fo.rgba = alb.p;
  fo.hit_t = ht.p;
  fo.normal = nrm.p;
  yv_status st = renderer_enqueue_unlit(r, &fo, s);
  if (st != YV_OK) return st;

  Shading sh;
  std::memset(&sh, 0, sizeof(sh));
  std::memcpy(sh.ambient, p->ambient, sizeof(sh.ambient));
  sh.spec_exp = p->specular_exp;
  sh.ssna = p->ssna ? 1 : 0;
  sh.show_normals = p->show_normals ? 1 : 0;
  for (int l = 0; l < YV_SSNA_MAX_LIGHTS; ++l) {
    const yv_point_light& L = p->lights[l];
    if (!L.enabled) continue;
    const int k = sh.nlights++;
    std::memcpy(sh.lpos[k], L.pos, 12);
    std::memcpy(sh.ldif[k], L.diffuse, 12);
    std::memcpy(sh.lspec[k], L.specular, 12);
    std::memcpy(sh.latt[k], L.attenuation, 12);
  }
  const BlurWeights bw = blur_weights();
  // pixel angle = fov / width in radians (RenderParams::pixelAng); pass i
  // blurs z <= 5 voxSize / (pixelAng * blurSize), blurSize = 3 (i + 1)
  const double pix = (double)rv.fov_deg * (3.14159265358979323846 / 180.0) / v.width;
  const float thr = p->edge_threshold;
  const float pad_thr = p->edge_pad * thr;

  const dim3 blk(kTX, kTY);
  const dim3 grd((unsigned)((v.width + kTile - 1) / kTile),
                 (unsigned)((v.height + kTile - 1) / kTile));
  depth_kernel<<<grd, blk, 0, s>>>(alb.as<uint32_t>(), ht.as<float>(), v, za.as<float>(),
                                   zmin.as<uint32_t>());
  if ((e = cudaGetLastError()) != cudaSuccess) return ssna_fail(e, "depth launch");
  PassLimits pl;
  pl.n = passes;
  float* src = za.as<float>();
  float* dst = zb.as<float>();
  for (int i = 0; i < passes; ++i) {
    pl.z[i] = (float)(5.0 * p->voxel_size / (pix * 3.0 * (i + 1)));
    blur_kernel<<<grd, blk, 0, s>>>(src, dst, v.width, v.height, pl.z[i], thr, pad_thr, bw,
                                    zmin.as<uint32_t>());
    if ((e = cudaGetLastError()) != cudaSuccess) return ssna_fail(e, "blur launch");
    float* t = src;
    src = dst;
    dst = t;
  }
  shade_kernel<<<grd, blk, 0, s>>>(alb.as<uint32_t>(), za.as<float>(), zb.as<float>(), pl,
                                   zmin.as<uint32_t>(), nrm.as<float>(), v, sh,
                                   static_cast<uint32_t*>(device_rgba),
                                   static_cast<float*>(device_depth),
                                   static_cast<float*>(device_normals));
  if ((e = cudaGetLastError()) != cudaSuccess) return ssna_fail(e, "shade launch");
  return YV_OK;
}

yv_status yv_renderer_trace_dump(yv_renderer* r, float* host_dist, uint32_t* host_color,
                                 float* host_normal) {
  if (!r) return YV_ERR_INVALID_ARG;
  yv_renderer_view rv;
  if (!renderer_view(r, &rv)) return YV_ERR_NO_SCENE;
  const int w = rv.fa.width, h = rv.fa.height;
  const size_t px = (size_t)w * (size_t)h;
  cudaStream_t s = nullptr;
  DevBuf alb, ht, nrm, dist;
  cudaError_t e;
  if ((e = alb.alloc(px * 4, s)) != cudaSuccess || (e = ht.alloc(px * 4, s)) != cudaSuccess ||
      (e = nrm.alloc(px * 12, s)) != cudaSuccess || (e = dist.alloc(px * 4, s)) != cudaSuccess)
    return ssna_fail(e, "scratch");
  yv_frame_outputs fo;
  std::memset(&fo, 0, sizeof(fo));
  fo.rgba = alb.p;
  fo.hit_t = ht.p;
  fo.normal = nrm.p;
  yv_status st = renderer_enqueue_unlit(r, &fo, s);
  if (st != YV_OK) return st;
  const dim3 blk(32, 8);
  const dim3 grd((unsigned)((w + 31) / 32), (unsigned)((h + 7) / 8));
  dump_kernel<<<grd, blk, 0, s>>>(alb.as<uint32_t>(), ht.as<float>(), w, h, dist.as<float>());
  if ((e = cudaGetLastError()) != cudaSuccess) return ssna_fail(e, "dump launch");
  yv_frame_stats fs;
  st = yv_renderer_frame_stats(r, &fs);  // synchronises the stream
  if (st != YV_OK) return st;
  if (host_dist && (e = cudaMemcpy(host_dist, dist.p, px * 4, cudaMemcpyDeviceToHost)))
    return ssna_fail(e, "read dist");
  if (host_color && (e = cudaMemcpy(host_color, alb.p, px * 4, cudaMemcpyDeviceToHost)))
    return ssna_fail(e, "read color");
  if (host_normal && (e = cudaMemcpy(host_normal, nrm.p, px * 12, cudaMemcpyDeviceToHost)))
    return ssna_fail(e, "read normal");
  return YV_OK;
}

}  // extern "C"
