// brick_kernels.cu - brick-volume ray-march (ntree layout) for sm_103a:
// forward compositing, its adjoint, and apron maintenance.
//
// March (restating castRay / walkBrick / intersect of
// reaction/trace/trace.cu:42-139 over the N=4 grid tree of volume_host.cpp):
//  * clip the ray to the unit cube, t_enter = max(t_enter, 0);
//  * DDA over brick cells; cell c spans [t_in, t_out) with t_in = the
//    previous cell's t_out, so cells partition the ray;
//  * in an occupied cell, samples sit at the global multiples t = k*dt
//    (trace.cu:47), dt = step_vox lattice cells;
//  * sample = software FP32 trilinear of density and albedo inside the brick
//    (the 9^3 apron lattice keeps all 8 corners in the brick);
//  * alpha = saturate(alpha_scale * density), front-to-back pre-multiplied
//    accumulation C += (1-A)*alpha*albedo, A += (1-A)*alpha (trace.cu:58),
//    stop once A > 0.99 (trace.cu:59).
// Every float operation of the march is an explicit round-to-nearest
// intrinsic so the forward and the backward kernels replay bit-identical
// values (the adjoint relies on reaching the forward's exact final colour).
//
// Adjoint: the backward kernel re-marches each ray instead of storing
// per-sample state.  With T = 1 - A before sample j and the forward output
// (C, A) of the ray:
//   d out_k / d alpha_j = T c_jk - (out_k - out_k after j) / (1 - alpha_j)
//   d out_k / d c_jk    = T alpha_j            (c_A = 1)
// Gradients for the 8 trilinear corners are coalesced in registers while
// consecutive samples of a ray stay in the same trilinear cell, then flushed
// with FP32 atomics (red.global.add.f32).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "yv_volume.h"

namespace yv {
namespace {

constexpr int kL = 9;
constexpr int kL3 = 729;
constexpr uint32_t kEmpty = 0x80000000u;
constexpr uint32_t kBrick = 0x40000000u;
constexpr int kSmemGrids = 65;  // root + up to 64 level-1 grid nodes

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float lerpf_(float a, float b, float t) { return ffma(t, fsub(b, a), a); }

template <int P>
struct Voxel;

// precision 0: fp16 density, uchar4 albedo
template <>
struct Voxel<0> {
  __device__ static __forceinline__ float den(const void* p, uint32_t i) {
    return __half2float(__ushort_as_half(__ldg(static_cast<const unsigned short*>(p) + i)));
  }
  __device__ static __forceinline__ void alb(const void* p, uint32_t i, float* c) {
    const uint32_t v = __ldg(static_cast<const unsigned int*>(p) + i);
    const float s = 1.0f / 255.0f;
    c[0] = fmul((float)(v & 0xFFu), s);
    c[1] = fmul((float)((v >> 8) & 0xFFu), s);
    c[2] = fmul((float)((v >> 16) & 0xFFu), s);
  }
};

// precision 1: fp32 density, fp32 RGB albedo (learnable)
template <>
struct Voxel<1> {
  __device__ static __forceinline__ float den(const void* p, uint32_t i) {
    return __ldg(static_cast<const float*>(p) + i);
  }
  __device__ static __forceinline__ void alb(const void* p, uint32_t i, float* c) {
    const float* q = static_cast<const float*>(p) + 3 * (size_t)i;
    c[0] = __ldg(q);
    c[1] = __ldg(q + 1);
    c[2] = __ldg(q + 2);
  }
};

struct SampleCtx {
  uint32_t base;  // brick*729 + corner-000 lattice index
  float fx, fy, fz;
  float sigma, alpha;
  float col[3];
};

// lx, ly, lz: brick-local lattice coordinates of the sample, in [0, 8].
template <int P>
__device__ __forceinline__ void eval_sample(const VolumeArgs& a, int b, float lx, float ly,
                                            float lz, SampleCtx& s) {
  float l[3] = {lx, ly, lz};
  int i0[3];
  float f[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    int k = __float2int_rd(l[i]);
    k = k < 0 ? 0 : (k > 7 ? 7 : k);
    float fi = fsub(l[i], (float)k);
    fi = fi < 0.f ? 0.f : (fi > 1.f ? 1.f : fi);
    i0[i] = k;
    f[i] = fi;
  }
  s.fx = f[0];
  s.fy = f[1];
  s.fz = f[2];
  s.base = (uint32_t)b * (uint32_t)kL3 + (uint32_t)((i0[2] * kL + i0[1]) * kL + i0[0]);
  float d[8];
  float c[8][3];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const uint32_t idx = s.base + (uint32_t)(((j >> 2) * kL + ((j >> 1) & 1)) * kL + (j & 1));
    d[j] = Voxel<P>::den(a.density, idx);
    Voxel<P>::alb(a.albedo, idx, c[j]);
  }
  // lerp along x, then y, then z (corner j: bit0 x, bit1 y, bit2 z)
  float dx0 = lerpf_(d[0], d[1], f[0]), dx1 = lerpf_(d[2], d[3], f[0]);
  float dx2 = lerpf_(d[4], d[5], f[0]), dx3 = lerpf_(d[6], d[7], f[0]);
  s.sigma = lerpf_(lerpf_(dx0, dx1, f[1]), lerpf_(dx2, dx3, f[1]), f[2]);
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) {
    float x0 = lerpf_(c[0][ch], c[1][ch], f[0]), x1 = lerpf_(c[2][ch], c[3][ch], f[0]);
    float x2 = lerpf_(c[4][ch], c[5][ch], f[0]), x3 = lerpf_(c[6][ch], c[7][ch], f[0]);
    s.col[ch] = lerpf_(lerpf_(x0, x1, f[1]), lerpf_(x2, x3, f[1]), f[2]);
  }
  float al = fmul(s.sigma, a.alpha_scale);
  s.alpha = al < 0.f ? 0.f : (al > 1.f ? 1.f : al);
}

// Tree descent for brick cell `cell` (ntree/ntree/nodes.h:56-99 offsets).
// Top grid nodes come from shared memory.  Returns brick id, -1 if empty,
// -2 if the pool is malformed.
__device__ __forceinline__ int lookup(const VolumeArgs& a, const uint32_t* sg, uint32_t nsg,
                                      const int* cell) {
  uint32_t node = 0;
  for (int lev = 0; lev < a.levels; ++lev) {
    const int sh = 2 * (a.levels - 1 - lev);
    const uint32_t c = (uint32_t)((((cell[2] >> sh) & 3) * 4 + ((cell[1] >> sh) & 3)) * 4 +
                                  ((cell[0] >> sh) & 3));
    if (node >= a.ngrids) return -2;
    const uint32_t ref = node < nsg ? sg[node * 64 + c] : __ldg(a.grids + (size_t)node * 64 + c);
    if (ref & kEmpty) return -1;
    if (ref & kBrick) {
      const uint32_t b = ref & 0x3FFFFFFFu;
      return (lev == a.levels - 1 && b < a.nbricks) ? (int)b : -2;
    }
    if (lev == a.levels - 1) return -2;
    node = ref;
  }
  return -1;
}

struct RayOut {
  float c[3];
  float a;
  uint32_t samples;
  uint32_t bricks;
  bool bad;
};

// One ray; `Vis` is called per sample with (sample, T, C before).
template <int P, class Vis>
__device__ __forceinline__ void march(const VolumeArgs& a, const uint32_t* sg, uint32_t nsg,
                                      const float* o, const float* d, Vis& vis, RayOut& r) {
  r.c[0] = r.c[1] = r.c[2] = 0.f;
  r.a = 0.f;
  r.samples = 0;
  r.bricks = 0;
  r.bad = false;
  float inv[3], t1[3], t2[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    inv[i] = __fdiv_rn(1.f, d[i]);
    const float lo = fmul(fsub(0.f, o[i]), inv[i]);
    const float hi = fmul(fsub(1.f, o[i]), inv[i]);
    t1[i] = lo < hi ? lo : hi;
    t2[i] = lo < hi ? hi : lo;
  }
  float t_enter = fmaxf(fmaxf(t1[0], t1[1]), t1[2]);
  const float t_exit = fminf(fminf(t2[0], t2[1]), t2[2]);
  if (t_enter < 0.f) t_enter = 0.f;
  if (t_exit < 0.f || t_enter > t_exit) return;
  const float h = a.cell_size;  // world size of a brick cell
  int cell[3], step[3];
  float Q[3], D[3];  // lattice-space origin and direction
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float q = __fdiv_rn(fadd(o[i], fmul(t_enter, d[i])), h);
    int k = __float2int_rd(q);
    k = k < 0 ? 0 : (k > a.nb - 1 ? a.nb - 1 : k);
    cell[i] = k;
    step[i] = d[i] > 0.f ? 1 : -1;
    Q[i] = fmul(o[i], a.S);
    D[i] = fmul(d[i], a.S);
  }
  float t_in = t_enter;
  float A = 0.f, C0 = 0.f, C1 = 0.f, C2 = 0.f;
  for (int guard = 0; guard < 4 * 4096; ++guard) {
    float tx[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float plane = fmul((float)(d[i] > 0.f ? cell[i] + 1 : cell[i]), h);
      tx[i] = fmul(fsub(plane, o[i]), inv[i]);
    }
    int e = 0;
    if (tx[1] < tx[e]) e = 1;
    if (tx[2] < tx[e]) e = 2;
    const float t_out = tx[e];
    const int b = lookup(a, sg, nsg, cell);
    if (b == -2) {
      r.bad = true;
      break;
    }
    if (b >= 0) {
      ++r.bricks;
      // Q - 8c is exact (8c is a multiple of ulp(Q)), so fma(t, D, Q - 8c)
      // rounds the brick-local coordinate in [0, 8] once: the sample point
      // is accurate to ulp(8) instead of ulp(|Q|).
      const float L0 = fsub(Q[0], (float)(8 * cell[0]));
      const float L1 = fsub(Q[1], (float)(8 * cell[1]));
      const float L2 = fsub(Q[2], (float)(8 * cell[2]));
      int k = __float2int_ru(fmul(t_in, a.inv_dt));
      for (int it = 0; it < 1 << 16; ++it, ++k) {
        const float t = fmul((float)k, a.dt);
        if (!(t < t_out)) break;
        SampleCtx s;
        eval_sample<P>(a, b, ffma(t, D[0], L0), ffma(t, D[1], L1), ffma(t, D[2], L2), s);
        const float T = fsub(1.f, A);
        vis(s, T, A, C0, C1, C2);
        const float w = fmul(T, s.alpha);
        C0 = ffma(w, s.col[0], C0);
        C1 = ffma(w, s.col[1], C1);
        C2 = ffma(w, s.col[2], C2);
        A = fadd(A, w);
        ++r.samples;
        if (A > 0.99f) goto done;
      }
    }
    t_in = t_out;
    cell[e] += step[e];
    if (cell[e] < 0 || cell[e] >= a.nb) break;
  }
done:
  r.c[0] = C0;
  r.c[1] = C1;
  r.c[2] = C2;
  r.a = A;
}

struct NoVis {
  __device__ __forceinline__ void operator()(const SampleCtx&, float, float, float, float,
                                             float) {}
};

__device__ __forceinline__ void pixel_ray(const VolumeArgs& a, int cam, int x, int y, float* o,
                                          float* d) {
  const CamBasis& c = a.cam[cam];
  const float fx = (float)x, fy = (float)y;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    o[i] = c.pos[i];
    d[i] = fadd(fadd(c.dir0[i], fmul(c.du[i], fx)), fmul(c.dv[i], fy));
  }
  const float len = __fsqrt_rn(fadd(fadd(fmul(d[0], d[0]), fmul(d[1], d[1])), fmul(d[2], d[2])));
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    d[i] = __fdiv_rn(d[i], len);
    if (fabsf(d[i]) < 1e-5f) d[i] = copysignf(1e-5f, d[i]);
  }
}

// tile mapping: warp w of the grid -> 8x4 pixel tile of one camera image
__device__ __forceinline__ bool ray_of_thread(const VolumeArgs& a, uint32_t tile, int& cam,
                                              int& x, int& y) {
  const int tx = (a.width + 7) >> 3, ty = (a.height + 3) >> 2;
  const uint32_t per_cam = (uint32_t)(tx * ty);
  cam = (int)(tile / per_cam);
  const uint32_t t = tile % per_cam;
  const int lane = threadIdx.x & 31;
  x = (int)(t % (uint32_t)tx) * 8 + (lane & 7);
  y = (int)(t / (uint32_t)tx) * 4 + (lane >> 3);
  return cam < a.ncams && x < a.width && y < a.height;
}

__device__ __forceinline__ uint32_t stage_grids(const VolumeArgs& a, uint32_t* sg) {
  const uint32_t nsg = a.ngrids < (uint32_t)kSmemGrids ? a.ngrids : (uint32_t)kSmemGrids;
  for (uint32_t i = threadIdx.x; i < nsg * 64; i += blockDim.x) sg[i] = __ldg(a.grids + i);
  __syncthreads();
  return nsg;
}

template <int P>
__global__ void __launch_bounds__(256) volume_forward_kernel(VolumeArgs a) {
  __shared__ uint32_t sg[kSmemGrids * 64];
  const uint32_t nsg = stage_grids(a, sg);
  const uint32_t n_tiles = (uint32_t)a.ncams * (uint32_t)(((a.width + 7) >> 3) * ((a.height + 3) >> 2));
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  bool bad = false;
  for (uint32_t tile = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); tile < n_tiles;
       tile += warps) {
    int cam, x, y;
    if (!ray_of_thread(a, tile, cam, x, y)) continue;
    float o[3], d[3];
    pixel_ray(a, cam, x, y, o, d);
    NoVis nv;
    RayOut r;
    march<P>(a, sg, nsg, o, d, nv, r);
    bad |= r.bad;
    const size_t off = ((size_t)cam * a.height + (size_t)y) * a.width + (size_t)x;
    if (a.rgba) reinterpret_cast<float4*>(a.rgba)[off] = make_float4(r.c[0], r.c[1], r.c[2], r.a);
    if (a.samples) a.samples[off] = r.samples;
    if (a.bricks_entered) a.bricks_entered[off] = r.bricks;
  }
  if (bad && a.status) atomicOr(a.status, 4u);
}

// Per-lane coalescing of corner gradients while consecutive samples share
// a trilinear cell; flushed with atomics.
struct GradVis {
  const VolumeArgs* a;
  float g[4];    // dL/d(r,g,b,a) of this ray
  float out[4];  // forward output of this ray
  uint32_t base;
  float gd[8];
  float ga[8][3];
  __device__ __forceinline__ void flush() {
    if (base == 0xFFFFFFFFu) return;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint32_t idx = base + (uint32_t)(((j >> 2) * kL + ((j >> 1) & 1)) * kL + (j & 1));
      if (gd[j] != 0.f) atomicAdd(a->grad_density + idx, gd[j]);
#pragma unroll
      for (int ch = 0; ch < 3; ++ch)
        if (ga[j][ch] != 0.f) atomicAdd(a->grad_albedo + 3 * (size_t)idx + ch, ga[j][ch]);
      gd[j] = 0.f;
      ga[j][0] = ga[j][1] = ga[j][2] = 0.f;
    }
  }
  __device__ __forceinline__ void operator()(const SampleCtx& s, float T, float A, float C0,
                                             float C1, float C2) {
    if (s.base != base) {
      flush();
      base = s.base;
    }
    const float w = fmul(T, s.alpha);
    const float om = fsub(1.f, s.alpha);
    const float Cb[3] = {C0, C1, C2};
    float dal = 0.f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float ck = k < 3 ? s.col[k] : 1.f;
      const float before = k < 3 ? Cb[k] : A;
      const float after = k < 3 ? ffma(w, ck, before) : fadd(A, w);
      float term = fmul(T, ck);
      if (om > 0.f) term = fsub(term, __fdiv_rn(fsub(out[k], after), om));
      dal = ffma(g[k], term, dal);
    }
    const float sa = fmul(s.sigma, a->alpha_scale);
    // saturate'(s) = 1 on [0, 1): right derivative at 0 so that empty lattice
    // points still receive gradient
    const float dsig = (sa >= 0.f && sa < 1.f) ? fmul(dal, a->alpha_scale) : 0.f;
    const float wx[2] = {fsub(1.f, s.fx), s.fx};
    const float wy[2] = {fsub(1.f, s.fy), s.fy};
    const float wz[2] = {fsub(1.f, s.fz), s.fz};
    const float gc[3] = {fmul(g[0], w), fmul(g[1], w), fmul(g[2], w)};
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const float wj = fmul(fmul(wx[j & 1], wy[(j >> 1) & 1]), wz[j >> 2]);
      gd[j] = ffma(wj, dsig, gd[j]);
#pragma unroll
      for (int ch = 0; ch < 3; ++ch) ga[j][ch] = ffma(wj, gc[ch], ga[j][ch]);
    }
  }
};

template <int P>
__global__ void __launch_bounds__(256) volume_backward_kernel(VolumeArgs a) {
  __shared__ uint32_t sg[kSmemGrids * 64];
  const uint32_t nsg = stage_grids(a, sg);
  const uint32_t n_tiles = (uint32_t)a.ncams * (uint32_t)(((a.width + 7) >> 3) * ((a.height + 3) >> 2));
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  bool bad = false;
  for (uint32_t tile = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); tile < n_tiles;
       tile += warps) {
    int cam, x, y;
    if (!ray_of_thread(a, tile, cam, x, y)) continue;
    const size_t off = ((size_t)cam * a.height + (size_t)y) * a.width + (size_t)x;
    const float4 g4 = reinterpret_cast<const float4*>(a.grad_rgba)[off];
    if (g4.x == 0.f && g4.y == 0.f && g4.z == 0.f && g4.w == 0.f) continue;
    const float4 o4 = reinterpret_cast<const float4*>(a.rgba_fwd)[off];
    float o[3], d[3];
    pixel_ray(a, cam, x, y, o, d);
    GradVis gv;
    gv.a = &a;
    gv.g[0] = g4.x; gv.g[1] = g4.y; gv.g[2] = g4.z; gv.g[3] = g4.w;
    gv.out[0] = o4.x; gv.out[1] = o4.y; gv.out[2] = o4.z; gv.out[3] = o4.w;
    gv.base = 0xFFFFFFFFu;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      gv.gd[j] = 0.f;
      gv.ga[j][0] = gv.ga[j][1] = gv.ga[j][2] = 0.f;
    }
    RayOut r;
    march<P>(a, sg, nsg, o, d, gv, r);
    gv.flush();
    bad |= r.bad;
  }
  if (bad && a.status) atomicOr(a.status, 4u);
}

// Apron fold, pass 1: every owned lattice point (x,y,z < 8) adds the
// gradient its copies received in the aprons of the lower neighbours.
__global__ void fold_gather_kernel(VolumeArgs a, int channels, float* g) {
  const uint32_t n = a.nbricks * 512u;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t b = i >> 9, p = i & 511u;
    const int x = (int)(p & 7u), y = (int)((p >> 3) & 7u), z = (int)(p >> 6);
    const uint32_t own = b * kL3 + (uint32_t)((z * kL + y) * kL + x);
    for (int ch = 0; ch < channels; ++ch) {
      float s = g[(size_t)own * channels + ch];
      for (int m = 1; m < 8; ++m) {
        const int dx = m & 1, dy = (m >> 1) & 1, dz = m >> 2;
        if ((dx && x) || (dy && y) || (dz && z)) continue;
        const int nb = a.nbr_dn[(size_t)b * 7 + (m - 1)];
        if (nb < 0) continue;
        const uint32_t cp = (uint32_t)nb * kL3 +
                            (uint32_t)(((z + 8 * dz) * kL + (y + 8 * dy)) * kL + (x + 8 * dx));
        s += g[(size_t)cp * channels + ch];
      }
      g[(size_t)own * channels + ch] = s;
    }
  }
}

// Apron fold, pass 2 (also the apron sync of parameters): every apron slot
// takes the value of the lattice point's owner, or 0 if the owner is absent.
__global__ void fold_scatter_kernel(VolumeArgs a, int channels, float* g) {
  const uint32_t n = a.nbricks * (uint32_t)kL3;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t b = i / kL3, p = i % kL3;
    const int x = (int)(p % kL), y = (int)((p / kL) % kL), z = (int)(p / (kL * kL));
    const int dx = x == 8, dy = y == 8, dz = z == 8;
    const int m = dx | (dy << 1) | (dz << 2);
    if (!m) continue;
    const int own = a.nbr_up[(size_t)b * 7 + (m - 1)];
    const uint32_t src = (uint32_t)own * kL3 +
                         (uint32_t)(((z - 8 * dz) * kL + (y - 8 * dy)) * kL + (x - 8 * dx));
    for (int ch = 0; ch < channels; ++ch)
      g[(size_t)i * channels + ch] = own >= 0 ? g[(size_t)src * channels + ch] : 0.f;
  }
}

}  // namespace

cudaError_t launch_volume_forward(const VolumeArgs& a, cudaStream_t s) {
  const uint32_t tiles = (uint32_t)a.ncams * (uint32_t)(((a.width + 7) >> 3) * ((a.height + 3) >> 2));
  const uint32_t blocks = (tiles + 7) / 8;
  if (blocks == 0) return cudaSuccess;
  if (a.precision == 0)
    volume_forward_kernel<0><<<blocks, 256, 0, s>>>(a);
  else
    volume_forward_kernel<1><<<blocks, 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_volume_backward(const VolumeArgs& a, cudaStream_t s) {
  const uint32_t tiles = (uint32_t)a.ncams * (uint32_t)(((a.width + 7) >> 3) * ((a.height + 3) >> 2));
  const uint32_t blocks = (tiles + 7) / 8;
  if (blocks == 0) return cudaSuccess;
  if (a.precision == 0)
    volume_backward_kernel<0><<<blocks, 256, 0, s>>>(a);
  else
    volume_backward_kernel<1><<<blocks, 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_apron_fold(const VolumeArgs& a, int channels, float* g, bool gather,
                              cudaStream_t s) {
  if (a.nbricks == 0) return cudaSuccess;
  const int blocks = 2 * device_sm_count_vol() * 8;
  if (gather) fold_gather_kernel<<<blocks, 256, 0, s>>>(a, channels, g);
  fold_scatter_kernel<<<blocks, 256, 0, s>>>(a, channels, g);
  return cudaGetLastError();
}

int device_sm_count_vol() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
    n = 1;
  return n;
}

}  // namespace yv
