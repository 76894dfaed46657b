// brick_march.cuh - device code of the brick-volume ray-march (ntree layout)
// for sm_103a, shared by brick_kernels.cu and batch_kernels.cu.
//
// March (restating castRay / walkBrick / intersect of
// reaction/trace/trace.cu:42-139 over the N=4 grid tree of volume_host.cpp):
//  * clip the ray to the unit cube, t_enter = max(t_enter, 0);
//  * DDA over brick cells; cell c spans [t_in, t_out) with t_in = the
//    previous cell's t_out, so cells partition the ray;
//  * in an occupied cell, samples sit at the global multiples t = k*dt
//    (trace.cu:47), dt = step_vox lattice cells;
//  * sample = software FP32 trilinear of density and albedo inside the brick
//    (the 9^3 apron lattice keeps all 8 corners in the brick), at a position
//    carried as a float pair (sample_coord) so the trilinear fractions are
//    accurate to ulp(1);
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
// with one 16-byte FP32 vector atomic per corner (brick_kernels.cu).
#pragma once
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

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float lerpf_(float a, float b, float t) { return ffma(t, fsub(b, a), a); }

// Exact conversions on the ALU / FMA pipes instead of the conversion unit
// (which runs at a fraction of their rate); used where they measured faster
// (the 8-byte packed format).
// Byte k of v as a float: 2^23 + byte assembled by one byte permute, minus
// 2^23 (exact).
__device__ __forceinline__ float byte_f(uint32_t v, int k) {
  return __fsub_rn(__uint_as_float(__byte_perm(v, 0x4B000000u, 0x7440u + (uint32_t)k)),
                   8388608.f);
}
// 0 <= n < 2^23 as a float (exact).
__device__ __forceinline__ float small_int_f(int n) {
  return __fsub_rn(__uint_as_float(0x4B000000u | (uint32_t)n), 8388608.f);
}
// Finite binary16 in the low 16 bits of h as a float: the half's exponent
// and mantissa bits placed in a float (a subnormal for every half) and
// scaled by 2^112, exact for normal and subnormal halves alike.  The fp16
// lattice formats hold finite values only (the upload saturates).
__device__ __forceinline__ float half_bits_f(uint32_t h) {
  const uint32_t m = ((h & 0x7FFFu) << 13) | ((h & 0x8000u) << 16);
  return __fmul_rn(__uint_as_float(m), __uint_as_float(0x77800000u));  // x 2^112
}

template <int P>
struct Voxel;

// Lattice formats (VolumeView::precision).  corner() loads one lattice
// point: density and the three albedo channels (raw 0..255 for the uint8
// formats, scaled once after interpolation by kAlbedoScale).
//   0: fp16 density array + uchar4 albedo array (two loads)
//   1: fp32 density array + fp32 RGB albedo array (learnable; four loads)
//   2: packed float4 (r, g, b, density) (one 16-byte load)
//   3: packed 8 bytes {fp16 density | r << 16 | g << 24, b} (one 8-byte load)
template <>
struct Voxel<0> {
  static constexpr float kAlbedoScale = 1.0f / 255.0f;
  __device__ static __forceinline__ void corner(const VolumeView& a, uint32_t i, float& d,
                                                float* c) {
    d = __half2float(__ushort_as_half(__ldg(static_cast<const unsigned short*>(a.density) + i)));
    const uint32_t v = __ldg(static_cast<const unsigned int*>(a.albedo) + i);
    c[0] = (float)(v & 0xFFu);
    c[1] = (float)((v >> 8) & 0xFFu);
    c[2] = (float)((v >> 16) & 0xFFu);
  }
};

template <>
struct Voxel<1> {
  static constexpr float kAlbedoScale = 1.0f;
  __device__ static __forceinline__ void corner(const VolumeView& a, uint32_t i, float& d,
                                                float* c) {
    d = __ldg(static_cast<const float*>(a.density) + i);
    const float* q = static_cast<const float*>(a.albedo) + 3 * (size_t)i;
    c[0] = __ldg(q);
    c[1] = __ldg(q + 1);
    c[2] = __ldg(q + 2);
  }
};

template <>
struct Voxel<2> {
  static constexpr float kAlbedoScale = 1.0f;
  __device__ static __forceinline__ void corner(const VolumeView& a, uint32_t i, float& d,
                                                float* c) {
    const float4 v = __ldg(static_cast<const float4*>(a.albedo) + i);
    c[0] = v.x;
    c[1] = v.y;
    c[2] = v.z;
    d = v.w;
  }
};

template <>
struct Voxel<3> {
  static constexpr float kAlbedoScale = 1.0f / 255.0f;
  __device__ static __forceinline__ void corner(const VolumeView& a, uint32_t i, float& d,
                                                float* c) {
    const uint2 v = __ldg(static_cast<const uint2*>(a.albedo) + i);
    d = half_bits_f(v.x);
    c[0] = byte_f(v.x, 2);
    c[1] = byte_f(v.x, 3);
    c[2] = byte_f(v.y, 0);
  }
};

struct SampleCtx {
  uint32_t base;  // brick*729 + corner-000 lattice index
  int brick;      // brick and brick-local corner-000 lattice coordinates
  int cell[3];
  float f[3];     // fractional position inside the trilinear cell
  float w[8];     // trilinear weights, corner j: bit0 +x, bit1 +y, bit2 +z
  float sigma, alpha;
  float col[3];
};

// Lattice offset of trilinear corner j inside a 9^3 brick.
__device__ __forceinline__ uint32_t corner_offset(int j) {
  return (uint32_t)(((j >> 2) * kL + ((j >> 1) & 1)) * kL + (j & 1));
}

// a + b as an exact float pair s + r (Knuth's TwoSum).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& r) {
  s = fadd(a, b);
  const float bb = fsub(s, a);
  r = fadd(fsub(a, fsub(s, bb)), fsub(b, bb));
}

// Brick-local lattice coordinate t D + (Lh + Ll) of a sample (in [0, 8]),
// Lh + Ll the brick-local origin o S - 8c as an exact pair (two_sum: o S is
// exact, but o S - 8c can need one bit more when it grows a binade), as a
// float pair l + e: p = t D rounded, e = its exact rounding error (one fma)
// plus Ll, l = p + Lh.  Once the origin is more than two bricks away, p and
// -Lh agree to a factor of two and l is exact (Sterbenz), so the fractional
// position inside the trilinear cell, (l - k) + e, is accurate to ulp(1)
// instead of ulp(8) or ulp(o S).  (Rounded once to ulp(8), and o S - 8c to
// ulp(o S), sample points on steep density edges moved low-opacity rays by
// up to 5e-5 relative.)
__device__ __forceinline__ void sample_coord(float t, float D, float Lh, float Ll, float& l,
                                             float& e) {
  const float p = fmul(t, D);
  e = fadd(ffma(t, D, -p), Ll);
  l = fadd(p, Lh);
}

// l + e: brick-local lattice coordinates of the sample (sample_coord), in
// [0, 8].
template <int P>
__device__ __forceinline__ void eval_sample(const VolumeView& a, int b, const float* l,
                                            const float* e, SampleCtx& s) {
  int i0[3];
  float f[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    int k = __float2int_rd(l[i]);
    k = k < 0 ? 0 : (k > 7 ? 7 : k);
    float fi = fadd(fsub(l[i], small_int_f(k)), e[i]);
    fi = fi < 0.f ? 0.f : (fi > 1.f ? 1.f : fi);
    i0[i] = k;
    f[i] = fi;
  }
  s.base = (uint32_t)b * (uint32_t)kL3 + (uint32_t)((i0[2] * kL + i0[1]) * kL + i0[0]);
  s.brick = b;
  s.cell[0] = i0[0];
  s.cell[1] = i0[1];
  s.cell[2] = i0[2];
  s.f[0] = f[0];
  s.f[1] = f[1];
  s.f[2] = f[2];
  const float gx = fsub(1.f, f[0]), gy = fsub(1.f, f[1]), gz = fsub(1.f, f[2]);
  const float w00 = fmul(gx, gy), w10 = fmul(f[0], gy), w01 = fmul(gx, f[1]),
              w11 = fmul(f[0], f[1]);
  s.w[0] = fmul(w00, gz);
  s.w[1] = fmul(w10, gz);
  s.w[2] = fmul(w01, gz);
  s.w[3] = fmul(w11, gz);
  s.w[4] = fmul(w00, f[2]);
  s.w[5] = fmul(w10, f[2]);
  s.w[6] = fmul(w01, f[2]);
  s.w[7] = fmul(w11, f[2]);
  float sig = 0.f, c0 = 0.f, c1 = 0.f, c2 = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float dj, c[3];
    Voxel<P>::corner(a, s.base + corner_offset(j), dj, c);
    sig = ffma(s.w[j], dj, sig);
    c0 = ffma(s.w[j], c[0], c0);
    c1 = ffma(s.w[j], c[1], c1);
    c2 = ffma(s.w[j], c[2], c2);
  }
  s.sigma = sig;
  s.col[0] = fmul(c0, Voxel<P>::kAlbedoScale);
  s.col[1] = fmul(c1, Voxel<P>::kAlbedoScale);
  s.col[2] = fmul(c2, Voxel<P>::kAlbedoScale);
  float al = fmul(s.sigma, a.alpha_scale);
  s.alpha = al < 0.f ? 0.f : (al > 1.f ? 1.f : al);
}

// Tree descent for brick cell `cell` (ntree/ntree/nodes.h:56-99 offsets).
// Grid nodes below nsg come from sg (a shared-memory copy; the kernels pass
// none and read every node through L1).  Returns brick id, -1 if empty,
// -2 if the pool is malformed.
__device__ __forceinline__ int lookup(const VolumeView& a, const uint32_t* sg, uint32_t nsg,
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

// One ray; `Vis` is called per sample with (sample, T, T alpha, A and C
// before the sample).
// kColor = false (the adjoint's replay): the composited colour is not
// accumulated (the visitor tracks what it needs; r.c stays 0).
// kSkip: the forward passes over the samples of cells the pool's
// cell_mask marks empty (compiled out for pools without one).
template <int P, class Vis, bool kColor = true, bool kSkip = kColor>
__device__ __forceinline__ void march(const VolumeView& a, const uint32_t* sg, uint32_t nsg,
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
  // The replay (kColor = false) keeps less live state for its tighter
  // register budget: the step direction of an axis is the sign of inv (d is
  // never 0), and the lattice-space origin o S is recomputed (the same
  // rounded product) at each occupied cell (cfg4 adjoint 7.10 -> 6.83 ms;
  // the forward measured faster holding them).
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
      const bool up = kColor ? d[i] > 0.f : inv[i] > 0.f;
      const float plane = fmul((float)(up ? cell[i] + 1 : cell[i]), h);
      tx[i] = fmul(fsub(plane, o[i]), inv[i]);
    }
    // exit axis = first argmin (selects, no dynamic register indexing)
    int e = 0;
    float t_out = tx[0];
    if (tx[1] < t_out) { e = 1; t_out = tx[1]; }
    if (tx[2] < t_out) { e = 2; t_out = tx[2]; }
    int b = -1;
    {
      // the tree is descended only where the brick bitmap (if any) says a
      // brick may be
      const uint32_t ci =
          ((uint32_t)cell[2] * (uint32_t)a.nb + (uint32_t)cell[1]) * (uint32_t)a.nb +
          (uint32_t)cell[0];
      if (!a.brick_bits || ((__ldg(a.brick_bits + (ci >> 5)) >> (ci & 31u)) & 1u))
        b = lookup(a, sg, nsg, cell);
    }
    if (b == -2) {
      r.bad = true;
      break;
    }
    if (b >= 0) {
      ++r.bricks;
      // the brick-local origin Q - 8c as an exact pair: the brick-local
      // coordinate t D + (Q - 8c) in [0, 8] is formed without the rounding
      // of |Q| (sample_coord)
      float Lh[3], Ll[3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
        two_sum(kColor ? Q[i] : fmul(o[i], a.S), -(float)(8 * cell[i]), Lh[i], Ll[i]);
      int k = __float2int_ru(fmul(t_in, a.inv_dt));
      for (int it = 0; it < 1 << 16; ++it, ++k) {
        const float t = fmul((float)k, a.dt);
        if (!(t < t_out)) break;
        float lc[3], le[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) sample_coord(t, D[i], Lh[i], Ll[i], lc[i], le[i]);
        if (kColor && kSkip && a.cell_mask) {
          // a cell whose 8 corners are all zero has sigma = 0, alpha = 0:
          // the sample adds exactly nothing (C, A unchanged), so the
          // forward passes over it; the replay of the adjoint, whose
          // density gradient reaches such samples, takes every sample
          int kc[3];
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            const int kk = __float2int_rd(lc[i]);
            kc[i] = kk < 0 ? 0 : (kk > 7 ? 7 : kk);
          }
          const uint32_t mw = __ldg(a.cell_mask + (size_t)b * 16u + (uint32_t)(kc[2] * 2 + (kc[1] >> 2)));
          if (!((mw >> (((kc[1] & 3) << 3) | kc[0])) & 1u)) {
            ++r.samples;
            continue;
          }
        }
        SampleCtx s;
        eval_sample<P>(a, b, lc, le, s);
        const float T = fsub(1.f, A);
        const float w = fmul(T, s.alpha);
        vis(s, T, w, A, C0, C1, C2);
        if (kColor) {
          C0 = ffma(w, s.col[0], C0);
          C1 = ffma(w, s.col[1], C1);
          C2 = ffma(w, s.col[2], C2);
        }
        A = fadd(A, w);
        ++r.samples;
        if (A > 0.99f) goto done;
      }
    }
    t_in = t_out;
    int ce;
    if (e == 0) ce = (cell[0] += kColor ? step[0] : (inv[0] > 0.f ? 1 : -1));
    else if (e == 1) ce = (cell[1] += kColor ? step[1] : (inv[1] > 0.f ? 1 : -1));
    else ce = (cell[2] += kColor ? step[2] : (inv[2] > 0.f ? 1 : -1));
    if (ce < 0 || ce >= a.nb) break;
  }
done:
  r.c[0] = C0;
  r.c[1] = C1;
  r.c[2] = C2;
  r.a = A;
}

struct NoVis {
  __device__ __forceinline__ void operator()(const SampleCtx&, float, float, float, float, float,
                                             float) {}
};

__device__ __forceinline__ void pixel_ray(const CamBasis& c, int x, int y, float* o, float* d) {
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

}  // namespace
}  // namespace yv
