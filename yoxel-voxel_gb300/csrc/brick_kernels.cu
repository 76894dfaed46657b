// brick_kernels.cu - brick-volume ray-march kernels (ntree layout) for
// sm_103a: forward compositing over many cameras, the re-marching adjoint,
// and apron maintenance.  Device helpers and the march are in
// brick_march.cuh.
#include "brick_march.cuh"

namespace yv {
namespace {

// Register budget of the adjoint (resident blocks of 256 per SM): its 16
// per-lane gradient accumulators live in registers (a shared-memory copy
// measured 1.25x slower).
constexpr int kBackwardMinBlocks = 3;
// Register budget of the forward march per lattice format: the fp16 +
// 8-bit colour formats (0, 3) run at 3 resident blocks (74 registers for the
// 8-byte format: 1.19 ms on the 1024^2 frame of a 512^3 volume, against 1.26
// ms at 4 blocks / 64 registers and 1.43 ms at 5 / 48 with spills); the fp32
// formats (1, 2) at 4 (the 64-camera 128^3 forward: 3.19 ms at 4 blocks,
// 3.29 ms at 3).  Measured while the grid nodes were staged in shared
// memory; re-measured for the 8-byte format without staging: 904 / 843 /
// 754 Mrays/s at 3 / 4 / 5 blocks.
template <int P>
struct ForwardBlocks {
  static constexpr int value = (P == 0 || P == 3) ? 3 : 4;
};

// tile mapping: warp w of the grid -> 8x4 pixel tile of one camera image;
// the 8 warps of a block take a 2x4-tile (16x16-pixel) square
__host__ __device__ __forceinline__ uint32_t tile_ids(const VolumeArgs& a) {
  const uint32_t tx = (uint32_t)((a.width + 7) >> 3), ty = (uint32_t)((a.height + 3) >> 2);
  return (uint32_t)a.ncams * ((tx + 1) >> 1) * ((ty + 3) >> 2) * 8u;
}
__device__ __forceinline__ bool ray_of_thread(const VolumeArgs& a, uint32_t tile, int& cam,
                                              int& x, int& y) {
  const uint32_t tx = (uint32_t)((a.width + 7) >> 3), ty = (uint32_t)((a.height + 3) >> 2);
  const uint32_t stx = (tx + 1) >> 1, sty = (ty + 3) >> 2;
  const uint32_t per_cam = stx * sty * 8u;
  cam = (int)(tile / per_cam);
  const uint32_t r = tile % per_cam, st = r >> 3, w = r & 7u;
  const int lane = threadIdx.x & 31;
  x = (int)(((st % stx) * 2u + (w & 1u)) * 8u) + (lane & 7);
  y = (int)(((st / stx) * 4u + (w >> 1)) * 4u) + (lane >> 3);
  return cam < a.ncams && x < a.width && y < a.height;
}

// RGBA8 pixel of a composited colour: each channel saturate(v) * 255
// truncated, R in the low byte (float2uint of reaction/trace/utils.h:37-44,
// the uchar4 image of RunTrace, ntree/ntree_trace.cuh:27).
__device__ __forceinline__ uint32_t rgba8_of(float r, float g, float b, float al) {
  const float v[4] = {r, g, b, al};
  uint32_t out = 0;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const float x = v[c] < 0.f ? 0.f : (v[c] > 1.f ? 1.f : v[c]);
    out |= __float2uint_rz(__fmul_rn(x, 255.f)) << (8 * c);
  }
  return out;
}

// kMinBlocks: resident blocks of 256 per SM the register allocation is
// sized for.
// kSkip: the pool carries a cell occupancy mask (a learnable pool does not).
template <int P, int kMinBlocks, bool kSkip>
__global__ void __launch_bounds__(256, kMinBlocks) volume_forward_kernel(VolumeArgs a) {
  // grid nodes are read through L1 (see prefer_l1)
  const uint32_t* sg = nullptr;
  const uint32_t nsg = 0;
  // the launch's tiles (a range of them for a frame split across GPUs)
  const uint32_t n_tiles = a.tile_end ? a.tile_end : tile_ids(a);
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  bool bad = false;
  for (uint32_t tile = a.tile_begin + blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
       tile < n_tiles; tile += warps) {
    int cam, x, y;
    if (!ray_of_thread(a, tile, cam, x, y)) continue;
    float o[3], d[3];
    pixel_ray(a.cam[cam], x, y, o, d);
    NoVis nv;
    RayOut r;
    march<P, NoVis, true, kSkip>(a.v, sg, nsg, o, d, nv, r);
    bad |= r.bad;
    const size_t off = ((size_t)cam * a.height + (size_t)y) * a.width + (size_t)x;
    if (a.rgba) reinterpret_cast<float4*>(a.rgba)[off] = make_float4(r.c[0], r.c[1], r.c[2], r.a);
    if (a.rgba8) a.rgba8[off] = rgba8_of(r.c[0], r.c[1], r.c[2], r.a);
    if (a.samples) a.samples[off] = r.samples;
    if (a.bricks_entered) a.bricks_entered[off] = r.bricks;
  }
  if (bad && a.status) atomicOr(a.status, 4u);
}

// Gradient of one sample w.r.t. its alpha (see the header), contracted with
// dL/d(rgba) = g of the ray up front:
//   sum_k g_k d out_k / d alpha = T (g.c) - (g.out - g.C_after) / (1 - alpha)
// with c_A = 1, C_after = C_before + T alpha c, g.out a per-ray constant
// (gout) and gb = g.C_before tracked along the ray (so the replay need not
// composite the colour).  Returns d(sigma) through saturate.  The colour
// gradient of the sample is g_k T alpha: g is constant along the ray, so
// only T alpha needs accumulating per corner.
__device__ __forceinline__ float sample_dsigma(const VolumeArgs* a, float gc, float gout,
                                               float gb, const SampleCtx& s, float T,
                                               float w) {
  const float ga = ffma(w, gc, gb);
  const float om = fsub(1.f, s.alpha);
  // the gradient bar is 1e-4 relative: the hardware reciprocal suffices
  const float inv_om = om > 0.f ? __fdividef(1.f, om) : 0.f;
  const float dal = ffma(T, gc, -fmul(fsub(gout, ga), inv_om));
  const float sa = fmul(s.sigma, a->v.alpha_scale);
  // saturate'(s) = 1 on [0, 1): right derivative at 0 so that empty lattice
  // points still receive gradient
  return (sa >= 0.f && sa < 1.f) ? fmul(dal, a->v.alpha_scale) : 0.f;
}

// Per-lane coalescing of corner gradients while consecutive samples share
// a trilinear cell: per corner, sum w_j dsigma (density) and sum w_j T alpha
// (colour, scaled by g at the flush), flushed with one 16-byte vector atomic
// per corner into the packed (albedo rgb, density) gradient of the lattice
// point.  The first sample of a cell sets the accumulators.  (Carrying the 4
// shared corners over a face-adjacent move halves the atomics but measured
// 1.3x slower: the per-axis cases diverge within a warp.)
struct GradVis {
  const VolumeArgs* a;
  float g[4];   // dL/d(r,g,b,a) of this ray
  float gout;   // g . (forward output of this ray)
  float gb;     // g . (r, g, b, A) composited before the current sample
  uint32_t base;
  float gd[8];  // density
  float gw[8];  // colour weight
  __device__ __forceinline__ void init() {
    base = 0xFFFFFFFFu;
    gb = 0.f;
  }
  __device__ __forceinline__ void flush() {
    if (base == 0xFFFFFFFFu) return;
#pragma unroll
    for (int j = 0; j < 8; ++j)
      atomicAdd(a->grad_packed + base + corner_offset(j),
                make_float4(fmul(g[0], gw[j]), fmul(g[1], gw[j]), fmul(g[2], gw[j]), gd[j]));
  }
  __device__ __forceinline__ void operator()(const SampleCtx& s, float T, float w, float, float,
                                             float, float) {
    const float gc = ffma(g[2], s.col[2], ffma(g[1], s.col[1], ffma(g[0], s.col[0], g[3])));
    const float ds = sample_dsigma(a, gc, gout, gb, s, T, w);
    gb = ffma(w, gc, gb);
    if (s.base != base) {
      flush();
      base = s.base;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        gd[j] = fmul(s.w[j], ds);
        gw[j] = fmul(s.w[j], w);
      }
    } else {
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        gd[j] = ffma(s.w[j], ds, gd[j]);
        gw[j] = ffma(s.w[j], w, gw[j]);
      }
    }
  }
};

// kMinBlocks: register budget (resident blocks of 256 per SM).
template <int P, int kMinBlocks>
// grid nodes are read through L1 (see prefer_l1)
__global__ void __launch_bounds__(256, kMinBlocks) volume_backward_kernel(VolumeArgs a) {
  const uint32_t* sg = nullptr;
  const uint32_t nsg = 0;
  const uint32_t n_tiles = tile_ids(a);
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
    pixel_ray(a.cam[cam], x, y, o, d);
    GradVis gv;
    gv.a = &a;
    gv.g[0] = g4.x; gv.g[1] = g4.y; gv.g[2] = g4.z; gv.g[3] = g4.w;
    gv.gout = ffma(g4.w, o4.w, ffma(g4.z, o4.z, ffma(g4.y, o4.y, fmul(g4.x, o4.x))));
    gv.init();
    RayOut r;
    march<P, GradVis, false>(a.v, sg, nsg, o, d, gv, r);
    gv.flush();
    bad |= r.bad;
  }
  if (bad && a.status) atomicOr(a.status, 4u);
}

// Cell occupancy mask: one warp per mask word - the 32 cells (x, y) of four
// rows of one z layer of a brick - sets the bit of every cell with a
// non-zero density corner, as the march reads the corners (format P).
template <int P>
__global__ void cell_mask_kernel(VolumeView v, uint32_t* mask) {
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= v.nbricks * 16u) return;  // uniform across the warp
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t b = warp >> 4, word = warp & 15u;
  const uint32_t z = word >> 1, y = (word & 1u) * 4u + (lane >> 3), x = lane & 7u;
  const uint32_t base = b * (uint32_t)kL3 + (z * kL + y) * kL + x;
  bool any = false;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float d, c[3];
    Voxel<P>::corner(v, base + corner_offset(j), d, c);
    any |= d != 0.f;
  }
  const uint32_t bits = __ballot_sync(0xFFFFFFFFu, any);
  if (lane == 0) mask[warp] = bits;
}

// Brick bitmap: one warp per word of 32 brick cells, a lane per cell, its
// bit set unless the tree descent finds the cell empty (a malformed ref
// keeps its bit, so the march's own descent still reports it).
__global__ void brick_bits_kernel(VolumeView v, uint32_t* bits, uint32_t nwords) {
  const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= nwords) return;  // uniform across the warp
  const uint32_t nb = (uint32_t)v.nb, n = nb * nb * nb;
  const uint32_t ci = w * 32u + (threadIdx.x & 31u);
  bool set = false;
  if (ci < n) {
    const int cell[3] = {(int)(ci % nb), (int)((ci / nb) % nb), (int)(ci / (nb * nb))};
    set = lookup(v, nullptr, 0u, cell) != -1;
  }
  const uint32_t word = __ballot_sync(0xFFFFFFFFu, set);
  if ((threadIdx.x & 31u) == 0) bits[w] = word;
}

// Apron fold, pass 1: every owned lattice point (x,y,z < 8) adds the
// gradient its copies received in the aprons of the lower neighbours.
__global__ void fold_gather_kernel(VolumeArgs a, int channels, float* g) {
  const uint32_t n = a.v.nbricks * 512u;
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
  const uint32_t n = a.v.nbricks * (uint32_t)kL3;
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

// The march reads the lattice and the grid nodes through L1, and the
// kernels use no shared memory, so they ask for the largest L1 (carveout 0).
// Measured against staging the root and level-1 grid nodes (16.6 KB a
// block) under the driver's default carveout: 64-camera 128^3 forward
// 1365 -> 1434 Mrays/s and adjoint 6.65 -> 6.40 ms; 512^3 fp16 + RGB8
// frame 875 -> 907 Mrays/s (the lowest carveout that still held the staged
// nodes gave half of these gains).
void prefer_l1() {
  static bool done[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64 || done[dev]) return;
  const cudaFuncAttribute k = cudaFuncAttributePreferredSharedMemoryCarveout;
  const cudaError_t e[10] = {
      cudaFuncSetAttribute(volume_forward_kernel<0, ForwardBlocks<0>::value, false>, k, 0),
      cudaFuncSetAttribute(volume_forward_kernel<0, ForwardBlocks<0>::value, true>, k, 0),
      cudaFuncSetAttribute(volume_forward_kernel<1, ForwardBlocks<1>::value, false>, k, 0),
      cudaFuncSetAttribute(volume_forward_kernel<1, ForwardBlocks<1>::value, true>, k, 0),
      cudaFuncSetAttribute(volume_forward_kernel<2, ForwardBlocks<2>::value, false>, k, 0),
      cudaFuncSetAttribute(volume_forward_kernel<2, ForwardBlocks<2>::value, true>, k, 0),
      cudaFuncSetAttribute(volume_forward_kernel<3, ForwardBlocks<3>::value, false>, k, 0),
      cudaFuncSetAttribute(volume_forward_kernel<3, ForwardBlocks<3>::value, true>, k, 0),
      cudaFuncSetAttribute(volume_backward_kernel<1, kBackwardMinBlocks>, k, 0),
      cudaFuncSetAttribute(volume_backward_kernel<2, kBackwardMinBlocks>, k, 0)};
  // a hint: a refusal keeps the default configuration and is not reported
  // as the next launch's error
  for (cudaError_t x : e)
    if (x != cudaSuccess) {
      cudaGetLastError();
      break;
    }
  done[dev] = true;
}

}  // namespace

uint32_t volume_tiles_per_camera(int width, int height) {
  const uint32_t tx = (uint32_t)((width + 7) >> 3), ty = (uint32_t)((height + 3) >> 2);
  return ((tx + 1) >> 1) * ((ty + 3) >> 2) * 8u;
}

cudaError_t launch_volume_forward(const VolumeArgs& a, cudaStream_t s) {
  const uint32_t end = a.tile_end ? a.tile_end : tile_ids(a);
  const uint32_t tiles = end > a.tile_begin ? end - a.tile_begin : 0u;
  const uint32_t blocks = (tiles + 7) / 8;
  if (blocks == 0) return cudaSuccess;
  prefer_l1();
  const bool skip = a.v.cell_mask != nullptr;
  switch (a.v.precision) {
    case 0:
      if (skip)
        volume_forward_kernel<0, ForwardBlocks<0>::value, true><<<blocks, 256, 0, s>>>(a);
      else
        volume_forward_kernel<0, ForwardBlocks<0>::value, false><<<blocks, 256, 0, s>>>(a);
      break;
    case 1:
      if (skip)
        volume_forward_kernel<1, ForwardBlocks<1>::value, true><<<blocks, 256, 0, s>>>(a);
      else
        volume_forward_kernel<1, ForwardBlocks<1>::value, false><<<blocks, 256, 0, s>>>(a);
      break;
    case 2:
      if (skip)
        volume_forward_kernel<2, ForwardBlocks<2>::value, true><<<blocks, 256, 0, s>>>(a);
      else
        volume_forward_kernel<2, ForwardBlocks<2>::value, false><<<blocks, 256, 0, s>>>(a);
      break;
    case 3:
      if (skip)
        volume_forward_kernel<3, ForwardBlocks<3>::value, true><<<blocks, 256, 0, s>>>(a);
      else
        volume_forward_kernel<3, ForwardBlocks<3>::value, false><<<blocks, 256, 0, s>>>(a);
      break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_volume_backward(const VolumeArgs& a, cudaStream_t s) {
  const uint32_t tiles = tile_ids(a);
  const uint32_t blocks = (tiles + 7) / 8;
  if (blocks == 0) return cudaSuccess;
  prefer_l1();
  // only fp32 (learnable) volumes have an adjoint
  if (a.v.precision == 1)
    volume_backward_kernel<1, kBackwardMinBlocks><<<blocks, 256, 0, s>>>(a);
  else if (a.v.precision == 2)
    volume_backward_kernel<2, kBackwardMinBlocks><<<blocks, 256, 0, s>>>(a);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_cell_mask(const VolumeView& v, uint32_t* mask, cudaStream_t s) {
  if (!v.nbricks) return cudaSuccess;
  const uint32_t threads = v.nbricks * 16u * 32u;
  const uint32_t blocks = (threads + 255u) / 256u;
  switch (v.precision) {
    case 0: cell_mask_kernel<0><<<blocks, 256, 0, s>>>(v, mask); break;
    case 1: cell_mask_kernel<1><<<blocks, 256, 0, s>>>(v, mask); break;
    case 2: cell_mask_kernel<2><<<blocks, 256, 0, s>>>(v, mask); break;
    default: cell_mask_kernel<3><<<blocks, 256, 0, s>>>(v, mask); break;
  }
  return cudaGetLastError();
}

cudaError_t launch_brick_bits(const VolumeView& v, uint32_t* bits, cudaStream_t s) {
  const uint64_t n = (uint64_t)v.nb * v.nb * v.nb;
  const uint32_t nwords = (uint32_t)((n + 31) / 32);
  brick_bits_kernel<<<(uint32_t)(((uint64_t)nwords * 32 + 255) / 256), 256, 0, s>>>(v, bits,
                                                                                   nwords);
  return cudaGetLastError();
}

cudaError_t launch_apron_fold(const VolumeArgs& a, int channels, float* g, bool gather,
                              cudaStream_t s) {
  if (a.v.nbricks == 0) return cudaSuccess;
  const int blocks = 2 * device_sm_count_vol() * 8;
  if (gather) fold_gather_kernel<<<blocks, 256, 0, s>>>(a, channels, g);
  fold_scatter_kernel<<<blocks, 256, 0, s>>>(a, channels, g);
  return cudaGetLastError();
}

__global__ void unpack_grads_kernel(const float4* __restrict__ p, uint32_t n, float* gd,
                                    float* ga) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 v = p[i];
    gd[i] += v.w;
    ga[3 * (size_t)i] += v.x;
    ga[3 * (size_t)i + 1] += v.y;
    ga[3 * (size_t)i + 2] += v.z;
  }
}

cudaError_t launch_unpack_grads(const float4* packed, uint32_t n, float* grad_density,
                                float* grad_albedo, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  unpack_grads_kernel<<<2 * device_sm_count_vol() * 8, 256, 0, s>>>(packed, n, grad_density,
                                                                     grad_albedo);
  return cudaGetLastError();
}

__global__ void pack_f32_kernel(const float* __restrict__ d, const float* __restrict__ c,
                                uint32_t n, float4* __restrict__ out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = make_float4(c[3 * (size_t)i], c[3 * (size_t)i + 1], c[3 * (size_t)i + 2], d[i]);
}

cudaError_t launch_pack_f32(const float* density, const float* albedo, uint32_t n,
                            float4* packed, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  pack_f32_kernel<<<2 * device_sm_count_vol() * 8, 256, 0, s>>>(density, albedo, n, packed);
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
