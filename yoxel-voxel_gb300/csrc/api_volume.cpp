// api_volume.cpp - C ABI of the brick-volume path: device upload of the
// ntree pool (BrickPool<T>, ntree/BrickManager.h:5-80), the multi-camera
// march (the working kernel behind ntree's RunTrace entry,
// ntree/ntree_trace.cuh:22-28) and its adjoint.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "yv_internal.h"
#include "yv_kernels.h"
#include "yv_volume.h"

using namespace yv;

struct yv_volume_gpu {
  int device = 0;
  yv_volume_device desc;
  void* mem[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  size_t cap[5] = {0, 0, 0, 0, 0};  // bytes allocated per array (reused by rebuilds)
  // acceleration arrays in one allocation: the cell occupancy mask (16
  // words per brick), then the brick bitmap (trees of up to 4 levels)
  uint32_t* mask = nullptr;
  size_t mask_cap = 0;
};

namespace {

yv_status fail(cudaError_t e, const char* what) {
  set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
  cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? YV_ERR_OUT_OF_MEMORY : YV_ERR_CUDA;
}

// IEEE binary32 -> binary16, round to nearest even, saturating at +-65504
// (the fp16 lattice formats hold finite values only; the device decodes
// them with exact bit arithmetic that assumes a finite half).  NaN -> 0.
uint16_t f32_to_f16(float f) {
  uint32_t x;
  std::memcpy(&x, &f, 4);
  const uint32_t sign = (x >> 16) & 0x8000u;
  const int32_t exp = (int32_t)((x >> 23) & 0xFFu);
  uint32_t man = x & 0x7FFFFFu;
  if (exp == 0xFF) return man ? (uint16_t)0 : (uint16_t)(sign | 0x7BFFu);
  int32_t e = exp - 127 + 15;
  if (e >= 0x1F) return (uint16_t)(sign | 0x7BFFu);
  if (e <= 0) {
    if (e < -10) return (uint16_t)sign;
    man |= 0x800000u;
    const int shift = 14 - e;
    uint32_t h = man >> shift;
    const uint32_t rem = man & ((1u << shift) - 1u), half = 1u << (shift - 1);
    if (rem > half || (rem == half && (h & 1u))) ++h;
    return (uint16_t)(sign | h);
  }
  uint32_t h = ((uint32_t)e << 10) | (man >> 13);
  const uint32_t rem = man & 0x1FFFu;
  if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
  if (h >= 0x7C00u) h = 0x7BFFu;
  return (uint16_t)(sign | h);
}

bool fill_args(const yv_volume_device* v, const yv_march_params* mp, int width, int height,
               VolumeArgs* a) {
  if (!v || !mp || !v->grids || v->levels < 1 || v->levels > 5 || width <= 0 || height <= 0 ||
      !(mp->step_vox > 0.f) || !std::isfinite(mp->alpha_scale) ||
      v->precision < YV_PRECISION_F16 || v->precision > YV_PRECISION_F16_PACKED)
    return false;
  // warp tiles of one launch (up to kMaxVolumeCams cameras, 16x16-pixel
  // squares of 8 tiles) are numbered with 32-bit ids
  const uint64_t sq_x = ((uint64_t)(width + 7) / 8 + 1) / 2;
  const uint64_t sq_y = ((uint64_t)(height + 3) / 4 + 3) / 4;
  if ((uint64_t)kMaxVolumeCams * sq_x * sq_y * 8u > 0x7FFFFFFFull) return false;
  // packed formats keep the whole lattice point in the albedo buffer
  const bool packed = v->precision >= YV_PRECISION_F32_PACKED;
  if (v->nbricks && (!v->albedo || (!packed && !v->density))) return false;
  std::memset(a, 0, sizeof(*a));
  a->v.grids = v->grids;
  a->v.ngrids = v->ngrids;
  a->v.levels = v->levels;
  a->v.nb = 1 << (2 * v->levels);
  a->v.density = v->density;
  a->v.albedo = v->albedo;
  a->v.nbricks = v->nbricks;
  a->v.precision = v->precision;
  a->v.cell_mask = v->cell_mask;
  a->v.brick_bits = v->brick_bits;
  a->nbr_up = v->nbr_up;
  a->nbr_dn = v->nbr_dn;
  a->v.S = (float)(8 * a->v.nb);
  a->v.cell_size = 8.0f / a->v.S;
  a->v.alpha_scale = mp->alpha_scale;
  a->v.dt = mp->step_vox / a->v.S;
  a->v.inv_dt = a->v.S / mp->step_vox;
  a->width = width;
  a->height = height;
  return true;
}

void set_cams(VolumeArgs* a, const yv_camera* cams, int n) {
  a->ncams = n;
  for (int i = 0; i < n; ++i) {
    CamBasis& b = a->cam[i];
    std::memcpy(b.pos, cams[i].pos, sizeof(b.pos));
    init_ray_dir(cams[i].dir, cams[i].up, cams[i].fov_deg, a->width, a->height, b.dir0, b.du,
                 b.dv);
  }
}

bool cams_ok(const yv_camera* c, int n) {
  if (!c || n <= 0) return false;
  for (int i = 0; i < n; ++i) {
    for (int k = 0; k < 3; ++k)
      if (!std::isfinite(c[i].pos[k]) || !std::isfinite(c[i].dir[k]) || !std::isfinite(c[i].up[k]))
        return false;
    if (!(c[i].fov_deg > 0.f && c[i].fov_deg < 180.f)) return false;
  }
  return true;
}

}  // namespace

namespace yv {

yv_status volume_gpu_from_device(void* mem[5], const size_t bytes[5], const yv_volume_device& d,
                                 yv_volume_gpu** out, uint32_t* accel) {
  yv_volume_gpu* g = new (std::nothrow) yv_volume_gpu();
  if (!g) {
    for (int i = 0; i < 5; ++i) cudaFree(mem[i]);
    cudaFree(accel);
    return YV_ERR_OUT_OF_MEMORY;
  }
  cudaGetDevice(&g->device);
  for (int i = 0; i < 5; ++i) {
    g->mem[i] = mem[i];
    g->cap[i] = mem[i] ? bytes[i] : 0;
  }
  g->desc = d;
  g->mask = accel;
  g->mask_cap = accel ? volume_accel_bytes(d.nbricks, d.levels) : 0;
  if (!accel) {
    g->desc.cell_mask = nullptr;
    g->desc.brick_bits = nullptr;
  }
  *out = g;
  return YV_OK;
}

size_t volume_accel_bytes(uint32_t nbricks, int levels) {
  if (!nbricks) return 0;
  const size_t bits = levels <= 4 ? (size_t)YV_BRICK_BITS_WORDS(levels) * 4u : 0u;
  return (size_t)nbricks * 16u * sizeof(uint32_t) + bits;
}

yv_status volume_gpu_accel_buffer(yv_volume_gpu* g, uint32_t nbricks, int levels, cudaStream_t s,
                                  uint32_t** mask, uint32_t** bits) {
  const size_t bytes = volume_accel_bytes(nbricks, levels);
  *mask = nullptr;
  *bits = nullptr;
  if (!bytes) return YV_OK;
  cudaError_t e = cudaSuccess;
  if (g->mask_cap < bytes) {
    // the old arrays may still be read by queued work on `s`
    if (g->mask) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) {
      cudaFree(g->mask);
      g->mask = nullptr;
      g->mask_cap = 0;
      g->desc.cell_mask = nullptr;
      g->desc.brick_bits = nullptr;
      e = cudaMalloc(&g->mask, bytes);
    }
    if (e != cudaSuccess) return fail(e, "acceleration arrays");
    g->mask_cap = bytes;
  }
  *mask = g->mask;
  if (levels <= 4) *bits = g->mask + (size_t)nbricks * 16u;
  return YV_OK;
}

yv_status volume_brick_bits(const yv_volume_device& d, uint32_t* bits, cudaStream_t s) {
  yv_march_params mp = {1.0f, 0.5f};
  VolumeArgs* a = new (std::nothrow) VolumeArgs;
  if (!a) return YV_ERR_OUT_OF_MEMORY;
  if (!fill_args(&d, &mp, 1, 1, a)) {
    delete a;
    return YV_ERR_INVALID_ARG;
  }
  const cudaError_t e = launch_brick_bits(a->v, bits, s);
  delete a;
  return e == cudaSuccess ? YV_OK : fail(e, "brick bits");
}

yv_status volume_gpu_refresh_mask(yv_volume_gpu* g, cudaStream_t s) {
  uint32_t *mask = nullptr, *bits = nullptr;
  yv_status st = volume_gpu_accel_buffer(g, g->desc.nbricks, g->desc.levels, s, &mask, &bits);
  g->desc.cell_mask = nullptr;
  g->desc.brick_bits = nullptr;
  if (st != YV_OK || !mask) return st;
  yv_march_params mp = {1.0f, 0.5f};
  VolumeArgs* a = new (std::nothrow) VolumeArgs;
  if (!a) return YV_ERR_OUT_OF_MEMORY;
  if (!fill_args(&g->desc, &mp, 1, 1, a)) {
    delete a;
    return YV_ERR_INVALID_ARG;
  }
  cudaError_t e = launch_cell_mask(a->v, mask, s);
  if (e == cudaSuccess && bits) e = launch_brick_bits(a->v, bits, s);
  delete a;
  if (e != cudaSuccess) return fail(e, "acceleration arrays");
  g->desc.cell_mask = mask;
  g->desc.brick_bits = bits;
  return YV_OK;
}

yv_status volume_gpu_arrays(yv_volume_gpu* g, void*** mem, size_t** cap, yv_volume_device** d) {
  if (!g) return YV_ERR_INVALID_ARG;
  *mem = g->mem;
  *cap = g->cap;
  *d = &g->desc;
  return YV_OK;
}

}  // namespace yv

extern "C" {

yv_status yv_volume_upload(const yv_volume_host* v, int32_t precision, yv_volume_gpu** out) {
  if (!v || !out || precision < YV_PRECISION_F16 || precision > YV_PRECISION_F16_PACKED)
    return YV_ERR_INVALID_ARG;
  *out = nullptr;
  yv_volume_gpu* g = new (std::nothrow) yv_volume_gpu();
  if (!g) return YV_ERR_OUT_OF_MEMORY;
  cudaGetDevice(&g->device);
  const uint32_t ng = yv_volume_grid_count(v), nb = yv_volume_brick_count(v);
  const size_t n = (size_t)nb * 729u;
  const float* den = yv_volume_density(v);
  const uint8_t* alb = yv_volume_albedo(v);
  // host-side validation of the refs (the kernels also bound-check)
  const uint32_t* grids = yv_volume_grids(v);
  for (size_t i = 0; i < (size_t)ng * 64; ++i) {
    uint32_t r = grids[i];
    if (r & 0x80000000u) continue;
    if ((r & 0x40000000u) ? (r & 0x3FFFFFFFu) >= nb : r >= ng) {
      delete g;
      set_last_error("volume child ref out of range");
      return YV_ERR_BAD_POOL;
    }
  }
  std::vector<uint8_t> dbuf, abuf;
  size_t dbytes, abytes;
  if (precision == YV_PRECISION_F16) {
    dbytes = n * 2;
    abytes = n * 4;
    dbuf.resize(dbytes);
    abuf.resize(abytes);
    uint16_t* d16 = reinterpret_cast<uint16_t*>(dbuf.data());
    for (size_t i = 0; i < n; ++i) {
      d16[i] = f32_to_f16(den[i]);
      abuf[i * 4] = alb[i * 3];
      abuf[i * 4 + 1] = alb[i * 3 + 1];
      abuf[i * 4 + 2] = alb[i * 3 + 2];
      abuf[i * 4 + 3] = 255;
    }
  } else if (precision == YV_PRECISION_F32) {
    dbytes = n * 4;
    abytes = n * 12;
    dbuf.resize(dbytes);
    abuf.resize(abytes);
    std::memcpy(dbuf.data(), den, dbytes);
    float* af = reinterpret_cast<float*>(abuf.data());
    for (size_t i = 0; i < n * 3; ++i) af[i] = (float)alb[i] * (1.0f / 255.0f);
  } else if (precision == YV_PRECISION_F32_PACKED) {
    // float4 (r, g, b, density) per lattice point; no separate density array
    dbytes = 0;
    abytes = n * 16;
    abuf.resize(abytes);
    float* af = reinterpret_cast<float*>(abuf.data());
    for (size_t i = 0; i < n; ++i) {
      for (int c = 0; c < 3; ++c) af[i * 4 + (size_t)c] = (float)alb[i * 3 + (size_t)c] * (1.0f / 255.0f);
      af[i * 4 + 3] = den[i];
    }
  } else {
    // 8 bytes per lattice point: {fp16 density | r << 16 | g << 24, b}
    dbytes = 0;
    abytes = n * 8;
    abuf.resize(abytes);
    uint32_t* au = reinterpret_cast<uint32_t*>(abuf.data());
    for (size_t i = 0; i < n; ++i) {
      au[i * 2] = (uint32_t)f32_to_f16(den[i]) | ((uint32_t)alb[i * 3] << 16) |
                  ((uint32_t)alb[i * 3 + 1] << 24);
      au[i * 2 + 1] = (uint32_t)alb[i * 3 + 2];
    }
  }
  const void* src[5] = {grids, dbuf.data(), abuf.data(), yv_volume_neighbors(v, 1),
                        yv_volume_neighbors(v, 0)};
  const size_t bytes[5] = {(size_t)ng * 256u, dbytes, abytes, (size_t)nb * 28u, (size_t)nb * 28u};
  for (int i = 0; i < 5; ++i) {
    if (!bytes[i]) continue;
    cudaError_t e = cudaMalloc(&g->mem[i], bytes[i]);
    if (e == cudaSuccess) g->cap[i] = bytes[i];
    if (e == cudaSuccess) e = cudaMemcpy(g->mem[i], src[i], bytes[i], cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      yv_volume_gpu_free(g);
      return fail(e, "volume upload");
    }
  }
  g->desc.grids = static_cast<const uint32_t*>(g->mem[0]);
  g->desc.ngrids = ng;
  g->desc.levels = yv_volume_levels(v);
  g->desc.density = g->mem[1];
  g->desc.albedo = g->mem[2];
  g->desc.nbricks = nb;
  g->desc.precision = precision;
  g->desc.nbr_up = static_cast<const int32_t*>(g->mem[3]);
  g->desc.nbr_dn = static_cast<const int32_t*>(g->mem[4]);
  g->desc.cell_mask = nullptr;
  g->desc.brick_bits = nullptr;
  yv_status st = volume_gpu_refresh_mask(g, nullptr);
  cudaError_t e = st == YV_OK ? cudaStreamSynchronize(nullptr) : cudaSuccess;
  if (st != YV_OK || e != cudaSuccess) {
    yv_volume_gpu_free(g);
    return st != YV_OK ? st : fail(e, "cell mask");
  }
  *out = g;
  return YV_OK;
}

void yv_volume_gpu_free(yv_volume_gpu* g) {
  if (!g) return;
  cudaSetDevice(g->device);
  for (void* p : g->mem) cudaFree(p);
  cudaFree(g->mask);
  delete g;
}

yv_status yv_volume_brick_bits(const yv_volume_device* v, uint32_t* bits, void* stream) {
  if (!v || !bits) return YV_ERR_INVALID_ARG;
  return volume_brick_bits(*v, bits, static_cast<cudaStream_t>(stream));
}

yv_status yv_volume_gpu_desc(const yv_volume_gpu* g, yv_volume_device* out) {
  if (!g || !out) return YV_ERR_INVALID_ARG;
  *out = g->desc;
  return YV_OK;
}

yv_status yv_volume_render(const yv_volume_device* vol, const yv_camera* cams, int32_t ncams,
                           int32_t width, int32_t height, const yv_march_params* mp, float* rgba,
                           uint32_t* samples, uint32_t* bricks, void* stream) {
  VolumeArgs* a = new (std::nothrow) VolumeArgs;
  if (!a) return YV_ERR_OUT_OF_MEMORY;
  if (!fill_args(vol, mp, width, height, a) || !cams_ok(cams, ncams) || !rgba) {
    delete a;
    return YV_ERR_INVALID_ARG;
  }
  const size_t px = (size_t)width * (size_t)height;
  for (int c0 = 0; c0 < ncams; c0 += kMaxVolumeCams) {
    const int n = ncams - c0 < kMaxVolumeCams ? ncams - c0 : kMaxVolumeCams;
    set_cams(a, cams + c0, n);
    a->rgba = rgba + (size_t)c0 * px * 4;
    a->samples = samples ? samples + (size_t)c0 * px : nullptr;
    a->bricks_entered = bricks ? bricks + (size_t)c0 * px : nullptr;
    cudaError_t e = launch_volume_forward(*a, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) {
      delete a;
      return fail(e, "volume forward launch");
    }
  }
  delete a;
  return YV_OK;
}

yv_status yv_volume_tile_count(int32_t width, int32_t height, uint32_t* tiles_per_camera) {
  if (width <= 0 || height <= 0 || !tiles_per_camera) return YV_ERR_INVALID_ARG;
  *tiles_per_camera = volume_tiles_per_camera(width, height);
  return YV_OK;
}

yv_status yv_volume_render_tiles(const yv_volume_device* vol, const yv_camera* cams,
                                 int32_t ncams, int32_t width, int32_t height,
                                 const yv_march_params* mp, uint32_t tile_begin,
                                 uint32_t tile_end, float* rgba, uint32_t* samples,
                                 uint32_t* bricks, void* stream) {
  if (ncams > kMaxVolumeCams) return YV_ERR_INVALID_ARG;
  VolumeArgs* a = new (std::nothrow) VolumeArgs;
  if (!a) return YV_ERR_OUT_OF_MEMORY;
  if (!fill_args(vol, mp, width, height, a) || !cams_ok(cams, ncams) || !rgba) {
    delete a;
    return YV_ERR_INVALID_ARG;
  }
  const uint64_t total = (uint64_t)volume_tiles_per_camera(width, height) * (uint64_t)ncams;
  if (tile_begin > tile_end || tile_end > total) {
    delete a;
    set_last_error("yv_volume_render_tiles: tile range outside the frames");
    return YV_ERR_INVALID_ARG;
  }
  if (tile_begin == tile_end) {
    delete a;
    return YV_OK;
  }
  set_cams(a, cams, ncams);
  a->rgba = rgba;
  a->samples = samples;
  a->bricks_entered = bricks;
  a->tile_begin = tile_begin;
  a->tile_end = tile_end;
  const cudaError_t e = launch_volume_forward(*a, static_cast<cudaStream_t>(stream));
  delete a;
  return e == cudaSuccess ? YV_OK : fail(e, "volume forward launch");
}

yv_status yv_volume_render_rgba8(const yv_volume_device* vol, const yv_camera* cams,
                                 int32_t ncams, int32_t width, int32_t height,
                                 const yv_march_params* mp, uint32_t* rgba8, void* stream) {
  VolumeArgs* a = new (std::nothrow) VolumeArgs;
  if (!a) return YV_ERR_OUT_OF_MEMORY;
  if (!fill_args(vol, mp, width, height, a) || !cams_ok(cams, ncams) || !rgba8) {
    delete a;
    return YV_ERR_INVALID_ARG;
  }
  const size_t px = (size_t)width * (size_t)height;
  for (int c0 = 0; c0 < ncams; c0 += kMaxVolumeCams) {
    const int n = ncams - c0 < kMaxVolumeCams ? ncams - c0 : kMaxVolumeCams;
    set_cams(a, cams + c0, n);
    a->rgba = nullptr;
    a->rgba8 = rgba8 + (size_t)c0 * px;
    a->samples = nullptr;
    a->bricks_entered = nullptr;
    cudaError_t e = launch_volume_forward(*a, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) {
      delete a;
      return fail(e, "volume forward launch");
    }
  }
  delete a;
  return YV_OK;
}

yv_status yv_volume_backward(const yv_volume_device* vol, const yv_camera* cams, int32_t ncams,
                             int32_t width, int32_t height, const yv_march_params* mp,
                             const float* rgba, const float* grad_rgba, float* grad_density,
                             float* grad_albedo, void* stream) {
  VolumeArgs* a = new (std::nothrow) VolumeArgs;
  if (!a) return YV_ERR_OUT_OF_MEMORY;
  if (!fill_args(vol, mp, width, height, a) || !cams_ok(cams, ncams) || !rgba || !grad_rgba ||
      !grad_density || !grad_albedo ||
      (vol->precision != YV_PRECISION_F32 && vol->precision != YV_PRECISION_F32_PACKED)) {
    delete a;
    return YV_ERR_INVALID_ARG;
  }
  const size_t px = (size_t)width * (size_t)height;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // Gradients accumulate in a packed (albedo rgb, density) float4 per
  // lattice point - one 16-byte atomic per corner - taken from the
  // stream-ordered pool and added into the caller's tensors at the end.
  const size_t npts = (size_t)vol->nbricks * 729u;
  float4* packed = nullptr;
  cudaError_t e = cudaSuccess;
  if (npts) {
    e = scratch_alloc(reinterpret_cast<void**>(&packed), npts * sizeof(float4), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(packed, 0, npts * sizeof(float4), s);
  }
  for (int c0 = 0; c0 < ncams && e == cudaSuccess && npts; c0 += kMaxVolumeCams) {
    const int n = ncams - c0 < kMaxVolumeCams ? ncams - c0 : kMaxVolumeCams;
    set_cams(a, cams + c0, n);
    a->rgba_fwd = rgba + (size_t)c0 * px * 4;
    a->grad_rgba = grad_rgba + (size_t)c0 * px * 4;
    a->grad_density = grad_density;
    a->grad_albedo = grad_albedo;
    a->grad_packed = packed;
    e = launch_volume_backward(*a, s);
  }
  if (e == cudaSuccess && npts)
    e = launch_unpack_grads(packed, (uint32_t)npts, grad_density, grad_albedo, s);
  if (packed) {
    cudaError_t ef = scratch_free(packed, s);
    if (e == cudaSuccess) e = ef;
  }
  delete a;
  return e == cudaSuccess ? YV_OK : fail(e, "volume backward");
}

yv_status yv_volume_fold_aprons(const yv_volume_device* vol, float* grad_density,
                                float* grad_albedo, void* stream) {
  if (!vol || !vol->nbr_up || !vol->nbr_dn) return YV_ERR_INVALID_ARG;
  VolumeArgs a;
  yv_march_params mp = {1.f, 1.f};
  if (!fill_args(vol, &mp, 1, 1, &a)) return YV_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaSuccess;
  if (grad_density) e = launch_apron_fold(a, 1, grad_density, true, s);
  if (e == cudaSuccess && grad_albedo) e = launch_apron_fold(a, 3, grad_albedo, true, s);
  return e == cudaSuccess ? YV_OK : fail(e, "apron fold");
}

yv_status yv_volume_sync_aprons(const yv_volume_device* vol, float* density, float* albedo,
                                void* stream) {
  if (!vol || !vol->nbr_up ||
      (vol->precision != YV_PRECISION_F32 && vol->precision != YV_PRECISION_F32_PACKED))
    return YV_ERR_INVALID_ARG;
  VolumeArgs a;
  yv_march_params mp = {1.f, 1.f};
  if (!fill_args(vol, &mp, 1, 1, &a)) return YV_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaSuccess;
  if (density) e = launch_apron_fold(a, 1, density, false, s);
  if (e == cudaSuccess && albedo) e = launch_apron_fold(a, 3, albedo, false, s);
  return e == cudaSuccess ? YV_OK : fail(e, "apron sync");
}

yv_status yv_volume_pack(const float* density, const float* albedo, uint32_t npoints,
                         float* packed, void* stream) {
  if (!npoints) return YV_OK;
  if (!density || !albedo || !packed || (reinterpret_cast<uintptr_t>(packed) & 15u))
    return YV_ERR_INVALID_ARG;
  cudaError_t e = launch_pack_f32(density, albedo, npoints, reinterpret_cast<float4*>(packed),
                                  static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? YV_OK : fail(e, "volume pack");
}

}  // extern "C"
