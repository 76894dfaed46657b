// svo_noalloc.cu - a frame entry point that allocates no device memory.
//
// Some callers cannot call cudaMalloc: code that runs while a CUDA stream is
// being captured into a graph (allocation is not a capturable operation),
// real-time render loops that cannot afford the device synchronisation an
// allocation may imply, and hosts whose device memory is owned by another
// allocator (a game engine's or a framework's pool) that hands out every
// buffer itself.  yv_render_svo_noalloc serves them: the scene (the
// reference VoxNode pool and its leaf attributes) and every output are the
// caller's device buffers, and the only scratch the frame kernel needs - its
// ray-queue counter, status word and hit counters - lives in the file-scope
// array below, which every GPU that loads the library holds until exit.
#include "svo_trace.cuh"

#include <cstring>
#include <mutex>
#include <string>

namespace yv {
namespace {

// 256 bytes: the stated maximum scratch of one allocation-free frame.
constexpr int kNoAllocScratchWords = 64;
static_assert(kSvoCounterWords <= kNoAllocScratchWords, "frame counters exceed the scratch");
static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocScratchWords];

// Device address of the scratch array for the current device.  In host code
// the array's name is only a host-side stand-in, so the address is looked up
// once per device, with that device current.
yv_status scratch_address(uint32_t** out) {
  static std::mutex mu;
  static uint32_t* addr[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) {
    set_last_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    cudaGetLastError();
    return YV_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lk(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      set_last_error(std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
      cudaGetLastError();
      return YV_ERR_CUDA;
    }
    addr[dev] = static_cast<uint32_t*>(p);
  }
  *out = addr[dev];
  return YV_OK;
}

}  // namespace
}  // namespace yv

using namespace yv;

extern "C" yv_status yv_render_svo_noalloc(const yv_vox_node* nodes, uint32_t count,
                                           uint32_t root, const yv_leaf_attr* attrs,
                                           uint32_t nattrs, const yv_camera* cam,
                                           const yv_light* light, int32_t width,
                                           int32_t height, const yv_frame_outputs* out,
                                           void* stream) {
  if (!cam || !light || !out || width <= 0 || height <= 0 ||
      (!(root & 0x80000000u) && (!nodes || root >= count)) || (nattrs && !attrs))
    return YV_ERR_INVALID_ARG;
  if (!(cam->fov_deg > 0.f && cam->fov_deg < 180.f)) return YV_ERR_INVALID_ARG;
  // The queue counter in the scratch array indexes rays in 8x4 tiles; a
  // frame whose padded ray count needs more than 31 bits does not fit.
  const uint64_t ids = (uint64_t)((width + 7) / 8) * (uint64_t)((height + 3) / 4) * 32u;
  if (ids > 0x7FFFFFFFull) {
    set_last_error("yv_render_svo_noalloc: frame larger than 2^31 rays (scratch counter range)");
    return YV_ERR_INVALID_ARG;
  }
  if (count > YV_MAX_DEVICE_NODES) {
    set_last_error("yv_render_svo_noalloc: node pool larger than 2^29 nodes");
    return YV_ERR_INVALID_ARG;
  }
  uint32_t* scratch = nullptr;
  yv_status st = scratch_address(&scratch);
  if (st != YV_OK) return st;

  SvoDeviceScene sc;
  sc.nodes = reinterpret_cast<const uint4*>(nodes);  // read as 40-byte VoxNode records
  sc.orig_id = nullptr;
  sc.attrs = attrs;
  sc.n_nodes = count;
  sc.n_attrs = nattrs;
  sc.root_word = (root & 0x80000000u) ? YV_DW_NULL : root;

  SvoFrameArgs a;
  std::memset(&a, 0, sizeof(a));
  std::memcpy(a.pos, cam->pos, sizeof(a.pos));
  init_ray_dir(cam->dir, cam->up, cam->fov_deg, width, height, a.dir0, a.du, a.dv);
  std::memcpy(a.light, light->dir, sizeof(a.light));
  std::memcpy(a.light_ray, light->dir, sizeof(a.light_ray));
  adjust_dir(a.light_ray);
  a.ambient = light->ambient;
  a.diffuse = light->diffuse;
  a.shadows = light->shadows ? 1 : 0;
  a.width = width;
  a.height = height;
  a.id_begin = 0;
  a.id_end = (uint32_t)ids;
  a.rgba = static_cast<uint32_t*>(out->rgba);
  a.hit = static_cast<uint32_t*>(out->hit);
  a.hit_t = static_cast<float*>(out->hit_t);
  a.fetches = static_cast<uint32_t*>(out->fetches);
  a.shadow_fetches = static_cast<uint32_t*>(out->shadow_fetches);
  a.normal = static_cast<float*>(out->normal);
  a.counters = scratch;

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // checked traversal of the caller's pool with the 4-frame shared-memory
  // ring (dynamic shared memory, 4 KB per warp: no allocation)
  constexpr int kRing = 4;
  constexpr size_t kSmem = (256 / 32) * kRing * 1024;
  auto kern = svo_frame_kernel<3, true, kRing, false>;
  int resident = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, kern, 256, kSmem);
  if (e == cudaSuccess && resident <= 0) e = cudaErrorInvalidConfiguration;
  // the counters start every frame at zero: the array keeps the last call's
  // contents
  if (e == cudaSuccess)
    e = cudaMemsetAsync(scratch, 0, kSvoCounterWords * sizeof(uint32_t), s);
  if (e == cudaSuccess) {
    kern<<<device_sm_count() * resident, 256, kSmem, s>>>(sc, a, 0u, 32u);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    set_last_error(std::string("yv_render_svo_noalloc: ") + cudaGetErrorString(e));
    cudaGetLastError();
    return YV_ERR_CUDA;
  }
  return YV_OK;
}

extern "C" yv_status yv_render_svo_noalloc_status(void* stream, uint32_t* device_bits) {
  uint32_t* scratch = nullptr;
  yv_status st = scratch_address(&scratch);
  if (st != YV_OK) return st;
  // word 1 of the scratch is the frame's status; a pageable host word makes
  // the copy complete before cudaMemcpyAsync returns, and nothing is
  // allocated
  uint32_t bits = 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemcpyAsync(&bits, scratch + 1, sizeof(bits), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    set_last_error(std::string("yv_render_svo_noalloc_status: ") + cudaGetErrorString(e));
    cudaGetLastError();
    return YV_ERR_CUDA;
  }
  if (device_bits) *device_bits = bits;
  if (bits & YV_DEV_ERR_POOL) return YV_ERR_BAD_POOL;
  if (bits & (YV_DEV_ERR_ITER | YV_DEV_ERR_DEPTH)) return YV_ERR_ITERATION_CAP;
  if (bits & YV_DEV_ERR_TIMEOUT) return YV_ERR_TIMEOUT;
  return YV_OK;
}
