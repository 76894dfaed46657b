// yv_internal.h - host-side internals shared by the C ABI implementation,
// the scene builders and the kernel launchers.  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "yv_c_api.h"

// ---------------------------------------------------------------------------
// Device layout of the SVO node pool.
//
// The reference pool is an array of 40-byte VoxNode records read through a
// 1D texture (reaction/report/main.tex:36-67).  On the device each node is
// re-laid as one 32-byte, 32-byte-aligned record of 8 child words, so a node
// is exactly one L2 sector (a traversal step reads the word it tests).  The leaf /
// null information of `flags` is folded into the words:
//   word & YV_DW_LEAF  -> leaf, low 31 bits = VoxData (leaf attribute index)
//   word & YV_DW_NULL  -> null child (EmptyNode / FullNode)
//   otherwise          -> device node index
// Nodes are renumbered breadth-first from the root, so the top levels are the
// first records (they are staged in shared memory); orig_id maps a device
// index back to the caller's node id for the hit output.
// ---------------------------------------------------------------------------
constexpr uint32_t YV_DW_LEAF = 0x80000000u;
constexpr uint32_t YV_DW_NULL = 0x40000000u;
constexpr int YV_MAX_DEPTH = 16;            // node levels a pool may have
constexpr uint32_t YV_MAX_DEVICE_NODES = 0x1FFFFFFFu;  // hit word = id<<3|c

// Device status bits (written with atomicOr by kernels).
constexpr uint32_t YV_DEV_ERR_ITER = 1u;    // per-ray iteration cap reached
constexpr uint32_t YV_DEV_ERR_DEPTH = 2u;   // stack depth exceeded
constexpr uint32_t YV_DEV_ERR_POOL = 4u;    // index outside the pool
constexpr uint32_t YV_DEV_ERR_TIMEOUT = 8u; // frame time budget elapsed

struct yv_svo_host {
  std::vector<yv_vox_node> nodes;
  std::vector<yv_leaf_attr> attrs;
  uint32_t root = YV_EMPTY_NODE;
  int depth = 0;
  bool lod = false;  // every node's `data` indexes its level-of-detail attribute
};

namespace yv {

// Breadth-first device re-layout of a reference pool (see above).
struct DeviceLayout {
  std::vector<uint32_t> words;     // 8 per node
  std::vector<uint32_t> orig_id;   // device index -> caller node id
  uint32_t root_word = YV_DW_NULL; // device word of the root
  int depth = 0;                   // node levels (root = level 0)
};

// Validates and converts; returns YV_OK or YV_ERR_BAD_POOL.
yv_status build_device_layout(const yv_vox_node* nodes, uint32_t count,
                              uint32_t root, uint32_t nattrs,
                              DeviceLayout* out, std::string* why);

// RendererBase::InitRayDir in float (cell/renderer_base.h:50-61).
void init_ray_dir(const float dir[3], const float up[3], float fov_deg,
                  int width, int height, float dir0[3], float du[3],
                  float dv[3]);
// AdjustDir with eps = 1e-5.
void adjust_dir(float d[3]);

// Thread-safe last-error text for diagnostics.
void set_last_error(const std::string& s);
const char* last_error_cstr();

// splitmix64 stream used by every seeded generator.
struct SplitMix64 {
  uint64_t s;
  explicit SplitMix64(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double u01() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};
uint64_t hash64(uint64_t x);

int hardware_threads();

// Scenes built on the device (api.cpp): renderer_scene_buffers waits for
// the renderer's last frame and returns its (reused or grown) buffers for nn
// node records (8 child words, id) and na 16-byte shading records;
// renderer_commit_scene then makes them the current scene.
yv_status renderer_scene_buffers(yv_renderer* r, uint32_t nn, uint32_t na, uint32_t** words,
                                 uint32_t** orig, void** attrs);
void renderer_commit_scene(yv_renderer* r, uint32_t nn, uint32_t na, uint32_t root_word);

// A host brick volume from parts built on the device (volume_host.cpp):
// grids (ngrids x 64 refs), fp32 lattice values and RGB per brick, brick
// cells; the apron neighbour tables are derived here.
yv_status volume_host_from_parts(int levels, std::vector<uint32_t>&& grids,
                                 std::vector<float>&& density, std::vector<uint8_t>&& albedo,
                                 std::vector<int32_t>&& cells, yv_volume_host** out);
// A yv_volume_gpu that owns device buffers mem[0..4] (grids, density,
// albedo, neighbours up, neighbours down) of bytes[0..4] bytes, described by
// d (api_volume.cpp), and, when `accel` is given, its acceleration arrays
// already computed there (volume_accel_bytes(d.nbricks, d.levels) bytes:
// d.cell_mask and d.brick_bits point into it).
yv_status volume_gpu_from_device(void* mem[5], const size_t bytes[5], const yv_volume_device& d,
                                 yv_volume_gpu** out, uint32_t* accel = nullptr);
// Bytes of a pool's acceleration arrays: the cell occupancy mask (16 words
// per brick), then the brick bitmap (YV_BRICK_BITS_WORDS(levels) words, for
// trees of up to 4 levels).  0 without bricks.
size_t volume_accel_bytes(uint32_t nbricks, int levels);
// The volume's acceleration arrays, grown to hold those of a pool of
// nbricks bricks and `levels` levels (the old ones are released after `s`
// drains): *mask and *bits (null for trees of more than 4 levels).
yv_status volume_gpu_accel_buffer(yv_volume_gpu* g, uint32_t nbricks, int levels, cudaStream_t s,
                                  uint32_t** mask, uint32_t** bits);
// The brick bitmap of d's tree into `bits` on `s`.
yv_status volume_brick_bits(const yv_volume_device& d, uint32_t* bits, cudaStream_t s);
// (Re)computes the acceleration arrays of a library-owned volume on `s`
// (after its pool changed) and points its descriptor at them.
yv_status volume_gpu_refresh_mask(yv_volume_gpu* g, cudaStream_t s);
// The owned buffers, their allocated sizes and the descriptor of a volume
// (for rebuilds in place).
yv_status volume_gpu_arrays(yv_volume_gpu* g, void*** mem, size_t** cap, yv_volume_device** d);

}  // namespace yv
