// svo_dynamic.cu - an editable SVO with incremental device sync: the
// DynamicSVO scheme of reaction/report/main.tex:67-71 (a node array managed
// by a free list of equal-size elements, split into pages of 256 nodes that
// each carry a version bumped on every modification, so that only changed
// pages are sent to the GPU copy) with its counters CountChangedPages /
// CountTransfrerSize (qtview.py:69-73) and the device update
// SVORenderer::UpdateSVO (demo/SVORenderer.cpp:39-53).
//
// The host pool keeps the reference VoxNode layout; the device mirror is the
// same array (plus the leaf attributes, paged the same way), so frames are
// traced directly from it by the caller-layout kernel of
// yv_render_svo_noalloc.  A sync gathers the changed pages into one pinned
// staging buffer, copies it with one host-to-device transfer and scatters
// the pages to their slots with one kernel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "yv_internal.h"
#include "yv_kernels.h"

namespace {

constexpr uint32_t kPage = 256;  // nodes (or attributes) per page

}  // namespace

struct yv_svo_dynamic {
  int device = 0;
  uint32_t cap_nodes = 0, cap_attrs = 0;
  std::vector<yv_vox_node> nodes;
  std::vector<yv_leaf_attr> attrs;
  std::vector<uint32_t> free_nodes;  // free list (stack) of node slots
  uint32_t n_nodes = 0;              // high-water mark of used node slots
  uint32_t n_attrs = 0;
  uint32_t root = YV_EMPTY_NODE;
  int depth = 0;
  // the state the device mirror holds (set by a sync)
  uint32_t synced_root = YV_EMPTY_NODE, synced_nodes = 0, synced_attrs = 0;
  // page versions: host (bumped on edit) and the version last sent
  std::vector<uint32_t> ver_n, sent_n, ver_a, sent_a;
  yv_vox_node* d_nodes = nullptr;
  yv_leaf_attr* d_attrs = nullptr;
  uint8_t* h_stage = nullptr;  // pinned staging for changed pages
  uint8_t* d_stage = nullptr;
  uint32_t* d_slots = nullptr;
  size_t stage_cap = 0;  // pages the staging buffers hold
};

namespace yv {
namespace {

void touch_node(yv_svo_dynamic* s, uint32_t id) { ++s->ver_n[id / kPage]; }
void touch_attr(yv_svo_dynamic* s, uint32_t i) { ++s->ver_a[i / kPage]; }

// Scatter: page p of the staging buffer (bytes per page `pb`) goes to slot
// slots[p] of `dst` (in pages).  One block per page, 16-byte words.
__global__ void scatter_pages_kernel(const uint4* stage, const uint32_t* slots, uint32_t pages,
                                     uint32_t words_per_page, uint4* dst) {
  for (uint32_t p = blockIdx.x; p < pages; p += gridDim.x) {
    const uint4* src = stage + (size_t)p * words_per_page;
    uint4* d = dst + (size_t)slots[p] * words_per_page;
    for (uint32_t w = threadIdx.x; w < words_per_page; w += blockDim.x) d[w] = src[w];
  }
}

yv_status dyn_fail(cudaError_t e, const char* what) {
  set_last_error(std::string("dynamic SVO: ") + what + ": " + cudaGetErrorString(e));
  cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? YV_ERR_OUT_OF_MEMORY : YV_ERR_CUDA;
}

uint32_t changed(const std::vector<uint32_t>& v, const std::vector<uint32_t>& s) {
  uint32_t n = 0;
  for (size_t i = 0; i < v.size(); ++i) n += v[i] != s[i];
  return n;
}

// Sends the changed pages of one array (node or attribute pages).
cudaError_t sync_array(yv_svo_dynamic* s, const uint8_t* host, size_t elem, uint32_t used,
                       std::vector<uint32_t>& ver, std::vector<uint32_t>& sent, void* dev,
                       cudaStream_t st) {
  const size_t pb = elem * kPage;  // bytes per page (multiple of 16)
  const uint32_t used_pages = (used + kPage - 1) / kPage;
  std::vector<uint32_t> pages;
  for (uint32_t p = 0; p < used_pages; ++p)
    if (ver[p] != sent[p]) pages.push_back(p);
  if (pages.empty()) return cudaSuccess;
  const size_t need = pages.size();
  // staging holds stage_cap pages of the larger (node) element plus slots
  if (need > s->stage_cap) {
    cudaFreeHost(s->h_stage);
    cudaFree(s->d_stage);
    cudaFree(s->d_slots);
    s->h_stage = s->d_stage = nullptr;
    s->d_slots = nullptr;
    s->stage_cap = 0;
    cudaError_t e = cudaMallocHost(&s->h_stage, need * kPage * sizeof(yv_vox_node) + need * 4);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_stage, need * kPage * sizeof(yv_vox_node));
    if (e == cudaSuccess) e = cudaMalloc(&s->d_slots, need * 4);
    if (e != cudaSuccess) return e;
    s->stage_cap = need;
  }
  // the previous sync's copies read the staging buffer: wait for them
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  uint32_t* h_slots = reinterpret_cast<uint32_t*>(s->h_stage + need * pb);
  for (size_t i = 0; i < need; ++i) {
    const uint32_t p = pages[i];
    const size_t first = (size_t)p * kPage;
    const size_t n = std::min<size_t>(kPage, (size_t)used - first);
    std::memcpy(s->h_stage + i * pb, host + first * elem, n * elem);
    if (n < kPage) std::memset(s->h_stage + i * pb + n * elem, 0, (kPage - n) * elem);
    h_slots[i] = p;
  }
  e = cudaMemcpyAsync(s->d_stage, s->h_stage, need * pb, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(s->d_slots, h_slots, need * 4, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  const uint32_t words = (uint32_t)(pb / 16);
  const uint32_t grid = need < 4096 ? (uint32_t)need : 4096u;
  scatter_pages_kernel<<<grid, 128, 0, st>>>(reinterpret_cast<const uint4*>(s->d_stage),
                                             s->d_slots, (uint32_t)need, words,
                                             static_cast<uint4*>(dev));
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  for (uint32_t p : pages) sent[p] = ver[p];
  return cudaSuccess;
}

}  // namespace
}  // namespace yv

using namespace yv;

extern "C" {

yv_status yv_svo_dynamic_create(uint32_t node_capacity, uint32_t attr_capacity,
                                yv_svo_dynamic** out) {
  if (!out || node_capacity == 0 || node_capacity > YV_MAX_DEVICE_NODES || attr_capacity == 0 ||
      attr_capacity > 0x7FFFFFFFu)
    return YV_ERR_INVALID_ARG;
  *out = nullptr;
  yv_svo_dynamic* s = new (std::nothrow) yv_svo_dynamic();
  if (!s) return YV_ERR_OUT_OF_MEMORY;
  // capacities rounded up to whole pages
  s->cap_nodes = (node_capacity + kPage - 1) / kPage * kPage;
  s->cap_attrs = (attr_capacity + kPage - 1) / kPage * kPage;
  try {
    s->nodes.assign(s->cap_nodes, yv_vox_node());
    s->attrs.assign(s->cap_attrs, yv_leaf_attr());
    // a page is sent once its version differs from the one last sent
    s->ver_n.assign(s->cap_nodes / kPage, 0);
    s->sent_n.assign(s->cap_nodes / kPage, 0);
    s->ver_a.assign(s->cap_attrs / kPage, 0);
    s->sent_a.assign(s->cap_attrs / kPage, 0);
  } catch (const std::bad_alloc&) {
    delete s;
    return YV_ERR_OUT_OF_MEMORY;
  }
  cudaError_t e = cudaGetDevice(&s->device);
  if (e == cudaSuccess) e = cudaMalloc(&s->d_nodes, (size_t)s->cap_nodes * sizeof(yv_vox_node));
  if (e == cudaSuccess) e = cudaMalloc(&s->d_attrs, (size_t)s->cap_attrs * sizeof(yv_leaf_attr));
  if (e != cudaSuccess) {
    cudaFree(s->d_nodes);
    cudaFree(s->d_attrs);
    delete s;
    return dyn_fail(e, "create");
  }
  *out = s;
  return YV_OK;
}

void yv_svo_dynamic_destroy(yv_svo_dynamic* s) {
  if (!s) return;
  cudaSetDevice(s->device);
  cudaFree(s->d_nodes);
  cudaFree(s->d_attrs);
  cudaFreeHost(s->h_stage);
  cudaFree(s->d_stage);
  cudaFree(s->d_slots);
  delete s;
}

yv_status yv_svo_dynamic_load(yv_svo_dynamic* s, const yv_svo_host* svo) {
  if (!s || !svo) return YV_ERR_INVALID_ARG;
  const uint32_t nn = yv_svo_node_count(svo), na = yv_svo_attr_count(svo);
  if (nn > s->cap_nodes || na > s->cap_attrs) return YV_ERR_UNSUPPORTED;
  std::memcpy(s->nodes.data(), yv_svo_nodes(svo), (size_t)nn * sizeof(yv_vox_node));
  std::memcpy(s->attrs.data(), yv_svo_attrs(svo), (size_t)na * sizeof(yv_leaf_attr));
  s->n_nodes = nn;
  s->n_attrs = na;
  s->free_nodes.clear();
  s->root = yv_svo_root(svo);
  s->depth = yv_svo_depth(svo);
  for (uint32_t p = 0; p < (nn + kPage - 1) / kPage; ++p) ++s->ver_n[p];
  for (uint32_t p = 0; p < (na + kPage - 1) / kPage; ++p) ++s->ver_a[p];
  return YV_OK;
}

yv_status yv_svo_dynamic_alloc_node(yv_svo_dynamic* s, uint32_t* id) {
  if (!s || !id) return YV_ERR_INVALID_ARG;
  uint32_t i;
  if (!s->free_nodes.empty()) {
    i = s->free_nodes.back();
    s->free_nodes.pop_back();
  } else {
    if (s->n_nodes >= s->cap_nodes) return YV_ERR_OUT_OF_MEMORY;
    i = s->n_nodes++;
  }
  std::memset(&s->nodes[i], 0, sizeof(yv_vox_node));
  for (int ch = 0; ch < 8; ++ch) s->nodes[i].child[ch] = YV_EMPTY_NODE;
  s->nodes[i].flags = 0xFF00u;
  touch_node(s, i);
  *id = i;
  return YV_OK;
}

yv_status yv_svo_dynamic_free_node(yv_svo_dynamic* s, uint32_t id) {
  if (!s || id >= s->n_nodes) return YV_ERR_INVALID_ARG;
  s->free_nodes.push_back(id);
  return YV_OK;
}

yv_status yv_svo_dynamic_set_node(yv_svo_dynamic* s, uint32_t id, const yv_vox_node* n) {
  if (!s || !n || id >= s->n_nodes) return YV_ERR_INVALID_ARG;
  s->nodes[id] = *n;
  touch_node(s, id);
  return YV_OK;
}

yv_status yv_svo_dynamic_get_node(const yv_svo_dynamic* s, uint32_t id, yv_vox_node* n) {
  if (!s || !n || id >= s->n_nodes) return YV_ERR_INVALID_ARG;
  *n = s->nodes[id];
  return YV_OK;
}

yv_status yv_svo_dynamic_add_attr(yv_svo_dynamic* s, const yv_leaf_attr* a, uint32_t* index) {
  if (!s || !a || !index) return YV_ERR_INVALID_ARG;
  if (s->n_attrs >= s->cap_attrs) return YV_ERR_OUT_OF_MEMORY;
  const uint32_t i = s->n_attrs++;
  s->attrs[i] = *a;
  touch_attr(s, i);
  *index = i;
  return YV_OK;
}

yv_status yv_svo_dynamic_set_attr(yv_svo_dynamic* s, uint32_t index, const yv_leaf_attr* a) {
  if (!s || !a || index >= s->n_attrs) return YV_ERR_INVALID_ARG;
  s->attrs[index] = *a;
  touch_attr(s, index);
  return YV_OK;
}

// Sets (a != NULL) or clears one voxel of a 2^depth grid: descends from the
// root, splitting EmptyNode / FullNode children into nodes where needed, and
// writes the leaf; nodes are not collapsed when they become empty.
yv_status yv_svo_dynamic_set_voxel(yv_svo_dynamic* s, int32_t depth, uint32_t x, uint32_t y,
                                   uint32_t z, const yv_leaf_attr* a) {
  if (!s || depth < 1 || depth > 16) return YV_ERR_INVALID_ARG;
  const uint32_t G = 1u << depth;
  if (x >= G || y >= G || z >= G) return YV_ERR_INVALID_ARG;
  if (s->root & 0x80000000u) {
    if (!a && s->root == YV_EMPTY_NODE) return YV_OK;
    const uint32_t fill = s->root;
    uint32_t r;
    yv_status st = yv_svo_dynamic_alloc_node(s, &r);
    if (st != YV_OK) return st;
    for (int ch = 0; ch < 8; ++ch) s->nodes[r].child[ch] = fill;
    s->root = r;
    s->depth = depth;
  }
  uint32_t node = s->root;
  for (int level = 0; level < depth - 1; ++level) {
    const int sh = depth - 1 - level;
    const int ch = (int)(((x >> sh) & 1u) | (((y >> sh) & 1u) << 1) | (((z >> sh) & 1u) << 2));
    yv_vox_node& n = s->nodes[node];
    if ((n.flags >> ch) & 1u) return YV_ERR_BAD_POOL;  // a leaf above the voxel level
    uint32_t w = n.child[ch];
    if (w & 0x80000000u) {
      if (!a && w == YV_EMPTY_NODE) return YV_OK;
      uint32_t c;
      yv_status st = yv_svo_dynamic_alloc_node(s, &c);
      if (st != YV_OK) return st;
      for (int k = 0; k < 8; ++k) s->nodes[c].child[k] = w;  // split the uniform region
      yv_vox_node& m = s->nodes[node];  // (the pool does not move: fixed capacity)
      m.child[ch] = c;
      m.flags &= ~(1u << (8 + ch));
      touch_node(s, node);
      w = c;
    } else if (w >= s->n_nodes) {
      return YV_ERR_BAD_POOL;
    }
    node = w;
  }
  const int ch = (int)((x & 1u) | ((y & 1u) << 1) | ((z & 1u) << 2));
  yv_vox_node& n = s->nodes[node];
  if (a) {
    if ((n.flags >> ch) & 1u) {
      s->attrs[n.child[ch]] = *a;
      touch_attr(s, n.child[ch]);
    } else {
      uint32_t idx;
      yv_status st = yv_svo_dynamic_add_attr(s, a, &idx);
      if (st != YV_OK) return st;
      n.child[ch] = idx;
      n.flags = (n.flags | (1u << ch)) & ~(1u << (8 + ch));
    }
  } else {
    n.child[ch] = YV_EMPTY_NODE;
    n.flags = (n.flags & ~(1u << ch)) | (1u << (8 + ch));
  }
  touch_node(s, node);
  return YV_OK;
}

// Copies the device mirror back (verification).
yv_status yv_svo_dynamic_download(const yv_svo_dynamic* s, yv_vox_node* nodes,
                                  yv_leaf_attr* attrs) {
  if (!s || !nodes || !attrs) return YV_ERR_INVALID_ARG;
  cudaError_t e = cudaSetDevice(s->device);
  if (e == cudaSuccess && s->n_nodes)
    e = cudaMemcpy(nodes, s->d_nodes, (size_t)s->n_nodes * sizeof(yv_vox_node),
                   cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && s->n_attrs)
    e = cudaMemcpy(attrs, s->d_attrs, (size_t)s->n_attrs * sizeof(yv_leaf_attr),
                   cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? YV_OK : dyn_fail(e, "download");
}

yv_status yv_svo_dynamic_set_root(yv_svo_dynamic* s, uint32_t root, int32_t depth) {
  if (!s || (!(root & 0x80000000u) && root >= s->n_nodes) || depth < 0 || depth > 16)
    return YV_ERR_INVALID_ARG;
  s->root = root;
  s->depth = depth;
  return YV_OK;
}

// CountChangedPages / CountTransfrerSize (qtview.py:69-73)
uint32_t yv_svo_dynamic_changed_pages(const yv_svo_dynamic* s) {
  if (!s) return 0;
  return changed(s->ver_n, s->sent_n) + changed(s->ver_a, s->sent_a);
}

uint64_t yv_svo_dynamic_transfer_bytes(const yv_svo_dynamic* s) {
  if (!s) return 0;
  return (uint64_t)changed(s->ver_n, s->sent_n) * kPage * sizeof(yv_vox_node) +
         (uint64_t)changed(s->ver_a, s->sent_a) * kPage * sizeof(yv_leaf_attr);
}

// SVORenderer::UpdateSVO: sends the changed pages on `stream`.
yv_status yv_svo_dynamic_sync(yv_svo_dynamic* s, void* stream) {
  if (!s) return YV_ERR_INVALID_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaSetDevice(s->device);
  if (e == cudaSuccess)
    e = sync_array(s, reinterpret_cast<const uint8_t*>(s->nodes.data()), sizeof(yv_vox_node),
                   s->n_nodes, s->ver_n, s->sent_n, s->d_nodes, st);
  if (e == cudaSuccess)
    e = sync_array(s, reinterpret_cast<const uint8_t*>(s->attrs.data()), sizeof(yv_leaf_attr),
                   s->n_attrs, s->ver_a, s->sent_a, s->d_attrs, st);
  if (e != cudaSuccess) return dyn_fail(e, "sync");
  s->synced_root = s->root;
  s->synced_nodes = s->n_nodes;
  s->synced_attrs = s->n_attrs;
  return YV_OK;
}

// The device mirror as of the last sync, for yv_render_svo_noalloc and the
// renderer (SVORenderer::UpdateSVO hands the tree to the kernels after the
// transfer, demo/SVORenderer.cpp:39-53).
yv_status yv_svo_dynamic_device(const yv_svo_dynamic* s, const yv_vox_node** nodes,
                                uint32_t* count, uint32_t* root, const yv_leaf_attr** attrs,
                                uint32_t* nattrs) {
  if (!s || !nodes || !count || !root || !attrs || !nattrs) return YV_ERR_INVALID_ARG;
  *nodes = s->d_nodes;
  *count = s->synced_nodes;
  *root = s->synced_root;
  *attrs = s->d_attrs;
  *nattrs = s->synced_attrs;
  return YV_OK;
}

yv_status yv_svo_dynamic_host_info(const yv_svo_dynamic* s, uint32_t* count, uint32_t* root,
                                   uint32_t* nattrs) {
  if (!s || !count || !root || !nattrs) return YV_ERR_INVALID_ARG;
  *count = s->n_nodes;
  *root = s->root;
  *nattrs = s->n_attrs;
  return YV_OK;
}

const yv_vox_node* yv_svo_dynamic_host_nodes(const yv_svo_dynamic* s) {
  return s ? s->nodes.data() : nullptr;
}
const yv_leaf_attr* yv_svo_dynamic_host_attrs(const yv_svo_dynamic* s) {
  return s ? s->attrs.data() : nullptr;
}

}  // extern "C"
