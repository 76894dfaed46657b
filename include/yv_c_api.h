/*
 * yv_c_api.h - C ABI of the GB300 sparse-voxel-octree / brick-volume ray caster.
 *
 * Plain C types only (pointers, sizes, PODs); no C++ or torch types cross this
 * boundary.  Every function returns a yv_status (0 = ok); nothing aborts and
 * no exception escapes.  One renderer object per host thread.
 *
 * Device pointers are passed as void* and streams as void* (a cudaStream_t;
 * NULL = legacy default stream).
 *
 * Reference interfaces replaced (paths inside znah/yoxel-voxel):
 *   ISVORenderer            cell/svorenderer.h:5-31
 *   RendererBase            cell/renderer_base.h:7-62
 *   CUDA SVORenderer        demo/SVORenderer.h:8-64, demo/SVORenderer.cpp:39-149
 *   SVOData / VoxNode       cell/svodata.h:22-55, reaction/report/main.tex:36-56
 *   ntree RunTrace C ABI    ntree/ntree_trace.cuh:22-28
 *   Python CudaRenderer     trace_cuda.py:17-120
 */
#ifndef YV_C_API_H
#define YV_C_API_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Status codes                                                             */
/* ------------------------------------------------------------------------ */
typedef int32_t yv_status;
#define YV_OK                 0
#define YV_ERR_INVALID_ARG    1  /* NULL pointer, bad size, bad enum          */
#define YV_ERR_NO_SCENE       2  /* render before a scene was set             */
                                 /* (RenderFrame returns NULL in the reference:
                                    cell/ppu_renderer.cpp:78-79)              */
#define YV_ERR_BAD_POOL       3  /* node/brick pool failed validation         */
#define YV_ERR_ITERATION_CAP  4  /* a ray hit the per-ray iteration cap       */
#define YV_ERR_TIMEOUT        5  /* the frame time budget ran out             */
#define YV_ERR_CUDA           6  /* a CUDA runtime call failed                */
#define YV_ERR_OUT_OF_MEMORY  7
#define YV_ERR_IO             8  /* file could not be read / written          */
#define YV_ERR_UNSUPPORTED    9

/* Human-readable name of a status code (static string). */
const char* yv_status_string(yv_status s);

/* Detail text of the last failure in this process (CUDA error string or the
 * validation failure); empty if none.  Valid until the next failing call. */
const char* yv_last_error(void);

/* ------------------------------------------------------------------------ */
/* Scene data: the reference SVO node layout                                */
/* ------------------------------------------------------------------------ */

/* VoxNode, 40 bytes (reaction/report/main.tex:38-52, cell/svodata.h:22-55).
 *   flags bits 0..7  : child i is a leaf (child[i] holds VoxData)
 *   flags bits 8..15 : child i is null (EmptyNode / FullNode)
 *   flags bit  19    : empty flag
 *   data             : coarse-LOD VoxData of the subtree (the level-of-detail
 *                      attribute index, see yv_svo_build_lod)
 *   child[i]         : node index, VoxData (leaf) or a null id (bit 31 set).
 * Child order: bit 0 of i = +x half, bit 1 = +y half, bit 2 = +z half.
 * VoxData of a leaf is an index into the leaf attribute array. */
typedef struct yv_vox_node {
  uint32_t flags;
  uint32_t data;
  uint32_t child[8];
} yv_vox_node;

#define YV_EMPTY_NODE 0x80000000u /* main.tex:54 */
#define YV_FULL_NODE  0x80000001u /* main.tex:55 */

/* Leaf attribute (8 bytes): uint8 RGB colour + int8x3 quantised normal
 * (127 * unit normal), the colour/normal pair of ore/src/main.cpp:37-51. */
typedef struct yv_leaf_attr {
  uint8_t r, g, b, a;
  int8_t nx, ny, nz, nw;
} yv_leaf_attr;

/* Host-side SVO container produced by a generator or a loader. */
typedef struct yv_svo_host yv_svo_host;

/* Seeded sphere-union scene in a 2^depth grid: n spheres, centres uniform in
 * the grid, radius uniform in [rmin, rmax] voxels, one random RGB per sphere;
 * surface voxel = inside the union with >= 1 of its 6 neighbours outside;
 * normal = normalize(voxel centre - centre of the first sphere holding it);
 * interior subtrees = FullNode.  (Surface rule of scene_gen.py:32-66.) */
yv_status yv_svo_gen_spheres(yv_svo_host** out, int depth, int n_spheres,
                             float rmin, float rmax, uint64_t seed);

/* Seeded terrain scene in a 2^depth grid: 6-octave value-noise heightfield
 * (amplitude 0.3 of the grid height, solid below the surface) plus n_cubes
 * floating axis-aligned cubes of side [cube_min, cube_max] voxels.  Normals
 * from heightfield central differences (scene_gen.py:49-53) or from the cube
 * centre. */
yv_status yv_svo_gen_terrain(yv_svo_host** out, int depth, int n_cubes,
                             int cube_min, int cube_max, uint64_t seed);

/* Copy caller arrays into a host container (caller keeps ownership). */
yv_status yv_svo_from_arrays(yv_svo_host** out, const yv_vox_node* nodes,
                             uint32_t count, uint32_t root,
                             const yv_leaf_attr* attrs, uint32_t nattrs);

/* A host container from a reference pool held in memory as SVOData holds it
 * (cell/svodata.h:20-55): leaves and every node's `data` carry the packed
 * VoxData of reaction/report/main.tex:38,65 (16-bit RGB565 colour, 16-bit
 * octahedral int8x2 normal), decoded into leaf attributes exactly as a .vox
 * file without an attribute section is (the scene then has level-of-detail
 * data).  Node ids are kept. */
yv_status yv_svo_from_packed(yv_svo_host** out, const yv_vox_node* nodes,
                             uint32_t count, uint32_t root);

/* .vox file (SVOData::Load, cell/svodata.h:31-50): little-endian
 * uint32 root, uint32, uint32, uint32 size, VoxNode[size]; followed by an
 * optional attribute section "YVAT" uint32 count, yv_leaf_attr[count], and
 * an optional marker "YVLD" saying that every node's `data` indexes its
 * level-of-detail attribute.  A file without the attribute section holds
 * the reference's packed VoxData (16-bit colour, 16-bit normal) in leaves
 * and in node `data`; both are decoded into attributes (the scene then has
 * level-of-detail data). */
yv_status yv_svo_load_vox(yv_svo_host** out, const char* path);
yv_status yv_svo_save_vox(const yv_svo_host* svo, const char* path);

/* Level-of-detail data (the node `data` field of
 * reaction/report/main.tex:61: the subtree shown at a coarser level): for
 * every node, the mean colour and mean normal of all leaves of its subtree
 * (each component the integer mean rounded half away from zero, alpha 255)
 * become a new attribute, appended after the existing ones in node order,
 * and the node's `data` indexes it. */
yv_status yv_svo_build_lod(yv_svo_host* svo);
/* 1 if every node's `data` is a level-of-detail attribute index. */
int       yv_svo_has_lod(const yv_svo_host* svo);

void               yv_svo_free(yv_svo_host* svo);
uint32_t           yv_svo_node_count(const yv_svo_host* svo);
uint32_t           yv_svo_root(const yv_svo_host* svo);
const yv_vox_node* yv_svo_nodes(const yv_svo_host* svo);
uint32_t           yv_svo_attr_count(const yv_svo_host* svo);
const yv_leaf_attr* yv_svo_attrs(const yv_svo_host* svo);
/* Tree depth (levels of nodes below the root that carry leaves); 0 if empty. */
int                yv_svo_depth(const yv_svo_host* svo);

/* GPU build of the canonical SVO from a dense density grid: the iso/raw
 * source form of DynamicSVO::BuildRange (ore/src/main.cpp:37-129,
 * demo/Demo.cpp:82-114).  density: DEVICE float array of (2^depth)^3
 * values, x fastest (index x + G*(y + G*z)); rgb: DEVICE uint8 RGB per voxel
 * or NULL (white).  Voxel solid iff density > iso; surface voxel = solid
 * with a 6-neighbour outside the grid or not solid (a leaf); regions without
 * surface voxels are EmptyNode / FullNode; nodes and leaves breadth-first.
 * Leaf normal = floor(127 u + 0.5) of u = the central difference
 * (d(x-1)-d(x+1), ...) (coordinates clamped to the grid) over its length,
 * every step FP32 round-to-nearest (zero for a zero or non-finite length).
 * 1 <= depth <= 11.  Runs on `stream`, then copies the pool into a new host
 * container. */
yv_status yv_svo_build_dense(const float* density, const uint8_t* rgb,
                             int32_t depth, float iso, void* stream,
                             yv_svo_host** out);

/* Host-side validation: child indices in range, leaf VoxData < nattrs,
 * depth <= 16, no cycles.  YV_OK or YV_ERR_BAD_POOL. */
yv_status yv_svo_validate(const yv_vox_node* nodes, uint32_t count,
                          uint32_t root, uint32_t nattrs);

/* ------------------------------------------------------------------------ */
/* SVO renderer (ISVORenderer / SVORenderer)                                */
/* ------------------------------------------------------------------------ */
typedef struct yv_renderer yv_renderer;

/* Directional light + shading (Lambert: ambient + diffuse * max(0, n.L)).
 * shadows != 0 casts one hard-shadow ray per primary hit toward dir. */
typedef struct yv_light {
  float dir[3];     /* direction toward the light (normalised by the caller) */
  float ambient;
  float diffuse;
  int32_t shadows;
} yv_light;

/* Output buffers of one frame, all DEVICE pointers, each optional (NULL):
 *   rgba      : uint32 per pixel, R | G<<8 | B<<16 | A<<24 (Color32)
 *   hit       : uint32 per pixel, (reference node id << 3) | child, or
 *               0xFFFFFFFF for a miss (TraceResult, cell/ppu_renderer.cpp:8-13)
 *   hit_t     : float per pixel, t of the hit (max(t1) of the leaf box)
 *   fetches   : uint32 per pixel, node dereferences of the primary ray
 *               (RecTrace calls that reach cell/ppu_renderer.cpp:23)
 *   shadow_fetches : uint32 per pixel, same for the shadow ray
 *   normal    : 3 floats per pixel, the unit normal of the hit leaf's
 *               attribute (0, 0, 0 for a miss)
 * Row-major, y*width + x. */
typedef struct yv_frame_outputs {
  void* rgba;
  void* hit;
  void* hit_t;
  void* fetches;
  void* shadow_fetches;
  void* normal;
} yv_frame_outputs;

/* Counters of the last frame (read by yv_renderer_frame_stats). */
typedef struct yv_frame_stats {
  uint64_t primary_rays;
  uint64_t hits;
  uint64_t shadow_rays;
  uint64_t shadowed;
  uint32_t status;       /* yv_status of the device side */
  uint32_t launches;     /* kernels launched for the frame */
} yv_frame_stats;

/* Launch configuration (the autotuned knobs).  Zero fields = defaults. */
typedef struct yv_launch_config {
  int32_t block_threads;   /* threads per block (multiple of 32)          */
  int32_t blocks_per_sm;   /* resident blocks per SM for the persistent grid */
  int32_t smem_nodes;      /* top-of-tree nodes staged in shared memory   */
  int32_t tile_rays;       /* rays a warp takes per queue pop (32|64|128) */
} yv_launch_config;

yv_status yv_renderer_create(yv_renderer** out);
void      yv_renderer_destroy(yv_renderer* r);

/* ISVORenderer::SetScene.  Copies the pool to the device in the renderer's
 * own layout; the caller keeps ownership of its arrays. */
yv_status yv_set_scene_svo(yv_renderer* r, const yv_vox_node* nodes,
                           uint32_t count, uint32_t root,
                           const yv_leaf_attr* attrs, uint32_t nattrs);
yv_status yv_set_scene_host(yv_renderer* r, const yv_svo_host* svo);
/* ISVORenderer::SetScene(SVOData*) for a pool in the reference's own packed
 * leaf format (yv_svo_from_packed): no separate attribute array needed.
 * Hit ids are the pool's node ids. */
yv_status yv_set_scene_svo_packed(yv_renderer* r, const yv_vox_node* nodes,
                                  uint32_t count, uint32_t root);
yv_status yv_load_scene_vox(yv_renderer* r, const char* path);
/* SVORenderer::SetScene(DynamicSVO*) (demo/SVORenderer.cpp:33-53): the
 * renderer keeps a non-owning pointer to an editable scene (declared below)
 * and traces its device mirror in place, as of the scene's last
 * yv_svo_dynamic_sync (UpdateSVO); hit words carry the pool's own node ids.
 * The scene must outlive the binding.  Not batchable; no level-of-detail
 * cut-off. */
typedef struct yv_svo_dynamic yv_svo_dynamic;
yv_status yv_set_scene_dynamic(yv_renderer* r, const yv_svo_dynamic* s);
/* The same GPU build (yv_svo_build_dense) straight into the renderer's
 * device layout: no host copy of the pool.  Node ids are the breadth-first
 * ids of yv_svo_build_dense. */
yv_status yv_set_scene_dense(yv_renderer* r, const float* density,
                             const uint8_t* rgb, int32_t depth, float iso,
                             void* stream);

/* Camera: ISVORenderer::SetViewPos/SetViewDir/SetViewUp/SetResolution/
 * GetResolution/SetFOV (cell/svorenderer.h:12-21).  Defaults follow
 * RendererBase (cell/renderer_base.h:25): up (0,0,1), fov 70, 640x480. */
yv_status yv_set_view_pos(yv_renderer* r, const float pos[3]);
yv_status yv_set_view_dir(yv_renderer* r, const float dir[3]);
yv_status yv_set_view_up(yv_renderer* r, const float up[3]);
yv_status yv_set_resolution(yv_renderer* r, int width, int height);
yv_status yv_get_resolution(const yv_renderer* r, int* width, int* height);
yv_status yv_set_fov(yv_renderer* r, float fov_deg);
yv_status yv_get_fov(const yv_renderer* r, float* fov_deg);  /* SVORenderer::GetFOV */
yv_status yv_set_light(yv_renderer* r, const yv_light* light);
/* SVORenderer::SetDetailCoef / GetDetailCoef (demo/SVORenderer.h:25-26):
 * level-of-detail cut-off.  With coef > 0 and a scene set from a host
 * container with level-of-detail data, a ray stops at a subtree whose cube
 * side is smaller than t * coef * radians(fov / 2) / width (t the distance
 * to the subtree's entry face; SVORenderer.cpp:104) and shades it with the
 * subtree's attribute; the hit word is then (parent << 3) | child slot, as
 * for a leaf in that slot.  0 (the default): exact leaves. */
yv_status yv_set_detail_coef(yv_renderer* r, float coef);
yv_status yv_get_detail_coef(const yv_renderer* r, float* coef);
/* Frame time budget of the persistent ray queue (no reference counterpart:
 * the reference renders a frame to completion).  With microseconds > 0, a
 * warp of the frame kernel takes no new rays once that long has passed
 * since its block started (the GPU global timer); rays in flight finish,
 * pixels of rays never taken are left unwritten, and the frame's status
 * (yv_renderer_frame_stats, yv_render_frame) is YV_ERR_TIMEOUT.  Applies
 * to yv_render_frame, yv_render_frame_async and yv_render_frame_tiles.
 * 0 (the default): no budget. */
yv_status yv_set_frame_budget(yv_renderer* r, uint32_t microseconds);
yv_status yv_get_frame_budget(const yv_renderer* r, uint32_t* microseconds);
yv_status yv_set_launch_config(yv_renderer* r, const yv_launch_config* cfg);
yv_status yv_get_launch_config(const yv_renderer* r, yv_launch_config* cfg);

/* ISVORenderer::RenderFrame.  Synchronous.  Writes RGBA8 to host_rgba
 * and/or device_rgba (either may be NULL; width*height uint32 each) on the
 * given stream, waits for it and returns the device status. */
yv_status yv_render_frame(yv_renderer* r, uint32_t* host_rgba,
                          void* device_rgba, void* stream);

/* Asynchronous form of SVORenderer::Render(void* d_dstBuf): enqueues the
 * frame on `stream` writing the requested device outputs.  No host sync;
 * the status is read later with yv_renderer_frame_stats. */
yv_status yv_render_frame_async(yv_renderer* r, const yv_frame_outputs* out,
                                void* stream);

/* Tiles [tile_begin, tile_end) of the frame only: the frame is cut into
 * 8x4-pixel tiles numbered row-major (yv_get_tile_count), and just the
 * pixels of the given range are traced and written (outputs are full-frame
 * device buffers as for yv_render_frame_async).  The work split of the
 * reference's threaded renderer, which gives each thread a band of rows
 * (TreadedRenderer::RenderFrame, cell/ppu_renderer.cpp:121-144), and of its
 * SPU renderer, which gives each SPE a stride of 16x16 tiles
 * (cell/spu/trace_spu.cpp:162-177): a frame split into tile ranges over
 * several GPUs (or calls) and merged gives the full frame bit for bit.
 * yv_renderer_frame_stats then counts the range's pixels. */
#define YV_TILE_W 8
#define YV_TILE_H 4
yv_status yv_render_frame_tiles(yv_renderer* r, uint32_t tile_begin,
                                uint32_t tile_end, const yv_frame_outputs* out,
                                void* stream);
yv_status yv_get_tile_count(const yv_renderer* r, uint32_t* tiles_x,
                            uint32_t* tiles_y);

/* Synchronises the last frame's stream and returns its counters. */
yv_status yv_renderer_frame_stats(yv_renderer* r, yv_frame_stats* stats);

/* Fills the camera basis the kernels use (RendererBase::InitRayDir,
 * cell/renderer_base.h:50-61): dir0, du, dv (3 floats each). */
yv_status yv_get_ray_basis(const yv_renderer* r, float dir0[3], float du[3],
                           float dv[3]);

/* Number of nodes of the device copy and bytes it occupies. */
yv_status yv_get_device_scene_info(const yv_renderer* r, uint64_t* nodes,
                                   uint64_t* device_bytes);

/* ------------------------------------------------------------------------ */
/* Brick volumes: the ntree layout (ntree/ntree/gpu_nodes.h:6-21,            */
/* ntree/ntree/nodes.h:13-100, ntree/BrickManager.h:5-80)                   */
/* ------------------------------------------------------------------------ */
/* Tree of N^3 grid nodes, N = 4; child c = (z*4 + y)*4 + x
 * (ntree/ntree/nodes.h:99).  A child ref is 0x80000000 (empty Const node),
 * 0x40000000 | b (brick b, last grid level only) or a grid node index.
 * Scene size = 8 * 4^levels lattice cells (CalcSceneSize with B = 8).
 * A brick is a 9^3 lattice (8^3 cells + the far-side apron repeating the
 * first layer of its +x/+y/+z neighbours), index (z*9 + y)*9 + x. */
typedef struct yv_volume_host yv_volume_host;

/* Seeded noise volume: density = clamp(amplitude*n(p) - offset, 0, 1) with
 * n a normalised 4-octave 3D value noise, albedo = per-lattice-point uint8
 * RGB from three further noise fields; bricks whose 9^3 lattice is all zero
 * are culled (empty refs). */
yv_status yv_volume_gen_noise(yv_volume_host** out, int levels, float offset,
                              float amplitude, uint64_t seed);
/* RangeBuilder (ntree/ntree/ntree.h:11-63) from a dense (S+1)^3 lattice,
 * x fastest; albedo_rgb may be NULL (white). */
yv_status yv_volume_from_dense(yv_volume_host** out, int levels,
                               const float* density, const uint8_t* albedo_rgb);
void            yv_volume_free(yv_volume_host* v);
int             yv_volume_levels(const yv_volume_host* v);
uint32_t        yv_volume_grid_count(const yv_volume_host* v);
const uint32_t* yv_volume_grids(const yv_volume_host* v);
uint32_t        yv_volume_brick_count(const yv_volume_host* v);
const float*    yv_volume_density(const yv_volume_host* v);   /* nbricks*729 */
const uint8_t*  yv_volume_albedo(const yv_volume_host* v);    /* nbricks*729*3 */
const int32_t*  yv_volume_brick_cells(const yv_volume_host* v); /* nbricks*3 */
/* Apron neighbour table, nbricks*7 (-1 = absent), index m-1 for the offset
 * m = dx | dy<<1 | dz<<2: upper != 0 -> brick at +offset (owner of my
 * apron slots), upper == 0 -> brick at -offset. */
const int32_t*  yv_volume_neighbors(const yv_volume_host* v, int upper);

#define YV_PRECISION_F16 0  /* fp16 density, uchar4 albedo (render only) */
#define YV_PRECISION_F32 1  /* fp32 density, fp32 RGB albedo (learnable)  */
/* Packed lattice points: the whole point in `albedo`, density == NULL.   */
#define YV_PRECISION_F32_PACKED 2 /* float4 (r, g, b, density) (learnable) */
#define YV_PRECISION_F16_PACKED 3 /* 8 B {fp16 density | r<<16 | g<<24, b},
                                     RGB8 (render only)                     */

/* GPU build of the brick volume from a dense DEVICE lattice of (S+1)^3
 * floats, S = 8 * 4^levels, x fastest (index x + (S+1)*(y + (S+1)*z)), with
 * an optional DEVICE uint8 RGB lattice (NULL: white): the result of
 * yv_volume_from_dense (RangeBuilder, ntree/ntree/ntree.h:11-63), bit for
 * bit, built on `stream` and copied into a new host container.  1 <= levels
 * <= 4. */
yv_status yv_volume_build_dense(const float* density, const uint8_t* rgb,
                                int32_t levels, void* stream,
                                yv_volume_host** out);

/* Device view of a volume: all pointers are device pointers. */
typedef struct yv_volume_device {
  const uint32_t* grids;
  uint32_t ngrids;
  int32_t levels;
  const void* density;
  const void* albedo;
  uint32_t nbricks;
  int32_t precision;
  const int32_t* nbr_up;
  const int32_t* nbr_dn;
  /* optional (NULL = none): per brick 16 words, bit (y & 3) * 8 + x of word
   * z * 2 + (y >> 2) set where trilinear cell (x, y, z) has a non-zero
   * density corner.  The forward march passes over the samples of cells
   * without one (they add nothing: alpha 0), counting them as taken.  Pools
   * owned by the library (yv_volume_upload, yv_volume_upload_dense,
   * yv_volume_rebuild_dense) carry it; a pool whose densities change between
   * frames (the learnable tensors) leaves it NULL. */
  const uint32_t* cell_mask;
  /* optional (NULL = none): one bit per brick cell of the tree, bit
   * (ci & 31) of word ci >> 5 for ci = (cz * nb + cy) * nb + cx, nb =
   * 4^levels, set unless the tree holds no brick there.  The march tests it
   * before descending the tree for a cell, so the empty cells a ray crosses
   * cost one load instead of a descent.  It depends on the grids only
   * (yv_volume_brick_bits computes it); library-owned pools of up to 4
   * levels carry it. */
  const uint32_t* brick_bits;
} yv_volume_device;

/* Words of the brick_bits array of a tree of `levels` levels:
 * ceil(4^(3 levels) / 32). */
#define YV_BRICK_BITS_WORDS(levels) \
  ((((uint64_t)1 << (6 * (levels))) + 31u) / 32u)

/* Computes the brick_bits array of v's tree (v->grids, ngrids, levels,
 * nbricks) into `bits` (device, YV_BRICK_BITS_WORDS(levels) words), on
 * `stream`.  v->brick_bits is not read.  No reference counterpart (the
 * reference descends the tree for every cell). */
yv_status yv_volume_brick_bits(const yv_volume_device* v, uint32_t* bits, void* stream);

/* Device copy owned by the library (BrickPool<T>, ntree/BrickManager.h). */
typedef struct yv_volume_gpu yv_volume_gpu;
yv_status yv_volume_upload(const yv_volume_host* v, int32_t precision,
                           yv_volume_gpu** out);
void      yv_volume_gpu_free(yv_volume_gpu* g);
/* The same GPU build straight into a device pool of the given precision
 * (the brick-pool construction of reaction/voxtree/density.cu:30-284 and
 * BrickPool::Update, reaction/voxtree/brickpool/BrickPool.cpp:21-62): no host
 * copy of the pool; equal to yv_volume_upload of yv_volume_from_dense. */
yv_status yv_volume_upload_dense(const float* density, const uint8_t* rgb,
                                 int32_t levels, int32_t precision, void* stream,
                                 yv_volume_gpu** out);
/* BrickPool::Update in place: rebuilds `vol` (same precision) from a new
 * lattice on `stream`, reusing its device arrays when they are large enough
 * (growing them otherwise).  Work already queued that reads `vol` must be
 * ordered before this call by the caller (same stream, or a sync), and a
 * yv_volume_device taken from `vol` before the call is stale after it:
 * take it again with yv_volume_gpu_desc. */
yv_status yv_volume_rebuild_dense(yv_volume_gpu* vol, const float* density,
                                  const uint8_t* rgb, int32_t levels,
                                  void* stream);
yv_status yv_volume_gpu_desc(const yv_volume_gpu* g, yv_volume_device* out);

/* Pinhole camera (RendererBase fields, cell/renderer_base.h:13-21). */
typedef struct yv_camera {
  float pos[3];
  float dir[3];
  float up[3];
  float fov_deg;
} yv_camera;

/* March parameters: alpha = saturate(alpha_scale * density) per sample,
 * samples every step_vox lattice cells (reaction/trace/trace.cu:44). */
typedef struct yv_march_params {
  float alpha_scale;
  float step_vox;
} yv_march_params;

/* Front-to-back composited RGBA (4 floats per pixel, camera-major) of
 * ncams cameras; the volume counterpart of RunTrace
 * (ntree/ntree_trace.cuh:27).  samples / bricks (optional, uint32 per
 * pixel) count samples taken and occupied bricks entered. */
yv_status yv_volume_render(const yv_volume_device* vol, const yv_camera* cams,
                           int32_t ncams, int32_t width, int32_t height,
                           const yv_march_params* mp, float* rgba,
                           uint32_t* samples, uint32_t* bricks, void* stream);

/* A frame split into ranges of warp tiles (the multi-GPU shards of one
 * frame, as the SVO frames' yv_render_frame_tiles; no reference
 * counterpart).  The march takes 8x4-pixel tiles in 16x16-pixel squares of
 * 8: tile id = (square row * squares per row + square column) * 8 + (tile
 * row within the square) * 2 + tile column within the square, camera-major
 * over the ncams frames.  yv_volume_tile_count gives the tiles of one
 * camera's frame. */
yv_status yv_volume_tile_count(int32_t width, int32_t height, uint32_t* tiles_per_camera);
/* yv_volume_render over tiles [tile_begin, tile_end) of the ncams (<= 64)
 * frames only: the other pixels of rgba / samples / bricks are left as
 * they are.  Ranges that start on a multiple of 8 keep each block of the
 * launch on one 16x16-pixel square. */
yv_status yv_volume_render_tiles(const yv_volume_device* vol, const yv_camera* cams,
                                 int32_t ncams, int32_t width, int32_t height,
                                 const yv_march_params* mp, uint32_t tile_begin,
                                 uint32_t tile_end, float* rgba, uint32_t* samples,
                                 uint32_t* bricks, void* stream);

/* Adjoint of yv_volume_render (fp32 volumes, plain or packed): re-marches
 * every ray and accumulates dL/ddensity and dL/dalbedo (pool layout, ADDED
 * to the buffers) from dL/drgba, given the forward output rgba. */
/* RunTrace(const RenderParams&, uchar4* img, float*) (ntree/ntree_trace.cuh:
 * 22-28): the same march written as RGBA8 pixels, each channel
 * saturate(v) * 255 truncated, R in the low byte (float2uint,
 * reaction/trace/utils.h:37-44); rgba8: ncams*height*width uint32 (device). */
yv_status yv_volume_render_rgba8(const yv_volume_device* vol, const yv_camera* cams,
                                 int32_t ncams, int32_t width, int32_t height,
                                 const yv_march_params* mp, uint32_t* rgba8,
                                 void* stream);
yv_status yv_volume_backward(const yv_volume_device* vol,
                             const yv_camera* cams, int32_t ncams,
                             int32_t width, int32_t height,
                             const yv_march_params* mp, const float* rgba,
                             const float* grad_rgba, float* grad_density,
                             float* grad_albedo, void* stream);

/* Sums the gradient of every apron copy into its lattice point's owner and
 * writes the total back to all copies (zero where the owner brick is
 * absent), so that copies of a parameter stay equal under any update. */
yv_status yv_volume_fold_aprons(const yv_volume_device* vol,
                                float* grad_density, float* grad_albedo,
                                void* stream);
/* Copies owner values into the apron slots of fp32 density / albedo. */
yv_status yv_volume_sync_aprons(const yv_volume_device* vol, float* density,
                                float* albedo, void* stream);
/* packed[i] = (albedo[3i], albedo[3i+1], albedo[3i+2], density[i]) for
 * npoints lattice points (device pointers, packed 16-byte aligned): the
 * YV_PRECISION_F32_PACKED pool of fp32 parameters, rebuilt per step. */
yv_status yv_volume_pack(const float* density, const float* albedo,
                         uint32_t npoints, float* packed, void* stream);

/* ------------------------------------------------------------------------ */
/* Batched persistent render (no reference code; nearest structure is the   */
/* SPU tile loop, cell/spu/trace_spu.cpp:162-177)                           */
/* ------------------------------------------------------------------------ */
/* Up to 64 scenes+cameras of uneven depth and resolution - SVO first-hit
 * frames and brick-volume composites - traced in ONE persistent launch whose
 * warps pop 8x4-pixel tiles from a global ray queue (largest scenes first).
 * Per-ray results are bit-identical to the per-scene launches. */
typedef struct yv_batch yv_batch;
yv_status yv_batch_create(yv_batch** out);
void      yv_batch_destroy(yv_batch* b);
yv_status yv_batch_clear(yv_batch* b);
/* Adds the renderer's current scene, camera, light and resolution (a
 * snapshot; the renderer must outlive the batch); output: device RGBA8. */
yv_status yv_batch_add_svo(yv_batch* b, const yv_renderer* r, void* d_rgba);
/* The same with any of the renderer's per-pixel device outputs
 * (yv_frame_outputs: rgba, hit ids, hit t, fetch counts, shadow fetch
 * counts, normals), so a batched frame reports the hit voxel of every ray
 * ((node << 3) | child, TraceResult of cell/ppu_renderer.cpp:8-13) as a
 * per-scene launch does. */
yv_status yv_batch_add_svo_outputs(yv_batch* b, const yv_renderer* r,
                                   const yv_frame_outputs* out);
/* Adds one camera of a device volume; output: device RGBA float4. */
yv_status yv_batch_add_volume(yv_batch* b, const yv_volume_device* vol,
                              const yv_camera* cam, int32_t width,
                              int32_t height, const yv_march_params* mp,
                              float* d_rgba);
yv_status yv_batch_set_launch_config(yv_batch* b, const yv_launch_config* cfg);
/* One persistent launch for the whole batch on `stream`; use_graph != 0
 * replays a captured CUDA graph (re-captured after the batch changes). */
yv_status yv_batch_render(yv_batch* b, int32_t use_graph, void* stream);
/* The same work as one plain launch per scene (the batch's baseline). */
yv_status yv_batch_render_separate(yv_batch* b, void* stream);
yv_status yv_batch_info(const yv_batch* b, uint32_t* n_items, uint64_t* rays);

/* ------------------------------------------------------------------------ */
/* Allocation-free frame (no counterpart in the reference)                  */
/* ------------------------------------------------------------------------ */
/* For callers that cannot call cudaMalloc: code running while a stream is
 * captured into a CUDA graph, real-time loops that cannot take the device
 * synchronisation an allocation may cost, and hosts whose device memory is
 * owned by another allocator.  Renders one frame of an SVO that the caller
 * holds in DEVICE memory in the reference layout (nodes: count VoxNode
 * records, attrs: nattrs leaf attributes) into the caller's device outputs,
 * with the same results as yv_render_frame_async (hit ids are the pool's own
 * node indices).  Nothing is allocated: the frame's scratch (ray-queue
 * counter, status word, hit counters) is a 256-byte static device array that
 * every GPU loading the library keeps until exit.  The first call on a
 * device looks up that array's address (cudaGetSymbolAddress); make it
 * before any stream capture.  Every call shares the array and clears it on
 * `stream` first, so calls that overlap on the GPU (other streams, other
 * threads) race and must be serialised by the caller.  Asynchronous: returns
 * launch errors only; malformed pools are contained by the kernel's bounds
 * checks (validate the host copy with yv_svo_validate), and the frame's
 * device status is read with yv_render_svo_noalloc_status.  Frames needing more
 * than 2^31 rays (8x4-tile padded) or pools over 2^29 nodes return
 * YV_ERR_INVALID_ARG. */
yv_status yv_render_svo_noalloc(const yv_vox_node* nodes, uint32_t count,
                                uint32_t root, const yv_leaf_attr* attrs,
                                uint32_t nattrs, const yv_camera* cam,
                                const yv_light* light, int32_t width,
                                int32_t height, const yv_frame_outputs* out,
                                void* stream);
/* Device status of the last allocation-free frame on the current device:
 * waits for `stream` (the stream of that frame), reads the status word of
 * the static scratch array and returns YV_ERR_BAD_POOL (a child index outside
 * the pool, or a leaf attribute index outside attrs), YV_ERR_ITERATION_CAP
 * (a ray reached the fetch cap or the 16-level depth cap: a cycle or a
 * too-deep pool) or YV_OK; device_bits (optional) receives the raw bits.
 * Allocates nothing.  The word belongs to whichever call ran last on the
 * device, so it must be read before the next allocation-free frame starts. */
yv_status yv_render_svo_noalloc_status(void* stream, uint32_t* device_bits);

/* ------------------------------------------------------------------------ */
/* Editable SVO with incremental device sync (DynamicSVO,                   */
/* reaction/report/main.tex:67-71; SVORenderer::UpdateSVO,                  */
/* demo/SVORenderer.cpp:39-53; CountChangedPages / CountTransfrerSize,      */
/* qtview.py:69-73)                                                         */
/* ------------------------------------------------------------------------ */
/* A host VoxNode pool of fixed capacity (free list of node slots) and its
 * device mirror, both split into pages of 256 nodes (and 256 leaf
 * attributes) with a version per page bumped on every edit; a sync sends
 * only the pages changed since the last one (gathered into one pinned
 * staging copy and scattered on the device).  Frames are traced from the
 * mirror with yv_render_svo_noalloc (caller node ids) or by a renderer bound
 * with yv_set_scene_dynamic (type declared above).  Not thread-safe. */
yv_status yv_svo_dynamic_create(uint32_t node_capacity, uint32_t attr_capacity,
                                yv_svo_dynamic** out);
void      yv_svo_dynamic_destroy(yv_svo_dynamic* s);
/* Replaces the contents with a host scene (all its pages become dirty). */
yv_status yv_svo_dynamic_load(yv_svo_dynamic* s, const yv_svo_host* svo);
yv_status yv_svo_dynamic_alloc_node(yv_svo_dynamic* s, uint32_t* id);
yv_status yv_svo_dynamic_free_node(yv_svo_dynamic* s, uint32_t id);
yv_status yv_svo_dynamic_set_node(yv_svo_dynamic* s, uint32_t id,
                                  const yv_vox_node* n);
yv_status yv_svo_dynamic_get_node(const yv_svo_dynamic* s, uint32_t id,
                                  yv_vox_node* n);
yv_status yv_svo_dynamic_add_attr(yv_svo_dynamic* s, const yv_leaf_attr* a,
                                  uint32_t* index);
yv_status yv_svo_dynamic_set_attr(yv_svo_dynamic* s, uint32_t index,
                                  const yv_leaf_attr* a);
yv_status yv_svo_dynamic_set_root(yv_svo_dynamic* s, uint32_t root,
                                  int32_t depth);
/* Sets (a != NULL) or clears one voxel of a 2^depth grid, splitting
 * EmptyNode / FullNode regions on the way down (no collapse on clear). */
yv_status yv_svo_dynamic_set_voxel(yv_svo_dynamic* s, int32_t depth,
                                   uint32_t x, uint32_t y, uint32_t z,
                                   const yv_leaf_attr* a);
uint32_t  yv_svo_dynamic_changed_pages(const yv_svo_dynamic* s);
uint64_t  yv_svo_dynamic_transfer_bytes(const yv_svo_dynamic* s);
/* Sends the changed pages on `stream` (UpdateSVO). */
yv_status yv_svo_dynamic_sync(yv_svo_dynamic* s, void* stream);
/* The device mirror as of the last sync (pointers, node slots in use, root,
 * attributes in use) and the host pool.  yv_svo_dynamic_host_info gives the
 * host pool's current node slots in use, root and attribute count
 * (download and host arrays are sized by them). */
yv_status yv_svo_dynamic_host_info(const yv_svo_dynamic* s, uint32_t* count,
                                   uint32_t* root, uint32_t* nattrs);
yv_status yv_svo_dynamic_device(const yv_svo_dynamic* s,
                                const yv_vox_node** nodes, uint32_t* count,
                                uint32_t* root, const yv_leaf_attr** attrs,
                                uint32_t* nattrs);
const yv_vox_node*  yv_svo_dynamic_host_nodes(const yv_svo_dynamic* s);
const yv_leaf_attr* yv_svo_dynamic_host_attrs(const yv_svo_dynamic* s);
/* Copies the device mirror back into host arrays (verification). */
yv_status yv_svo_dynamic_download(const yv_svo_dynamic* s, yv_vox_node* nodes,
                                  yv_leaf_attr* attrs);

/* ------------------------------------------------------------------------ */
/* Screen-space normal approximation and point-light shading                */
/* (SVORenderer::Render with m_ssna, demo/SVORenderer.cpp:88-146; the blur  */
/* kernel of InitBlur, :55-78; the limited Gaussian depth blur and the      */
/* depth normals of demo/dumps/ztools.py:23-43, 154-233, 252-266;           */
/* LightParams as Demo.cpp:141-147 fills them; DumpTraceData, :158-186)     */
/* ------------------------------------------------------------------------ */
#define YV_SSNA_MAX_LIGHTS 4

/* Point light: attenuation = 1 / (a0 + a1 d + a2 d^2) at distance d. */
typedef struct yv_point_light {
  float pos[3];
  float diffuse[3];
  float specular[3];
  float attenuation[3];
  int32_t enabled;
} yv_point_light;

typedef struct yv_ssna_params {
  int32_t ssna;           /* 1: blur the depth, normals from the depth;
                             0: the leaves' stored normals              */
  int32_t show_normals;   /* 1: output the normal as colour n/2 + 1/2  */
  int32_t blur_passes;    /* depth blur passes (5)                      */
  float voxel_size;       /* world size of a finest voxel (1/2048)      */
  float edge_threshold;   /* depth step treated as an edge (4/2048)     */
  float edge_pad;         /* far taps replaced by d + edge_pad*thr (0.3) */
  float ambient[3];       /* (0.1, 0.1, 0.1)                            */
  float specular_exp;     /* Phong exponent (10)                        */
  yv_point_light lights[YV_SSNA_MAX_LIGHTS];
} yv_ssna_params;

/* The reference's values; lights[0] = a white light at the eye
 * (diffuse 0.7, specular 0.3, attenuation (1, 0, 0.5)), others disabled. */
yv_status yv_ssna_defaults(const yv_renderer* r, yv_ssna_params* p);

/* One frame: an unlit trace (albedo, hit distance, stored normals), the
 * view depth z = t / |u| (u the pixel's unnormalised ray, forward
 * component 1), blur_passes limited 5x5 Gaussian passes (pass i blurs the
 * pixels with z <= 5 voxel_size / (pixel_angle * 3 (i + 1))), normals from
 * the depth and Phong shading with the point lights.  device_rgba (Color32,
 * required), device_depth (blurred z, 0 for a miss) and device_normals (3
 * floats per pixel) are device pointers; the last two are optional.  Async
 * on `stream`; the trace's counters are read with yv_renderer_frame_stats. */
yv_status yv_render_ssna(yv_renderer* r, const yv_ssna_params* p,
                         void* device_rgba, void* device_depth,
                         void* device_normals, void* stream);

/* DumpTraceData into host arrays (each optional): dist = the hit's ray
 * distance (0 for a miss), color = the hit leaf's Color32 (0 for a miss),
 * normal = its unit normal (3 floats, 0 for a miss).  Synchronous. */
yv_status yv_renderer_trace_dump(yv_renderer* r, float* host_dist,
                                 uint32_t* host_color, float* host_normal);

#ifdef __cplusplus
}
#endif

#endif /* YV_C_API_H */
