/*
 * yv_oracle.h - CPU oracle for the SVO ray cast and the brick ray-march.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the CUDA path is compared
 * against (and the timed CPU baseline); the product library never links,
 * loads or calls it.
 *
 * It restates, in plain C, the reference CPU renderer of znah/yoxel-voxel:
 *   RendererBase::InitRayDir       cell/renderer_base.h:50-61
 *   PPURendererBase::RenderRect    cell/ppu_renderer.cpp:43-70
 *   PPURendererBase::RecTrace      cell/ppu_renderer.cpp:18-41
 *   FindFirstChild / GoNext        cell/spu/trace_spu.cpp:48-93
 *   AdjustDir / SetupTrace         cell/spu/trace_spu.c_:66-105,
 *                                  reaction/report/voxel.tex:309-326
 *   brick march castRay/walkBrick  reaction/trace/trace.cu:42-139
 * Pinned against the reference itself: oracle/build_ref.py compiles the
 * reference's own renderer code on the host (cell/ppu_renderer.cpp with
 * renderer_base.h and svodata.h, cell/spu/trace_spu.cpp, and
 * reaction/trace/trace.cu), with stand-ins (oracle/ref_shim/) only for the
 * headers its snapshot lacks (cpp/, Boost, the Cell SDK, CUDA).  The float
 * instantiation reproduces that renderer's camera basis, every pixel's hit
 * leaf, hit t and node-fetch count bit for bit, and the double march under
 * trace.cu's fixed transfer agrees with its castRay to 1e-5
 * (tests/test_ref_pin.py, fixtures tests/golden/ref_*.npz).  What the
 * snapshot does not define - SetupTrace / AdjustDir, the shading, the
 * configs' transfer and the ntree lattice layout - is restated, as the
 * comments below say.
 */
#ifndef YV_ORACLE_H
#define YV_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Camera basis, RendererBase::InitRayDir (cell/renderer_base.h:50-61). */
void orc_init_ray_dir_f32(const float dir[3], const float up[3], float fov_deg,
                          int width, int height, float dir0[3], float du[3],
                          float dv[3]);
void orc_init_ray_dir_f64(const double dir[3], const double up[3],
                          double fov_deg, int width, int height, double dir0[3],
                          double du[3], double dv[3]);

/*
 * SVO render of rows [y0, y1) (RenderRect).  nodes = count*10 uint32 (the
 * 40-byte VoxNode), attrs = nattrs*8 bytes.  Outputs are full-frame arrays
 * (width*height), any may be NULL.  light = direction toward the light.
 * Returns 0, or 3 if the pool is malformed (index out of range / too deep).
 */
int orc_svo_render_f32(const uint32_t* nodes, uint32_t count, uint32_t root,
                       const uint8_t* attrs, uint32_t nattrs,
                       const float pos[3], const float dir0[3],
                       const float du[3], const float dv[3], int width,
                       int height, const float light[3], float ambient,
                       float diffuse, int shadows, int y0, int y1,
                       uint32_t* rgba, uint32_t* hit, float* hit_t,
                       uint32_t* fetches, uint32_t* shadow_fetches,
                       uint8_t* shadowed);

/* The same with the level-of-detail cut-off of SVORenderer (detailCoef):
 * a subtree ahead of the ray whose cube side 2^-(level+1) is below
 * max(t_enter, 0) * lod_coef ends the ray there; it is shaded with the
 * attribute its node's `data` word indexes, and reported as the hit
 * (parent << 3 | child slot).  lod_coef = 0: orc_svo_render_f32. */
int orc_svo_render_lod_f32(const uint32_t* nodes, uint32_t count, uint32_t root,
                           const uint8_t* attrs, uint32_t nattrs,
                           const float pos[3], const float dir0[3],
                           const float du[3], const float dv[3], int width,
                           int height, const float light[3], float ambient,
                           float diffuse, int shadows, float lod_coef, int y0,
                           int y1, uint32_t* rgba, uint32_t* hit, float* hit_t,
                           uint32_t* fetches, uint32_t* shadow_fetches,
                           uint8_t* shadowed);

/* Same over all rows on nthreads POSIX threads in row bands
 * (TreadedRenderer, cell/ppu_renderer.cpp:121-144). */
int orc_svo_render_mt(int nthreads, const uint32_t* nodes, uint32_t count,
                      uint32_t root, const uint8_t* attrs, uint32_t nattrs,
                      const float pos[3], const float dir0[3],
                      const float du[3], const float dv[3], int width,
                      int height, const float light[3], float ambient,
                      float diffuse, int shadows, uint32_t* rgba,
                      uint32_t* hit, float* hit_t, uint32_t* fetches,
                      uint32_t* shadow_fetches, uint8_t* shadowed);

/* The same with the level-of-detail cut-off (see orc_svo_render_lod_f32). */
int orc_svo_render_mt_lod(int nthreads, const uint32_t* nodes, uint32_t count,
                          uint32_t root, const uint8_t* attrs, uint32_t nattrs,
                          const float pos[3], const float dir0[3],
                          const float du[3], const float dv[3], int width,
                          int height, const float light[3], float ambient,
                          float diffuse, int shadows, float lod_coef, uint32_t* rgba,
                          uint32_t* hit, float* hit_t, uint32_t* fetches,
                          uint32_t* shadow_fetches, uint8_t* shadowed);

/* FP64 evaluation of the primary hits (camera basis recomputed in double);
 * used to count rays whose hit voxel is decided by a float rounding tie. */
int orc_svo_hits_f64(const uint32_t* nodes, uint32_t count, uint32_t root,
                     const double pos[3], const double dir[3],
                     const double up[3], double fov_deg, int width, int height,
                     int y0, int y1, uint32_t* hit, double* hit_t);

/* Single-ray entry points used by the known-answer tests. */
int orc_svo_trace_ray_f32(const uint32_t* nodes, uint32_t count, uint32_t root,
                          const float pos[3], const float dir[3],
                          int cull_behind, uint32_t* hit, float* hit_t,
                          uint32_t* fetches, int* level);
void orc_find_first_child_f32(float t1[3], float t2[3], int* child);
int orc_go_next_f32(int* child, float t1[3], float t2[3]);
int orc_setup_trace_f32(const float pos[3], const float dir[3], float t1[3],
                        float t2[3], uint32_t* dir_flags);

/*
 * Brick volume ray-march (ntree layout).
 *   grids   : ngrids*64 uint32 child refs of N=4 grid nodes; ref encoding
 *             0x80000000 = empty, 0x40000000|b = brick b, else grid index.
 *   density : nbricks*729 values (9^3 lattice incl. the +1 apron), float
 *             (f64 oracle reads float input, computes in double)
 *   albedo  : nbricks*729*3 floats in [0,1]
 *   levels  : grid levels (scene size = 4^levels * 8 lattice cells)
 * Output rgba: 4 doubles per pixel.  samples / bricks: per-pixel counters
 * (optional).  Rows [y0, y1).
 */
int orc_brick_render_f64(const uint32_t* grids, uint32_t ngrids,
                         const float* density, const float* albedo,
                         uint32_t nbricks, int levels, const double pos[3],
                         const double dir0[3], const double du[3],
                         const double dv[3], int width, int height,
                         double alpha_scale, double step_vox, int y0, int y1,
                         double* rgba, uint32_t* samples, uint32_t* bricks);
/* FP64 march of the FP32-generated primary rays (float camera basis).
 * ties (optional): 1 where the ray's sample set or its early exit is decided
 * by a rounding tie - a sample within 1e-6 (relative) of a cell boundary,
 * two exit planes of a cell within 1e-6 of each other, the entry cell's
 * coordinate within 1e-6 of an integer, or the opacity within 1e-5 of the
 * 0.99 early-exit threshold after a sample - so that an FP32 march may take
 * a different sample set. */
int orc_brick_render_f64_f32ray(const uint32_t* grids, uint32_t ngrids,
                                const float* density, const float* albedo,
                                uint32_t nbricks, int levels, const float pos[3],
                                const float dir0[3], const float du[3],
                                const float dv[3], int width, int height,
                                double alpha_scale, double step_vox, int y0,
                                int y1, double* rgba, uint32_t* samples,
                                uint32_t* bricks, uint8_t* ties);
int orc_brick_render_f32(const uint32_t* grids, uint32_t ngrids,
                         const float* density, const float* albedo,
                         uint32_t nbricks, int levels, const float pos[3],
                         const float dir0[3], const float du[3],
                         const float dv[3], int width, int height,
                         float alpha_scale, float step_vox, int y0, int y1,
                         float* rgba, uint32_t* samples, uint32_t* bricks);
int orc_brick_render_mt_f32(int nthreads, const uint32_t* grids,
                            uint32_t ngrids, const float* density,
                            const float* albedo, uint32_t nbricks, int levels,
                            const float pos[3], const float dir0[3],
                            const float du[3], const float dv[3], int width,
                            int height, float alpha_scale, float step_vox,
                            float* rgba, uint32_t* samples, uint32_t* bricks);

/* FP64 adjoint of the brick march for an L2-style loss: given dL/drgba per
 * pixel (4 doubles), accumulates dL/ddensity (nbricks*729) and dL/dalbedo
 * (nbricks*729*3) in pool layout (apron slots receive their own share). */
int orc_brick_backward_f64(const uint32_t* grids, uint32_t ngrids,
                           const float* density, const float* albedo,
                           uint32_t nbricks, int levels, const double pos[3],
                           const double dir0[3], const double du[3],
                           const double dv[3], int width, int height,
                           double alpha_scale, double step_vox,
                           const double* grad_rgba, double* grad_density,
                           double* grad_albedo);

/* Row-parallel forms of the checks above, for full-size frames: interleaved
 * rows on nthreads POSIX threads, each with its own context.  The adjoint
 * keeps per-thread gradient accumulators and adds them into grad_density /
 * grad_albedo in thread order (deterministic for a given nthreads). */
int orc_svo_hits_f64_mt(int nthreads, const uint32_t* nodes, uint32_t count,
                        uint32_t root, const double pos[3], const double dir[3],
                        const double up[3], double fov_deg, int width,
                        int height, uint32_t* hit, double* hit_t);
int orc_brick_render_f64_f32ray_mt(int nthreads, const uint32_t* grids, uint32_t ngrids,
                                   const float* density, const float* albedo,
                                   uint32_t nbricks, int levels, const float pos[3],
                                   const float dir0[3], const float du[3],
                                   const float dv[3], int width, int height,
                                   double alpha_scale, double step_vox, double* rgba,
                                   uint32_t* samples, uint32_t* bricks, uint8_t* ties);
int orc_brick_backward_f64_mt(int nthreads, const uint32_t* grids, uint32_t ngrids,
                              const float* density, const float* albedo,
                              uint32_t nbricks, int levels, const double pos[3],
                              const double dir0[3], const double du[3],
                              const double dv[3], int width, int height,
                              double alpha_scale, double step_vox,
                              const double* grad_rgba, double* grad_density,
                              double* grad_albedo);
/* The same checks over the FP32 primary rays (float camera basis, as the
 * CUDA path generates them) promoted to double: the FP64 traversal of those
 * rays (its hits differ from the float traversal only where a rounding tie
 * inside the traversal decides the hit) and the FP64 adjoint of the march
 * along them. */
int orc_svo_hits_f64_f32ray(const uint32_t* nodes, uint32_t count, uint32_t root,
                            const float pos[3], const float dir0[3], const float du[3],
                            const float dv[3], int width, int height, int y0, int y1,
                            uint32_t* hit, double* hit_t);
int orc_svo_hits_f64_f32ray_mt(int nthreads, const uint32_t* nodes, uint32_t count,
                               uint32_t root, const float pos[3], const float dir0[3],
                               const float du[3], const float dv[3], int width, int height,
                               uint32_t* hit, double* hit_t);
int orc_brick_backward_f64_f32ray_mt(int nthreads, const uint32_t* grids, uint32_t ngrids,
                                     const float* density, const float* albedo,
                                     uint32_t nbricks, int levels, const float pos[3],
                                     const float dir0[3], const float du[3],
                                     const float dv[3], int width, int height,
                                     double alpha_scale, double step_vox,
                                     const double* grad_rgba, double* grad_density,
                                     double* grad_albedo);
/* FP64 march (FP64 rays, as orc_brick_render_f64) of the pixel window
 * [x0, x1) x [y0, y1) only; rgba (4 doubles per pixel) and samples (optional,
 * samples taken per ray) are full-frame arrays, pixels outside the window
 * are left untouched.  Used for central
 * differences, where a lattice point reaches only the rays of a few pixels. */
int orc_brick_render_f64_rect(const uint32_t* grids, uint32_t ngrids,
                              const float* density, const float* albedo,
                              uint32_t nbricks, int levels, const double pos[3],
                              const double dir0[3], const double du[3],
                              const double dv[3], int width, int height,
                              double alpha_scale, double step_vox, int x0, int x1,
                              int y0, int y1, double* rgba, uint32_t* samples);

/* The same window over the FP32 primary rays promoted to double. */
int orc_brick_render_f64_f32ray_rect(const uint32_t* grids, uint32_t ngrids,
                                     const float* density, const float* albedo,
                                     uint32_t nbricks, int levels, const float pos[3],
                                     const float dir0[3], const float du[3],
                                     const float dv[3], int width, int height,
                                     double alpha_scale, double step_vox, int x0, int x1,
                                     int y0, int y1, double* rgba, uint32_t* samples);

/* FP64 march of n rays with the given origins and directions (3 doubles
 * each; directions need not be unit: t is their parameter).  transfer 0:
 * the configs' (alpha = saturate(alpha_scale * density), albedo colour);
 * 1: the fixed transfer of reaction/trace/trace.cu:52-56 (s = saturate(2 v
 * - 0.9), alpha = s / 2, colour s), used to pin the march against the
 * reference's own castRay.  rgba: 4 doubles per ray. */
int orc_brick_march_rays_f64(const uint32_t* grids, uint32_t ngrids, const float* density,
                             const float* albedo, uint32_t nbricks, int levels,
                             double alpha_scale, double step_vox, int transfer,
                             const double* origins, const double* dirs, int n, double* rgba,
                             uint32_t* samples);

/* SVO build from a dense density grid (yv_oracle_build.c): 2^depth grid,
 * solid = density > iso, canonical breadth-first pool (nodes: 10 uint32 per
 * VoxNode, attrs: 8 bytes per leaf).  Returns 0; 1 if node_cap / attr_cap
 * are too small (n_nodes / n_attrs then hold the sizes needed); 2 bad
 * arguments; 3 out of memory.  An empty (full) grid gives root EmptyNode
 * (FullNode) and no nodes. */
int orc_svo_build_dense(const float* density, const uint8_t* rgb, int depth, float iso,
                        uint32_t* nodes, uint32_t node_cap, uint8_t* attrs,
                        uint32_t attr_cap, uint32_t* n_nodes, uint32_t* n_attrs,
                        uint32_t* root);

#ifdef __cplusplus
}
#endif

#endif /* YV_ORACLE_H */
