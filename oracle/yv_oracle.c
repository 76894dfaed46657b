/*
 * yv_oracle.c - CPU oracle (test infrastructure only; see yv_oracle.h).
 *
 * Instantiates the traversal / march restatement for float (the reference's
 * own FP32 path, bit-comparable with the CUDA kernels) and for double (the
 * FP64 oracle used for tie counting, composited radiance and gradients).
 */
#include "yv_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ---- float instantiation ---- */
#define REAL float
#define SFX f32
#define SQRT sqrtf
#define TAN tanf
#define FLOOR floorf
#define CEIL ceilf
#define COPYSIGN copysignf
#define LDEXP ldexpf
#include "yv_oracle_impl.h"
#undef REAL
#undef SFX
#undef SQRT
#undef TAN
#undef FLOOR
#undef CEIL
#undef COPYSIGN
#undef LDEXP
#undef V3

/* ---- double instantiation ---- */
#define REAL double
#define SFX f64
#define SQRT sqrt
#define TAN tan
#define FLOOR floor
#define CEIL ceil
#define COPYSIGN copysign
#define LDEXP ldexp
#include "yv_oracle_impl.h"

/* ------------------------------------------------------------------------ */
/* SVO shading and rendering (float path)                                   */
/* ------------------------------------------------------------------------ */

/* Lambert shading of a leaf (the shading model of
 * reaction/report/voxel.tex:97-99 reduced to ambient + one directional
 * diffuse term): I = ambient + diffuse*max(0, n.L), or ambient when the
 * shadow ray is blocked; Color32 with alpha 255. */
static uint32_t shade_f32(const uint8_t* attr, const float* light,
                          float ambient, float diffuse, int shadowed) {
  float nx = (float)(int8_t)attr[4];
  float ny = (float)(int8_t)attr[5];
  float nz = (float)(int8_t)attr[6];
  float len2 = (nx * nx + ny * ny) + nz * nz;
  float ndl = 0.0f;
  if (len2 > 0.0f) {
    float len = sqrtf(len2);
    float ux = nx / len, uy = ny / len, uz = nz / len;
    ndl = (ux * light[0] + uy * light[1]) + uz * light[2];
  }
  float dif = ndl > 0.0f ? ndl : 0.0f;
  float inten = shadowed ? ambient : ambient + diffuse * dif;
  uint32_t out = 0xFF000000u;
  for (int c = 0; c < 3; ++c) {
    float v = (float)attr[c] * inten + 0.5f;
    uint32_t u = v >= 255.0f ? 255u : (uint32_t)v;
    out |= u << (8 * c);
  }
  return out;
}

/* Shadow-ray origin: the hit point p = pos + dir*t moved half a leaf out of
 * the entry face (face axis = first argmax of the leaf box's t1). */
static void shadow_origin_f32(const float* pos, const float* dir,
                              const hit_rec_f32* h, uint32_t dir_flags,
                              float* o) {
  for (int i = 0; i < 3; ++i) o[i] = pos[i] + dir[i] * h->t;
  int e = 0;
  if (h->t1[1] > h->t1[e]) e = 1;
  if (h->t1[2] > h->t1[e]) e = 2;
  float half = ldexpf(0.5f, -(h->level + 1));
  float off = ((dir_flags >> e) & 1u) ? half : -half;
  o[e] = o[e] + off;
}

int orc_svo_render_f32(const uint32_t* nodes, uint32_t count, uint32_t root,
                       const uint8_t* attrs, uint32_t nattrs,
                       const float pos[3], const float dir0[3],
                       const float du[3], const float dv[3], int width,
                       int height, const float light[3], float ambient,
                       float diffuse, int shadows, int y0, int y1,
                       uint32_t* rgba, uint32_t* hit, float* hit_t,
                       uint32_t* fetches, uint32_t* shadow_fetches,
                       uint8_t* shadowed) {
  return orc_svo_render_lod_f32(nodes, count, root, attrs, nattrs, pos, dir0, du, dv, width,
                                height, light, ambient, diffuse, shadows, 0.0f, y0, y1, rgba,
                                hit, hit_t, fetches, shadow_fetches, shadowed);
}

int orc_svo_render_lod_f32(const uint32_t* nodes, uint32_t count, uint32_t root,
                           const uint8_t* attrs, uint32_t nattrs,
                           const float pos[3], const float dir0[3],
                           const float du[3], const float dv[3], int width,
                           int height, const float light[3], float ambient,
                           float diffuse, int shadows, float lod_coef, int y0,
                           int y1, uint32_t* rgba, uint32_t* hit, float* hit_t,
                           uint32_t* fetches, uint32_t* shadow_fetches,
                           uint8_t* shadowed) {
  if (y0 < 0) y0 = 0;
  if (y1 > height) y1 = height;
  float ldir[3] = {light[0], light[1], light[2]};
  adjust_dir_f32(ldir);
  for (int y = y0; y < y1; ++y) {
    for (int x = 0; x < width; ++x) {
      size_t off = (size_t)y * (size_t)width + (size_t)x;
      if (rgba) rgba[off] = 0;
      if (hit) hit[off] = 0xFFFFFFFFu;
      if (hit_t) hit_t[off] = 0.0f;
      if (shadow_fetches) shadow_fetches[off] = 0;
      if (shadowed) shadowed[off] = 0;
      float d[3];
      pixel_dir_f32(dir0, du, dv, x, y, d);
      adjust_dir_f32(d);
      trace_ctx_f32 c = {nodes, count, 0, 0, 0, lod_coef};
      hit_rec_f32 h;
      uint32_t dir_flags = 0;
      int ok = trace_one_f32(&c, root, pos, d, &h, &dir_flags);
      if (c.err) return c.err;
      if (fetches) fetches[off] = c.fetches;
      if (!ok) continue;
      uint32_t vd = nodes[(size_t)h.node * 10u + 2u + (uint32_t)h.child];
      /* a level-of-detail hit shades with the subtree's data attribute */
      if (h.lod) vd = nodes[(size_t)vd * 10u + 1u];
      if (vd >= nattrs) return 3;
      if (hit) hit[off] = (h.node << 3) | (uint32_t)h.child;
      if (hit_t) hit_t[off] = h.t;
      int sh = 0;
      if (shadows) {
        float so[3];
        shadow_origin_f32(pos, d, &h, dir_flags, so);
        trace_ctx_f32 cs = {nodes, count, 1, 0, 0, lod_coef};
        hit_rec_f32 hs;
        sh = trace_one_f32(&cs, root, so, ldir, &hs, 0);
        if (cs.err) return cs.err;
        if (shadow_fetches) shadow_fetches[off] = cs.fetches;
        if (shadowed) shadowed[off] = (uint8_t)sh;
      }
      if (rgba)
        rgba[off] = shade_f32(attrs + (size_t)vd * 8u, light, ambient,
                              diffuse, sh);
    }
  }
  return 0;
}

/* ---- row-band threading (TreadedRenderer) ---- */
typedef struct {
  int kind;
  int y0, y1;
  int status;
  /* svo */
  const uint32_t* nodes;
  uint32_t count, root;
  const uint8_t* attrs;
  uint32_t nattrs;
  const float *pos, *dir0, *du, *dv, *light;
  int width, height;
  float ambient, diffuse;
  int shadows;
  float lod_coef;
  uint32_t *rgba, *hit, *fetches, *shadow_fetches;
  float* hit_t;
  uint8_t* shadowed;
  /* bricks */
  const uint32_t* grids;
  uint32_t ngrids;
  const float *density, *albedo;
  uint32_t nbricks;
  int levels;
  float alpha_scale, step_vox;
  float* frgba;
  uint32_t *samples, *bricks;
} band_job;

static void* band_main(void* arg) {
  band_job* j = (band_job*)arg;
  /* rows y0, y0+stride, ... (interleaved rows keep threads balanced) */
  for (int y = j->y0; y < j->height && !j->status; y += j->y1) {
    if (j->kind == 0) {
      j->status = orc_svo_render_lod_f32(
          j->nodes, j->count, j->root, j->attrs, j->nattrs, j->pos, j->dir0,
          j->du, j->dv, j->width, j->height, j->light, j->ambient, j->diffuse,
          j->shadows, j->lod_coef, y, y + 1, j->rgba, j->hit, j->hit_t, j->fetches,
          j->shadow_fetches, j->shadowed);
    } else {
      j->status = orc_brick_render_f32(
          j->grids, j->ngrids, j->density, j->albedo, j->nbricks, j->levels,
          j->pos, j->dir0, j->du, j->dv, j->width, j->height, j->alpha_scale,
          j->step_vox, y, y + 1, j->frgba, j->samples, j->bricks);
    }
  }
  return NULL;
}

static int run_bands(band_job* proto, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  band_job* jobs = (band_job*)calloc((size_t)nthreads, sizeof(band_job));
  pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
  char* created = (char*)calloc((size_t)nthreads, 1);
  if (!jobs || !th || !created) {
    free(jobs);
    free(th);
    free(created);
    return 7;
  }
  /* thread i renders rows i, i+n, i+2n, ... (y0 = first row, y1 = stride) */
  int st = 0;
  for (int i = 0; i < nthreads; ++i) {
    jobs[i] = *proto;
    jobs[i].y0 = i;
    jobs[i].y1 = nthreads;
    jobs[i].status = 0;
    created[i] = pthread_create(&th[i], NULL, band_main, &jobs[i]) == 0;
  }
  for (int i = 0; i < nthreads; ++i) {
    if (created[i])
      pthread_join(th[i], NULL);
    else
      band_main(&jobs[i]);
    if (jobs[i].status && !st) st = jobs[i].status;
  }
  free(jobs);
  free(th);
  free(created);
  return st;
}

int orc_svo_render_mt(int nthreads, const uint32_t* nodes, uint32_t count,
                      uint32_t root, const uint8_t* attrs, uint32_t nattrs,
                      const float pos[3], const float dir0[3],
                      const float du[3], const float dv[3], int width,
                      int height, const float light[3], float ambient,
                      float diffuse, int shadows, uint32_t* rgba,
                      uint32_t* hit, float* hit_t, uint32_t* fetches,
                      uint32_t* shadow_fetches, uint8_t* shadowed) {
  return orc_svo_render_mt_lod(nthreads, nodes, count, root, attrs, nattrs, pos, dir0, du, dv,
                               width, height, light, ambient, diffuse, shadows, 0.0f, rgba,
                               hit, hit_t, fetches, shadow_fetches, shadowed);
}

int orc_svo_render_mt_lod(int nthreads, const uint32_t* nodes, uint32_t count,
                          uint32_t root, const uint8_t* attrs, uint32_t nattrs,
                          const float pos[3], const float dir0[3],
                          const float du[3], const float dv[3], int width,
                          int height, const float light[3], float ambient,
                          float diffuse, int shadows, float lod_coef, uint32_t* rgba,
                          uint32_t* hit, float* hit_t, uint32_t* fetches,
                          uint32_t* shadow_fetches, uint8_t* shadowed) {
  band_job p;
  memset(&p, 0, sizeof(p));
  p.kind = 0;
  p.nodes = nodes;
  p.count = count;
  p.root = root;
  p.attrs = attrs;
  p.nattrs = nattrs;
  p.pos = pos;
  p.dir0 = dir0;
  p.du = du;
  p.dv = dv;
  p.width = width;
  p.height = height;
  p.light = light;
  p.ambient = ambient;
  p.diffuse = diffuse;
  p.shadows = shadows;
  p.rgba = rgba;
  p.hit = hit;
  p.hit_t = hit_t;
  p.fetches = fetches;
  p.shadow_fetches = shadow_fetches;
  p.shadowed = shadowed;
  p.lod_coef = lod_coef;
  return run_bands(&p, nthreads);
}

int orc_brick_render_mt_f32(int nthreads, const uint32_t* grids,
                            uint32_t ngrids, const float* density,
                            const float* albedo, uint32_t nbricks, int levels,
                            const float pos[3], const float dir0[3],
                            const float du[3], const float dv[3], int width,
                            int height, float alpha_scale, float step_vox,
                            float* rgba, uint32_t* samples, uint32_t* bricks) {
  band_job p;
  memset(&p, 0, sizeof(p));
  p.kind = 1;
  p.grids = grids;
  p.ngrids = ngrids;
  p.density = density;
  p.albedo = albedo;
  p.nbricks = nbricks;
  p.levels = levels;
  p.pos = pos;
  p.dir0 = dir0;
  p.du = du;
  p.dv = dv;
  p.width = width;
  p.height = height;
  p.alpha_scale = alpha_scale;
  p.step_vox = step_vox;
  p.frgba = rgba;
  p.samples = samples;
  p.bricks = bricks;
  return run_bands(&p, nthreads);
}

/* ---- FP64 hits ---- */
int orc_svo_hits_f64(const uint32_t* nodes, uint32_t count, uint32_t root,
                     const double pos[3], const double dir[3],
                     const double up[3], double fov_deg, int width, int height,
                     int y0, int y1, uint32_t* hit, double* hit_t) {
  double dir0[3], du[3], dv[3];
  orc_init_ray_dir_f64(dir, up, fov_deg, width, height, dir0, du, dv);
  if (y0 < 0) y0 = 0;
  if (y1 > height) y1 = height;
  for (int y = y0; y < y1; ++y)
    for (int x = 0; x < width; ++x) {
      size_t off = (size_t)y * (size_t)width + (size_t)x;
      double d[3];
      pixel_dir_f64(dir0, du, dv, x, y, d);
      adjust_dir_f64(d);
      trace_ctx_f64 c = {nodes, count, 0, 0, 0};
      hit_rec_f64 h;
      int ok = trace_one_f64(&c, root, pos, d, &h, 0);
      if (c.err) return c.err;
      if (hit) hit[off] = ok ? ((h.node << 3) | (uint32_t)h.child) : 0xFFFFFFFFu;
      if (hit_t) hit_t[off] = ok ? h.t : 0.0;
    }
  return 0;
}

/* ---- single-ray / helper entry points for known-answer tests ---- */
int orc_svo_trace_ray_f32(const uint32_t* nodes, uint32_t count, uint32_t root,
                          const float pos[3], const float dir[3],
                          int cull_behind, uint32_t* hit, float* hit_t,
                          uint32_t* fetches, int* level) {
  float d[3] = {dir[0], dir[1], dir[2]};
  adjust_dir_f32(d);
  trace_ctx_f32 c = {nodes, count, cull_behind, 0, 0};
  hit_rec_f32 h;
  int ok = trace_one_f32(&c, root, pos, d, &h, 0);
  if (c.err) return -c.err;
  if (hit) *hit = ok ? ((h.node << 3) | (uint32_t)h.child) : 0xFFFFFFFFu;
  if (hit_t) *hit_t = ok ? h.t : 0.0f;
  if (fetches) *fetches = c.fetches;
  if (level) *level = ok ? h.level : -1;
  return ok;
}

void orc_find_first_child_f32(float t1[3], float t2[3], int* child) {
  *child = ffc_f32(t1, t2);
}

int orc_go_next_f32(int* child, float t1[3], float t2[3]) {
  return go_next_f32(child, t1, t2);
}

int orc_setup_trace_f32(const float pos[3], const float dir[3], float t1[3],
                        float t2[3], uint32_t* dir_flags) {
  float d[3] = {dir[0], dir[1], dir[2]};
  adjust_dir_f32(d);
  return setup_trace_f32(pos, d, t1, t2, dir_flags);
}

/* FP64 march of the FP32 primary rays: the ray directions are generated
 * exactly as the float path does (InitRayDir, RenderRect, AdjustDir in
 * float), then promoted; the march itself runs in double.  This isolates
 * the accuracy of the march arithmetic from ray generation. */
int orc_brick_render_f64_f32ray(const uint32_t* grids, uint32_t ngrids,
                                const float* density, const float* albedo,
                                uint32_t nbricks, int levels, const float pos[3],
                                const float dir0[3], const float du[3],
                                const float dv[3], int width, int height,
                                double alpha_scale, double step_vox, int y0,
                                int y1, double* rgba, uint32_t* samples,
                                uint32_t* bricks, uint8_t* ties) {
  brick_ctx_f64 c;
  if (brick_ctx_init_f64(&c, grids, ngrids, density, albedo, nbricks, levels,
                         alpha_scale, step_vox))
    return 1;
  if (y0 < 0) y0 = 0;
  if (y1 > height) y1 = height;
  double o[3] = {pos[0], pos[1], pos[2]};
  for (int y = y0; y < y1; ++y)
    for (int x = 0; x < width; ++x) {
      size_t off = (size_t)y * (size_t)width + (size_t)x;
      float df[3];
      pixel_dir_f32(dir0, du, dv, x, y, df);
      adjust_dir_f32(df);
      double d[3] = {df[0], df[1], df[2]};
      double out[4];
      uint32_t ns = 0, nbk = 0;
      int st = brick_march_f64(&c, o, d, out, &ns, &nbk, 0, 0);
      if (st) return st;
      if (rgba)
        for (int i = 0; i < 4; ++i) rgba[off * 4 + (size_t)i] = out[i];
      if (samples) samples[off] = ns;
      if (bricks) bricks[off] = nbk;
      if (ties) ties[off] = (uint8_t)c.tie;
    }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* FP64 adjoint of the brick march                                          */
/* ------------------------------------------------------------------------ */
typedef struct {
  const double* g;      /* dL/d(r,g,b,a) of this ray */
  const double* out;    /* forward (C, A) of this ray */
  double alpha_scale;
  double* grad_density;
  double* grad_albedo;
} bwd_user;

/* For output channel k with per-sample colour c (c_A = 1):
 *   d out_k / d alpha_j = T_j c_jk - (out_k - out_k,after j) / (1 - alpha_j)
 *   d out_k / d c_jk    = T_j alpha_j
 * with T_j = 1 - A before sample j. */
static void bwd_sample(void* user, const uint32_t* idx, const double* w,
                       double sigma, const double* col, double alpha,
                       double acc_a, const double* acc_c) {
  bwd_user* u = (bwd_user*)user;
  double T = 1.0 - acc_a;
  double wgt = T * alpha;
  double one_m = 1.0 - alpha;
  double dalpha = 0.0;
  for (int k = 0; k < 4; ++k) {
    double ck = k < 3 ? col[k] : 1.0;
    double after = k < 3 ? acc_c[k] + wgt * ck : acc_a + wgt;
    double term = T * ck;
    if (one_m > 0.0) term -= (u->out[k] - after) / one_m;
    dalpha += u->g[k] * term;
  }
  double s = sigma * u->alpha_scale;
  /* saturate'(s): 1 on [0, 1) (right derivative at 0, so empty lattice
   * points still receive gradient), 0 elsewhere */
  double dsigma = (s >= 0.0 && s < 1.0) ? dalpha * u->alpha_scale : 0.0;
  for (int j = 0; j < 8; ++j) {
    u->grad_density[idx[j]] += w[j] * dsigma;
    for (int k = 0; k < 3; ++k)
      u->grad_albedo[(size_t)idx[j] * 3u + (uint32_t)k] += w[j] * u->g[k] * wgt;
  }
}

int orc_brick_backward_f64(const uint32_t* grids, uint32_t ngrids,
                           const float* density, const float* albedo,
                           uint32_t nbricks, int levels, const double pos[3],
                           const double dir0[3], const double du[3],
                           const double dv[3], int width, int height,
                           double alpha_scale, double step_vox,
                           const double* grad_rgba, double* grad_density,
                           double* grad_albedo) {
  brick_ctx_f64 c;
  if (brick_ctx_init_f64(&c, grids, ngrids, density, albedo, nbricks, levels,
                         alpha_scale, step_vox))
    return 1;
  for (int y = 0; y < height; ++y)
    for (int x = 0; x < width; ++x) {
      size_t off = (size_t)y * (size_t)width + (size_t)x;
      double d[3];
      pixel_dir_f64(dir0, du, dv, x, y, d);
      adjust_dir_f64(d);
      double out[4];
      int st = brick_march_f64(&c, pos, d, out, 0, 0, 0, 0);
      if (st) return st;
      bwd_user u = {grad_rgba + off * 4, out, alpha_scale, grad_density,
                    grad_albedo};
      double out2[4];
      st = brick_march_f64(&c, pos, d, out2, 0, 0, bwd_sample, &u);
      if (st) return st;
    }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Row-parallel drivers for full-size checks (POSIX threads, interleaved    */
/* rows; every thread owns its own context and, for the adjoint, its own    */
/* gradient accumulators, summed in thread order at the end, so the result  */
/* depends only on nthreads)                                                */
/* ------------------------------------------------------------------------ */
typedef int (*row_fn)(void* ctx, int y, int tid);
typedef struct {
  row_fn fn;
  void* ctx;
  int tid, nthreads, height, status;
} row_job;

static void* row_main(void* arg) {
  row_job* j = (row_job*)arg;
  for (int y = j->tid; y < j->height && !j->status; y += j->nthreads)
    j->status = j->fn(j->ctx, y, j->tid);
  return NULL;
}

static int run_rows(int nthreads, int height, row_fn fn, void* ctx) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  row_job* jobs = (row_job*)calloc((size_t)nthreads, sizeof(row_job));
  pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
  char* created = (char*)calloc((size_t)nthreads, 1);
  if (!jobs || !th || !created) {
    free(jobs);
    free(th);
    free(created);
    return 7;
  }
  int st = 0;
  for (int i = 0; i < nthreads; ++i) {
    jobs[i].fn = fn;
    jobs[i].ctx = ctx;
    jobs[i].tid = i;
    jobs[i].nthreads = nthreads;
    jobs[i].height = height;
    created[i] = pthread_create(&th[i], NULL, row_main, &jobs[i]) == 0;
  }
  for (int i = 0; i < nthreads; ++i) {
    if (created[i])
      pthread_join(th[i], NULL);
    else
      row_main(&jobs[i]);
    if (jobs[i].status && !st) st = jobs[i].status;
  }
  free(jobs);
  free(th);
  free(created);
  return st;
}

/* ---- FP64 traversal of the FP32 primary rays: directions generated as
 * the float path generates them (InitRayDir, RenderRect, AdjustDir in
 * float), promoted, then traced in double; rays whose hit differs from the
 * float traversal are the rays a rounding tie inside the traversal decides */
int orc_svo_hits_f64_f32ray(const uint32_t* nodes, uint32_t count, uint32_t root,
                            const float pos[3], const float dir0[3], const float du[3],
                            const float dv[3], int width, int height, int y0, int y1,
                            uint32_t* hit, double* hit_t) {
  if (y0 < 0) y0 = 0;
  if (y1 > height) y1 = height;
  const double o[3] = {pos[0], pos[1], pos[2]};
  for (int y = y0; y < y1; ++y)
    for (int x = 0; x < width; ++x) {
      size_t off = (size_t)y * (size_t)width + (size_t)x;
      float df[3];
      pixel_dir_f32(dir0, du, dv, x, y, df);
      adjust_dir_f32(df);
      double d[3] = {df[0], df[1], df[2]};
      trace_ctx_f64 c = {nodes, count, 0, 0, 0};
      hit_rec_f64 h;
      int ok = trace_one_f64(&c, root, o, d, &h, 0);
      if (c.err) return c.err;
      if (hit) hit[off] = ok ? ((h.node << 3) | (uint32_t)h.child) : 0xFFFFFFFFu;
      if (hit_t) hit_t[off] = ok ? h.t : 0.0;
    }
  return 0;
}

typedef struct {
  const uint32_t* nodes;
  uint32_t count, root;
  const float *pos, *dir0, *du, *dv;
  int width, height;
  uint32_t* hit;
  double* hit_t;
} hits32_job;

static int hits32_row(void* ctx, int y, int tid) {
  (void)tid;
  hits32_job* j = (hits32_job*)ctx;
  return orc_svo_hits_f64_f32ray(j->nodes, j->count, j->root, j->pos, j->dir0, j->du, j->dv,
                                 j->width, j->height, y, y + 1, j->hit, j->hit_t);
}

/* ---- FP64 primary hits on threads ---- */
typedef struct {
  const uint32_t* nodes;
  uint32_t count, root;
  const double *pos, *dir, *up;
  double fov;
  int width, height;
  uint32_t* hit;
  double* hit_t;
} hits_job;

static int hits_row(void* ctx, int y, int tid) {
  (void)tid;
  hits_job* j = (hits_job*)ctx;
  return orc_svo_hits_f64(j->nodes, j->count, j->root, j->pos, j->dir, j->up, j->fov,
                          j->width, j->height, y, y + 1, j->hit, j->hit_t);
}

int orc_svo_hits_f64_f32ray_mt(int nthreads, const uint32_t* nodes, uint32_t count,
                               uint32_t root, const float pos[3], const float dir0[3],
                               const float du[3], const float dv[3], int width, int height,
                               uint32_t* hit, double* hit_t) {
  hits32_job j = {nodes, count, root, pos, dir0, du, dv, width, height, hit, hit_t};
  return run_rows(nthreads, height, hits32_row, &j);
}

int orc_svo_hits_f64_mt(int nthreads, const uint32_t* nodes, uint32_t count,
                        uint32_t root, const double pos[3], const double dir[3],
                        const double up[3], double fov_deg, int width,
                        int height, uint32_t* hit, double* hit_t) {
  hits_job j = {nodes, count, root, pos, dir, up, fov_deg, width, height, hit, hit_t};
  return run_rows(nthreads, height, hits_row, &j);
}

/* ---- FP64 march of the FP32 primary rays on threads ---- */
typedef struct {
  const uint32_t* grids;
  uint32_t ngrids;
  const float *density, *albedo;
  uint32_t nbricks;
  int levels;
  const float *pos, *dir0, *du, *dv;
  int width, height;
  double alpha_scale, step_vox;
  double* rgba;
  uint32_t *samples, *bricks;
  uint8_t* ties;
} march32_job;

static int march32_row(void* ctx, int y, int tid) {
  (void)tid;
  march32_job* j = (march32_job*)ctx;
  return orc_brick_render_f64_f32ray(j->grids, j->ngrids, j->density, j->albedo, j->nbricks,
                                     j->levels, j->pos, j->dir0, j->du, j->dv, j->width,
                                     j->height, j->alpha_scale, j->step_vox, y, y + 1,
                                     j->rgba, j->samples, j->bricks, j->ties);
}

int orc_brick_render_f64_f32ray_mt(int nthreads, const uint32_t* grids, uint32_t ngrids,
                                   const float* density, const float* albedo,
                                   uint32_t nbricks, int levels, const float pos[3],
                                   const float dir0[3], const float du[3],
                                   const float dv[3], int width, int height,
                                   double alpha_scale, double step_vox, double* rgba,
                                   uint32_t* samples, uint32_t* bricks, uint8_t* ties) {
  march32_job j = {grids, ngrids, density, albedo, nbricks, levels, pos, dir0, du, dv,
                   width, height, alpha_scale, step_vox, rgba, samples, bricks, ties};
  return run_rows(nthreads, height, march32_row, &j);
}

/* ---- FP64 march of a pixel window [x0, x1) x [y0, y1) (FP64 rays, as
 * orc_brick_render_f64 and the FP64 adjoint cast them) ---- */
int orc_brick_render_f64_rect(const uint32_t* grids, uint32_t ngrids,
                              const float* density, const float* albedo,
                              uint32_t nbricks, int levels, const double pos[3],
                              const double dir0[3], const double du[3],
                              const double dv[3], int width, int height,
                              double alpha_scale, double step_vox, int x0, int x1,
                              int y0, int y1, double* rgba, uint32_t* samples) {
  brick_ctx_f64 c;
  if (brick_ctx_init_f64(&c, grids, ngrids, density, albedo, nbricks, levels,
                         alpha_scale, step_vox))
    return 1;
  if (x0 < 0) x0 = 0;
  if (y0 < 0) y0 = 0;
  if (x1 > width) x1 = width;
  if (y1 > height) y1 = height;
  for (int y = y0; y < y1; ++y)
    for (int x = x0; x < x1; ++x) {
      size_t off = (size_t)y * (size_t)width + (size_t)x;
      double d[3];
      pixel_dir_f64(dir0, du, dv, x, y, d);
      adjust_dir_f64(d);
      double out[4];
      uint32_t ns = 0;
      int st = brick_march_f64(&c, pos, d, out, &ns, 0, 0, 0);
      if (st) return st;
      for (int i = 0; i < 4; ++i) rgba[off * 4 + (size_t)i] = out[i];
      if (samples) samples[off] = ns;
    }
  return 0;
}

int orc_brick_render_f64_f32ray_rect(const uint32_t* grids, uint32_t ngrids,
                                     const float* density, const float* albedo,
                                     uint32_t nbricks, int levels, const float pos[3],
                                     const float dir0[3], const float du[3],
                                     const float dv[3], int width, int height,
                                     double alpha_scale, double step_vox, int x0, int x1,
                                     int y0, int y1, double* rgba, uint32_t* samples) {
  brick_ctx_f64 c;
  if (brick_ctx_init_f64(&c, grids, ngrids, density, albedo, nbricks, levels,
                         alpha_scale, step_vox))
    return 1;
  if (x0 < 0) x0 = 0;
  if (y0 < 0) y0 = 0;
  if (x1 > width) x1 = width;
  if (y1 > height) y1 = height;
  const double o[3] = {pos[0], pos[1], pos[2]};
  for (int y = y0; y < y1; ++y)
    for (int x = x0; x < x1; ++x) {
      size_t off = (size_t)y * (size_t)width + (size_t)x;
      float df[3];
      pixel_dir_f32(dir0, du, dv, x, y, df);
      adjust_dir_f32(df);
      double d[3] = {df[0], df[1], df[2]};
      double out[4];
      uint32_t ns = 0;
      int st = brick_march_f64(&c, o, d, out, &ns, 0, 0, 0);
      if (st) return st;
      for (int i = 0; i < 4; ++i) rgba[off * 4 + (size_t)i] = out[i];
      if (samples) samples[off] = ns;
    }
  return 0;
}

/* ---- FP64 adjoint on threads ---- */
typedef struct {
  brick_ctx_f64 proto;
  const double *pos, *dir0, *du, *dv;
  /* FP32 rays (orc_brick_backward_f64_f32ray_mt): float basis, or NULL */
  const float *fdir0, *fdu, *fdv;
  int width;
  double alpha_scale;
  const double* grad_rgba;
  double** gd;  /* per-thread accumulators */
  double** ga;
} bwd_job;

static int bwd_row(void* ctx, int y, int tid) {
  bwd_job* j = (bwd_job*)ctx;
  brick_ctx_f64 c = j->proto;
  for (int x = 0; x < j->width; ++x) {
    size_t off = (size_t)y * (size_t)j->width + (size_t)x;
    double d[3];
    if (j->fdir0) {
      float df[3];
      pixel_dir_f32(j->fdir0, j->fdu, j->fdv, x, y, df);
      adjust_dir_f32(df);
      d[0] = df[0];
      d[1] = df[1];
      d[2] = df[2];
    } else {
      pixel_dir_f64(j->dir0, j->du, j->dv, x, y, d);
      adjust_dir_f64(d);
    }
    double out[4];
    int st = brick_march_f64(&c, j->pos, d, out, 0, 0, 0, 0);
    if (st) return st;
    bwd_user u = {j->grad_rgba + off * 4, out, j->alpha_scale, j->gd[tid], j->ga[tid]};
    double out2[4];
    st = brick_march_f64(&c, j->pos, d, out2, 0, 0, bwd_sample, &u);
    if (st) return st;
  }
  return 0;
}

static int backward_mt(int nthreads, bwd_job* jp, const uint32_t* grids, uint32_t ngrids,
                       const float* density, const float* albedo, uint32_t nbricks,
                       int levels, int width, int height, double alpha_scale,
                       double step_vox, const double* grad_rgba, double* grad_density,
                       double* grad_albedo);

int orc_brick_backward_f64_mt(int nthreads, const uint32_t* grids, uint32_t ngrids,
                              const float* density, const float* albedo,
                              uint32_t nbricks, int levels, const double pos[3],
                              const double dir0[3], const double du[3],
                              const double dv[3], int width, int height,
                              double alpha_scale, double step_vox,
                              const double* grad_rgba, double* grad_density,
                              double* grad_albedo) {
  bwd_job j;
  memset(&j, 0, sizeof(j));
  j.pos = pos;
  j.dir0 = dir0;
  j.du = du;
  j.dv = dv;
  return backward_mt(nthreads, &j, grids, ngrids, density, albedo, nbricks, levels, width,
                     height, alpha_scale, step_vox, grad_rgba, grad_density, grad_albedo);
}

int orc_brick_backward_f64_f32ray_mt(int nthreads, const uint32_t* grids, uint32_t ngrids,
                                     const float* density, const float* albedo,
                                     uint32_t nbricks, int levels, const float pos[3],
                                     const float dir0[3], const float du[3],
                                     const float dv[3], int width, int height,
                                     double alpha_scale, double step_vox,
                                     const double* grad_rgba, double* grad_density,
                                     double* grad_albedo) {
  bwd_job j;
  memset(&j, 0, sizeof(j));
  const double o[3] = {pos[0], pos[1], pos[2]};
  j.pos = o;
  j.fdir0 = dir0;
  j.fdu = du;
  j.fdv = dv;
  return backward_mt(nthreads, &j, grids, ngrids, density, albedo, nbricks, levels, width,
                     height, alpha_scale, step_vox, grad_rgba, grad_density, grad_albedo);
}

static int backward_mt(int nthreads, bwd_job* jp, const uint32_t* grids, uint32_t ngrids,
                       const float* density, const float* albedo, uint32_t nbricks,
                       int levels, int width, int height, double alpha_scale,
                       double step_vox, const double* grad_rgba, double* grad_density,
                       double* grad_albedo) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  bwd_job j = *jp;
  if (brick_ctx_init_f64(&j.proto, grids, ngrids, density, albedo, nbricks, levels,
                         alpha_scale, step_vox))
    return 1;
  const size_t nd = (size_t)nbricks * 729u, na = nd * 3u;
  j.width = width;
  j.alpha_scale = alpha_scale;
  j.grad_rgba = grad_rgba;
  j.gd = (double**)calloc((size_t)nthreads, sizeof(double*));
  j.ga = (double**)calloc((size_t)nthreads, sizeof(double*));
  int st = (j.gd && j.ga) ? 0 : 7;
  for (int i = 0; i < nthreads && !st; ++i) {
    j.gd[i] = (double*)calloc(nd ? nd : 1, sizeof(double));
    j.ga[i] = (double*)calloc(na ? na : 1, sizeof(double));
    if (!j.gd[i] || !j.ga[i]) st = 7;
  }
  if (!st) st = run_rows(nthreads, height, bwd_row, &j);
  if (!st)
    for (int i = 0; i < nthreads; ++i) {
      for (size_t k = 0; k < nd; ++k) grad_density[k] += j.gd[i][k];
      for (size_t k = 0; k < na; ++k) grad_albedo[k] += j.ga[i][k];
    }
  for (int i = 0; i < nthreads; ++i) {
    if (j.gd) free(j.gd[i]);
    if (j.ga) free(j.ga[i]);
  }
  free(j.gd);
  free(j.ga);
  return st;
}

/* ---- FP64 march of arbitrary rays (origins and directions given) ---- */
int orc_brick_march_rays_f64(const uint32_t* grids, uint32_t ngrids, const float* density,
                             const float* albedo, uint32_t nbricks, int levels,
                             double alpha_scale, double step_vox, int transfer,
                             const double* origins, const double* dirs, int n, double* rgba,
                             uint32_t* samples) {
  brick_ctx_f64 c;
  if (brick_ctx_init_f64(&c, grids, ngrids, density, albedo, nbricks, levels, alpha_scale,
                         step_vox))
    return 1;
  c.transfer = transfer;
  for (int i = 0; i < n; ++i) {
    uint32_t ns = 0;
    int st = brick_march_f64(&c, origins + 3 * (size_t)i, dirs + 3 * (size_t)i,
                             rgba + 4 * (size_t)i, &ns, 0, 0, 0);
    if (st) return st;
    if (samples) samples[i] = ns;
  }
  return 0;
}
