/*
 * yv_oracle_impl.h - body of the CPU oracle, included once per scalar type
 * by yv_oracle.c with REAL (float|double) and SFX (f32|f64) defined.
 *
 * TEST INFRASTRUCTURE ONLY (see yv_oracle.h).  Compiled with
 * -ffp-contract=off so the float instantiation performs exactly one IEEE
 * rounding per written operation, the same sequence the CUDA kernels issue
 * with __fadd_rn/__fmul_rn/__fdiv_rn/__fsqrt_rn.
 */

#define CAT2(a, b) a##_##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(name, SFX)

typedef struct { REAL v[3]; } FN(vec3);
#define V3 FN(vec3)

static inline REAL FN(max3)(const REAL* a) {
  /* max_vec_float3: max(max(x, y), z) */
  REAL m = a[0] > a[1] ? a[0] : a[1];
  return m > a[2] ? m : a[2];
}
static inline REAL FN(min3)(const REAL* a) {
  REAL m = a[0] < a[1] ? a[0] : a[1];
  return m < a[2] ? m : a[2];
}

/* RendererBase::InitRayDir (cell/renderer_base.h:50-61):
 *   vfwd = normalized(dir); vright = normalized(vfwd ^ up);
 *   vup = vright ^ vfwd; da = tan(fov/2) / width;
 *   du = 2*vright*da; dv = -2*vup*da;
 *   dir0 = vfwd - du*width/2 - dv*height/2.                                */
static void FN(cross)(const REAL* a, const REAL* b, REAL* r) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}
static void FN(normalize)(REAL* v) {
  REAL len = SQRT((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
  v[0] = v[0] / len;
  v[1] = v[1] / len;
  v[2] = v[2] / len;
}

void CAT(orc_init_ray_dir, SFX)(const REAL dir[3], const REAL up[3],
                                REAL fov_deg, int width, int height,
                                REAL dir0[3], REAL du[3], REAL dv[3]) {
  REAL vfwd[3] = {dir[0], dir[1], dir[2]};
  FN(normalize)(vfwd);
  REAL vright[3];
  FN(cross)(vfwd, up, vright);
  FN(normalize)(vright);
  REAL vup[3];
  FN(cross)(vright, vfwd, vup);
  REAL half = fov_deg / (REAL)2;
  REAL rad = half * (REAL)(3.14159265358979323846 / 180.0);
  REAL da = TAN(rad) / (REAL)width;
  for (int i = 0; i < 3; ++i) {
    du[i] = ((REAL)2 * vright[i]) * da;
    dv[i] = ((REAL)-2 * vup[i]) * da;
  }
  for (int i = 0; i < 3; ++i) {
    REAL a = (du[i] * (REAL)width) / (REAL)2;
    REAL b = (dv[i] * (REAL)height) / (REAL)2;
    dir0[i] = (vfwd[i] - a) - b;
  }
}

/* Per-pixel direction, RenderRect (cell/ppu_renderer.cpp:56):
 *   dir = normalized(dir0 + du*x + dv*y)                                   */
static inline void FN(pixel_dir)(const REAL* dir0, const REAL* du,
                                 const REAL* dv, int x, int y, REAL* d) {
  REAL fx = (REAL)x, fy = (REAL)y;
  for (int i = 0; i < 3; ++i) d[i] = (dir0[i] + du[i] * fx) + dv[i] * fy;
  FN(normalize)(d);
}

/* AdjustDir: |d_i| < eps -> copysign(eps, d_i), eps = 1e-5
 * (cell/spu/trace_spu.c_:80-82, reaction/report/voxel.tex:316-318).       */
static inline void FN(adjust_dir)(REAL* d) {
  const REAL eps = (REAL)1e-5f;
  for (int i = 0; i < 3; ++i) {
    REAL a = d[i] < 0 ? -d[i] : d[i];
    if (a < eps) d[i] = COPYSIGN(eps, d[i]);
  }
}

/* SetupTrace: octant mirroring into the unit cube
 * (reaction/report/voxel.tex:312-326, cell/spu/trace_spu.c_:79-99):
 *   d_i < 0 -> p_i = 1 - p_i, d_i = -d_i, dirFlags |= 1<<i
 *   t1 = (0 - p) / d, t2 = (1 - p) / d; trace iff max(t1) < min(t2).      */
static inline int FN(setup_trace)(const REAL* pos, const REAL* dir, REAL* t1,
                                  REAL* t2, uint32_t* dir_flags) {
  uint32_t flags = 0;
  for (int i = 0; i < 3; ++i) {
    REAL p = pos[i], d = dir[i];
    if (d < 0) {
      p = (REAL)1 - p;
      d = -d;
      flags |= 1u << i;
    }
    t1[i] = ((REAL)0 - p) / d;
    t2[i] = ((REAL)1 - p) / d;
  }
  *dir_flags = flags;
  return FN(max3)(t1) < FN(min3)(t2);
}

/* FindFirstChild (cell/spu/trace_spu.cpp:48-68):
 *   tm = 0.5*(t1+t2); tEnter = max(t1); bit i set iff tEnter > tm_i;
 *   set bits: t1_i = tm_i, clear bits: t2_i = tm_i.                       */
static inline int FN(ffc)(REAL* t1, REAL* t2) {
  REAL te = FN(max3)(t1);
  int ch = 0;
  for (int i = 0; i < 3; ++i) {
    REAL tm = (REAL)0.5f * (t1[i] + t2[i]);
    if (te > tm) {
      ch |= 1 << i;
      t1[i] = tm;
    } else {
      t2[i] = tm;
    }
  }
  return ch;
}

/* GoNext (cell/spu/trace_spu.cpp:70-93): exit plane = argmin(t2) with the
 * tie order of :75-78; leave the node if that bit is already set; else flip
 * it and step the slab: dt = t2-t1, t1 = t2, t2 += dt.                    */
static inline int FN(go_next)(int* ch, REAL* t1, REAL* t2) {
  int e;
  if (t2[0] > t2[1])
    e = (t2[1] < t2[2]) ? 1 : 2;
  else
    e = (t2[0] < t2[2]) ? 0 : 2;
  int mask = 1 << e;
  if (*ch & mask) return 0;
  *ch ^= mask;
  REAL dt = t2[e] - t1[e];
  t1[e] = t2[e];
  t2[e] = t2[e] + dt;
  return 1;
}

typedef struct {
  uint32_t node;
  int child;
  REAL t;
  int level;
  REAL t1[3];
  int lod;         /* 1: stopped at the subtree in (node, child) */
} FN(hit_rec);

typedef struct {
  const uint32_t* nodes;
  uint32_t count;
  int cull_behind; /* shadow rays: leaves entirely behind the origin skip */
  int err;
  uint32_t fetches;
  REAL lod_coef;   /* > 0: level-of-detail cut-off (see rec_trace) */
} FN(trace_ctx);

/* RecTrace (cell/ppu_renderer.cpp:18-41), recursive as in the reference.  */
static int FN(rec_trace)(FN(trace_ctx) * c, uint32_t node_id, REAL* pt1,
                         REAL* pt2, uint32_t dir_flags, int level,
                         FN(hit_rec) * res) {
  REAL t1[3] = {pt1[0], pt1[1], pt1[2]};
  REAL t2[3] = {pt2[0], pt2[1], pt2[2]};
  if ((node_id & 0x80000000u) || FN(min3)(t2) <= 0) return 0;
  if (node_id >= c->count || level > 30) {
    c->err = 3;
    return 0;
  }
  const uint32_t* node = c->nodes + (size_t)node_id * 10u;
  c->fetches++;
  int ch = FN(ffc)(t1, t2);
  for (;;) {
    int cc = ch ^ (int)dir_flags;
    if ((node[0] >> cc) & 1u) {
      if (!c->cull_behind || FN(min3)(t2) > 0) {
        res->node = node_id;
        res->child = cc;
        res->t = FN(max3)(t1);
        res->level = level;
        res->t1[0] = t1[0];
        res->t1[1] = t1[1];
        res->t1[2] = t1[2];
        res->lod = 0;
        return 1;
      }
    } else {
      /* Level-of-detail cut-off (SVORenderer::SetDetailCoef,
       * demo/SVORenderer.cpp:104; node data = the subtree at a coarser
       * level, reaction/report/main.tex:61): a subtree ahead of the ray
       * whose cube side 2^-(level+1) is below max(t_enter, 0) * lod_coef
       * ends the ray there.  Sides are powers of two (exact). */
      uint32_t sub = node[2 + cc];
      if (c->lod_coef > 0 && !(sub & 0x80000000u) && FN(min3)(t2) > 0) {
        REAL side = LDEXP((REAL)1, -(level + 1));
        REAL te = FN(max3)(t1);
        if (te < 0) te = 0;
        if (side < te * c->lod_coef) {
          res->node = node_id;
          res->child = cc;
          res->t = FN(max3)(t1);
          res->level = level;
          res->t1[0] = t1[0];
          res->t1[1] = t1[1];
          res->t1[2] = t1[2];
          res->lod = 1;
          return 1;
        }
      }
      if (FN(rec_trace)(c, sub, t1, t2, dir_flags, level + 1, res)) return 1;
    }
    if (c->err) return 0;
    if (!FN(go_next)(&ch, t1, t2)) return 0;
  }
}

/* One ray from pos along dir (already adjusted).  Returns 1 on a hit. */
static int FN(trace_one)(FN(trace_ctx) * c, uint32_t root, const REAL* pos,
                         const REAL* dir, FN(hit_rec) * res,
                         uint32_t* dir_flags_out) {
  REAL t1[3], t2[3];
  uint32_t dir_flags;
  if (!FN(setup_trace)(pos, dir, t1, t2, &dir_flags)) return 0;
  if (dir_flags_out) *dir_flags_out = dir_flags;
  return FN(rec_trace)(c, root, t1, t2, dir_flags, 0, res);
}

/* ------------------------------------------------------------------------ */
/* Brick volume ray-march (ntree layout), restating castRay / walkBrick /    */
/* intersect of reaction/trace/trace.cu:42-139 over an N=4 grid tree whose   */
/* last level points to 9^3-lattice bricks (8^3 cells + far-side apron).     */
/* ------------------------------------------------------------------------ */
typedef struct {
  const uint32_t* grids;
  uint32_t ngrids;
  const float* density;
  const float* albedo;
  uint32_t nbricks;
  int levels;
  int nb;          /* brick cells per axis = 4^levels */
  REAL S;          /* lattice cells per axis = 8 * nb */
  REAL alpha_scale;
  REAL dt;         /* world-space step = step_vox / S */
  REAL inv_dt;
  int err;
  /* set by brick_march when the ray's sample set or its early exit is
   * decided by a rounding tie: a sample within TIE_T (relative) of a cell
   * boundary, two exit planes of a cell within TIE_T of each other, the
   * entry cell's coordinate within TIE_T of an integer, or the opacity
   * within TIE_A of the early-exit threshold after a sample */
  int tie;
  /* 0: the configs' transfer, alpha = saturate(alpha_scale * density) and
   * the interpolated albedo as colour; 1: the reference's fixed transfer of
   * reaction/trace/trace.cu:52-56, s = saturate(2 v - 0.9), alpha = s / 2,
   * colour (s, s, s) */
  int transfer;
} FN(brick_ctx);

/* Tree descent for brick cell c (ntree/ntree/nodes.h:56-99 child offsets
 * (z*N + y)*N + x).  Returns the brick index, -1 for an empty cell. */
static int FN(brick_lookup)(FN(brick_ctx) * c, const int* cell) {
  uint32_t node = 0;
  for (int lev = 0; lev < c->levels; ++lev) {
    int sh = 2 * (c->levels - 1 - lev);
    int ix = (cell[0] >> sh) & 3, iy = (cell[1] >> sh) & 3,
        iz = (cell[2] >> sh) & 3;
    if (node >= c->ngrids) {
      c->err = 3;
      return -1;
    }
    uint32_t ref = c->grids[(size_t)node * 64u + (uint32_t)((iz * 4 + iy) * 4 + ix)];
    if (ref & 0x80000000u) return -1;
    if (ref & 0x40000000u) {
      uint32_t b = ref & 0x3FFFFFFFu;
      if (lev != c->levels - 1 || b >= c->nbricks) {
        c->err = 3;
        return -1;
      }
      return (int)b;
    }
    if (lev == c->levels - 1) {
      c->err = 3;
      return -1;
    }
    node = ref;
  }
  return -1;
}

/* Trilinear corner indices and weights of local lattice point l in [0,8]^3
 * (software trilinear: the reference's tex3D linear filter, trace.cu:51). */
static inline void FN(brick_corners)(const REAL* l, uint32_t base,
                                     uint32_t* idx, REAL* w) {
  int i0[3];
  REAL f[3];
  for (int i = 0; i < 3; ++i) {
    REAL li = l[i];
    int k = (int)FLOOR(li);
    if (k < 0) k = 0;
    if (k > 7) k = 7;
    REAL fi = li - (REAL)k;
    if (fi < 0) fi = 0;
    if (fi > 1) fi = 1;
    i0[i] = k;
    f[i] = fi;
  }
  int n = 0;
  for (int dz = 0; dz < 2; ++dz)
    for (int dy = 0; dy < 2; ++dy)
      for (int dx = 0; dx < 2; ++dx) {
        REAL wx = dx ? f[0] : (REAL)1 - f[0];
        REAL wy = dy ? f[1] : (REAL)1 - f[1];
        REAL wz = dz ? f[2] : (REAL)1 - f[2];
        idx[n] = base + (uint32_t)(((i0[2] + dz) * 9 + (i0[1] + dy)) * 9 + (i0[0] + dx));
        w[n] = (wx * wy) * wz;
        ++n;
      }
}

/* Visitor over the samples of one ray, front to back.  Calls `on_sample`
 * (if set) with the sample state; returns the composited RGBA.  Sample
 * positions are the global multiples t = k*dt (trace.cu:47), restricted to
 * occupied bricks; each brick cell spans [t_in, t_out) with t_in the
 * previous cell's t_out, so the cells partition the ray. */
typedef void (*FN(sample_fn))(void* user, const uint32_t* idx, const REAL* w,
                              REAL sigma, const REAL* col, REAL alpha,
                              REAL acc_a_before, const REAL* acc_c_before);

#ifndef YV_ORC_TIES
#define YV_ORC_TIES
#define TIE_T 1e-6
#define TIE_A 1e-5
#endif
static inline int FN(near_rel)(REAL a, REAL b) {
  REAL d = a - b, m = a < 0 ? -a : a;
  if (d < 0) d = -d;
  return d <= (REAL)TIE_T * (m > (REAL)1e-3 ? m : (REAL)1e-3);
}

static int FN(brick_march)(FN(brick_ctx) * c, const REAL* o, const REAL* d,
                           REAL* out, uint32_t* n_samples,
                           uint32_t* n_bricks, FN(sample_fn) fn, void* user) {
  REAL inv[3], t1[3], t2[3];
  c->tie = 0;
  for (int i = 0; i < 4; ++i) out[i] = 0;
  for (int i = 0; i < 3; ++i) {
    inv[i] = (REAL)1 / d[i];
    REAL a = ((REAL)0 - o[i]) * inv[i];
    REAL b = ((REAL)1 - o[i]) * inv[i];
    t1[i] = a < b ? a : b;
    t2[i] = a < b ? b : a;
  }
  REAL t_enter = FN(max3)(t1), t_exit = FN(min3)(t2);
  if (t_enter < 0) t_enter = 0;
  if (t_exit < 0 || t_enter > t_exit) return 0;
  const REAL h = (REAL)8 / c->S; /* world size of a brick cell (2^-k) */
  int cell[3], step[3];
  for (int i = 0; i < 3; ++i) {
    REAL q = (o[i] + t_enter * d[i]) / h;
    int k = (int)FLOOR(q);
    /* near an interior cell plane (the entry face itself is clamped) */
    if ((k > 0 && k < c->nb && FN(near_rel)(q, (REAL)k)) ||
        (k + 1 < c->nb && FN(near_rel)(q, (REAL)(k + 1))))
      c->tie = 1;
    if (k < 0) k = 0;
    if (k > c->nb - 1) k = c->nb - 1;
    cell[i] = k;
    step[i] = d[i] > 0 ? 1 : -1;
  }
  REAL acc_c[3] = {0, 0, 0}, acc_a = 0;
  REAL t_in = t_enter;
  uint32_t ns = 0, nbk = 0;
  int done = 0;
  while (!done) {
    REAL tx[3];
    for (int i = 0; i < 3; ++i) {
      REAL plane = (REAL)(d[i] > 0 ? cell[i] + 1 : cell[i]) * h;
      tx[i] = (plane - o[i]) * inv[i];
    }
    int e = 0;
    if (tx[1] < tx[e]) e = 1;
    if (tx[2] < tx[e]) e = 2;
    REAL t_out = tx[e];
    for (int i = 0; i < 3; ++i)
      if (i != e && FN(near_rel)(tx[i], t_out)) c->tie = 1;
    int b = FN(brick_lookup)(c, cell);
    if (c->err) return c->err;
    if (b >= 0) {
      ++nbk;
      int64_t k = (int64_t)CEIL(t_in * c->inv_dt);
      /* the sample just before the cell's first one may fall inside it in
       * another precision */
      if (FN(near_rel)((REAL)(k - 1) * c->dt, t_in)) c->tie = 1;
      for (;; ++k) {
        REAL t = (REAL)k * c->dt;
        if (FN(near_rel)(t, t_in) || FN(near_rel)(t, t_out)) c->tie = 1;
        if (!(t < t_out)) break;
        REAL l[3];  /* brick-local lattice coordinates */
        for (int i = 0; i < 3; ++i)
          l[i] = t * (d[i] * c->S) + (o[i] * c->S - (REAL)(8 * cell[i]));
        uint32_t idx[8];
        REAL w[8];
        FN(brick_corners)(l, (uint32_t)b * 729u, idx, w);
        REAL sigma = 0, col[3] = {0, 0, 0};
        for (int j = 0; j < 8; ++j) {
          sigma += w[j] * (REAL)c->density[idx[j]];
          for (int ch = 0; ch < 3; ++ch)
            col[ch] += w[j] * (REAL)c->albedo[(size_t)idx[j] * 3u + (uint32_t)ch];
        }
        REAL alpha;
        if (c->transfer == 1) {
          REAL sv = (REAL)2 * sigma - (REAL)0.9;
          if (sv < 0) sv = 0;
          if (sv > 1) sv = 1;
          alpha = (REAL)0.5 * sv;
          col[0] = col[1] = col[2] = sv;
        } else {
          alpha = sigma * c->alpha_scale;
          if (alpha < 0) alpha = 0;
          if (alpha > 1) alpha = 1;
        }
        if (fn) fn(user, idx, w, sigma, col, alpha, acc_a, acc_c);
        REAL wgt = ((REAL)1 - acc_a) * alpha;
        for (int ch = 0; ch < 3; ++ch) acc_c[ch] += wgt * col[ch];
        acc_a += wgt;
        ++ns;
        {
          REAL da = acc_a - (REAL)0.99f;
          if (da < (REAL)TIE_A && da > -(REAL)TIE_A) c->tie = 1;
        }
        if (acc_a > (REAL)0.99f) {
          done = 1;
          break;
        }
      }
    }
    t_in = t_out;
    cell[e] += step[e];
    if (cell[e] < 0 || cell[e] >= c->nb) break;
  }
  out[0] = acc_c[0];
  out[1] = acc_c[1];
  out[2] = acc_c[2];
  out[3] = acc_a;
  if (n_samples) *n_samples = ns;
  if (n_bricks) *n_bricks = nbk;
  return 0;
}

static int FN(brick_ctx_init)(FN(brick_ctx) * c, const uint32_t* grids,
                              uint32_t ngrids, const float* density,
                              const float* albedo, uint32_t nbricks,
                              int levels, REAL alpha_scale, REAL step_vox) {
  if (levels < 1 || levels > 8 || ngrids == 0) return 1;
  c->grids = grids;
  c->ngrids = ngrids;
  c->density = density;
  c->albedo = albedo;
  c->nbricks = nbricks;
  c->levels = levels;
  c->nb = 1 << (2 * levels);
  c->S = (REAL)(8 * c->nb);
  c->alpha_scale = alpha_scale;
  c->dt = step_vox / c->S;
  c->inv_dt = c->S / step_vox;
  c->err = 0;
  c->tie = 0;
  c->transfer = 0;
  return 0;
}

static int FN(brick_render_rows)(FN(brick_ctx) * c, const REAL* pos,
                                 const REAL* dir0, const REAL* du,
                                 const REAL* dv, int width, int y0, int y1,
                                 REAL* rgba, uint32_t* samples,
                                 uint32_t* bricks) {
  for (int y = y0; y < y1; ++y)
    for (int x = 0; x < width; ++x) {
      size_t off = (size_t)y * (size_t)width + (size_t)x;
      REAL d[3];
      FN(pixel_dir)(dir0, du, dv, x, y, d);
      FN(adjust_dir)(d);
      REAL out[4];
      uint32_t ns = 0, nbk = 0;
      int st = FN(brick_march)(c, pos, d, out, &ns, &nbk, 0, 0);
      if (st) return st;
      if (rgba)
        for (int i = 0; i < 4; ++i) rgba[off * 4 + (size_t)i] = out[i];
      if (samples) samples[off] = ns;
      if (bricks) bricks[off] = nbk;
    }
  return 0;
}

int CAT(orc_brick_render, SFX)(const uint32_t* grids, uint32_t ngrids,
                               const float* density, const float* albedo,
                               uint32_t nbricks, int levels, const REAL pos[3],
                               const REAL dir0[3], const REAL du[3],
                               const REAL dv[3], int width, int height,
                               REAL alpha_scale, REAL step_vox, int y0, int y1,
                               REAL* rgba, uint32_t* samples,
                               uint32_t* bricks) {
  FN(brick_ctx) c;
  if (FN(brick_ctx_init)(&c, grids, ngrids, density, albedo, nbricks, levels,
                         alpha_scale, step_vox))
    return 1;
  if (y0 < 0) y0 = 0;
  if (y1 > height) y1 = height;
  return FN(brick_render_rows)(&c, pos, dir0, du, dv, width, y0, y1, rgba,
                               samples, bricks);
}
