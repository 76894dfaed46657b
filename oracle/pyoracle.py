"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker, and by bench.py's CPU-baseline / reference legs.  The product
(libyoxel.so and the yoxel package) never imports it.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_library(build_if_missing=True):
    path = os.path.join(HERE, "liboracle.so")
    if build_if_missing:
        import importlib.util
        spec = importlib.util.spec_from_file_location("_oracle_build", os.path.join(HERE, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        try:
            mod.build()
        except Exception:
            if not os.path.exists(path):
                raise
    lib = C.CDLL(path)
    P = C.c_void_p
    F = C.c_float
    D = C.c_double
    I = C.c_int
    U = C.c_uint32
    sig = {
        "orc_init_ray_dir_f32": (None, [P, P, F, I, I, P, P, P]),
        "orc_init_ray_dir_f64": (None, [P, P, D, I, I, P, P, P]),
        "orc_svo_render_f32": (I, [P, U, U, P, U, P, P, P, P, I, I, P, F, F, I, I, I,
                                   P, P, P, P, P, P]),
        "orc_svo_render_lod_f32": (I, [P, U, U, P, U, P, P, P, P, I, I, P, F, F, I, F, I, I,
                                       P, P, P, P, P, P]),
        "orc_svo_render_mt": (I, [I, P, U, U, P, U, P, P, P, P, I, I, P, F, F, I,
                                  P, P, P, P, P, P]),
        "orc_svo_render_mt_lod": (I, [I, P, U, U, P, U, P, P, P, P, I, I, P, F, F, I, F,
                                      P, P, P, P, P, P]),
        "orc_svo_hits_f64": (I, [P, U, U, P, P, P, D, I, I, I, I, P, P]),
        "orc_svo_trace_ray_f32": (I, [P, U, U, P, P, I, P, P, P, P]),
        "orc_find_first_child_f32": (None, [P, P, P]),
        "orc_go_next_f32": (I, [P, P, P]),
        "orc_setup_trace_f32": (I, [P, P, P, P, P]),
        "orc_brick_render_f64": (I, [P, U, P, P, U, I, P, P, P, P, I, I, D, D, I, I, P, P, P]),
        "orc_brick_render_f32": (I, [P, U, P, P, U, I, P, P, P, P, I, I, F, F, I, I, P, P, P]),
        "orc_brick_render_f64_f32ray": (I, [P, U, P, P, U, I, P, P, P, P, I, I, D, D, I, I,
                                            P, P, P, P]),
        "orc_brick_render_mt_f32": (I, [I, P, U, P, P, U, I, P, P, P, P, I, I, F, F, P, P, P]),
        "orc_brick_backward_f64": (I, [P, U, P, P, U, I, P, P, P, P, I, I, D, D, P, P, P]),
        "orc_svo_build_dense": (I, [P, P, I, F, P, U, P, U, P, P, P]),
        "orc_svo_hits_f64_mt": (I, [I, P, U, U, P, P, P, D, I, I, P, P]),
        "orc_brick_march_rays_f64": (I, [P, U, P, P, U, I, D, D, I, P, P, I, P, P]),
        "orc_svo_hits_f64_f32ray_mt": (I, [I, P, U, U, P, P, P, P, I, I, P, P]),
        "orc_brick_backward_f64_f32ray_mt": (I, [I, P, U, P, P, U, I, P, P, P, P, I, I, D, D,
                                                 P, P, P]),
        "orc_brick_render_f64_f32ray_mt": (I, [I, P, U, P, P, U, I, P, P, P, P, I, I, D, D,
                                               P, P, P, P]),
        "orc_brick_backward_f64_mt": (I, [I, P, U, P, P, U, I, P, P, P, P, I, I, D, D, P, P,
                                          P]),
        "orc_brick_render_f64_rect": (I, [P, U, P, P, U, I, P, P, P, P, I, I, D, D, I, I, I, I,
                                          P, P]),
        "orc_brick_render_f64_f32ray_rect": (I, [P, U, P, P, U, I, P, P, P, P, I, I, D, D, I, I,
                                                 I, I, P, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = load_library()
    return _lib


_KEEP = []


def _p(a):
    """Pointer to a numpy array's data.  The array is kept alive until the
    next _release() so temporaries survive the ctypes call."""
    if a is None:
        return None
    _KEEP.append(a)
    return C.c_void_p(a.ctypes.data)


def _release():
    del _KEEP[:]


def _keeps(fn):
    def w(*a, **k):
        mark = len(_KEEP)
        try:
            return fn(*a, **k)
        finally:
            del _KEEP[mark:]
    w.__name__ = fn.__name__
    w.__doc__ = fn.__doc__
    return w


def f32(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.float32).reshape(-1))


def f64(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(-1))


@_keeps
def init_ray_dir_f32(dir_, up, fov, width, height):
    d0, du, dv = (np.zeros(3, np.float32) for _ in range(3))
    lib().orc_init_ray_dir_f32(_p(f32(dir_)), _p(f32(up)), float(fov), width, height,
                               _p(d0), _p(du), _p(dv))
    return d0, du, dv


@_keeps
def init_ray_dir_f64(dir_, up, fov, width, height):
    d0, du, dv = (np.zeros(3, np.float64) for _ in range(3))
    lib().orc_init_ray_dir_f64(_p(f64(dir_)), _p(f64(up)), float(fov), width, height,
                               _p(d0), _p(du), _p(dv))
    return d0, du, dv


@_keeps
def svo_render(nodes_u32, root, attrs_u8, pos, dir_, up, fov, width, height, light,
               ambient=0.15, diffuse=0.85, shadows=False, threads=1, rows=None, lod_coef=0.0):
    """FP32 oracle render.  Returns dict of numpy arrays (rgba u32, hit u32,
    hit_t f32, fetches u32, shadow_fetches u32, shadowed u8).  lod_coef > 0:
    the level-of-detail cut-off."""
    nodes_u32 = np.ascontiguousarray(nodes_u32, dtype=np.uint32)
    attrs_u8 = np.ascontiguousarray(attrs_u8, dtype=np.uint8)
    count = len(nodes_u32) // 10
    nattrs = len(attrs_u8) // 8
    d0, du, dv = init_ray_dir_f32(dir_, up, fov, width, height)
    n = width * height
    out = dict(rgba=np.zeros(n, np.uint32), hit=np.full(n, 0xFFFFFFFF, np.uint32),
               hit_t=np.zeros(n, np.float32), fetches=np.zeros(n, np.uint32),
               shadow_fetches=np.zeros(n, np.uint32), shadowed=np.zeros(n, np.uint8))
    ps, lt = f32(pos), f32(light)
    if threads <= 1 or rows is not None:
        y0, y1 = (0, height) if rows is None else rows
        st = lib().orc_svo_render_lod_f32(_p(nodes_u32), count, root, _p(attrs_u8), nattrs,
                                          _p(ps), _p(d0), _p(du), _p(dv), width, height,
                                          _p(lt), ambient, diffuse, 1 if shadows else 0,
                                          float(lod_coef), y0, y1,
                                          _p(out["rgba"]), _p(out["hit"]), _p(out["hit_t"]),
                                          _p(out["fetches"]), _p(out["shadow_fetches"]),
                                          _p(out["shadowed"]))
    else:
        st = lib().orc_svo_render_mt_lod(threads, _p(nodes_u32), count, root, _p(attrs_u8),
                                         nattrs, _p(ps), _p(d0), _p(du), _p(dv), width,
                                         height, _p(lt), ambient, diffuse,
                                         1 if shadows else 0, float(lod_coef),
                                         _p(out["rgba"]), _p(out["hit"]), _p(out["hit_t"]),
                                         _p(out["fetches"]), _p(out["shadow_fetches"]),
                                         _p(out["shadowed"]))
    if st != 0:
        raise RuntimeError(f"oracle svo render failed: {st}")
    return {k: v.reshape(height, width) for k, v in out.items()}


@_keeps
def svo_hits_f64(nodes_u32, root, pos, dir_, up, fov, width, height, rows=None, threads=1):
    nodes_u32 = np.ascontiguousarray(nodes_u32, dtype=np.uint32)
    n = width * height
    hit = np.full(n, 0xFFFFFFFF, np.uint32)
    t = np.zeros(n, np.float64)
    if threads > 1 and rows is None:
        st = lib().orc_svo_hits_f64_mt(int(threads), _p(nodes_u32), len(nodes_u32) // 10, root,
                                       _p(f64(pos)), _p(f64(dir_)), _p(f64(up)), float(fov),
                                       width, height, _p(hit), _p(t))
        if st != 0:
            raise RuntimeError(f"oracle f64 hits failed: {st}")
        return hit.reshape(height, width), t.reshape(height, width)
    y0, y1 = (0, height) if rows is None else rows
    st = lib().orc_svo_hits_f64(_p(nodes_u32), len(nodes_u32) // 10, root, _p(f64(pos)),
                                _p(f64(dir_)), _p(f64(up)), float(fov), width, height, y0, y1,
                                _p(hit), _p(t))
    if st != 0:
        raise RuntimeError(f"oracle f64 hits failed: {st}")
    return hit.reshape(height, width), t.reshape(height, width)


@_keeps
def svo_hits_f64_f32ray(nodes_u32, root, pos, dir_, up, fov, width, height, threads=1):
    """FP64 traversal of the FP32 primary rays (hits differ from the float
    traversal only where a rounding tie inside the traversal decides)."""
    nodes_u32 = np.ascontiguousarray(nodes_u32, dtype=np.uint32)
    d0, du, dv = init_ray_dir_f32(dir_, up, fov, width, height)
    n = width * height
    hit = np.full(n, 0xFFFFFFFF, np.uint32)
    t = np.zeros(n, np.float64)
    st = lib().orc_svo_hits_f64_f32ray_mt(max(1, int(threads)), _p(nodes_u32),
                                          len(nodes_u32) // 10, root, _p(f32(pos)), _p(d0),
                                          _p(du), _p(dv), width, height, _p(hit), _p(t))
    if st != 0:
        raise RuntimeError(f"oracle f64 hits failed: {st}")
    return hit.reshape(height, width), t.reshape(height, width)


@_keeps
def brick_backward_f64_f32ray(grids, density, albedo, levels, pos, dir_, up, fov, width,
                              height, grad_rgba, alpha_scale=1.0, step_vox=0.5, threads=1):
    """FP64 adjoint along the FP32 primary rays (the rays the CUDA path
    casts); pool layout, apron slots holding their own share."""
    g, d, a = _vol_arrays(grids, density, albedo)
    d0, du, dv = init_ray_dir_f32(dir_, up, fov, width, height)
    gr = np.ascontiguousarray(np.asarray(grad_rgba, np.float64).reshape(-1))
    gd = np.zeros(len(d), np.float64)
    ga = np.zeros(len(a), np.float64)
    st = lib().orc_brick_backward_f64_f32ray_mt(max(1, int(threads)), _p(g), len(g) // 64,
                                                _p(d), _p(a), len(d) // 729, levels,
                                                _p(f32(pos)), _p(d0), _p(du), _p(dv), width,
                                                height, float(alpha_scale), float(step_vox),
                                                _p(gr), _p(gd), _p(ga))
    if st != 0:
        raise RuntimeError(f"oracle brick backward failed: {st}")
    return gd, ga


@_keeps
def trace_ray_f32(nodes_u32, root, pos, dir_, cull_behind=False):
    nodes_u32 = np.ascontiguousarray(nodes_u32, dtype=np.uint32)
    hit = np.zeros(1, np.uint32)
    t = np.zeros(1, np.float32)
    f = np.zeros(1, np.uint32)
    lv = np.zeros(1, np.int32)
    ok = lib().orc_svo_trace_ray_f32(_p(nodes_u32), len(nodes_u32) // 10, root, _p(f32(pos)),
                                     _p(f32(dir_)), 1 if cull_behind else 0, _p(hit), _p(t),
                                     _p(f), _p(lv))
    if ok < 0:
        raise RuntimeError(f"oracle trace failed: {-ok}")
    return bool(ok), int(hit[0]), float(t[0]), int(f[0]), int(lv[0])


@_keeps
def find_first_child(t1, t2):
    a, b = f32(t1).copy(), f32(t2).copy()
    ch = np.zeros(1, np.int32)
    lib().orc_find_first_child_f32(_p(a), _p(b), _p(ch))
    return int(ch[0]), a, b


@_keeps
def go_next(ch, t1, t2):
    a, b = f32(t1).copy(), f32(t2).copy()
    c = np.array([ch], np.int32)
    ok = lib().orc_go_next_f32(_p(c), _p(a), _p(b))
    return bool(ok), int(c[0]), a, b


@_keeps
def setup_trace(pos, dir_):
    t1, t2 = np.zeros(3, np.float32), np.zeros(3, np.float32)
    fl = np.zeros(1, np.uint32)
    ok = lib().orc_setup_trace_f32(_p(f32(pos)), _p(f32(dir_)), _p(t1), _p(t2), _p(fl))
    return bool(ok), t1, t2, int(fl[0])


def _vol_arrays(grids, density, albedo):
    g = np.ascontiguousarray(np.asarray(grids).reshape(-1).view(np.uint32)
                             if np.asarray(grids).dtype != np.uint32 else np.asarray(grids).reshape(-1))
    d = np.ascontiguousarray(np.asarray(density, np.float32).reshape(-1))
    a = np.ascontiguousarray(np.asarray(albedo, np.float32).reshape(-1))
    return g, d, a


@_keeps
def brick_render_f64(grids, density, albedo, levels, pos, dir_, up, fov, width, height,
                     alpha_scale=1.0, step_vox=0.5, rows=None):
    """FP64 brick march.  density (nb,729) float, albedo (nb,729,3) float in
    [0,1].  Returns (h,w,4) float64 rgba, samples, bricks (h,w) uint32."""
    g, d, a = _vol_arrays(grids, density, albedo)
    d0, du, dv = init_ray_dir_f64(dir_, up, fov, width, height)
    rgba = np.zeros(width * height * 4, np.float64)
    ns = np.zeros(width * height, np.uint32)
    nb = np.zeros(width * height, np.uint32)
    y0, y1 = (0, height) if rows is None else rows
    st = lib().orc_brick_render_f64(_p(g), len(g) // 64, _p(d), _p(a), len(d) // 729, levels,
                                    _p(f64(pos)), _p(d0), _p(du), _p(dv), width, height,
                                    float(alpha_scale), float(step_vox), y0, y1, _p(rgba),
                                    _p(ns), _p(nb))
    if st != 0:
        raise RuntimeError(f"oracle brick render failed: {st}")
    return rgba.reshape(height, width, 4), ns.reshape(height, width), nb.reshape(height, width)


@_keeps
def brick_render_f32_mt(grids, density, albedo, levels, pos, dir_, up, fov, width, height,
                        alpha_scale=1.0, step_vox=0.5, threads=1):
    g, d, a = _vol_arrays(grids, density, albedo)
    d0, du, dv = init_ray_dir_f32(dir_, up, fov, width, height)
    rgba = np.zeros(width * height * 4, np.float32)
    ns = np.zeros(width * height, np.uint32)
    nb = np.zeros(width * height, np.uint32)
    st = lib().orc_brick_render_mt_f32(threads, _p(g), len(g) // 64, _p(d), _p(a),
                                       len(d) // 729, levels, _p(f32(pos)), _p(d0), _p(du),
                                       _p(dv), width, height, float(alpha_scale),
                                       float(step_vox), _p(rgba), _p(ns), _p(nb))
    if st != 0:
        raise RuntimeError(f"oracle brick render failed: {st}")
    return rgba.reshape(height, width, 4), ns.reshape(height, width), nb.reshape(height, width)


@_keeps
def brick_backward_f64(grids, density, albedo, levels, pos, dir_, up, fov, width, height,
                       grad_rgba, alpha_scale=1.0, step_vox=0.5, threads=1):
    """FP64 adjoint: returns (grad_density (nb*729), grad_albedo (nb*729*3))
    in pool layout, apron slots holding their own share.  threads > 1: row-
    parallel, per-thread accumulators summed in thread order."""
    g, d, a = _vol_arrays(grids, density, albedo)
    d0, du, dv = init_ray_dir_f64(dir_, up, fov, width, height)
    gr = np.ascontiguousarray(np.asarray(grad_rgba, np.float64).reshape(-1))
    gd = np.zeros(len(d), np.float64)
    ga = np.zeros(len(a), np.float64)
    if threads > 1:
        st = lib().orc_brick_backward_f64_mt(int(threads), _p(g), len(g) // 64, _p(d), _p(a),
                                             len(d) // 729, levels, _p(f64(pos)), _p(d0),
                                             _p(du), _p(dv), width, height, float(alpha_scale),
                                             float(step_vox), _p(gr), _p(gd), _p(ga))
        if st != 0:
            raise RuntimeError(f"oracle brick backward failed: {st}")
        return gd, ga
    st = lib().orc_brick_backward_f64(_p(g), len(g) // 64, _p(d), _p(a), len(d) // 729, levels,
                                      _p(f64(pos)), _p(d0), _p(du), _p(dv), width, height,
                                      float(alpha_scale), float(step_vox), _p(gr), _p(gd), _p(ga))
    if st != 0:
        raise RuntimeError(f"oracle brick backward failed: {st}")
    return gd, ga


@_keeps
def brick_render_f64_f32ray(grids, density, albedo, levels, pos, dir_, up, fov, width, height,
                            alpha_scale=1.0, step_vox=0.5, rows=None, threads=1, ties=False):
    """FP64 march of the FP32-generated primary rays (the rays the CUDA path
    casts), so the comparison measures the march arithmetic alone.  Returns
    (rgba, samples, bricks), and with ties=True also the per-ray flag of a
    sample set or early exit decided by a rounding tie (yv_oracle.h)."""
    g, d, a = _vol_arrays(grids, density, albedo)
    d0, du, dv = init_ray_dir_f32(dir_, up, fov, width, height)
    rgba = np.zeros(width * height * 4, np.float64)
    ns = np.zeros(width * height, np.uint32)
    nb = np.zeros(width * height, np.uint32)
    tf = np.zeros(width * height, np.uint8)
    if threads > 1 and rows is None:
        st = lib().orc_brick_render_f64_f32ray_mt(int(threads), _p(g), len(g) // 64, _p(d),
                                                  _p(a), len(d) // 729, levels, _p(f32(pos)),
                                                  _p(d0), _p(du), _p(dv), width, height,
                                                  float(alpha_scale), float(step_vox),
                                                  _p(rgba), _p(ns), _p(nb), _p(tf))
    else:
        y0, y1 = (0, height) if rows is None else rows
        st = lib().orc_brick_render_f64_f32ray(_p(g), len(g) // 64, _p(d), _p(a),
                                               len(d) // 729, levels, _p(f32(pos)), _p(d0),
                                               _p(du), _p(dv), width, height,
                                               float(alpha_scale), float(step_vox), y0, y1,
                                               _p(rgba), _p(ns), _p(nb), _p(tf))
    if st != 0:
        raise RuntimeError(f"oracle brick render failed: {st}")
    out = (rgba.reshape(height, width, 4), ns.reshape(height, width), nb.reshape(height, width))
    return out + (tf.reshape(height, width).astype(bool),) if ties else out


@_keeps
def brick_march_rays_f64(grids, density, albedo, levels, origins, dirs, alpha_scale=1.0,
                         step_vox=0.5, transfer=0):
    """FP64 march of rays (n x 3 origins and directions); transfer 1 is the
    fixed transfer of reaction/trace/trace.cu.  Returns (rgba (n, 4),
    samples (n,))."""
    g, d, a = _vol_arrays(grids, density, albedo)
    o = np.ascontiguousarray(origins, np.float64).reshape(-1, 3)
    dv = np.ascontiguousarray(dirs, np.float64).reshape(-1, 3)
    n = len(o)
    rgba = np.zeros((n, 4), np.float64)
    ns = np.zeros(n, np.uint32)
    st = lib().orc_brick_march_rays_f64(_p(g), len(g) // 64, _p(d), _p(a), len(d) // 729,
                                        levels, float(alpha_scale), float(step_vox),
                                        int(transfer), _p(o), _p(dv), n, _p(rgba), _p(ns))
    if st != 0:
        raise RuntimeError(f"oracle brick march failed: {st}")
    return rgba, ns


class BrickWindow:
    """FP64 march of pixel windows of one camera over a volume whose arrays
    are modified in place between calls (central differences).  Holds the
    float32 copies the oracle reads; `density` / `albedo` are those arrays."""

    def __init__(self, grids, density, albedo, levels, pos, dir_, up, fov, width, height,
                 alpha_scale=1.0, step_vox=0.5, f32ray=False):
        self.g, self.density, self.albedo = _vol_arrays(grids, density, albedo)
        self.density = self.density.copy()
        self.albedo = self.albedo.copy()
        self.levels, self.width, self.height = levels, width, height
        # f32ray: the FP32 primary rays (as the CUDA path casts them), promoted
        self.f32ray = bool(f32ray)
        if self.f32ray:
            self.pos = f32(pos)
            self.d0, self.du, self.dv = init_ray_dir_f32(dir_, up, fov, width, height)
        else:
            self.pos = f64(pos)
            self.d0, self.du, self.dv = init_ray_dir_f64(dir_, up, fov, width, height)
        self.alpha_scale, self.step_vox = float(alpha_scale), float(step_vox)
        self.rgba = np.zeros(width * height * 4, np.float64)
        self.samples = np.zeros(width * height, np.uint32)

    def render(self, x0, x1, y0, y1):
        """(y1-y0, x1-x0, 4) radiance of the window; the samples each ray took
        are left in self.samples (full-frame, row-major)."""
        fn = (lib().orc_brick_render_f64_f32ray_rect if self.f32ray
              else lib().orc_brick_render_f64_rect)
        st = fn(
            self.g.ctypes.data, len(self.g) // 64, self.density.ctypes.data,
            self.albedo.ctypes.data, len(self.density) // 729, self.levels,
            self.pos.ctypes.data, self.d0.ctypes.data, self.du.ctypes.data,
            self.dv.ctypes.data, self.width, self.height, self.alpha_scale, self.step_vox,
            x0, x1, y0, y1, self.rgba.ctypes.data, self.samples.ctypes.data)
        if st != 0:
            raise RuntimeError(f"oracle brick window failed: {st}")
        return self.rgba.reshape(self.height, self.width, 4)[y0:y1, x0:x1].copy()

    def window_samples(self, x0, x1, y0, y1):
        """Samples per ray of the last render of the window."""
        return self.samples.reshape(self.height, self.width)[y0:y1, x0:x1].copy()


def svo_build_dense(density, depth, iso=0.0, rgb=None):
    """CPU build of the canonical SVO from a dense (2^depth)^3 float32 grid
    (x fastest).  Returns (nodes uint32 (n, 10), attrs uint8 (m, 8), root)."""
    G = 1 << depth
    d = np.ascontiguousarray(density, dtype=np.float32).reshape(-1)
    assert d.size == G ** 3
    c = None if rgb is None else np.ascontiguousarray(rgb, dtype=np.uint8).reshape(-1)
    assert c is None or c.size == 3 * G ** 3
    L = lib()
    nn, na, root = C.c_uint32(0), C.c_uint32(0), C.c_uint32(0)
    cap_n, cap_a = 1 << 16, 1 << 16
    while True:
        nodes = np.zeros((cap_n, 10), np.uint32)
        attrs = np.zeros((cap_a, 8), np.uint8)
        st = L.orc_svo_build_dense(d.ctypes.data, None if c is None else c.ctypes.data, depth,
                                   float(iso), nodes.ctypes.data, cap_n, attrs.ctypes.data,
                                   cap_a, C.byref(nn), C.byref(na), C.byref(root))
        if st == 1:
            cap_n, cap_a = max(nn.value, 1), max(na.value, 1)
            continue
        if st != 0:
            raise RuntimeError(f"orc_svo_build_dense: {st}")
        return nodes[:nn.value].copy(), attrs[:na.value].copy(), root.value
