"""ctypes binding of oracle/_ref/libyvref.so: the reference's own renderer
code (cell/ppu_renderer.cpp, cell/spu/trace_spu.cpp, reaction/trace/trace.cu)
compiled on the host by oracle/build_ref.py.

TEST INFRASTRUCTURE ONLY: the tests use it to pin the oracle (and, through
the fixtures tests/golden/make_ref_golden.py writes, the CUDA path) against
the reference itself.  It exists only where the reference checkout is
present; available() says so.
"""
import ctypes as C
import importlib.util
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


def _builder():
    spec = importlib.util.spec_from_file_location("_ref_build", os.path.join(HERE,
                                                                          "build_ref.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def available():
    """True if the reference library can be built or is built here."""
    return _builder().available()


def lib():
    global _lib
    if _lib is None:
        path = _builder().build()
        if path is None:
            raise RuntimeError("reference checkout not present: oracle/_ref is not built")
        L = C.CDLL(path)
        P, I, U, F = C.c_void_p, C.c_int, C.c_uint32, C.c_float
        sig = {
            "yvref_ray_basis": (I, [P, P, F, I, I, P, P, P]),
            "yvref_ppu_render": (I, [C.c_char_p, P, P, P, F, I, I, I, P, P, P]),
            "yvref_spu_frame": (I, [P, U, U, P, P, P, F, I, I, P, P, P]),
            "yvref_cast_rays": (I, [P, I, I, I, P, P, P, I, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _f32(v):
    return np.ascontiguousarray(np.asarray(v, np.float32).reshape(-1))


def ray_basis(dir_, up, fov, width, height):
    """RendererBase::InitRayDir of the reference: (dir0, du, dv) float32."""
    d0, du, dv = (np.zeros(3, np.float32) for _ in range(3))
    a, b = _f32(dir_), _f32(up)
    st = lib().yvref_ray_basis(a.ctypes.data, b.ctypes.data, float(fov), width, height,
                               d0.ctypes.data, du.ctypes.data, dv.ctypes.data)
    assert st == 0
    return d0, du, dv


def ppu_render(vox_path, pos, dir_, up, fov, width, height, threaded=False):
    """The reference CPU renderer over a .vox file (SVOData::Load): per pixel
    the hit leaf's VoxData (0xFFFFFFFF for a miss), t, and node fetches."""
    n = width * height
    data = np.zeros(n, np.uint32)
    t = np.zeros(n, np.float32)
    f = np.zeros(n, np.uint32)
    p, d, u = _f32(pos), _f32(dir_), _f32(up)
    st = lib().yvref_ppu_render(os.fsencode(vox_path), p.ctypes.data, d.ctypes.data,
                                u.ctypes.data, float(fov), width, height, 1 if threaded else 0,
                                data.ctypes.data, t.ctypes.data,
                                None if threaded else f.ctypes.data)
    if st != 0:
        raise RuntimeError(f"reference render failed: {st}")
    return data.reshape(height, width), t.reshape(height, width), f.reshape(height, width)


def spu_render(nodes_u32, root, pos, dir_, up, fov, width, height):
    """The reference SPU tracer (16x16 blocks, FetchNode node cache) on the
    CPU renderer's camera basis: per pixel VoxData, t, node fetches."""
    nodes = np.ascontiguousarray(nodes_u32, np.uint32).reshape(-1)
    n = width * height
    data = np.zeros(n, np.uint32)
    t = np.zeros(n, np.float32)
    f = np.zeros(n, np.uint32)
    p, d, u = _f32(pos), _f32(dir_), _f32(up)
    st = lib().yvref_spu_frame(nodes.ctypes.data, len(nodes) // 10, root, p.ctypes.data,
                               d.ctypes.data, u.ctypes.data, float(fov), width, height,
                               data.ctypes.data, t.ctypes.data, f.ctypes.data)
    if st != 0:
        raise RuntimeError(f"reference SPU render failed: {st}")
    return data.reshape(height, width), t.reshape(height, width), f.reshape(height, width)


def cast_rays(volume_u8, marks_u8, eye, dirs):
    """castRay of reaction/trace/trace.cu: volume (nz, ny, nx) uint8 over
    [0, 1]^3 in normalized texture coordinates, brick marks (64, 64, 64)
    uint8, rays from `eye` along unit `dirs` (n x 3).  Returns (n, 4) RGBA."""
    vol = np.ascontiguousarray(volume_u8, np.uint8)
    marks = np.ascontiguousarray(marks_u8, np.uint8)
    assert marks.shape == (64, 64, 64)
    dv = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
    out = np.zeros((len(dv), 4), np.float32)
    e = _f32(eye)
    st = lib().yvref_cast_rays(vol.ctypes.data, vol.shape[2], vol.shape[1], vol.shape[0],
                               marks.ctypes.data, e.ctypes.data, dv.ctypes.data, len(dv),
                               out.ctypes.data)
    assert st == 0
    return out
