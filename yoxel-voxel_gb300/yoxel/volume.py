"""Brick volumes in the ntree layout and the differentiable ray-march.

`BrickVolume` wraps the host tree + brick pool (ntree::Node / RangeBuilder /
BrickPool<T>, ntree/ntree/nodes.h, ntree/ntree/ntree.h, ntree/BrickManager.h);
`render_volume` is the multi-camera march (the kernel behind ntree's RunTrace
entry, ntree/ntree_trace.cuh:27); `VolumeMarch` is a torch.autograd.Function
whose backward re-marches every ray in the CUDA adjoint kernel.
"""
import ctypes as C

import numpy as np

from . import _lib as L


def _torch():
    import torch
    return torch


def _stream(stream):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


class BrickVolume:
    """Host brick volume (grid tree + 9^3-lattice brick pool)."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            L.lib.yv_volume_free(h)
            self._h = C.c_void_p(None)

    @classmethod
    def noise(cls, levels=3, offset=0.4, amplitude=1.0, seed=1234):
        h = C.c_void_p()
        L.check(L.lib.yv_volume_gen_noise(C.byref(h), levels, offset, amplitude, seed),
                "yv_volume_gen_noise")
        return cls(h.value)

    @classmethod
    def build_dense(cls, density, levels, rgb=None, stream=None):
        """GPU build of yv_volume_from_dense from a dense CUDA lattice
        ((8*4^levels + 1)^3 float32, x fastest; rgb optional uint8 x 3),
        copied into a host container."""
        _check_lattice(density, levels, rgb)
        h = C.c_void_p()
        L.check(L.lib.yv_volume_build_dense(C.c_void_p(density.data_ptr()),
                                            None if rgb is None else C.c_void_p(rgb.data_ptr()),
                                            levels, _stream(stream), C.byref(h)),
                "yv_volume_build_dense")
        return cls(h.value)

    @classmethod
    def from_dense(cls, levels, density, albedo=None):
        density = np.ascontiguousarray(density, np.float32)
        s = 8 * 4 ** levels + 1
        if density.shape != (s, s, s):
            raise ValueError(f"density must be {(s, s, s)} (z, y, x) lattice")
        a = None
        if albedo is not None:
            albedo = np.ascontiguousarray(albedo, np.uint8)
            if albedo.shape != (s, s, s, 3):
                raise ValueError("albedo must be (S+1)^3 x 3 uint8")
            a = albedo.ctypes.data
        h = C.c_void_p()
        L.check(L.lib.yv_volume_from_dense(C.byref(h), levels, density.ctypes.data, a),
                "yv_volume_from_dense")
        return cls(h.value)

    @property
    def handle(self):
        return self._h

    @property
    def levels(self):
        return int(L.lib.yv_volume_levels(self._h))

    @property
    def size(self):
        """Lattice cells per axis (CalcSceneSize with N = 4, B = 8)."""
        return 8 * 4 ** self.levels

    @property
    def nbricks(self):
        return int(L.lib.yv_volume_brick_count(self._h))

    @property
    def ngrids(self):
        return int(L.lib.yv_volume_grid_count(self._h))

    def _view(self, ptr, ctype, count, shape):
        if count == 0:
            return np.zeros(shape, np.dtype(ctype))
        buf = (ctype * count).from_address(ptr)
        a = np.frombuffer(buf, dtype=np.dtype(ctype)).reshape(shape)
        a.flags.writeable = False
        return a

    @property
    def grids(self):
        return self._view(L.lib.yv_volume_grids(self._h), C.c_uint32, self.ngrids * 64,
                          (self.ngrids, 64))

    @property
    def density(self):
        return self._view(L.lib.yv_volume_density(self._h), C.c_float, self.nbricks * 729,
                          (self.nbricks, 729))

    @property
    def albedo_u8(self):
        return self._view(L.lib.yv_volume_albedo(self._h), C.c_uint8, self.nbricks * 2187,
                          (self.nbricks, 729, 3))

    @property
    def cells(self):
        return self._view(L.lib.yv_volume_brick_cells(self._h), C.c_int32, self.nbricks * 3,
                          (self.nbricks, 3))

    def neighbors(self, upper):
        return self._view(L.lib.yv_volume_neighbors(self._h, 1 if upper else 0), C.c_int32,
                          self.nbricks * 7, (self.nbricks, 7))

    @property
    def occupancy(self):
        return self.nbricks / float(4 ** (3 * self.levels))

    def upload(self, precision=L.YV_PRECISION_F16):
        return VolumeGPU(self, precision)

    def to_torch(self, device="cuda"):
        """Learnable fp32 copy: dict of torch tensors (grids, density (nb,729),
        albedo (nb,729,3) in [0,1], nbr_up, nbr_dn) on `device`."""
        torch = _torch()
        tv = dict(
            levels=self.levels,
            grids=torch.from_numpy(self.grids.astype(np.int32)).to(device),
            density=torch.from_numpy(self.density.copy()).to(device),
            albedo=torch.from_numpy((self.albedo_u8.astype(np.float32) *
                                     np.float32(1.0 / 255.0))).to(device),
            nbr_up=torch.from_numpy(self.neighbors(True).copy()).to(device),
            nbr_dn=torch.from_numpy(self.neighbors(False).copy()).to(device),
        )
        tv["brick_bits"] = brick_bits(torch_desc(tv)) if self.levels <= 4 else None
        return tv


def _check_lattice(density, levels, rgb):
    n = 8 * 4 ** int(levels) + 1
    if not (density.is_cuda and density.is_contiguous() and str(density.dtype) == "torch.float32"
            and density.numel() == n ** 3):
        raise ValueError(f"density must be a contiguous CUDA float32 tensor of {n}^3 values")
    if rgb is not None and not (rgb.is_cuda and rgb.is_contiguous() and
                                str(rgb.dtype) == "torch.uint8" and rgb.numel() == 3 * n ** 3):
        raise ValueError(f"rgb must be a contiguous CUDA uint8 tensor of {n}^3 x 3 values")


class VolumeGPU:
    """Library-owned device copy of a BrickVolume (any YV_PRECISION_* pool)."""

    def __init__(self, vol, precision, handle=None):
        h = C.c_void_p(handle) if handle is not None else C.c_void_p()
        if handle is None:
            L.check(L.lib.yv_volume_upload(vol.handle, precision, C.byref(h)),
                    "yv_volume_upload")
        self._h = h
        self.precision = precision

    @classmethod
    def from_dense(cls, density, levels, precision=L.YV_PRECISION_F16, rgb=None, stream=None):
        """GPU build from a dense CUDA lattice ((8*4^levels + 1)^3 float32, x
        fastest; rgb optional uint8 x 3) straight into a device pool."""
        _check_lattice(density, levels, rgb)
        h = C.c_void_p()
        L.check(L.lib.yv_volume_upload_dense(C.c_void_p(density.data_ptr()),
                                             None if rgb is None else C.c_void_p(rgb.data_ptr()),
                                             levels, precision, _stream(stream), C.byref(h)),
                "yv_volume_upload_dense")
        return cls(None, precision, h.value)

    def rebuild_dense(self, density, levels, rgb=None, stream=None):
        """BrickPool::Update in place: rebuild this device pool from a new
        lattice on `stream`, reusing its device arrays where they fit."""
        _check_lattice(density, levels, rgb)
        L.check(L.lib.yv_volume_rebuild_dense(self._h, C.c_void_p(density.data_ptr()),
                                              None if rgb is None else
                                              C.c_void_p(rgb.data_ptr()), levels,
                                              _stream(stream)), "yv_volume_rebuild_dense")
        return self

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            L.lib.yv_volume_gpu_free(h)
            self._h = C.c_void_p(None)

    def desc(self):
        d = L.VolumeDevice()
        L.check(L.lib.yv_volume_gpu_desc(self._h, C.byref(d)), "yv_volume_gpu_desc")
        return d


def torch_desc(tv, density=None, albedo=None, packed=None):
    """VolumeDevice over torch tensors from BrickVolume.to_torch(): fp32
    density + albedo, or (packed given) the float4 (r, g, b, density) pool
    that pack_volume() builds from them."""
    d = L.VolumeDevice()
    d.grids = tv["grids"].data_ptr()
    d.ngrids = tv["grids"].shape[0]
    d.levels = tv["levels"]
    if packed is not None:
        d.density = None
        d.albedo = packed.data_ptr()
        d.nbricks = packed.shape[0]
        d.precision = L.YV_PRECISION_F32_PACKED
    else:
        density = tv["density"] if density is None else density
        albedo = tv["albedo"] if albedo is None else albedo
        d.density = density.data_ptr()
        d.albedo = albedo.data_ptr()
        d.nbricks = density.shape[0]
        d.precision = L.YV_PRECISION_F32
    d.nbr_up = tv["nbr_up"].data_ptr()
    d.nbr_dn = tv["nbr_dn"].data_ptr()
    bits = tv.get("brick_bits")
    d.brick_bits = None if bits is None else bits.data_ptr()
    return d


def brick_bits(desc, stream=None):
    """The brick bitmap of a volume's tree (int32 CUDA tensor of
    ceil(4^(3 levels) / 32) words: bit (ci & 31) of word ci >> 5 set where
    brick cell ci = (cz nb + cy) nb + cx may hold a brick), from its grids;
    VolumeDevice.brick_bits takes its pointer."""
    torch = _torch()
    words = ((1 << (6 * int(desc.levels))) + 31) // 32
    out = torch.empty(words, dtype=torch.int32, device="cuda")
    L.check(L.lib.yv_volume_brick_bits(C.byref(desc), C.c_void_p(out.data_ptr()),
                                       _stream(stream)), "yv_volume_brick_bits")
    return out


def pack_volume(density, albedo, out=None, stream=None):
    """(nbricks, 729, 4) float32 CUDA tensor of (r, g, b, density) per lattice
    point, from contiguous fp32 density (nbricks, 729) and albedo
    (nbricks, 729, 3): one 16-byte load per trilinear corner in the march."""
    torch = _torch()
    nb = density.shape[0]
    if out is None:
        out = torch.empty((nb, 729, 4), dtype=torch.float32, device=density.device)
    L.check(L.lib.yv_volume_pack(C.c_void_p(density.data_ptr()), C.c_void_p(albedo.data_ptr()),
                                 nb * 729, C.c_void_p(out.data_ptr()), _stream(stream)),
            "yv_volume_pack")
    return out


def cameras(cams):
    """ctypes array of yv_camera from (pos, dir, up, fov_deg) tuples."""
    arr = (L.Camera * len(cams))()
    for i, (p, d, u, f) in enumerate(cams):
        arr[i].pos = L.F3(*[float(v) for v in p])
        arr[i].dir = L.F3(*[float(v) for v in d])
        arr[i].up = L.F3(*[float(v) for v in u])
        arr[i].fov_deg = float(f)
    return arr


def sphere_cameras(n, radius=1.5, fov=60.0, center=(0.5, 0.5, 0.5)):
    """n cameras on a Fibonacci sphere looking at the centre."""
    cams = []
    ga = np.pi * (3.0 - np.sqrt(5.0))
    c = np.asarray(center, np.float64)
    for i in range(n):
        z = 1.0 - 2.0 * (i + 0.5) / n
        r = np.sqrt(max(0.0, 1.0 - z * z))
        d = np.array([np.cos(ga * i) * r, np.sin(ga * i) * r, z])
        pos = c + radius * d
        up = (0, 0, 1) if abs(d[2]) < 0.99 else (0, 1, 0)
        cams.append((pos.astype(np.float32), (-d).astype(np.float32), up, fov))
    return cams


def render_volume(desc, cams, width, height, alpha_scale=1.0, step_vox=0.5, out=None,
                  samples=None, bricks=None, stream=None):
    """Composited RGBA, (ncams, h, w, 4) float32 CUDA tensor."""
    torch = _torch()
    ca = cams if isinstance(cams, C.Array) else cameras(cams)
    n = len(ca)
    if out is None:
        out = torch.empty((n, height, width, 4), dtype=torch.float32, device="cuda")
    mp = L.MarchParams(float(alpha_scale), float(step_vox))
    L.check(L.lib.yv_volume_render(C.byref(desc), ca, n, width, height, C.byref(mp),
                                   C.c_void_p(out.data_ptr()),
                                   None if samples is None else C.c_void_p(samples.data_ptr()),
                                   None if bricks is None else C.c_void_p(bricks.data_ptr()),
                                   _stream(stream)), "yv_volume_render")
    return out


def volume_tile_count(width, height):
    """Warp tiles of one camera's frame in the march's order (8x4-pixel
    tiles in 16x16-pixel squares of 8)."""
    n = C.c_uint32()
    L.check(L.lib.yv_volume_tile_count(int(width), int(height), C.byref(n)),
            "yv_volume_tile_count")
    return n.value


def render_volume_tiles(desc, cams, width, height, tile_begin, tile_end, out,
                        alpha_scale=1.0, step_vox=0.5, samples=None, bricks=None,
                        stream=None):
    """render_volume over warp tiles [tile_begin, tile_end) only (camera-major
    ids; volume_tile_count per camera) into full-frame tensors: the other
    pixels are left as they are (one shard of a frame split across GPUs)."""
    ca = cams if isinstance(cams, C.Array) else cameras(cams)
    mp = L.MarchParams(float(alpha_scale), float(step_vox))
    L.check(L.lib.yv_volume_render_tiles(
        C.byref(desc), ca, len(ca), width, height, C.byref(mp), int(tile_begin), int(tile_end),
        C.c_void_p(out.data_ptr()),
        None if samples is None else C.c_void_p(samples.data_ptr()),
        None if bricks is None else C.c_void_p(bricks.data_ptr()), _stream(stream)),
        "yv_volume_render_tiles")
    return out


def render_volume_rgba8(desc, cams, width, height, alpha_scale=1.0, step_vox=0.5, out=None,
                        stream=None):
    """RGBA8 frames (ntree RunTrace's uchar4 image): (ncams, h, w) int32 CUDA
    tensor, R in the low byte, each channel saturate(v) * 255 truncated."""
    torch = _torch()
    ca = cams if isinstance(cams, C.Array) else cameras(cams)
    n = len(ca)
    if out is None:
        out = torch.empty((n, height, width), dtype=torch.int32, device="cuda")
    mp = L.MarchParams(float(alpha_scale), float(step_vox))
    L.check(L.lib.yv_volume_render_rgba8(C.byref(desc), ca, n, width, height, C.byref(mp),
                                         C.c_void_p(out.data_ptr()), _stream(stream)),
            "yv_volume_render_rgba8")
    return out


def volume_backward(desc, cams, width, height, rgba, grad_rgba, grad_density, grad_albedo,
                    alpha_scale=1.0, step_vox=0.5, fold=True, stream=None):
    ca = cams if isinstance(cams, C.Array) else cameras(cams)
    mp = L.MarchParams(float(alpha_scale), float(step_vox))
    L.check(L.lib.yv_volume_backward(C.byref(desc), ca, len(ca), width, height, C.byref(mp),
                                     C.c_void_p(rgba.data_ptr()),
                                     C.c_void_p(grad_rgba.data_ptr()),
                                     C.c_void_p(grad_density.data_ptr()),
                                     C.c_void_p(grad_albedo.data_ptr()), _stream(stream)),
            "yv_volume_backward")
    if fold:
        L.check(L.lib.yv_volume_fold_aprons(C.byref(desc), C.c_void_p(grad_density.data_ptr()),
                                            C.c_void_p(grad_albedo.data_ptr()),
                                            _stream(stream)), "yv_volume_fold_aprons")


def _make_function():
    torch = _torch()

    class VolumeMarch(torch.autograd.Function):
        """rgba = march(density, albedo); backward re-marches each ray.

        The parameters are packed once per forward into the float4
        (r, g, b, density) pool, which both passes read."""

        @staticmethod
        def forward(ctx, density, albedo, tv, cams, width, height, alpha_scale, step_vox):
            density = density.contiguous()
            albedo = albedo.contiguous()
            packed = pack_volume(density, albedo)
            desc = torch_desc(tv, packed=packed)
            ca = cams if isinstance(cams, C.Array) else cameras(cams)
            rgba = render_volume(desc, ca, width, height, alpha_scale, step_vox)
            ctx.save_for_backward(packed, rgba)
            ctx.meta = (tv, ca, width, height, alpha_scale, step_vox, density.shape, albedo.shape)
            return rgba

        @staticmethod
        def backward(ctx, grad_rgba):
            packed, rgba = ctx.saved_tensors
            tv, ca, width, height, alpha_scale, step_vox, dshape, ashape = ctx.meta
            gd = torch.zeros(dshape, dtype=torch.float32, device=packed.device)
            ga = torch.zeros(ashape, dtype=torch.float32, device=packed.device)
            desc = torch_desc(tv, packed=packed)
            volume_backward(desc, ca, width, height, rgba, grad_rgba.contiguous(), gd, ga,
                            alpha_scale, step_vox)
            return gd, ga, None, None, None, None, None, None

    return VolumeMarch


_VolumeMarch = None


def volume_march(density, albedo, tv, cams, width, height, alpha_scale=1.0, step_vox=0.5):
    """Differentiable multi-camera march (torch.autograd)."""
    global _VolumeMarch
    if _VolumeMarch is None:
        _VolumeMarch = _make_function()
    return _VolumeMarch.apply(density, albedo, tv, cams, width, height, alpha_scale, step_vox)
