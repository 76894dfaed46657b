"""Host-side SVO scenes (SVOData, cell/svodata.h:22-55).

An `SVOScene` owns a yv_svo_host container of the C library and exposes its
40-byte VoxNode records and 8-byte leaf attributes as numpy views.
"""
import ctypes as C

import numpy as np

from . import _lib as L

NODE_DTYPE = np.dtype([("flags", "<u4"), ("data", "<u4"), ("child", "<u4", (8,))])
ATTR_DTYPE = np.dtype([("rgb", "u1", (4,)), ("n", "i1", (4,))])


class SVOScene:
    """A sparse voxel octree: `nodes` (VoxNode records), `attrs` (leaf colour +
    quantised normal), `root` and `depth`."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            L.lib.yv_svo_free(h)
            self._h = C.c_void_p(None)

    # ---- constructors -------------------------------------------------
    @classmethod
    def spheres(cls, depth=8, n_spheres=200, rmin=4.0, rmax=24.0, seed=1234):
        """Seeded sphere-union scene (the 200-spheres-in-256^3 workload)."""
        h = C.c_void_p()
        L.check(L.lib.yv_svo_gen_spheres(C.byref(h), depth, n_spheres, rmin, rmax, seed),
                "yv_svo_gen_spheres")
        return cls(h.value)

    @classmethod
    def terrain(cls, depth=11, n_cubes=10000, cube_min=2, cube_max=16, seed=1234):
        """Seeded value-noise terrain + floating cubes (the 2048^3 workload)."""
        h = C.c_void_p()
        L.check(L.lib.yv_svo_gen_terrain(C.byref(h), depth, n_cubes, cube_min, cube_max,
                                         seed), "yv_svo_gen_terrain")
        return cls(h.value)

    @classmethod
    def from_arrays(cls, nodes, root, attrs):
        nodes = np.ascontiguousarray(nodes, dtype=NODE_DTYPE)
        attrs = np.ascontiguousarray(attrs, dtype=ATTR_DTYPE)
        h = C.c_void_p()
        L.check(L.lib.yv_svo_from_arrays(C.byref(h), nodes.ctypes.data, len(nodes), root,
                                         attrs.ctypes.data, len(attrs)),
                "yv_svo_from_arrays")
        return cls(h.value)

    @classmethod
    def from_packed(cls, nodes, root):
        """A pool as the reference's SVOData holds it in memory: leaves and
        node data carry the packed 16-bit colour + 16-bit normal VoxData,
        decoded into leaf attributes (node ids kept)."""
        nodes = np.ascontiguousarray(nodes, dtype=NODE_DTYPE)
        h = C.c_void_p()
        L.check(L.lib.yv_svo_from_packed(C.byref(h), nodes.ctypes.data, len(nodes), root),
                "yv_svo_from_packed")
        return cls(h.value)

    @classmethod
    def build_dense(cls, density, depth, iso=0.0, rgb=None, stream=None):
        """GPU build from a dense CUDA float32 grid of (2^depth)^3 values
        (x fastest, e.g. a (G, G, G) tensor indexed [z, y, x]); rgb: CUDA
        uint8 (G, G, G, 3) or None (white).  Solid = density > iso; surface
        voxels become leaves; the canonical pool is copied to the host."""
        _check_dense(density, depth, rgb)
        h = C.c_void_p()
        L.check(L.lib.yv_svo_build_dense(C.c_void_p(density.data_ptr()),
                                         None if rgb is None else C.c_void_p(rgb.data_ptr()),
                                         depth, float(iso), _stream(stream), C.byref(h)),
                "yv_svo_build_dense")
        return cls(h.value)

    @classmethod
    def load(cls, path):
        """SVOData::Load of a .vox file."""
        h = C.c_void_p()
        L.check(L.lib.yv_svo_load_vox(C.byref(h), str(path).encode()), "yv_svo_load_vox")
        return cls(h.value)

    def save(self, path):
        L.check(L.lib.yv_svo_save_vox(self._h, str(path).encode()), "yv_svo_save_vox")

    def build_lod(self):
        """Level-of-detail data (reaction/report/main.tex:61): every node's
        `data` indexes a new attribute holding the mean colour and normal
        of its subtree's leaves.  Returns self."""
        L.check(L.lib.yv_svo_build_lod(self._h), "yv_svo_build_lod")
        return self

    @property
    def has_lod(self):
        return bool(L.lib.yv_svo_has_lod(self._h))

    # ---- views --------------------------------------------------------
    @property
    def handle(self):
        return self._h

    @property
    def root(self):
        return int(L.lib.yv_svo_root(self._h))

    @property
    def depth(self):
        return int(L.lib.yv_svo_depth(self._h))

    @property
    def node_count(self):
        return int(L.lib.yv_svo_node_count(self._h))

    @property
    def attr_count(self):
        return int(L.lib.yv_svo_attr_count(self._h))

    @property
    def nodes(self):
        """(count,) structured view of the VoxNode records (no copy)."""
        n = self.node_count
        if n == 0:
            return np.zeros(0, NODE_DTYPE)
        buf = (C.c_uint8 * (n * 40)).from_address(L.lib.yv_svo_nodes(self._h))
        a = np.frombuffer(buf, dtype=NODE_DTYPE)
        a.flags.writeable = False
        return a

    @property
    def nodes_u32(self):
        """(count*10,) uint32 view of the node pool."""
        return self.nodes.view(np.uint32).reshape(-1)

    @property
    def attrs(self):
        n = self.attr_count
        if n == 0:
            return np.zeros(0, ATTR_DTYPE)
        buf = (C.c_uint8 * (n * 8)).from_address(L.lib.yv_svo_attrs(self._h))
        a = np.frombuffer(buf, dtype=ATTR_DTYPE)
        a.flags.writeable = False
        return a

    @property
    def attrs_u8(self):
        return self.attrs.view(np.uint8).reshape(-1)

    def validate(self):
        return L.lib.yv_svo_validate(L.lib.yv_svo_nodes(self._h), self.node_count, self.root,
                                     self.attr_count)

    def nbytes(self):
        return self.node_count * 40 + self.attr_count * 8


def _check_dense(density, depth, rgb):
    G = 1 << int(depth)
    if not (density.is_cuda and density.is_contiguous() and str(density.dtype) == "torch.float32"
            and density.numel() == G ** 3):
        raise ValueError(f"density must be a contiguous CUDA float32 tensor of {G}^3 values")
    if rgb is not None and not (rgb.is_cuda and rgb.is_contiguous() and
                                str(rgb.dtype) == "torch.uint8" and rgb.numel() == 3 * G ** 3):
        raise ValueError(f"rgb must be a contiguous CUDA uint8 tensor of {G}^3 x 3 values")


def _stream(stream):
    if stream is None:
        import torch
        stream = torch.cuda.current_stream()
    return C.c_void_p(stream.cuda_stream)
