"""Editable SVO with incremental device sync (DynamicSVO of
reaction/report/main.tex:67-71; SVORenderer::UpdateSVO,
demo/SVORenderer.cpp:39-53; CountChangedPages / CountTransfrerSize,
qtview.py:69-73) over the C ABI.  Frames are traced from the device mirror
by the caller-layout kernel (yv_render_svo_noalloc), so hit ids are the
pool's own node ids."""
import ctypes as C

import numpy as np

from . import _lib as L
from .svo import ATTR_DTYPE, NODE_DTYPE


def _stream(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


class DynamicSVO:
    def __init__(self, node_capacity, attr_capacity):
        h = C.c_void_p()
        L.check(L.lib.yv_svo_dynamic_create(int(node_capacity), int(attr_capacity),
                                            C.byref(h)), "yv_svo_dynamic_create")
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            L.lib.yv_svo_dynamic_destroy(h)
            self._h = C.c_void_p(None)

    def load(self, scene):
        L.check(L.lib.yv_svo_dynamic_load(self._h, scene.handle), "yv_svo_dynamic_load")

    def set_voxel(self, depth, x, y, z, rgb=None, normal=(0, 0, 127)):
        """Sets the voxel to a leaf of colour rgb (None: clears it)."""
        a = None
        if rgb is not None:
            at = np.zeros(1, ATTR_DTYPE)
            at["rgb"][0] = [rgb[0], rgb[1], rgb[2], 255]
            at["n"][0] = [normal[0], normal[1], normal[2], 0]
            a = at.ctypes.data
        L.check(L.lib.yv_svo_dynamic_set_voxel(self._h, depth, x, y, z, a),
                "yv_svo_dynamic_set_voxel")

    def changed_pages(self):
        return int(L.lib.yv_svo_dynamic_changed_pages(self._h))

    def transfer_bytes(self):
        return int(L.lib.yv_svo_dynamic_transfer_bytes(self._h))

    def sync(self, stream=None):
        L.check(L.lib.yv_svo_dynamic_sync(self._h, _stream(stream)), "yv_svo_dynamic_sync")

    def _device(self):
        n, a = C.c_void_p(), C.c_void_p()
        cnt, root, na = C.c_uint32(), C.c_uint32(), C.c_uint32()
        L.check(L.lib.yv_svo_dynamic_device(self._h, C.byref(n), C.byref(cnt), C.byref(root),
                                            C.byref(a), C.byref(na)), "yv_svo_dynamic_device")
        return n, cnt.value, root.value, a, na.value

    def _host(self):
        cnt, root, na = C.c_uint32(), C.c_uint32(), C.c_uint32()
        L.check(L.lib.yv_svo_dynamic_host_info(self._h, C.byref(cnt), C.byref(root),
                                               C.byref(na)), "yv_svo_dynamic_host_info")
        return cnt.value, root.value, na.value

    @property
    def root(self):
        """Root of the host pool (the device mirror takes it at the next sync)."""
        return self._host()[1]

    def host_arrays(self):
        """Copies of the host pool: (nodes, root, attrs) structured arrays."""
        cnt, root, na = self._host()
        nodes = np.frombuffer((C.c_uint8 * (cnt * 40)).from_address(
            L.lib.yv_svo_dynamic_host_nodes(self._h)), dtype=NODE_DTYPE).copy()
        attrs = np.frombuffer((C.c_uint8 * (na * 8)).from_address(
            L.lib.yv_svo_dynamic_host_attrs(self._h)), dtype=ATTR_DTYPE).copy()
        return nodes, root, attrs

    def download(self):
        """The device mirror copied back: (nodes, attrs), sized like the host
        pool (equal to it after a sync)."""
        cnt, _, na = self._host()
        nodes = np.zeros(cnt, NODE_DTYPE)
        attrs = np.zeros(na, ATTR_DTYPE)
        L.check(L.lib.yv_svo_dynamic_download(self._h, nodes.ctypes.data, attrs.ctypes.data),
                "yv_svo_dynamic_download")
        return nodes, attrs

    def render(self, pos, view, up, fov, width, height, light, ambient=0.15, diffuse=0.85,
               shadows=False, stream=None):
        """One frame from the device mirror: dict of CUDA tensors (rgba, hit,
        hit_t, fetches, shadow_fetches).

        The frame runs through the allocation-free entry point, whose scratch
        (ray-queue counter, status word, hit counters) is one static device
        array shared by every such frame: frames in flight at the same time,
        on different streams or host threads, race on it and come out wrong.
        Serialise them, or bind the scene to a Renderer
        (Renderer.SetSceneDynamic), which has counters of its own.  The
        frame's device status is read with `status()`."""
        import torch
        n, cnt, root, a, na = self._device()
        cam = L.Camera(L.F3(*[float(v) for v in pos]), L.F3(*[float(v) for v in view]),
                       L.F3(*[float(v) for v in up]), float(fov))
        lt = L.Light(L.F3(*[float(v) for v in light]), float(ambient), float(diffuse),
                     1 if shadows else 0)
        dev = torch.device("cuda", torch.cuda.current_device())
        out = {k: torch.empty((height, width), dtype=torch.int32 if k != "hit_t" else
                              torch.float32, device=dev)
               for k in ("rgba", "hit", "hit_t", "fetches", "shadow_fetches")}
        o = L.FrameOutputs(*[C.c_void_p(out[k].data_ptr()) for k in
                             ("rgba", "hit", "hit_t", "fetches", "shadow_fetches")])
        L.check(L.lib.yv_render_svo_noalloc(n, cnt, root, a, na, C.byref(cam), C.byref(lt),
                                            width, height, C.byref(o), _stream(stream)),
                "yv_render_svo_noalloc")
        return out

    @staticmethod
    def status(stream=None):
        """Device status of the last frame rendered by `render` (waits for
        `stream`): raises YvError on YV_ERR_BAD_POOL or YV_ERR_ITERATION_CAP,
        else returns the raw status bits (0)."""
        bits = C.c_uint32()
        L.check(L.lib.yv_render_svo_noalloc_status(_stream(stream), C.byref(bits)),
                "yv_render_svo_noalloc_status")
        return bits.value
