"""Batched persistent render (yv_batch_* of the C ABI).

Many scenes and cameras of uneven depth and resolution - SVO first-hit
frames and brick-volume composites - traced in one persistent launch fed by a
global ray queue, optionally replayed from a captured CUDA graph.
"""
import ctypes as C

from . import _lib as L
from .volume import cameras


def _stream(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


class Batch:
    def __init__(self):
        h = C.c_void_p()
        L.check(L.lib.yv_batch_create(C.byref(h)), "yv_batch_create")
        self._h = h
        self._keep = []  # renderers / tensors the batch points into

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            L.lib.yv_batch_destroy(h)
            self._h = C.c_void_p(None)

    def clear(self):
        L.check(L.lib.yv_batch_clear(self._h), "yv_batch_clear")
        self._keep = []

    def add_svo(self, renderer, rgba, hit=None, hit_t=None, fetches=None, shadow_fetches=None):
        """Snapshot of `renderer` (scene, camera, light, resolution) into the
        (h, w) int32 CUDA tensor `rgba`, and optionally the per-pixel hit ids
        ((node << 3) | child), hit t, fetch and shadow-fetch counts, as a
        per-scene frame reports them."""
        if hit is None and hit_t is None and fetches is None and shadow_fetches is None:
            L.check(L.lib.yv_batch_add_svo(self._h, renderer.handle,
                                           C.c_void_p(rgba.data_ptr())), "yv_batch_add_svo")
        else:
            def ptr(t):
                return None if t is None else C.c_void_p(t.data_ptr())
            o = L.FrameOutputs(ptr(rgba), ptr(hit), ptr(hit_t), ptr(fetches),
                               ptr(shadow_fetches), None)
            L.check(L.lib.yv_batch_add_svo_outputs(self._h, renderer.handle, C.byref(o)),
                    "yv_batch_add_svo_outputs")
        self._keep += [renderer, rgba, hit, hit_t, fetches, shadow_fetches]

    def add_volume(self, desc, cam, width, height, rgba, alpha_scale=1.0, step_vox=0.5):
        """One camera (pos, dir, up, fov) of a device volume into the
        (h, w, 4) float32 CUDA tensor `rgba`."""
        ca = cameras([cam])
        mp = L.MarchParams(float(alpha_scale), float(step_vox))
        L.check(L.lib.yv_batch_add_volume(self._h, C.byref(desc), ca, width, height,
                                          C.byref(mp), C.c_void_p(rgba.data_ptr())),
                "yv_batch_add_volume")
        self._keep += [desc, rgba]

    def set_launch_config(self, block_threads=0, blocks_per_sm=0):
        cfg = L.LaunchConfig(block_threads, blocks_per_sm, -1, 0)
        L.check(L.lib.yv_batch_set_launch_config(self._h, C.byref(cfg)), "batch config")

    def render(self, graph=True, stream=None):
        L.check(L.lib.yv_batch_render(self._h, 1 if graph else 0, _stream(stream)),
                "yv_batch_render")

    def render_separate(self, stream=None):
        L.check(L.lib.yv_batch_render_separate(self._h, _stream(stream)),
                "yv_batch_render_separate")

    def info(self):
        n, r = C.c_uint32(), C.c_uint64()
        L.check(L.lib.yv_batch_info(self._h, C.byref(n), C.byref(r)), "yv_batch_info")
        return n.value, r.value
