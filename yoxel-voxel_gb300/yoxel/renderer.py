"""SVO renderers over the C ABI.

`Renderer` mirrors ISVORenderer (cell/svorenderer.h:5-24): SetScene,
SetViewPos/Dir/Up, SetResolution/GetResolution, SetFOV, RenderFrame (None
without a scene, as RenderFrame returns NULL, cell/ppu_renderer.cpp:78-79).

`CudaRenderer` mirrors the Python driver trace_cuda.CudaRenderer
(trace_cuda.py:17-120): updateScene, setLightPos, getViewSize, render,
getImage.  Frames live in CUDA memory as torch tensors; torch provides the
device buffers and streams only, all computation is in libyoxel.so.
"""
import ctypes as C
import time

import numpy as np

from . import _lib as L
from .svo import SVOScene


def _f3(v):
    v = [float(x) for x in v]
    if len(v) != 3:
        raise ValueError("expected 3 components")
    return L.F3(*v)


def _torch():
    import torch
    return torch


def _stream_ptr(stream):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


class Renderer:
    """ISVORenderer on the GPU."""

    def __init__(self):
        h = C.c_void_p()
        L.check(L.lib.yv_renderer_create(C.byref(h)), "yv_renderer_create")
        self._h = h
        self._scene = None
        self._fov = 70.0  # RendererBase default (cell/renderer_base.h:25)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            L.lib.yv_renderer_destroy(h)
            self._h = C.c_void_p(None)

    @property
    def handle(self):
        return self._h

    # ---- ISVORenderer ---------------------------------------------------
    def SetScene(self, scene: SVOScene):
        L.check(L.lib.yv_set_scene_host(self._h, scene.handle), "SetScene")
        self._scene = scene

    def SetSceneDense(self, density, depth, iso=0.0, rgb=None, stream=None):
        """Builds the scene on the GPU from a dense CUDA float32 grid (see
        SVOScene.build_dense) straight into the renderer's device layout."""
        from .svo import _check_dense
        _check_dense(density, depth, rgb)
        L.check(L.lib.yv_set_scene_dense(self._h, C.c_void_p(density.data_ptr()),
                                         None if rgb is None else C.c_void_p(rgb.data_ptr()),
                                         depth, float(iso), _stream_ptr(stream)),
                "SetSceneDense")
        self._scene = None

    def SetSceneDynamic(self, dyn):
        """SVORenderer::SetScene(DynamicSVO*): trace an editable scene's device
        mirror in place (as of its last sync); the renderer keeps a
        reference to it."""
        L.check(L.lib.yv_set_scene_dynamic(self._h, dyn._h), "SetSceneDynamic")
        self._scene = dyn

    def SetSceneArrays(self, nodes, root, attrs):
        from .svo import ATTR_DTYPE, NODE_DTYPE
        nodes = np.ascontiguousarray(nodes, dtype=NODE_DTYPE)
        attrs = np.ascontiguousarray(attrs, dtype=ATTR_DTYPE)
        L.check(L.lib.yv_set_scene_svo(self._h, nodes.ctypes.data, len(nodes), root,
                                       attrs.ctypes.data, len(attrs)), "SetSceneArrays")
        self._scene = (nodes, attrs)

    def SetSceneSVOPacked(self, nodes, root):
        """ISVORenderer::SetScene for a pool in the reference's packed leaf
        format (SVOScene.from_packed), without a separate attribute array."""
        from .svo import NODE_DTYPE
        nodes = np.ascontiguousarray(nodes, dtype=NODE_DTYPE)
        L.check(L.lib.yv_set_scene_svo_packed(self._h, nodes.ctypes.data, len(nodes), root),
                "SetSceneSVOPacked")
        self._scene = (nodes,)

    def SetViewPos(self, pos):
        L.check(L.lib.yv_set_view_pos(self._h, _f3(pos)), "SetViewPos")

    def SetViewDir(self, d):
        L.check(L.lib.yv_set_view_dir(self._h, _f3(d)), "SetViewDir")

    def SetViewUp(self, up):
        L.check(L.lib.yv_set_view_up(self._h, _f3(up)), "SetViewUp")

    def SetResolution(self, width, height):
        L.check(L.lib.yv_set_resolution(self._h, int(width), int(height)), "SetResolution")

    def GetResolution(self):
        w, h = C.c_int(), C.c_int()
        L.check(L.lib.yv_get_resolution(self._h, C.byref(w), C.byref(h)), "GetResolution")
        return (w.value, h.value)

    def SetFOV(self, fov):
        L.check(L.lib.yv_set_fov(self._h, float(fov)), "SetFOV")
        self._fov = float(np.float32(fov))

    def GetFOV(self):
        f = C.c_float()
        L.check(L.lib.yv_get_fov(self._h, C.byref(f)), "GetFOV")
        return f.value

    def SetDetailCoef(self, coef):
        """SVORenderer::SetDetailCoef: level-of-detail cut-off (0 = exact
        leaves; needs a scene with level-of-detail data)."""
        L.check(L.lib.yv_set_detail_coef(self._h, float(coef)), "SetDetailCoef")

    def GetDetailCoef(self):
        c = C.c_float()
        L.check(L.lib.yv_get_detail_coef(self._h, C.byref(c)), "GetDetailCoef")
        return c.value

    def SetFrameBudget(self, microseconds):
        """Frame time budget of the persistent ray queue (0 = none): past it
        the kernel takes no new rays, unwritten pixels keep their contents
        and the frame status is YV_ERR_TIMEOUT."""
        L.check(L.lib.yv_set_frame_budget(self._h, int(microseconds)), "SetFrameBudget")

    def GetFrameBudget(self):
        v = C.c_uint32()
        L.check(L.lib.yv_get_frame_budget(self._h, C.byref(v)), "GetFrameBudget")
        return v.value

    def lod_coef(self):
        """The per-frame cut-off coefficient detail * radians(fov / 2) /
        width, as the frame uses it (float32)."""
        import math
        w, _ = self.GetResolution()
        f = C.c_float()
        L.check(L.lib.yv_get_detail_coef(self._h, C.byref(f)), "GetDetailCoef")
        return float(np.float32(float(f.value) * float(np.float32(self._fov)) *
                                (math.pi / 360.0) / float(w)))

    def SetLight(self, direction, ambient=0.15, diffuse=0.85, shadows=False):
        lt = L.Light(_f3(direction), float(ambient), float(diffuse), 1 if shadows else 0)
        L.check(L.lib.yv_set_light(self._h, C.byref(lt)), "SetLight")

    def SetLaunchConfig(self, block_threads=0, blocks_per_sm=0, smem_nodes=-1, tile_rays=0):
        cfg = L.LaunchConfig(block_threads, blocks_per_sm, smem_nodes, tile_rays)
        L.check(L.lib.yv_set_launch_config(self._h, C.byref(cfg)), "SetLaunchConfig")

    def GetLaunchConfig(self):
        cfg = L.LaunchConfig()
        L.check(L.lib.yv_get_launch_config(self._h, C.byref(cfg)), "GetLaunchConfig")
        return dict(block_threads=cfg.block_threads, blocks_per_sm=cfg.blocks_per_sm,
                    smem_nodes=cfg.smem_nodes, tile_rays=cfg.tile_rays)

    def RenderFrame(self):
        """Synchronous frame into host memory: (h, w, 4) uint8 RGBA, or None
        when no scene is set."""
        w, h = self.GetResolution()
        out = np.empty((h, w), np.uint32)
        st = L.lib.yv_render_frame(self._h, out.ctypes.data, None, None)
        if st == L.YV_ERR_NO_SCENE:
            return None
        L.check(st, "RenderFrame")
        return out.view(np.uint8).reshape(h, w, 4)

    # ---- device-side API ----------------------------------------------------
    def ray_basis(self):
        d0, du, dv = L.F3(), L.F3(), L.F3()
        L.check(L.lib.yv_get_ray_basis(self._h, d0, du, dv), "yv_get_ray_basis")
        return np.array(d0, np.float32), np.array(du, np.float32), np.array(dv, np.float32)

    def render_async(self, rgba=None, hit=None, hit_t=None, fetches=None,
                     shadow_fetches=None, normal=None, stream=None):
        """Enqueues a frame into caller-owned CUDA tensors (each optional;
        normal is (h, w, 3) float32)."""
        def ptr(t):
            return None if t is None else C.c_void_p(t.data_ptr())
        o = L.FrameOutputs(ptr(rgba), ptr(hit), ptr(hit_t), ptr(fetches), ptr(shadow_fetches),
                           ptr(normal))
        L.check(L.lib.yv_render_frame_async(self._h, C.byref(o), _stream_ptr(stream)),
                "yv_render_frame_async")

    def tile_count(self):
        """(tiles_x, tiles_y) of the frame's 8x4-pixel tiles."""
        tx, ty = C.c_uint32(), C.c_uint32()
        L.check(L.lib.yv_get_tile_count(self._h, C.byref(tx), C.byref(ty)), "yv_get_tile_count")
        return tx.value, ty.value

    def render_tiles(self, tile_begin, tile_end, rgba=None, hit=None, hit_t=None, fetches=None,
                     shadow_fetches=None, normal=None, stream=None):
        """Enqueues tiles [tile_begin, tile_end) of the frame (8x4-pixel
        tiles, row-major) into full-frame CUDA tensors; pixels outside the
        range are left as they are (the work split of the reference's
        threaded renderer, cell/ppu_renderer.cpp:121-144)."""
        def ptr(t):
            return None if t is None else C.c_void_p(t.data_ptr())
        o = L.FrameOutputs(ptr(rgba), ptr(hit), ptr(hit_t), ptr(fetches), ptr(shadow_fetches),
                           ptr(normal))
        L.check(L.lib.yv_render_frame_tiles(self._h, int(tile_begin), int(tile_end), C.byref(o),
                                            _stream_ptr(stream)), "yv_render_frame_tiles")

    def frame_stats(self, check=True):
        s = L.FrameStats()
        st = L.lib.yv_renderer_frame_stats(self._h, C.byref(s))
        if check:
            L.check(st, "frame")
        return dict(primary_rays=s.primary_rays, hits=s.hits, shadow_rays=s.shadow_rays,
                    shadowed=s.shadowed, status=s.status, launches=s.launches)

    def render_outputs(self, stream=None, stats=True):
        """Renders into fresh CUDA tensors and returns them with the counters:
        rgba (h,w) int32, hit (h,w) int32, hit_t (h,w) float32, fetches and
        shadow_fetches (h,w) int32."""
        torch = _torch()
        w, h = self.GetResolution()
        dev = torch.device("cuda", torch.cuda.current_device())
        out = dict(
            rgba=torch.empty((h, w), dtype=torch.int32, device=dev),
            hit=torch.empty((h, w), dtype=torch.int32, device=dev),
            hit_t=torch.empty((h, w), dtype=torch.float32, device=dev),
            fetches=torch.empty((h, w), dtype=torch.int32, device=dev),
            shadow_fetches=torch.empty((h, w), dtype=torch.int32, device=dev),
        )
        self.render_async(stream=stream, **out)
        if stats:
            out["stats"] = self.frame_stats()
        return out

    def device_scene_info(self):
        n, b = C.c_uint64(), C.c_uint64()
        L.check(L.lib.yv_get_device_scene_info(self._h, C.byref(n), C.byref(b)),
                "yv_get_device_scene_info")
        return n.value, b.value

    # ---- screen-space normals + point lights (SVORenderer::Render) ----------
    def ssna_params(self):
        """The reference's SSNA defaults (5 blur passes, voxel 1/2048,
        ambient 0.1, specular exponent 10, a white light at the eye) as a
        mutable L.SsnaParams."""
        p = L.SsnaParams()
        L.check(L.lib.yv_ssna_defaults(self._h, C.byref(p)), "yv_ssna_defaults")
        return p

    @staticmethod
    def set_point_light(params, i, pos, diffuse=(0.7, 0.7, 0.7), specular=(0.3, 0.3, 0.3),
                        attenuation=(1.0, 0.0, 0.5), enabled=True):
        """SVORenderer::SetLigth (demo/SVORenderer.h:34) on a params block."""
        if not 0 <= i < L.YV_SSNA_MAX_LIGHTS:
            raise ValueError("light index out of range")
        lp = params.lights[i]
        lp.pos[:] = [float(v) for v in pos]
        lp.diffuse[:] = [float(v) for v in diffuse]
        lp.specular[:] = [float(v) for v in specular]
        lp.attenuation[:] = [float(v) for v in attenuation]
        lp.enabled = 1 if enabled else 0

    def render_ssna(self, params=None, rgba=None, depth=None, normals=None, stream=None):
        """Enqueues an SSNA frame into CUDA tensors: rgba (h, w) int32
        (allocated when None), optional depth (h, w) float32 and normals
        (h, w, 3) float32.  Returns rgba."""
        torch = _torch()
        w, h = self.GetResolution()
        if params is None:
            params = self.ssna_params()
        if rgba is None:
            rgba = torch.empty((h, w), dtype=torch.int32,
                               device=torch.device("cuda", torch.cuda.current_device()))
        for t, shape in ((rgba, (h, w)), (depth, (h, w)), (normals, (h, w, 3))):
            if t is not None and (tuple(t.shape) != shape or not t.is_cuda
                                  or not t.is_contiguous() or t.element_size() != 4):
                raise ValueError("render_ssna outputs must be contiguous 4-byte CUDA tensors "
                                 "of shape %s" % (shape,))

        def ptr(t):
            return None if t is None else C.c_void_p(t.data_ptr())
        L.check(L.lib.yv_render_ssna(self._h, C.byref(params), ptr(rgba), ptr(depth),
                                     ptr(normals), _stream_ptr(stream)), "yv_render_ssna")
        return rgba

    def trace_dump(self):
        """DumpTraceData into arrays: dist (h, w) float32, color (h, w, 4)
        uint8, normal (h, w, 3) float32 (zero for misses)."""
        w, h = self.GetResolution()
        dist = np.empty((h, w), np.float32)
        color = np.empty((h, w), np.uint32)
        normal = np.empty((h, w, 3), np.float32)
        L.check(L.lib.yv_renderer_trace_dump(self._h, dist.ctypes.data, color.ctypes.data,
                                             normal.ctypes.data), "yv_renderer_trace_dump")
        return dist, color.view(np.uint8).reshape(h, w, 4), normal

    def DumpTraceData(self, fnbase):
        """SVORenderer::DumpTraceData (demo/SVORenderer.cpp:158-186): writes
        <fnbase>_<w>x<h>.dist (float32), .color (Color32) and .normal (3
        float32) per pixel, row-major."""
        w, h = self.GetResolution()
        dist, color, normal = self.trace_dump()
        base = "%s_%dx%d" % (fnbase, w, h)
        dist.tofile(base + ".dist")
        color.tofile(base + ".color")
        normal.tofile(base + ".normal")
        return base


class CudaRenderer:
    """trace_cuda.CudaRenderer (trace_cuda.py:17-120) on libyoxel."""

    def __init__(self, res=(640, 480)):
        self.resx, self.resy = int(res[0]), int(res[1])
        self._r = Renderer()
        self._r.SetResolution(self.resx, self.resy)
        self._r.SetFOV(70.0)
        self.detailCoef = 10.0
        self._img = None
        self.setLightPos((0.5, 0.5, 1))

    def updateScene(self, scene):
        self._r.SetScene(scene)

    def setLightPos(self, pos):
        """Directional light toward `pos` seen from the scene centre."""
        self.lightPos = tuple(float(v) for v in pos)
        d = np.array(self.lightPos, np.float64) - 0.5
        n = np.linalg.norm(d)
        d = d / n if n > 0 else np.array([0.0, 0.0, 1.0])
        self._r.SetLight(d)

    def getViewSize(self):
        return (self.resx, self.resy)

    def render(self, eyePos, viewDir, first=False):
        torch = _torch()
        self._r.SetViewPos(eyePos)
        self._r.SetViewDir(viewDir)
        # trace_cuda.py:93 passes radians(1) / detailCoef as the cut-off
        # angle; as the renderer's coefficient of radians(fov / 2) / width:
        import math
        if self.detailCoef > 0:
            self._r.SetDetailCoef(math.radians(1.0) / self.detailCoef * self.resx /
                                  math.radians(self._r.GetFOV() / 2))
        else:
            self._r.SetDetailCoef(0.0)
        if self._img is None:
            self._img = torch.empty((self.resy, self.resx), dtype=torch.int32, device="cuda")
        t0 = time.perf_counter()
        self._r.render_async(rgba=self._img)
        st = self._r.frame_stats()
        dt = time.perf_counter() - t0
        return ("gpu time: %.2f ms\n" % (dt * 1000) +
                "hits: %d of %d\n" % (st["hits"], st["primary_rays"]) +
                "detailCoef: %f\n" % self.detailCoef)

    def getImage(self):
        a = self._img.cpu().numpy().view(np.uint8).reshape(self.resy, self.resx, 4)
        return a[..., :3]
