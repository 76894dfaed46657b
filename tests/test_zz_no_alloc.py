"""The allocation-free frame entry point, yv_render_svo_noalloc.

It exists for callers that cannot call cudaMalloc (stream capture into a
CUDA graph, real-time loops, hosts whose device memory belongs to another
allocator).  They keep the scene in their own device memory in the reference
VoxNode layout; the frame's only scratch is a static device array shared by
all calls.  Here the caller's buffers are torch CUDA tensors (the caller
allocates; the library does not).  Two calls in a row check that the shared
scratch is cleared between frames: the outputs are pre-filled with garbage
before each call, so a frame that traced nothing would fail the comparison.
Bar: bit-exact with the renderer entry point (yv_render_frame_async), the
same bar as the other SVO parity tests.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import LIGHT, camera_for

pytestmark = pytest.mark.gpu


def _frame_outputs(t):
    from yoxel import _lib as L
    return L.FrameOutputs(*[C.c_void_p(t[k].data_ptr()) for k in
                            ("rgba", "hit", "hit_t", "fetches", "shadow_fetches")])


def test_noalloc_frame_matches_renderer_on_two_calls(yoxel_mod):
    import torch
    from yoxel import _lib as L
    scene = yoxel_mod.SVOScene.spheres(7, 60, 2.0, 12.0, 4321)
    pos, view = camera_for()
    w, h = 160, 120
    r = yoxel_mod.Renderer()
    r.SetScene(scene)
    r.SetViewPos(pos)
    r.SetViewDir(view)
    r.SetResolution(w, h)
    r.SetFOV(60.0)
    r.SetLight(LIGHT, 0.15, 0.85, True)
    ref = r.render_outputs()
    assert ref["stats"]["hits"] > 0

    # the caller's own device copy of the reference pool and attributes
    d_nodes = torch.from_numpy(scene.nodes_u32.copy().view(np.int32)).cuda()
    d_attrs = torch.from_numpy(scene.attrs_u8.copy()).cuda()
    cam = L.Camera(L.F3(*pos), L.F3(*view), L.F3(0, 0, 1), 60.0)
    light = L.Light(L.F3(*LIGHT), 0.15, 0.85, 1)
    stream = torch.cuda.current_stream()
    for call in range(2):
        out = dict(rgba=torch.full((h, w), -7, dtype=torch.int32, device="cuda"),
                   hit=torch.full((h, w), -7, dtype=torch.int32, device="cuda"),
                   hit_t=torch.full((h, w), -7.0, dtype=torch.float32, device="cuda"),
                   fetches=torch.full((h, w), -7, dtype=torch.int32, device="cuda"),
                   shadow_fetches=torch.full((h, w), -7, dtype=torch.int32, device="cuda"))
        fo = _frame_outputs(out)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        st = L.lib.yv_render_svo_noalloc(C.c_void_p(d_nodes.data_ptr()), scene.node_count,
                                         scene.root, C.c_void_p(d_attrs.data_ptr()),
                                         scene.attr_count, C.byref(cam), C.byref(light), w, h,
                                         C.byref(fo), C.c_void_p(stream.cuda_stream))
        assert st == L.YV_OK, L.status_string(st)
        torch.cuda.synchronize()
        if call == 1:
            # the warm call takes no device memory
            assert torch.cuda.mem_get_info()[0] == free_before
        for k in ("rgba", "hit", "fetches", "shadow_fetches"):
            assert torch.equal(out[k], ref[k]), f"call {call}: {k} differs"
        assert torch.equal(out["hit_t"].view(torch.int32), ref["hit_t"].view(torch.int32))


def test_noalloc_rejects_frames_beyond_the_scratch_range(yoxel_mod):
    from yoxel import _lib as L
    cam = L.Camera(L.F3(2, 2, 2), L.F3(-1, -1, -1), L.F3(0, 0, 1), 60.0)
    light = L.Light(L.F3(0, 0, 1), 0.15, 0.85, 0)
    fo = L.FrameOutputs()
    st = L.lib.yv_render_svo_noalloc(None, 0, 0x80000000, None, 0, C.byref(cam),
                                     C.byref(light), 65536, 65536, C.byref(fo), None)
    assert st == L.YV_ERR_INVALID_ARG
    assert "2^31" in L.last_error()
