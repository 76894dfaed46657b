"""Device status of caller-held pools.

A pool the library did not build (the caller's device VoxNode array of the
allocation-free frame, or an editable scene's mirror) is traversed with
range, depth and fetch checks.  A malformed pool - corrupted on the host
here, never on the device - must end in a status code, not a fault: a child
index past the pool is caught before any load (YV_ERR_BAD_POOL), a cycle by
the 16-level depth cap (YV_ERR_ITERATION_CAP).  Rays that never reach the
bad node render exactly as the FP32 oracle renders the intact pool; rays
that do end as misses.  The reference has no such checks (SVOData::Load
does not validate, cell/svodata.h:31-50)."""
import ctypes as C

import numpy as np
import pytest

from conftest import LIGHT, camera_for

pytestmark = pytest.mark.gpu

W, H = 160, 120


def _scene(yoxel):
    return yoxel.SVOScene.spheres(7, 60, 2.0, 12.0, 4321)


def _corrupt(scene, oracle, mode):
    """A copy of the pool with one subtree broken.  P = the parent of the
    most frequently hit leaves.  Mode "range": the slot pointing at P points
    past the pool.  Mode "cycle": P's eight children all point at P (no
    leaves on the cycle, so a ray entering P descends until the depth cap)."""
    pos, view = camera_for()
    ref = oracle.svo_render(scene.nodes_u32, scene.root, scene.attrs_u8, pos, view, [0, 0, 1],
                            60.0, W, H, LIGHT, shadows=False)
    hits = ref["hit"][ref["hit"] != 0xFFFFFFFF]
    parents, counts = np.unique(hits >> 3, return_counts=True)
    nodes = scene.nodes_u32.reshape(-1, 10).copy()
    # the node whose child slot points at the busiest parent
    for p in parents[np.argsort(-counts)]:
        ref_slots = np.argwhere((nodes[:, 2:] == p) & ~((nodes[:, :1] >> np.arange(8)) & 1)
                                .astype(bool))
        if len(ref_slots):
            q, c = ref_slots[0]
            break
    if mode == "range":
        nodes[q, 2 + c] = scene.node_count + 5
    else:
        nodes[p, 0] = 0
        nodes[p, 2:] = p
    return nodes.reshape(-1), ref


def _noalloc(yoxel, scene, nodes_u32):
    import torch
    from yoxel import _lib as L
    d_nodes = torch.from_numpy(nodes_u32.copy().view(np.int32)).cuda()
    d_attrs = torch.from_numpy(scene.attrs_u8.copy()).cuda()
    pos, view = camera_for()
    cam = L.Camera(L.F3(*pos), L.F3(*view), L.F3(0, 0, 1), 60.0)
    light = L.Light(L.F3(*LIGHT), 0.15, 0.85, 0)
    out = {k: torch.full((H, W), -7, dtype=torch.int32, device="cuda")
           for k in ("rgba", "hit", "hit_t", "fetches", "shadow_fetches")}
    fo = L.FrameOutputs(*[C.c_void_p(out[k].data_ptr()) for k in
                          ("rgba", "hit", "hit_t", "fetches", "shadow_fetches")])
    stream = torch.cuda.current_stream()
    st = L.lib.yv_render_svo_noalloc(C.c_void_p(d_nodes.data_ptr()), scene.node_count,
                                     scene.root, C.c_void_p(d_attrs.data_ptr()),
                                     scene.attr_count, C.byref(cam), C.byref(light), W, H,
                                     C.byref(fo), C.c_void_p(stream.cuda_stream))
    assert st == L.YV_OK
    bits = C.c_uint32()
    status = L.lib.yv_render_svo_noalloc_status(C.c_void_p(stream.cuda_stream), C.byref(bits))
    return status, bits.value, {k: v.cpu().numpy().view(np.uint32) for k, v in out.items()}


def _check_frame(got, ref):
    """Rays that never reach the broken slot equal the oracle on the intact
    pool; the others are misses."""
    diff = got["hit"] != ref["hit"]
    assert 0 < diff.sum() < 0.5 * diff.size
    assert (got["hit"][diff] == 0xFFFFFFFF).all()
    same = ~diff
    assert np.array_equal(got["rgba"][same], ref["rgba"][same])
    assert np.array_equal(got["fetches"][same], ref["fetches"][same])


@pytest.mark.parametrize("mode,expect", [("range", 3), ("cycle", 4)])
def test_noalloc_malformed_pool_reports_status(yoxel_mod, oracle, mode, expect):
    from yoxel import _lib as L
    scene = _scene(yoxel_mod)
    bad, ref = _corrupt(scene, oracle, mode)
    status, bits, got = _noalloc(yoxel_mod, scene, bad)
    assert status == expect, (L.status_string(status), bits)
    _check_frame(got, ref)
    # the next frame over the intact pool starts from a cleared status
    status, bits, got = _noalloc(yoxel_mod, scene, scene.nodes_u32)
    assert status == L.YV_OK and bits == 0
    assert np.array_equal(got["hit"], ref["hit"])


@pytest.mark.parametrize("mode,expect", [("range", 3), ("cycle", 4)])
def test_dynamic_scene_malformed_pool_reports_status(yoxel_mod, oracle, mode, expect):
    import torch
    from yoxel import _lib as L
    scene = _scene(yoxel_mod)
    bad, ref = _corrupt(scene, oracle, mode)
    dyn = yoxel_mod.DynamicSVO(scene.node_count + 64, scene.attr_count + 64)
    dyn.load(scene)
    nodes = bad.reshape(-1, 10)
    changed = np.argwhere((nodes != scene.nodes_u32.reshape(-1, 10)).any(axis=1)).ravel()
    for i in changed:
        vn = L.VoxNode()
        vn.flags = int(nodes[i, 0])
        vn.data = int(nodes[i, 1])
        for c in range(8):
            vn.child[c] = int(nodes[i, 2 + c])
        L.check(L.lib.yv_svo_dynamic_set_node(dyn._h, int(i), C.byref(vn)), "set_node")
    dyn.sync()
    pos, view = camera_for()
    # the editable scene's own frame (allocation-free path) ...
    g = dyn.render(pos, view, [0, 0, 1], 60.0, W, H, LIGHT)
    with pytest.raises(L.YvError) as e:
        dyn.status()
    assert e.value.status == expect
    _check_frame({k: v.cpu().numpy().view(np.uint32) for k, v in g.items()}, ref)
    # ... and a renderer bound to it (SVORenderer::SetScene(DynamicSVO*))
    r = yoxel_mod.Renderer()
    r.SetSceneDynamic(dyn)
    r.SetViewPos(pos)
    r.SetViewDir(view)
    r.SetResolution(W, H)
    r.SetFOV(60.0)
    r.SetLight(LIGHT, 0.15, 0.85, False)
    out = {k: torch.empty((H, W), dtype=torch.int32, device="cuda")
           for k in ("rgba", "hit", "fetches")}
    r.render_async(**out)
    st = r.frame_stats(check=False)
    assert st["status"] == expect
    _check_frame({k: v.cpu().numpy().view(np.uint32) for k, v in out.items()}, ref)


def test_frame_budget_times_out_and_frame_recovers(yoxel_mod):
    """The persistent queue's time budget: with a 1 us budget the frame
    kernel stops taking rays after the first ones its warps took, the frame
    reports YV_ERR_TIMEOUT, every pixel it wrote equals the unbudgeted
    frame's, the others keep their contents; with the budget removed the
    next frame is complete and the status clean."""
    import torch
    from yoxel import _lib as L
    scene = yoxel_mod.SVOScene.spheres(8, 200, 4.0, 24.0, 1234)
    pos, view = camera_for()
    w, h = 1024, 1024
    r = yoxel_mod.Renderer()
    r.SetScene(scene)
    r.SetViewPos(pos)
    r.SetViewDir(view)
    r.SetResolution(w, h)
    r.SetFOV(60.0)
    r.SetLight(LIGHT, 0.15, 0.85, True)
    assert r.GetFrameBudget() == 0
    full = r.render_outputs()
    assert full.pop("stats")["status"] == L.YV_OK
    r.SetFrameBudget(1)
    assert r.GetFrameBudget() == 1
    out = {k: torch.full((h, w), -7, dtype=torch.float32 if k == "hit_t" else torch.int32,
                         device="cuda") for k in full}
    r.render_async(**out)
    st = r.frame_stats(check=False)
    assert st["status"] == L.YV_ERR_TIMEOUT
    with pytest.raises(L.YvError) as e:
        r.frame_stats()
    assert e.value.status == L.YV_ERR_TIMEOUT
    got = {k: v.cpu().numpy() for k, v in out.items()}
    ref = {k: v.cpu().numpy().view(np.uint32) for k, v in full.items()}
    written = got["fetches"] != -7
    assert 0 < written.sum() < w * h
    for k in got:
        assert np.array_equal(got[k].view(np.uint32)[written], ref[k][written]), k
        assert (got[k][~written] == -7).all(), k
    r.SetFrameBudget(0)
    again = r.render_outputs()
    assert again.pop("stats")["status"] == L.YV_OK
    for k in again:
        assert torch.equal(again[k].view(torch.int32), full[k].view(torch.int32)), k
