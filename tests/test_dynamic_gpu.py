"""Editable SVO with incremental device sync: after loads and voxel edits
only the changed 256-node pages travel, the device mirror equals the host
pool byte for byte, and frames traced from the mirror equal the FP32
oracle's frames of the host pool (hit ids are the pool's own node ids)."""
import numpy as np
import pytest

from conftest import LIGHT, camera_for

pytestmark = pytest.mark.gpu


def check_mirror_and_frame(yoxel_mod, oracle, dyn, shadows):
    import torch
    dyn.sync()
    torch.cuda.synchronize()
    assert dyn.changed_pages() == 0 and dyn.transfer_bytes() == 0
    nodes, root, attrs = dyn.host_arrays()
    dn, da = dyn.download()
    assert np.array_equal(dn.view(np.uint32), nodes.view(np.uint32))
    assert np.array_equal(da.view(np.uint8), attrs.view(np.uint8))
    pos, view = camera_for()
    up = np.array([0, 0, 1], np.float32)
    g = dyn.render(pos, view, up, 60.0, 80, 64, LIGHT, shadows=shadows)
    o = oracle.svo_render(nodes.view(np.uint32), root, attrs.view(np.uint8), pos, view, up,
                          60.0, 80, 64, LIGHT, shadows=shadows)
    for k in ("hit", "rgba", "fetches"):
        got = g[k].cpu().numpy().view(np.uint32).reshape(-1)
        assert np.array_equal(got, o[k].reshape(-1)), k
    return o


def test_dynamic_sync_and_edits(yoxel_mod, oracle):
    depth = 6
    scene = yoxel_mod.SVOScene.spheres(depth, 30, 2.0, 8.0, 21)
    dyn = yoxel_mod.DynamicSVO(scene.node_count + 4096, scene.attr_count + 8192)
    dyn.load(scene)
    total = dyn.changed_pages()
    assert total > 0
    o0 = check_mirror_and_frame(yoxel_mod, oracle, dyn, True)
    # a few edits touch a few pages
    rng = np.random.default_rng(3)
    G = 1 << depth
    for _ in range(40):
        x, y, z = (int(v) for v in rng.integers(G // 4, 3 * G // 4, 3))
        dyn.set_voxel(depth, x, y, z, rgb=tuple(int(c) for c in rng.integers(0, 256, 3)),
                      normal=(0, 127, 0))
    for _ in range(40):
        x, y, z = (int(v) for v in rng.integers(0, G, 3))
        dyn.set_voxel(depth, x, y, z, None)
    changed = dyn.changed_pages()
    assert 0 < changed < total + 40
    assert dyn.transfer_bytes() < (scene.node_count + 4096) * 40 + (scene.attr_count + 8192) * 8
    o1 = check_mirror_and_frame(yoxel_mod, oracle, dyn, True)
    assert not np.array_equal(o0["hit"], o1["hit"])


def test_dynamic_from_empty_and_paging(yoxel_mod, oracle):
    dyn = yoxel_mod.DynamicSVO(600, 600)
    # build a small scene voxel by voxel from nothing
    for i in range(300):
        dyn.set_voxel(5, 8 + i % 16, 8 + (i // 16) % 16, 10 + i // 256, rgb=(200, 50, 20))
    assert dyn.root == 0
    check_mirror_and_frame(yoxel_mod, oracle, dyn, False)
    # one more voxel: only the pages it touched travel
    dyn.set_voxel(5, 31, 31, 31, rgb=(1, 2, 3))
    assert 1 <= dyn.changed_pages() <= 4
    check_mirror_and_frame(yoxel_mod, oracle, dyn, False)


def test_renderer_bound_to_editable_scene(yoxel_mod, oracle):
    """SVORenderer::SetScene(DynamicSVO*) + UpdateSVO: the renderer traces
    the mirror in place as of the last sync; edits show after a sync."""
    import torch
    depth = 6
    scene = yoxel_mod.SVOScene.spheres(depth, 30, 2.0, 8.0, 21)
    dyn = yoxel_mod.DynamicSVO(scene.node_count + 4096, scene.attr_count + 8192)
    dyn.load(scene)
    dyn.sync()
    r = yoxel_mod.Renderer()
    r.SetSceneDynamic(dyn)
    pos, view = camera_for()
    up = np.array([0, 0, 1], np.float32)
    r.SetViewPos(pos)
    r.SetViewDir(view)
    r.SetViewUp(up)
    r.SetResolution(80, 64)
    r.SetFOV(60.0)
    r.SetLight(LIGHT, 0.15, 0.85, True)

    def frame():
        o = r.render_outputs()
        o.pop("stats")
        return {k: v.cpu().numpy().view(np.uint32).reshape(-1)
                for k, v in o.items() if k in ("hit", "rgba", "fetches")}

    def oracle_frame():
        nodes, root, attrs = dyn.host_arrays()
        return oracle.svo_render(nodes.view(np.uint32), root, attrs.view(np.uint8), pos, view,
                                 up, 60.0, 80, 64, LIGHT, shadows=True)

    g0 = frame()
    o0 = oracle_frame()
    for k in g0:
        assert np.array_equal(g0[k], o0[k].reshape(-1)), k
    # edit: until the sync the renderer still shows the synced state
    rng = np.random.default_rng(5)
    G = 1 << depth
    for _ in range(60):
        x, y, z = (int(v) for v in rng.integers(G // 4, 3 * G // 4, 3))
        dyn.set_voxel(depth, x, y, z, rgb=(250, 20, 20), normal=(0, 0, 127))
    g1 = frame()
    for k in g0:
        assert np.array_equal(g1[k], g0[k]), k
    dyn.sync()
    torch.cuda.synchronize()
    g2 = frame()
    o2 = oracle_frame()
    for k in g2:
        assert np.array_equal(g2[k], o2[k].reshape(-1)), k
    assert not np.array_equal(g2["hit"], g0["hit"])
    # the screen-space pipeline runs on the bound scene too
    rgba = r.render_ssna()
    r.frame_stats()
    assert (rgba.cpu().numpy().view(np.uint32) >> 24).any()
    # batching a renderer bound to an editable scene is refused
    from yoxel import _lib as L
    b = yoxel_mod.Batch()
    out = torch.empty((64, 80), dtype=torch.int32, device="cuda")
    with pytest.raises(L.YvError):
        b.add_svo(r, out)
