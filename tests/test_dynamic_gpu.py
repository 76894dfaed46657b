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
