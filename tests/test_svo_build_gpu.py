"""GPU SVO build from a dense density grid vs the CPU oracle of the build:
the canonical pool (nodes, leaf attributes, root) must be bit-identical, and
a renderer whose scene was built on the GPU must render exactly the frame of
the oracle-built pool."""
import numpy as np
import pytest

from conftest import LIGHT, camera_for

pytestmark = pytest.mark.gpu

EMPTY, FULL = 0x80000000, 0x80000001


def density_field(kind, depth, seed):
    G = 1 << depth
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(G, dtype=np.float32), np.arange(G, dtype=np.float32),
                          np.arange(G, dtype=np.float32), indexing="ij")
    if kind == "noise":
        return rng.standard_normal((G, G, G)).astype(np.float32)
    if kind == "blob":
        return (G * 0.3 - np.sqrt((x - G / 2) ** 2 + (y - G / 2 + 0.5) ** 2 +
                                  (z - G / 2) ** 2)).astype(np.float32)
    d = np.full((G, G, G), -1e9, np.float32)
    for _ in range(8):
        c = rng.uniform(0, G, 3).astype(np.float32)
        r = np.float32(rng.uniform(1, G / 4))
        d = np.maximum(d, r - np.sqrt((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2))
    return d.astype(np.float32)


def gpu_build(yoxel_mod, d, depth, iso, rgb):
    import torch
    td = torch.from_numpy(d).cuda()
    tr = None if rgb is None else torch.from_numpy(rgb).cuda()
    s = yoxel_mod.SVOScene.build_dense(td, depth, iso, tr)
    torch.cuda.synchronize()
    return s


@pytest.mark.parametrize("kind,depth,seed,with_rgb", [
    ("blob", 3, 1, True), ("noise", 4, 2, True), ("spheres", 5, 3, False),
    ("spheres", 6, 4, True), ("noise", 6, 5, False), ("spheres", 8, 6, True)])
def test_gpu_build_matches_oracle(yoxel_mod, oracle, kind, depth, seed, with_rgb):
    d = density_field(kind, depth, seed)
    G = 1 << depth
    rgb = (np.random.default_rng(seed + 100).integers(0, 256, (G, G, G, 3), dtype=np.uint8)
           if with_rgb else None)
    nodes, attrs, root = oracle.svo_build_dense(d, depth, 0.0, rgb)
    s = gpu_build(yoxel_mod, d, depth, 0.0, rgb)
    assert s.root == root
    assert np.array_equal(s.nodes_u32.reshape(-1, 10), nodes)
    assert np.array_equal(s.attrs_u8.reshape(-1, 8), attrs)
    assert len(nodes) > 0


def test_gpu_build_edge_cases(yoxel_mod, oracle):
    for depth, fill in ((3, 0.0), (4, 1.0), (1, 1.0), (1, 0.0)):
        G = 1 << depth
        d = np.full((G, G, G), fill, np.float32)
        n, a, r = oracle.svo_build_dense(d, depth, 0.5)
        s = gpu_build(yoxel_mod, d, depth, 0.5, None)
        assert s.root == r
        assert np.array_equal(s.nodes_u32.reshape(-1, 10), n)
        assert np.array_equal(s.attrs_u8.reshape(-1, 8), a)
    d = np.zeros((8, 8, 8), np.float32)
    d[5, 2, 6] = 1.0
    s = gpu_build(yoxel_mod, d, 3, 0.5, None)
    n, a, r = oracle.svo_build_dense(d, 3, 0.5)
    assert np.array_equal(s.nodes_u32.reshape(-1, 10), n) and len(a) == 1


def test_renderer_scene_built_on_gpu(yoxel_mod, oracle):
    import torch
    depth = 7
    d = density_field("spheres", depth, 11)
    G = 1 << depth
    rgb = np.random.default_rng(12).integers(0, 256, (G, G, G, 3), dtype=np.uint8)
    nodes, attrs, root = oracle.svo_build_dense(d, depth, 0.0, rgb)
    pos, view = camera_for()
    w, h = 96, 72
    r = yoxel_mod.Renderer()
    r.SetSceneDense(torch.from_numpy(d).cuda(), depth, 0.0, torch.from_numpy(rgb).cuda())
    r.SetViewPos(pos)
    r.SetViewDir(view)
    r.SetResolution(w, h)
    r.SetFOV(60.0)
    r.SetLight(LIGHT, 0.15, 0.85, True)
    got = r.render_outputs()
    ref = oracle.svo_render(nodes.reshape(-1), root, attrs.reshape(-1), pos, view,
                            np.array([0, 0, 1], np.float32), 60.0, w, h, LIGHT, 0.15, 0.85, True)
    hit = got["hit"].cpu().numpy().view(np.uint32).reshape(-1)
    rgba = got["rgba"].cpu().numpy().view(np.uint32).reshape(-1)
    assert np.array_equal(hit, ref["hit"].reshape(-1))
    assert np.array_equal(rgba, ref["rgba"].reshape(-1))
    assert (hit != 0xFFFFFFFF).sum() > 100
    # the same pool uploaded from the host renders the same frame
    r2 = yoxel_mod.Renderer()
    from yoxel.svo import ATTR_DTYPE, NODE_DTYPE
    r2.SetSceneArrays(nodes.reshape(-1).view(NODE_DTYPE), root, attrs.reshape(-1).view(ATTR_DTYPE))
    r2.SetViewPos(pos)
    r2.SetViewDir(view)
    r2.SetResolution(w, h)
    r2.SetFOV(60.0)
    r2.SetLight(LIGHT, 0.15, 0.85, True)
    got2 = r2.render_outputs()
    assert torch.equal(got2["hit"], got["hit"]) and torch.equal(got2["rgba"], got["rgba"])
