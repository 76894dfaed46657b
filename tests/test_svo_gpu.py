"""GPU parity of the SVO ray cast against the CPU oracle, through the C ABI.

Bar: hit voxel index (node id, child) bit-exact with the FP32 restatement of
the reference renderer; hit t, fetch counts, RGBA8 colour and shadow results
bit-exact too (the kernel issues the same IEEE operations).  Against the FP64
oracle, rays whose hit differs (float ties at cell boundaries) must stay
under 1e-4 of all rays."""
import os

import numpy as np
import pytest

from conftest import LIGHT, ROOT, camera_for

pytestmark = pytest.mark.gpu

TIE_BUDGET = 1e-4


def render_gpu(yoxel, scene, pos, view, w, h, fov=60.0, shadows=False, cfg=None,
               arrays=None):
    r = yoxel.Renderer()
    if arrays is not None:
        r.SetSceneArrays(*arrays)
    else:
        r.SetScene(scene)
    r.SetViewPos(pos)
    r.SetViewDir(view)
    r.SetViewUp([0, 0, 1])
    r.SetResolution(w, h)
    r.SetFOV(fov)
    r.SetLight(LIGHT, 0.15, 0.85, shadows)
    if cfg:
        r.SetLaunchConfig(**cfg)
    o = r.render_outputs()
    stats = o.pop("stats")
    out = {k: v.cpu().numpy() for k, v in o.items()}
    out["hit"] = out["hit"].view(np.uint32)
    out["rgba"] = out["rgba"].view(np.uint32)
    out["fetches"] = out["fetches"].view(np.uint32)
    out["shadow_fetches"] = out["shadow_fetches"].view(np.uint32)
    return out, stats


def assert_bit_exact(g, o, shadows):
    miss = g["hit"] != o["hit"]
    assert miss.sum() == 0, f"{miss.sum()} hit ids differ, first at {np.argwhere(miss)[:3]}"
    assert np.array_equal(g["hit_t"].view(np.uint32), o["hit_t"].view(np.uint32))
    assert np.array_equal(g["fetches"], o["fetches"])
    assert np.array_equal(g["rgba"], o["rgba"])
    if shadows:
        assert np.array_equal(g["shadow_fetches"], o["shadow_fetches"])


@pytest.fixture(scope="module")
def spheres(yoxel_mod):
    return yoxel_mod.SVOScene.spheres(8, 200, 4.0, 24.0, 1234)


@pytest.mark.parametrize("shadows", [False, True])
def test_spheres_256_parity(yoxel_mod, oracle, spheres, shadows):
    """200 spheres in 256^3 (depth 8), 512x512, FOV 60, Lambert."""
    pos, view = camera_for()
    g, st = render_gpu(yoxel_mod, spheres, pos, view, 512, 512, shadows=shadows)
    o = oracle.svo_render(spheres.nodes_u32, spheres.root, spheres.attrs_u8, pos, view,
                          [0, 0, 1], 60.0, 512, 512, LIGHT, shadows=shadows, threads=8)
    assert_bit_exact(g, o, shadows)
    hits = int((o["hit"] != 0xFFFFFFFF).sum())
    assert st["hits"] == hits and st["primary_rays"] == 512 * 512
    if shadows:
        assert st["shadow_rays"] == hits and st["shadowed"] == int(o["shadowed"].sum())
    h64, _ = oracle.svo_hits_f64(spheres.nodes_u32, spheres.root, pos, view, [0, 0, 1], 60.0,
                                 512, 512)
    ties = (h64 != g["hit"]).mean()
    assert ties < TIE_BUDGET, f"FP64 tie rate {ties}"


def test_terrain_parity_with_shadows(yoxel_mod, oracle):
    s = yoxel_mod.SVOScene.terrain(9, 2500, 2, 8, 77)
    pos, view = camera_for()
    g, _ = render_gpu(yoxel_mod, s, pos, view, 320, 180, shadows=True)
    o = oracle.svo_render(s.nodes_u32, s.root, s.attrs_u8, pos, view, [0, 0, 1], 60.0, 320,
                          180, LIGHT, shadows=True, threads=8)
    assert_bit_exact(g, o, True)
    assert (o["hit"] != 0xFFFFFFFF).mean() > 0.3


@pytest.mark.parametrize("name", ["svo_spheres_d5", "svo_terrain_d6"])
def test_golden_fixtures(yoxel_mod, name):
    gf = np.load(os.path.join(ROOT, "tests", "golden", name + ".npz"))
    nodes = gf["nodes"].view(yoxel_mod.NODE_DTYPE)
    attrs = gf["attrs"].view(yoxel_mod.ATTR_DTYPE)
    g, _ = render_gpu(yoxel_mod, None, gf["pos"], gf["view"], int(gf["width"]),
                      int(gf["height"]), float(gf["fov"]), bool(gf["shadows"]),
                      arrays=(nodes, int(gf["root"]), attrs))
    expect = {k: gf[k] for k in ("rgba", "hit", "hit_t", "fetches", "shadow_fetches")}
    assert_bit_exact(g, expect, True)


@pytest.mark.parametrize("cfg", [
    dict(smem_nodes=0), dict(smem_nodes=9), dict(smem_nodes=4096),
    dict(block_threads=64), dict(block_threads=128, blocks_per_sm=2),
])
def test_launch_configs_give_identical_results(yoxel_mod, spheres, cfg):
    pos, view = camera_for()
    base, _ = render_gpu(yoxel_mod, spheres, pos, view, 200, 150, shadows=True)
    g, _ = render_gpu(yoxel_mod, spheres, pos, view, 200, 150, shadows=True, cfg=cfg)
    for k in ("hit", "rgba", "fetches", "shadow_fetches"):
        assert np.array_equal(base[k], g[k]), k


@pytest.mark.parametrize("case", ["inside", "axis", "ragged", "tiny", "wide_fov"])
def test_edge_cases(yoxel_mod, oracle, spheres, case):
    pos, view = camera_for()
    w, h, fov = 64, 48, 60.0
    if case == "inside":       # camera inside the volume (reference quirk path)
        pos = np.array([0.41, 0.47, 0.52], np.float32)
        view = np.array([0.3, -1.0, 0.2], np.float32)
    elif case == "axis":       # axis-aligned view: AdjustDir epsilon path
        pos = np.array([0.5, 0.5, 2.0], np.float32)
        view = np.array([0.0, 0.0, -1.0], np.float32)
        w, h = 65, 65
    elif case == "ragged":     # width/height not multiples of the 8x4 tile
        w, h = 37, 23
    elif case == "tiny":
        w, h = 1, 1
    elif case == "wide_fov":
        fov = 150.0
    g, _ = render_gpu(yoxel_mod, spheres, pos, view, w, h, fov=fov, shadows=True)
    o = oracle.svo_render(spheres.nodes_u32, spheres.root, spheres.attrs_u8, pos, view,
                          [0, 0, 1], fov, w, h, LIGHT, shadows=True)
    assert_bit_exact(g, o, True)


def test_empty_and_single_voxel_scenes(yoxel_mod, oracle):
    EMPTY = 0x80000000
    pos, view = camera_for()
    empty = np.zeros(0, yoxel_mod.NODE_DTYPE)
    g, st = render_gpu(yoxel_mod, None, pos, view, 32, 32,
                       arrays=(empty, EMPTY, np.zeros(0, yoxel_mod.ATTR_DTYPE)))
    assert (g["hit"] == 0xFFFFFFFF).all() and (g["rgba"] == 0).all() and st["hits"] == 0
    # one leaf: root child 6 of a depth-1 tree
    node = np.zeros(1, yoxel_mod.NODE_DTYPE)
    node["child"][0] = [EMPTY] * 6 + [0, EMPTY]
    node["flags"][0] = (1 << 6) | (0xBF << 8)
    attrs = np.zeros(1, yoxel_mod.ATTR_DTYPE)
    attrs["rgb"][0] = [200, 100, 50, 255]
    attrs["n"][0] = [0, 0, 127, 0]
    g, st = render_gpu(yoxel_mod, None, pos, view, 48, 48, shadows=True,
                       arrays=(node, 0, attrs))
    o = oracle.svo_render(node.view(np.uint32), 0, attrs.view(np.uint8), pos, view, [0, 0, 1],
                          60.0, 48, 48, LIGHT, shadows=True)
    assert_bit_exact(g, o, True)
    assert st["hits"] > 0


def test_render_frame_host_matches_device(yoxel_mod, spheres):
    pos, view = camera_for()
    g, _ = render_gpu(yoxel_mod, spheres, pos, view, 96, 64)
    r = yoxel_mod.Renderer()
    r.SetScene(spheres)
    r.SetViewPos(pos)
    r.SetViewDir(view)
    r.SetResolution(96, 64)
    r.SetFOV(60.0)
    r.SetLight(LIGHT, 0.15, 0.85, False)
    img = r.RenderFrame()
    assert img.shape == (64, 96, 4)
    assert np.array_equal(img.reshape(-1, 4).view(np.uint32).reshape(64, 96), g["rgba"])


def test_status_codes(yoxel_mod):
    r = yoxel_mod.Renderer()
    assert r.RenderFrame() is None  # no scene: RenderFrame returns NULL
    # a pool with a cycle is rejected by validation
    node = np.zeros(1, yoxel_mod.NODE_DTYPE)
    node["child"][0] = [0] + [0x80000000] * 7
    with pytest.raises(yoxel_mod.YvError) as e:
        r.SetSceneArrays(node, 0, np.zeros(0, yoxel_mod.ATTR_DTYPE))
    assert e.value.status == 3
    # frames up to 2^31 rays in 8x4 tiles (the ray ids are 32-bit); a thin
    # frame counts its padding
    from yoxel import _lib as L
    r.SetResolution(8, 4 * ((1 << 26) - 1))
    assert r.GetResolution() == (8, 4 * ((1 << 26) - 1))
    for w, h in [(8, 1 << 28), (1, 1 << 28), (46341, 46341)]:
        with pytest.raises(yoxel_mod.YvError) as e:
            r.SetResolution(w, h)
        assert e.value.status == L.YV_ERR_INVALID_ARG


def test_vox_roundtrip_renders_identically(yoxel_mod, spheres, tmp_path):
    p = tmp_path / "scene.vox"
    spheres.save(p)
    s2 = yoxel_mod.SVOScene.load(p)
    pos, view = camera_for()
    a, _ = render_gpu(yoxel_mod, spheres, pos, view, 64, 64)
    b, _ = render_gpu(yoxel_mod, s2, pos, view, 64, 64)
    assert np.array_equal(a["hit"], b["hit"]) and np.array_equal(a["rgba"], b["rgba"])


def test_cuda_renderer_driver(yoxel_mod, spheres):
    """trace_cuda.CudaRenderer-style driver."""
    cr = yoxel_mod.CudaRenderer((128, 96))
    cr.updateScene(spheres)
    cr.setLightPos((0.5, 0.5, 1.0))
    pos, view = camera_for()
    stat = cr.render(pos, view)
    assert "gpu time" in stat
    img = cr.getImage()
    assert img.shape == (96, 128, 3) and img.max() > 0


def deep_random_tree(rng, levels=16):
    """Random sparse pool with `levels` node levels: 1-3 node children per
    node (more near the root), 1-4 leaves per bottom node."""
    EMPTY = 0x80000000
    nodes, attrs = [], []

    def make(level):
        idx = len(nodes)
        nodes.append(None)
        flags, child = 0, [EMPTY] * 8
        if level == levels - 1:
            for ch in rng.choice(8, int(rng.integers(1, 5)), replace=False):
                flags |= 1 << int(ch)
                child[int(ch)] = len(attrs)
                attrs.append(list(rng.integers(0, 256, 4)) + list(rng.integers(-127, 128, 3)) + [0])
        else:
            k = int(rng.integers(2, 5)) if level < 4 else int(rng.integers(1, 3))
            for ch in rng.choice(8, k, replace=False):
                child[int(ch)] = make(level + 1)
        for ch in range(8):
            if not (flags >> ch) & 1 and child[ch] & 0x80000000:
                flags |= 1 << (8 + ch)
        nodes[idx] = (flags, child)
        return idx

    make(0)
    n = np.zeros(len(nodes), dtype=np.dtype([("flags", "<u4"), ("data", "<u4"),
                                             ("child", "<u4", (8,))]))
    for i, (f, c) in enumerate(nodes):
        n["flags"][i] = f
        n["child"][i] = c
    a = np.array(attrs, dtype=np.int64).astype(np.int8).view(np.uint8).reshape(-1, 8)
    return n, a


def test_deepest_tree_16_levels(yoxel_mod, oracle):
    """16 node levels (the maximum): deep frame stacks spill out of the
    shared-memory ring into local memory and back; hits, hit distances,
    colours and per-ray fetch counts stay bit-exact."""
    n, a = deep_random_tree(np.random.default_rng(5))
    attrs = a.reshape(-1).view(yoxel_mod.ATTR_DTYPE)
    nodes = n.view(yoxel_mod.NODE_DTYPE)
    assert yoxel_mod.SVOScene.from_arrays(nodes, 0, attrs).depth == 16
    pos = np.array([1.3, 1.1, 0.9], np.float32)
    for view in ([-0.8, -0.6, -0.4], [-1.0, -0.2, -0.3]):
        view = np.array(view, np.float32)
        g, _ = render_gpu(yoxel_mod, None, pos, view, 128, 96, fov=70.0, shadows=True,
                          arrays=(nodes, 0, attrs))
        o = oracle.svo_render(nodes.view(np.uint32), 0, attrs.view(np.uint8), pos, view,
                              [0, 0, 1], 70.0, 128, 96, LIGHT, shadows=True)
        assert_bit_exact(g, o, True)
        assert o["fetches"].max() >= 16


@pytest.mark.parametrize("name", ["ref_svo_spheres_d6", "ref_svo_terrain_d6",
                                  "ref_svo_inside_d5", "ref_svo_axis_d5", "ref_svo_deep16"])
def test_reference_renderer_fixtures(yoxel_mod, name):
    """The CUDA path against outputs of the reference's own CPU renderer
    (cell/ppu_renderer.cpp compiled on the host, tests/golden/
    make_ref_golden.py): every pixel's hit leaf (its VoxData), t and node
    fetches bit-exact."""
    gf = np.load(os.path.join(ROOT, "tests", "golden", name + ".npz"))
    nodes = gf["nodes"].view(yoxel_mod.NODE_DTYPE)
    attrs = gf["attrs"].reshape(-1).view(yoxel_mod.ATTR_DTYPE)
    r = yoxel_mod.Renderer()
    r.SetSceneArrays(nodes, int(gf["root"]), attrs)
    r.SetViewPos(gf["pos"])
    r.SetViewDir(gf["view"])
    r.SetViewUp(gf["up"])
    r.SetResolution(int(gf["width"]), int(gf["height"]))
    r.SetFOV(float(gf["fov"]))
    r.SetLight(LIGHT, 0.15, 0.85, False)
    o = r.render_outputs()
    hit = o["hit"].cpu().numpy().view(np.uint32)
    pool = gf["nodes"].reshape(-1, 10)
    data = np.full(hit.shape, 0xFFFFFFFF, np.uint32)
    m = hit != 0xFFFFFFFF
    data[m] = pool[hit[m] >> 3, 2 + (hit[m] & 7)]
    assert np.array_equal(data, gf["data"])
    assert np.array_equal(o["hit_t"].cpu().numpy().view(np.uint32), gf["t"].view(np.uint32))
    assert np.array_equal(o["fetches"].cpu().numpy().view(np.uint32), gf["fetches"])
