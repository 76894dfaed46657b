"""GPU parity of the level-of-detail cut-off (SVORenderer::SetDetailCoef,
demo/SVORenderer.cpp:104) against the FP32 oracle through the C ABI: hit
words, hit t, fetch counts, colours and shadow results bit-exact."""
import numpy as np
import pytest

from conftest import LIGHT, camera_for

pytestmark = pytest.mark.gpu


def render(yoxel, scene, detail, shadows, w=192, h=128, dist=1.5):
    r = yoxel.Renderer()
    r.SetScene(scene)
    pos, view = camera_for(dist=dist)
    r.SetViewPos(pos)
    r.SetViewDir(view)
    r.SetViewUp([0, 0, 1])
    r.SetResolution(w, h)
    r.SetFOV(60.0)
    r.SetLight(LIGHT, 0.15, 0.85, shadows)
    r.SetDetailCoef(detail)
    o = r.render_outputs()
    o.pop("stats")
    out = {k: v.cpu().numpy() for k, v in o.items()}
    for k in ("rgba", "hit", "fetches", "shadow_fetches"):
        out[k] = out[k].view(np.uint32)
    return out, r, pos, view


def oracle_frame(oracle, scene, pos, view, w, h, shadows, coef):
    return oracle.svo_render(scene.nodes_u32, scene.root, scene.attrs_u8, pos, view,
                             np.float32([0, 0, 1]), 60.0, w, h, LIGHT, 0.15, 0.85, shadows,
                             lod_coef=coef)


def assert_same(g, o, shadows):
    bad = g["hit"] != o["hit"]
    assert bad.sum() == 0, f"{bad.sum()} hit words differ, first at {np.argwhere(bad)[:3]}"
    assert np.array_equal(g["hit_t"].view(np.uint32), o["hit_t"].view(np.uint32))
    assert np.array_equal(g["fetches"], o["fetches"])
    assert np.array_equal(g["rgba"], o["rgba"])
    if shadows:
        assert np.array_equal(g["shadow_fetches"], o["shadow_fetches"])


@pytest.fixture(scope="module")
def spheres_lod(yoxel_mod):
    return yoxel_mod.SVOScene.spheres(8, 200, 4.0, 24.0, 1234).build_lod()


@pytest.fixture(scope="module")
def terrain_lod(yoxel_mod):
    return yoxel_mod.SVOScene.terrain(9, 400, 2, 12, 77).build_lod()


@pytest.mark.parametrize("detail", [0.5, 2.0, 8.0])
@pytest.mark.parametrize("shadows", [False, True])
def test_lod_matches_oracle_spheres(yoxel_mod, oracle, spheres_lod, detail, shadows):
    g, r, pos, view = render(yoxel_mod, spheres_lod, detail, shadows)
    o = oracle_frame(oracle, spheres_lod, pos, view, 192, 128, shadows, r.lod_coef())
    assert_same(g, o, shadows)


@pytest.mark.parametrize("detail", [1.0, 6.0])
def test_lod_matches_oracle_terrain(yoxel_mod, oracle, terrain_lod, detail):
    g, r, pos, view = render(yoxel_mod, terrain_lod, detail, True, dist=1.2)
    o = oracle_frame(oracle, terrain_lod, pos, view, 192, 128, True, r.lod_coef())
    assert_same(g, o, True)


def test_lod_cuts_work_and_stops_at_subtrees(yoxel_mod, spheres_lod):
    exact, _, _, _ = render(yoxel_mod, spheres_lod, 0.0, False)
    coarse, _, _, _ = render(yoxel_mod, spheres_lod, 8.0, False)
    assert coarse["fetches"].mean() < exact["fetches"].mean()
    assert np.all(coarse["fetches"] <= exact["fetches"])
    hit = coarse["hit"] != 0xFFFFFFFF
    nn = spheres_lod.nodes_u32.reshape(-1, 10)
    ids, ch = coarse["hit"][hit] >> 3, coarse["hit"][hit] & 7
    assert ((nn[ids, 0] >> ch) & 1 == 0).any()


def test_detail_without_lod_data_is_exact(yoxel_mod, oracle):
    s = yoxel_mod.SVOScene.spheres(7, 60, 2.0, 12.0, 11)  # no build_lod
    g, r, pos, view = render(yoxel_mod, s, 8.0, False)
    assert r.GetDetailCoef() == 8.0
    o = oracle_frame(oracle, s, pos, view, 192, 128, False, 0.0)
    assert_same(g, o, False)
