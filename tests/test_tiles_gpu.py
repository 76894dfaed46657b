"""Tile-range frames (yv_render_frame_tiles): a frame split into contiguous
ranges of 8x4-pixel tiles - the row bands of the reference's threaded
renderer (cell/ppu_renderer.cpp:121-144), or the cost-balanced ranges the
multi-GPU partitioner hands to each rank - renders the full frame bit for
bit once the ranges are merged, and a range writes only its own pixels."""
import numpy as np
import pytest

from conftest import LIGHT, camera_for

pytestmark = pytest.mark.gpu

KEYS = ("rgba", "hit", "hit_t", "fetches", "shadow_fetches")


def make_renderer(yoxel, scene, w, h, shadows=True):
    pos, view = camera_for()
    r = yoxel.Renderer()
    r.SetScene(scene)
    r.SetViewPos(pos)
    r.SetViewDir(view)
    r.SetResolution(w, h)
    r.SetFOV(60.0)
    r.SetLight(LIGHT, 0.15, 0.85, shadows)
    return r


def sentinel_outputs(torch, w, h):
    return {k: torch.full((h, w), -3, dtype=torch.float32 if k == "hit_t" else torch.int32,
                          device="cuda") for k in KEYS}


def tile_mask(w, h, tb, te):
    """Pixels of tiles [tb, te) (row-major 8x4 tiles)."""
    tx = (w + 7) // 8
    m = np.zeros((h, w), bool)
    for t in range(tb, te):
        x0, y0 = (t % tx) * 8, (t // tx) * 4
        m[y0:y0 + 4, x0:x0 + 8] = True
    return m


@pytest.fixture(scope="module")
def spheres(yoxel_mod):
    return yoxel_mod.SVOScene.spheres(8, 200, 4.0, 24.0, 1234)


@pytest.mark.parametrize("size,parts", [((512, 512), 4), ((333, 211), 3), ((64, 48), 7)])
def test_tile_ranges_merge_to_the_full_frame(yoxel_mod, spheres, size, parts):
    import torch
    from yoxel.parallel import partition_tiles
    w, h = size
    r = make_renderer(yoxel_mod, spheres, w, h)
    full = r.render_outputs()
    full_stats = full.pop("stats")
    tx, ty = r.tile_count()
    assert (tx, ty) == ((w + 7) // 8, (h + 3) // 4)
    # cost-balanced ranges from the full frame's per-tile fetch counts
    f = full["fetches"].cpu().numpy().astype(np.int64) + full["shadow_fetches"].cpu().numpy()
    fp = np.zeros((ty * 4, tx * 8), np.int64)
    fp[:h, :w] = f
    costs = fp.reshape(ty, 4, tx, 8).sum(axis=(1, 3)).reshape(-1) + 1
    ranges = partition_tiles(costs, parts)
    assert ranges[0][0] == 0 and ranges[-1][1] == tx * ty
    out = sentinel_outputs(torch, w, h)
    pixels = 0
    for k, (tb, te) in enumerate(ranges):
        r.render_tiles(tb, te, **out)
        st = r.frame_stats()
        m = tile_mask(w, h, tb, te)
        assert st["primary_rays"] == int(m.sum())
        pixels += st["primary_rays"]
        if k == 0:
            # nothing outside the first range was written
            got = out["rgba"].cpu().numpy()
            assert (got[~m] == -3).all() and (got[m] != -3).any() == bool(m.sum())
    assert pixels == w * h
    for key in KEYS:
        a = out[key].cpu().numpy().view(np.uint32)
        b = full[key].cpu().numpy().view(np.uint32)
        assert np.array_equal(a, b), key
    assert full_stats["primary_rays"] == w * h


def test_row_bands_as_the_threaded_renderer(yoxel_mod, spheres):
    """Four row bands (TreadedRenderer's split): each band is a contiguous
    tile range when its row count is a multiple of the tile height."""
    import torch
    w, h = 256, 192
    r = make_renderer(yoxel_mod, spheres, w, h, shadows=False)
    full = r.render_outputs()
    full.pop("stats")
    tx, _ = r.tile_count()
    out = sentinel_outputs(torch, w, h)
    band = h // 4
    for i in range(4):
        r.render_tiles(tx * (i * band // 4), tx * ((i + 1) * band // 4), **out)
    torch.cuda.synchronize()
    for key in KEYS:
        assert torch.equal(out[key].view(torch.int32), full[key].view(torch.int32)), key


def test_tile_range_arguments(yoxel_mod, spheres):
    import torch
    from yoxel import _lib as L
    r = make_renderer(yoxel_mod, spheres, 40, 20)
    tx, ty = r.tile_count()
    out = sentinel_outputs(torch, 40, 20)
    with pytest.raises(L.YvError) as e:
        r.render_tiles(0, tx * ty + 1, **out)
    assert e.value.status == L.YV_ERR_INVALID_ARG
    with pytest.raises(L.YvError):
        r.render_tiles(5, 4, **out)
    # an empty range writes nothing
    r.render_tiles(3, 3, **out)
    assert r.frame_stats()["primary_rays"] == 0
    assert (out["rgba"].cpu().numpy() == -3).all()
