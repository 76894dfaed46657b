"""Batched persistent render: one launch over mixed SVO / brick scenes must
give bit-identical frames to the per-scene launches (graph and plain
launch), and the autotuner must pick a configuration and cache it."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def build_batch(yoxel_mod, torch):
    from yoxel import workloads as W
    batch = yoxel_mod.Batch()
    keep, outs = [], []
    for i, (depth, res) in enumerate([(5, (64, 64)), (6, (96, 80)), (7, (130, 70))]):
        s = W.spheres(depth, seed=100 + i, n_spheres=40)
        r = yoxel_mod.Renderer()
        r.SetScene(s)
        pos, view = W.camera((1.0, 0.2 + 0.3 * i, 0.6))
        r.SetViewPos(pos)
        r.SetViewDir(view)
        r.SetResolution(*res)
        r.SetFOV(55.0)
        r.SetLight(W.LIGHT, 0.15, 0.85, i == 2)
        o = torch.zeros((res[1], res[0]), dtype=torch.int32, device="cuda")
        batch.add_svo(r, o)
        keep += [s, r]
        outs.append(("svo", r, o))
    for i, (levels, prec, res) in enumerate([(1, 0, (72, 40)), (2, 1, (100, 100)),
                                              (1, 3, (40, 56)), (2, 2, (64, 48))]):
        v = yoxel_mod.BrickVolume.noise(levels, 0.4, 1.4, 7 + i)
        g = v.upload(prec)
        pos, view = W.camera((0.3, 1.0, 0.4 + 0.2 * i))
        cam = (pos, view, (0, 0, 1), 60.0)
        o = torch.zeros((res[1], res[0], 4), dtype=torch.float32, device="cuda")
        batch.add_volume(g.desc(), cam, res[0], res[1], o, alpha_scale=1.5)
        keep += [v, g]
        outs.append(("brick", (g, cam, res), o))
    return batch, outs, keep


def test_batch_matches_separate_launches_and_renderers(yoxel_mod):
    import torch
    batch, outs, keep = build_batch(yoxel_mod, torch)
    n, rays = batch.info()
    assert n == 7 and rays > 0
    results = {}
    for mode in ("separate", "plain", "graph", "graph_again"):
        for _, _, o in outs:
            o.fill_(-1) if o.dtype == torch.int32 else o.fill_(float("nan"))
        if mode == "separate":
            batch.render_separate()
        else:
            batch.render(graph=mode.startswith("graph"))
        torch.cuda.synchronize()
        results[mode] = [o.clone() for _, _, o in outs]
    for mode in ("plain", "graph", "graph_again"):
        for a, b in zip(results["separate"], results[mode]):
            assert torch.equal(a.view(torch.int32), b.view(torch.int32)), mode
    # against the standalone entry points
    for (kind, src, _), got in zip(outs, results["graph"]):
        if kind == "svo":
            ref = src.render_outputs()["rgba"]
            assert torch.equal(ref, got)
        else:
            g, cam, res = src
            ref = yoxel_mod.render_volume(g.desc(), [cam], res[0], res[1], alpha_scale=1.5)[0]
            assert torch.equal(ref.view(torch.int32), got.view(torch.int32))


def test_autotuner_picks_and_caches(yoxel_mod, tmp_path, monkeypatch):
    import torch
    from yoxel import autotune
    from yoxel import workloads as W
    monkeypatch.setenv("YOXEL_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    s = W.spheres(7, seed=3, n_spheres=60)
    r = yoxel_mod.Renderer()
    r.SetScene(s)
    pos, view = W.camera()
    r.SetViewPos(pos)
    r.SetViewDir(view)
    r.SetResolution(128, 128)
    r.SetFOV(60.0)
    ref = r.render_outputs()["hit"]
    space = dict(block_threads=[128, 256], blocks_per_sm=[2, 4], smem_nodes=[0, 73],
                 tile_rays=[32])
    best, times = autotune.tune_renderer(r, "spheres7-128", space=space, reps=2)
    assert len(times) == 8 and best in [json.loads(k) for k in times]
    assert r.GetLaunchConfig()["block_threads"] == best["block_threads"]
    assert torch.equal(r.render_outputs()["hit"], ref)
    cache = json.load(open(tmp_path / "tune.json"))
    assert any(k.endswith("svo|spheres7-128") for k in cache)
    # second call is served from the cache
    best2, _ = autotune.tune_renderer(r, "spheres7-128", space=space, reps=2)
    assert best2 == best
    batch, outs, keep = build_batch(yoxel_mod, torch)
    bb, bt = autotune.tune_batch(batch, "mixed5", reps=1)
    assert bb in [json.loads(k) for k in bt]


@pytest.mark.parametrize("blocks_per_sm", [2, 3, 4])
@pytest.mark.parametrize("formats", [(0, 0), (1, 1), (2, 2), (3, 3), (3, 0), ()])
def test_every_batch_kernel_variant_matches_separate_launches(yoxel_mod, formats,
                                                              blocks_per_sm):
    """The batch kernel is compiled per register budget and per brick lattice
    format (one format shared by every volume, or all four for a mixed
    batch; an SVO-only batch takes the 8-byte format's kernel): every
    variant gives the per-scene frames bit for bit."""
    import torch
    from yoxel import workloads as W
    batch = yoxel_mod.Batch()
    keep, outs = [], []
    s = W.spheres(6, seed=21, n_spheres=30)
    r = yoxel_mod.Renderer()
    r.SetScene(s)
    pos, view = W.camera((0.9, 0.4, 0.5))
    r.SetViewPos(pos)
    r.SetViewDir(view)
    r.SetResolution(88, 72)
    r.SetFOV(60.0)
    r.SetLight(W.LIGHT, 0.15, 0.85, True)
    o = torch.zeros((72, 88), dtype=torch.int32, device="cuda")
    batch.add_svo(r, o)
    keep += [s, r]
    outs.append(o)
    for i, prec in enumerate(formats):
        v = yoxel_mod.BrickVolume.noise(1 + i, 0.4, 1.4, 31 + i)
        g = v.upload(prec)
        pos, view = W.camera((0.4, 1.0, 0.3 + 0.3 * i))
        o = torch.zeros((60, 84, 4), dtype=torch.float32, device="cuda")
        batch.add_volume(g.desc(), (pos, view, (0, 0, 1), 60.0), 84, 60, o, alpha_scale=1.3)
        keep += [v, g]
        outs.append(o)
    batch.set_launch_config(block_threads=128, blocks_per_sm=blocks_per_sm)
    results = {}
    for mode in ("separate", "graph"):
        for o in outs:
            o.fill_(-1) if o.dtype == torch.int32 else o.fill_(float("nan"))
        if mode == "separate":
            batch.render_separate()
        else:
            batch.render(graph=True)
        torch.cuda.synchronize()
        results[mode] = [o.clone() for o in outs]
    for a, b in zip(results["separate"], results["graph"]):
        assert torch.equal(a.view(torch.int32), b.view(torch.int32))
    assert (results["graph"][0] != 0).any()
