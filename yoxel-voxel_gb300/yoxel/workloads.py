"""Seeded synthetic workloads (the reference ships no scene data).

cfg1: 200 spheres in 256^3 (SVO depth 8), 512x512, Lambert, one light.
cfg2: 2048^3 value-noise terrain + 10k cubes, 1920x1080 + shadow rays.
cfg3: N=4 brick tree, 512^3, fp16 density (~20% brick occupancy), 1024^2.
cfg4: 128^3 fp32 learnable volume, 64 cameras at 256^2, fwd + bwd.
cfg5: 32 scenes of cfg1/cfg3 type, depth 6..11, resolutions 128^2..1024^2,
      one persistent launch vs 32 per-scene launches.
"""
import numpy as np

LIGHT = (np.array([0.3, 0.5, 0.8]) / np.linalg.norm([0.3, 0.5, 0.8])).astype(np.float32)


def camera(direction=(1.0, 0.7, 0.5), dist=1.5, center=(0.5, 0.5, 0.5)):
    """Camera at centre + dist*normalize(direction) looking at the centre."""
    d = np.asarray(direction, np.float64)
    d = d / np.linalg.norm(d)
    c = np.asarray(center, np.float64)
    return (c + dist * d).astype(np.float32), (-d).astype(np.float32)


def spheres(depth, seed=1234, n_spheres=200):
    """cfg1-type scene at any depth: radii 4..24 voxels at 256^3, scaled
    with the grid."""
    from .svo import SVOScene
    s = 2.0 ** (depth - 8)
    return SVOScene.spheres(depth, n_spheres, 4.0 * s, 24.0 * s, seed)


def brick_levels_for_depth(depth):
    """Grid levels of a cfg3-type volume standing in for SVO depth d
    (scene size 8*4^levels: 32^3, 128^3 or 512^3)."""
    return int(min(3, max(1, (depth - 3) // 2)))


def cfg5_specs(seed=1234, n=32):
    """n scene specs: kind, depth, resolution, seed (seeded draws)."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n):
        kind = "svo" if rng.random() < 0.5 else "brick"
        depth = int(rng.integers(6, 12))
        res = int(rng.choice([128, 256, 512, 1024]))
        cam_dir = rng.normal(size=3)
        cam_dir[2] = abs(cam_dir[2]) + 0.3
        specs.append(dict(kind=kind, depth=depth, res=res, seed=int(seed * 1000 + i),
                          cam_dir=tuple(float(v) for v in cam_dir)))
    return specs


def cfg5_batch(specs, precision=3, hits=False, keep_scenes=False):
    """The batch of `specs` (cfg5_specs): one yoxel.Batch with an SVO frame
    (spheres scene, Lambert, no shadows) or a brick-volume composite per
    spec, in spec order.  Returns (batch, items); each item is a dict with
    kind, spec, res, cam (pos, view, up, fov) and out (the batch's output
    tensor), plus for SVO items the renderer (the host scene too with
    keep_scenes=True; a depth-11 scene holds about 0.6 GB of host memory) and,
    with hits=True, the hit / hit_t / fetches tensors the batch also writes;
    for brick items the host volume and its device pool."""
    import torch

    from .batch import Batch
    from .renderer import Renderer
    from .volume import BrickVolume
    batch = Batch()
    items = []
    for sp in specs:
        res = sp["res"]
        pos, view = camera(sp["cam_dir"])
        cam = (pos, view, (0, 0, 1), 60.0)
        it = dict(kind=sp["kind"], spec=sp, res=res, cam=cam)
        if sp["kind"] == "svo":
            s = spheres(sp["depth"], seed=sp["seed"])
            r = Renderer()
            r.SetScene(s)
            r.SetViewPos(pos)
            r.SetViewDir(view)
            r.SetResolution(res, res)
            r.SetFOV(60.0)
            r.SetLight(LIGHT, 0.15, 0.85, False)
            out = torch.empty((res, res), dtype=torch.int32, device="cuda")
            extra = {}
            if hits:
                extra = dict(hit=torch.empty((res, res), dtype=torch.int32, device="cuda"),
                             hit_t=torch.empty((res, res), dtype=torch.float32, device="cuda"),
                             fetches=torch.empty((res, res), dtype=torch.int32, device="cuda"))
            batch.add_svo(r, out, **extra)
            it.update(renderer=r, out=out, **extra)
            if keep_scenes:
                it["scene"] = s
            del s
        else:
            v = BrickVolume.noise(brick_levels_for_depth(sp["depth"]), 0.4, 1.4, sp["seed"])
            gv = v.upload(precision)
            out = torch.empty((res, res, 4), dtype=torch.float32, device="cuda")
            batch.add_volume(gv.desc(), cam, res, res, out)
            it.update(volume=v, gpu_volume=gv, out=out, precision=precision)
        items.append(it)
    return batch, items


def cfg4_problem(levels=2, ncams=64, seed=1234):
    """The differentiable-volume workload: the noise volume as torch tensors
    (yoxel.BrickVolume.to_torch), the target volume (density and albedo
    + N(0, 0.1) from a CUDA generator seeded with `seed`, clamped to [0, 1],
    owners perturbed then aprons synced) and the cameras (Fibonacci sphere,
    radius 1.5).  Returns (volume, tv, target_density, target_albedo, cams)."""
    import ctypes as C

    import torch

    from . import _lib as L
    from .volume import BrickVolume, sphere_cameras, torch_desc
    vol = BrickVolume.noise(levels, 0.4, 1.4, seed)
    tv = vol.to_torch()
    g = torch.Generator(device="cuda").manual_seed(seed)
    tgt_d = (tv["density"] + 0.1 * torch.randn(tv["density"].shape, generator=g,
                                               device="cuda")).clamp_(0, 1)
    tgt_a = (tv["albedo"] + 0.1 * torch.randn(tv["albedo"].shape, generator=g,
                                              device="cuda")).clamp_(0, 1)
    L.check(L.lib.yv_volume_sync_aprons(C.byref(torch_desc(tv, tgt_d, tgt_a)),
                                        C.c_void_p(tgt_d.data_ptr()),
                                        C.c_void_p(tgt_a.data_ptr()), None), "sync")
    return vol, tv, tgt_d, tgt_a, sphere_cameras(ncams)
