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
