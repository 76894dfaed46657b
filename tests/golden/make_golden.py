"""Generates the golden fixtures under tests/golden/ (run from the repo root:
`python tests/golden/make_golden.py`).

Each .npz holds a small seeded scene (its VoxNode pool and leaf attributes,
so the fixture does not depend on the generator staying the same), the
camera, and the FP32 oracle's outputs for it.  tests/test_oracle_kat.py checks
the oracle still reproduces them; the GPU tests compare the CUDA path with
them.  The reference ships no scene data and no tracing tests, so these
fixtures freeze the restatement rather than reference outputs.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "yoxel-voxel_gb300"))

import yoxel  # noqa: E402
from oracle import pyoracle  # noqa: E402


def camera(direction=(1.0, 0.7, 0.5), dist=1.5):
    d = np.asarray(direction, np.float64)
    d = d / np.linalg.norm(d)
    return (0.5 + dist * d).astype(np.float32), (-d).astype(np.float32)


def make(name, scene, width, height, fov, shadows):
    pos, view = camera()
    light = np.array([0.3, 0.5, 0.8]) / np.linalg.norm([0.3, 0.5, 0.8])
    light = light.astype(np.float32)
    o = pyoracle.svo_render(scene.nodes_u32, scene.root, scene.attrs_u8, pos, view,
                            [0, 0, 1], fov, width, height, light, shadows=shadows)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), nodes=scene.nodes_u32.copy(),
                        root=np.uint32(scene.root), attrs=scene.attrs_u8.copy(), pos=pos,
                        view=view, fov=np.float32(fov), width=width, height=height,
                        light=light, shadows=shadows, **o)
    print(name, scene.node_count, "nodes", (o["hit"] != 0xFFFFFFFF).mean(), "hit rate")


if __name__ == "__main__":
    make("svo_spheres_d5", yoxel.SVOScene.spheres(5, 12, 1.5, 5.0, 99), 64, 48, 60.0, True)
    make("svo_terrain_d6", yoxel.SVOScene.terrain(6, 40, 1, 4, 5), 48, 40, 60.0, True)
