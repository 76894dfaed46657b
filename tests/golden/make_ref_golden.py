"""Generates the reference-produced fixtures tests/golden/ref_*.npz (run
from the repo root where the reference checkout is present:
`python tests/golden/make_ref_golden.py`).

Unlike make_golden.py (the oracle's own outputs), these hold outputs of the
reference's code itself, compiled on the host by oracle/build_ref.py:

* ref_svo_*.npz - a seeded scene (VoxNode pool and leaf attributes), a
  camera, and per pixel what the reference CPU renderer
  (cell/ppu_renderer.cpp SimpleRenderer over a .vox file read by
  SVOData::Load, with the SPU FindFirstChild / GoNext) returns: the hit
  leaf's VoxData (0xFFFFFFFF for a miss), the hit t and the node fetches of
  RecTrace; the camera basis of RendererBase::InitRayDir too.
* ref_march_*.npz - a uint8 volume, its 64^3 brick marks, an eye point and
  unit ray directions, and the RGBA castRay (reaction/trace/trace.cu) returns
  for them, with the volume's texture filtered in software.

tests/test_ref_pin.py checks the oracle against them on any machine, and
tests/test_svo_gpu.py checks the CUDA path against the SVO ones, so both are
pinned to the reference without it being present.
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "yoxel-voxel_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import yoxel  # noqa: E402
from oracle import pyoracle, pyref  # noqa: E402


def camera(direction=(1.0, 0.7, 0.5), dist=1.5):
    d = np.asarray(direction, np.float64)
    d = d / np.linalg.norm(d)
    return (0.5 + dist * d).astype(np.float32), (-d).astype(np.float32)


def svo_case(name, nodes, root, attrs, pos, view, up, fov, width, height):
    scene = yoxel.SVOScene.from_arrays(nodes.view(yoxel.NODE_DTYPE), root,
                                       attrs.reshape(-1).view(yoxel.ATTR_DTYPE))
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "scene.vox")
        scene.save(path)
        data, t, fetches = pyref.ppu_render(path, pos, view, up, fov, width, height)
    d0, du, dv = pyref.ray_basis(view, up, fov, width, height)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), nodes=scene.nodes_u32.copy(),
                        root=np.uint32(scene.root), attrs=scene.attrs_u8.copy(),
                        pos=np.asarray(pos, np.float32), view=np.asarray(view, np.float32),
                        up=np.asarray(up, np.float32), fov=np.float32(fov), width=width,
                        height=height, data=data, t=t, fetches=fetches, dir0=d0, du=du, dv=dv)
    print(name, scene.node_count, "nodes", (data != 0xFFFFFFFF).mean(), "hit rate")


def march_case(name, n, seed, eye, fov, res, mark_all, offset=0.15):
    """A smooth seeded uint8 volume with a zero border; marks: every brick,
    or the bricks whose texel footprint (one texel of margin) holds a
    non-zero texel (the brick skipping of castRay)."""
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(*(np.arange(n) / (n - 1),) * 3, indexing="ij")
    a = rng.uniform(3, 9, 4)
    b = rng.uniform(0, 6.3, 4)
    f = 0.5 + 0.3 * np.sin(a[0] * x + b[0]) * np.cos(a[1] * y + b[1]) \
        + 0.3 * np.sin(a[2] * z + b[2]) * np.cos(a[3] * x + b[3]) - offset
    vol = np.round(np.clip(f, 0, 1) * 255).astype(np.uint8)
    vol[[0, -1], :, :] = 0
    vol[:, [0, -1], :] = 0
    vol[:, :, [0, -1]] = 0
    if mark_all:
        marks = np.ones((64, 64, 64), np.uint8)
    else:
        marks = np.zeros((64, 64, 64), np.uint8)
        for bz in range(64):
            for by in range(64):
                for bx in range(64):
                    lo = [int(np.floor(c / 64 * n - 0.5)) - 1 for c in (bz, by, bx)]
                    hi = [int(np.ceil((c + 1) / 64 * n - 0.5)) + 1 for c in (bz, by, bx)]
                    lo = [max(0, v) for v in lo]
                    hi = [min(n - 1, v) + 1 for v in hi]
                    marks[bz, by, bx] = vol[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]].any()
    eye = np.asarray(eye, np.float32)
    d0, du, dv = pyoracle.init_ray_dir_f32(0.5 - eye, [0, 0, 1], fov, res, res)
    dirs = []
    for yy in range(res):
        for xx in range(res):
            d = (d0 + du * np.float32(xx)) + dv * np.float32(yy)
            dirs.append(d / np.sqrt((d * d).sum()))
    dirs = np.asarray(dirs, np.float32)
    rgba = pyref.cast_rays(vol, marks, eye, dirs)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), volume=vol, marks=marks, eye=eye,
                        dirs=dirs, rgba=rgba)
    print(name, "marked", marks.mean(), "A > 0.5:", (rgba[:, 3] > 0.5).mean())


if __name__ == "__main__":
    from test_svo_gpu import deep_random_tree

    light_dir = (1.0, 0.7, 0.5)
    s = yoxel.SVOScene.spheres(6, 40, 2.0, 8.0, 77)
    pos, view = camera(light_dir)
    svo_case("ref_svo_spheres_d6", s.nodes_u32, s.root, s.attrs_u8, pos, view, [0, 0, 1],
             60.0, 80, 60)
    s = yoxel.SVOScene.terrain(6, 60, 1, 5, 8)
    svo_case("ref_svo_terrain_d6", s.nodes_u32, s.root, s.attrs_u8, pos, view, [0, 0, 1],
             70.0, 72, 56)
    # camera inside the volume, and an axis-aligned view (AdjustDir epsilon)
    s = yoxel.SVOScene.spheres(5, 20, 1.5, 5.0, 5)
    svo_case("ref_svo_inside_d5", s.nodes_u32, s.root, s.attrs_u8,
             np.array([0.41, 0.47, 0.52], np.float32), np.array([0.3, -1.0, 0.2], np.float32),
             [0, 0, 1], 90.0, 48, 40)
    svo_case("ref_svo_axis_d5", s.nodes_u32, s.root, s.attrs_u8,
             np.array([0.5, 0.5, 2.0], np.float32), np.array([0.0, 0.0, -1.0], np.float32),
             [0, 1, 0], 60.0, 33, 33)
    n, a = deep_random_tree(np.random.default_rng(5), levels=16)
    svo_case("ref_svo_deep16", n.view(np.uint32).reshape(-1), 0, a.reshape(-1),
             np.array([1.3, 1.1, 0.9], np.float32), np.array([-0.8, -0.6, -0.4], np.float32),
             [0, 0, 1], 70.0, 64, 48)
    march_case("ref_march_all_marks", 33, 3, [1.6, 1.2, 1.0], 45.0, 40, True)
    march_case("ref_march_skip_marks", 33, 4, [-0.7, 1.4, 0.9], 50.0, 40, False, offset=0.45)
