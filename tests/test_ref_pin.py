"""The oracle pinned against the reference itself.

oracle/build_ref.py compiles the reference's own renderer code on the host
(cell/ppu_renderer.cpp with renderer_base.h and svodata.h, the SPU tracer
cell/spu/trace_spu.cpp, the brick march reaction/trace/trace.cu), standing in
only for the headers its snapshot lacks.  tests/golden/make_ref_golden.py
froze what it returns into tests/golden/ref_*.npz, so these checks run on any
machine; where the reference checkout is present, live renders of larger
scenes are compared as well.

Bars: the camera basis, every pixel's hit (the leaf's VoxData), its t and
its node-fetch count bit-exact between the FP32 oracle and the reference CPU
renderer (and its SPU tracer); the oracle's FP64 march under the reference's
fixed transfer within 1e-5 absolute of castRay (FP32, t accumulated by
t += dt where the oracle takes t = k dt).
"""
import glob
import os
import tempfile

import numpy as np
import pytest

from conftest import LIGHT, ROOT, camera_for

GOLDEN = os.path.join(ROOT, "tests", "golden")


def _leaf_data(nodes_u32, hit):
    """VoxData of the hit leaves ((node << 3) | child) of the oracle, or
    0xFFFFFFFF for a miss, as the reference renderer reports hits."""
    nodes = np.asarray(nodes_u32, np.uint32).reshape(-1, 10)
    h = np.asarray(hit, np.uint32)
    out = np.full(h.shape, 0xFFFFFFFF, np.uint32)
    m = h != 0xFFFFFFFF
    out[m] = nodes[h[m] >> 3, 2 + (h[m] & 7)]
    return out


def _svo_fixtures():
    return sorted(glob.glob(os.path.join(GOLDEN, "ref_svo_*.npz")))


@pytest.mark.parametrize("path", _svo_fixtures(), ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_matches_reference_renderer_fixture(oracle, path):
    g = np.load(path)
    w, h = int(g["width"]), int(g["height"])
    d0, du, dv = oracle.init_ray_dir_f32(g["view"], g["up"], float(g["fov"]), w, h)
    for a, b in ((d0, g["dir0"]), (du, g["du"]), (dv, g["dv"])):
        assert np.array_equal(a.view(np.uint32), np.asarray(b, np.float32).view(np.uint32))
    o = oracle.svo_render(g["nodes"], int(g["root"]), g["attrs"], g["pos"], g["view"], g["up"],
                          float(g["fov"]), w, h, LIGHT)
    assert np.array_equal(_leaf_data(g["nodes"], o["hit"]), g["data"])
    assert np.array_equal(o["hit_t"].view(np.uint32), g["t"].view(np.uint32))
    assert np.array_equal(o["fetches"], g["fetches"])
    assert g["fetches"].sum() > 0


def _march_fixtures():
    return sorted(glob.glob(os.path.join(GOLDEN, "ref_march_*.npz")))


def oracle_march_as_reference(oracle, yoxel, volume_u8, eye, dirs):
    """The oracle's FP64 march of castRay's rays under castRay's transfer.

    castRay samples an N^3 texture in normalized coordinates (texel centres
    at (i + 0.5) / N, trilinear); the oracle's lattice holds the same N^3
    values at vertices k / (N - 1) of its unit cube.  The affine map q =
    (p - 0.5 / N) N / (N - 1) takes one onto the other; applied to the ray
    (origin and direction) it keeps the ray parameter t, so castRay's step
    dt = 0.5 / 256 is step_vox = (N - 1) 0.5 / 256 lattice cells.  The zero
    border of the volume makes the clamped margin outside the lattice empty
    in both."""
    n = volume_u8.shape[0]
    S = n - 1
    levels = {32: 1, 128: 2, 512: 3}[S]
    v = yoxel.BrickVolume.from_dense(levels, volume_u8.astype(np.float32) / np.float32(255.0))
    c, k = 0.5 / n, n / (n - 1)
    o = np.tile((np.asarray(eye, np.float64) - c) * k, (len(dirs), 1))
    d = np.asarray(dirs, np.float64) * k
    rgba, _ = oracle.brick_march_rays_f64(v.grids, v.density,
                                          np.zeros((v.nbricks, 729, 3), np.float32), levels, o,
                                          d, step_vox=S * 0.5 / 256, transfer=1)
    return rgba


@pytest.mark.parametrize("path", _march_fixtures(), ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_march_matches_reference_castray_fixture(oracle, yoxel_mod, path):
    g = np.load(path)
    ours = oracle_march_as_reference(oracle, yoxel_mod, g["volume"], g["eye"], g["dirs"])
    ref = g["rgba"].astype(np.float64)
    assert (ref[:, 3] > 0.5).any()
    assert np.abs(ours - ref).max() <= 1e-5


# ---- live comparisons where the reference checkout is present -------------
def _pyref():
    from oracle import pyref
    if not pyref.available():
        pytest.skip("reference checkout not present")
    return pyref


@pytest.mark.parametrize("scene,size,cam", [
    ("spheres8", (160, 120), "std"), ("terrain9", (128, 72), "std"),
    ("spheres8", (64, 48), "inside"), ("terrain9", (96, 64), "wide"),
])
def test_oracle_matches_reference_renderer_live(oracle, yoxel_mod, scene, size, cam):
    pyref = _pyref()
    s = (yoxel_mod.SVOScene.spheres(8, 200, 4.0, 24.0, 1234) if scene == "spheres8"
         else yoxel_mod.SVOScene.terrain(9, 2500, 2, 8, 77))
    pos, view = camera_for()
    fov = 60.0
    if cam == "inside":
        pos = np.array([0.41, 0.47, 0.52], np.float32)
        view = np.array([0.3, -1.0, 0.2], np.float32)
    elif cam == "wide":
        fov = 150.0
    w, h = size
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "scene.vox")
        s.save(p)
        data, t, fetches = pyref.ppu_render(p, pos, view, [0, 0, 1], fov, w, h)
        if h % 4 == 0:
            # TreadedRenderer: four row bands (cell/ppu_renderer.cpp:121-144)
            d4, t4, _ = pyref.ppu_render(p, pos, view, [0, 0, 1], fov, w, h, threaded=True)
            assert np.array_equal(d4, data) and np.array_equal(t4.view(np.uint32),
                                                               t.view(np.uint32))
    o = oracle.svo_render(s.nodes_u32, s.root, s.attrs_u8, pos, view, [0, 0, 1], fov, w, h,
                          LIGHT, threads=4)
    assert np.array_equal(_leaf_data(s.nodes_u32, o["hit"]), data)
    assert np.array_equal(o["hit_t"].view(np.uint32), t.view(np.uint32))
    assert np.array_equal(o["fetches"], fetches)
    # the reference SPU tracer (node cache, 16x16 blocks) agrees with both
    sd, st, sf = pyref.spu_render(s.nodes_u32, s.root, pos, view, [0, 0, 1], fov, w, h)
    assert np.array_equal(sd, data) and np.array_equal(sf, fetches)
    assert np.array_equal(st.view(np.uint32), t.view(np.uint32))
    assert (data != 0xFFFFFFFF).mean() > 0.01


def test_reference_fixtures_are_current(oracle):
    """Regenerating a fixture with the reference library gives the stored
    outputs (the fixtures are what the reference code returns)."""
    pyref = _pyref()
    g = np.load(os.path.join(GOLDEN, "ref_svo_spheres_d6.npz"))
    import yoxel
    scene = yoxel.SVOScene.from_arrays(g["nodes"].view(yoxel.NODE_DTYPE), int(g["root"]),
                                       g["attrs"].reshape(-1).view(yoxel.ATTR_DTYPE))
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "scene.vox")
        scene.save(p)
        data, t, fetches = pyref.ppu_render(p, g["pos"], g["view"], g["up"], float(g["fov"]),
                                            int(g["width"]), int(g["height"]))
    assert np.array_equal(data, g["data"]) and np.array_equal(fetches, g["fetches"])
    m = np.load(os.path.join(GOLDEN, "ref_march_skip_marks.npz"))
    rgba = pyref.cast_rays(m["volume"], m["marks"], m["eye"], m["dirs"])
    assert np.array_equal(rgba.view(np.uint32), m["rgba"].view(np.uint32))


def test_oracle_march_matches_reference_castray_live_128(oracle, yoxel_mod):
    """A 129^3 volume (the oracle's 128^3 lattice), every brick marked."""
    pyref = _pyref()
    n = 129
    z, y, x = np.meshgrid(*(np.arange(n) / (n - 1),) * 3, indexing="ij")
    f = 0.5 + 0.25 * np.sin(7 * x + 1) * np.cos(5 * y + 2) + 0.25 * np.sin(6 * z + 0.5) * \
        np.cos(4 * x)
    vol = np.round(np.clip(f, 0, 1) * 255).astype(np.uint8)
    vol[[0, -1], :, :] = 0
    vol[:, [0, -1], :] = 0
    vol[:, :, [0, -1]] = 0
    eye = np.array([1.7, 1.3, 1.1], np.float32)
    d0, du, dv = oracle.init_ray_dir_f32(0.5 - eye, [0, 0, 1], 40.0, 40, 40)
    dirs = []
    for yy in range(40):
        for xx in range(40):
            d = (d0 + du * np.float32(xx)) + dv * np.float32(yy)
            dirs.append(d / np.sqrt((d * d).sum()))
    dirs = np.asarray(dirs, np.float32)
    ref = pyref.cast_rays(vol, np.ones((64, 64, 64), np.uint8), eye, dirs).astype(np.float64)
    ours = oracle_march_as_reference(oracle, yoxel_mod, vol, eye, dirs)
    assert (ref[:, 3] > 0.5).mean() > 0.5
    assert np.abs(ours - ref).max() <= 2e-5


def test_integration_subclass_compiles_against_the_reference_headers(tmp_path):
    """The ISVORenderer subclass INTEGRATION.md gives a maintainer compiles
    against the reference's own cell/svorenderer.h and svodata.h (with the
    stand-ins for the headers the snapshot lacks) and the C ABI header."""
    import re
    import subprocess
    from oracle import pyref
    if not pyref.available():
        pytest.skip("reference checkout not present")
    txt = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    block = re.search(r"```cpp\n(#include \"svorenderer.h\".*?)```", txt, re.S).group(1)
    src = tmp_path / "gb300_renderer.cpp"
    src.write_text('#include "stdafx.h"\n#include <map>\n' + block)
    ref = pyref._builder().reference_root()
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only",
                        "-I" + os.path.join(ROOT, "oracle", "ref_shim"),
                        "-I" + os.path.join(ref, "cell"), "-I" + os.path.join(ROOT, "include"),
                        str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
