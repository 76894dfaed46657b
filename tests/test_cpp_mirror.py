"""The C++ mirror of SVOData / ISVORenderer (include/yv_svo_renderer.hpp),
compiled into a small caller shaped like the reference's cell/main.cpp.

CPU: the host-side API (generator, .vox save / load round trip, failed load
keeps the contents) and the NULL frame without a device.  GPU: one frame
through ISVORenderer equals the FP32 oracle's frame bit for bit."""
import os
import subprocess

import numpy as np
import pytest

from conftest import PKG, ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "render_svo.cpp")


def _build(tmp_path):
    exe = str(tmp_path / "render_svo")
    libdir = os.path.join(PKG, "yoxel")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", libdir, "-lyoxel", "-Wl,-rpath," + libdir]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_cpp_mirror_host_side(tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("host-only path checks the no-device behaviour")
    exe = _build(tmp_path)
    p = subprocess.run([exe, "host", str(tmp_path / "s.vox")], capture_output=True, text=True,
                       timeout=120)
    assert p.returncode == 0, (p.returncode, p.stdout, p.stderr)
    assert "frame null" in p.stdout


@pytest.mark.gpu
def test_cpp_mirror_renders_oracle_frame(tmp_path, oracle):
    exe = _build(tmp_path)
    vox, raw = str(tmp_path / "s.vox"), str(tmp_path / "f.raw")
    p = subprocess.run([exe, "gpu", vox, raw], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, (p.returncode, p.stdout, p.stderr)
    got = np.fromfile(raw, dtype=np.uint32).reshape(48, 64)
    import yoxel
    s = yoxel.SVOScene.load(vox)
    lv = np.array([0.3, 0.5, 0.8])
    light = (lv / np.sqrt(lv[0] * lv[0] + lv[1] * lv[1] + lv[2] * lv[2])).astype(np.float32)
    f32 = lambda *v: np.array(v, np.float32)
    ref = oracle.svo_render(s.nodes_u32, s.root, s.attrs_u8, f32(1.1, 0.45, 0.72),
                            f32(-0.6, 0.05, -0.22), f32(0, 0, 1), 55.0, 64, 48, light, 0.15,
                            0.85, True)
    assert np.array_equal(got, ref["rgba"].reshape(48, 64).astype(np.uint32))
    # the trace dump: distances of the hits, colours with alpha set on hits
    dist = np.fromfile(raw + ".dmp_64x48.dist", np.float32).reshape(48, 64)
    color = np.fromfile(raw + ".dmp_64x48.color", np.uint32).reshape(48, 64)
    normal = np.fromfile(raw + ".dmp_64x48.normal", np.float32).reshape(48, 64, 3)
    hits = ref["hit"].reshape(48, 64) != 0xFFFFFFFF
    assert np.array_equal(dist[hits], ref["hit_t"].reshape(48, 64)[hits])
    assert np.array_equal((color >> 24) != 0, hits)
    nl = np.linalg.norm(normal[hits], axis=-1)
    assert np.all((np.abs(nl - 1.0) < 1e-5) | (nl == 0)) and (nl > 0).mean() > 0.9
