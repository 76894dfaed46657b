"""Boundary forms of the reference's interfaces.

* An SVO held in memory as the reference's SVOData holds it - leaves (and
  node data) carrying the packed 16-bit colour + 16-bit normal VoxData of
  reaction/report/main.tex:38,65 - is handed to the renderer directly
  (yv_set_scene_svo_packed): the frame equals that of the same pool read
  from a .vox file without an attribute section, and the FP32 oracle's frame
  of the decoded attributes.
* The brick march writes the uchar4 image of ntree's RunTrace
  (ntree/ntree_trace.cuh:27): every pixel float2uint (reaction/trace/
  utils.h:37-44) of the float frame, bit for bit."""
import numpy as np
import pytest

from conftest import LIGHT, camera_for

pytestmark = pytest.mark.gpu


def pack_pool(scene):
    """The scene's pool with every leaf's VoxData (and node data) in the
    reference's packed format: RGB565 colour, octahedral int8x2 normal."""
    nodes = scene.nodes_u32.reshape(-1, 10).copy()
    attrs = scene.attrs_u8.reshape(-1, 8)
    r, g, b = (attrs[:, i].astype(np.uint32) for i in range(3))
    c565 = ((r * 31 // 255) << 11) | ((g * 63 // 255) << 5) | (b * 31 // 255)
    n = attrs[:, 4:7].view(np.int8).astype(np.float64)
    n /= np.maximum(np.abs(n).sum(axis=1, keepdims=True), 1e-9)
    ox, oy = n[:, 0].copy(), n[:, 1].copy()
    neg = n[:, 2] < 0
    ox[neg], oy[neg] = ((1 - np.abs(n[neg, 1])) * np.sign(n[neg, 0]),
                        (1 - np.abs(n[neg, 0])) * np.sign(n[neg, 1]))
    qx = np.round(ox * 127).astype(np.int8).view(np.uint8).astype(np.uint32)
    qy = np.round(oy * 127).astype(np.int8).view(np.uint8).astype(np.uint32)
    packed = c565 | (qx << 16) | (qy << 24)
    for ch in range(8):
        leaf = ((nodes[:, 0] >> ch) & 1).astype(bool)
        nodes[leaf, 2 + ch] = packed[nodes[leaf, 2 + ch]]
    nodes[:, 1] = packed[0]  # node data: any packed value
    return nodes.reshape(-1)


def test_packed_pool_in_memory_renders_as_the_vox_file(yoxel_mod, oracle, tmp_path):
    import torch
    scene = yoxel_mod.SVOScene.spheres(7, 80, 2.0, 10.0, 31)
    packed = pack_pool(scene)
    pos, view = camera_for()
    w, h = 160, 120

    def frame(setup):
        r = yoxel_mod.Renderer()
        setup(r)
        r.SetViewPos(pos)
        r.SetViewDir(view)
        r.SetResolution(w, h)
        r.SetFOV(60.0)
        r.SetLight(LIGHT, 0.15, 0.85, True)
        o = r.render_outputs()
        o.pop("stats")
        return {k: v.cpu().numpy().view(np.uint32) for k, v in o.items()}

    root = scene.root
    a = frame(lambda r: r.SetSceneSVOPacked(packed.view(yoxel_mod.NODE_DTYPE), root))
    # the same pool as a .vox file without an attribute section
    p = tmp_path / "packed.vox"
    with open(p, "wb") as f:
        f.write(np.array([root, 0, 0, len(packed) // 10], np.uint32).tobytes())
        f.write(packed.astype(np.uint32).tobytes())
    b = frame(lambda r: r.SetScene(yoxel_mod.SVOScene.load(p)))
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    dec = yoxel_mod.SVOScene.from_packed(packed.view(yoxel_mod.NODE_DTYPE), root)
    o = oracle.svo_render(dec.nodes_u32, dec.root, dec.attrs_u8, pos, view, [0, 0, 1], 60.0, w,
                          h, LIGHT, shadows=True)
    for k in ("hit", "rgba", "fetches", "shadow_fetches"):
        assert np.array_equal(a[k], o[k]), k
    assert (a["hit"] != 0xFFFFFFFF).any()
    torch.cuda.synchronize()


def test_volume_rgba8_is_float2uint_of_the_float_frame(yoxel_mod):
    vol = yoxel_mod.BrickVolume.noise(2, 0.4, 1.4, 12)
    gv = vol.upload(3)
    cams = yoxel_mod.sphere_cameras(3)
    w, h = 96, 80
    f = yoxel_mod.render_volume(gv.desc(), cams, w, h).cpu().numpy()
    u8 = yoxel_mod.render_volume_rgba8(gv.desc(), cams, w, h).cpu().numpy().view(np.uint32)
    x = np.clip(f, np.float32(0), np.float32(1)).astype(np.float32)
    q = (x * np.float32(255.0)).astype(np.float32).astype(np.uint32)
    expect = q[..., 0] | (q[..., 1] << 8) | (q[..., 2] << 16) | (q[..., 3] << 24)
    assert np.array_equal(u8, expect)
    assert (q[..., 3] > 128).any()
