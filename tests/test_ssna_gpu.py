"""GPU parity of the screen-space normal approximation (SSNA) post passes
(yv_render_ssna) and the trace dump (yv_renderer_trace_dump) through the C
ABI.

Inputs of the oracle are the device's own unlit trace (albedo, hit distance,
stored normal), itself bit-exact with the FP32 trace oracle (test_svo_gpu).
Bar: blurred depth and normals bit-exact with the FP32 numpy restatement
(every step is a correctly rounded FP32 operation on both sides); colour
within 1 of 255 per channel (the specular power is powf on both sides, a few
ulp apart) and equal on at least 99.9 % of the pixels."""
import numpy as np
import pytest

from conftest import LIGHT, camera_for
from oracle import ssna as O

pytestmark = pytest.mark.gpu

W, H, FOV = 256, 192, 60.0


@pytest.fixture(scope="module")
def spheres(yoxel_mod):
    return yoxel_mod.SVOScene.spheres(8, 200, 4.0, 24.0, 1234)


def make_renderer(yoxel, scene, dist=1.5, direction=(1.0, 0.7, 0.5)):
    r = yoxel.Renderer()
    r.SetScene(scene)
    pos, view = camera_for(direction=direction, dist=dist)
    r.SetViewPos(pos)
    r.SetViewDir(view)
    r.SetViewUp([0, 0, 1])
    r.SetResolution(W, H)
    r.SetFOV(FOV)
    r.SetLight(LIGHT, 1.0, 0.0, False)  # unlit: rgba = albedo
    return r, pos


def unlit_trace(r):
    import torch
    dev = torch.device("cuda", 0)
    o = dict(rgba=torch.empty((H, W), dtype=torch.int32, device=dev),
             hit=torch.empty((H, W), dtype=torch.int32, device=dev),
             hit_t=torch.empty((H, W), dtype=torch.float32, device=dev),
             normal=torch.empty((H, W, 3), dtype=torch.float32, device=dev))
    r.render_async(**o)
    r.frame_stats()
    out = {k: v.cpu().numpy() for k, v in o.items()}
    out["rgba"] = out["rgba"].view(np.uint32)
    out["hit"] = out["hit"].view(np.uint32)
    return out


def run_ssna(r, params):
    import torch
    dev = torch.device("cuda", 0)
    dep = torch.empty((H, W), dtype=torch.float32, device=dev)
    nrm = torch.empty((H, W, 3), dtype=torch.float32, device=dev)
    rgba = r.render_ssna(params, depth=dep, normals=nrm)
    r.frame_stats()
    return rgba.cpu().numpy().view(np.uint32), dep.cpu().numpy(), nrm.cpu().numpy()


def oracle_frame(r, pos, tr, p):
    d0, du, dv = r.ray_basis()
    lights = [dict(pos=list(lt.pos), diffuse=list(lt.diffuse), specular=list(lt.specular),
                   attenuation=list(lt.attenuation)) for lt in p.lights if lt.enabled]
    return O.ssna_frame(tr["rgba"], tr["hit_t"], tr["normal"], pos, d0, du, dv,
                        float(np.float32(FOV)), passes=p.blur_passes,
                        voxel_size=p.voxel_size, edge_threshold=p.edge_threshold,
                        edge_pad=p.edge_pad, ssna=bool(p.ssna),
                        show_normals=bool(p.show_normals), ambient=list(p.ambient),
                        specular_exp=p.specular_exp, lights=lights)


def assert_close(got, want):
    g_rgba, g_dep, g_n = got
    o_rgba, o_dep, o_n = want
    bad_d = g_dep.view(np.uint32) != o_dep.view(np.uint32)
    assert bad_d.sum() == 0, f"{bad_d.sum()} depths differ, first {np.argwhere(bad_d)[:3]}"
    bad_n = (g_n.view(np.uint32) != o_n.view(np.uint32)).any(-1)
    assert bad_n.sum() == 0, f"{bad_n.sum()} normals differ, first {np.argwhere(bad_n)[:3]}"
    gc = g_rgba.view(np.uint8).reshape(H, W, 4).astype(np.int32)
    oc = o_rgba.view(np.uint8).reshape(H, W, 4).astype(np.int32)
    assert np.abs(gc - oc).max() <= 1
    assert (g_rgba == o_rgba).mean() >= 0.999


def fine_voxel(p):
    # a 2^8 scene's voxel size: the near pixels fall under the blur limits
    p.voxel_size = 1.0 / 256
    p.edge_threshold = 4.0 / 256


@pytest.mark.parametrize("case", ["default", "fine_voxel", "two_lights", "show_normals",
                                  "stored_normals", "close_up", "one_pass", "many_passes"])
def test_ssna_matches_oracle(yoxel_mod, spheres, case):
    r, pos = make_renderer(yoxel_mod, spheres, dist=0.9 if case == "close_up" else 1.5)
    p = r.ssna_params()
    if case != "default":
        fine_voxel(p)
    if case == "two_lights":
        r.set_point_light(p, 2, (0.2, 0.9, 1.1), diffuse=(1.0, 0.8, 0.6),
                          specular=(0.5, 0.5, 0.5), attenuation=(1.0, 10.0, 400.0))
        p.specular_exp = 24.0
        p.ambient[:] = [0.05, 0.1, 0.15]
    if case == "show_normals":
        p.show_normals = 1
    if case == "stored_normals":
        p.ssna = 0
    if case == "one_pass":
        p.blur_passes = 1
    if case == "many_passes":
        # more passes than the fused one-launch chain takes: one launch per pass
        p.blur_passes = 9
    tr = unlit_trace(r)
    hits = (tr["rgba"] >> 24) != 0
    assert hits.mean() > 0.2
    got = run_ssna(r, p)
    want = oracle_frame(r, pos, tr, p)
    assert_close(got, want)
    if case in ("fine_voxel", "close_up", "many_passes"):
        # the blur changed the depth of some pixels
        z0 = O.depth(tr["rgba"], tr["hit_t"], *r.ray_basis())
        assert (got[1][hits] != z0[hits]).mean() > 0.05


@pytest.mark.parametrize("passes", [3, 24])
def test_passes_beyond_the_nearest_depth_are_skipped_exactly(yoxel_mod, spheres, passes):
    """The nearest hit lies between the pass limits: the leading passes blur,
    the rest are skipped by the kernels (the limits fall below the frame's
    smallest depth), and the result is still the oracle's."""
    r, pos = make_renderer(yoxel_mod, spheres, dist=0.9)
    p = r.ssna_params()
    fine_voxel(p)
    p.blur_passes = passes
    tr = unlit_trace(r)
    hits = (tr["rgba"] >> 24) != 0
    z0 = O.depth(tr["rgba"], tr["hit_t"], *r.ray_basis())
    zl = O.zlimits(passes, p.voxel_size, float(np.float32(FOV)), W)
    zmin = z0[hits].min()
    if passes == 24:
        assert zl[0] >= zmin > zl[-1]  # some passes run, some do not
    got = run_ssna(r, p)
    want = oracle_frame(r, pos, tr, p)
    assert_close(got, want)


def test_frame_normal_output_is_the_leaf_normal(yoxel_mod, spheres):
    r, _ = make_renderer(yoxel_mod, spheres)
    tr = unlit_trace(r)
    hits = tr["hit"] != 0xFFFFFFFF
    ids, ch = tr["hit"][hits] >> 3, tr["hit"][hits] & 7
    nodes = spheres.nodes_u32.reshape(-1, 10)
    leaf = nodes[ids, 2 + ch]
    at = spheres.attrs[leaf]
    n = at["n"][:, :3].astype(np.float32)
    len2 = (n[:, 0] * n[:, 0] + n[:, 1] * n[:, 1]) + n[:, 2] * n[:, 2]
    ln = np.sqrt(len2)
    want = np.where(len2[:, None] > 0, n / np.where(ln > 0, ln, 1)[:, None], 0).astype(np.float32)
    assert np.array_equal(tr["normal"][hits].view(np.uint32), want.view(np.uint32))
    assert not tr["normal"][~hits].any()


def test_trace_dump_matches_frame(yoxel_mod, spheres, tmp_path):
    r, _ = make_renderer(yoxel_mod, spheres)
    tr = unlit_trace(r)
    hits = (tr["rgba"] >> 24) != 0
    dist, color, normal = r.trace_dump()
    assert np.array_equal(dist[hits].view(np.uint32), tr["hit_t"][hits].view(np.uint32))
    assert not dist[~hits].any()
    assert np.array_equal(color.reshape(H, W, 4).view(np.uint32)[..., 0], tr["rgba"])
    assert np.array_equal(normal.view(np.uint32), tr["normal"].view(np.uint32))
    base = r.DumpTraceData(str(tmp_path / "dmp_0"))
    assert base.endswith("_%dx%d" % (W, H))
    assert np.array_equal(np.fromfile(base + ".dist", np.float32).reshape(H, W), dist)
    assert np.fromfile(base + ".normal", np.float32).size == H * W * 3


def test_ssna_without_scene_is_an_error(yoxel_mod):
    from yoxel import _lib as L
    r = yoxel_mod.Renderer()
    r.SetResolution(8, 8)
    p = r.ssna_params()
    with pytest.raises(L.YvError):
        r.render_ssna(p)
