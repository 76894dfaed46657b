"""Parity at the benchmarked sizes: every workload bench.py times, on the
same seeded scenes and cameras, against the CPU oracle.

* cfg2: the 2048^3 terrain frame at 1920x1080 with one shadow ray per hit -
  hit ids, hit t, node-fetch counts of primary and shadow rays and RGBA8
  bit-exact with the FP32 oracle (the restatement of cell/ppu_renderer.cpp
  :18-70); rays whose hit a rounding tie inside the traversal decides (the
  FP64 traversal of the same FP32 rays disagrees) counted: 1.3e-4 at this
  depth, bounded here by 2e-4.
* cfg3: the 512^3 fp16 brick volume at 1024^2 - composited radiance within
  1e-5 relative (1e-6 absolute) of the FP64 march of the same FP32 rays
  (reaction/trace/trace.cu:83-139), except rays whose sample set a rounding
  tie decides (test_volume_gpu.compare_radiance), which stay under 1e-3.
* cfg4: the 128^3 learnable volume with its 64 cameras at 256^2 - forward
  radiance as cfg3; the adjoint of the L2 loss against the FP64 adjoint
  along the same rays over the whole pool (relative L2 error <= 1e-4);
  FP64 central differences of the loss of 8 of the cameras on 1000 seeded
  lattice points, against the FP64 adjoint and the GPU adjoint (relative L2
  error <= 1e-4).  Tie rays carry no gradient in these checks (their
  dL/drgba is set to 0 for every side).
* cfg5: the 32-scene batch of seed 1234 - every SVO frame (hit ids, hit t,
  fetch counts, RGBA8) bit-exact with the FP32 oracle, every brick frame
  within the cfg3 tolerance of the FP64 march.
"""
import os

import numpy as np
import pytest

from test_volume_gpu import compare_radiance, gpu_inputs
from volume_util import central_differences, gradient_at

pytestmark = pytest.mark.gpu

THREADS = max(1, os.cpu_count() or 1)
TIE_BUDGET = 1e-4


def to_np(t, view=None):
    a = t.cpu().numpy()
    return a.view(view) if view is not None else a


def test_cfg2_full_frame_bit_exact(yoxel_mod, oracle):
    from yoxel import workloads as W
    s = yoxel_mod.SVOScene.terrain(11, 10000, 2, 16, 1234)
    pos, view = W.camera()
    w, h = 1920, 1080
    r = yoxel_mod.Renderer()
    r.SetScene(s)
    r.SetViewPos(pos)
    r.SetViewDir(view)
    r.SetViewUp([0, 0, 1])
    r.SetResolution(w, h)
    r.SetFOV(60.0)
    r.SetLight(W.LIGHT, 0.15, 0.85, True)
    o = r.render_outputs()
    st = o.pop("stats")
    g = {k: to_np(v) for k, v in o.items()}
    ref = oracle.svo_render(s.nodes_u32, s.root, s.attrs_u8, pos, view, [0, 0, 1], 60.0, w, h,
                            W.LIGHT, shadows=True, threads=THREADS)
    for k in ("hit", "rgba", "fetches", "shadow_fetches"):
        diff = g[k].view(np.uint32) != ref[k]
        assert not diff.any(), f"{k}: {int(diff.sum())} pixels differ, first {np.argwhere(diff)[:3]}"
    assert np.array_equal(g["hit_t"].view(np.uint32), ref["hit_t"].view(np.uint32))
    hits = int((ref["hit"] != 0xFFFFFFFF).sum())
    assert st["hits"] == hits and st["shadow_rays"] == hits
    assert st["shadowed"] == int(ref["shadowed"].sum())
    assert hits > 0.3 * w * h
    # rounding ties inside the traversal: rays whose hit the FP64 traversal
    # of the same FP32 rays decides otherwise.  The kernel reproduces the
    # FP32 restatement on every ray (above), so this counts where the
    # reference's own FP32 arithmetic (slab midpoints carried down 11
    # levels, a few ulps of error each) decides the hit voxel: 1.3e-4 of the
    # rays of this 2048^3 frame, 5.7e-5 of the 256^3 one.
    h64, _ = oracle.svo_hits_f64_f32ray(s.nodes_u32, s.root, pos, view, [0, 0, 1], 60.0, w, h,
                                        threads=THREADS)
    ties = float((h64 != ref["hit"]).mean())
    assert ties < 2 * TIE_BUDGET, f"traversal tie rate {ties}"
    # and with the camera basis and ray directions in FP64 as well (ray
    # generation rounding moves rays by ~1e-7 relative: a looser bound)
    h64b, _ = oracle.svo_hits_f64(s.nodes_u32, s.root, pos, view, [0, 0, 1], 60.0, w, h,
                                  threads=THREADS)
    assert float((h64b != ref["hit"]).mean()) < 1e-3


def test_cfg3_full_frame_radiance(yoxel_mod, oracle):
    import torch
    from yoxel import workloads as W
    vol = yoxel_mod.BrickVolume.noise(3, 0.4, 1.4, 1234)
    gv = vol.upload(3)
    pos, view = W.camera()
    cam = (pos, view, (0, 0, 1), 60.0)
    w = h = 1024
    ns = torch.zeros((1, h, w), dtype=torch.int32, device="cuda")
    out = to_np(yoxel_mod.render_volume(gv.desc(), [cam], w, h, alpha_scale=1.0, step_vox=0.5,
                                        samples=ns))[0]
    ns = to_np(ns, np.uint32)[0]
    den, alb = gpu_inputs(vol, 3)
    ref, ns_ref, _, ties = oracle.brick_render_f64_f32ray(vol.grids, den, alb, vol.levels, pos,
                                                          view, (0, 0, 1), 60.0, w, h,
                                                          alpha_scale=1.0, step_vox=0.5,
                                                          threads=THREADS, ties=True)
    real, tie, worst = compare_radiance(out, ref, ns, ns_ref, ties)
    assert real == 0, f"{real} rays beyond tolerance (worst rel {worst:.3g})"
    assert tie <= 1e-3 * w * h, f"{tie} tie rays"
    assert (ref[..., 3] > 0.01).mean() > 0.2 and int(ns.sum()) > 0


@pytest.fixture(scope="module")
def cfg4(yoxel_mod, oracle):
    """The cfg4 problem of bench.py: volume, target, 64 cameras at 256^2,
    the forward of the learnable volume, dL/drgba of the L2 loss, and per
    camera the FP64 march of the same rays with its tie flags."""
    import torch
    from yoxel import workloads as W
    vol, tv, tgt_d, tgt_a, cams = W.cfg4_problem(2, 64, 1234)
    w = h = 256
    target = yoxel_mod.render_volume(yoxel_mod.torch_desc(tv, tgt_d, tgt_a),
                                     yoxel_mod.cameras(cams), w, h, 1.0, 0.5)
    packed = yoxel_mod.pack_volume(tv["density"], tv["albedo"])
    desc = yoxel_mod.torch_desc(tv, packed=packed)
    ns = torch.zeros((len(cams), h, w), dtype=torch.int32, device="cuda")
    rgba = yoxel_mod.render_volume(desc, yoxel_mod.cameras(cams), w, h, 1.0, 0.5, samples=ns)
    grad = 2.0 * (rgba - target)
    torch.cuda.synchronize()
    den, alb = gpu_inputs(vol, 1)
    refs = []
    for (p, d, up, fov) in cams:
        refs.append(oracle.brick_render_f64_f32ray(vol.grids, den, alb, vol.levels, p, d, up,
                                                   fov, w, h, alpha_scale=1.0, step_vox=0.5,
                                                   threads=THREADS, ties=True))
    ns = to_np(ns, np.uint32)
    # rays whose sample set a rounding tie decides carry no gradient below
    tie_rays = np.stack([(ns[i] != r[1]) | r[3] for i, r in enumerate(refs)])
    g_np = to_np(grad)
    g_np[tie_rays] = 0.0
    grad_nt = torch.from_numpy(g_np).cuda()
    return dict(vol=vol, tv=tv, cams=cams, w=w, h=h, desc=desc, rgba=rgba, grad=grad_nt,
                grad_np=g_np.astype(np.float64), ns=ns, refs=refs, tie_rays=tie_rays, den=den,
                alb=alb)


def test_cfg4_forward_radiance(cfg4):
    out = to_np(cfg4["rgba"])
    tie_total = 0
    for i, (ref, ns_ref, _, ties) in enumerate(cfg4["refs"]):
        real, tie, worst = compare_radiance(out[i], ref, cfg4["ns"][i], ns_ref, ties)
        assert real == 0, f"camera {i}: {real} rays beyond tolerance (worst rel {worst:.3g})"
        tie_total += tie
    w, h = cfg4["w"], cfg4["h"]
    assert tie_total <= 1e-3 * len(cfg4["cams"]) * w * h
    # the FP64 tie flags are conservative (a sample within 1e-6 relative of
    # any cell boundary): 6 % of these rays, the gradient checks keep the rest
    assert cfg4["tie_rays"].mean() < 0.1


def _gpu_adjoint(yoxel_mod, cfg4, cam_ids):
    import torch
    cams = [cfg4["cams"][i] for i in cam_ids]
    idx = torch.tensor(cam_ids, device="cuda")
    gd = torch.zeros_like(cfg4["tv"]["density"])
    ga = torch.zeros_like(cfg4["tv"]["albedo"])
    yoxel_mod.volume_backward(cfg4["desc"], yoxel_mod.cameras(cams), cfg4["w"], cfg4["h"],
                              cfg4["rgba"][idx].contiguous(), cfg4["grad"][idx].contiguous(),
                              gd, ga, 1.0, 0.5, fold=False)
    torch.cuda.synchronize()
    return (to_np(gd).reshape(-1).astype(np.float64), to_np(ga).reshape(-1).astype(np.float64))


def _oracle_adjoint(oracle, cfg4, cam_ids):
    vol, w, h = cfg4["vol"], cfg4["w"], cfg4["h"]
    rd = np.zeros(vol.nbricks * 729)
    ra = np.zeros(vol.nbricks * 729 * 3)
    for i in cam_ids:
        p, d, up, fov = cfg4["cams"][i]
        a, b = oracle.brick_backward_f64_f32ray(vol.grids, cfg4["den"], cfg4["alb"], vol.levels,
                                                p, d, up, fov, w, h, cfg4["grad_np"][i],
                                                alpha_scale=1.0, step_vox=0.5, threads=THREADS)
        rd += a
        ra += b
    return rd, ra


def test_cfg4_adjoint_all_cameras_matches_fp64(yoxel_mod, oracle, cfg4):
    ids = list(range(len(cfg4["cams"])))
    gd, ga = _gpu_adjoint(yoxel_mod, cfg4, ids)
    rd, ra = _oracle_adjoint(oracle, cfg4, ids)
    ed = np.linalg.norm(gd - rd) / np.linalg.norm(rd)
    ea = np.linalg.norm(ga - ra) / np.linalg.norm(ra)
    assert ed <= 1e-4 and ea <= 1e-4, (ed, ea)


def test_cfg4_central_differences_1000_voxels(yoxel_mod, oracle, cfg4):
    """L = sum over 8 of the cameras of dL/drgba . rgba (dL/drgba of the full
    L2 loss held fixed).  FP64 central differences (h = 1e-3, the float32
    perturbation actually stored taken as the step) on 1000 seeded owned
    lattice points, density and albedo (green), every copy of a point
    perturbed, against the FP64 adjoint and the GPU adjoint of the same L
    (kinks left out: volume_util.central_differences)."""
    vol, w, h = cfg4["vol"], cfg4["w"], cfg4["h"]
    cam_ids = list(range(0, 64, 8))
    rd, ra = _oracle_adjoint(oracle, cfg4, cam_ids)
    gd, ga = _gpu_adjoint(yoxel_mod, cfg4, cam_ids)
    rng = np.random.default_rng(1234)
    pts = [(int(rng.integers(0, vol.nbricks)),) + tuple(int(v) for v in rng.integers(0, 8, 3))
           for _ in range(1000)]
    fds, kinks = central_differences(oracle, vol, cfg4["den"], cfg4["alb"],
                                     [cfg4["cams"][i] for i in cam_ids],
                                     [cfg4["grad_np"][i] for i in cam_ids], w, h, pts,
                                     f32ray=True)
    for kind, ch, rg, gg in (("d", 1, rd, gd), ("a", 3, ra, ga)):
        fd = np.array([f for (_, f, _) in fds[kind]])
        an = np.array([gradient_at(rg, sl, ch, 0 if kind == "d" else 1)
                       for (_, _, sl) in fds[kind]])
        gp = np.array([gradient_at(gg, sl, ch, 0 if kind == "d" else 1)
                       for (_, _, sl) in fds[kind]])
        assert len(fd) > 500 and np.abs(fd).max() > 0, (kind, len(fd))
        e_ref = np.linalg.norm(an - fd) / np.linalg.norm(fd)
        e_gpu = np.linalg.norm(gp - fd) / np.linalg.norm(fd)
        zero = np.array([cfg4["den"][p[0], (p[1] * 9 + p[2]) * 9 + p[3]] == 0
                         for (p, _, _) in fds[kind]])
        info = (kind, e_ref, e_gpu, "zero-density points", int(zero.sum()),
                float(np.linalg.norm((gp - an)[zero]) / (np.linalg.norm(an[zero]) + 1e-30)),
                float(np.linalg.norm((gp - an)[~zero]) / (np.linalg.norm(an[~zero]) + 1e-30)))
        assert e_ref <= 1e-4, ("FP64 adjoint vs FD",) + info
        assert e_gpu <= 1e-4, ("GPU adjoint vs FD",) + info
    assert kinks < 0.5 * len(pts), kinks


def test_cfg5_batch_every_scene_matches_oracle(yoxel_mod, oracle):
    import torch
    from yoxel import workloads as W
    specs = W.cfg5_specs(1234, 32)
    batch, items = W.cfg5_batch(specs, 3, hits=True, keep_scenes=True)
    batch.render(graph=True)
    torch.cuda.synchronize()
    n_svo = n_brick = 0
    for k, it in enumerate(items):
        res = it["res"]
        pos, view, up, fov = it["cam"]
        if it["kind"] == "svo":
            s = it["scene"]
            ref = oracle.svo_render(s.nodes_u32, s.root, s.attrs_u8, pos, view, up, fov, res,
                                    res, W.LIGHT, shadows=False, threads=THREADS)
            for key, ref_v in (("hit", ref["hit"]), ("out", ref["rgba"]),
                               ("fetches", ref["fetches"])):
                diff = to_np(it[key], np.uint32) != ref_v
                assert not diff.any(), f"scene {k} ({it['spec']}): {key} differs at " \
                                       f"{int(diff.sum())} pixels"
            assert np.array_equal(to_np(it["hit_t"], np.uint32), ref["hit_t"].view(np.uint32))
            n_svo += 1
            it.pop("scene")
        else:
            vol = it["volume"]
            den, alb = gpu_inputs(vol, it["precision"])
            ref, ns_ref, _, ties = oracle.brick_render_f64_f32ray(
                vol.grids, den, alb, vol.levels, pos, view, up, fov, res, res,
                alpha_scale=1.0, step_vox=0.5, threads=THREADS, ties=True)
            ns = torch.zeros((1, res, res), dtype=torch.int32, device="cuda")
            yoxel_mod.render_volume(it["gpu_volume"].desc(), [it["cam"]], res, res,
                                    samples=ns)
            real, tie, worst = compare_radiance(to_np(it["out"]), ref,
                                                to_np(ns, np.uint32)[0], ns_ref, ties)
            assert real == 0, f"scene {k}: {real} rays beyond tolerance (worst {worst:.3g})"
            assert tie <= 1e-3 * res * res
            n_brick += 1
    assert n_svo + n_brick == 32 and n_svo > 0 and n_brick > 0
