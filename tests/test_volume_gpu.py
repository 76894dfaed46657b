"""GPU brick-volume march, adjoint and apron maintenance vs the FP64 oracle.

Bars: composited radiance within 1e-5 relative (+1e-6 absolute for values
near zero) of the FP64 oracle, except rays whose sample set differs by a
rounding tie (early-exit threshold or a cell boundary hit exactly), which are
counted and must stay under 1e-3 of the rays; gradient relative error
(L2 over the pool) <= 1e-4 against the FP64 adjoint."""
import numpy as np
import pytest

from volume_util import fold_numpy

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-5, 1e-6


def gpu_inputs(vol, precision):
    """Oracle-side float copies of exactly the values the GPU reads
    (precisions 0 and 3 store fp16 density, all store 8-bit albedo scaled by
    the fp32 constant 1/255)."""
    if precision in (0, 3):
        den = vol.density.astype(np.float16).astype(np.float32)
        alb = vol.albedo_u8.astype(np.float32) * np.float32(1.0 / 255.0)
    else:
        den = vol.density.astype(np.float32)
        alb = vol.albedo_u8.astype(np.float32) * np.float32(1.0 / 255.0)
    return den, alb


def cam_at(pos, fov=60.0):
    pos = np.asarray(pos, np.float32)
    return (pos, (0.5 - pos).astype(np.float32), (0, 0, 1), fov)


def compare_radiance(g, ref, ns_g, ns_ref, ties=None):
    """(rays beyond tolerance that no rounding tie explains, tie rays beyond
    tolerance, worst relative error of the former).  A tie ray samples a
    different set of points in FP32 and FP64: its sample count differs, or
    the FP64 march flags a sample, a cell exit or the early exit within a
    rounding step of a boundary (`ties`, oracle brick_render_f64_f32ray)."""
    g = g.astype(np.float64)
    err = np.abs(g - ref)
    ok = err <= RTOL * np.abs(ref) + ATOL
    bad_rays = ~ok.all(axis=-1)
    tie_rays = ns_g != ns_ref
    if ties is not None:
        tie_rays = tie_rays | ties
    tie = bad_rays & tie_rays
    real = bad_rays & ~tie
    rel = (err / (RTOL * np.abs(ref) + ATOL)).max(axis=-1) * RTOL
    worst = float(rel[real].max()) if real.any() else 0.0
    return int(real.sum()), int(tie.sum()), worst


@pytest.mark.parametrize("precision", [0, 1, 2, 3])
def test_forward_matches_fp64_oracle(yoxel_mod, oracle, precision):
    import torch
    vol = yoxel_mod.BrickVolume.noise(2, 0.4, 1.4, 21)
    gv = vol.upload(precision)
    desc = gv.desc()
    w, h = 96, 80
    cams = [cam_at([1.6, 1.3, 1.1]), cam_at([-0.7, 0.4, 0.9], 50.0)]
    ns = torch.zeros((len(cams), h, w), dtype=torch.int32, device="cuda")
    out = yoxel_mod.render_volume(desc, cams, w, h, alpha_scale=1.0, step_vox=0.5,
                                  samples=ns).cpu().numpy()
    ns = ns.cpu().numpy().view(np.uint32)
    den, alb = gpu_inputs(vol, precision)
    tot_rays = 0
    for i, (p, d, up, fov) in enumerate(cams):
        # FP64 march of the same FP32 primary rays (ray generation itself is
        # pinned bit-exactly by the SVO tests)
        ref, ns_ref, _ = oracle.brick_render_f64_f32ray(vol.grids, den, alb, vol.levels, p, d,
                                                        up, fov, w, h, alpha_scale=1.0,
                                                        step_vox=0.5)
        real, tie, worst = compare_radiance(out[i], ref, ns[i], ns_ref)
        assert real == 0, f"cam {i}: {real} rays beyond tolerance (worst rel {worst:.3g})"
        assert tie <= 1e-3 * w * h, f"cam {i}: {tie} tie rays"
        assert ref[..., 3].max() > 0.5
        tot_rays += w * h


def test_forward_known_answer(yoxel_mod):
    """Constant density 0.5, alpha_scale 1: A = 1 - 0.5^7 after 7 samples."""
    s = 33
    vol = yoxel_mod.BrickVolume.from_dense(1, np.full((s, s, s), 0.5, np.float32),
                                           np.full((s, s, s, 3), 128, np.uint8))
    gv = vol.upload(1)
    out = yoxel_mod.render_volume(gv.desc(), [cam_at([-1.0, 0.5, 0.5], 10.0)], 4, 4,
                                  alpha_scale=1.0).cpu().numpy()
    a = np.float32(0.0)
    for _ in range(7):
        a = np.float32(a + np.float32(np.float32(1) - a) * np.float32(0.5))
    assert np.all(out[..., 3] == a)
    assert np.allclose(out[..., 0], (128 / 255) * (1 - 0.5 ** 7), rtol=1e-6)


def test_samples_and_bricks_counters(yoxel_mod, oracle):
    import torch
    vol = yoxel_mod.BrickVolume.noise(1, 0.4, 1.4, 3)
    gv = vol.upload(1)
    w, h = 48, 48
    ns = torch.zeros((1, h, w), dtype=torch.int32, device="cuda")
    nb = torch.zeros((1, h, w), dtype=torch.int32, device="cuda")
    c = cam_at([1.6, 1.3, 1.1])
    yoxel_mod.render_volume(gv.desc(), [c], w, h, samples=ns, bricks=nb)
    den, alb = gpu_inputs(vol, 1)
    _, ns_ref, nb_ref = oracle.brick_render_f64(vol.grids, den, alb, 1, c[0], c[1], c[2], c[3],
                                                w, h)
    ns = ns.cpu().numpy()[0].view(np.uint32)
    nb = nb.cpu().numpy()[0].view(np.uint32)
    assert (ns != ns_ref).mean() < 1e-2 and (nb != nb_ref).mean() < 1e-2
    assert ns.sum() > 0


def test_pack_volume_bit_exact(yoxel_mod):
    import torch
    vol = yoxel_mod.BrickVolume.noise(1, 0.4, 1.4, 3)
    tv = vol.to_torch()
    p = yoxel_mod.pack_volume(tv["density"], tv["albedo"])
    torch.cuda.synchronize()
    ref = np.concatenate([tv["albedo"].cpu().numpy().reshape(-1, 3),
                          tv["density"].cpu().numpy().reshape(-1, 1)], axis=1)
    assert p.shape == (vol.nbricks, 729, 4)
    assert np.array_equal(p.cpu().numpy().reshape(-1, 4).view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("packed", [False, True])
def test_backward_matches_fp64_adjoint(yoxel_mod, oracle, packed):
    import torch
    vol = yoxel_mod.BrickVolume.noise(1, 0.4, 1.4, 3)
    tv = vol.to_torch()
    if packed:
        pk = yoxel_mod.pack_volume(tv["density"], tv["albedo"])
        desc = yoxel_mod.torch_desc(tv, packed=pk)
    else:
        desc = yoxel_mod.torch_desc(tv)
    w, h = 40, 32
    cams = [cam_at([1.6, 1.3, 1.1]), cam_at([-0.8, 0.3, 0.2], 45.0)]
    rgba = yoxel_mod.render_volume(desc, cams, w, h, alpha_scale=2.0)
    rng = np.random.default_rng(5)
    g = rng.standard_normal((len(cams), h, w, 4)).astype(np.float32)
    gd = torch.zeros_like(tv["density"])
    ga = torch.zeros_like(tv["albedo"])
    yoxel_mod.volume_backward(desc, cams, w, h, rgba, torch.from_numpy(g).cuda(), gd, ga,
                              alpha_scale=2.0, fold=False)
    den, alb = gpu_inputs(vol, 1)
    rd = np.zeros(vol.nbricks * 729)
    ra = np.zeros(vol.nbricks * 729 * 3)
    for i, (p, d, up, fov) in enumerate(cams):
        a, b = oracle.brick_backward_f64(vol.grids, den, alb, 1, p, d, up, fov, w, h,
                                         g[i].astype(np.float64), alpha_scale=2.0)
        rd += a
        ra += b
    gd = gd.cpu().numpy().reshape(-1).astype(np.float64)
    ga = ga.cpu().numpy().reshape(-1).astype(np.float64)
    ed = np.linalg.norm(gd - rd) / np.linalg.norm(rd)
    ea = np.linalg.norm(ga - ra) / np.linalg.norm(ra)
    assert ed < 1e-4 and ea < 1e-4, (ed, ea)


def test_apron_fold_and_sync(yoxel_mod):
    import torch
    vol = yoxel_mod.BrickVolume.noise(1, 0.4, 1.4, 4)
    tv = vol.to_torch()
    desc = yoxel_mod.torch_desc(tv)
    rng = np.random.default_rng(2)
    gd = rng.standard_normal(vol.nbricks * 729).astype(np.float32)
    ga = rng.standard_normal(vol.nbricks * 729 * 3).astype(np.float32)
    tgd = torch.from_numpy(gd.copy()).cuda()
    tga = torch.from_numpy(ga.copy()).cuda()
    import ctypes as C
    from yoxel import _lib as L
    L.check(L.lib.yv_volume_fold_aprons(C.byref(desc), C.c_void_p(tgd.data_ptr()),
                                        C.c_void_p(tga.data_ptr()), None), "fold")
    torch.cuda.synchronize()
    assert np.allclose(tgd.cpu().numpy(), fold_numpy(vol, gd, 1), atol=1e-5)
    assert np.allclose(tga.cpu().numpy(), fold_numpy(vol, ga, 3), atol=1e-5)
    # sync: perturb owners, then aprons must repeat them again
    den = tv["density"].clone()
    den[:, 0] += 0.25
    L.check(L.lib.yv_volume_sync_aprons(C.byref(yoxel_mod.torch_desc(tv, den)),
                                        C.c_void_p(den.data_ptr()), None, None), "sync")
    d = den.cpu().numpy().reshape(-1, 9, 9, 9)
    up = vol.neighbors(True)
    for b in range(vol.nbricks):
        if up[b, 0] >= 0:
            assert np.array_equal(d[b, :, :, 8], d[up[b, 0], :, :, 0])


def naive_torch_march(torch, vol, den_t, alb_t, cam, w, h, alpha_scale, step_vox, oracle):
    """Plain PyTorch FP64 ray-marcher over the same sample positions (found
    by a Python restatement of the DDA) for the autograd cross-check."""
    d0, du, dv = oracle.init_ray_dir_f64(cam[1], cam[2], cam[3], w, h)
    S = 8 * 4 ** vol.levels
    grids = vol.grids
    nbc = 4 ** vol.levels
    dt = step_vox / S

    def lookup(c):
        node = 0
        for lev in range(vol.levels):
            sh = 2 * (vol.levels - 1 - lev)
            r = int(grids[node, ((((c[2] >> sh) & 3) * 4 + ((c[1] >> sh) & 3)) * 4 +
                                 ((c[0] >> sh) & 3))])
            if r & 0x80000000:
                return -1
            if r & 0x40000000:
                return r & 0x3FFFFFFF
            node = r
        return -1

    out = []
    o = np.asarray(cam[0], np.float64)
    for y in range(h):
        for x in range(w):
            d = d0 + du * x + dv * y
            d = d / np.sqrt((d * d).sum())
            d = np.where(np.abs(d) < 1e-5, np.copysign(1e-5, d), d)
            inv = 1.0 / d
            lo, hi = (0 - o) * inv, (1 - o) * inv
            t1, t2 = np.minimum(lo, hi), np.maximum(lo, hi)
            te, tx_ = max(t1.max(), 0.0), t2.min()
            C = torch.zeros(3, dtype=torch.float64)
            A = torch.zeros((), dtype=torch.float64)
            if tx_ >= 0 and te <= tx_:
                h_ = 8.0 / S
                cell = [min(max(int(np.floor((o[i] + te * d[i]) / h_)), 0), nbc - 1)
                        for i in range(3)]
                t_in, done = te, False
                while not done:
                    txs = [((cell[i] + 1 if d[i] > 0 else cell[i]) * h_ - o[i]) * inv[i]
                           for i in range(3)]
                    e = int(np.argmin(txs))
                    t_out = txs[e]
                    b = lookup(cell)
                    if b >= 0:
                        k = int(np.ceil(t_in / dt))
                        while k * dt < t_out:
                            t = k * dt
                            ll = (o + t * d) * S - 8 * np.asarray(cell)
                            i0 = np.clip(np.floor(ll).astype(int), 0, 7)
                            f = np.clip(ll - i0, 0, 1)
                            sig = 0
                            col = 0
                            for j in range(8):
                                dx_, dy_, dz_ = j & 1, (j >> 1) & 1, j >> 2
                                wgt = ((f[0] if dx_ else 1 - f[0]) * (f[1] if dy_ else 1 - f[1]) *
                                       (f[2] if dz_ else 1 - f[2]))
                                idx = b * 729 + ((i0[2] + dz_) * 9 + i0[1] + dy_) * 9 + i0[0] + dx_
                                sig = sig + wgt * den_t[idx]
                                col = col + wgt * alb_t[idx]
                            a = torch.clamp(sig * alpha_scale, 0, 1)
                            wt = (1 - A) * a
                            C = C + wt * col
                            A = A + wt
                            k += 1
                            if A.item() > 0.99:
                                done = True
                                break
                    if done:
                        break
                    t_in = t_out
                    cell[e] += 1 if d[e] > 0 else -1
                    if not 0 <= cell[e] < nbc:
                        break
            out.append(torch.cat([C, A.reshape(1)]))
    return torch.stack(out).reshape(h, w, 4)


def test_autograd_function_matches_naive_torch_marcher(yoxel_mod, oracle):
    import torch
    vol = yoxel_mod.BrickVolume.noise(1, 0.4, 1.4, 3)
    tv = vol.to_torch()
    den = tv["density"].clone().requires_grad_(True)
    alb = tv["albedo"].clone().requires_grad_(True)
    w, h = 10, 8
    cam = cam_at([1.6, 1.3, 1.1], 40.0)
    rgba = yoxel_mod.volume_march(den, alb, tv, [cam], w, h, 2.0, 0.5)
    rng = np.random.default_rng(9)
    wts = torch.from_numpy(rng.standard_normal((1, h, w, 4)).astype(np.float32)).cuda()
    (rgba * wts).sum().backward()
    # naive marcher differentiates every pool slot separately; fold its result
    den64 = torch.from_numpy(den.detach().cpu().numpy().reshape(-1).astype(np.float64))
    alb64 = torch.from_numpy(alb.detach().cpu().numpy().reshape(-1, 3).astype(np.float64))
    den64.requires_grad_(True)
    alb64.requires_grad_(True)
    ref = naive_torch_march(torch, vol, den64, alb64, cam, w, h, 2.0, 0.5, oracle)
    assert np.allclose(ref.detach().numpy(), rgba.detach().cpu().numpy()[0], rtol=1e-4,
                       atol=1e-6)
    (ref * wts.cpu().double()[0]).sum().backward()
    gref_d = fold_numpy(vol, den64.grad.numpy(), 1)
    gref_a = fold_numpy(vol, alb64.grad.numpy().reshape(-1), 3)
    gd = den.grad.cpu().numpy().reshape(-1)
    ga = alb.grad.cpu().numpy().reshape(-1)
    assert np.linalg.norm(gd - gref_d) / np.linalg.norm(gref_d) < 1e-4
    assert np.linalg.norm(ga - gref_a) / np.linalg.norm(gref_a) < 1e-4


def test_more_cameras_than_one_launch_holds(yoxel_mod):
    """70 cameras run as launches of 64 + 6: the frames equal per-camera
    renders bit for bit, and the adjoint of all 70 equals the sum of the
    adjoints of the two groups."""
    import torch
    vol = yoxel_mod.BrickVolume.noise(1, 0.4, 1.4, 8)
    tv = vol.to_torch()
    desc = yoxel_mod.torch_desc(tv)
    cams = yoxel_mod.sphere_cameras(70)
    w, h = 16, 12
    out = yoxel_mod.render_volume(desc, cams, w, h)
    for i in (0, 63, 64, 69):
        one = yoxel_mod.render_volume(desc, [cams[i]], w, h)[0]
        assert torch.equal(one.view(torch.int32), out[i].view(torch.int32))
    g = torch.randn(out.shape, generator=torch.Generator(device="cuda").manual_seed(3),
                    device="cuda")
    gd = torch.zeros_like(tv["density"])
    ga = torch.zeros_like(tv["albedo"])
    yoxel_mod.volume_backward(desc, cams, w, h, out, g, gd, ga, fold=False)
    gd2 = torch.zeros_like(gd)
    ga2 = torch.zeros_like(ga)
    for lo, hi in ((0, 40), (40, 70)):
        yoxel_mod.volume_backward(desc, cams[lo:hi], w, h, out[lo:hi].contiguous(),
                                  g[lo:hi].contiguous(), gd2, ga2, fold=False)
    # atomics add in a different order: compare as relative L2 error
    assert float((gd - gd2).norm() / gd.norm()) < 1e-5
    assert float((ga - ga2).norm() / ga.norm()) < 1e-5
    assert gd.abs().sum() > 0


@pytest.mark.parametrize("precision", [0, 1, 2, 3])
def test_cell_mask_and_empty_cell_skipping(yoxel_mod, precision):
    """The occupancy mask of a library-owned pool marks exactly the trilinear
    cells with a non-zero density corner (as stored: fp16 formats round),
    and skipping the samples of unmarked cells changes no output bit: the
    same frame, sample counts included, with the mask removed."""
    import torch
    vol = yoxel_mod.BrickVolume.noise(2, 0.4, 1.4, 17)
    gv = vol.upload(precision)
    desc = gv.desc()
    assert desc.cell_mask
    nb = vol.nbricks

    class _DeviceWords:  # a view of the library's device array
        __cuda_array_interface__ = {"shape": (nb * 16,), "typestr": "<i4",
                                    "data": (desc.cell_mask, False), "version": 2}

    got = torch.as_tensor(_DeviceWords(), device="cuda").cpu().numpy().view(np.uint32)
    den, _ = gpu_inputs(vol, precision)
    nz = den.reshape(nb, 9, 9, 9) != 0
    cell = np.zeros((nb, 8, 8, 8), bool)
    for j in range(8):
        dx, dy, dz = j & 1, (j >> 1) & 1, j >> 2
        cell |= nz[:, dz:dz + 8, dy:dy + 8, dx:dx + 8]
    expect = np.zeros((nb, 16), np.uint32)
    for z in range(8):
        for y in range(8):
            for x in range(8):
                expect[:, z * 2 + (y >> 2)] |= cell[:, z, y, x].astype(np.uint32) << np.uint32(
                    ((y & 3) << 3) | x)
    assert np.array_equal(got.reshape(nb, 16), expect)
    assert 0 < cell.mean() < 1
    cams = [cam_at([1.6, 1.3, 1.1]), cam_at([-0.7, 0.4, 0.9], 50.0)]
    w, h = 96, 80
    outs = []
    for use_mask in (True, False):
        d = gv.desc()
        if not use_mask:
            d.cell_mask = None
        ns = torch.zeros((2, h, w), dtype=torch.int32, device="cuda")
        rgba = yoxel_mod.render_volume(d, cams, w, h, samples=ns)
        outs.append((rgba.cpu().numpy().view(np.uint32), ns.cpu().numpy()))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def _device_words(ptr, n):
    import torch

    class _Words:  # a view of the library's device array
        __cuda_array_interface__ = {"shape": (n,), "typestr": "<i4", "data": (ptr, False),
                                    "version": 2}

    return torch.as_tensor(_Words(), device="cuda").cpu().numpy().view(np.uint32)


def expected_brick_bits(vol):
    nb = 4 ** vol.levels
    bits = np.zeros(((nb ** 3 + 31) // 32,), np.uint32)
    c = np.asarray(vol.cells, np.int64).reshape(-1, 3)
    ci = (c[:, 2] * nb + c[:, 1]) * nb + c[:, 0]
    np.bitwise_or.at(bits, ci >> 5, (np.uint32(1) << (ci & 31).astype(np.uint32)))
    return bits


@pytest.mark.parametrize("precision", [0, 1, 2, 3])
def test_brick_bits_and_cheap_empty_cells(yoxel_mod, precision):
    """The brick bitmap of a library-owned pool has exactly the cells of its
    bricks set (uploads, device builds and the learnable copy alike), and
    rendering without it gives the same frame bit for bit, sample and brick
    counters included."""
    import torch
    vol = yoxel_mod.BrickVolume.noise(2, 0.4, 1.4, 23)
    want = expected_brick_bits(vol)
    assert 0 < np.unpackbits(want.view(np.uint8)).sum() < 4 ** 6
    gv = vol.upload(precision)
    desc = gv.desc()
    assert desc.brick_bits
    assert np.array_equal(_device_words(desc.brick_bits, len(want)), want)
    tv = vol.to_torch()
    assert np.array_equal(tv["brick_bits"].cpu().numpy().view(np.uint32), want)
    cams = [cam_at([1.6, 1.3, 1.1]), cam_at([-0.7, 0.4, 0.9], 50.0), cam_at([0.5, 0.5, 0.5])]
    w, h = 96, 80
    outs = []
    for use_bits in (True, False):
        d = gv.desc()
        if not use_bits:
            d.brick_bits = None
        ns = torch.zeros((len(cams), h, w), dtype=torch.int32, device="cuda")
        nbk = torch.zeros((len(cams), h, w), dtype=torch.int32, device="cuda")
        rgba = yoxel_mod.render_volume(d, cams, w, h, samples=ns, bricks=nbk)
        outs.append([rgba.cpu().numpy().view(np.uint32), ns.cpu().numpy(), nbk.cpu().numpy()])
    for a, b in zip(*outs):
        assert np.array_equal(a, b)
    assert outs[0][2].sum() > 0


@pytest.mark.parametrize("levels", [1, 3])
def test_brick_bits_other_tree_depths(yoxel_mod, levels):
    """The bitmap at the smallest tree (4^3 brick cells, two words) and at a
    512^3 volume; an empty tree gives an all-zero bitmap."""
    import torch
    from yoxel import _lib as L
    vol = yoxel_mod.BrickVolume.noise(levels, 0.4, 1.4, 29)
    want = expected_brick_bits(vol)
    gv = vol.upload(3)
    assert np.array_equal(_device_words(gv.desc().brick_bits, len(want)), want)
    got = yoxel_mod.brick_bits(gv.desc()).cpu().numpy().view(np.uint32)
    assert np.array_equal(got, want)
    n = 8 * 4 ** levels + 1
    empty = yoxel_mod.BrickVolume.from_dense(levels, np.zeros((n, n, n), np.float32))
    assert empty.nbricks == 0
    tv = empty.to_torch()
    assert not tv["brick_bits"].any()
    d = yoxel_mod.torch_desc(tv)
    out = yoxel_mod.render_volume(d, [cam_at([1.6, 1.3, 1.1])], 16, 16)
    assert not out.any()


@pytest.mark.parametrize("world", [1, 3, 4])
def test_volume_tile_ranges_merge_to_the_full_frame(yoxel_mod, world):
    """A volume frame split into warp-tile ranges of equal estimated cost
    (the multi-GPU shards of one frame) renders the full frame bit for bit
    once the ranges are merged - radiance, samples and bricks - and a range
    writes only its own tiles."""
    import torch
    from yoxel import _lib as L
    from yoxel import parallel as P
    vol = yoxel_mod.BrickVolume.noise(2, 0.4, 1.4, 31)
    gv = vol.upload(3)  # the device pool lives as long as this object
    d = gv.desc()
    cams = [cam_at([1.6, 1.3, 1.1]), cam_at([-0.7, 0.4, 0.9], 50.0)]
    w, h = 100, 60
    ns = torch.zeros((2, h, w), dtype=torch.int32, device="cuda")
    nb = torch.zeros((2, h, w), dtype=torch.int32, device="cuda")
    full = yoxel_mod.render_volume(d, cams, w, h, samples=ns, bricks=nb)
    per_cam = yoxel_mod.volume_tile_count(w, h)
    costs = P.volume_tile_costs(ns.cpu().numpy(), w, h)
    assert len(costs) == 2 * per_cam
    ranges = P.partition_volume_tiles(costs, world)
    out = torch.full((2, h, w, 4), -5.0, device="cuda")
    ns2 = torch.full((2, h, w), -5, dtype=torch.int32, device="cuda")
    nb2 = torch.full((2, h, w), -5, dtype=torch.int32, device="cuda")
    ox, oy = P.volume_tile_order(w, h)
    for k, (tb, te) in enumerate(ranges):
        yoxel_mod.render_volume_tiles(d, cams, w, h, tb, te, out, samples=ns2, bricks=nb2)
        if k == 0 and world > 1:
            written = np.zeros((2, h, w), bool)
            for t in range(tb, te):
                c, i = divmod(t, per_cam)
                written[c, oy[i] * 4:oy[i] * 4 + 4, ox[i] * 8:ox[i] * 8 + 8] = True
            got = ns2.cpu().numpy()
            assert (got[~written] == -5).all() and (got[written] != -5).all()
    assert torch.equal(out.view(torch.int32), full.view(torch.int32))
    assert torch.equal(ns2, ns) and torch.equal(nb2, nb)
    # an empty range writes nothing; a range past the frames is refused
    out.fill_(-5.0)
    yoxel_mod.render_volume_tiles(d, cams, w, h, 8, 8, out)
    assert (out == -5.0).all()
    with pytest.raises(L.YvError) as e:
        yoxel_mod.render_volume_tiles(d, cams, w, h, 0, 2 * per_cam + 1, out)
    assert e.value.status == L.YV_ERR_INVALID_ARG
