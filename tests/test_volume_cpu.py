"""Brick volumes on the CPU: ntree layout invariants, analytic march known
answers for the FP64 oracle, and the oracle adjoint pinned to FP64 central
finite differences."""
import numpy as np
import pytest

from volume_util import copies_of, fold_numpy, owned_points


def cam(pos, d, fov=60.0):
    return np.asarray(pos, np.float64), np.asarray(d, np.float64), fov


@pytest.fixture(scope="module")
def small(yoxel_mod):
    return yoxel_mod.BrickVolume.noise(levels=1, offset=0.4, amplitude=1.4, seed=3)


def test_noise_volume_is_deterministic_and_culled(yoxel_mod):
    a = yoxel_mod.BrickVolume.noise(2, 0.4, 1.4, 11)
    b = yoxel_mod.BrickVolume.noise(2, 0.4, 1.4, 11)
    assert a.nbricks == b.nbricks > 0
    assert np.array_equal(a.grids, b.grids) and np.array_equal(a.density, b.density)
    assert np.array_equal(a.albedo_u8, b.albedo_u8)
    # every stored brick has a non-zero lattice value, densities in [0, 1]
    assert (a.density.max(axis=1) > 0).all()
    assert a.density.min() >= 0 and a.density.max() <= 1
    assert 0 < a.occupancy < 1


def test_tree_refs_and_brick_cells_agree(yoxel_mod):
    v = yoxel_mod.BrickVolume.noise(2, 0.4, 1.4, 5)
    g = v.grids
    seen = set()
    # walk the tree, recompute each brick's cell, compare with the table
    stack = [(0, 0, 0, 0, 0)]
    while stack:
        node, lvl, x, y, z = stack.pop()
        for c in range(64):
            r = int(g[node, c])
            cx, cy, cz = x * 4 + (c & 3), y * 4 + ((c >> 2) & 3), z * 4 + (c >> 4)
            if r & 0x80000000:
                continue
            if r & 0x40000000:
                assert lvl == v.levels - 1
                b = r & 0x3FFFFFFF
                assert tuple(v.cells[b]) == (cx, cy, cz)
                seen.add(b)
            else:
                stack.append((r, lvl + 1, cx, cy, cz))
    assert seen == set(range(v.nbricks))


def test_aprons_repeat_neighbour_lattice(yoxel_mod):
    v = yoxel_mod.BrickVolume.noise(2, 0.4, 1.4, 5)
    d = v.density.reshape(-1, 9, 9, 9)
    up = v.neighbors(True)
    for b in range(0, v.nbricks, 7):
        nx = up[b, 0]  # +x neighbour
        if nx >= 0:
            assert np.array_equal(d[b, :, :, 8], d[nx, :, :, 0])
        elif v.cells[b][0] + 1 < 4 ** v.levels:
            # culled interior neighbour: its (shared) low face is all zero
            assert (d[b, :, :, 8] == 0).all()


def test_from_dense_matches_lattice(yoxel_mod):
    rng = np.random.default_rng(0)
    s = 33
    dense = np.zeros((s, s, s), np.float32)
    dense[4:20, 6:30, 2:11] = rng.random((16, 24, 9), dtype=np.float32)
    v = yoxel_mod.BrickVolume.from_dense(1, dense)
    assert v.nbricks > 0
    for b in range(v.nbricks):
        cx, cy, cz = v.cells[b]
        blk = dense[cz * 8:cz * 8 + 9, cy * 8:cy * 8 + 9, cx * 8:cx * 8 + 9]
        assert np.array_equal(v.density[b].reshape(9, 9, 9), blk)


def const_volume(yoxel_mod, value, albedo=128):
    s = 33
    dense = np.full((s, s, s), value, np.float32)
    alb = np.full((s, s, s, 3), albedo, np.uint8)
    return yoxel_mod.BrickVolume.from_dense(1, dense, alb)


def test_march_known_answers(oracle, yoxel_mod):
    """alpha = 0.5 per sample: A = 1 - 0.5^n stops at n = 7 (A > 0.99);
    constant albedo a gives C = a*A.  alpha = 1: one sample, A = 1."""
    v = const_volume(yoxel_mod, 0.5, 128)
    alb = v.albedo_u8.astype(np.float64) / 255.0
    pos, d, fov = cam([-1.0, 0.5, 0.5], [1, 0, 0], 10.0)
    rgba, ns, nb = oracle.brick_render_f64(v.grids, v.density, alb, v.levels, pos, d,
                                           [0, 0, 1], fov, 4, 4, alpha_scale=1.0)
    assert (ns == 7).all()
    assert np.allclose(rgba[..., 3], 1 - 0.5 ** 7, rtol=0, atol=1e-15)
    assert np.allclose(rgba[..., 0], 128 / 255 * (1 - 0.5 ** 7), atol=1e-15)
    rgba, ns, _ = oracle.brick_render_f64(v.grids, v.density, alb, v.levels, pos, d,
                                          [0, 0, 1], fov, 4, 4, alpha_scale=4.0)
    assert (ns == 1).all() and np.allclose(rgba[..., 3], 1.0)
    # a ray that misses the cube composites nothing
    rgba, ns, _ = oracle.brick_render_f64(v.grids, v.density, alb, v.levels,
                                          np.array([-1.0, 3.0, 0.5]), d, [0, 0, 1], fov, 4, 4)
    assert (ns == 0).all() and (rgba == 0).all()


def test_march_sample_count_matches_path_length(oracle, yoxel_mod):
    """Thin density: no early exit; samples = lattice path length / step."""
    v = const_volume(yoxel_mod, 0.001, 255)
    alb = v.albedo_u8.astype(np.float64) / 255.0
    pos, d, fov = cam([-1.0, 0.55, 0.45], [1, 0, 0], 1.0)
    _, ns, nb = oracle.brick_render_f64(v.grids, v.density, alb, v.levels, pos, d, [0, 0, 1],
                                        fov, 1, 1, step_vox=0.5)
    # 32 lattice cells crossed along x at 0.5-cell steps
    assert abs(int(ns[0, 0]) - 64) <= 1
    assert nb[0, 0] == 4


def test_f32_oracle_close_to_f64(oracle, small):
    alb = small.albedo_u8.astype(np.float64) / 255.0
    pos = np.array([1.6, 1.3, 1.1])
    d = 0.5 - pos
    r64, _, _ = oracle.brick_render_f64(small.grids, small.density, alb, 1, pos, d, [0, 0, 1],
                                        60.0, 32, 32)
    r32, _, _ = oracle.brick_render_f32_mt(small.grids, small.density, alb, 1, pos, d,
                                           [0, 0, 1], 60.0, 32, 32, threads=2)
    assert r64[..., 3].max() > 0.05
    assert np.abs(r64 - r32).max() < 1e-4


def test_oracle_adjoint_matches_central_differences(oracle, small):
    """FP64 adjoint vs FP64 central differences (h = 1e-3) of
    L = sum(w * rgba) on random lattice points (all copies perturbed)."""
    rng = np.random.default_rng(1)
    alb = small.albedo_u8.astype(np.float64) / 255.0
    den = small.density.astype(np.float64)
    pos = np.array([1.6, 1.3, 1.1])
    d = 0.5 - pos
    w, h = 24, 24
    wts = rng.standard_normal((h, w, 4))
    gd, ga = oracle.brick_backward_f64(small.grids, den, alb, 1, pos, d, [0, 0, 1], 60.0, w, h,
                                       wts, alpha_scale=2.0)
    gd = fold_numpy(small, gd, 1)
    ga = fold_numpy(small, ga, 3)

    def loss(dd, aa):
        r, _, _ = oracle.brick_render_f64(small.grids, dd, aa, 1, pos, d, [0, 0, 1], 60.0, w, h,
                                          alpha_scale=2.0)
        return float((r * wts).sum())

    eps = 1e-3
    l0 = loss(den, alb)
    errs, refs, kinks = [], [], 0

    def perturbed(slots, kind, delta):
        dd, aa = den.copy(), alb.copy()
        for (bb, s) in slots:
            if kind == "d":
                dd[bb, s] += delta
            else:
                aa[bb, s, 1] += delta
        return loss(dd, aa)

    for (b, z, y, x) in owned_points(small, rng, 60):
        slots = copies_of(small, b, z, y, x)
        i = b * 729 + (z * 9 + y) * 9 + x
        for kind in ("d", "a"):
            an = gd[i] if kind == "d" else ga[i * 3 + 1]
            if kind == "d" and den[b, (z * 9 + y) * 9 + x] == 0.0:
                # density 0 sits on the saturate kink: the adjoint returns
                # the right derivative; check it with a Richardson-extrapolated
                # forward difference
                r1 = (perturbed(slots, kind, eps) - l0) / eps
                r2 = (perturbed(slots, kind, eps / 2) - l0) / (eps / 2)
                fd = 2 * r2 - r1
            else:
                lp, lm = perturbed(slots, kind, eps), perturbed(slots, kind, -eps)
                fd = (lp - lm) / (2 * eps)
                right, left = (lp - l0) / eps, (l0 - lm) / eps
                # saturation at 1 or an early-exit jump: one-sided slopes differ
                if abs(right - left) > 1e-2 * (abs(right) + abs(left)) + 1e-6:
                    kinks += 1
                    continue
            errs.append(an - fd)
            refs.append(fd)
    errs, refs = np.array(errs), np.array(refs)
    assert len(refs) > 60 and np.abs(refs).max() > 0 and kinks < len(refs)
    rel = np.linalg.norm(errs) / np.linalg.norm(refs)
    assert rel < 1e-4, rel


def test_oracle_adjoint_matches_central_differences_cfg4_volume(oracle, yoxel_mod):
    """The FP64 adjoint on the full 128^3 differentiable volume (seed 1234)
    with 4 of its 64 cameras at 256^2 and a seeded dL/drgba, against FP64
    central differences on 150 seeded lattice points (density and albedo),
    kinks left out (volume_util.central_differences)."""
    import os
    from volume_util import central_differences, gradient_at
    vol = yoxel_mod.BrickVolume.noise(2, 0.4, 1.4, 1234)
    cams = [yoxel_mod.sphere_cameras(64)[i] for i in (0, 16, 32, 48)]
    den = vol.density.astype(np.float32)
    alb = vol.albedo_u8.astype(np.float32) * np.float32(1.0 / 255.0)
    w = h = 256
    rng = np.random.default_rng(11)
    grads = [rng.standard_normal((h, w, 4)) for _ in cams]
    threads = max(1, os.cpu_count() or 1)
    rd = np.zeros(vol.nbricks * 729)
    ra = np.zeros(vol.nbricks * 729 * 3)
    for c, g in zip(cams, grads):
        a, b = oracle.brick_backward_f64(vol.grids, den, alb, vol.levels, *c, w, h, g,
                                         threads=threads)
        rd += a
        ra += b
    pts = owned_points(vol, np.random.default_rng(1234), 150)
    fds, kinks = central_differences(oracle, vol, den, alb, cams, grads, w, h, pts)
    for kind, ch, rg in (("d", 1, rd), ("a", 3, ra)):
        fd = np.array([f for (_, f, _) in fds[kind]])
        an = np.array([gradient_at(rg, sl, ch, 0 if kind == "d" else 1)
                       for (_, _, sl) in fds[kind]])
        assert len(fd) > 100 and np.abs(fd).max() > 0
        assert np.linalg.norm(an - fd) / np.linalg.norm(fd) < 1e-4, kind
    assert kinks < 40
