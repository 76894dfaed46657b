"""The SSNA oracle on analytic depth maps (no GPU): the blur kernel of
SVORenderer::InitBlur, depth-limited blurring, edge preservation and the
depth-reconstructed normals of a plane."""
import math

import numpy as np

from oracle import ssna as O


def basis(w, h, fov=60.0, fwd=(1.0, 0.0, 0.0), up=(0.0, 0.0, 1.0)):
    """RendererBase::InitRayDir in float64 then float32 (enough for these
    analytic checks)."""
    f = np.asarray(fwd, np.float64)
    f /= np.linalg.norm(f)
    right = np.cross(f, up)
    right /= np.linalg.norm(right)
    vup = np.cross(right, f)
    da = math.tan(math.radians(fov / 2)) / w
    du, dv = 2 * right * da, -2 * vup * da
    d0 = f - du * w / 2 - dv * h / 2
    return d0.astype(np.float32), du.astype(np.float32), dv.astype(np.float32), f


def test_blur_weights_are_init_blur():
    k = O.blur_weights()
    assert k.shape == (5, 5)
    assert abs(float(k.sum(dtype=np.float64)) - 1.0) < 1e-6
    assert np.array_equal(k, k.T) and np.array_equal(k, k[::-1, ::-1])
    t = np.arange(5) - 2.0
    ref = np.exp(-(t[None] ** 2 + t[:, None] ** 2))
    assert np.allclose(k, ref / ref.sum(), rtol=1e-6)


def test_zlimits_follow_the_pass_schedule():
    zl = O.zlimits(5, 1.0 / 2048, 70.0, 640)
    pix = math.radians(70.0) / 640
    for i, z in enumerate(zl):
        assert abs(z - 5.0 / 2048 / (pix * 3 * (i + 1))) <= 1e-6 * z
    assert all(a > b for a, b in zip(zl, zl[1:]))


def test_constant_depth_is_a_fixed_point():
    z = np.full((20, 30), 0.5, np.float32)
    out = O.blur_pass(z, 1.0, 4.0 / 2048, 0.3 * 4.0 / 2048, O.blur_weights())
    assert np.allclose(out, z, rtol=1e-6, atol=0)


def test_only_pixels_under_the_limit_blur():
    rng = np.random.default_rng(5)
    z = (0.5 + 0.001 * rng.standard_normal((24, 24))).astype(np.float32)
    z[:, 12:] += 1.0  # far half
    out = O.blur_pass(z, 1.0, 0.01, 0.003, O.blur_weights())
    assert np.array_equal(out[:, 12:], z[:, 12:])
    assert not np.array_equal(out[:, :12], z[:, :12])
    assert np.abs(out[:, :12] - 0.5).std() < np.abs(z[:, :12] - 0.5).std()


def test_depth_edges_are_kept():
    z = np.full((16, 16), 0.4, np.float32)
    z[:, 8:] = 0.6  # a step far above the threshold
    thr, pad = np.float32(0.01), np.float32(0.3)
    out = O.blur_pass(z, 1.0, thr, pad * thr, O.blur_weights())
    # near side: far taps clamp to d + pad*thr, so at most that much pull
    eps = 1e-6
    assert np.all(out[:, :8] >= 0.4 - eps)
    assert np.all(out[:, :8] <= np.float32(0.4) + pad * thr + eps)
    # far side: near taps are replaced by their (far) mirror
    assert np.allclose(out[:, 8:], 0.6, rtol=1e-6)


def test_misses_are_never_blurred_or_mixed_in():
    z = np.full((10, 10), O.K_FAR, np.float32)
    z[3:7, 3:7] = 0.5
    out = O.blur_pass(z, 1.0, 0.01, 0.003, O.blur_weights())
    assert np.all(out[z == O.K_FAR] == O.K_FAR)
    assert np.all(out[3:7, 3:7] <= np.float32(0.5) + np.float32(0.003) + 1e-6)


def test_plane_normal_faces_the_eye():
    w, h = 40, 30
    d0, du, dv, fwd = basis(w, h, fwd=(1.0, 0.4, -0.2))
    # a plane perpendicular to the view axis: constant view depth
    z = np.full((h, w), 2.0, np.float32)
    alb = np.full((h, w), 0xFF808080, np.uint32)
    stored = np.zeros((h, w, 3), np.float32)
    rgba, dep, n = O.shade(alb, z, stored, (0, 0, 0), d0, du, dv, ssna=True)
    assert np.allclose(n, -fwd[None, None, :], atol=1e-5)
    assert np.array_equal(dep, z)
    # a lit plane head-on with a light at the eye: diffuse 0.7 + specular 0.3
    light = dict(pos=(0, 0, 0), diffuse=(0.7,) * 3, specular=(0.3,) * 3,
                 attenuation=(1.0, 0.0, 0.0))
    rgba, _, _ = O.shade(alb, z, stored, (0, 0, 0), d0, du, dv, lights=[light],
                         ambient=(0.0,) * 3)
    c = rgba.view(np.uint8).reshape(h, w, 4)
    centre = c[h // 2, w // 2]
    assert centre[3] == 255
    assert abs(int(centre[0]) - round(255 * (128 / 255 * 0.7 + 0.3))) <= 2


def test_tilted_plane_normal():
    w, h = 64, 48
    d0, du, dv, fwd = basis(w, h)
    # world plane x + 0.5 z = 2 seen from the origin along +x
    nrm = np.array([1.0, 0.0, 0.5]) / math.sqrt(1.25)
    ys, xs = np.mgrid[:h, :w]
    u = O.ray_u(d0, du, dv, xs, ys).astype(np.float64)
    t = 2.0 / (u[..., 0] + 0.5 * u[..., 2])  # z along u (forward component 1)
    z = t.astype(np.float32)
    alb = np.full((h, w), 0xFFFFFFFF, np.uint32)
    _, _, n = O.shade(alb, z, np.zeros((h, w, 3), np.float32), (0, 0, 0), d0, du, dv)
    assert np.allclose(n[2:-2, 2:-2], -nrm[None, None, :], atol=1e-3)


def test_stored_normals_without_ssna():
    w, h = 8, 6
    d0, du, dv, _ = basis(w, h)
    z = np.full((h, w), 1.0, np.float32)
    alb = np.full((h, w), 0xFF102030, np.uint32)
    alb[0, 0] = 0  # a miss
    stored = np.zeros((h, w, 3), np.float32)
    stored[..., 2] = 1.0
    rgba, dep, n = O.shade(alb, z, stored, (0, 0, 0), d0, du, dv, ssna=False)
    assert np.array_equal(n[1:, 1:], stored[1:, 1:])
    assert rgba[0, 0] == 0 and dep[0, 0] == 0 and not n[0, 0].any()
