"""CPU oracle of the screen-space normal approximation (SSNA) post passes.

TEST INFRASTRUCTURE ONLY: the checker of the CUDA passes behind
yv_render_ssna; the product library never imports or calls it.

Restates, in numpy FP32 with every operation rounded to nearest in the order
the device passes use:
  - the blur kernel of SVORenderer::InitBlur (demo/SVORenderer.cpp:55-78)
    with BlurZKernSize 5 (the kernel size of ztools.multipassGaussBlur,
    demo/dumps/ztools.py:257): weights exp(-(dx^2 + dy^2)) / sum;
  - the pass schedule of SVORenderer::Render (demo/SVORenderer.cpp:124-140):
    pass i (blurSize = 3 (i + 1)) blurs the pixels with
    0 < z <= 5 voxSize / (pixelAng * blurSize);
  - limitedGaussBlur mode 2 (ztools.py:154-233): a far tap (s > d + thr)
    is replaced by d + edgePad * thr, a near tap (d > s + thr) by its mirror
    across the pixel unless the mirror is near too (then its weight is 0);
    here the mirror is clamped like a far tap and taps outside the frame are
    left out;
  - calcNormals (ztools.py:23-43): per axis the neighbour difference with the
    smaller |dz| (absMin); here the exact cross product of the reconstructed
    positions z * u instead of its small-angle form, turned toward the eye;
  - Phong point lights with LightParams (Demo.cpp:141-147):
    albedo * (ambient + diffuse * max(n.L, 0) * att)
    + specular * max(R.V, 0)^e * att, att = 1 / (a0 + a1 d + a2 d^2),
    evaluated as n.L = (n.lv) / d and R.V = (lv.u - 2 (n.L) (n.u) d) / (d |u|)
    (lv = light - P, u the pixel's ray, R = 2 (n.L) n - L, V = -u / |u|).
Parity status: the reference's BlurZ / ShadeSimple CUDA kernels are absent
from its snapshot, so this restatement is unpinned against reference outputs;
it pins the device passes to this specification.
"""
import math

import numpy as np

F = np.float32
K_FAR = F(1e30)
FLT_MAX = F(3.402823466e38)


def blur_weights():
    """(5, 5) float32 weights indexed [oy + 2, ox + 2]."""
    t = np.arange(5, dtype=np.float64) - 2.0
    w = np.exp(-(t[None, :] ** 2 + t[:, None] ** 2))
    return (w / w.sum()).astype(F)


def ray_u(dir0, du, dv, xs, ys):
    """Unnormalised pixel rays (..., 3): (dir0 + du x) + dv y."""
    fx, fy = xs.astype(F), ys.astype(F)
    return np.stack([(F(dir0[i]) + F(du[i]) * fx) + F(dv[i]) * fy for i in range(3)], -1)


def _dot(a, b):
    return (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]) + a[..., 2] * b[..., 2]


def depth(albedo, hit_t, dir0, du, dv):
    """View depth z = t / |u| for hits (alpha != 0), K_FAR for misses."""
    h, w = hit_t.shape
    ys, xs = np.mgrid[:h, :w]
    u = ray_u(dir0, du, dv, xs, ys)
    hit = (albedo.astype(np.uint32) >> 24) != 0
    z = hit_t.astype(F) / np.sqrt(_dot(u, u))
    return np.where(hit, z, K_FAR).astype(F)


def _shift(zp, ox, oy, h, w):
    return zp[2 + oy:2 + oy + h, 2 + ox:2 + ox + w]


def blur_pass(z, zlimit, thr, pad_thr, kern):
    z = z.astype(F)
    h, w = z.shape
    zlimit, thr, pad_thr = F(zlimit), F(thr), F(pad_thr)
    zp = np.full((h + 4, w + 4), K_FAR, F)
    zp[2:-2, 2:-2] = z
    ys, xs = np.mgrid[:h, :w]
    d = z
    d_far = d + thr
    d_pad = d + pad_thr
    acc = np.zeros_like(d)
    c = np.zeros_like(d)
    with np.errstate(over="ignore", invalid="ignore"):
        for oy in range(-2, 3):
            for ox in range(-2, 3):
                tap_ok = (xs + ox >= 0) & (xs + ox < w) & (ys + oy >= 0) & (ys + oy < h)
                m_ok = (xs - ox >= 0) & (xs - ox < w) & (ys - oy >= 0) & (ys - oy < h)
                s = _shift(zp, ox, oy, h, w)
                m = _shift(zp, -ox, -oy, h, w)
                k = np.full_like(d, kern[oy + 2, ox + 2])
                far = s > d_far
                near = ~far & (d > s + thr)
                k_zero = near & (~m_ok | (d > m + thr))
                take_m = near & ~k_zero
                s2 = np.where(far, d_pad, np.where(take_m, np.where(m > d_far, d_pad, m), s))
                k2 = np.where(k_zero, F(0), k)
                acc = np.where(tap_ok, acc + s2 * k2, acc)
                c = np.where(tap_ok, c + k2, c)
        blurred = acc / c
    return np.where((d > 0) & (d <= zlimit), blurred, d).astype(F)


def zlimits(passes, voxel_size, fov_deg, width):
    pix = fov_deg * (math.pi / 180.0) / width
    return [F(5.0 * float(F(voxel_size)) / (pix * 3.0 * (i + 1))) for i in range(passes)]


def _tangent(z, u, p, axis):
    """Tangent along x (axis 1) or y (axis 0) and whether a hit neighbour
    exists."""
    h, w = z.shape
    zp = np.full((h + 2, w + 2), K_FAR, F)
    zp[1:-1, 1:-1] = z
    up = np.zeros((h + 2, w + 2, 3), F)
    up[1:-1, 1:-1] = u
    if axis == 1:
        zl, zh = zp[1:-1, :-2], zp[1:-1, 2:]
        ul, uh = up[1:-1, :-2], up[1:-1, 2:]
    else:
        zl, zh = zp[:-2, 1:-1], zp[2:, 1:-1]
        ul, uh = up[:-2, 1:-1], up[2:, 1:-1]
    has_lo = zl < K_FAR
    has_hi = zh < K_FAR
    with np.errstate(over="ignore", invalid="ignore"):
        use_hi = has_hi & (~has_lo | (np.abs(zh - z) < np.abs(z - zl)))
        t_hi = zh[..., None] * uh - p
        t_lo = p - zl[..., None] * ul
    return np.where(use_hi[..., None], t_hi, t_lo), has_lo | has_hi


def _to_u8(c):
    c = np.fmin(np.fmax(c, F(0)), F(1))
    return np.trunc(c * F(255) + F(0.5)).astype(np.uint32)


def shade(albedo, z, stored_n, pos, dir0, du, dv, ssna=True, show_normals=False,
          ambient=(0.1, 0.1, 0.1), specular_exp=10.0, lights=()):
    """rgba (h, w) uint32, depth (h, w) f32 and normals (h, w, 3) f32.
    lights: dicts with pos, diffuse, specular, attenuation (enabled only)."""
    albedo = albedo.astype(np.uint32)
    h, w = z.shape
    ys, xs = np.mgrid[:h, :w]
    u = ray_u(dir0, du, dv, xs, ys)
    p = z[..., None] * u
    n = stored_n.astype(F).copy()
    hit = (albedo >> 24) != 0
    with np.errstate(over="ignore", invalid="ignore", divide="ignore"):
        if ssna:
            tx, okx = _tangent(z, u, p, 1)
            ty, oky = _tangent(z, u, p, 0)
            cr = np.stack([tx[..., 1] * ty[..., 2] - tx[..., 2] * ty[..., 1],
                           tx[..., 2] * ty[..., 0] - tx[..., 0] * ty[..., 2],
                           tx[..., 0] * ty[..., 1] - tx[..., 1] * ty[..., 0]], -1)
            flip = _dot(cr, u) > 0
            cr = np.where(flip[..., None], -cr, cr)
            len2 = _dot(cr, cr)
            ok = okx & oky & (len2 > 0) & (len2 <= FLT_MAX)
            inv = F(1) / np.sqrt(len2)
            nn = cr * inv[..., None]
            n = np.where(ok[..., None], nn, n)
        if show_normals:
            rgb = [_to_u8(n[..., i] * F(0.5) + F(0.5)) for i in range(3)]
        else:
            a = [((albedo >> (8 * i)) & 0xFF).astype(F) * (F(1) / F(255)) for i in range(3)]
            col = [a[i] * F(ambient[i]) for i in range(3)]
            ulen = np.sqrt(_dot(u, u))
            nu = _dot(n, u)
            for lt in lights:
                lpos = np.asarray(lt["pos"], F)
                lv = np.stack([F(lpos[i]) - (F(pos[i]) + p[..., i]) for i in range(3)], -1)
                d2 = _dot(lv, lv)
                d = np.sqrt(d2)
                ndl = _dot(n, lv) / d
                dok = (d > 0) & (ndl > 0)
                at = np.asarray(lt["attenuation"], F)
                den = (at[0] + at[1] * d) + at[2] * d2
                att = np.where(den > 0, F(1) / den, F(0))
                na = ndl * att
                dif = np.asarray(lt["diffuse"], F)
                for i in range(3):
                    col[i] = np.where(dok, col[i] + a[i] * (na * dif[i]), col[i])
                num = _dot(lv, u) - ((F(2) * ndl) * nu) * d
                rv = num / (d * ulen)
                sok = dok & (rv > 0)
                sp = np.power(np.where(sok, rv, F(1)), F(specular_exp)).astype(F) * att
                spec = np.asarray(lt["specular"], F)
                for i in range(3):
                    col[i] = np.where(sok, col[i] + spec[i] * sp, col[i])
            rgb = [_to_u8(col[i]) for i in range(3)]
    rgba = np.uint32(0xFF000000) | rgb[0] | (rgb[1] << 8) | (rgb[2] << 16)
    rgba = np.where(hit, rgba, np.uint32(0)).astype(np.uint32)
    dep = np.where(hit, z, F(0)).astype(F)
    nout = np.where(hit[..., None], n, F(0)).astype(F)
    return rgba, dep, nout


def ssna_frame(albedo, hit_t, stored_n, pos, dir0, du, dv, fov_deg, passes=5,
               voxel_size=1.0 / 2048, edge_threshold=4.0 / 2048, edge_pad=0.3, ssna=True,
               **shade_kw):
    """The whole post chain from an unlit trace (albedo, hit_t, stored normals)."""
    h, w = hit_t.shape
    z = depth(albedo, hit_t, dir0, du, dv)
    if ssna:
        kern = blur_weights()
        thr = F(edge_threshold)
        pad_thr = F(edge_pad) * thr
        for zl in zlimits(passes, voxel_size, fov_deg, w):
            z = blur_pass(z, zl, thr, pad_thr, kern)
    return shade(albedo, z, stored_n, pos, dir0, du, dv, ssna=ssna, **shade_kw)
