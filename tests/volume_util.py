"""Helpers shared by the brick-volume tests."""
import numpy as np


def fold_numpy(vol, g, channels):
    """CPU restatement of the apron fold: totals per lattice point written to
    every copy (zero where the owner brick is absent).  g: (nb*729*channels)."""
    nb = vol.nbricks
    g = np.asarray(g, np.float64).reshape(nb, 9, 9, 9, channels).copy()
    up = vol.neighbors(True)
    dn = vol.neighbors(False)
    out = g.copy()
    # owners gather copies from lower neighbours' aprons
    for b in range(nb):
        for m in range(1, 8):
            dx, dy, dz = m & 1, (m >> 1) & 1, (m >> 2) & 1
            n = dn[b, m - 1]
            if n < 0:
                continue
            xs = slice(0, 1) if dx else slice(0, 8)
            ys = slice(0, 1) if dy else slice(0, 8)
            zs = slice(0, 1) if dz else slice(0, 8)
            xa = slice(8, 9) if dx else slice(0, 8)
            ya = slice(8, 9) if dy else slice(0, 8)
            za = slice(8, 9) if dz else slice(0, 8)
            out[b, zs, ys, xs] += g[n, za, ya, xa]
    # aprons copy owners
    res = out.copy()
    for b in range(nb):
        for m in range(1, 8):
            dx, dy, dz = m & 1, (m >> 1) & 1, (m >> 2) & 1
            # apron slots whose "==8" axes are exactly m
            xs = np.arange(9) if not dx else np.array([8])
            ys = np.arange(9) if not dy else np.array([8])
            zs = np.arange(9) if not dz else np.array([8])
            if not dx:
                xs = xs[xs < 8]
            if not dy:
                ys = ys[ys < 8]
            if not dz:
                zs = zs[zs < 8]
            own = up[b, m - 1]
            for z in zs:
                for y in ys:
                    for x in xs:
                        if own >= 0:
                            res[b, z, y, x] = out[own, z - 8 * dz, y - 8 * dy, x - 8 * dx]
                        else:
                            res[b, z, y, x] = 0.0
    return res.reshape(-1)


def owned_points(vol, rng, n):
    """n random (brick, z, y, x) owned lattice points (x,y,z < 8)."""
    nb = vol.nbricks
    b = rng.integers(0, nb, n)
    z = rng.integers(0, 8, n)
    y = rng.integers(0, 8, n)
    x = rng.integers(0, 8, n)
    return list(zip(b.tolist(), z.tolist(), y.tolist(), x.tolist()))


def copies_of(vol, b, z, y, x):
    """All pool slots (brick, slot) holding lattice point (b; z,y,x)."""
    dn = vol.neighbors(False)
    out = [(b, (z * 9 + y) * 9 + x)]
    for m in range(1, 8):
        dx, dy, dz = m & 1, (m >> 1) & 1, (m >> 2) & 1
        if (dx and x) or (dy and y) or (dz and z):
            continue
        n = dn[b, m - 1]
        if n >= 0:
            out.append((n, ((z + 8 * dz) * 9 + (y + 8 * dy)) * 9 + (x + 8 * dx)))
    return out


def support_window(p_lo, p_hi, cam, w, h, oracle):
    """Pixel window (x0, x1, y0, y1) holding every FP64 primary ray of `cam`
    that can cross the world box [p_lo, p_hi]: the box corners projected
    with the camera basis of InitRayDir (dir = dir0 + du x + dv y), widened by
    2 pixels; the whole frame if a corner is not in front of the camera."""
    pos, d, up, fov = cam
    d0, du, dv = oracle.init_ray_dir_f64(d, up, fov, w, h)
    fwd = d0 + du * (w / 2.0) + dv * (h / 2.0)
    xs, ys = [], []
    for k in range(8):
        c = np.array([p_hi[0] if k & 1 else p_lo[0], p_hi[1] if k & 2 else p_lo[1],
                      p_hi[2] if k & 4 else p_lo[2]]) - np.asarray(pos, np.float64)
        s = c @ fwd / (fwd @ fwd)
        if s <= 0:
            return 0, w, 0, h
        # c = s (dir0 + du x + dv y), dir0 . du = -|du|^2 w / 2 (du, dv and the
        # view direction are orthogonal)
        xs.append((c @ du) / (s * (du @ du)) + w / 2.0)
        ys.append((c @ dv) / (s * (dv @ dv)) + h / 2.0)
    x0 = max(0, int(np.floor(min(xs))) - 2)
    x1 = min(w, int(np.ceil(max(xs))) + 3)
    y0 = max(0, int(np.floor(min(ys))) - 2)
    y1 = min(h, int(np.ceil(max(ys))) + 3)
    return x0, max(x0, x1), y0, max(y0, y1)


def central_differences(oracle, vol, den, alb, cams, grads, w, h, pts, alpha_scale=1.0,
                        step_vox=0.5, eps=1e-3, kink_tol=1e-3, f32ray=False):
    """FP64 central differences of L = sum_c grads[c] . rgba_c (the FP64 march
    of cameras `cams` at w x h; FP32 primary rays promoted with f32ray, as
    the CUDA path casts them) with respect to the density and the green
    albedo of the owned lattice points `pts` ((brick, z, y, x)), every copy of
    a point perturbed.  Only the pixels whose rays can reach the 8 cells
    around a point are re-marched (support_window), so the sum is that of
    the whole frames.  The float32 value actually stored on either side sets
    the step.  A point is a kink and is skipped when an early exit moves
    between the evaluations (a ray's sample count changes) or its one-sided
    slopes differ by more than kink_tol (relative; saturation at 1); a
    density within h of 0 (the saturate kink) gets a Richardson-extrapolated
    forward difference (the right derivative, which the adjoint returns).
    Returns {"d": [(point, fd, slots)], "a": [...]} and the number of
    kinks."""
    wins = [oracle.BrickWindow(vol.grids, den, alb, vol.levels, *c, w, h,
                               alpha_scale=alpha_scale, step_vox=step_vox, f32ray=f32ray)
            for c in cams]
    S = 8 * 4 ** vol.levels
    cells = vol.cells
    den2 = np.asarray(den, np.float32).reshape(vol.nbricks, 729)
    alb2 = np.asarray(alb, np.float32).reshape(vol.nbricks, 729, 3)

    def loss(rects):
        """L over the windows, and the samples every ray of them took (an
        early exit that moves between two evaluations is a jump of L)."""
        tot, ns = 0.0, []
        for k, (x0, x1, y0, y1) in enumerate(rects):
            if x0 < x1 and y0 < y1:
                r = wins[k].render(x0, x1, y0, y1)
                tot += float((r * grads[k][y0:y1, x0:x1]).sum())
                ns.append(wins[k].window_samples(x0, x1, y0, y1))
        return tot, (np.concatenate([n.ravel() for n in ns]) if ns else np.zeros(0))

    def set_value(slots, kind, val):
        for (bb, s) in slots:
            for wn in wins:
                if kind == "d":
                    wn.density[bb * 729 + s] = val
                else:
                    wn.albedo[(bb * 729 + s) * 3 + 1] = val

    out = {"d": [], "a": []}
    kinks = 0
    for (b, z, y, x) in pts:
        slots = copies_of(vol, b, z, y, x)
        lp = (np.asarray(cells[b], np.float64) * 8 + np.array([x, y, z], np.float64))
        rects = [support_window((lp - 1.0001) / S, (lp + 1.0001) / S, c, w, h, oracle)
                 for c in cams]
        i = (z * 9 + y) * 9 + x
        l0, n0 = loss(rects)
        for kind in ("d", "a"):
            x0v = np.float32(den2[b, i] if kind == "d" else alb2[b, i, 1])
            up_v = np.float32(x0v + np.float32(eps))
            dn_v = np.float32(x0v - np.float32(eps))
            hp, hm = float(up_v) - float(x0v), float(x0v) - float(dn_v)
            set_value(slots, kind, up_v)
            lp_, np_ = loss(rects)
            if kind == "d" and dn_v < 0.0:
                # within h of the saturate kink at 0: the adjoint returns the
                # right derivative, checked by forward differences over h and
                # h/2, Richardson-extrapolated
                half = np.float32(x0v + np.float32(eps / 2))
                set_value(slots, kind, half)
                lh, nh = loss(rects)
                set_value(slots, kind, x0v)
                r1, r2 = (lp_ - l0) / hp, (lh - l0) / (float(half) - float(x0v))
                # a kink inside [x, x + h]: an early exit moved, or forward
                # slopes over h and h/2 that disagree
                if (not np.array_equal(n0, np_) or not np.array_equal(n0, nh) or
                        abs(r1 - r2) > kink_tol * (abs(r1) + abs(r2)) + 1e-9):
                    kinks += 1
                    continue
                fd = 2 * r2 - r1
            else:
                set_value(slots, kind, dn_v)
                lm, nm = loss(rects)
                set_value(slots, kind, x0v)
                fd = (lp_ - lm) / (hp + hm)
                right, left = (lp_ - l0) / hp, (l0 - lm) / hm
                if (not np.array_equal(n0, np_) or not np.array_equal(n0, nm) or
                        abs(right - left) > kink_tol * (abs(right) + abs(left)) + 1e-9):
                    kinks += 1
                    continue
            out[kind].append(((b, z, y, x), fd, slots))
    return out, kinks


def gradient_at(g, slots, channels, channel=0):
    """Total gradient of a lattice point: the sum over its pool copies."""
    return float(sum(g[(bb * 729 + s) * channels + channel] for (bb, s) in slots))
