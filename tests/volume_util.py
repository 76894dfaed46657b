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
