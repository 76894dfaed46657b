"""The CPU oracle of the dense SVO build, pinned against a numpy restatement
of the same rules: decoding the built tree gives exactly the surface voxels
(solid with a 6-neighbour outside the grid or not solid), each leaf with the
voxel's colour and quantised central-difference normal; regions without
surface voxels are EmptyNode / FullNode; node ids are breadth-first."""
import numpy as np
import pytest

EMPTY, FULL = 0x80000000, 0x80000001


def surface_numpy(d, iso):
    s = d > iso
    pad = np.pad(s, 1, constant_values=False)
    out = np.zeros_like(s)
    for ax in range(3):
        for sh in (1, -1):
            out |= ~np.roll(pad, sh, axis=ax)[1:-1, 1:-1, 1:-1]
    return s & out


def normals_numpy(d):
    """(z, y, x) float32 grid -> int8 normals (z, y, x, 3) of the rule."""
    p = np.pad(d, 1, mode="edge")
    fx = (p[1:-1, 1:-1, :-2] - p[1:-1, 1:-1, 2:]).astype(np.float32)
    fy = (p[1:-1, :-2, 1:-1] - p[1:-1, 2:, 1:-1]).astype(np.float32)
    fz = (p[:-2, 1:-1, 1:-1] - p[2:, 1:-1, 1:-1]).astype(np.float32)
    v = np.stack([fx, fy, fz], -1)
    ln2 = (v[..., 0] * v[..., 0] + v[..., 1] * v[..., 1]) + v[..., 2] * v[..., 2]
    ok = (ln2 > 0) & np.isfinite(ln2)
    ln = np.sqrt(np.where(ok, ln2, np.float32(1)))
    u = np.where(ok[..., None], v / ln[..., None], np.float32(0)).astype(np.float32)
    q = np.clip(np.floor(np.float32(127) * u + np.float32(0.5)), -127, 127)
    return q.astype(np.int8)


def decode(nodes, attrs, root, depth):
    """Walk the pool: leaf voxel -> attr row, plus the null regions."""
    G = 1 << depth
    leaves, nulls = {}, []
    order = []

    def rec(nid, x0, y0, z0, s):
        order.append((s, nid))
        n = nodes[nid]
        h = s // 2
        for ch in range(8):
            x, y, z = x0 + (ch & 1) * h, y0 + ((ch >> 1) & 1) * h, z0 + ((ch >> 2) & 1) * h
            w = int(n[2 + ch])
            if (n[0] >> ch) & 1:
                assert h == 1
                leaves[(x, y, z)] = attrs[w]
            elif w & 0x80000000:
                assert (n[0] >> (8 + ch)) & 1
                nulls.append((w, x, y, z, h))
            else:
                rec(w, x, y, z, h)

    if not root & 0x80000000:
        rec(root, 0, 0, 0, G)
    return leaves, nulls, order


@pytest.mark.parametrize("depth,seed,kind", [(3, 1, "blob"), (4, 2, "blob"), (5, 3, "noise"),
                                             (5, 4, "spheres"), (6, 5, "spheres")])
def test_oracle_dense_build_matches_rules(oracle, depth, seed, kind):
    G = 1 << depth
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(G), np.arange(G), np.arange(G), indexing="ij")
    if kind == "noise":
        d = rng.standard_normal((G, G, G)).astype(np.float32)
    elif kind == "blob":
        d = (G * 0.3 - np.sqrt((x - G / 2) ** 2 + (y - G / 2 + 0.5) ** 2 +
                               (z - G / 2) ** 2)).astype(np.float32)
    else:
        d = np.full((G, G, G), -1e9, np.float32)
        for _ in range(6):
            c = rng.uniform(0, G, 3)
            r = rng.uniform(1, G / 4)
            d = np.maximum(d, (r - np.sqrt((x - c[0]) ** 2 + (y - c[1]) ** 2 +
                                           (z - c[2]) ** 2)).astype(np.float32))
    rgb = rng.integers(0, 256, (G, G, G, 3), dtype=np.uint8)
    nodes, attrs, root = oracle.svo_build_dense(d, depth, 0.0, rgb)
    surf = surface_numpy(d, 0.0)
    nrm = normals_numpy(d)
    leaves, nulls, order = decode(nodes, attrs, root, depth)
    want = {(int(a), int(b), int(c)) for c, b, a in zip(*np.nonzero(surf))}
    assert set(leaves) == want
    for (vx, vy, vz), a in leaves.items():
        assert tuple(a[:3]) == tuple(rgb[vz, vy, vx]) and a[3] == 255
        assert tuple(a[4:7].view(np.int8)) == tuple(nrm[vz, vy, vx]) and a[7] == 0
    solid = d > 0.0
    for w, x0, y0, z0, h in nulls:
        blk_s = surf[z0:z0 + h, y0:y0 + h, x0:x0 + h]
        blk = solid[z0:z0 + h, y0:y0 + h, x0:x0 + h]
        assert not blk_s.any()
        assert (w == FULL and blk.all()) or (w == EMPTY and not blk.any())
    # breadth-first ids: region sizes never grow along the id order
    ids = [nid for _, nid in sorted(order, key=lambda t: t[1])]
    assert ids == list(range(len(nodes)))
    sizes = [s for s, nid in sorted(order, key=lambda t: t[1])]
    assert sizes == sorted(sizes, reverse=True)


def test_oracle_dense_build_edge_cases(oracle):
    G = 8
    n, a, r = oracle.svo_build_dense(np.zeros((G, G, G), np.float32), 3)
    assert r == EMPTY and len(n) == 0
    n, a, r = oracle.svo_build_dense(np.ones((2, 2, 2), np.float32), 1)
    # a full 2^3 grid: every voxel touches the grid border, so all are leaves
    assert r == 0 and len(n) == 1 and n[0][0] == 0xFF and len(a) == 8
    d = np.zeros((G, G, G), np.float32)
    d[5, 2, 6] = 1.0  # one voxel (z, y, x)
    n, a, r = oracle.svo_build_dense(d, 3)
    assert len(n) == 3 and len(a) == 1
    assert tuple(a[0][:4]) == (255, 255, 255, 255) and tuple(a[0][4:7]) == (0, 0, 0)
