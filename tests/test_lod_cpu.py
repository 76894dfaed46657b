"""Level-of-detail data and the level-of-detail cut-off (no GPU).

yv_svo_build_lod against a Python restatement of the node-data rule of
reaction/report/main.tex:61 (mean colour and normal of all leaves of the
subtree); .vox round trips; the reference's packed-VoxData file form; and
the cut-off in the FP32 oracle (SVORenderer::SetDetailCoef,
demo/SVORenderer.cpp:104)."""
import struct

import numpy as np
import pytest

from conftest import LIGHT, camera_for


def mean_round(s, n):
    return (2 * s + n) // (2 * n) if s >= 0 else -((-2 * s + n) // (2 * n))


def lod_restated(nodes_u32, attrs_u8):
    """Per node: the attribute the rule gives (8 bytes)."""
    nodes = nodes_u32.reshape(-1, 10).astype(np.int64)
    attrs = attrs_u8.reshape(-1, 8)
    memo = {}

    def sums(i):
        if i in memo:
            return memo[i]
        flags = int(nodes[i, 0])
        acc = np.zeros(7, np.int64)
        for ch in range(8):
            c = int(nodes[i, 2 + ch])
            if (flags >> ch) & 1:
                a = attrs[c]
                acc[:3] += a[:3].astype(np.int64)
                acc[3:6] += a[4:7].view(np.int8).astype(np.int64)
                acc[6] += 1
            elif not (c & 0x80000000):
                acc += sums(c)
        memo[i] = acc
        return acc

    out = []
    for i in range(len(nodes)):
        a = sums(i)
        n = int(a[6])
        if n == 0:
            out.append(bytes(8))
            continue
        rgb = [mean_round(int(v), n) for v in a[:3]]
        nrm = [mean_round(int(v), n) for v in a[3:6]]
        out.append(struct.pack("BBBBbbbb", *rgb, 255, *nrm, 0))
    return out


@pytest.mark.parametrize("kind", ["spheres", "terrain"])
def test_build_lod_matches_rule(yoxel_mod, kind):
    s = (yoxel_mod.SVOScene.spheres(5, 12, 1.0, 6.0, 3) if kind == "spheres"
         else yoxel_mod.SVOScene.terrain(6, 20, 1, 4, 5))
    na0, nn = s.attr_count, s.node_count
    nodes0 = s.nodes_u32.reshape(-1, 10).copy()
    attrs0 = s.attrs_u8.copy()
    assert not s.has_lod
    s.build_lod()
    assert s.has_lod
    assert s.attr_count == na0 + nn
    nodes = s.nodes_u32.reshape(-1, 10)
    # only the data words change; attributes are appended in node order
    assert np.array_equal(np.delete(nodes, 1, axis=1), np.delete(nodes0, 1, axis=1))
    assert np.array_equal(nodes[:, 1], np.arange(na0, na0 + nn, dtype=np.uint32))
    assert np.array_equal(s.attrs_u8[:na0 * 8], attrs0)
    want = lod_restated(nodes0.reshape(-1), attrs0)
    got = s.attrs_u8.reshape(-1, 8)[na0:]
    for i in range(nn):
        assert bytes(got[i]) == want[i], f"node {i}"


def test_lod_survives_save_and_load(yoxel_mod, tmp_path):
    s = yoxel_mod.SVOScene.spheres(5, 12, 1.0, 6.0, 3).build_lod()
    p = tmp_path / "lod.vox"
    s.save(p)
    t = yoxel_mod.SVOScene.load(p)
    assert t.has_lod
    assert np.array_equal(t.nodes_u32, s.nodes_u32)
    assert np.array_equal(t.attrs_u8, s.attrs_u8)
    u = yoxel_mod.SVOScene.spheres(5, 12, 1.0, 6.0, 3)
    u.save(tmp_path / "plain.vox")
    assert not yoxel_mod.SVOScene.load(tmp_path / "plain.vox").has_lod


def test_reference_packed_file_decodes_node_data(yoxel_mod, tmp_path):
    """A file in the reference's own form (no attribute section): leaves and
    node data hold packed VoxData; both become attributes and the scene has
    level-of-detail data."""
    def packed(r5, g6, b5, ox, oy):
        return (r5 << 11 | g6 << 5 | b5) | ((ox & 0xFF) << 16) | ((oy & 0xFF) << 24)
    # root with one child node (slot 0) and one leaf (slot 7); child node
    # with two leaves
    root = [0x80, packed(31, 0, 0, 0, 0)] + [1] + [0x80000000] * 6 + [packed(0, 63, 0, 127, 0)]
    root[0] = (1 << 7) | (0x7E << 8)
    child = [(1 << 0) | (1 << 3) | (0xF6 << 8), packed(0, 0, 31, 0, 127),
             packed(31, 63, 31, 0, 0)] + [0x80000000] * 2 + [packed(31, 0, 0, 0, -127)] + \
        [0x80000000] * 4
    hdr = struct.pack("<4I", 0, 0, 0, 2)
    body = struct.pack("<10I", *root) + struct.pack("<10I", *child)
    p = tmp_path / "ref.vox"
    p.write_bytes(hdr + body)
    s = yoxel_mod.SVOScene.load(p)
    assert s.has_lod
    nodes = s.nodes_u32.reshape(-1, 10)
    attrs = s.attrs_u8.reshape(-1, 8)
    # node 0's data decodes to pure red, node 1's to pure blue
    assert tuple(attrs[nodes[0, 1]][:4]) == (255, 0, 0, 255)
    assert tuple(attrs[nodes[1, 1]][:4]) == (0, 0, 255, 255)
    # leaves still decode as before
    assert tuple(attrs[nodes[0, 2 + 7]][:3]) == (0, 255, 0)


def test_oracle_cut_off(oracle, yoxel_mod):
    s = yoxel_mod.SVOScene.spheres(7, 60, 2.0, 12.0, 11).build_lod()
    pos, view = camera_for()
    nodes, attrs = s.nodes_u32, s.attrs_u8
    args = (nodes, s.root, attrs, pos, view, np.float32([0, 0, 1]), 60.0, 96, 64, LIGHT)
    exact = oracle.svo_render(*args)
    zero = oracle.svo_render(*args, lod_coef=0.0)
    for k in exact:
        assert np.array_equal(exact[k], zero[k])
    prev = exact
    nn = nodes.reshape(-1, 10)
    for coef in (0.002, 0.01, 0.05):
        lod = oracle.svo_render(*args, lod_coef=coef)
        # a cut only shortens a ray's descent
        assert np.all(lod["fetches"] <= prev["fetches"])
        hit = lod["hit"] != 0xFFFFFFFF
        assert np.all(hit >= (prev["hit"] != 0xFFFFFFFF))
        ids, ch = lod["hit"][hit] >> 3, lod["hit"][hit] & 7
        is_leaf = (nn[ids, 0] >> ch) & 1
        if coef >= 0.01:
            assert (is_leaf == 0).any()  # some rays stopped at a subtree
        prev = lod
    assert prev["fetches"].mean() < exact["fetches"].mean()
