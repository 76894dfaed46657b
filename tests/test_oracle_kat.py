"""Known-answer tests that pin the CPU oracle's restatement of the reference
traversal (FindFirstChild / GoNext of cell/spu/trace_spu.cpp:48-93, SetupTrace
of reaction/report/voxel.tex:312-326, RecTrace of cell/ppu_renderer.cpp:18-41).

The reference's own tests cover no tracing code, so these hand-derived cases
(answers worked out from the algorithm text, not from running the oracle) and
the committed golden fixtures are the pins."""
import os

import numpy as np
import pytest

from conftest import ROOT, camera_for, LIGHT

EMPTY, FULL = 0x80000000, 0x80000001


def make_node(children, leaf_mask=0):
    """VoxNode as 10 uint32: flags, data, child[8]."""
    flags = leaf_mask
    for i, c in enumerate(children):
        if not (leaf_mask >> i) & 1 and (c & 0x80000000):
            flags |= 1 << (8 + i)
    return [flags, 0] + list(children)


def pool(*nodes):
    return np.array(sum(nodes, []), np.uint32)


# ---------------------------------------------------------------- primitives
def test_find_first_child_known_answers(oracle):
    # entry through the low corner: all halves low
    ch, t1, t2 = oracle.find_first_child([0, 0, 0], [2, 4, 8])
    assert ch == 0
    assert list(t1) == [0, 0, 0] and list(t2) == [1, 2, 4]
    # tEnter = 3 > tm_z = 1 only
    ch, t1, t2 = oracle.find_first_child([3, 1, 0], [5, 9, 2])
    assert ch == 4
    assert list(t1) == [3, 1, 1] and list(t2) == [4, 5, 2]
    # tEnter equal to a midpoint is not "greater": the low half is chosen
    ch, t1, t2 = oracle.find_first_child([2, 0, 0], [4, 4, 4])
    assert ch == 0


def test_go_next_known_answers(oracle):
    ok, ch, t1, t2 = oracle.go_next(0, [0, 0, 0], [1, 2, 3])
    assert ok and ch == 1 and list(t1) == [1, 0, 0] and list(t2) == [2, 2, 3]
    # exit axis already stepped -> leave the node
    ok, ch, _, _ = oracle.go_next(1, [0, 0, 0], [1, 2, 3])
    assert not ok and ch == 1
    # tie order (trace_spu.cpp:75-78): t2x == t2y -> x unless z smaller
    ok, ch, _, _ = oracle.go_next(0, [0, 0, 0], [2, 2, 3])
    assert ok and ch == 1
    # t2x > t2y == t2z -> z
    ok, ch, _, _ = oracle.go_next(0, [0, 0, 0], [3, 2, 2])
    assert ok and ch == 4
    # all equal -> z
    ok, ch, _, _ = oracle.go_next(0, [0, 0, 0], [2, 2, 2])
    assert ok and ch == 4


def test_setup_trace_mirrors_negative_axes(oracle):
    ok, t1, t2, flags = oracle.setup_trace([0.5, 0.5, 2.0], [0, 0, -1])
    assert ok and flags == 0b100 | 0  # z mirrored; x,y adjusted to +1e-5
    # mirrored z: p = 1-2 = -1, d = 1 -> t1 = 1, t2 = 2
    assert t1[2] == 1.0 and t2[2] == 2.0
    # x,y: eps direction 1e-5 from 0.5: t1 = -0.5/1e-5, t2 = +0.5/1e-5
    assert t1[0] == np.float32(-0.5) / np.float32(1e-5)
    # beside the cube: the x slab interval lies entirely before the y slab
    ok, *_ = oracle.setup_trace([2.0, 0.5, 0.5], [0, 1, 0])
    assert not ok
    # behind the cube still sets up (max(t1) < min(t2)); RecTrace rejects it
    ok, t1, t2, _ = oracle.setup_trace([2.0, 2.0, 2.0], [1, 1, 1])
    assert ok and t2.max() < 0


# --------------------------------------------------------------- hand scenes
def test_single_leaf_hit(oracle):
    # root whose child 0 ([0,.5]^3) is a leaf with VoxData 0
    nodes = pool(make_node([0, EMPTY, EMPTY, EMPTY, EMPTY, EMPTY, EMPTY, EMPTY], 0b1))
    hit, word, t, f, lvl = oracle.trace_ray_f32(nodes, 0, [0.25, 0.25, -1.0], [0, 0, 1])
    assert hit and word == (0 << 3) | 0 and t == 1.0 and f == 1 and lvl == 0
    # x in the upper half: passes child 1 then child 5 (both empty) -> miss
    hit, *_ = oracle.trace_ray_f32(nodes, 0, [0.75, 0.25, -1.0], [0, 0, 1])
    assert not hit


def test_front_to_back_order(oracle):
    # leaves at children 0 and 4 (z low and z high); ray along +z hits 0 at
    # t=1, ray along -z hits 4 at t=1 (entering z=1 from above)
    nodes = pool(make_node([0, EMPTY, EMPTY, EMPTY, 1, EMPTY, EMPTY, EMPTY], 0b10001))
    hit, word, t, *_ = oracle.trace_ray_f32(nodes, 0, [0.25, 0.25, -1.0], [0, 0, 1])
    assert hit and word == 0 and t == 1.0
    hit, word, t, *_ = oracle.trace_ray_f32(nodes, 0, [0.25, 0.25, 2.0], [0, 0, -1])
    assert hit and word == 4 and t == 1.0


def test_two_level_descent_and_fetch_count(oracle):
    # root -> child 7 is node 1; node 1 has a leaf at its child 0, i.e. the
    # voxel [0.5,0.75]^3.  A ray along +x at y=z=0.6 enters root child 6
    # (empty) then child 7 -> node 1 child 0 at x = 0.5 -> t = 1.5 from x=-1.
    root = make_node([EMPTY] * 7 + [1])
    n1 = make_node([7, EMPTY, EMPTY, EMPTY, EMPTY, EMPTY, EMPTY, EMPTY], 0b1)
    nodes = pool(root, n1)
    hit, word, t, f, lvl = oracle.trace_ray_f32(nodes, 0, [-1.0, 0.6, 0.6], [1, 0, 0])
    assert hit and word == (1 << 3) | 0 and t == 1.5 and f == 2 and lvl == 1
    # at y = 0.9 the ray is in node 1's child 2 (empty): miss after 2 fetches
    hit, word, t, f, lvl = oracle.trace_ray_f32(nodes, 0, [-1.0, 0.9, 0.6], [1, 0, 0])
    assert not hit and f == 2


def test_full_and_empty_nodes_are_null(oracle):
    # FullNode children are treated as null (IsNull covers bit 31)
    nodes = pool(make_node([FULL] * 7 + [0], 0b10000000))
    hit, word, t, *_ = oracle.trace_ray_f32(nodes, 0, [0.75, 0.75, -1.0], [0, 0, 1])
    assert hit and word == 7 and t == 1.5  # passes FULL child 3, hits leaf 7
    hit, *_ = oracle.trace_ray_f32(pool(make_node([EMPTY] * 8)), 0, [0.5, 0.5, -1], [0, 0, 1])
    assert not hit
    hit, *_ = oracle.trace_ray_f32(pool(make_node([EMPTY] * 8)), EMPTY, [0.5, 0.5, -1], [0, 0, 1])
    assert not hit


def test_behind_origin_leaf_quirk_and_cull(oracle):
    # RecTrace reports the first leaf on the line even if it lies behind the
    # origin (no t2 test before the leaf check, cell/ppu_renderer.cpp:28-33).
    # Shadow rays use the culling variant that skips such leaves.
    nodes = pool(make_node([0, EMPTY, EMPTY, EMPTY, EMPTY, EMPTY, EMPTY, EMPTY], 0b1))
    hit, word, t, *_ = oracle.trace_ray_f32(nodes, 0, [0.25, 0.25, 0.9], [0, 0, 1])
    assert hit and word == 0 and t < 0
    hit, *_ = oracle.trace_ray_f32(nodes, 0, [0.25, 0.25, 0.9], [0, 0, 1], cull_behind=True)
    assert not hit


def test_malformed_pool_reports_error(oracle):
    nodes = pool(make_node([5] + [EMPTY] * 7))  # child index outside the pool
    with pytest.raises(RuntimeError):
        oracle.trace_ray_f32(nodes, 0, [0.25, 0.25, -1.0], [0, 0, 1])


def test_camera_basis_matches_formula(oracle):
    d0, du, dv = oracle.init_ray_dir_f64([1, 0, 0], [0, 0, 1], 90.0, 4, 2)
    # vfwd = x, vright = x^z = -y, vup = vright^vfwd = z; da = tan(45)/4
    da = 1.0 / 4
    assert np.allclose(du, [0, -2 * da, 0]) and np.allclose(dv, [0, 0, -2 * da])
    assert np.allclose(d0, [1, 2 * da * 2, 2 * da * 1])


# ------------------------------------------------------------ golden pinning
GOLDEN = os.path.join(ROOT, "tests", "golden")


@pytest.mark.parametrize("name", ["svo_spheres_d5", "svo_terrain_d6"])
def test_oracle_reproduces_golden_fixture(oracle, name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    o = oracle.svo_render(g["nodes"], int(g["root"]), g["attrs"], g["pos"], g["view"],
                          [0, 0, 1], float(g["fov"]), int(g["width"]), int(g["height"]),
                          g["light"], shadows=bool(g["shadows"]))
    for k in ("rgba", "hit", "hit_t", "fetches", "shadow_fetches"):
        assert np.array_equal(o[k], g[k]), k


def test_f32_and_f64_oracles_agree_up_to_ties(oracle, yoxel_mod):
    s = yoxel_mod.SVOScene.spheres(6, 40, 2.0, 8.0, 7)
    pos, view = camera_for()
    o = oracle.svo_render(s.nodes_u32, s.root, s.attrs_u8, pos, view, [0, 0, 1], 60, 96, 96,
                          LIGHT)
    h64, _ = oracle.svo_hits_f64(s.nodes_u32, s.root, pos, view, [0, 0, 1], 60, 96, 96)
    assert (o["hit"] != h64).mean() < 1e-3
    assert (o["hit"] != 0xFFFFFFFF).mean() > 0.1
