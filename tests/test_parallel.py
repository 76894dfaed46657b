"""Multi-GPU host logic, exercised on CPU ranks (gloo, world size 2).

The ray caster shards with no data-path collective (scene replicas, tile or
scene partitions, a gather of frames at the end); training is data-parallel
over cameras with one exchange step, a sum all-reduce of the gradients."""
import os
import socket
import sys

import numpy as np
import pytest

from conftest import PKG, ROOT


def test_partition_scenes_balances_and_covers():
    from yoxel import parallel as P
    costs = [100, 80, 60, 55, 40, 30, 20, 10, 5, 1]
    parts = P.partition_scenes(costs, 3)
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(costs)))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(costs)
    assert P.partition_scenes(costs, 3) == parts  # deterministic


def test_partition_tiles_contiguous_and_balanced():
    from yoxel import parallel as P
    rng = np.random.default_rng(0)
    c = rng.random(1000) * 10
    parts = P.partition_tiles(c, 4)
    assert parts[0][0] == 0 and parts[-1][1] == 1000
    for (a, b), (a2, _) in zip(parts, parts[1:]):
        assert b == a2 and a <= b
    sums = [c[a:b].sum() for a, b in parts]
    assert max(sums) - min(sums) <= 2 * c.max()
    assert P.partition_tiles([], 3) == [(0, 0)] * 3


def test_partition_cameras():
    from yoxel import parallel as P
    assert P.partition_cameras(64, 2) == [(0, 32), (32, 64)]
    assert P.partition_cameras(5, 3) == [(0, 2), (2, 4), (4, 5)]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    sys.path[:0] = [ROOT, PKG]
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from yoxel import parallel as P
    # data-parallel gradient: rank r holds the gradient of its camera shard
    cams = P.partition_cameras(8, world)[rank]
    g = torch.zeros(6, dtype=torch.float64)
    for c in range(*cams):
        g += torch.arange(6, dtype=torch.float64) * (c + 1)
    P.sum_gradients([g])
    # frame gather: every rank renders its tile band (here: a fake frame)
    frame = torch.full((4,), float(rank), dtype=torch.float32)
    frames = P.gather_to_root(frame, world, rank)
    q.put((rank, g.tolist(), None if frames is None else [f.tolist() for f in frames]))
    dist.destroy_process_group()


def test_gloo_gradient_sum_and_frame_gather():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(2):
        rank, g, frames = q.get(timeout=120)
        res[rank] = (g, frames)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    full = (np.arange(6) * sum(range(1, 9))).tolist()
    assert res[0][0] == full and res[1][0] == full
    assert res[0][1] == [[0.0] * 4, [1.0] * 4] and res[1][1] is None


def _shard_worker(rank, world, port, q):
    """A sharded frame as bench.py runs it: every rank derives the same tile
    ranges from the same cost map (no communication), paints the pixels of
    its ranges, and rank 0 gathers the frames."""
    sys.path[:0] = [ROOT, PKG]
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from yoxel import parallel as P
    w, h = 37, 23
    cost = np.random.default_rng(7).integers(1, 60, (h, w))
    ranges = P.partition_tiles(P.tile_costs(cost, w, h), world)
    tb, te = ranges[rank]
    tx = (w + 7) // 8
    frame = torch.full((h, w), -1.0)
    for t in range(tb, te):
        frame[(t // tx) * 4:(t // tx) * 4 + 4, (t % tx) * 8:(t % tx) * 8 + 8] = float(rank)
    y0, y1 = P.tile_rows((tb, te), w, h)
    painted_rows = torch.nonzero((frame >= 0).any(dim=1)).flatten().tolist()
    frames = P.gather_to_root(frame, world, rank)
    q.put((rank, ranges, (y0, y1), painted_rows,
           None if frames is None else [f.numpy() for f in frames]))
    dist.destroy_process_group()


def test_gloo_sharded_frame_tiles_cover_the_frame_once():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    world = 3
    procs = [ctx.Process(target=_shard_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(world):
        rank, ranges, rows, painted, frames = q.get(timeout=120)
        res[rank] = (ranges, rows, painted, frames)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert all(res[r][0] == res[0][0] for r in range(world))
    frames = res[0][3]
    merged = np.full(frames[0].shape, -1.0)
    for r, f in enumerate(frames):
        mine = f >= 0
        assert (merged[mine] < 0).all()  # no pixel painted twice
        merged[mine] = f[mine]
        painted = res[r][2]
        y0, y1 = res[r][1]
        assert all(y0 <= y < y1 for y in painted)  # the rows read back hold the tiles
    assert (merged >= 0).all()  # every pixel painted once


def test_volume_tile_order_covers_the_frame_in_squares():
    """The march's tile order: every 8x4 tile of the (padded) frame once,
    8 consecutive ids on one 16x16-pixel square; costs follow the order and
    ranges split on square boundaries cover every tile once."""
    from yoxel import parallel as P
    for w, h in [(64, 32), (33, 17), (1024, 1024), (100, 60)]:
        ox, oy = P.volume_tile_order(w, h)
        tx, ty = (w + 7) // 8, (h + 3) // 4
        assert len(ox) % 8 == 0
        seen = set(zip(ox.tolist(), oy.tolist()))
        assert len(seen) == len(ox)
        assert {(x, y) for x in range(tx) for y in range(ty)} <= seen
        sq = np.stack([ox // 2, oy // 4], 1).reshape(-1, 8, 2)
        assert (sq == sq[:, :1]).all()
        cost = np.random.default_rng(w).random((2, h, w))
        c = P.volume_tile_costs(cost, w, h)
        assert len(c) == 2 * len(ox)
        k = len(ox) // 2 + 3
        x0, y0 = ox[k] * 8, oy[k] * 4
        assert np.isclose(c[len(ox) + k] - 1.0, cost[1, y0:y0 + 4, x0:x0 + 8].sum())
        for world in (1, 2, 3, 5):
            rs = P.partition_volume_tiles(c, world)
            assert rs[0][0] == 0 and rs[-1][1] == len(c)
            assert all(b % 8 == 0 and e % 8 == 0 and b <= e for b, e in rs)
            assert all(rs[i][1] == rs[i + 1][0] for i in range(world - 1))


def test_volume_tile_rows_hold_the_range():
    """The rows a rank of a split brick frame reads back hold every pixel of
    its tile range (one camera)."""
    from yoxel import parallel as P
    for w, h in [(1024, 1024), (100, 60), (33, 17)]:
        ox, oy = P.volume_tile_order(w, h)
        n = len(ox)
        for world in (2, 3, 4):
            for tb, te in P.partition_volume_tiles(np.ones(n), world):
                y0, y1 = P.volume_tile_rows((tb, te), w, h)
                for t in range(tb, te):
                    if ox[t] * 8 < w and oy[t] * 4 < h:
                        assert y0 <= oy[t] * 4 and min(h, oy[t] * 4 + 4) <= y1

