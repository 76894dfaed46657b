"""Multi-GPU host logic: partitioning and the training exchange step.

Rays are independent, so rendering shards with no data-path collective:
every GPU holds a replica of the scene and renders its share - whole scenes
of a batch (largest-first greedy on a cost estimate) or bands of 8x4-pixel
tiles of one frame (contiguous ranges of equal estimated cost) - and the
frames are gathered to one rank at the end.  The differentiable volume is
data-parallel over cameras with one exchange step per iteration: a sum
all-reduce of the density / albedo gradient tensors.  torch.distributed
(NCCL on GPUs, gloo on CPUs) carries the gather and the all-reduce.
"""
import numpy as np


def partition_scenes(costs, world):
    """Scene indices per rank: greedy longest-processing-time assignment of
    `costs` (e.g. pixels x depth) to `world` ranks.  Deterministic."""
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    load = [0.0] * world
    out = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        out[r].append(i)
        load[r] += float(costs[i])
    for lst in out:
        lst.sort()
    return out


def partition_tiles(tile_costs, world):
    """Contiguous [begin, end) tile ranges per rank with near-equal summed
    cost (prefix-sum split); every tile is assigned exactly once."""
    c = np.asarray(tile_costs, np.float64)
    n = len(c)
    if n == 0:
        return [(0, 0)] * world
    pref = np.concatenate([[0.0], np.cumsum(c)])
    total = pref[-1]
    bounds = [0]
    for r in range(1, world):
        target = total * r / world
        k = int(np.searchsorted(pref, target, side="left"))
        k = min(max(k, bounds[-1]), n)
        bounds.append(k)
    bounds.append(n)
    return [(bounds[r], bounds[r + 1]) for r in range(world)]


def tile_costs(pixel_cost, width, height):
    """Cost per 8x4-pixel tile (row-major tiles, the order of
    yv_render_frame_tiles) from a per-pixel cost map (h, w), e.g. the node
    fetches of a previous frame; every tile costs at least 1."""
    c = np.asarray(pixel_cost, np.float64).reshape(height, width)
    tx, ty = (width + 7) // 8, (height + 3) // 4
    pad = np.zeros((ty * 4, tx * 8), np.float64)
    pad[:height, :width] = c
    return pad.reshape(ty, 4, tx, 8).sum(axis=(1, 3)).reshape(-1) + 1.0


def tile_rows(tile_range, width, height):
    """Pixel rows [y0, y1) covered by a range of 8x4 tiles."""
    tb, te = tile_range
    tx = (width + 7) // 8
    if te <= tb:
        return 0, 0
    return (tb // tx) * 4, min(height, ((te - 1) // tx + 1) * 4)


def volume_tile_order(width, height):
    """Tile coordinates (tile column, tile row) of the warp tiles of one
    camera's volume frame in the march's order (yv_volume_render_tiles):
    16x16-pixel squares row-major, 8 tiles of 8x4 pixels per square (tile
    column within the square fastest).  Padding tiles lie outside the
    frame."""
    tx, ty = (width + 7) // 8, (height + 3) // 4
    stx, sty = (tx + 1) // 2, (ty + 3) // 4
    ids = np.arange(stx * sty * 8)
    st, w = ids >> 3, ids & 7
    return (st % stx) * 2 + (w & 1), (st // stx) * 4 + (w >> 1)


def volume_tile_costs(pixel_cost, width, height):
    """Cost per warp tile of volume frames in the march's order, camera-major,
    from a per-pixel cost map ((ncams,) h, w), e.g. the samples of a previous
    frame; every tile costs at least 1 (padding tiles too)."""
    c = np.asarray(pixel_cost, np.float64).reshape(-1, height, width)
    n = c.shape[0]
    tx, ty = (width + 7) // 8, (height + 3) // 4
    stx, sty = (tx + 1) // 2, (ty + 3) // 4
    pad = np.zeros((n, sty * 16, stx * 16), np.float64)
    pad[:, :height, :width] = c
    per_tile = pad.reshape(n, sty * 4, 4, stx * 2, 8).sum(axis=(2, 4))
    ox, oy = volume_tile_order(width, height)
    return per_tile[:, oy, ox].reshape(-1) + 1.0


def partition_volume_tiles(tile_costs, world):
    """partition_tiles with every boundary on a multiple of 8 tiles (one
    16x16-pixel square, the footprint of a block of the march)."""
    c = np.asarray(tile_costs, np.float64)
    n = len(c)
    sq = c.reshape(-1, 8).sum(axis=1) if n % 8 == 0 else c
    if n % 8:
        raise ValueError("volume tile counts are multiples of 8")
    return [(8 * b, 8 * e) for b, e in partition_tiles(sq, world)]


def volume_tile_rows(tile_range, width, height):
    """Pixel rows [y0, y1) of one camera's frame covered by a range of warp
    tiles of the march's order (within one camera: ids < volume_tile_count)."""
    tb, te = tile_range
    if te <= tb:
        return 0, 0
    stx = ((width + 7) // 8 + 1) // 2
    return (tb // 8 // stx) * 16, min(height, ((te - 1) // 8 // stx + 1) * 16)


def partition_cameras(ncams, world):
    """Contiguous camera ranges per rank (data parallelism over views)."""
    base, extra = divmod(ncams, world)
    out, start = [], 0
    for r in range(world):
        k = base + (1 if r < extra else 0)
        out.append((start, start + k))
        start += k
    return out


def sum_gradients(tensors, group=None):
    """The exchange step of data-parallel training: in-place sum all-reduce."""
    import torch.distributed as dist
    for t in tensors:
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return tensors


def gather_to_root(tensor, world, rank, group=None):
    """Gathers equally shaped per-rank tensors to rank 0 (list on rank 0,
    None elsewhere)."""
    import torch
    import torch.distributed as dist
    if rank == 0:
        bufs = [torch.empty_like(tensor) for _ in range(world)]
        dist.gather(tensor, gather_list=bufs, dst=0, group=group)
        return bufs
    dist.gather(tensor, dst=0, group=group)
    return None
