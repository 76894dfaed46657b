"""GPU brick-volume build from a dense lattice vs the host RangeBuilder
(yv_volume_from_dense): identical grids, brick order, lattice values,
colours, cells and neighbour tables; device pools built straight from the
lattice render exactly like uploads of the host build, in every format."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def lattice(levels, seed, kind):
    n = 8 * 4 ** levels + 1
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(*(np.arange(n, dtype=np.float32),) * 3, indexing="ij")
    if kind == "blobs":
        d = np.zeros((n, n, n), np.float32)
        for _ in range(5):
            c = rng.uniform(0, n, 3).astype(np.float32)
            r = np.float32(rng.uniform(n / 10, n / 4))
            d = np.maximum(d, np.clip(1 - np.sqrt((x - c[0]) ** 2 + (y - c[1]) ** 2 +
                                                  (z - c[2]) ** 2) / r, 0, 1))
        return d.astype(np.float32)
    d = rng.random((n, n, n)).astype(np.float32)
    d[d < 0.995] = 0.0  # sparse specks
    return d


@pytest.mark.parametrize("levels,seed,kind,with_rgb", [(1, 1, "blobs", True),
                                                       (2, 2, "blobs", False),
                                                       (2, 3, "specks", True)])
def test_gpu_volume_build_matches_host(yoxel_mod, levels, seed, kind, with_rgb):
    import torch
    d = lattice(levels, seed, kind)
    n = d.shape[0]
    rgb = (np.random.default_rng(seed + 9).integers(0, 256, (n, n, n, 3), dtype=np.uint8)
           if with_rgb else None)
    host = yoxel_mod.BrickVolume.from_dense(levels, d, rgb)
    g = yoxel_mod.BrickVolume.build_dense(torch.from_numpy(d).cuda(), levels,
                                          None if rgb is None else torch.from_numpy(rgb).cuda())
    assert g.nbricks == host.nbricks and g.ngrids == host.ngrids and host.nbricks > 0
    assert np.array_equal(g.grids, host.grids)
    assert np.array_equal(g.cells, host.cells)
    assert np.array_equal(g.density.view(np.uint32), host.density.view(np.uint32))
    assert np.array_equal(g.albedo_u8, host.albedo_u8)
    for up in (True, False):
        assert np.array_equal(g.neighbors(up), host.neighbors(up))


@pytest.mark.parametrize("precision", [0, 1, 2, 3])
def test_device_pool_from_lattice_renders_like_upload(yoxel_mod, precision):
    import torch
    levels = 2
    d = lattice(levels, 4, "blobs")
    n = d.shape[0]
    rgb = np.random.default_rng(5).integers(0, 256, (n, n, n, 3), dtype=np.uint8)
    host = yoxel_mod.BrickVolume.from_dense(levels, d, rgb)
    up = host.upload(precision)
    gv = yoxel_mod.VolumeGPU.from_dense(torch.from_numpy(d).cuda(), levels, precision,
                                        torch.from_numpy(rgb).cuda())
    cams = yoxel_mod.sphere_cameras(3)
    a = yoxel_mod.render_volume(up.desc(), cams, 40, 32)
    b = yoxel_mod.render_volume(gv.desc(), cams, 40, 32)
    assert torch.equal(a.view(torch.int32), b.view(torch.int32))
    assert a[..., 3].max() > 0.1


@pytest.mark.parametrize("levels", [1, 2])
def test_gpu_volume_build_empty_lattice(yoxel_mod, levels):
    import torch
    n = 8 * 4 ** levels + 1
    host = yoxel_mod.BrickVolume.from_dense(levels, np.zeros((n, n, n), np.float32))
    g = yoxel_mod.BrickVolume.build_dense(torch.zeros((n, n, n), device="cuda"), levels)
    assert g.nbricks == 0 == host.nbricks and np.array_equal(g.grids, host.grids)


@pytest.mark.parametrize("precision", [2, 3])
def test_rebuild_in_place_renders_like_fresh_build(yoxel_mod, precision):
    """BrickPool::Update: rebuilding a device pool in place from a new
    lattice (smaller, then larger than the first) renders exactly like a
    fresh build of that lattice."""
    import torch
    levels = 2
    a = lattice(levels, 11, "blobs")
    b = lattice(levels, 3, "specks")  # fewer bricks
    c = lattice(levels, 12, "blobs")
    cams = yoxel_mod.sphere_cameras(3)
    vol = yoxel_mod.VolumeGPU.from_dense(torch.from_numpy(a).cuda(), levels, precision)
    for nxt in (b, c, a):
        t = torch.from_numpy(nxt).cuda()
        vol.rebuild_dense(t, levels)
        fresh = yoxel_mod.VolumeGPU.from_dense(t, levels, precision)
        assert vol.desc().nbricks == fresh.desc().nbricks
        x = yoxel_mod.render_volume(vol.desc(), cams, 40, 32)
        y = yoxel_mod.render_volume(fresh.desc(), cams, 40, 32)
        assert torch.equal(x.view(torch.int32), y.view(torch.int32))


def device_mask(desc):
    """The cell occupancy mask words of a device pool (a view of the
    library's array)."""
    import torch
    n = desc.nbricks * 16

    class _Words:
        __cuda_array_interface__ = {"shape": (n,), "typestr": "<i4",
                                    "data": (desc.cell_mask, False), "version": 2}

    return torch.as_tensor(_Words(), device="cuda").cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("precision", [0, 1, 2, 3])
def test_pack_kernel_cell_mask_matches_upload(yoxel_mod, precision):
    """The occupancy mask the pack kernel builds with a device pool (from a
    lattice, and rebuilt in place) equals the mask computed from the stored
    corners of an upload of the host build - lattice values that the fp16
    formats round to zero included."""
    import torch
    levels = 2
    d = lattice(levels, 6, "blobs")
    rng = np.random.default_rng(7)
    tiny = rng.random(d.shape) < 0.002
    d[tiny] = np.float32(1e-9)  # non-zero in fp32, zero once stored as fp16
    host = yoxel_mod.BrickVolume.from_dense(levels, d)
    up = host.upload(precision)
    gv = yoxel_mod.VolumeGPU.from_dense(torch.from_numpy(d).cuda(), levels, precision)
    assert gv.desc().cell_mask and gv.desc().nbricks == host.nbricks
    want = device_mask(up.desc())
    assert np.array_equal(device_mask(gv.desc()), want)
    assert 0 < np.unpackbits(want.view(np.uint8)).mean() < 1
    # in place, over a pool that held other bricks
    other = yoxel_mod.VolumeGPU.from_dense(torch.from_numpy(lattice(levels, 12, "blobs")).cuda(),
                                           levels, precision)
    other.rebuild_dense(torch.from_numpy(d).cuda(), levels)
    assert np.array_equal(device_mask(other.desc()), want)


def test_device_build_brick_bits_match_upload(yoxel_mod):
    """The brick bitmap of a pool built from a lattice on the device (fresh
    and rebuilt in place) equals that of an upload of the host build."""
    import torch
    levels = 2
    d = lattice(levels, 8, "blobs")
    host = yoxel_mod.BrickVolume.from_dense(levels, d)
    up = host.upload(3)
    n = (4 ** (3 * levels) + 31) // 32

    def bits(desc):
        class _Words:
            __cuda_array_interface__ = {"shape": (n,), "typestr": "<i4",
                                        "data": (desc.brick_bits, False), "version": 2}
        return torch.as_tensor(_Words(), device="cuda").cpu().numpy()

    want = bits(up.desc())
    gv = yoxel_mod.VolumeGPU.from_dense(torch.from_numpy(d).cuda(), levels, 3)
    assert np.array_equal(bits(gv.desc()), want)
    other = yoxel_mod.VolumeGPU.from_dense(torch.from_numpy(lattice(levels, 3, "specks")).cuda(),
                                           levels, 3)
    other.rebuild_dense(torch.from_numpy(d).cuda(), levels)
    assert np.array_equal(bits(other.desc()), want)
