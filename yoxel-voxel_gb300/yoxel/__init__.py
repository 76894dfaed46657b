"""yoxel - GB300-native sparse-voxel-octree and brick-volume ray caster.

Python side of the C ABI in include/yv_c_api.h (libyoxel.so, built in-tree by
yoxel-voxel_gb300/build.py).  Mirrors the reference's Python driver
trace_cuda.CudaRenderer and its ISVORenderer interface.
"""
from . import _lib
from ._lib import YvError, LIB_PATH
from .svo import SVOScene, NODE_DTYPE, ATTR_DTYPE
from .renderer import Renderer, CudaRenderer
from .volume import (BrickVolume, VolumeGPU, render_volume, render_volume_rgba8,
                     volume_backward, volume_march, torch_desc, pack_volume, brick_bits,
                     render_volume_tiles, volume_tile_count,
                     cameras, sphere_cameras)

from .batch import Batch
from .dynamic import DynamicSVO

__all__ = ["SVOScene", "Renderer", "CudaRenderer", "YvError", "LIB_PATH", "Batch",
           "NODE_DTYPE", "ATTR_DTYPE", "DynamicSVO", "BrickVolume", "VolumeGPU", "render_volume",
           "render_volume_rgba8", "render_volume_tiles", "volume_tile_count",
           "volume_backward", "volume_march", "torch_desc", "pack_volume", "brick_bits",
           "cameras", "sphere_cameras"]
