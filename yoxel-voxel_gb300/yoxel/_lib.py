"""ctypes binding of libyoxel.so (the C ABI declared in include/yv_c_api.h).

The shared library is built in-tree by yoxel-voxel_gb300/build.py.  There is
no fallback: if the library is missing, importing this module raises.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libyoxel.so")

# status codes (yv_c_api.h)
YV_OK = 0
YV_ERR_INVALID_ARG = 1
YV_ERR_NO_SCENE = 2
YV_ERR_BAD_POOL = 3
YV_ERR_ITERATION_CAP = 4
YV_ERR_TIMEOUT = 5
YV_ERR_CUDA = 6
YV_ERR_OUT_OF_MEMORY = 7
YV_ERR_IO = 8
YV_ERR_UNSUPPORTED = 9

YV_EMPTY_NODE = 0x80000000
YV_FULL_NODE = 0x80000001


class YvError(RuntimeError):
    """A yv_status other than YV_OK."""

    def __init__(self, status, what=""):
        self.status = status
        msg = f"{what}: {status_string(status)} ({status})"
        detail = last_error()
        if detail:
            msg += f" - {detail}"
        super().__init__(msg)


class VoxNode(C.Structure):
    _fields_ = [("flags", C.c_uint32), ("data", C.c_uint32), ("child", C.c_uint32 * 8)]


class LeafAttr(C.Structure):
    _fields_ = [("r", C.c_uint8), ("g", C.c_uint8), ("b", C.c_uint8), ("a", C.c_uint8),
                ("nx", C.c_int8), ("ny", C.c_int8), ("nz", C.c_int8), ("nw", C.c_int8)]


class Light(C.Structure):
    _fields_ = [("dir", C.c_float * 3), ("ambient", C.c_float), ("diffuse", C.c_float),
                ("shadows", C.c_int32)]


class FrameOutputs(C.Structure):
    _fields_ = [("rgba", C.c_void_p), ("hit", C.c_void_p), ("hit_t", C.c_void_p),
                ("fetches", C.c_void_p), ("shadow_fetches", C.c_void_p),
                ("normal", C.c_void_p)]


YV_SSNA_MAX_LIGHTS = 4


class PointLight(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("diffuse", C.c_float * 3),
                ("specular", C.c_float * 3), ("attenuation", C.c_float * 3),
                ("enabled", C.c_int32)]


class SsnaParams(C.Structure):
    _fields_ = [("ssna", C.c_int32), ("show_normals", C.c_int32),
                ("blur_passes", C.c_int32), ("voxel_size", C.c_float),
                ("edge_threshold", C.c_float), ("edge_pad", C.c_float),
                ("ambient", C.c_float * 3), ("specular_exp", C.c_float),
                ("lights", PointLight * YV_SSNA_MAX_LIGHTS)]


class FrameStats(C.Structure):
    _fields_ = [("primary_rays", C.c_uint64), ("hits", C.c_uint64),
                ("shadow_rays", C.c_uint64), ("shadowed", C.c_uint64),
                ("status", C.c_uint32), ("launches", C.c_uint32)]


class LaunchConfig(C.Structure):
    _fields_ = [("block_threads", C.c_int32), ("blocks_per_sm", C.c_int32),
                ("smem_nodes", C.c_int32), ("tile_rays", C.c_int32)]


class VolumeDevice(C.Structure):
    _fields_ = [("grids", C.c_void_p), ("ngrids", C.c_uint32), ("levels", C.c_int32),
                ("density", C.c_void_p), ("albedo", C.c_void_p), ("nbricks", C.c_uint32),
                ("precision", C.c_int32), ("nbr_up", C.c_void_p), ("nbr_dn", C.c_void_p),
                ("cell_mask", C.c_void_p), ("brick_bits", C.c_void_p)]


class Camera(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("dir", C.c_float * 3), ("up", C.c_float * 3),
                ("fov_deg", C.c_float)]


class MarchParams(C.Structure):
    _fields_ = [("alpha_scale", C.c_float), ("step_vox", C.c_float)]


YV_PRECISION_F16 = 0
YV_PRECISION_F32 = 1
YV_PRECISION_F32_PACKED = 2
YV_PRECISION_F16_PACKED = 3

F3 = C.c_float * 3
P = C.c_void_p
U32 = C.c_uint32
I32 = C.c_int
S = C.c_int32  # yv_status

# name -> (restype, argtypes); every symbol include/yv_c_api.h declares
_SIGS = {
    "yv_status_string": (C.c_char_p, [S]),
    "yv_last_error": (C.c_char_p, []),
    "yv_svo_gen_spheres": (S, [C.POINTER(P), I32, I32, C.c_float, C.c_float, C.c_uint64]),
    "yv_svo_gen_terrain": (S, [C.POINTER(P), I32, I32, I32, I32, C.c_uint64]),
    "yv_svo_from_arrays": (S, [C.POINTER(P), P, U32, U32, P, U32]),
    "yv_svo_load_vox": (S, [C.POINTER(P), C.c_char_p]),
    "yv_svo_save_vox": (S, [P, C.c_char_p]),
    "yv_svo_build_lod": (S, [P]),
    "yv_svo_has_lod": (I32, [P]),
    "yv_svo_free": (None, [P]),
    "yv_svo_node_count": (U32, [P]),
    "yv_svo_root": (U32, [P]),
    "yv_svo_nodes": (P, [P]),
    "yv_svo_attr_count": (U32, [P]),
    "yv_svo_attrs": (P, [P]),
    "yv_svo_depth": (I32, [P]),
    "yv_svo_validate": (S, [P, U32, U32, U32]),
    "yv_svo_build_dense": (S, [P, P, C.c_int32, C.c_float, P, C.POINTER(P)]),
    "yv_renderer_create": (S, [C.POINTER(P)]),
    "yv_renderer_destroy": (None, [P]),
    "yv_set_scene_svo": (S, [P, P, U32, U32, P, U32]),
    "yv_set_scene_host": (S, [P, P]),
    "yv_load_scene_vox": (S, [P, C.c_char_p]),
    "yv_set_scene_dense": (S, [P, P, P, C.c_int32, C.c_float, P]),
    "yv_set_scene_dynamic": (S, [P, P]),
    "yv_set_scene_svo_packed": (S, [P, P, U32, U32]),
    "yv_svo_from_packed": (S, [C.POINTER(P), P, U32, U32]),
    "yv_set_view_pos": (S, [P, F3]),
    "yv_set_view_dir": (S, [P, F3]),
    "yv_set_view_up": (S, [P, F3]),
    "yv_set_resolution": (S, [P, I32, I32]),
    "yv_get_resolution": (S, [P, C.POINTER(I32), C.POINTER(I32)]),
    "yv_set_fov": (S, [P, C.c_float]),
    "yv_get_fov": (S, [P, C.POINTER(C.c_float)]),
    "yv_set_detail_coef": (S, [P, C.c_float]),
    "yv_get_detail_coef": (S, [P, C.POINTER(C.c_float)]),
    "yv_set_frame_budget": (S, [P, C.c_uint32]),
    "yv_get_frame_budget": (S, [P, C.POINTER(C.c_uint32)]),
    "yv_set_light": (S, [P, C.POINTER(Light)]),
    "yv_set_launch_config": (S, [P, C.POINTER(LaunchConfig)]),
    "yv_get_launch_config": (S, [P, C.POINTER(LaunchConfig)]),
    "yv_render_frame": (S, [P, P, P, P]),
    "yv_render_frame_async": (S, [P, C.POINTER(FrameOutputs), P]),
    "yv_render_frame_tiles": (S, [P, U32, U32, C.POINTER(FrameOutputs), P]),
    "yv_get_tile_count": (S, [P, C.POINTER(U32), C.POINTER(U32)]),
    "yv_renderer_frame_stats": (S, [P, C.POINTER(FrameStats)]),
    "yv_get_ray_basis": (S, [P, F3, F3, F3]),
    "yv_get_device_scene_info": (S, [P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "yv_volume_gen_noise": (S, [C.POINTER(P), I32, C.c_float, C.c_float, C.c_uint64]),
    "yv_volume_from_dense": (S, [C.POINTER(P), I32, P, P]),
    "yv_volume_free": (None, [P]),
    "yv_volume_levels": (I32, [P]),
    "yv_volume_grid_count": (U32, [P]),
    "yv_volume_grids": (P, [P]),
    "yv_volume_brick_count": (U32, [P]),
    "yv_volume_density": (P, [P]),
    "yv_volume_albedo": (P, [P]),
    "yv_volume_brick_cells": (P, [P]),
    "yv_volume_neighbors": (P, [P, I32]),
    "yv_volume_upload": (S, [P, C.c_int32, C.POINTER(P)]),
    "yv_volume_gpu_free": (None, [P]),
    "yv_volume_build_dense": (S, [P, P, C.c_int32, P, C.POINTER(P)]),
    "yv_volume_upload_dense": (S, [P, P, C.c_int32, C.c_int32, P, C.POINTER(P)]),
    "yv_volume_rebuild_dense": (S, [P, P, P, C.c_int32, P]),
    "yv_volume_gpu_desc": (S, [P, C.POINTER(VolumeDevice)]),
    "yv_volume_brick_bits": (S, [C.POINTER(VolumeDevice), P, P]),
    "yv_volume_tile_count": (S, [C.c_int32, C.c_int32, C.POINTER(C.c_uint32)]),
    "yv_volume_render_tiles": (S, [C.POINTER(VolumeDevice), C.POINTER(Camera), C.c_int32,
                                   C.c_int32, C.c_int32, C.POINTER(MarchParams), C.c_uint32,
                                   C.c_uint32, P, P, P, P]),
    "yv_volume_render": (S, [C.POINTER(VolumeDevice), C.POINTER(Camera), C.c_int32, C.c_int32,
                             C.c_int32, C.POINTER(MarchParams), P, P, P, P]),
    "yv_volume_render_rgba8": (S, [C.POINTER(VolumeDevice), C.POINTER(Camera), C.c_int32,
                                   C.c_int32, C.c_int32, C.POINTER(MarchParams), P, P]),
    "yv_volume_backward": (S, [C.POINTER(VolumeDevice), C.POINTER(Camera), C.c_int32,
                               C.c_int32, C.c_int32, C.POINTER(MarchParams), P, P, P, P, P]),
    "yv_volume_fold_aprons": (S, [C.POINTER(VolumeDevice), P, P, P]),
    "yv_volume_sync_aprons": (S, [C.POINTER(VolumeDevice), P, P, P]),
    "yv_volume_pack": (S, [P, P, C.c_uint32, P, P]),
    "yv_batch_create": (S, [C.POINTER(P)]),
    "yv_batch_destroy": (None, [P]),
    "yv_batch_clear": (S, [P]),
    "yv_batch_add_svo": (S, [P, P, P]),
    "yv_batch_add_svo_outputs": (S, [P, P, C.POINTER(FrameOutputs)]),
    "yv_batch_add_volume": (S, [P, C.POINTER(VolumeDevice), C.POINTER(Camera), C.c_int32,
                                C.c_int32, C.POINTER(MarchParams), P]),
    "yv_batch_set_launch_config": (S, [P, C.POINTER(LaunchConfig)]),
    "yv_batch_render": (S, [P, C.c_int32, P]),
    "yv_batch_render_separate": (S, [P, P]),
    "yv_batch_info": (S, [P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint64)]),
    "yv_svo_dynamic_create": (S, [U32, U32, C.POINTER(P)]),
    "yv_svo_dynamic_destroy": (None, [P]),
    "yv_svo_dynamic_load": (S, [P, P]),
    "yv_svo_dynamic_alloc_node": (S, [P, C.POINTER(U32)]),
    "yv_svo_dynamic_free_node": (S, [P, U32]),
    "yv_svo_dynamic_set_node": (S, [P, U32, P]),
    "yv_svo_dynamic_get_node": (S, [P, U32, P]),
    "yv_svo_dynamic_add_attr": (S, [P, P, C.POINTER(U32)]),
    "yv_svo_dynamic_set_attr": (S, [P, U32, P]),
    "yv_svo_dynamic_set_root": (S, [P, U32, C.c_int32]),
    "yv_svo_dynamic_set_voxel": (S, [P, C.c_int32, U32, U32, U32, P]),
    "yv_svo_dynamic_changed_pages": (U32, [P]),
    "yv_svo_dynamic_transfer_bytes": (C.c_uint64, [P]),
    "yv_svo_dynamic_sync": (S, [P, P]),
    "yv_svo_dynamic_device": (S, [P, C.POINTER(P), C.POINTER(U32), C.POINTER(U32),
                                  C.POINTER(P), C.POINTER(U32)]),
    "yv_svo_dynamic_host_nodes": (P, [P]),
    "yv_svo_dynamic_host_attrs": (P, [P]),
    "yv_svo_dynamic_download": (S, [P, P, P]),
    "yv_svo_dynamic_host_info": (S, [P, C.POINTER(U32), C.POINTER(U32), C.POINTER(U32)]),
    "yv_render_svo_noalloc": (S, [P, U32, U32, P, U32, C.POINTER(Camera), C.POINTER(Light),
                                  C.c_int32, C.c_int32, C.POINTER(FrameOutputs), P]),
    "yv_render_svo_noalloc_status": (S, [P, C.POINTER(U32)]),
    "yv_ssna_defaults": (S, [P, C.POINTER(SsnaParams)]),
    "yv_render_ssna": (S, [P, C.POINTER(SsnaParams), P, P, P, P]),
    "yv_renderer_trace_dump": (S, [P, P, P, P]),
}


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build it with "
            "`python yoxel-voxel_gb300/build.py` (or __graft_entry__.build())")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


def status_string(s):
    return lib.yv_status_string(s).decode()


def last_error():
    v = lib.yv_last_error()
    return v.decode() if v else ""


def check(status, what=""):
    if status != YV_OK:
        raise YvError(status, what)
    return status


def declared_symbols():
    """Names of all C ABI entry points this binding declares."""
    return sorted(_SIGS)
