"""ctypes bindings of libgbr.so (the C ABI declared in include/gbr.h,
include/gbr_replay.h, include/gbr_noise.h and include/gbr_hbao.h)."""
import ctypes
import os

from . import build as _build

c_float_p = ctypes.POINTER(ctypes.c_float)


class Config(ctypes.Structure):
    _fields_ = [("flags", ctypes.c_uint32), ("tile_size", ctypes.c_int32 * 2),
                ("tile_count", ctypes.c_int32 * 2), ("max_light_count", ctypes.c_uint32),
                ("ambient_factor", ctypes.c_float), ("cuda_device", ctypes.c_int32),
                ("standalone_flags", ctypes.c_uint32), ("planes", ctypes.c_uint32),
                ("draw_mode", ctypes.c_uint32), ("scene_count", ctypes.c_uint32),
                ("viewports", ctypes.POINTER(ctypes.c_int32))]


class MeshData(ctypes.Structure):
    _fields_ = [("vertex_count", ctypes.c_uint32), ("positions", ctypes.c_void_p),
                ("colors", ctypes.c_void_p), ("texcoords", ctypes.c_void_p),
                ("object_ids", ctypes.c_void_p), ("index_count", ctypes.c_uint32),
                ("indices", ctypes.c_void_p), ("normals", ctypes.c_void_p)]


class TextureData(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32), ("layers", ctypes.c_int32),
                ("rgba8", ctypes.c_void_p), ("filter", ctypes.c_int32),
                ("wrap_s", ctypes.c_int32), ("wrap_t", ctypes.c_int32),
                ("min_filter", ctypes.c_int32), ("mip_filter", ctypes.c_int32),
                ("levels", ctypes.c_int32), ("generate_mipmap", ctypes.c_int32)]


class MaterialData(ctypes.Structure):
    _fields_ = [("color", ctypes.c_float * 4), ("texture", ctypes.c_uint32),
                ("layer", ctypes.c_uint32), ("matrix", ctypes.c_float * 9),
                ("shaded", ctypes.c_int32)]


class MeshView(ctypes.Structure):
    _fields_ = [("mesh", ctypes.c_uint32), ("index_offset", ctypes.c_uint32),
                ("index_count", ctypes.c_uint32), ("material", ctypes.c_uint32),
                ("transform", ctypes.c_float * 16)]


class SceneStatsInfo(ctypes.Structure):
    _fields_ = [("node_count", ctypes.c_uint64), ("draw_count", ctypes.c_uint64),
                ("draw_batch_count", ctypes.c_uint64)]


class Tuning(ctypes.Structure):
    _fields_ = [("threads", ctypes.c_int32), ("region_width", ctypes.c_int32),
                ("region_height", ctypes.c_int32), ("small_area", ctypes.c_int32),
                ("ctas_per_sm", ctypes.c_int32), ("plain_region_width", ctypes.c_int32),
                ("plain_region_height", ctypes.c_int32), ("occlusion_culling", ctypes.c_int32),
                ("queue_fill_percent", ctypes.c_int32)]


class DrawStats(ctypes.Structure):
    _fields_ = [("scenes", ctypes.c_uint64), ("draws", ctypes.c_uint64),
                ("visible_draws", ctypes.c_uint64), ("triangles", ctypes.c_uint64),
                ("kernel_launches", ctypes.c_uint64), ("prepare_ms", ctypes.c_float),
                ("raster_ms", ctypes.c_float)]


class HbaoConfig(ctypes.Structure):
    _fields_ = [("intensity", ctypes.c_float), ("bias", ctypes.c_float),
                ("radius", ctypes.c_float), ("blur_sharpness", ctypes.c_float),
                ("no_blur", ctypes.c_int32), ("special_blur", ctypes.c_int32),
                ("algorithm", ctypes.c_int32)]


class ReplayConfig(ctypes.Structure):
    _fields_ = [("num_environments", ctypes.c_uint32), ("gpu_device_id", ctypes.c_int32),
                ("standalone", ctypes.c_int32), ("enable_frustum_culling", ctypes.c_int32),
                ("enable_hbao", ctypes.c_int32), ("sensor_uuid", ctypes.c_char_p),
                ("resolution", ctypes.c_int32 * 2), ("hfov_degrees", ctypes.c_float),
                ("near_plane", ctypes.c_float), ("far_plane", ctypes.c_float),
                ("orthographic", ctypes.c_int32), ("ortho_scale", ctypes.c_float),
                ("max_light_count", ctypes.c_uint32), ("ambient_factor", ctypes.c_float),
                ("draw_mode", ctypes.c_uint32), ("quiet", ctypes.c_uint32)]


_P = ctypes.c_void_p
_U32 = ctypes.c_uint32
_I32 = ctypes.c_int32
_U64 = ctypes.c_uint64
_ST = ctypes.c_int

PROTOTYPES = {
    "gbr_config_init": (None, [ctypes.POINTER(Config)]),
    "gbr_create": (_ST, [ctypes.POINTER(Config), ctypes.POINTER(_P)]),
    "gbr_destroy": (None, [_P]),
    "gbr_last_error": (ctypes.c_char_p, []),
    "gbr_tile_size_count": (_ST, [_P, ctypes.POINTER(_I32), ctypes.POINTER(_I32)]),
    "gbr_scene_count": (_ST, [_P, ctypes.POINTER(_U32)]),
    "gbr_framebuffer_size": (_ST, [_P, ctypes.POINTER(ctypes.c_int64)]),
    "gbr_scene_viewport": (_ST, [_P, _U32, ctypes.POINTER(ctypes.c_int64)]),
    "gbr_add_file": (_ST, [_P, ctypes.c_char_p, _U32, ctypes.c_char_p]),
    "gbr_add_mesh": (_ST, [_P, ctypes.POINTER(MeshData), ctypes.POINTER(_U32)]),
    "gbr_add_texture": (_ST, [_P, ctypes.POINTER(TextureData), ctypes.POINTER(_U32)]),
    "gbr_add_material": (_ST, [_P, ctypes.POINTER(MaterialData), ctypes.POINTER(_U32)]),
    "gbr_add_node_hierarchy_template": (_ST, [_P, ctypes.c_char_p, _U32, ctypes.POINTER(MeshView)]),
    "gbr_add_light": (_ST, [_P, _U32, _U64, _U32, ctypes.POINTER(_U64)]),
    "gbr_clear_lights": (_ST, [_P, _U32]),
    "gbr_light_colors": (_ST, [_P, _U32, ctypes.POINTER(c_float_p), ctypes.POINTER(_U64)]),
    "gbr_light_ranges": (_ST, [_P, _U32, ctypes.POINTER(c_float_p), ctypes.POINTER(_U64)]),
    "gbr_set_scene_sources": (_ST, [_P, _U32, _U32, ctypes.POINTER(_U32)]),
    "gbr_set_scene_enabled": (_ST, [_P, _U32, _I32]),
    "gbr_remove_mesh": (_ST, [_P, _U32]),
    "gbr_remove_texture": (_ST, [_P, _U32]),
    "gbr_remove_node_hierarchy_template": (_ST, [_P, ctypes.c_char_p]),
    "gbr_memory_usage": (_ST, [_P, ctypes.POINTER(_U64), ctypes.POINTER(_U64)]),
    "gbr_has_node_hierarchy": (_ST, [_P, ctypes.c_char_p, ctypes.POINTER(_I32)]),
    "gbr_add_node_hierarchy": (_ST, [_P, _U32, ctypes.c_char_p, c_float_p, ctypes.POINTER(_U64)]),
    "gbr_add_empty_node": (_ST, [_P, _U32, ctypes.POINTER(_U64)]),
    "gbr_clear": (_ST, [_P, _U32]),
    "gbr_set_semantic_id": (_ST, [_P, _U32, _U64, _U32]),
    "gbr_update_camera": (_ST, [_P, _U32, c_float_p, c_float_p]),
    "gbr_update_cameras": (_ST, [_P, _U32, _U32, c_float_p, c_float_p]),
    "gbr_camera": (_ST, [_P, _U32, c_float_p]),
    "gbr_camera_depth_unprojection": (_ST, [_P, _U32, c_float_p]),
    "gbr_transformations": (_ST, [_P, _U32, ctypes.POINTER(c_float_p), ctypes.POINTER(_U64)]),
    "gbr_draw": (_ST, [_P, _P]),
    "gbr_draw_mode": (_ST, [_P, _P, _U32, _I32]),
    "gbr_scene_stats": (_ST, [_P, _U32, ctypes.POINTER(SceneStatsInfo)]),
    "gbr_image_into": (_ST, [_P, _U32, ctypes.POINTER(_I32), _P, _U64]),
    "gbr_color_image_into": (_ST, [_P, ctypes.POINTER(_I32), _P, _U64]),
    "gbr_image_into_async": (_ST, [_P, _U32, ctypes.POINTER(_I32), _P, _U64]),
    "gbr_readback_wait": (_ST, [_P]),
    "gbr_scenes_into_async": (_ST, [_P, _U32, _U32, _U32, _P]),
    "gbr_depth_image_into": (_ST, [_P, ctypes.POINTER(_I32), _P, _U64]),
    "gbr_semantic_image_into": (_ST, [_P, ctypes.POINTER(_I32), _P, _U64]),
    "gbr_linear_depth_image_into": (_ST, [_P, ctypes.POINTER(_I32), _P, _U64]),
    "gbr_scene_image_into": (_ST, [_P, _U32, _U32, _P, _U64]),
    "gbr_plane_device_pointer": (_ST, [_P, _U32, ctypes.POINTER(_P), ctypes.POINTER(_U64)]),
    "gbr_plane_dlpack": (_ST, [_P, _U32, ctypes.POINTER(_P)]),
    "gbr_unproject_depth": (_ST, [c_float_p, c_float_p, _U64, _U64, _U64]),
    "gbr_unproject_depth_device": (_ST, [c_float_p, _P, _U64, _U64, _U64, _P]),
    "gbr_get_tuning": (_ST, [_P, ctypes.POINTER(Tuning)]),
    "gbr_set_tuning": (_ST, [_P, ctypes.POINTER(Tuning)]),
    "gbr_last_draw_stats": (_ST, [_P, ctypes.POINTER(DrawStats)]),
    "gbr_set_kernel_timing": (_ST, [_P, _I32]),
    "gbr_set_device_memory_limit": (_ST, [_P, _U64]),
    "gbr_device_memory": (_ST, [_P, ctypes.POINTER(_U64), ctypes.POINTER(_U64)]),
    "gbr_debug_corrupt_parent": (_ST, [_P, _U32, _U64, _I32]),
    "gbr_render_mesh_no_alloc": (_ST, [_P, _P, _P, _U32, _U32, c_float_p, c_float_p, _U32, _I32,
                                       _I32, _I32, _P, _P, _P, _P, _P]),
    # include/gbr_replay.h
    "gbr_replay_config_init": (None, [ctypes.POINTER(ReplayConfig)]),
    "gbr_replay_create": (_ST, [ctypes.POINTER(ReplayConfig), ctypes.POINTER(_P)]),
    "gbr_replay_destroy": (None, [_P]),
    "gbr_replay_close": (_ST, [_P]),
    "gbr_replay_renderer": (_ST, [_P, ctypes.POINTER(_P)]),
    "gbr_replay_environment_grid_size": (_ST, [_I32, ctypes.POINTER(_I32)]),
    "gbr_replay_preload_file": (_ST, [_P, ctypes.c_char_p]),
    "gbr_replay_environment_count": (_ST, [_P, ctypes.POINTER(_U32)]),
    "gbr_replay_sensor_size": (_ST, [_P, _U32, ctypes.POINTER(_I32)]),
    "gbr_replay_clear_environment": (_ST, [_P, _U32]),
    "gbr_replay_set_environment_keyframe": (_ST, [_P, _U32, ctypes.c_char_p, _U64]),
    "gbr_replay_set_environment_keyframe_unwrapped": (_ST, [_P, _U32, ctypes.c_char_p, _U64]),
    "gbr_replay_set_keyframes": (_ST, [_P, _U32, ctypes.c_char_p, _U64]),
    "gbr_replay_set_environment_keyframes": (_ST, [_P, _U32, _U32, ctypes.POINTER(ctypes.c_char_p),
                                                  ctypes.POINTER(_U64), ctypes.c_char_p]),
    "gbr_replay_set_keyframe_index": (_ST, [_P, _U32, _I32]),
    "gbr_replay_keyframe_count": (_ST, [_P, _U32, ctypes.POINTER(_I32), ctypes.POINTER(_I32)]),
    "gbr_replay_user_transform": (_ST, [_P, _U32, ctypes.c_char_p, c_float_p, c_float_p,
                                        ctypes.POINTER(_I32)]),
    "gbr_replay_set_sensor_transform": (_ST, [_P, _U32, ctypes.c_char_p, c_float_p]),
    "gbr_replay_set_sensor_transforms_from_keyframe": (_ST, [_P, _U32, ctypes.c_char_p]),
    "gbr_replay_render": (_ST, [_P, _P, _U32, ctypes.POINTER(_P), _U64, _U32, ctypes.POINTER(_P),
                                _U64]),
    "gbr_replay_unproject": (_ST, [_P, _U32, _I32, _I32, c_float_p, c_float_p]),
    # include/gbr_noise.h
    "gbr_redwood_noise_create": (_ST, [c_float_p, _I32, _I32, _I32, ctypes.c_float, _U64,
                                       ctypes.POINTER(_P)]),
    "gbr_redwood_noise_destroy": (None, [_P]),
    "gbr_redwood_noise_simulate_device": (_ST, [_P, _P, _I32, _I32, _P, _P]),
    "gbr_redwood_noise_simulate_host": (_ST, [_P, c_float_p, _I32, _I32, c_float_p]),
    "gbr_redwood_noise_simulate_tiles": (_ST, [_P, _P, _P, ctypes.c_int64, _I32, _I32, _I32, _I32,
                                               _P]),
    "gbr_redwood_noise_simulate_images": (_ST, [_P, _P, _P, ctypes.POINTER(ctypes.c_int64), _I32, _P]),
    "gbr_redwood_noise_set_state": (_ST, [_P, _U64, _U64]),
    "gbr_redwood_noise_get_state": (_ST, [_P, ctypes.POINTER(_U64), ctypes.POINTER(_U64)]),
    "gbr_normal_quantile_table": (_ST, [c_float_p, _U32]),
    # include/gbr_hbao.h
    "gbr_hbao_config_init": (None, [ctypes.POINTER(HbaoConfig)]),
    "gbr_hbao_draw": (_ST, [_P, ctypes.POINTER(HbaoConfig), _P]),
    "gbr_hbao_apply": (_ST, [ctypes.POINTER(HbaoConfig), c_float_p, _P, _P, _I32, _I32,
                             ctypes.c_int64, _P]),
    "gbr_hbao_jitter_table": (_ST, [c_float_p]),
}

_lib = None


def library_path():
    return _build.LIB


def load():
    """Load libgbr.so (compiling it first if its sources changed)."""
    global _lib
    if _lib is None:
        path = _build.build()
        lib = ctypes.CDLL(path)
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


class GbrError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"[gbr status {status}] {message}")
        self.status = status


def check(status):
    if status != 0:
        raise GbrError(status, load().gbr_last_error().decode(errors="replace"))
