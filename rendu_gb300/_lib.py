"""ctypes binding of ``librendu_gb300.so`` (the C-ABI declared in include/rendu_gb300.h).

The library is the only compute path: if it is missing or cannot be loaded, every entry
point raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "librendu_gb300.so")

RT_OK = 0
RT_ERR_ARG = 1
RT_ERR_OOM = 2
RT_ERR_CUDA = 3
RT_ERR_TIMEOUT = 4
RT_ERR_STATE = 5
RT_ERR_OVERFLOW = 6
RT_FLAG_DEVICE_PTRS = 0x1
PT_MODE_REFERENCE = 0
PT_MODE_EXTENDED = 1
PT_BG_COLOR = 0
PT_BG_IMAGE = 1
PT_BG_SKYBOX = 2
PT_BG_ATMOSPHERE = 3
RT_NO_HIT = 0xFFFFFFFF
PT_RANK_TILE_PIXELS = 4096

_STATUS_NAMES = {1: "RT_ERR_ARG", 2: "RT_ERR_OOM", 3: "RT_ERR_CUDA", 4: "RT_ERR_TIMEOUT", 5: "RT_ERR_STATE",
                 6: "RT_ERR_OVERFLOW"}


class RenduError(RuntimeError):
    def __init__(self, code: int, func: str, msg: str):
        super().__init__(f"{func}: {_STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class rt_stats(C.Structure):
    _fields_ = [("triangles", C.c_uint64), ("vertices", C.c_uint64), ("meshes", C.c_uint64), ("nodes", C.c_uint64),
                ("leaves", C.c_uint64), ("device_bytes", C.c_uint64), ("build_ms", C.c_float),
                ("sah_cost", C.c_float)]


class pt_mesh_desc(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("normals", C.c_void_p), ("tangents", C.c_void_p),
                ("bitangents", C.c_void_p), ("texcoords", C.c_void_p), ("vertex_count", C.c_size_t),
                ("indices", C.c_void_p), ("index_count", C.c_size_t)]


class pt_material_desc(C.Structure):
    _fields_ = [("type", C.c_int32), ("masked", C.c_int32), ("tex", C.c_uint32 * 3)]


class pt_light_desc(C.Structure):
    _fields_ = [("type", C.c_int32), ("cast_shadows", C.c_int32), ("color", C.c_float * 3),
                ("position", C.c_float * 3), ("direction", C.c_float * 3), ("radius", C.c_float),
                ("inner_angle", C.c_float), ("outer_angle", C.c_float)]


class pt_camera_desc(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("center", C.c_float * 3), ("up", C.c_float * 3), ("fov", C.c_float),
                ("ratio", C.c_float)]


class pt_render_options(C.Structure):
    _fields_ = [("mode", C.c_int32), ("clamp", C.c_float), ("accum_fp64", C.c_int32), ("aov", C.c_void_p),
                ("ranks", C.c_uint32), ("rank", C.c_uint32), ("profile", C.c_int32)]


class pt_batch_job(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("camera", pt_camera_desc), ("samples", C.c_uint32), ("depth", C.c_uint32),
                ("seed", C.c_uint64), ("image", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32),
                ("components", C.c_uint32)]


class pt_batch_tuning(C.Structure):
    _fields_ = [("wave_paths", C.c_uint32), ("tile_pixels", C.c_uint32), ("max_samples", C.c_uint32)]


class pt_render_stats(C.Structure):
    _fields_ = [("primary_rays", C.c_uint64), ("bounce_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("paths", C.c_uint64), ("device_ms", C.c_float), ("kernel_ms", C.c_float * 5)]


class dn_layer(C.Structure):
    _fields_ = [("cin0", C.c_uint32), ("cin1", C.c_uint32), ("cout", C.c_uint32), ("up0", C.c_int32),
                ("relu", C.c_int32), ("level", C.c_int32), ("weight_offset", C.c_uint64), ("bias_offset", C.c_uint64)]


DN_FEATURES = 11

_lib = None
_lock = threading.Lock()

_VP = C.c_void_p
_SIGS = {
    "rt_create": ([C.POINTER(C.c_void_p), C.c_int], C.c_int),
    "rt_destroy": ([_VP], C.c_int),
    "rt_add_mesh": ([_VP, _VP, C.c_size_t, _VP, C.c_size_t, _VP, C.POINTER(C.c_uint32)], C.c_int),
    "rt_update_hierarchy": ([_VP], C.c_int),
    "rt_intersect": ([_VP, _VP, C.c_size_t, _VP, _VP, C.c_uint32], C.c_int),
    "rt_intersect_any": ([_VP, _VP, C.c_size_t, _VP, _VP, C.c_uint32], C.c_int),
    "rt_visible": ([_VP, _VP, C.c_size_t, _VP, _VP, C.c_uint32], C.c_int),
    "rt_prim_info": ([_VP, C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)], C.c_int),
    "rt_hit_info": ([_VP, _VP, C.c_size_t, _VP, _VP, _VP, C.c_uint32], C.c_int),
    "rt_get_status": ([_VP, _VP, C.POINTER(C.c_uint32)], C.c_int),
    "rt_set_traversal_stack": ([_VP, C.c_uint32], C.c_int),
    "rt_get_stats": ([_VP, C.POINTER(rt_stats)], C.c_int),
    "rt_count_visits": ([_VP, _VP, C.c_size_t, _VP, _VP, _VP, C.c_uint32], C.c_int),
    "rt_last_error": ([], C.c_char_p),
    "pt_scene_create": ([C.POINTER(C.c_void_p), C.c_int], C.c_int),
    "pt_scene_destroy": ([_VP], C.c_int),
    "pt_scene_add_texture": ([_VP, C.c_uint32, C.c_uint32, C.c_uint32, _VP, C.POINTER(C.c_uint32)], C.c_int),
    "pt_scene_add_mesh": ([_VP, C.POINTER(pt_mesh_desc), C.POINTER(C.c_uint32)], C.c_int),
    "pt_scene_add_material": ([_VP, C.POINTER(pt_material_desc), C.POINTER(C.c_uint32)], C.c_int),
    "pt_scene_add_object": ([_VP, C.c_uint32, C.c_uint32, _VP, C.POINTER(C.c_uint32)], C.c_int),
    "pt_scene_add_light": ([_VP, C.POINTER(pt_light_desc)], C.c_int),
    "pt_scene_set_background": ([_VP, C.c_int32, _VP, _VP], C.c_int),
    "pt_scene_commit": ([_VP], C.c_int),
    "pt_render": ([_VP, C.POINTER(pt_camera_desc), C.c_uint32, C.c_uint32, C.c_uint64, _VP, C.c_uint32, C.c_uint32,
                   C.c_uint32, _VP, C.c_uint32], C.c_int),
    "pt_get_render_stats": ([_VP, C.POINTER(pt_render_stats)], C.c_int),
    "pt_scene_set_environment": ([_VP, C.c_uint32, C.c_float], C.c_int),
    "pt_render_ex": ([_VP, C.POINTER(pt_camera_desc), C.c_uint32, C.c_uint32, C.c_uint64, _VP, C.c_uint32, C.c_uint32,
                      C.c_uint32, C.POINTER(pt_render_options), _VP, C.c_uint32], C.c_int),
    "rt_visible_noalloc": ([_VP, _VP, C.c_size_t, _VP, _VP], C.c_int),
    "pt_batch_create": ([C.POINTER(C.c_void_p), C.c_int], C.c_int),
    "pt_batch_destroy": ([_VP], C.c_int),
    "pt_batch_render": ([_VP, _VP, C.c_size_t, C.POINTER(pt_render_options), C.POINTER(pt_batch_tuning), _VP,
                         C.c_uint32], C.c_int),
    "pt_batch_autotune": ([_VP, _VP, C.c_size_t, C.POINTER(pt_render_options), C.c_char_p,
                           C.POINTER(pt_batch_tuning)], C.c_int),
    "pt_batch_get_stats": ([_VP, C.POINTER(pt_render_stats)], C.c_int),
    "pt_scene_raycaster": ([_VP], _VP),
    "pt_material_eval": ([_VP, C.c_size_t, _VP, C.c_int], C.c_int),
    "pt_material_sample": ([_VP, _VP, C.c_size_t, _VP, C.c_int], C.c_int),
    "pt_scene_set_sky_table": ([_VP, _VP, C.c_uint32, C.c_uint32], C.c_int),
    "pt_image_save": ([_VP, C.c_uint32, C.c_uint32, C.c_uint32, C.c_char_p, C.c_int32], C.c_int),
    "rt_hierarchy_boxes": ([_VP, _VP, _VP, C.c_size_t, C.POINTER(C.c_size_t)], C.c_int),
    "rt_ray_levels": ([_VP, _VP, _VP, _VP, C.c_size_t, C.POINTER(C.c_size_t), _VP], C.c_int),
    "pt_png_unfilter": ([_VP, C.c_uint32, C.c_uint32, C.c_uint32, _VP], C.c_int),
    "pt_jpeg_decode": ([_VP, C.c_size_t, C.c_uint32, _VP, C.c_size_t, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)],
                       C.c_int),
    "pt_sky_table": ([C.c_uint32, C.c_uint32, C.c_int32, _VP, C.c_int], C.c_int),
    "pt_sky_eval": ([_VP, C.c_uint32, C.c_uint32, _VP, C.c_size_t, _VP, C.c_int], C.c_int),
    "dn_create": ([C.POINTER(C.c_void_p), C.c_int], C.c_int),
    "dn_destroy": ([_VP], C.c_int),
    "dn_init": ([_VP, C.c_uint64], C.c_int),
    "dn_layer_count": ([_VP, C.POINTER(C.c_uint32)], C.c_int),
    "dn_layer_info": ([_VP, C.c_uint32, C.POINTER(dn_layer)], C.c_int),
    "dn_param_count": ([_VP, C.POINTER(C.c_size_t)], C.c_int),
    "dn_get_params": ([_VP, _VP, C.c_size_t], C.c_int),
    "dn_set_params": ([_VP, _VP, C.c_size_t], C.c_int),
    "dn_get_grads": ([_VP, _VP, C.c_size_t], C.c_int),
    "dn_read_grads": ([_VP, _VP, C.c_size_t, _VP, C.c_uint32], C.c_int),
    "dn_write_grads": ([_VP, _VP, C.c_size_t, _VP, C.c_uint32], C.c_int),
    "dn_denoise": ([_VP, _VP, C.c_uint32, C.c_uint32, C.c_uint32, _VP, _VP, C.c_uint32], C.c_int),
    "dn_backward": ([_VP, _VP, _VP, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(C.c_float), _VP, C.c_uint32],
                    C.c_int),
    "dn_adam_step": ([_VP, C.c_float, _VP], C.c_int),
    "dn_train_step": ([_VP, _VP, _VP, C.c_uint32, C.c_uint32, C.c_uint32, C.c_float, C.POINTER(C.c_float), _VP,
                       C.c_uint32], C.c_int),
    "dn_conv3x3": ([_VP, C.c_uint32, C.c_int32, _VP, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, _VP, _VP,
                    C.c_uint32, C.c_int32, _VP, C.c_int32, _VP], C.c_int),
    "dn_conv3x3_backward": ([_VP, C.c_uint32, C.c_int32, _VP, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, _VP,
                             C.c_uint32, _VP, _VP, _VP, _VP], C.c_int),
}


def lib():
    """Load the library once; raise if it is absent (build it with rendu_gb300.build.build())."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(f"{LIB_PATH} is missing: the CUDA library must be built (rendu_gb300.build)")
            h = C.CDLL(LIB_PATH)
            for name, (args, res) in _SIGS.items():
                f = getattr(h, name)
                f.argtypes = args
                f.restype = res
            _lib = h
    return _lib


def check(code: int, func: str):
    if code != RT_OK:
        msg = lib().rt_last_error()
        raise RenduError(code, func, msg.decode() if msg else "")


def call(func: str, *args):
    check(getattr(lib(), func)(*args), func)
