"""ctypes binding of libatx.so (include/atx.h).

The library must have been built (``python -m ataraxia_gb300.build``); there
is no fallback: loading fails with an error that says so.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libatx.so"

# Same layout as atx_sphere / atx_material / atx_light (and the reference's
# Sphere 20 B, Material 52 B, Light 28 B).
SPHERE_DTYPE = np.dtype([("center", "<f4", (3,)), ("radius", "<f4"), ("material", "<i4")])
MATERIAL_DTYPE = np.dtype([
    ("albedo", "<f4", (3,)), ("roughness", "<f4"), ("metallic", "<f4"), ("f0", "<f4", (3,)),
    ("emission_color", "<f4", (3,)), ("emission_intensity", "<f4"), ("id", "<i4"),
])
LIGHT_DTYPE = np.dtype([("position", "<f4", (3,)), ("color", "<f4", (3,)), ("intensity", "<f4")])
assert SPHERE_DTYPE.itemsize == 20 and MATERIAL_DTYPE.itemsize == 52 and LIGHT_DTYPE.itemsize == 28

STATUS = {
    0: "ATX_OK", 1: "ATX_ERR_INVALID_ARG", 2: "ATX_ERR_OUT_OF_MEMORY", 3: "ATX_ERR_CUDA",
    4: "ATX_ERR_TIMEOUT", 5: "ATX_ERR_BUSY", 6: "ATX_ERR_NOT_FOUND", 7: "ATX_ERR_CANCELLED",
    8: "ATX_ERR_NO_DEVICE", 9: "ATX_ERR_PARSE",
}


class AtxError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status
        self.message = message


class Settings(C.Structure):
    _fields_ = [("accumulation", C.c_uint8), ("sky_light", C.c_uint8), ("reserved", C.c_uint8 * 2),
                ("max_bounces", C.c_int32)]


class CameraDesc(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("direction", C.c_float * 3), ("fov_deg", C.c_float),
                ("near_clip", C.c_float), ("far_clip", C.c_float)]


class CameraInput(C.Structure):
    _fields_ = [("mouse", C.c_float * 2), ("right_button", C.c_uint8), ("key_w", C.c_uint8), ("key_s", C.c_uint8),
                ("key_a", C.c_uint8), ("key_d", C.c_uint8), ("key_q", C.c_uint8), ("key_e", C.c_uint8),
                ("reserved", C.c_uint8)]


IMAGE_PPM, IMAGE_PAM, IMAGE_PFM = 1, 2, 3


class SceneInfo(C.Structure):
    _fields_ = [("n_spheres", C.c_uint32), ("n_materials", C.c_uint32), ("n_lights", C.c_uint32),
                ("n_nodes", C.c_uint32), ("camera", CameraDesc), ("settings", Settings)]


class Config(C.Structure):
    _fields_ = [("device", C.c_int32), ("wave_paths", C.c_uint32), ("threads", C.c_uint32),
                ("bvh_threshold", C.c_uint32), ("bvh_leaf_size", C.c_uint32), ("flags", C.c_uint32),
                ("hbm_budget_bytes", C.c_uint64)]


class Stats(C.Structure):
    _fields_ = [("frames", C.c_uint64), ("paths", C.c_uint64), ("extension_rays", C.c_uint64),
                ("shadow_rays", C.c_uint64), ("kernel_launches", C.c_uint64), ("device_bytes", C.c_uint64),
                ("last_render_ms", C.c_double), ("bvh_in_use", C.c_uint32), ("reserved", C.c_uint32),
                ("shaded_first", C.c_uint64)]


class Tuning(C.Structure):
    _fields_ = [("bvh_leaf_size", C.c_uint32), ("lanes", C.c_uint32), ("wave_paths", C.c_uint32),
                ("threads", C.c_uint32), ("wave_spp", C.c_uint32), ("path_kernel", C.c_uint32),
                ("from_cache", C.c_uint32), ("cell_res", C.c_uint32), ("ms", C.c_double)]


class KernelTimes(C.Structure):
    _fields_ = [("extend_ms", C.c_double), ("shadow_ms", C.c_double), ("accumulate_ms", C.c_double),
                ("other_ms", C.c_double), ("extend_launches", C.c_uint64), ("shadow_launches", C.c_uint64),
                ("accumulate_launches", C.c_uint64), ("other_launches", C.c_uint64)]


class BatchScene(C.Structure):
    _fields_ = [("spheres", C.c_void_p), ("n_spheres", C.c_uint32), ("materials", C.c_void_p),
                ("n_materials", C.c_uint32), ("lights", C.c_void_p), ("n_lights", C.c_uint32),
                ("camera", CameraDesc), ("width", C.c_uint32), ("height", C.c_uint32), ("settings", Settings)]


class BatchStats(C.Structure):
    _fields_ = [("passes", C.c_uint64), ("paths", C.c_uint64), ("extension_rays", C.c_uint64),
                ("shadow_rays", C.c_uint64), ("kernel_launches", C.c_uint64), ("graph_launches", C.c_uint64),
                ("device_bytes", C.c_uint64), ("last_pass_ms", C.c_double), ("scenes", C.c_uint32),
                ("waves_last_pass", C.c_uint32)]


class BatchTuning(C.Structure):
    _fields_ = [("lanes", C.c_uint32), ("lane_wave_paths", C.c_uint32), ("threads", C.c_uint32),
                ("bvh_threshold", C.c_uint32), ("bvh_leaf_size", C.c_uint32), ("primary_cache", C.c_uint32),
                ("reserved", C.c_uint32 * 2)]


class ServerConfig(C.Structure):
    _fields_ = [("base", Config), ("max_active_jobs", C.c_uint32), ("pass_spp", C.c_uint32),
                ("max_pass_paths", C.c_uint64), ("max_pending", C.c_uint32), ("host_fail_pass", C.c_uint32),
                ("policy", C.c_uint32)]


ADMIT_ARRIVAL, ADMIT_SMALLEST = 0, 1


class JobInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("frames_done", C.c_uint32), ("target_spp", C.c_uint32),
                ("width", C.c_uint32), ("height", C.c_uint32), ("reserved", C.c_uint32),
                ("submit_s", C.c_double), ("admit_s", C.c_double), ("done_s", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("admitted", C.c_uint64), ("completed", C.c_uint64),
                ("cancelled", C.c_uint64), ("failed", C.c_uint64), ("rejected", C.c_uint64),
                ("passes", C.c_uint64), ("paths", C.c_uint64), ("busy_s", C.c_double),
                ("device_bytes", C.c_uint64), ("active", C.c_uint32), ("queued", C.c_uint32)]


JOB_STATES = {0: "queued", 1: "active", 2: "done", 3: "cancelled", 4: "failed"}

FLAG_NO_GRAPHS = 1
FLAG_PROFILE_KERNELS = 2
FLAG_HOST_EXECUTOR = 4
FLAG_OVERLAP_RENDERS = 8

assert C.sizeof(Settings) == 8 and C.sizeof(CameraDesc) == 36

_P = C.c_void_p
_F = C.POINTER(C.c_float)
_U32 = C.c_uint32
_U64 = C.c_uint64
_ST = C.c_int

# name -> (restype, argtypes)
SIGNATURES = {
    "atx_abi_version": (C.c_int, []),
    "atx_status_string": (C.c_char_p, [C.c_int]),
    "atx_last_error": (C.c_char_p, []),
    "atx_device_count": (_ST, [C.POINTER(C.c_int32)]),
    "atx_renderer_create": (_ST, [C.POINTER(Config), C.POINTER(_P)]),
    "atx_renderer_destroy": (_ST, [_P]),
    "atx_resize": (_ST, [_P, _U32, _U32]),
    "atx_set_scene": (_ST, [_P, _P, _U32, _P, _U32, _P, _U32]),
    "atx_set_settings": (_ST, [_P, C.POINTER(Settings)]),
    "atx_get_settings": (_ST, [_P, C.POINTER(Settings)]),
    "atx_reset_frame_index": (_ST, [_P]),
    "atx_get_frame_index": (_ST, [_P, C.POINTER(C.c_uint32)]),
    "atx_set_camera": (_ST, [_P, C.POINTER(CameraDesc)]),
    "atx_set_camera_matrices": (_ST, [_P, _P, _P, _P]),
    "atx_render": (_ST, [_P, _U32]),
    "atx_synchronize": (_ST, [_P]),
    "atx_join": (_ST, [_P]),
    "atx_read_image_async": (_ST, [_P, _P, _U64, C.POINTER(_U64)]),
    "atx_wait_read": (_ST, [_P, _U64]),
    "atx_read_accumulation": (_ST, [_P, _P, _U64]),
    "atx_read_image": (_ST, [_P, _P, _U64]),
    "atx_device_buffers": (_ST, [_P, C.POINTER(_P), C.POINTER(_P)]),
    "atx_get_stats": (_ST, [_P, C.POINTER(Stats)]),
    "atx_get_kernel_times": (_ST, [_P, C.POINTER(KernelTimes)]),
    "atx_reset_kernel_times": (_ST, [_P]),
    "atx_get_stream": (_ST, [_P, C.POINTER(_P)]),
    "atx_autotune": (_ST, [_P, _U32, _U32, C.c_int32, C.POINTER(Tuning)]),
    "atx_get_tuning": (_ST, [_P, C.POINTER(Tuning)]),
    "atx_set_tuning": (_ST, [_P, C.POINTER(Tuning)]),
    "atx_host_alloc": (_ST, [_U64, C.POINTER(_P)]),
    "atx_host_free": (_ST, [_P]),
    "atx_camera_matrices": (_ST, [C.POINTER(CameraDesc), _U32, _U32, _P, _P, _P, _P]),
    "atx_batch_create": (_ST, [C.POINTER(Config), C.POINTER(_P)]),
    "atx_batch_destroy": (_ST, [_P]),
    "atx_batch_add_scene": (_ST, [_P, C.POINTER(BatchScene), C.POINTER(C.c_uint32)]),
    "atx_batch_remove_scene": (_ST, [_P, _U32]),
    "atx_batch_set_spp": (_ST, [_P, _U32, _U32]),
    "atx_batch_reset": (_ST, [_P, _U32]),
    "atx_batch_frame_index": (_ST, [_P, _U32, C.POINTER(C.c_uint32)]),
    "atx_batch_run": (_ST, [_P]),
    "atx_batch_synchronize": (_ST, [_P]),
    "atx_batch_read_accumulation": (_ST, [_P, _U32, _P, _U64]),
    "atx_batch_read_image": (_ST, [_P, _U32, _P, _U64]),
    "atx_batch_get_stats": (_ST, [_P, C.POINTER(BatchStats)]),
    "atx_batch_set_tuning": (_ST, [_P, C.POINTER(BatchTuning)]),
    "atx_batch_set_camera": (_ST, [_P, _U32, C.POINTER(CameraDesc)]),
    "atx_batch_autotune": (_ST, [_P, _U32, C.POINTER(BatchTuning)]),
    "atx_batch_get_tuning": (_ST, [_P, C.POINTER(BatchTuning)]),
    "atx_server_create": (_ST, [C.POINTER(ServerConfig), C.POINTER(_P)]),
    "atx_server_destroy": (_ST, [_P]),
    "atx_server_submit": (_ST, [_P, C.POINTER(BatchScene), _U32, C.POINTER(C.c_uint32)]),
    "atx_server_poll": (_ST, [_P, _U32, C.POINTER(JobInfo)]),
    "atx_server_wait": (_ST, [_P, _U32, _U32]),
    "atx_server_read_image": (_ST, [_P, _U32, _P, _U64]),
    "atx_server_read_accumulation": (_ST, [_P, _U32, _P, _U64]),
    "atx_server_cancel": (_ST, [_P, _U32]),
    "atx_server_set_camera": (_ST, [_P, _U32, C.POINTER(CameraDesc)]),
    "atx_server_release": (_ST, [_P, _U32]),
    "atx_server_get_stats": (_ST, [_P, C.POINTER(ServerStats)]),
    "atx_server_now": (_ST, [_P, C.POINTER(C.c_double)]),
    "atx_render_noalloc": (_ST, [_P, _U32, _P, _U32, _P, _U32, _P, _P, _P, _U32, _U32, C.POINTER(Settings), _U32,
                                 _U32, _P, _P, _P]),
    "atx_trace_nearest": (_ST, [_P, _P, _P, _U64, _P, _P]),
    "atx_primary_directions": (_ST, [_P, _P, _U64]),
    "atx_scene_create": (_ST, [C.POINTER(_P)]),
    "atx_scene_destroy": (_ST, [_P]),
    "atx_scene_parse_json": (_ST, [C.c_char_p, _U64, C.POINTER(_P)]),
    "atx_scene_load": (_ST, [C.c_char_p, C.POINTER(_P)]),
    "atx_scene_to_json": (_ST, [_P, _P, _U64, C.POINTER(C.c_uint64)]),
    "atx_scene_save": (_ST, [_P, C.c_char_p]),
    "atx_scene_get_info": (_ST, [_P, C.POINTER(SceneInfo)]),
    "atx_scene_flatten": (_ST, [_P, _P, _U64]),
    "atx_scene_get_materials": (_ST, [_P, _P, _U64]),
    "atx_scene_get_lights": (_ST, [_P, _P, _U64]),
    "atx_scene_add_node": (_ST, [_P, _U32, C.c_char_p, C.POINTER(C.c_uint32)]),
    "atx_scene_set_transform": (_ST, [_P, _U32, _P, _P, _P]),
    "atx_scene_add_spheres": (_ST, [_P, _U32, _P, _U32]),
    "atx_scene_set_materials": (_ST, [_P, _P, _U32]),
    "atx_scene_set_lights": (_ST, [_P, _P, _U32]),
    "atx_scene_set_camera": (_ST, [_P, C.POINTER(CameraDesc)]),
    "atx_scene_set_settings": (_ST, [_P, C.POINTER(Settings)]),
    "atx_set_scene_graph": (_ST, [_P, _P]),
    "atx_camera_on_update": (_ST, [C.POINTER(CameraDesc), _F, C.POINTER(CameraInput), C.c_float,
                                   C.POINTER(C.c_int32)]),
    "atx_update_camera": (_ST, [_P, C.POINTER(CameraDesc), _F, C.POINTER(CameraInput), C.c_float,
                                C.POINTER(C.c_int32)]),
    "atx_write_rgba8": (_ST, [C.c_char_p, _P, _U32, _U32, C.c_int32]),
    "atx_write_pfm": (_ST, [C.c_char_p, _P, _U32, _U32]),
    "atx_save_image": (_ST, [_P, C.c_char_p, C.c_int32]),
}

_lib = None


def lib():
    """Loads libatx.so once and declares every entry point's signature."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is not built; run `python -m ataraxia_gb300.build` "
                               "(there is no CPU fallback)")
        h = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        _lib = h
    return _lib


def check(status: int) -> None:
    if status != 0:
        msg = lib().atx_last_error()
        raise AtxError(status, msg.decode() if msg else "")


def ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "arrays passed to libatx must be C-contiguous"
    return C.c_void_p(a.ctypes.data)
