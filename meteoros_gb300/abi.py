"""ctypes mirror of include/meteoros.h and the loader of the in-tree library.

The structures here are byte-for-byte the C structures of the header; the
layout asserts at the bottom fail loudly if the two ever drift apart.  The
library is the in-tree ``meteoros_gb300/_build/libmeteoros_gb300.so`` built by
``meteoros_gb300.build``; there is no fallback implementation: when the
library is missing, :func:`load_library` raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "_build" / "libmeteoros_gb300.so"

MT_BASE_N = 128
MT_DETAIL_N = 32
MT_CURL_N = 128
MT_WEATHER_N = 512
MT_MAX_WEATHER_SLOTS = 256
MT_MAX_DIM = 16384
MT_NOALLOC_MAX_VIEWS = 64
MT_LDR_RGBA8 = 0
MT_VOLUME_BASE = 0
MT_VOLUME_DETAIL = 1
MT_TGA_MAX_SLICE_BYTES = 200000
MT_LDR_RGBA32F = 1
MT_NOALLOC_MAX_TILES = 32768

MT_OK = 0
MT_ERR_INVALID_ARG = 1
MT_ERR_NO_VOLUMES = 2
MT_ERR_CUDA = 3
MT_ERR_OUT_OF_MEMORY = 4
MT_ERR_UNSUPPORTED = 5
MT_ERR_BUDGET = 6
MT_ERR_TIMEOUT = 7

MT_STORAGE_U8 = 0
MT_STORAGE_F16 = 1
MT_STORAGE_BF16 = 2

MT_RENDER_CHECKERBOARD = 0
MT_RENDER_FULL = 1
MT_RENDER_COUNT = 2


class CameraUBO(C.Structure):
    """CameraUBO (camera.h:12-18): view, proj (column-major), eye, tanFovBy2."""

    _fields_ = [
        ("view", C.c_float * 16),
        ("proj", C.c_float * 16),
        ("eye", C.c_float * 4),
        ("tan_fov_by_2", C.c_float * 2),
        ("_pad", C.c_float * 2),
    ]


class TimeUBO(C.Structure):
    """TimeUBO (Scene.h:12-21): 16 Halton values, (dt, t), frame index mod 16."""

    _fields_ = [
        ("halton_seq1", C.c_float * 4),
        ("halton_seq2", C.c_float * 4),
        ("halton_seq3", C.c_float * 4),
        ("halton_seq4", C.c_float * 4),
        ("time", C.c_float * 2),
        ("frame_count_mod16", C.c_int32),
        ("_pad", C.c_int32),
    ]


class Params(C.Structure):
    _fields_ = [
        ("earth_radius", C.c_float),
        ("shell_inner_radius", C.c_float),
        ("shell_outer_radius", C.c_float),
        ("noise_period", C.c_float),
        ("steps_min", C.c_int32),
        ("steps_max", C.c_int32),
        ("accum_limit", C.c_float),
        ("coverage_mode", C.c_int32),
        ("coverage", C.c_float),
        ("height_gradient", C.c_int32),
        ("weather_scale", C.c_float),
        ("weather_slot", C.c_int32),
        ("wind_dir", C.c_float * 3),
        ("wind_speed", C.c_float),
        ("skew_dir", C.c_float * 3),
        ("cloud_top_offset", C.c_float),
        ("sun_light_pos", C.c_float * 3),
        ("sky_sun_pos", C.c_float * 3),
        ("eye_sign", C.c_float),
        ("feedback_min", C.c_float),
        ("feedback_max", C.c_float),
        ("slot_x", C.c_int32 * 16),
        ("slot_y", C.c_int32 * 16),
        ("storage", C.c_int32),
        ("fp64_shells", C.c_int32),
        ("_reserved", C.c_int32 * 7),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("primary_samples", C.c_uint64),
        ("light_samples", C.c_uint64),
        ("marched_rays", C.c_uint64),
        ("pixels", C.c_uint64),
    ]


class Tuning(C.Structure):
    _fields_ = [("march_lanes", C.c_int32), ("fused_resolve", C.c_int32), ("batch_tile_w", C.c_int32),
                ("batch_tile_h", C.c_int32), ("batch_lanes", C.c_int32), ("batch_direct", C.c_int32),
                ("reproject_serial", C.c_int32), ("march_block", C.c_int32),
                ("march_order", C.c_int32), ("batch_order", C.c_int32), ("_reserved", C.c_int32 * 2)]


class KernelTimes(C.Structure):
    _fields_ = [("reproject_ms", C.c_float), ("march_ms", C.c_float), ("txaa_ms", C.c_float),
                ("resolve_ms", C.c_float)]


class View(C.Structure):
    _fields_ = [
        ("camera", CameraUBO),
        ("camera_old", CameraUBO),
        ("time", TimeUBO),
        ("params", Params),
        ("prev_rgba", C.c_void_p),
        ("cur_rgba", C.c_void_p),
        ("godray_mask", C.c_void_p),
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("flags", C.c_uint32),
        ("_pad", C.c_int32),
    ]


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("max_batch", C.c_int32), ("streams", C.c_int32),
                ("batch_lanes", C.c_int32), ("per_request", C.c_int32), ("use_graph", C.c_int32),
                ("admission_wait_ms", C.c_int32)]


class RequestInfo(C.Structure):
    _fields_ = [("id", C.c_uint64), ("session", C.c_int64), ("submit_s", C.c_double), ("start_s", C.c_double),
                ("done_s", C.c_double), ("batch_size", C.c_int32), ("status", C.c_int32)]


assert C.sizeof(CameraUBO) == 160
assert C.sizeof(TimeUBO) == 80
assert C.sizeof(Params) == 280, C.sizeof(Params)

# Every function the header declares, with its ctypes signature.
_P = C.c_void_p
SIGNATURES = {
    "mt_abi_version": (C.c_int, []),
    "mt_create": (C.c_int, [C.POINTER(_P), C.c_int]),
    "mt_destroy": (None, [_P]),
    "mt_last_error": (C.c_char_p, [_P]),
    "mt_params_reference": (None, [C.POINTER(Params)]),
    "mt_params_config": (None, [C.POINTER(Params)]),
    "mt_time_init": (None, [C.POINTER(TimeUBO)]),
    "mt_time_advance": (None, [C.POINTER(TimeUBO), C.c_float]),
    "mt_camera_look_at": (None, [C.POINTER(CameraUBO), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                 C.c_float, C.c_float, C.c_float, C.c_float]),
    "mt_halton": (C.c_float, [C.c_int, C.c_int]),
    "mt_upload_volumes": (C.c_int, [_P, _P, _P, _P, _P]),
    "mt_upload_weather": (C.c_int, [_P, C.c_int, _P]),
    "mt_generate_volumes": (C.c_int, [_P, C.c_uint64, _P]),
    "mt_generate_weather": (C.c_int, [_P, C.c_int, C.c_uint64, _P]),
    "mt_download_volumes": (C.c_int, [_P, _P, _P, _P, _P, C.c_int]),
    "mt_download_volumes_16": (C.c_int, [_P, C.c_int, _P, _P, _P, _P, C.c_int]),
    "mt_render": (C.c_int, [_P, C.POINTER(CameraUBO), C.POINTER(CameraUBO), C.POINTER(TimeUBO),
                            C.POINTER(Params), _P, _P, _P, C.c_int, C.c_int, C.c_uint32, _P]),
    "mt_render_frame": (C.c_int, [_P, C.POINTER(CameraUBO), C.POINTER(CameraUBO), C.POINTER(TimeUBO),
                                  C.POINTER(Params), _P, _P, _P, _P, _P, C.c_int, C.c_int, C.c_uint32, _P]),
    "mt_txaa": (C.c_int, [_P, C.POINTER(CameraUBO), C.POINTER(CameraUBO), C.POINTER(TimeUBO),
                          C.POINTER(Params), _P, _P, _P, C.c_int, C.c_int, _P]),
    "mt_render_batch": (C.c_int, [_P, C.POINTER(View), C.c_int, _P]),
    "mt_set_sample_trace": (C.c_int, [_P, _P]),
    "mt_get_stats": (C.c_int, [_P, C.POINTER(Stats), C.c_int, _P]),
    "mt_autotune_batch": (C.c_int, [_P, C.POINTER(View), C.c_int, _P, C.POINTER(Tuning)]),
    "mt_render_batch_noalloc": (C.c_int, [_P, C.POINTER(View), C.c_int, _P]),
    "mt_decode_tga_volume": (C.c_int, [_P, C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_size_t), C.c_int, _P]),
    "mt_godrays": (C.c_int, [_P, C.POINTER(CameraUBO), C.POINTER(C.c_float), _P, _P, _P, C.c_int, C.c_int, _P]),
    "mt_tonemap": (C.c_int, [_P, C.POINTER(TimeUBO), _P, _P, C.c_int, C.c_int, C.c_int, _P]),
    "mt_server_clock": (C.c_double, []),
    "mt_server_create": (C.c_int, [_P, C.POINTER(ServerConfig), C.POINTER(_P)]),
    "mt_server_destroy": (None, [_P]),
    "mt_server_last_error": (C.c_char_p, [_P]),
    "mt_server_open_session": (C.c_int, [_P, C.c_int, C.c_int, C.POINTER(Params), C.POINTER(C.c_int64)]),
    "mt_server_close_session": (C.c_int, [_P, C.c_int64]),
    "mt_server_submit": (C.c_int, [_P, C.c_int64, C.POINTER(CameraUBO), C.POINTER(TimeUBO),
                                   C.POINTER(C.c_uint64)]),
    "mt_server_wait": (C.c_int, [_P, C.c_uint64, C.c_int, C.POINTER(RequestInfo)]),
    "mt_server_read_frame": (C.c_int, [_P, C.c_int64, _P, _P]),
    "mt_server_memory": (C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "mt_set_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
    "mt_get_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
    "mt_selftest_division": (C.c_int, [_P, _P, _P, _P, _P, C.c_int, _P]),
    "mt_set_timing": (C.c_int, [_P, C.c_int]),
    "mt_get_kernel_times": (C.c_int, [_P, C.POINTER(KernelTimes)]),
}

_lib = None


def load_library(path: os.PathLike | str | None = None) -> C.CDLL:
    """Load the in-tree C-ABI library (no fallback: raises if it is missing)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"meteoros_gb300: CUDA library {p} is missing; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class MeteorosError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[mt_status {status}] {message}")
        self.status = status


def params_reference() -> Params:
    p = Params()
    load_library().mt_params_reference(C.byref(p))
    return p


def params_config() -> Params:
    p = Params()
    load_library().mt_params_config(C.byref(p))
    return p


def time_init() -> TimeUBO:
    t = TimeUBO()
    load_library().mt_time_init(C.byref(t))
    return t


def time_advance(t: TimeUBO, dt: float) -> TimeUBO:
    load_library().mt_time_advance(C.byref(t), C.c_float(dt))
    return t


def camera_look_at(eye, ref, fovy_deg: float, aspect: float, near: float = 0.1,
                   far: float = 1000.0) -> CameraUBO:
    cam = CameraUBO()
    e = (C.c_float * 3)(*eye)
    r = (C.c_float * 3)(*ref)
    load_library().mt_camera_look_at(C.byref(cam), e, r, fovy_deg, aspect, near, far)
    return cam
