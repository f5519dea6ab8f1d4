"""TEST INFRASTRUCTURE — ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, and only as the checker (bench.py also times it as the CPU
baseline).  The product path never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

from meteoros_gb300 import abi

ORACLE_DIR = Path(__file__).resolve().parent
BUILD_DIR = ORACLE_DIR / "_build"
LIB = BUILD_DIR / "liboracle.so"
SOURCES = [ORACLE_DIR / "meteoros_oracle.cpp", ORACLE_DIR / "noise_oracle.cpp", ORACLE_DIR / "post_oracle.cpp",
           ORACLE_DIR / "asset_oracle.cpp", ORACLE_DIR / "uniform_oracle.cpp"]
HEADERS = [ORACLE_DIR / "oracle_math.hpp", ORACLE_DIR.parent / "include" / "meteoros.h"]

CXXFLAGS = ["-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c++17"]


def build(force: bool = False) -> Path:
    """Compile the oracle with g++ (no FMA contraction, OpenMP over pixels)."""
    BUILD_DIR.mkdir(exist_ok=True)
    newest = max(p.stat().st_mtime for p in SOURCES + HEADERS)
    if force or not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = LIB.with_suffix(f".so.{os.getpid()}")
        cmd = ["g++", *CXXFLAGS, *map(str, SOURCES), "-o", str(tmp)]
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    return LIB


class OrcVolumes(C.Structure):
    _fields_ = [("base", C.c_void_p), ("detail", C.c_void_p), ("curl", C.c_void_p),
                ("weather", C.c_void_p), ("fmt", C.c_int32), ("_pad", C.c_int32)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P = C.c_void_p
        cam = C.POINTER(abi.CameraUBO)
        tm = C.POINTER(abi.TimeUBO)
        par = C.POINTER(abi.Params)
        for name in ("orc_render_f32", "orc_render_f64"):
            f = getattr(L, name)
            f.restype = C.c_int
            f.argtypes = [C.POINTER(OrcVolumes), cam, cam, tm, par, P, P, P, C.c_int, C.c_int,
                          C.c_uint, C.c_int, P]
        for name in ("orc_txaa_f32", "orc_txaa_f64"):
            f = getattr(L, name)
            f.restype = C.c_int
            f.argtypes = [cam, cam, tm, par, P, P, P, C.c_int, C.c_int, C.c_int]
        for name in ("orc_march_pixels_f32", "orc_march_pixels_f64"):
            f = getattr(L, name)
            f.restype = C.c_int
            f.argtypes = [C.POINTER(OrcVolumes), cam, tm, par, C.c_int, C.c_int, P, C.c_longlong, P, P, P, C.c_int]
        L.orc_godrays_f32.restype = C.c_int
        L.orc_godrays_f32.argtypes = [cam, P, P, P, P, C.c_int, C.c_int]
        L.orc_tonemap_f32.restype = C.c_int
        L.orc_tonemap_f32.argtypes = [C.c_float, P, P, P, C.c_int, C.c_int]
        L.orc_decode_tga.restype = C.c_int
        L.orc_decode_tga.argtypes = [P, C.c_size_t, C.POINTER(C.c_int), C.POINTER(C.c_int), P]
        L.orc_wang_hash_noise.restype = C.c_float
        L.orc_wang_hash_noise.argtypes = [C.c_uint32] * 3
        L.orc_generate_volumes.restype = None
        L.orc_generate_volumes.argtypes = [C.c_uint64] + [P] * 12
        L.orc_wang.restype = C.c_uint32
        L.orc_wang.argtypes = [C.c_uint32] * 3
        L.orc_f2h.restype = C.c_uint16
        L.orc_f2h.argtypes = [C.c_float]
        L.orc_f2bf.restype = C.c_uint16
        L.orc_f2bf.argtypes = [C.c_float]
        L.orc_hg.restype = C.c_float
        L.orc_hg.argtypes = [C.c_float, C.c_float]
        L.orc_light_energy.restype = C.c_float
        L.orc_light_energy.argtypes = [C.c_float] * 7
        L.orc_godray_value.restype = C.c_float
        L.orc_godray_value.argtypes = [C.c_float, C.c_float]
        L.orc_ray_sphere.restype = C.c_int
        L.orc_ray_sphere.argtypes = [P, P, P, C.c_float, P]
        L.orc_tex3.restype = None
        L.orc_tex3.argtypes = [P, C.c_int, C.c_int, P, P]
        for name, n in (("orc_height_gradient", 2), ("orc_remap", 5), ("orc_remap_clamped", 5),
                        ("orc_remap_clamped_ba", 5)):
            getattr(L, name).restype = C.c_float
            getattr(L, name).argtypes = [C.c_float] * n
        L.orc_halton.restype = C.c_float
        L.orc_halton.argtypes = [C.c_int, C.c_int]
        L.orc_time_init.restype = None
        L.orc_time_init.argtypes = [tm]
        L.orc_camera_look_at.restype = None
        L.orc_camera_look_at.argtypes = [cam, C.POINTER(C.c_float), C.POINTER(C.c_float)] + [C.c_float] * 4
        L.orc_params_reference.restype = None
        L.orc_params_reference.argtypes = [par]
        L.orc_params_config.restype = None
        L.orc_params_config.argtypes = [par]
        _lib = L
    return _lib


# ---------------------------------------------------------------------------
# Uniform producers and presets, restated (uniform_oracle.cpp).  Same names and
# signatures as meteoros_gb300.abi's, so scene builders can take either.
# ---------------------------------------------------------------------------
def halton(index: int, base: int) -> float:
    return lib().orc_halton(index, base)


def time_init() -> abi.TimeUBO:
    t = abi.TimeUBO()
    lib().orc_time_init(C.byref(t))
    return t


def camera_look_at(eye, ref, fovy_deg: float, aspect: float, near: float = 0.1,
                   far: float = 1000.0) -> abi.CameraUBO:
    cam = abi.CameraUBO()
    lib().orc_camera_look_at(C.byref(cam), (C.c_float * 3)(*eye), (C.c_float * 3)(*ref), fovy_deg, aspect, near,
                             far)
    return cam


def params_reference() -> abi.Params:
    p = abi.Params()
    lib().orc_params_reference(C.byref(p))
    return p


def params_config() -> abi.Params:
    p = abi.Params()
    lib().orc_params_config(C.byref(p))
    return p


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Volumes:
    """Noise volumes in host memory: uint8 RGBA (fmt 0) or float texel values (fmt 1)."""

    def __init__(self, base, detail, curl, weather):
        arrs = [np.ascontiguousarray(a) for a in (base, detail, curl, weather)]
        self.base, self.detail, self.curl, self.weather = arrs
        self.fmt = 0 if self.base.dtype == np.uint8 else 1
        if self.fmt == 1:
            self.base, self.detail, self.curl, self.weather = [
                np.ascontiguousarray(a, dtype=np.float32) for a in arrs]

    def c(self) -> OrcVolumes:
        return OrcVolumes(_ptr(self.base), _ptr(self.detail), _ptr(self.curl), _ptr(self.weather),
                          self.fmt, 0)


def generate_volumes(seed: int) -> dict:
    """All generator outputs: u8, f16 (uint16 bits) and bf16 (uint16 bits)."""
    N, D, Cn, Wn = abi.MT_BASE_N, abi.MT_DETAIL_N, abi.MT_CURL_N, abi.MT_WEATHER_N
    shapes = {"base": (N, N, N, 4), "detail": (D, D, D, 4), "curl": (Cn, Cn, 4), "weather": (Wn, Wn, 4)}
    out = {}
    for k, s in shapes.items():
        out[k] = np.zeros(s, np.uint8)
        out[k + "_h16"] = np.zeros(s, np.uint16)
        out[k + "_b16"] = np.zeros(s, np.uint16)
    lib().orc_generate_volumes(
        C.c_uint64(seed & 0xFFFFFFFFFFFFFFFF),
        *[_ptr(out[k]) for k in ("base", "detail", "curl", "weather")],
        *[_ptr(out[k + "_h16"]) for k in ("base", "detail", "curl", "weather")],
        *[_ptr(out[k + "_b16"]) for k in ("base", "detail", "curl", "weather")])
    return out


def half_bits_to_float(bits: np.ndarray) -> np.ndarray:
    return bits.view(np.float16).astype(np.float32)


def bf16_bits_to_float(bits: np.ndarray) -> np.ndarray:
    return (bits.astype(np.uint32) << 16).view(np.float32)


def render(vol: Volumes, cam, cam_old, tm, params, prev, width: int, height: int, flags: int,
           dtype=np.float32, nthreads: int = 0):
    """CPU render of one frame.  Returns (rgba[H,W,4], mask[H,W], counters[4]).

    The mask holds NaN where the frame did not write it."""
    cur = np.zeros((height, width, 4), dtype)
    mask = np.full((height, width), np.nan, dtype)
    if prev is not None:
        prev = np.ascontiguousarray(prev, dtype=dtype)
    counters = np.zeros(4, np.uint64)
    fn = lib().orc_render_f32 if dtype == np.float32 else lib().orc_render_f64
    v = vol.c()
    rc = fn(C.byref(v), C.byref(cam), C.byref(cam_old), C.byref(tm), C.byref(params), _ptr(prev),
            _ptr(cur), _ptr(mask), width, height, flags, nthreads, _ptr(counters))
    if rc != 0:
        raise RuntimeError(f"orc_render failed ({rc})")
    return cur, mask, counters


def march_pixels(vol: Volumes, cam, tm, params, width: int, height: int, xy: np.ndarray, dtype=np.float64,
                 nthreads: int = 0, counts: bool = False):
    """Full-raymarch colour and god-ray value of the listed pixels (xy: n x 2
    int32); with counts=True also each ray's trace as an (n, 4) uint32 array:
    primary samples, in-cloud samples, control-flow signature, 0."""
    xy = np.ascontiguousarray(xy, np.int32)
    n = xy.shape[0]
    rgba = np.zeros((n, 4), dtype)
    mask = np.zeros(n, dtype)
    cnt = np.zeros((n, 4), np.uint32) if counts else None
    fn = lib().orc_march_pixels_f32 if dtype == np.float32 else lib().orc_march_pixels_f64
    v = vol.c()
    rc = fn(C.byref(v), C.byref(cam), C.byref(tm), C.byref(params), width, height, _ptr(xy), n, _ptr(rgba),
            _ptr(mask), _ptr(cnt), nthreads)
    if rc != 0:
        raise RuntimeError(f"orc_march_pixels failed ({rc})")
    return (rgba, mask, cnt) if counts else (rgba, mask)


def volumes_16(vols: dict, storage: str) -> Volumes:
    """The texel values of the half ('h16') or bfloat16 ('b16') copies, as float32 (exact)."""
    conv = half_bits_to_float if storage == "h16" else bf16_bits_to_float
    return Volumes(*(conv(vols[k + "_" + storage]) for k in ("base", "detail", "curl", "weather")))


def txaa(cam, cam_old, tm, params, current, history, dtype=np.float32, nthreads: int = 0):
    current = np.ascontiguousarray(current, dtype=dtype)
    history = np.ascontiguousarray(history, dtype=dtype)
    h, w = current.shape[:2]
    out = np.zeros_like(current)
    fn = lib().orc_txaa_f32 if dtype == np.float32 else lib().orc_txaa_f64
    rc = fn(C.byref(cam), C.byref(cam_old), C.byref(tm), C.byref(params), _ptr(current), _ptr(history),
            _ptr(out), w, h, nthreads)
    if rc != 0:
        raise RuntimeError(f"orc_txaa failed ({rc})")
    return out


def godrays(cam, light_color, mask, rgba):
    """God-ray radial blur added to (H, W, 4) `rgba` (restatement, FP32)."""
    rgba = np.ascontiguousarray(rgba, np.float32)
    mask = np.ascontiguousarray(mask, np.float32)
    h, w = rgba.shape[:2]
    out = np.empty_like(rgba)
    light = np.ascontiguousarray(light_color, np.float32)
    if lib().orc_godrays_f32(C.byref(cam), _ptr(light), _ptr(mask), _ptr(rgba), _ptr(out), w, h) != 0:
        raise RuntimeError("orc_godrays_f32 failed")
    return out


def tonemap(time_y: float, rgba, fill4=np.nan, fill8=0):
    """Tone map + dither.  Returns (float RGBA (H, W, 4), RGBA8 (H, W, 4) uint8);
    pixels no fragment stores to keep the fill values."""
    rgba = np.ascontiguousarray(rgba, np.float32)
    h, w = rgba.shape[:2]
    out4 = np.full((h, w, 4), fill4, np.float32)
    out8 = np.full((h, w, 4), fill8, np.uint8)
    if lib().orc_tonemap_f32(C.c_float(time_y), _ptr(rgba), _ptr(out4), _ptr(out8), w, h) != 0:
        raise RuntimeError("orc_tonemap_f32 failed")
    return out4, out8


def decode_tga(data: bytes) -> np.ndarray:
    """TGA file bytes -> (H, W, 4) uint8 RGBA, top row first (restatement)."""
    buf = np.frombuffer(data, np.uint8)
    w, h = C.c_int(), C.c_int()
    if lib().orc_decode_tga(_ptr(buf), len(data), C.byref(w), C.byref(h), None) != 0:
        raise ValueError("TGA outside the accepted subset")
    out = np.zeros((h.value, w.value, 4), np.uint8)
    lib().orc_decode_tga(_ptr(buf), len(data), C.byref(w), C.byref(h), _ptr(out))
    return out
