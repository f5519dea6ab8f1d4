"""TEST INFRASTRUCTURE — ctypes binding of oracle/_ref/libmeteoros_ref.so, the
reference's own shader source compiled as C++ (oracle/ref_build.py).

Available only where the reference tree exists (this is how the oracle
restatement is pinned and how the golden fixtures in tests/golden/ are made);
:func:`available` says whether it is.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from meteoros_gb300 import abi
from oracle import ref_build

_lib = None


def available() -> bool:
    try:
        return ref_build.build() is not None
    except Exception:
        return False


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = ref_build.build()
        if path is None:
            raise RuntimeError("reference tree not present: oracle/_ref cannot be built")
        L = C.CDLL(str(path))
        P = C.c_void_p
        cam = C.POINTER(abi.CameraUBO)
        tm = C.POINTER(abi.TimeUBO)
        L.ref_cloud_raymarch.restype = C.c_int
        L.ref_cloud_raymarch.argtypes = [P, P, P, P, C.c_int, cam, tm, P, P, C.c_int, C.c_int, C.c_int]
        L.ref_reprojection.restype = C.c_int
        L.ref_reprojection.argtypes = [cam, cam, tm, P, P, C.c_int, C.c_int, C.c_int]
        L.ref_txaa.restype = C.c_int
        L.ref_txaa.argtypes = [cam, cam, tm, P, P, P, C.c_int, C.c_int, C.c_int]
        L.ref_godrays.restype = C.c_int
        L.ref_godrays.argtypes = [cam, P, P, P, P, C.c_int, C.c_int]
        L.ref_tonemap.restype = C.c_int
        L.ref_tonemap.argtypes = [tm, P, P, C.c_int, C.c_int]
        for name, n in (("ref_height_gradient", 2), ("ref_remap", 5), ("ref_remap_clamped", 5),
                        ("ref_remap_clamped_ba", 5)):
            getattr(L, name).restype = C.c_float
            getattr(L, name).argtypes = [C.c_float] * n
        L.ref_wang_hash_noise.restype = C.c_float
        L.ref_wang_hash_noise.argtypes = [C.c_uint, C.c_uint, C.c_uint]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


_BIT_DEC = np.float32(1.0) / np.array([1.0, 255.0, 65025.0, 16581375.0], np.float32)


def decode_godray(rgba: np.ndarray) -> np.ndarray:
    """dot(x, 1/bitEnc) of postProcess_GodRays.frag:36-43, in float32 left to right."""
    x = rgba.astype(np.float32)
    d = _BIT_DEC
    return ((x[..., 0] * d[0] + x[..., 1] * d[1]) + x[..., 2] * d[2]) + x[..., 3] * d[3]


def frame(volumes, cam, cam_old, tm, prev, width, height, nthreads=0):
    """One compute command buffer of the reference: the reprojection dispatch
    then the raymarch dispatch (Renderer.cpp:688-716), raymarch writes last.

    Returns (rgba[H,W,4] float32, mask[H,W] float32 with NaN where unwritten)."""
    cur = np.zeros((height, width, 4), np.float32)
    if prev is not None:
        prev = np.ascontiguousarray(prev, np.float32)
        lib().ref_reprojection(C.byref(cam), C.byref(cam_old), C.byref(tm), _p(prev), _p(cur), width, height,
                               nthreads)
    god = np.full((height, width, 4), np.nan, np.float32)
    lib().ref_cloud_raymarch(_p(volumes.base), _p(volumes.detail), _p(volumes.curl), _p(volumes.weather),
                             volumes.fmt, C.byref(cam), C.byref(tm), _p(cur), _p(god), width, height, nthreads)
    return cur, decode_godray(god)


def txaa(cam, cam_old, tm, current, history, nthreads=0):
    current = np.ascontiguousarray(current, np.float32)
    history = np.ascontiguousarray(history, np.float32)
    h, w = current.shape[:2]
    out = np.zeros_like(current)
    lib().ref_txaa(C.byref(cam), C.byref(cam_old), C.byref(tm), _p(history), _p(current), _p(out), w, h, nthreads)
    return out


def wang_hash_noise(u: int, v: int, s: int) -> float:
    return lib().ref_wang_hash_noise(u, v, s)


def godrays(cam, light_color, mask, rgba):
    """postProcess_GodRays.frag over (H, W, 4) `rgba` with the (H, W) mask."""
    rgba = np.ascontiguousarray(rgba, np.float32)
    mask = np.ascontiguousarray(mask, np.float32)
    h, w = rgba.shape[:2]
    out = np.empty_like(rgba)
    light = np.ascontiguousarray(light_color, np.float32)
    lib().ref_godrays(C.byref(cam), _p(light), _p(mask), _p(rgba), _p(out), w, h)
    return out


def tonemap(tm, rgba, fill=np.nan):
    """postProcess_ToneMap.frag: the float values stored, `fill` where no fragment stores."""
    rgba = np.ascontiguousarray(rgba, np.float32)
    h, w = rgba.shape[:2]
    out = np.full((h, w, 4), fill, np.float32)
    lib().ref_tonemap(C.byref(tm), _p(rgba), _p(out), w, h)
    return out


_stbi = None


def stbi_available() -> bool:
    try:
        return ref_build.build_stbi() is not None
    except Exception:
        return False


def stbi_load_rgba(data: bytes) -> np.ndarray | None:
    """The reference's stb_image decode of a TGA or PNG file to (H, W, 4)
    RGBA8 (None when stb_image rejects it)."""
    global _stbi
    if _stbi is None:
        path = ref_build.build_stbi()
        if path is None:
            raise RuntimeError("reference tree not present: stb_image cannot be built")
        L = C.CDLL(str(path))
        L.ref_stbi_load_rgba.restype = C.c_int
        L.ref_stbi_load_rgba.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_void_p,
                                         C.c_longlong]
        _stbi = L
    buf = np.frombuffer(data, np.uint8)
    w, h = C.c_int(), C.c_int()
    if data[:8] == b"\x89PNG\r\n\x1a\n" and len(data) >= 24:  # IHDR width, height (big-endian)
        cap = 4 * int.from_bytes(data[16:20], "big") * int.from_bytes(data[20:24], "big")
    else:  # TGA header width, height (little-endian)
        cap = 4 * (data[12] | data[13] << 8) * (data[14] | data[15] << 8) if len(data) >= 18 else 0
    cap = max(cap, 4)
    out = np.zeros(cap, np.uint8)
    rc = _stbi.ref_stbi_load_rgba(_p(buf), len(data), C.byref(w), C.byref(h), _p(out), cap)
    if rc != 0:
        return None
    return out[: w.value * h.value * 4].reshape(h.value, w.value, 4).copy()
