"""Seeded scene builders: the uniform blocks of the benchmark configurations.

The reference drives its uniforms from an interactive window (main.cpp:172-186:
keyboard-rotated camera, wall-clock time); these builders produce the same
uniform blocks deterministically from a seed:

  reference_frame   the reference's own camera (main.cpp:157-160: eye (0,0,2)
                    looking toward (0,0,1), fovy 45 deg) with optional pitch
  config_view       a camera at 100 m altitude, FOV 60 deg, yaw in [0,360),
                    pitch in [5,30] deg, sun uniform on the upper hemisphere,
                    wind 10 m/s at heading 45 deg (mt_params_config)
  config_sequence   16 frames yawing 0.5 deg/frame with t += 0.16 s/frame

`uniforms` names the module that produces the uniform blocks and presets:
meteoros_gb300.abi (the library's mt_camera_look_at, mt_time_init,
mt_params_config, mt_params_reference) by default; any module with functions
of the same names and signatures can stand in (a host-only caller that must
not load the CUDA library passes its own).
"""
from __future__ import annotations

import math

import numpy as np

from . import abi


def _forward(yaw_deg: float, pitch_deg: float):
    y, p = math.radians(yaw_deg), math.radians(pitch_deg)
    return (math.cos(p) * math.sin(y), math.sin(p), -math.cos(p) * math.cos(y))


def look(eye, yaw_deg: float, pitch_deg: float, fovy_deg: float, width: int, height: int,
         uniforms=abi) -> abi.CameraUBO:
    f = _forward(yaw_deg, pitch_deg)
    ref = tuple(e + d for e, d in zip(eye, f))
    return uniforms.camera_look_at(eye, ref, fovy_deg, width / height, 0.1, 1000.0)


def sun_direction(rng: np.random.Generator):
    """Uniform on the upper hemisphere (y up)."""
    y = float(rng.uniform(0.0, 1.0))
    phi = float(rng.uniform(0.0, 2.0 * math.pi))
    r = math.sqrt(max(0.0, 1.0 - y * y))
    return (r * math.cos(phi), y, r * math.sin(phi))


def set_sun(params: abi.Params, direction, distance: float = 1.0e9) -> abi.Params:
    for i in range(3):
        params.sun_light_pos[i] = direction[i] * distance
        params.sky_sun_pos[i] = direction[i] * distance
    return params


def reference_frame(width: int, height: int, pitch_deg: float = 0.0, frame: int = 0, t: float = 0.0,
                    uniforms=abi):
    """The reference's camera and constants (REF preset)."""
    cam = look((0.0, 0.0, 2.0), 0.0, pitch_deg, 45.0, width, height, uniforms)
    tm = uniforms.time_init()
    tm.frame_count_mod16 = frame % 16
    tm.time[1] = t
    return cam, tm, uniforms.params_reference()


def config_view(seed: int, width: int, height: int, steps: int | None = None, uniforms=abi):
    """Camera, time and params of one benchmark view (configs 0, 2, 3)."""
    rng = np.random.default_rng(seed)
    yaw = float(rng.uniform(0.0, 360.0))
    pitch = float(rng.uniform(5.0, 30.0))
    cam = look((0.0, 100.0, 0.0), yaw, pitch, 60.0, width, height, uniforms)
    params = set_sun(uniforms.params_config(), sun_direction(rng))
    if steps is not None:
        params.steps_min = params.steps_max = int(steps)
    tm = uniforms.time_init()
    return cam, tm, params, (yaw, pitch)


def config_sequence(seed: int, width: int, height: int, frames: int = 16, yaw_step: float = 0.5,
                    dt: float = 0.16, uniforms=abi):
    """Per-frame (camera, camera_old, time, params) of the reprojected sequence (config 1)."""
    cam0, tm, params, (yaw, pitch) = config_view(seed, width, height, uniforms=uniforms)
    out = []
    old = cam0
    for i in range(frames):
        cam = look((0.0, 100.0, 0.0), yaw + yaw_step * i, pitch, 60.0, width, height, uniforms)
        t = abi.TimeUBO()
        C_copy(t, tm)
        t.frame_count_mod16 = i % 16
        t.time[0] = dt if i > 0 else 0.0
        t.time[1] = dt * i
        out.append((cam, old, t, params))
        old = cam
    return out


def C_copy(dst, src):
    import ctypes

    ctypes.memmove(ctypes.addressof(dst), ctypes.addressof(src), ctypes.sizeof(src))
    return dst


CONFIG3_RESOLUTIONS = ((256, 256), (640, 360), (960, 540), (1280, 720), (1920, 1080))


def config3_views(seed: int, n_views: int = 64, resolutions=CONFIG3_RESOLUTIONS):
    """The batched workload (config 3): per view a resolution drawn uniformly
    from `resolutions`, a camera/sun/time drawn as in config 0, a step budget
    drawn from U{64..128} and its own weather map (generated from seed + view
    id into weather slot view id).  Returns [(width, height, camera, time, params)]."""
    rng = np.random.default_rng(seed)
    out = []
    for v in range(n_views):
        w, h = resolutions[int(rng.integers(0, len(resolutions)))]
        cam, tm, params, _ = config_view(seed * 1000 + v, w, h, steps=int(rng.integers(64, 129)))
        params.weather_slot = v
        out.append((w, h, cam, tm, params))
    return out


def make_view(cam, cam_old, tm, params, cur, prev=None, mask=None, flags: int = 1) -> abi.View:
    """An mt_view over device tensors (cur/prev: (H, W, 4) float32, mask: (H, W))."""
    v = abi.View()
    v.camera, v.camera_old, v.time, v.params = cam, cam_old, tm, params
    v.prev_rgba = None if prev is None else prev.data_ptr()
    v.cur_rgba = cur.data_ptr()
    v.godray_mask = None if mask is None else mask.data_ptr()
    v.height, v.width = int(cur.shape[0]), int(cur.shape[1])
    v.flags = flags
    return v
