"""Host-side mirror of the reference renderer's compute path over the C ABI.

`Context` stands where the reference's Renderer + Sky pair stands for the
compute stage (Renderer.cpp:89-192, Sky.cpp:25-58): it owns the noise
volumes and records the two compute dispatches of a frame (`render`) and the
TXAA pass (`txaa`).  `Session` holds one view's temporal state -- the
previous raymarched frame and the previous resolved frame -- and performs the
ping-pong swap the reference does with its two pre-recorded command buffers
(Renderer.cpp:131-136, 191).

Images are torch CUDA tensors (torch is the allocator and stream provider
here, nothing more); every computation happens in the CUDA kernels behind
the C ABI.  There is no fallback: without the library every call raises.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi


def _ptr(t) -> int | None:
    if t is None:
        return None
    if isinstance(t, int):
        return t
    return t.data_ptr()


def _stream(stream) -> int | None:
    if stream is None:
        import torch

        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


class Context:
    """An mt_ctx: noise volumes on one GPU plus the compute-stage launches."""

    def __init__(self, device: int = 0):
        self.lib = abi.load_library()
        h = C.c_void_p()
        st = self.lib.mt_create(C.byref(h), device)
        if st != abi.MT_OK:
            raise abi.MeteorosError(st, self.lib.mt_last_error(None).decode())
        self.handle = h
        self.device = device

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.mt_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, st: int) -> None:
        if st != abi.MT_OK:
            raise abi.MeteorosError(st, self.lib.mt_last_error(self.handle).decode())

    # ---- volumes -----------------------------------------------------------
    def generate_volumes(self, seed: int, stream=None) -> None:
        self._check(self.lib.mt_generate_volumes(self.handle, C.c_uint64(seed & (2**64 - 1)), _stream(stream)))

    def generate_weather(self, slot: int, seed: int, stream=None) -> None:
        self._check(self.lib.mt_generate_weather(self.handle, slot, C.c_uint64(seed & (2**64 - 1)), _stream(stream)))

    def upload_volumes(self, base=None, detail=None, curl=None, weather=None) -> None:
        arrs = [None if a is None else np.ascontiguousarray(a, np.uint8) for a in (base, detail, curl, weather)]
        self._check(self.lib.mt_upload_volumes(self.handle, *[None if a is None else a.ctypes.data for a in arrs]))

    def upload_weather(self, slot: int, weather) -> None:
        a = np.ascontiguousarray(weather, np.uint8)
        self._check(self.lib.mt_upload_weather(self.handle, slot, a.ctypes.data))

    def download_volumes(self, weather_slot: int = 0) -> dict:
        N, D, Cn, Wn = abi.MT_BASE_N, abi.MT_DETAIL_N, abi.MT_CURL_N, abi.MT_WEATHER_N
        out = {"base": np.zeros((N, N, N, 4), np.uint8), "detail": np.zeros((D, D, D, 4), np.uint8),
               "curl": np.zeros((Cn, Cn, 4), np.uint8), "weather": np.zeros((Wn, Wn, 4), np.uint8)}
        self._check(self.lib.mt_download_volumes(self.handle, out["base"].ctypes.data, out["detail"].ctypes.data,
                                                 out["curl"].ctypes.data, out["weather"].ctypes.data, weather_slot))
        return out

    def download_volumes_16(self, storage: int, weather_slot: int = 0) -> dict:
        N, D, Cn, Wn = abi.MT_BASE_N, abi.MT_DETAIL_N, abi.MT_CURL_N, abi.MT_WEATHER_N
        out = {"base": np.zeros((N, N, N, 4), np.uint16), "detail": np.zeros((D, D, D, 4), np.uint16),
               "curl": np.zeros((Cn, Cn, 4), np.uint16), "weather": np.zeros((Wn, Wn, 4), np.uint16)}
        self._check(self.lib.mt_download_volumes_16(self.handle, storage, out["base"].ctypes.data,
                                                    out["detail"].ctypes.data, out["curl"].ctypes.data,
                                                    out["weather"].ctypes.data, weather_slot))
        return out

    # ---- the compute stage -------------------------------------------------
    def render(self, camera: abi.CameraUBO, camera_old: abi.CameraUBO, time: abi.TimeUBO, params: abi.Params,
               prev, cur, mask=None, flags: int = abi.MT_RENDER_CHECKERBOARD, stream=None) -> None:
        h, w = int(cur.shape[0]), int(cur.shape[1])
        self._check(self.lib.mt_render(self.handle, C.byref(camera), C.byref(camera_old), C.byref(time),
                                       C.byref(params), _ptr(prev), _ptr(cur), _ptr(mask), w, h, flags,
                                       _stream(stream)))

    def render_frame(self, camera, camera_old, time, params, prev, cur, history, out, mask=None,
                     flags: int = abi.MT_RENDER_CHECKERBOARD, stream=None) -> None:
        """Raymarch, reprojection and TXAA of one frame: the reprojection and the
        TXAA history taps run beside the raymarch, the TXAA resolve after it."""
        h, w = int(cur.shape[0]), int(cur.shape[1])
        self._check(self.lib.mt_render_frame(self.handle, C.byref(camera), C.byref(camera_old), C.byref(time),
                                             C.byref(params), _ptr(prev), _ptr(cur), _ptr(history), _ptr(out),
                                             _ptr(mask), w, h, flags, _stream(stream)))

    def txaa(self, camera, camera_old, time, params, current, history, out, stream=None) -> None:
        h, w = int(current.shape[0]), int(current.shape[1])
        self._check(self.lib.mt_txaa(self.handle, C.byref(camera), C.byref(camera_old), C.byref(time),
                                     C.byref(params), _ptr(current), _ptr(history), _ptr(out), w, h,
                                     _stream(stream)))

    def godrays(self, camera, light_color, mask, inp, out, stream=None) -> None:
        """God-ray radial blur of `mask` (H, W) added to `inp` (H, W, 4) into `out` (may be `inp`)."""
        h, w = int(inp.shape[0]), int(inp.shape[1])
        light = (C.c_float * 4)(*[float(x) for x in light_color])
        self._check(self.lib.mt_godrays(self.handle, C.byref(camera), light, _ptr(mask), _ptr(inp), _ptr(out), w, h,
                                        _stream(stream)))

    def tonemap(self, time, inp, out, out_format: int = abi.MT_LDR_RGBA8, stream=None) -> None:
        """Tone map + dither of `inp` (H, W, 4) into `out`: (H, W, 4) uint8 for
        MT_LDR_RGBA8, (H, W, 4) float32 for MT_LDR_RGBA32F."""
        h, w = int(inp.shape[0]), int(inp.shape[1])
        self._check(self.lib.mt_tonemap(self.handle, C.byref(time), _ptr(inp), _ptr(out), w, h, int(out_format),
                                        _stream(stream)))

    def render_batch(self, views: list[abi.View], stream=None) -> None:
        arr = (abi.View * len(views))(*views)
        self._check(self.lib.mt_render_batch(self.handle, arr, len(views), _stream(stream)))

    def autotune_batch(self, views: list[abi.View], stream=None) -> abi.Tuning:
        arr = (abi.View * len(views))(*views)
        t = abi.Tuning()
        self._check(self.lib.mt_autotune_batch(self.handle, arr, len(views), _stream(stream), C.byref(t)))
        return t

    def set_tuning(self, march_lanes: int | None = None, fused_resolve: bool | None = None,
                   batch_tile: tuple[int, int] | None = None, batch_lanes: int | None = None,
                   batch_direct: bool | None = None, reproject_serial: bool | None = None,
                   march_block: int | None = None, march_order: int | None = None,
                   batch_order: int | None = None) -> abi.Tuning:
        t = abi.Tuning()
        self._check(self.lib.mt_get_tuning(self.handle, C.byref(t)))
        if march_lanes is not None:
            t.march_lanes = march_lanes
        if fused_resolve is not None:
            t.fused_resolve = 1 if fused_resolve else 0
        if batch_tile is not None:
            t.batch_tile_w, t.batch_tile_h = batch_tile
        if batch_lanes is not None:
            t.batch_lanes = batch_lanes
        if batch_direct is not None:
            t.batch_direct = 1 if batch_direct else 0
        if reproject_serial is not None:
            t.reproject_serial = 1 if reproject_serial else 0
        if march_block is not None:
            t.march_block = march_block
        if march_order is not None:
            t.march_order = march_order
        if batch_order is not None:
            t.batch_order = batch_order
        self._check(self.lib.mt_set_tuning(self.handle, C.byref(t)))
        return t

    def set_sample_trace(self, counts=None) -> None:
        """Per-pixel control-flow trace of later renders (mt_set_sample_trace):
        `counts` an (H, W, 4) int32 device tensor, or None to stop."""
        self._check(self.lib.mt_set_sample_trace(self.handle, _ptr(counts)))
        self._trace = counts  # kept alive while the library may write it

    def set_timing(self, enabled: bool) -> None:
        self._check(self.lib.mt_set_timing(self.handle, 1 if enabled else 0))

    def kernel_times(self) -> abi.KernelTimes:
        t = abi.KernelTimes()
        self._check(self.lib.mt_get_kernel_times(self.handle, C.byref(t)))
        return t

    def stats(self, reset: bool = True, stream=None) -> abi.Stats:
        s = abi.Stats()
        self._check(self.lib.mt_get_stats(self.handle, C.byref(s), 1 if reset else 0, _stream(stream)))
        return s


@dataclass
class FrameInputs:
    camera: abi.CameraUBO
    camera_old: abi.CameraUBO
    time: abi.TimeUBO
    params: abi.Params


class Session:
    """One view's temporal state on the device: raw frames for reprojection,
    resolved frames for TXAA history, and the god-ray masks.  Every buffer is
    double-buffered, so a frame's results can be read back while the next
    frame renders."""

    def __init__(self, ctx: Context, width: int, height: int, txaa: bool = True):
        import torch

        self.ctx, self.width, self.height, self.use_txaa = ctx, width, height, txaa
        dev = torch.device("cuda", ctx.device)
        self.raw = [torch.zeros((height, width, 4), dtype=torch.float32, device=dev) for _ in range(2)]
        self.resolved = [torch.zeros((height, width, 4), dtype=torch.float32, device=dev) for _ in range(2)]
        self.masks = [torch.zeros((height, width), dtype=torch.float32, device=dev) for _ in range(2)]
        self.parity = 0
        self.frames = 0

    @property
    def mask(self):
        """The last frame's god-ray mask."""
        return self.masks[self.parity ^ 1]

    @property
    def output(self):
        """The last frame's result: the resolved image with TXAA, else the raw one."""
        if self.use_txaa:
            return self.resolved[self.parity ^ 1]
        return self.raw[self.parity ^ 1]

    def frame(self, f: FrameInputs, flags: int = abi.MT_RENDER_CHECKERBOARD, stream=None) -> None:
        """Record one frame: checkerboard render (the first frame of a session
        marches every pixel: there is no previous frame to reproject), then TXAA."""
        cur, prev = self.raw[self.parity], self.raw[self.parity ^ 1]
        fl = flags if self.frames > 0 else (flags | abi.MT_RENDER_FULL)
        if self.use_txaa and self.frames > 0:
            self.ctx.render_frame(f.camera, f.camera_old, f.time, f.params, prev, cur, self.resolved[self.parity ^ 1],
                                  self.resolved[self.parity], self.masks[self.parity], fl, stream)
        else:
            self.ctx.render(f.camera, f.camera_old, f.time, f.params, prev, cur, self.masks[self.parity], fl, stream)
            if self.use_txaa:  # first frame: the frame is its own history
                self.ctx.txaa(f.camera, f.camera_old, f.time, f.params, cur, cur, self.resolved[self.parity], stream)
        self.parity ^= 1
        self.frames += 1
