"""Python mirror of the serving loop (mt_server_* in include/meteoros.h).

A Server owns a native worker thread that batches per-session frame requests
as they arrive (continuous batching, up to two batches overlapping on the
device) over one Context's shared noise volumes.  Sessions keep their
previous frame resident in HBM and are admitted while their state fits the
server's HBM budget.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi


@dataclass
class RequestInfo:
    id: int
    session: int
    submit_s: float
    start_s: float
    done_s: float
    batch_size: int
    status: int

    @property
    def latency_s(self) -> float:
        return self.done_s - self.submit_s


class Server:
    def __init__(self, ctx, max_batch: int = 64, streams: int = 2, hbm_budget_bytes: int = 40 << 30,
                 batch_lanes: int = 0, per_request: bool = False, use_graph: bool = False,
                 admission_wait_ms: int = 0):
        self.ctx = ctx
        self.lib = ctx.lib
        cfg = abi.ServerConfig()
        cfg.hbm_budget_bytes = int(hbm_budget_bytes)
        cfg.max_batch = int(max_batch)
        cfg.streams = int(streams)
        cfg.batch_lanes = int(batch_lanes)
        cfg.per_request = 1 if per_request else 0
        cfg.use_graph = 1 if use_graph else 0
        cfg.admission_wait_ms = int(admission_wait_ms)
        h = C.c_void_p()
        st = self.lib.mt_server_create(ctx.handle, C.byref(cfg), C.byref(h))
        if st != abi.MT_OK:
            raise abi.MeteorosError(st, self.lib.mt_last_error(ctx.handle).decode() or "mt_server_create failed")
        self.handle = h
        self.sessions: dict[int, tuple[int, int]] = {}

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.mt_server_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, st: int) -> None:
        if st != abi.MT_OK:
            raise abi.MeteorosError(st, self.lib.mt_server_last_error(self.handle).decode())

    @staticmethod
    def clock() -> float:
        """The server's clock (seconds, monotonic), the one request times use."""
        return abi.load_library().mt_server_clock()

    def open_session(self, width: int, height: int, params: abi.Params) -> int:
        sid = C.c_int64()
        self._check(self.lib.mt_server_open_session(self.handle, width, height, C.byref(params), C.byref(sid)))
        self.sessions[sid.value] = (width, height)
        return sid.value

    def close_session(self, session: int) -> None:
        self._check(self.lib.mt_server_close_session(self.handle, C.c_int64(session)))
        self.sessions.pop(session, None)

    def submit(self, session: int, camera: abi.CameraUBO, time: abi.TimeUBO) -> int:
        rid = C.c_uint64()
        self._check(self.lib.mt_server_submit(self.handle, C.c_int64(session), C.byref(camera), C.byref(time),
                                              C.byref(rid)))
        return rid.value

    def wait(self, request: int, timeout_ms: int = 30000) -> RequestInfo:
        info = abi.RequestInfo()
        st = self.lib.mt_server_wait(self.handle, C.c_uint64(request), int(timeout_ms), C.byref(info))
        if st == abi.MT_ERR_TIMEOUT:
            raise abi.MeteorosError(st, f"request {request} not done within {timeout_ms} ms")
        out = RequestInfo(info.id, info.session, info.submit_s, info.start_s, info.done_s, info.batch_size,
                          info.status)
        if st != abi.MT_OK:
            raise abi.MeteorosError(st, self.lib.mt_server_last_error(self.handle).decode())
        return out

    def read_frame(self, session: int) -> tuple[np.ndarray, np.ndarray]:
        """The session's last frame (H, W, 4) and god-ray mask (H, W), in host memory."""
        w, h = self.sessions[session]
        rgba = np.empty((h, w, 4), np.float32)
        mask = np.empty((h, w), np.float32)
        self._check(self.lib.mt_server_read_frame(self.handle, C.c_int64(session),
                                                  rgba.ctypes.data_as(C.c_void_p), mask.ctypes.data_as(C.c_void_p)))
        return rgba, mask

    def memory(self) -> tuple[int, int]:
        used, budget = C.c_uint64(), C.c_uint64()
        self._check(self.lib.mt_server_memory(self.handle, C.byref(used), C.byref(budget)))
        return used.value, budget.value
