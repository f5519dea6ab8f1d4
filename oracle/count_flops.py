"""TEST INFRASTRUCTURE — algorithmic FLOPs of the raymarch, counted by the
op-counting build of the oracle (oracle/flop_count.cpp).

Marches a sample of the marched pixels of a 1920x1080 reprojected frame and
of a 960x540 full frame (the config-1 and config-0 views) with every FP32
+, -, *, /, sqrt, exp, pow, acos and cos counted, and fits

    FLOPs = P * pixels + R * rays + S * primary samples + L * light samples

over the per-pixel counts (pixels: every pixel the raymarch visits; rays:
those that march the cloud layer).  bench.py turns the GPU's exact sample
counters into algorithmic FLOPs with these four constants.

Usage: python oracle/count_flops.py
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

from meteoros_gb300 import abi, scenes  # noqa: E402
from oracle import pyoracle  # noqa: E402

LIB = pyoracle.BUILD_DIR / "libflops.so"
SRC = [pyoracle.ORACLE_DIR / "flop_count.cpp", pyoracle.ORACLE_DIR / "meteoros_oracle.cpp",
       pyoracle.ORACLE_DIR / "oracle_math.hpp"]


def build() -> Path:
    pyoracle.BUILD_DIR.mkdir(exist_ok=True)
    newest = max(p.stat().st_mtime for p in SRC)
    if not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = LIB.with_suffix(f".so.{os.getpid()}")
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
                        f"-I{pyoracle.ORACLE_DIR}", str(SRC[0]), "-o", str(tmp)], check=True)
        os.replace(tmp, LIB)
    return LIB


def count(vol, cam, tm, params, w, h, xy) -> np.ndarray:
    """Per pixel: [flops, primary, light, rays]."""
    L = C.CDLL(str(build()))
    L.orc_count_flops.restype = C.c_int
    L.orc_count_flops.argtypes = [C.POINTER(pyoracle.OrcVolumes), C.POINTER(abi.CameraUBO),
                                  C.POINTER(abi.TimeUBO), C.POINTER(abi.Params), C.c_int, C.c_int, C.c_void_p,
                                  C.c_longlong, C.c_void_p]
    xy = np.ascontiguousarray(xy, np.int32)
    out = np.zeros((len(xy), 4), np.uint64)
    v = vol.c()
    rc = L.orc_count_flops(C.byref(v), C.byref(cam), C.byref(tm), C.byref(params), w, h,
                           xy.ctypes.data_as(C.c_void_p), len(xy), out.ctypes.data_as(C.c_void_p))
    if rc:
        raise RuntimeError("orc_count_flops failed")
    return out.astype(np.float64)


def fit():
    """(P, R, S, L) and the per-pixel count rows."""
    g = pyoracle.generate_volumes(2017)
    vol = pyoracle.Volumes(g["base"], g["detail"], g["curl"], g["weather"])
    rows = []
    # config 1: the marched (slot) pixels of a 1080p checkerboard frame, every 4th block
    W, H = 1920, 1080
    cam, old, tm, params = scenes.config_sequence(2017, W, H, frames=3)[2]
    sx, sy = params.slot_x[tm.frame_count_mod16], params.slot_y[tm.frame_count_mod16]
    bx, by = np.meshgrid(np.arange(0, W // 4, 2), np.arange(0, H // 4, 2))
    xy = np.stack([bx.ravel() * 4 + sx, by.ravel() * 4 + sy], 1)
    rows.append(count(vol, cam, tm, params, W, H, xy))
    # config 0: a 960x540 full frame, every 8th pixel
    W0, H0 = 960, 540
    cam0, tm0, params0, _ = scenes.config_view(11, W0, H0)
    ys, xs = np.mgrid[0:H0:8, 0:W0:8]
    rows.append(count(vol, cam0, tm0, params0, W0, H0, np.stack([xs.ravel(), ys.ravel()], 1)))
    d = np.concatenate(rows)
    A = np.stack([np.ones(len(d)), d[:, 3], d[:, 1], d[:, 2]], 1)
    coef, *_ = np.linalg.lstsq(A, d[:, 0], rcond=None)
    return coef, d, A


def main() -> int:
    coef, d, A = fit()
    pred = A @ coef
    rel = np.abs(pred.sum() - d[:, 0].sum()) / d[:, 0].sum()
    print(f"pixels {len(d)}, rays {int(d[:, 3].sum())}, primary {int(d[:, 1].sum())}, light {int(d[:, 2].sum())}")
    print(f"FLOPs per pixel {coef[0]:.1f}, per ray {coef[1]:.1f}, per primary sample {coef[2]:.1f}, "
          f"per light sample {coef[3]:.1f}; total misfit {rel:.2e}; "
          f"mean FLOPs per primary sample (all in) {d[:, 0].sum() / d[:, 1].sum():.1f}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
