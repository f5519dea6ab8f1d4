"""Build the in-tree C-ABI library meteoros_gb300/_build/libmeteoros_gb300.so.

Every CUDA translation unit is compiled by nvcc for sm_103a only
(`-gencode arch=compute_103a,code=sm_103a`), in parallel, then linked into one
shared library with the CUDA runtime linked statically.  The kernels of the
FP32 form are compiled with -fmad=false and IEEE division/square root: their
results must follow the reference's operation order exactly (no contraction
into fused multiply-adds).  The precision-form kernels (FP16/BF16 volumes)
are compiled with --use_fast_math.

Usage: python -m meteoros_gb300.build [--force] [--verbose-ptxas]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libmeteoros_gb300.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          f"-I{INCLUDE}"]
EXACT = ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]
# The precision form is measured against the FP64 oracle statistically, not
# bit for bit: its FP32 arithmetic may contract and use the fast intrinsics
# (errors ~1e-6 relative, far below the half-precision interpolation's).
FAST = ["--use_fast_math"]

# translation unit -> extra flags
UNITS = {
    "mt_host.cpp": ["-x", "cu", "-Xcompiler", "-ffp-contract=off"],
    "mt_capi.cu": [],
    "mt_server.cpp": ["-x", "cu"],
    "mt_render.cu": EXACT,
    "mt_march_u8.cu": EXACT,
    "mt_march_f16.cu": FAST,
    "mt_march_bf16.cu": FAST,
    "mt_noise.cu": EXACT,
    "mt_post.cu": EXACT,
    "mt_assets.cu": [],
    "mt_consts.cpp": ["-x", "cu", "-Xcompiler", "-ffp-contract=off"],
}


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found")
    return exe


def _deps() -> list[Path]:
    return sorted(CSRC.glob("*")) + sorted(INCLUDE.glob("*.h")) + [Path(__file__)]


def build(force: bool = False, verbose_ptxas: bool = False, jobs: int | None = None) -> Path:
    OUT.mkdir(exist_ok=True)
    newest = max(p.stat().st_mtime for p in _deps())
    if not force and LIB.exists() and LIB.stat().st_mtime >= newest:
        return LIB
    exe = nvcc()
    objs = []
    cmds = []
    for unit, extra in UNITS.items():
        obj = OUT / (unit + ".o")
        objs.append(obj)
        cmd = [exe, *ARCH, *COMMON, *extra, "-c", str(CSRC / unit), "-o", str(obj)]
        if verbose_ptxas and unit.endswith(".cu"):
            cmd += ["-Xptxas", "-v"]
        cmds.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        results = list(ex.map(run, cmds))
    for cmd, r in results:
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose_ptxas:
            sys.stderr.write(r.stderr)
    tmp = LIB.with_suffix(f".so.{os.getpid()}")
    link = [exe, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(link)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def main() -> int:
    ap = argparse.ArgumentParser(description="build libmeteoros_gb300.so for sm_103a")
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose-ptxas", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose_ptxas=a.verbose_ptxas))
    return 0


if __name__ == "__main__":
    sys.exit(main())
