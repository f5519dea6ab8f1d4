"""TEST INFRASTRUCTURE — compile the reference's own GLSL shader source as C++.

The reference's compute stage exists only as GLSL (src/CloudScapes/shaders/*),
and no graphics stack or SPIR-V toolchain exists here, so the shaders cannot
run through Vulkan.  Their source can still be compiled as C++: this script
reads each shader from the reference tree, applies a small mechanical
rewrite (below), wraps it in a namespace of the GLSL environment in
oracle/glsl_shim.hpp, and compiles it together with a dispatch driver
(oracle/ref_driver.cpp) into oracle/_ref/libmeteoros_ref.so.  Nothing is
copied into the repository: the generated sources live in oracle/_ref/gen
(git-ignored) and are rebuilt from the reference tree.

The rewrite only changes syntax that C++ spells differently from GLSL:
  * `#version`, `#extension` and `layout(local_size...) in;` are dropped;
  * `layout(...) uniform <block> {...} name;` becomes a struct variable, an
    anonymous block becomes plain variables; images and samplers become
    variables of the shim's image2D / sampler2D / sampler3D types;
  * `layout(location=N) in/out T x;` becomes a thread_local variable;
  * parameter qualifiers: `in T x` -> `T x`, `out/inout T x` -> `T& x`;
  * float literals get an `f` suffix (GLSL literals are single precision);
  * swizzles `.xyz`/`.rgb`/... become `.sw<0,1,2>()` (or `.swref<...>()` when
    assigned to); single `.r/.g/.b/.a` become `.x/.y/.z/.w`;
  * scalar struct members get a `{}` initialiser (GLSL leaves an unset
    Intersection.t undefined; here it is 0, as in the oracle);
  * `void main(` becomes `void shader_main(`.

Run: python oracle/ref_build.py [--reference /path/to/reference]
"""
from __future__ import annotations

import argparse
import os
import re
import subprocess
import sys
from pathlib import Path

ORACLE = Path(__file__).resolve().parent
OUT = ORACLE / "_ref"
GEN = OUT / "gen"
LIB = OUT / "libmeteoros_ref.so"
# The reference tree: $METEOROS_REFERENCE, else a checkout named "reference"
# beside this repository's directory.
DEFAULT_REF = Path(os.environ.get("METEOROS_REFERENCE", ORACLE.parents[1] / "reference"))
SHADERS = {
    "cloudRayMarch": "src/CloudScapes/shaders/cloudRayMarch.comp",
    "reprojection": "src/CloudScapes/shaders/reprojection.comp",
    "txaa": "src/CloudScapes/shaders/postProcess_TXAA.frag",
    "tonemap": "src/CloudScapes/shaders/postProcess_ToneMap.frag",
    "godrays": "src/CloudScapes/shaders/postProcess_GodRays.frag",
}

_SWZ = {"x": 0, "y": 1, "z": 2, "w": 3, "r": 0, "g": 1, "b": 2, "a": 3}
_FLOAT = re.compile(r"(?<![\w.])(\d+\.\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])")


def _swizzle(m: re.Match) -> str:
    idx = ",".join(str(_SWZ[c]) for c in m.group(1))
    return f".swref<{idx}>()" if m.group(2) else f".sw<{idx}>()"


def transform(src: str) -> str:
    s = src
    s = re.sub(r"^\s*#\s*(version|extension)[^\n]*$", "", s, flags=re.M)
    s = re.sub(r"layout\s*\([^)]*\)\s*in\s*;", "", s)

    def block(m: re.Match) -> str:
        name, body, inst = m.group(1), m.group(2), m.group(3)
        return f"struct {name} {{{body}}} {inst};" if inst else body

    s = re.sub(r"layout\s*\([^)]*\)\s*uniform\s+(\w+)\s*\{([^}]*)\}\s*(\w*)\s*;", block, s)
    s = re.sub(r"layout\s*\([^)]*\)\s*uniform\s+(?:(?:writeonly|readonly)\s+)*(image2D|sampler2D|sampler3D)\s+(\w+)\s*;",
               r"\1 \2;", s)
    s = re.sub(r"layout\s*\([^)]*\)\s*(?:in|out)\s+(\w+)\s+(\w+)\s*;", r"thread_local \1 \2;", s)
    # parameter qualifiers: on one line only (a comment's "in this" followed
    # by a line break must stay a comment)
    s = re.sub(r"\binout[ \t]+(\w+)[ \t]+(\w+)", r"\1& \2", s)
    s = re.sub(r"\bout[ \t]+(\w+)[ \t]+(\w+)", r"\1& \2", s)
    s = re.sub(r"\bin[ \t]+(\w+)[ \t]+(\w+)", r"\1 \2", s)
    s = _FLOAT.sub(lambda m: m.group(1) + "f", s)
    s = re.sub(r"(?<=[\w\)\]])\.([xyzw]{2,4}|[rgba]{2,4})\b(?=(\s*(?:\+=|-=|\*=|/=|=(?!=)))?)", _swizzle, s)
    s = re.sub(r"(?<=[\w\)\]])\.([rgba])\b(?!\w)", lambda m: "." + "xyzw"[_SWZ[m.group(1)]], s)

    def init_members(m: re.Match) -> str:
        body = re.sub(r"\b(bool|float|int|uint)\s+(\w+)\s*;", r"\1 \2{};", m.group(2))
        return f"struct {m.group(1)} {{{body}}}"

    s = re.sub(r"struct\s+(\w+)\s*\{([^}]*)\}", init_members, s)
    s = re.sub(r"\bvoid\s+main\s*\(", "void shader_main(", s)
    return s


def generate(reference: Path) -> None:
    GEN.mkdir(parents=True, exist_ok=True)
    for name, rel in SHADERS.items():
        src = (reference / rel).read_text()
        text = f"// generated by oracle/ref_build.py from {rel}; do not edit\n" + transform(src)
        (GEN / f"{name}.inc").write_text(text)


def build(reference: Path = DEFAULT_REF, force: bool = False) -> Path | None:
    """Build oracle/_ref/libmeteoros_ref.so; None when the reference is absent."""
    if not (reference / SHADERS["cloudRayMarch"]).exists():
        return None
    inputs = [reference / r for r in SHADERS.values()] + [
        ORACLE / "glsl_shim.hpp", ORACLE / "ref_driver.cpp", Path(__file__)]
    newest = max(p.stat().st_mtime for p in inputs)
    if not force and LIB.exists() and LIB.stat().st_mtime >= newest:
        return LIB
    generate(reference)
    tmp = LIB.with_suffix(f".so.{os.getpid()}")
    cmd = ["g++", "-O2", "-fopenmp", "-ffp-contract=off", "-std=c++17", "-fPIC", "-shared",
           "-w", f"-I{ORACLE}", f"-I{GEN}", str(ORACLE / "ref_driver.cpp"), "-o", str(tmp)]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


STBI_LIB = OUT / "libstbi_ref.so"
STBI_HEADER = "external/stb_image.h"


def build_stbi(reference: Path = DEFAULT_REF, force: bool = False) -> Path | None:
    """Build oracle/_ref/libstbi_ref.so: the reference's vendored stb_image
    (external/stb_image.h, included from the reference tree) behind
    oracle/ref_stbi.c.  None when the reference is absent."""
    header = reference / STBI_HEADER
    if not header.exists():
        return None
    OUT.mkdir(parents=True, exist_ok=True)
    inputs = [header, ORACLE / "ref_stbi.c", Path(__file__)]
    newest = max(p.stat().st_mtime for p in inputs)
    if not force and STBI_LIB.exists() and STBI_LIB.stat().st_mtime >= newest:
        return STBI_LIB
    tmp = STBI_LIB.with_suffix(f".so.{os.getpid()}")
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-w", f"-I{header.parent}", str(ORACLE / "ref_stbi.c"), "-o", str(tmp)]
    subprocess.run(cmd, check=True)
    os.replace(tmp, STBI_LIB)
    return STBI_LIB


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--reference", type=Path, default=DEFAULT_REF)
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    lib = build(a.reference, a.force)
    build_stbi(a.reference, a.force)
    if lib is None:
        print(f"reference shaders not found under {a.reference}; nothing built")
        return 1
    print(lib)
    return 0


if __name__ == "__main__":
    sys.exit(main())
