"""Make tests/golden/golden.npz from the reference's own shader source.

The reference has no tests, fixtures or golden images.  The golden vectors
here are produced by running its GLSL shaders -- compiled as C++ by
oracle/ref_build.py from the reference tree -- on seeded synthetic inputs:

  repro_f{k}, mask_f{k}   cloudRayMarch.comp + reprojection.comp, REF constants,
                          a 64x36 16-frame checkerboard sequence starting from a
                          seeded random previous frame (k = 0, 7, 15 kept)
  quirk_rgba, quirk_mask  a 130x18 frame: floor(130/4) = 32 blocks is a whole
                          number of 32-wide groups, so the reference's dispatch
                          (Renderer.cpp:713-716) never marches columns 128-129
  txaa_out                postProcess_TXAA.frag on seeded current/history images
  wang_uvs, wang_val      WangHashNoise (postProcess_ToneMap.frag:52-66)
  godray_*                postProcess_GodRays.frag over frame 15 of the sequence
                          with the god-ray mask every frame of the sequence left
                          (each frame writes its marched pixels; the image keeps
                          the rest), light colour (1, 1, 0.57, 1) (Sky.cpp:71)
  tonemap_*               postProcess_ToneMap.frag over the god-ray output,
                          time.y = 2.75 (NaN where no fragment stores)
  tga_sha256_base/detail  SHA-256 of the shipped noise volumes as the reference's
                          loader builds them (stb_image on each TGA slice, slice z
                          from "<name>(z+1).tga", ImageLoadingUtility.cpp:75-139)
  gen_sha256_*            SHA-256 of the seed-7 generator volumes (pins the
                          generator bit for bit across hosts)
  ref_assets.npz          (a file of its own) REF-preset frames on volumes built
                          from the reference's shipped noise assets, for the
                          GPU test, which has no reference tree: the TGA bytes
                          of all 32 HighFrequency slices and of LowFrequency
                          slices 1-2 (the base stack repeats them 64 times:
                          the whole 128-slice stack is 8.4 MB of noise that no
                          compressor shrinks), curlNoise.png as stb_image
                          decodes it, SHA-256 of the two volumes as stb_image
                          decodes the stacks, and for each view the uniform
                          bytes plus the reference shaders' checkerboard frame
                          and god-ray mask
  *_ubo                   the exact uniform-block bytes every golden was made
                          with: cameras are built with tan/sin/cos of the host's
                          libm, which may differ by an ulp between hosts, and an
                          ulp in a ray direction can move a density-threshold
                          crossing; tests read these bytes instead of
                          rebuilding the uniforms

The noise volumes fed to the shaders come from the seed-7 generator, with
the base shape's R channel scaled by 0.8 (`golden_volumes`): under the
reference's constants the unscaled volume gives a fully overcast sky, where
every ray saturates and the god-ray mask is identically zero.  The run
needs the reference tree ($METEOROS_REFERENCE, else a checkout named
"reference" beside this repository); the tests only read the .npz.

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from meteoros_gb300 import abi, build, scenes  # noqa: E402
from oracle import pyoracle, pyref  # noqa: E402

OUT = Path(__file__).resolve().parent / "golden.npz"
OUT_ASSETS = Path(__file__).resolve().parent / "ref_assets.npz"
ASSET_LOW_SLICES = 2  # LowFrequency(1..2).tga, stacked 64 times into the 128-slice base volume
ASSET_W, ASSET_H = 64, 36
# (yaw, pitch, checkerboard slot, time.y) of the REF frames on the shipped assets
ASSET_VIEWS = ((0.0, 8.0, 3, 3.5), (35.0, 22.0, 12, 17.25), (-60.0, 4.0, 9, 0.0))

SEQ_W, SEQ_H, SEQ_PITCH = 64, 36, 20.0
QUIRK_W, QUIRK_H, QUIRK_FRAME = 130, 18, 5
KEEP = (0, 7, 15)
GODRAY_LIGHT = np.array([1.0, 1.0, 0.57, 1.0], np.float32)


def sequence_inputs():
    """Cameras and times of the 16-frame REF sequence (camera yaws 0.25 deg/frame)."""
    frames = []
    old = scenes.look((0.0, 0.0, 2.0), 0.0, SEQ_PITCH, 45.0, SEQ_W, SEQ_H)
    for f in range(16):
        cam = scenes.look((0.0, 0.0, 2.0), 0.25 * f, SEQ_PITCH, 45.0, SEQ_W, SEQ_H)
        tm = abi.time_init()
        tm.frame_count_mod16 = f
        tm.time[0] = 0.016
        tm.time[1] = 0.016 * f
        frames.append((cam, old, tm))
        old = cam
    return frames


def ubo_bytes(*structs) -> np.ndarray:
    import ctypes

    return np.frombuffer(b"".join(ctypes.string_at(ctypes.addressof(x), ctypes.sizeof(x)) for x in structs),
                         np.uint8).copy()


def ubos_from(blob: np.ndarray, *types):
    out, off = [], 0
    raw = bytes(np.asarray(blob, np.uint8))
    for t in types:
        import ctypes

        n = ctypes.sizeof(t)
        out.append(t.from_buffer_copy(raw[off:off + n]))
        off += n
    return out


def golden_sequence(golden: dict):
    """The 16 (camera, camera_old, time) triples the sequence golden was made with."""
    return [tuple(ubos_from(golden[f"seq_ubo_f{f}"], abi.CameraUBO, abi.CameraUBO, abi.TimeUBO))
            for f in range(16)]


def golden_volumes(v: dict) -> pyoracle.Volumes:
    base = v["base"].copy()
    base[..., 0] = np.floor(base[..., 0].astype(np.float32) * 0.8).astype(np.uint8)
    return pyoracle.Volumes(base, v["detail"], v["curl"], v["weather"])


def initial_prev():
    return np.random.default_rng(0).random((SEQ_H, SEQ_W, 4), dtype=np.float32)


def txaa_inputs():
    rng = np.random.default_rng(1)
    cur = (rng.random((SEQ_H, SEQ_W, 4), dtype=np.float32) * 2.0).astype(np.float32)
    hist = (rng.random((SEQ_H, SEQ_W, 4), dtype=np.float32) * 2.0).astype(np.float32)
    old = scenes.look((0.0, 0.0, 2.0), 0.0, SEQ_PITCH, 45.0, SEQ_W, SEQ_H)
    cam = scenes.look((0.0, 0.0, 2.0), 0.5, SEQ_PITCH + 0.3, 45.0, SEQ_W, SEQ_H)
    tm = abi.time_init()
    tm.frame_count_mod16 = 9
    return cam, old, tm, cur, hist


def wang_inputs():
    return np.random.default_rng(2).integers(0, 2**32, size=(256, 3), dtype=np.uint64).astype(np.uint32)


def mg_textures() -> Path:
    from oracle import ref_build

    return ref_build.DEFAULT_REF / "src/CloudScapes/textures/CloudTextures"


def asset_stack_order():
    """Shipped slice file of each base-volume slice z: LowFrequency((z % 2) + 1)."""
    return [z % ASSET_LOW_SLICES for z in range(abi.MT_BASE_N)]


def asset_prev(k: int):
    return np.random.default_rng(40 + k).random((ASSET_H, ASSET_W, 4), dtype=np.float32)


def unpack_files(blob: np.ndarray, offsets: np.ndarray) -> list[bytes]:
    raw = bytes(np.asarray(blob, np.uint8))
    return [raw[int(a):int(b)] for a, b in zip(offsets[:-1], offsets[1:])]


def make_ref_assets() -> dict:
    """The fixture of REF frames on volumes from the shipped assets (see the module docstring)."""
    tex = mg_textures()
    low = [(tex / "LowFrequency" / f"LowFrequency({z + 1}).tga").read_bytes() for z in range(ASSET_LOW_SLICES)]
    high = [(tex / "HighFrequency" / f"HighFrequency({z + 1}).tga").read_bytes() for z in range(abi.MT_DETAIL_N)]
    out = {}
    for key, files in (("low", low), ("high", high)):
        out[f"{key}_tga"] = np.frombuffer(b"".join(files), np.uint8).copy()
        out[f"{key}_offsets"] = np.cumsum([0] + [len(f) for f in files]).astype(np.int64)
    low_dec = [pyref.stbi_load_rgba(f) for f in low]
    base = np.stack([low_dec[i] for i in asset_stack_order()])
    detail = np.stack([pyref.stbi_load_rgba(f) for f in high])
    curl = pyref.stbi_load_rgba((tex / "curlNoise.png").read_bytes())
    weather = np.zeros((abi.MT_WEATHER_N, abi.MT_WEATHER_N, 4), np.uint8)  # the REF preset never reads it
    out["curl_rgba8"] = curl
    out["base_sha256"] = np.frombuffer(hashlib.sha256(base.tobytes()).digest(), np.uint8)
    out["detail_sha256"] = np.frombuffer(hashlib.sha256(detail.tobytes()).digest(), np.uint8)
    vol = pyoracle.Volumes(base, detail, curl, weather)
    for k, (yaw, pitch, slot, t) in enumerate(ASSET_VIEWS):
        cam = scenes.look((0.0, 0.0, 2.0), yaw, pitch, 45.0, ASSET_W, ASSET_H)
        old = scenes.look((0.0, 0.0, 2.0), yaw - 0.25, pitch, 45.0, ASSET_W, ASSET_H)
        tm = abi.time_init()
        tm.frame_count_mod16 = slot
        tm.time[0] = 0.016
        tm.time[1] = t
        out[f"view{k}_ubo"] = ubo_bytes(cam, old, tm)
        out[f"view{k}_rgba"], out[f"view{k}_mask"] = pyref.frame(vol, cam, old, tm, asset_prev(k), ASSET_W, ASSET_H)
    return out


def main() -> int:
    build.build()
    if not pyref.available():
        print("reference tree not found: cannot make golden vectors")
        return 1
    v = pyoracle.generate_volumes(7)
    vol = golden_volumes(v)
    out = {}
    prev = initial_prev()
    mask_image = np.zeros((SEQ_H, SEQ_W), np.float32)
    for f, (cam, old, tm) in enumerate(sequence_inputs()):
        out[f"seq_ubo_f{f}"] = ubo_bytes(cam, old, tm)
        rgba, mask = pyref.frame(vol, cam, old, tm, prev, SEQ_W, SEQ_H)
        if f in KEEP:
            out[f"repro_f{f}"] = rgba
            out[f"mask_f{f}"] = mask
        mask_image = np.where(np.isnan(mask), mask_image, mask).astype(np.float32)
        prev = rgba
    out["godray_ubo"] = ubo_bytes(cam)
    out["godray_mask"] = mask_image
    out["godray_out"] = pyref.godrays(cam, GODRAY_LIGHT, mask_image, prev)
    tm = abi.time_init()
    tm.time[1] = 2.75
    out["tonemap_ubo"] = ubo_bytes(tm)
    out["tonemap_out"] = pyref.tonemap(tm, out["godray_out"])
    cam = scenes.look((0.0, 0.0, 2.0), 0.0, SEQ_PITCH, 45.0, QUIRK_W, QUIRK_H)
    tm = abi.time_init()
    tm.frame_count_mod16 = QUIRK_FRAME
    qprev = np.random.default_rng(3).random((QUIRK_H, QUIRK_W, 4), dtype=np.float32)
    out["quirk_ubo"] = ubo_bytes(cam, tm)
    out["quirk_rgba"], out["quirk_mask"] = pyref.frame(vol, cam, cam, tm, qprev, QUIRK_W, QUIRK_H)
    cam, old, tm, cur, hist = txaa_inputs()
    out["txaa_ubo"] = ubo_bytes(cam, old, tm)
    out["txaa_out"] = pyref.txaa(cam, old, tm, cur, hist)
    uvs = wang_inputs()
    out["wang_uvs"] = uvs
    out["wang_val"] = np.array([pyref.wang_hash_noise(int(a), int(b), int(c)) for a, b, c in uvs], np.float32)
    tex = mg_textures()
    for kind, n, key in (("LowFrequency", 128, "tga_sha256_base"), ("HighFrequency", 32, "tga_sha256_detail")):
        vol = np.stack([pyref.stbi_load_rgba((tex / kind / f"{kind}({z + 1}).tga").read_bytes()) for z in range(n)])
        out[key] = np.frombuffer(hashlib.sha256(vol.tobytes()).digest(), np.uint8)
    for k in ("base", "detail", "curl", "weather"):
        for suffix in ("", "_h16", "_b16"):
            out[f"gen_sha256_{k}{suffix}"] = np.frombuffer(
                hashlib.sha256(np.ascontiguousarray(v[k + suffix]).tobytes()).digest(), np.uint8)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")
    np.savez_compressed(OUT_ASSETS, **make_ref_assets())
    print(f"wrote {OUT_ASSETS} ({OUT_ASSETS.stat().st_size} bytes)")
    return 0


if __name__ == "__main__":
    sys.exit(main())
