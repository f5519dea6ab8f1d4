"""TGA slice decoding (the noise-volume asset path) on the CPU: the
restatement against the reference's own decoder (stb_image v2.16 as vendored
by the reference) on every shipped slice and on synthetic files, and the
golden hashes of the shipped volumes."""
import glob
import hashlib
from pathlib import Path

import numpy as np
import pytest

from tests.tga_util import encode_tga, runs_image

from oracle.ref_build import DEFAULT_REF

REF_TEXTURES = DEFAULT_REF / "src/CloudScapes/textures/CloudTextures"


@pytest.fixture(scope="module")
def stbi():
    from oracle import pyref

    if not pyref.stbi_available():
        pytest.skip("reference tree not present")
    return pyref


@pytest.mark.parametrize("rle,bpp,top_left", [(True, 32, False), (True, 24, False), (False, 32, True),
                                              (False, 24, False), (True, 32, True)])
def test_round_trip(oracle, rle, bpp, top_left):
    img = runs_image(37, 53, seed=bpp + 2 * rle + 4 * top_left)
    if bpp == 24:
        img[..., 3] = 255
    data = encode_tga(img, rle=rle, bpp=bpp, top_left=top_left, seed=5, image_id=b"meteoros")
    assert np.array_equal(oracle.decode_tga(data), img)


def test_truncated_rle_reads_zero_bytes(oracle, stbi):
    img = runs_image(16, 16, seed=3)
    data = encode_tga(img, rle=True, seed=1)
    for cut in (18, 40, len(data) // 2, len(data) - 1):
        a = oracle.decode_tga(data[:cut])
        b = stbi.stbi_load_rgba(data[:cut])
        assert np.array_equal(a, b), cut


def test_rejects_files_outside_the_subset(oracle):
    img = runs_image(8, 8, seed=0)
    good = bytearray(encode_tga(img))
    for byte, value in ((1, 1), (2, 3), (2, 1), (16, 16), (16, 8)):
        bad = bytearray(good)
        bad[byte] = value
        with pytest.raises(ValueError):
            oracle.decode_tga(bytes(bad))


@pytest.mark.parametrize("seed", range(6))
def test_synthetic_files_match_reference_decoder(oracle, stbi, seed):
    rng = np.random.default_rng(seed)
    img = runs_image(int(rng.integers(1, 70)), int(rng.integers(1, 70)), seed)
    for rle in (True, False):
        for bpp in (24, 32):
            data = encode_tga(img, rle=rle, bpp=bpp, top_left=bool(seed & 1), seed=seed)
            assert np.array_equal(oracle.decode_tga(data), stbi.stbi_load_rgba(data))


def shipped_volume(decode, kind, n):
    slices = [decode(Path(REF_TEXTURES, kind, f"{kind}({z + 1}).tga").read_bytes()) for z in range(n)]
    return np.stack(slices)


def test_every_shipped_slice_matches_reference_decoder(oracle, stbi):
    files = sorted(glob.glob(str(REF_TEXTURES / "*" / "*.tga")))
    assert len(files) == 160
    for f in files:
        data = Path(f).read_bytes()
        assert np.array_equal(oracle.decode_tga(data), stbi.stbi_load_rgba(data)), f


def test_shipped_volumes_match_golden_hashes(oracle, stbi, golden):
    for kind, n, key in (("LowFrequency", 128, "tga_sha256_base"), ("HighFrequency", 32, "tga_sha256_detail")):
        vol = shipped_volume(oracle.decode_tga, kind, n)
        assert hashlib.sha256(vol.tobytes()).digest() == golden[key].tobytes(), kind


def test_ref_frame_with_shipped_assets_matches_reference_source(oracle, stbi):
    """The REF preset on the reference's own noise assets (TGA slices decoded
    by the restatement, curl and weather maps by the reference's stb_image):
    the restatement's frame equals the reference shader source's, bit for bit."""
    from meteoros_gb300 import abi
    from oracle import pyref

    base = shipped_volume(oracle.decode_tga, "LowFrequency", 128)
    detail = shipped_volume(oracle.decode_tga, "HighFrequency", 32)
    curl = stbi.stbi_load_rgba((REF_TEXTURES / "curlNoise.png").read_bytes())
    weather = stbi.stbi_load_rgba((REF_TEXTURES / "weatherMap.png").read_bytes())
    assert base.shape == (128, 128, 128, 4) and detail.shape == (32, 32, 32, 4)
    assert curl.shape == (128, 128, 4) and weather.shape == (512, 512, 4)
    vol = oracle.Volumes(base, detail, curl, weather)
    w, h = 72, 40
    prev = np.random.default_rng(9).random((h, w, 4), dtype=np.float32)
    for pitch, slot in ((5.0, 3), (25.0, 12)):
        cam = __import__("meteoros_gb300.scenes", fromlist=["look"]).look((0.0, 0.0, 2.0), 10.0, pitch, 45.0, w, h)
        tm = abi.time_init()
        tm.frame_count_mod16 = slot
        tm.time[1] = 3.5
        a, am, _ = oracle.render(vol, cam, cam, tm, abi.params_reference(), prev, w, h, 0)
        b, bm = pyref.frame(vol, cam, cam, tm, prev, w, h)
        for x, y, what in ((a, b, "rgba"), (am, bm, "mask")):
            na, nb = np.isnan(x), np.isnan(y)
            assert np.array_equal(na, nb), what
            assert np.array_equal(np.where(na, 0, x).view(np.uint32), np.where(nb, 0, y).view(np.uint32)), what
