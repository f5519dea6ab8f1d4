"""REF-preset frames on volumes built from the reference's shipped noise
assets (Sky.cpp:25-58), against frames of the reference's own shader source
(tests/golden/ref_assets.npz, made by tests/golden/make_golden.py).

The fixture holds the TGA bytes of all 32 HighFrequency slices and of
LowFrequency slices 1-2 (repeated through the 128-slice base stack: the
whole stack is 8.4 MB of noise), and curlNoise.png as the reference's
stb_image decodes it.  On the GPU the TGA files are decoded on the device
(mt_decode_tga_volume), the curl map uploaded, and the REF checkerboard
frames rendered through the C ABI; on the CPU the oracle restatement does the
same.  The golden frames come from the reference's shaders compiled as C++."""
import ctypes as C
import hashlib

import numpy as np
import pytest

from meteoros_gb300 import abi
from tests.golden import make_golden as mg
from tests.gpu_util import assert_bits_equal, assert_hdr_close, to_dev

ASSETS = mg.OUT_ASSETS


@pytest.fixture(scope="module")
def fixture():
    if not ASSETS.exists():
        pytest.fail(f"{ASSETS} is missing; run tests/golden/make_golden.py")
    d = dict(np.load(ASSETS))
    low = mg.unpack_files(d["low_tga"], d["low_offsets"])
    high = mg.unpack_files(d["high_tga"], d["high_offsets"])
    base_files = [low[i] for i in mg.asset_stack_order()]
    return d, base_files, high


def views(d):
    for k, _ in enumerate(mg.ASSET_VIEWS):
        cam, old, tm = mg.ubos_from(d[f"view{k}_ubo"], abi.CameraUBO, abi.CameraUBO, abi.TimeUBO)
        yield k, cam, old, tm, d[f"view{k}_rgba"], d[f"view{k}_mask"]


def test_fixture_frames_have_clouds(fixture):
    d, _, _ = fixture
    for k, *_, rgba, mask in views(d):
        marched = ~np.isnan(mask)
        assert marched.sum() > 0 and (mask[marched] > 0).any(), f"view {k}: no god-ray signal"


def test_oracle_on_shipped_assets_equals_reference_frames(oracle, fixture):
    """CPU: the restatement's TGA decoder and renderer give the reference
    shaders' frames bit for bit (pins the fixture itself)."""
    d, base_files, high = fixture
    base = np.stack([oracle.decode_tga(f) for f in base_files])
    detail = np.stack([oracle.decode_tga(f) for f in high])
    assert hashlib.sha256(base.tobytes()).digest() == d["base_sha256"].tobytes()
    assert hashlib.sha256(detail.tobytes()).digest() == d["detail_sha256"].tobytes()
    weather = np.zeros((abi.MT_WEATHER_N, abi.MT_WEATHER_N, 4), np.uint8)
    vol = oracle.Volumes(base, detail, d["curl_rgba8"], weather)
    for k, cam, old, tm, rgba, mask in views(d):
        a, am, _ = oracle.render(vol, cam, old, tm, abi.params_reference(), mg.asset_prev(k), mg.ASSET_W, mg.ASSET_H, 0)
        assert_bits_equal(a, rgba, f"view {k} rgba")
        assert_bits_equal(am, mask, f"view {k} mask")


@pytest.mark.gpu
def test_gpu_on_shipped_assets_matches_reference_frames(lib, fixture):
    """GPU: TGA slices decoded on the device equal stb_image's volumes (by
    hash), and the REF checkerboard frames rendered on them match the
    reference shaders' frames: reprojected pixels and god-ray values bit for
    bit, colour within the HDR bar."""
    torch = pytest.importorskip("torch")
    from meteoros_gb300.renderer import Context

    d, base_files, high = fixture
    with Context(0) as ctx:
        for volume, files in ((abi.MT_VOLUME_BASE, base_files), (abi.MT_VOLUME_DETAIL, high)):
            arr = (C.c_void_p * len(files))(*[C.cast(C.c_char_p(f), C.c_void_p) for f in files])
            sizes = (C.c_size_t * len(files))(*[len(f) for f in files])
            st = ctx.lib.mt_decode_tga_volume(ctx.handle, volume, arr, sizes, len(files), None)
            assert st == abi.MT_OK, ctx.lib.mt_last_error(ctx.handle).decode()
        weather = np.zeros((abi.MT_WEATHER_N, abi.MT_WEATHER_N, 4), np.uint8)
        ctx.upload_volumes(None, None, d["curl_rgba8"], weather)
        got = ctx.download_volumes()
        assert hashlib.sha256(got["base"].tobytes()).digest() == d["base_sha256"].tobytes()
        assert hashlib.sha256(got["detail"].tobytes()).digest() == d["detail_sha256"].tobytes()
        for k, cam, old, tm, rgba, mask in views(d):
            w, h = mg.ASSET_W, mg.ASSET_H
            cur = torch.full((h, w, 4), float("nan"), dtype=torch.float32, device="cuda")
            gmask = torch.full((h, w), float("nan"), dtype=torch.float32, device="cuda")
            ctx.render(cam, old, tm, abi.params_reference(), to_dev(mg.asset_prev(k), torch), cur, gmask,
                       abi.MT_RENDER_CHECKERBOARD)
            g, gm = cur.cpu().numpy(), gmask.cpu().numpy()
            m = ~np.isnan(mask)
            assert_bits_equal(g[~m], rgba[~m], f"view {k} reprojected")
            assert_hdr_close(g, rgba, f"view {k} rgba")
            assert_bits_equal(gm, mask, f"view {k} god-ray mask")
