"""The downstream passes on the GPU against the CPU oracle, through the C ABI
(GB300 only): god-ray radial blur (bit for bit: the same FP32 operations in
the same order, no transcendental functions) and tone map + dither (the
float values within 3e-7 relative, powf of libdevice vs the host's libm; the
RGBA8 image equal except where a value straddles a rounding boundary)."""
import numpy as np
import pytest

from meteoros_gb300 import abi, scenes
from tests.gpu_util import assert_bits_equal, to_dev
from tests.golden import make_golden as mg

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

LIGHT = (1.0, 1.0, 0.57, 1.0)


@pytest.fixture(scope="module")
def ctx(lib):
    from meteoros_gb300.renderer import Context

    c = Context(0)
    yield c
    c.close()


def gpu_godrays(ctx, cam, mask, img, in_place=False):
    inp = to_dev(img, torch)
    m = to_dev(mask, torch)
    out = inp if in_place else torch.full_like(inp, float("nan"))
    ctx.godrays(cam, LIGHT, m, inp, out)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_godrays_golden(ctx, oracle, golden):
    (cam,) = mg.ubos_from(golden["godray_ubo"], abi.CameraUBO)
    got = gpu_godrays(ctx, cam, golden["godray_mask"], golden["repro_f15"])
    assert_bits_equal(got, golden["godray_out"], "god rays vs golden")


@pytest.mark.parametrize("size", [(1, 1), (2, 3), (61, 35), (160, 90), (333, 127)])
def test_godrays_vs_oracle(ctx, oracle, size):
    w, h = size
    rng = np.random.default_rng(w * 7 + h)
    img = rng.random((h, w, 4), dtype=np.float32) * 3.0
    mask = rng.random((h, w), dtype=np.float32) * 1.25
    light = np.array(LIGHT, np.float32)
    for yaw, pitch in ((0.0, 0.0), (30.0, 25.0), (-50.0, 60.0), (10.0, -40.0)):
        cam = scenes.look((0.0, 0.0, 2.0), yaw, pitch, 45.0, w, h)
        want = oracle.godrays(cam, light, mask, img)
        assert_bits_equal(gpu_godrays(ctx, cam, mask, img), want, f"{size} yaw {yaw} pitch {pitch}")
        assert_bits_equal(gpu_godrays(ctx, cam, mask, img, in_place=True), want, f"{size} in place")


def test_godrays_sun_behind_leaves_image(ctx):
    """A camera above the static sun at (0, 1, 0): blendFactor < 0, no store."""
    w, h = 64, 36
    img = np.random.default_rng(1).random((h, w, 4), dtype=np.float32)
    mask = np.ones((h, w), np.float32)
    cam = scenes.look((0.0, 100.0, 0.0), 0.0, 10.0, 60.0, w, h)
    assert_bits_equal(gpu_godrays(ctx, cam, mask, img), img, "sun behind")


def test_godrays_1080p_vs_oracle(ctx, oracle):
    w, h = 1920, 1080
    rng = np.random.default_rng(3)
    img = rng.random((h, w, 4), dtype=np.float32) * 2.0
    mask = rng.random((h, w), dtype=np.float32)
    cam = scenes.look((0.0, 0.0, 2.0), 5.0, 12.0, 45.0, w, h)
    want = oracle.godrays(cam, np.array(LIGHT, np.float32), mask, img)
    assert_bits_equal(gpu_godrays(ctx, cam, mask, img), want, "1080p")


def gpu_tonemap(ctx, tm, img, fmt):
    inp = to_dev(img, torch)
    if fmt == abi.MT_LDR_RGBA8:
        out = torch.full((img.shape[0], img.shape[1], 4), 77, dtype=torch.uint8, device="cuda")
    else:
        out = torch.full((img.shape[0], img.shape[1], 4), float("nan"), dtype=torch.float32, device="cuda")
    ctx.tonemap(tm, inp, out, fmt)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def check_tonemap(ctx, oracle, tm, img, what):
    want4, want8 = oracle.tonemap(tm.time[1], img, fill8=77)
    got4 = gpu_tonemap(ctx, tm, img, abi.MT_LDR_RGBA32F)
    stored = ~np.isnan(want4[..., 3])
    assert np.array_equal(stored, ~np.isnan(got4[..., 3])), f"{what}: stored-pixel pattern"
    a, b = got4[stored], want4[stored]
    assert np.array_equal(np.isnan(a), np.isnan(b)), f"{what}: NaN pattern"
    ok = ~np.isnan(b)
    np.testing.assert_allclose(a[ok], b[ok], rtol=3e-7, atol=0, err_msg=what)
    got8 = gpu_tonemap(ctx, tm, img, abi.MT_LDR_RGBA8)
    assert (got8[~stored] == 77).all(), f"{what}: a pixel no fragment stores to was written"
    d = np.abs(got8.astype(np.int16) - want8.astype(np.int16))
    assert d.max() <= 1, f"{what}: RGBA8 differs by {d.max()}"
    assert (d > 0).mean() < 1e-3, f"{what}: {int((d > 0).sum())} RGBA8 values differ"


def test_tonemap_golden(ctx, oracle, golden):
    (tm,) = mg.ubos_from(golden["tonemap_ubo"], abi.TimeUBO)
    got4 = gpu_tonemap(ctx, tm, golden["godray_out"], abi.MT_LDR_RGBA32F)
    ref = golden["tonemap_out"]
    assert np.array_equal(np.isnan(got4), np.isnan(ref))
    ok = ~np.isnan(ref)
    np.testing.assert_allclose(got4[ok], ref[ok], rtol=3e-7, atol=0)


@pytest.mark.parametrize("size", [(1, 1), (3, 2), (59, 37), (1920, 1080)])
def test_tonemap_vs_oracle(ctx, oracle, size):
    w, h = size
    img = (np.random.default_rng(w + h).random((h, w, 4), dtype=np.float32) * 20.0).astype(np.float32)
    img[0, 0] = 0.0
    for t in (0.0, 1.5, 977.25):
        tm = abi.time_init()
        tm.time[1] = t
        check_tonemap(ctx, oracle, tm, img, f"{size} t={t}")


def test_post_argument_errors(ctx):
    img = torch.zeros((8, 8, 4), dtype=torch.float32, device="cuda")
    mask = torch.zeros((8, 8), dtype=torch.float32, device="cuda")
    cam = scenes.look((0.0, 0.0, 2.0), 0.0, 0.0, 45.0, 8, 8)
    with pytest.raises(abi.MeteorosError):
        ctx.godrays(cam, LIGHT, None, img, img)
    with pytest.raises(abi.MeteorosError):
        ctx.tonemap(abi.time_init(), img, img, abi.MT_LDR_RGBA32F)  # out must differ from in
    out = torch.zeros((8, 8, 4), dtype=torch.uint8, device="cuda")
    with pytest.raises(abi.MeteorosError):
        ctx.tonemap(abi.time_init(), img, out, 7)
