"""The oracle (CPU restatement) against the golden vectors produced by the
reference's own shader source, and -- where the reference tree is present --
against that source directly.  CPU only."""
import numpy as np
import pytest

from meteoros_gb300 import abi
from tests.golden import make_golden as mg


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def assert_bit_exact(a, b, what):
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    assert a.shape == b.shape, what
    nan_a, nan_b = np.isnan(a), np.isnan(b)
    assert np.array_equal(nan_a, nan_b), f"{what}: written-pixel pattern differs"
    diff = bits(np.where(nan_a, 0, a)) != bits(np.where(nan_b, 0, b))
    assert not diff.any(), f"{what}: {int(diff.sum())} values differ, max {np.nanmax(np.abs(a - b))}"


def test_sequence_matches_golden(oracle, volumes_seed7, golden, lib):
    vol = mg.golden_volumes(volumes_seed7)
    params = abi.params_reference()
    prev = mg.initial_prev()
    for f, (cam, old, tm) in enumerate(mg.golden_sequence(golden)):
        rgba, mask, _ = oracle.render(vol, cam, old, tm, params, prev, mg.SEQ_W, mg.SEQ_H,
                                      abi.MT_RENDER_CHECKERBOARD)
        if f in mg.KEEP:
            assert_bit_exact(rgba, golden[f"repro_f{f}"], f"frame {f} rgba")
            assert_bit_exact(mask, golden[f"mask_f{f}"], f"frame {f} mask")
        prev = rgba


def test_dispatch_quirk_matches_golden(oracle, volumes_seed7, golden, lib):
    vol = mg.golden_volumes(volumes_seed7)
    cam, tm = mg.ubos_from(golden["quirk_ubo"], abi.CameraUBO, abi.TimeUBO)
    prev = np.random.default_rng(3).random((mg.QUIRK_H, mg.QUIRK_W, 4), dtype=np.float32)
    rgba, mask, _ = oracle.render(vol, cam, cam, tm, abi.params_reference(), prev, mg.QUIRK_W, mg.QUIRK_H, 0)
    assert_bit_exact(rgba, golden["quirk_rgba"], "quirk rgba")
    assert_bit_exact(mask, golden["quirk_mask"], "quirk mask")
    # columns 128 and 129 are never marched by the reference's dispatch
    assert np.isnan(mask[:, 128:]).all()


def test_txaa_matches_golden(oracle, golden, lib):
    _, _, _, cur, hist = mg.txaa_inputs()
    cam, old, tm = mg.ubos_from(golden["txaa_ubo"], abi.CameraUBO, abi.CameraUBO, abi.TimeUBO)
    out = oracle.txaa(cam, old, tm, abi.params_reference(), cur, hist)
    assert_bit_exact(out, golden["txaa_out"], "txaa")


def test_wang_hash_matches_reference(oracle, golden):
    uvs = golden["wang_uvs"]
    h = np.array([oracle.lib().orc_wang(int(a), int(b), int(c)) for a, b, c in uvs], np.uint32)
    # WangHashNoise returns float(seed) * (1.0 / 4294967296.0) in float32
    val = h.astype(np.float32) * np.float32(1.0 / 4294967296.0)
    assert_bit_exact(val, golden["wang_val"], "WangHashNoise")


def test_uniforms_rebuild_identically_here(golden, lib):
    """On the host that made the goldens the uniform builders reproduce the
    stored bytes (on another host libm may differ by an ulp, hence the bytes)."""
    for f, (cam, old, tm) in enumerate(mg.sequence_inputs()):
        same = np.array_equal(mg.ubo_bytes(cam, old, tm), golden[f"seq_ubo_f{f}"])
        if not same:
            pytest.skip("uniforms differ on this host (libm); tests use the stored bytes")


def test_generator_matches_golden_hashes(volumes_seed7, golden):
    import hashlib

    for k in ("base", "detail", "curl", "weather"):
        for suffix in ("", "_h16", "_b16"):
            digest = hashlib.sha256(np.ascontiguousarray(volumes_seed7[k + suffix]).tobytes()).digest()
            assert digest == golden[f"gen_sha256_{k}{suffix}"].tobytes(), f"{k}{suffix}"


# ---- directly against the reference's shader source (needs the reference tree) ----

@pytest.fixture(scope="module")
def pyref():
    from oracle import pyref

    if not pyref.available():
        pytest.skip("reference tree not present")
    return pyref


@pytest.mark.parametrize("size", [(48, 28), (67, 41)])
def test_every_frame_slot_matches_reference_source(oracle, pyref, volumes_seed7, lib, size):
    w, h = size
    vol = mg.golden_volumes(volumes_seed7)
    rng = np.random.default_rng(w)
    prev = rng.random((h, w, 4), dtype=np.float32) * 3.0
    old = mg.scenes.look((0.0, 0.0, 2.0), 3.0, 14.0, 45.0, w, h)
    cam = mg.scenes.look((0.0, 0.0, 2.0), 4.0, 15.0, 45.0, w, h)
    for f in range(16):
        tm = abi.time_init()
        tm.frame_count_mod16 = f
        tm.time[1] = 1.7 * f
        a, am, _ = oracle.render(vol, cam, old, tm, abi.params_reference(), prev, w, h, 0)
        b, bm = pyref.frame(vol, cam, old, tm, prev, w, h)
        assert_bit_exact(a, b, f"frame slot {f} rgba")
        assert_bit_exact(am, bm, f"frame slot {f} mask")


def test_txaa_matches_reference_source(oracle, pyref, lib):
    rng = np.random.default_rng(11)
    w, h = 57, 33
    cur = rng.random((h, w, 4), dtype=np.float32) * 5.0
    hist = rng.random((h, w, 4), dtype=np.float32) * 5.0
    old = mg.scenes.look((0.0, 0.0, 2.0), 0.0, 10.0, 45.0, w, h)
    cam = mg.scenes.look((0.0, 0.0, 2.0), 2.0, 11.0, 45.0, w, h)
    for f in (0, 5, 13):
        tm = abi.time_init()
        tm.frame_count_mod16 = f
        a = oracle.txaa(cam, old, tm, abi.params_reference(), cur, hist)
        b = pyref.txaa(cam, old, tm, cur, hist)
        assert_bit_exact(a, b, f"txaa slot {f}")


# ---- downstream passes: god-ray radial blur and tone map ----

def test_godrays_match_golden(oracle, golden, lib):
    (cam,) = mg.ubos_from(golden["godray_ubo"], abi.CameraUBO)
    out = oracle.godrays(cam, mg.GODRAY_LIGHT, golden["godray_mask"], golden["repro_f15"])
    assert_bit_exact(out, golden["godray_out"], "god rays")
    assert np.abs(out - golden["repro_f15"]).max() > 0.1  # the blur adds light


def test_tonemap_matches_golden(oracle, golden, lib):
    (tm,) = mg.ubos_from(golden["tonemap_ubo"], abi.TimeUBO)
    out4, out8 = oracle.tonemap(tm.time[1], golden["godray_out"])
    ref = golden["tonemap_out"]
    assert np.array_equal(np.isnan(out4), np.isnan(ref)), "stored-pixel pattern differs"
    # powf of the host's libm: equal where the goldens were made, within 2 ulp elsewhere
    ok = ~np.isnan(ref)
    np.testing.assert_allclose(out4[ok], ref[ok], rtol=3e-7, atol=0)
    # the RGBA8 image is the UNORM conversion of the stored values
    conv = np.rint(np.clip(np.nan_to_num(out4, nan=0.0), 0.0, 1.0) * np.float32(255.0)).astype(np.uint8)
    stored = ~np.isnan(out4[..., 3])
    assert np.array_equal(out8[stored], conv[stored])


def test_godray_and_tonemap_fragment_mapping(oracle):
    """pixelPos = clamp(round(dim * in_uv)): column and row 0 receive no store,
    the last column and row receive two (the later fragment wins)."""
    w, h = 33, 17
    img = np.random.default_rng(5).random((h, w, 4), dtype=np.float32)
    out4, _ = oracle.tonemap(0.0, img)
    stored = ~np.isnan(out4[..., 3])
    assert not stored[0, :].any() and not stored[:, 0].any()
    assert stored[-1, -1]


def test_godrays_match_reference_source(oracle, pyref, lib):
    rng = np.random.default_rng(21)
    w, h = 61, 35
    img = rng.random((h, w, 4), dtype=np.float32) * 3.0
    mask = rng.random((h, w), dtype=np.float32) * 1.25
    light = np.array([1.0, 1.0, 0.57, 1.0], np.float32)
    for yaw, pitch in ((0.0, 0.0), (30.0, 25.0), (-50.0, 60.0), (10.0, -40.0), (180.0, 10.0)):
        cam = mg.scenes.look((0.0, 0.0, 2.0), yaw, pitch, 45.0, w, h)
        a = oracle.godrays(cam, light, mask, img)
        b = pyref.godrays(cam, light, mask, img)
        assert_bit_exact(a, b, f"god rays yaw {yaw} pitch {pitch}")


def test_tonemap_matches_reference_source(oracle, pyref, lib):
    rng = np.random.default_rng(22)
    w, h = 59, 37
    img = (rng.random((h, w, 4), dtype=np.float32) * 20.0).astype(np.float32)
    img[3, 4] = 0.0  # black: the curve's zero crossing
    for t in (0.0, 1.5, 977.25):
        tm = abi.time_init()
        tm.time[1] = t
        a, _ = oracle.tonemap(t, img)
        b = pyref.tonemap(tm, img)
        assert_bit_exact(a, b, f"tone map t={t}")


# ---- the CONFIG-only terms, against the reference's own functions ----

def _grid_heights():
    """Relative heights around every remap breakpoint of the gradient (0, 0.01,
    0.1, 0.2, 0.25, 0.3, 0.6, 0.65, 0.95, 1) plus a dense sweep and out-of-range
    values (the function clamps them)."""
    h = [np.linspace(-0.5, 1.5, 4001, dtype=np.float32)]
    for b in (0.0, 0.01, 0.1, 0.2, 0.25, 0.3, 0.6, 0.65, 0.95, 1.0):
        c = np.float32(b)
        h.append(np.array([np.nextafter(c, np.float32(-1)), c, np.nextafter(c, np.float32(2))], np.float32))
    h.append(np.random.default_rng(31).random(20000, dtype=np.float32))
    return np.concatenate(h)


def test_height_gradient_matches_reference_source(oracle, pyref):
    """getDensityHeightGradientForPoint (cloudRayMarch.comp:475-487) is dead
    code in the reference; the CONFIG presets switch it on.  The oracle's
    restatement equals the shader's own function bit for bit over heights x
    cloud types (the weather map's B channel: every 8-bit value, as the
    sampler sees it after filtering, and the configs' 0, 0.5, 1)."""
    L = oracle.lib()
    R = pyref.lib()
    heights = _grid_heights()
    types = np.concatenate([np.arange(256, dtype=np.float32) / np.float32(255.0),
                            np.random.default_rng(32).random(64, dtype=np.float32),
                            np.array([0.0, 0.5, 1.0, -0.25, 1.25], np.float32)])
    mism = 0
    for t in types:
        a = np.array([L.orc_height_gradient(float(h), float(t)) for h in heights[::7]], np.float32)
        b = np.array([R.ref_height_gradient(float(h), float(t)) for h in heights[::7]], np.float32)
        mism += int((a.view(np.uint32) != b.view(np.uint32)).sum())
    for t in (0.0, 0.5, 1.0):
        a = np.array([L.orc_height_gradient(float(h), t) for h in heights], np.float32)
        b = np.array([R.ref_height_gradient(float(h), t) for h in heights], np.float32)
        mism += int((a.view(np.uint32) != b.view(np.uint32)).sum())
        assert (b > 0).any()  # the gradient is not trivially zero on this grid
    assert mism == 0, f"{mism} height-gradient values differ from the reference's function"


def test_remaps_match_reference_source(oracle, pyref):
    """remap / remapClamped / remapClampedBeforeAndAfter (cloudRayMarch.comp:153-169)
    on the CONFIG preset's inputs: the base-shape remap (lo = fbm - 0.9), the
    weather coverage remap (lo = 1 - R for every weather byte R) and the
    erosion remap (lo = modifier * 0.005), plus random arguments."""
    L = oracle.lib()
    R = pyref.lib()
    rng = np.random.default_rng(33)
    vals = np.concatenate([rng.random(400, dtype=np.float32) * np.float32(1.4) - np.float32(0.2),
                           np.array([0.0, 1.0, -0.0, 1e-30, 0.5], np.float32)])
    los = np.concatenate([np.float32(1.0) - np.arange(256, dtype=np.float32) / np.float32(255.0),  # coverage
                          rng.random(32, dtype=np.float32) - np.float32(0.9),  # base shape
                          rng.random(32, dtype=np.float32) * np.float32(0.005)])  # erosion
    cases = [(v, lo, 1.0, 0.0, 1.0) for lo in los for v in vals[::3]]
    cases += [tuple(float(x) for x in rng.normal(size=5).astype(np.float32)) for _ in range(3000)]
    for name in ("remap", "remap_clamped", "remap_clamped_ba"):
        fa, fb = getattr(L, "orc_" + name), getattr(R, "ref_" + name)
        a = np.array([fa(*map(float, c)) for c in cases], np.float32)
        b = np.array([fb(*map(float, c)) for c in cases], np.float32)
        same = (a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))
        assert same.all(), f"{name}: {(~same).sum()} of {len(cases)} differ"
