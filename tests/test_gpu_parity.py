"""CUDA kernels vs the oracle, through the C ABI (GB300 only)."""
import ctypes as C

import numpy as np
import pytest

from meteoros_gb300 import abi, scenes
from tests.golden import make_golden as mg
from tests.gpu_util import assert_bits_equal, assert_hdr_close, to_dev

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def ctx(lib):
    from meteoros_gb300.renderer import Context

    c = Context(0)
    c.generate_volumes(7)
    torch.cuda.synchronize()
    yield c
    c.close()


def gpu_render(ctx, cam, old, tm, params, prev, w, h, flags):
    cur = torch.full((h, w, 4), float("nan"), dtype=torch.float32, device="cuda")
    mask = torch.full((h, w), float("nan"), dtype=torch.float32, device="cuda")
    prev_d = None if prev is None else to_dev(prev.astype(np.float32), torch)
    ctx.render(cam, old, tm, params, prev_d, cur, mask, flags | abi.MT_RENDER_COUNT)
    st = ctx.stats(reset=True)
    return cur.cpu().numpy(), mask.cpu().numpy(), st


def marched(mask):
    return ~np.isnan(mask)


def check_frame(oracle, vol, ctx, cam, old, tm, params, prev, w, h, flags, what):
    a, am, cnt = oracle.render(vol, cam, old, tm, params, prev, w, h, flags)
    g, gm, st = gpu_render(ctx, cam, old, tm, params, prev, w, h, flags)
    m = marched(am)
    # reprojected pixels: no transcendental is involved, so bit-exact
    if not (flags & abi.MT_RENDER_FULL):
        assert_bits_equal(g[~m], a[~m], what + " reprojected")
    assert_hdr_close(g, a, what + " rgba")
    assert_hdr_close(gm, am, what + " mask")
    # identical control flow: the executed-sample counters agree exactly
    assert (st.primary_samples, st.light_samples, st.marched_rays) == (int(cnt[0]), int(cnt[1]), int(cnt[2]))
    assert st.pixels == w * h if not (flags & abi.MT_RENDER_FULL) else st.pixels == int(cnt[3])
    return g, gm


def test_generator_bit_exact(ctx, volumes_seed7):
    got = ctx.download_volumes()
    for k in ("base", "detail", "curl", "weather"):
        assert np.array_equal(got[k], volumes_seed7[k]), k
    for storage, suffix in ((abi.MT_STORAGE_F16, "_h16"), (abi.MT_STORAGE_BF16, "_b16")):
        got16 = ctx.download_volumes_16(storage)
        for k in ("base", "detail", "curl", "weather"):
            assert np.array_equal(got16[k], volumes_seed7[k + suffix]), k + suffix


def test_generated_weather_slots(ctx, oracle):
    ctx.generate_weather(3, 1234)
    got = ctx.download_volumes(weather_slot=3)["weather"]
    want = oracle.generate_volumes(1234)["weather"]
    assert np.array_equal(got, want)


@pytest.fixture(scope="module")
def ref_ctx(lib, volumes_seed7):
    """A context holding the golden (sparse-cloud) volumes."""
    from meteoros_gb300.renderer import Context

    c = Context(0)
    vol = mg.golden_volumes(volumes_seed7)
    c.upload_volumes(vol.base, vol.detail, vol.curl, vol.weather)
    got = c.download_volumes()
    assert np.array_equal(got["base"], vol.base) and np.array_equal(got["weather"], vol.weather)
    yield c, vol
    c.close()


def test_reference_sequence_each_frame(ref_ctx, oracle, golden):
    """16 checkerboard frames, REF constants: each frame from the same previous image."""
    ctx, vol = ref_ctx
    params = abi.params_reference()
    prev = mg.initial_prev()
    for f, (cam, old, tm) in enumerate(mg.golden_sequence(golden)):
        a, _, _ = oracle.render(vol, cam, old, tm, params, prev, mg.SEQ_W, mg.SEQ_H, 0)
        check_frame(oracle, vol, ctx, cam, old, tm, params, prev, mg.SEQ_W, mg.SEQ_H, 0, f"frame {f}")
        prev = a


def test_reference_sequence_against_golden(ref_ctx, golden):
    """The GPU's own 16-frame chain against the reference shaders' golden frames."""
    ctx, vol = ref_ctx
    params = abi.params_reference()
    prev = to_dev(mg.initial_prev(), torch)
    for f, (cam, old, tm) in enumerate(mg.golden_sequence(golden)):
        cur = torch.zeros((mg.SEQ_H, mg.SEQ_W, 4), dtype=torch.float32, device="cuda")
        mask = torch.full((mg.SEQ_H, mg.SEQ_W), float("nan"), dtype=torch.float32, device="cuda")
        ctx.render(cam, old, tm, params, prev, cur, mask, 0)
        if f in mg.KEEP:
            assert_hdr_close(cur.cpu().numpy(), golden[f"repro_f{f}"], f"golden frame {f}")
            assert_hdr_close(mask.cpu().numpy(), golden[f"mask_f{f}"], f"golden mask {f}")
        prev = cur


def test_dispatch_quirk_against_golden(ref_ctx, golden):
    ctx, vol = ref_ctx
    cam, tm = mg.ubos_from(golden["quirk_ubo"], abi.CameraUBO, abi.TimeUBO)
    prev = np.random.default_rng(3).random((mg.QUIRK_H, mg.QUIRK_W, 4), dtype=np.float32)
    g, gm, _ = gpu_render(ctx, cam, cam, tm, abi.params_reference(), prev, mg.QUIRK_W, mg.QUIRK_H, 0)
    assert_hdr_close(g, golden["quirk_rgba"], "quirk")
    assert_hdr_close(gm, golden["quirk_mask"], "quirk mask")
    assert np.isnan(gm[:, 128:]).all()


def test_txaa_bit_exact(ctx, oracle, golden):
    _, _, _, cur, hist = mg.txaa_inputs()
    cam, old, tm = mg.ubos_from(golden["txaa_ubo"], abi.CameraUBO, abi.CameraUBO, abi.TimeUBO)
    for params in (abi.params_reference(), abi.params_config()):
        want = oracle.txaa(cam, old, tm, params, cur, hist)
        out = torch.zeros_like(to_dev(cur, torch))
        ctx.txaa(cam, old, tm, params, to_dev(cur, torch), to_dev(hist, torch), out)
        assert_bits_equal(out.cpu().numpy(), want, "txaa")
    out = torch.zeros_like(to_dev(cur, torch))
    ctx.txaa(cam, old, tm, abi.params_reference(), to_dev(cur, torch), to_dev(hist, torch), out)
    assert_bits_equal(out.cpu().numpy(), golden["txaa_out"], "txaa golden")


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_config_full_frame_small(ctx, oracle, volumes_seed7, seed):
    vol = oracle.Volumes(volumes_seed7["base"], volumes_seed7["detail"], volumes_seed7["curl"],
                         volumes_seed7["weather"])
    w, h = 192, 108
    cam, tm, params, _ = scenes.config_view(seed, w, h)
    check_frame(oracle, vol, ctx, cam, cam, tm, params, None, w, h, abi.MT_RENDER_FULL, f"config seed {seed}")


def test_config0_full_size(ctx, oracle, volumes_seed7):
    """Config 0 at its own size: 960x540, every pixel marched, 128 steps."""
    vol = oracle.Volumes(volumes_seed7["base"], volumes_seed7["detail"], volumes_seed7["curl"],
                         volumes_seed7["weather"])
    w, h = 960, 540
    cam, tm, params, _ = scenes.config_view(11, w, h)
    check_frame(oracle, vol, ctx, cam, cam, tm, params, None, w, h, abi.MT_RENDER_FULL, "config0 960x540")


def test_config1_frame_full_size(ctx, oracle, volumes_seed7):
    """One reprojected 1920x1080 frame of config 1 (checkerboard + TXAA)."""
    vol = oracle.Volumes(volumes_seed7["base"], volumes_seed7["detail"], volumes_seed7["curl"],
                         volumes_seed7["weather"])
    w, h = 1920, 1080
    seq = scenes.config_sequence(5, w, h, frames=3)
    prev = np.random.default_rng(9).random((h, w, 4), dtype=np.float32)
    cam, old, tm, params = seq[2]
    g, _ = check_frame(oracle, vol, ctx, cam, old, tm, params, prev, w, h, 0, "config1 1080p")
    hist = np.random.default_rng(10).random((h, w, 4), dtype=np.float32)
    want = oracle.txaa(cam, old, tm, params, g, hist)
    out = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    ctx.txaa(cam, old, tm, params, to_dev(g, torch), to_dev(hist, torch), out)
    assert_bits_equal(out.cpu().numpy(), want, "config1 txaa")


@pytest.mark.parametrize("size", [(1, 1), (3, 5), (7, 3), (17, 9), (130, 18)])
def test_edge_sizes(ctx, oracle, volumes_seed7, size):
    vol = oracle.Volumes(volumes_seed7["base"], volumes_seed7["detail"], volumes_seed7["curl"],
                         volumes_seed7["weather"])
    w, h = size
    cam, tm, params, _ = scenes.config_view(3, w, h)
    prev = np.random.default_rng(w * h).random((h, w, 4), dtype=np.float32)
    for f in (0, 5, 15):
        tm.frame_count_mod16 = f
        check_frame(oracle, vol, ctx, cam, cam, tm, params, prev, w, h, 0, f"{w}x{h} slot {f}")
    check_frame(oracle, vol, ctx, cam, cam, tm, params, None, w, h, abi.MT_RENDER_FULL, f"{w}x{h} full")


def test_deterministic(ctx):
    w, h = 256, 144
    cam, tm, params, _ = scenes.config_view(4, w, h)
    outs = []
    for _ in range(2):
        cur = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
        ctx.render(cam, cam, tm, params, None, cur, None, abi.MT_RENDER_FULL)
        outs.append(cur.cpu().numpy())
    assert_bits_equal(outs[0], outs[1], "repeat")


def test_argument_errors(ctx, lib):
    w, h = 16, 16
    cam, tm, params, _ = scenes.config_view(0, w, h)
    a = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    b = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    raw = torch.zeros(h * w * 4 + 1, dtype=torch.float32, device="cuda")

    def status(fn):
        try:
            fn()
        except abi.MeteorosError as e:
            return e.status
        return abi.MT_OK

    assert status(lambda: ctx.render(cam, cam, tm, params, None, a, None, 0)) == abi.MT_ERR_INVALID_ARG
    assert status(lambda: ctx.render(cam, cam, tm, params, a, a, None, 0)) == abi.MT_ERR_INVALID_ARG
    misaligned = raw.data_ptr() + 4
    st = ctx.lib.mt_render(ctx.handle, C.byref(cam), C.byref(cam), C.byref(tm), C.byref(params), b.data_ptr(),
                           misaligned, None, w, h, 0, None)
    assert st == abi.MT_ERR_INVALID_ARG
    bad_tm = abi.time_init()
    bad_tm.frame_count_mod16 = 16
    assert status(lambda: ctx.render(cam, cam, bad_tm, params, b, a, None, 0)) == abi.MT_ERR_INVALID_ARG
    bad = abi.params_config()
    bad.weather_slot = 77  # never generated
    assert status(lambda: ctx.render(cam, cam, tm, bad, b, a, None, 0)) == abi.MT_ERR_NO_VOLUMES
    bad = abi.params_config()
    bad.steps_max = 0
    assert status(lambda: ctx.render(cam, cam, tm, bad, b, a, None, 0)) == abi.MT_ERR_INVALID_ARG
    assert status(lambda: ctx.txaa(cam, cam, tm, params, a, b, a)) == abi.MT_ERR_INVALID_ARG
    assert status(lambda: ctx.render(cam, cam, tm, params, b, a, None, 0x80)) == abi.MT_ERR_INVALID_ARG
    assert ctx.lib.mt_last_error(ctx.handle)
    from meteoros_gb300.renderer import Context

    empty = Context(0)
    assert status(lambda: empty.render(cam, cam, tm, params, b, a, None, 0)) == abi.MT_ERR_NO_VOLUMES
    empty.close()
    torch.cuda.synchronize()
