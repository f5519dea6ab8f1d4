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
    # the god-ray mask is a function of the accumulated density alone (no
    # transcendental on its path), so it is bit-exact: this pins the density
    # arithmetic (samplers, remaps, erosion) operation for operation
    assert_bits_equal(gm, am, what + " mask")
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


def test_txaa_signed_and_special_values_bit_exact(ctx, oracle, golden):
    """Blocks whose neighbourhoods hold negative values, -0, NaN or infinity
    take the compare-select path of the resolve, the others the min/max path:
    both equal the oracle bit for bit."""
    _, _, _, cur, hist = mg.txaa_inputs()
    cam, old, tm = mg.ubos_from(golden["txaa_ubo"], abi.CameraUBO, abi.CameraUBO, abi.TimeUBO)
    cur = cur.copy()
    h, w = cur.shape[:2]
    rng = np.random.default_rng(17)
    n = max(8, (h * w) // 500)
    ys, xs = rng.integers(0, h, n), rng.integers(0, w, n)
    special = np.array([-0.0, -1.5, -1e-30, np.inf, np.nan, 0.0], np.float32)
    cur[ys, xs, rng.integers(0, 4, n)] = special[rng.integers(0, len(special), n)]
    cur[: h // 3, : w // 3] *= -1.0  # a negative region
    for params in (abi.params_reference(), abi.params_config()):
        want = oracle.txaa(cam, old, tm, params, cur, hist)
        out = torch.zeros_like(to_dev(cur, torch))
        ctx.txaa(cam, old, tm, params, to_dev(cur, torch), to_dev(hist, torch), out)
        assert_bits_equal(out.cpu().numpy(), want, "txaa with special values")


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


@pytest.mark.parametrize("size", [(abi.MT_MAX_DIM, 8), (8, abi.MT_MAX_DIM)])
def test_maximum_dimensions(ctx, oracle, volumes_seed7, size):
    """The largest width and height the ABI accepts (index arithmetic at the
    limit); one above is rejected."""
    vol = oracle.Volumes(volumes_seed7["base"], volumes_seed7["detail"], volumes_seed7["curl"],
                         volumes_seed7["weather"])
    w, h = size
    cam, tm, params, _ = scenes.config_view(9, w, h)
    prev = np.random.default_rng(5).random((h, w, 4), dtype=np.float32)
    tm.frame_count_mod16 = 6
    check_frame(oracle, vol, ctx, cam, cam, tm, params, prev, w, h, 0, f"{w}x{h} checkerboard")
    check_frame(oracle, vol, ctx, cam, cam, tm, params, None, w, h, abi.MT_RENDER_FULL, f"{w}x{h} full")
    big = torch.zeros((h, w + 1, 4) if w > h else (h + 1, w, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(abi.MeteorosError) as e:
        ctx.render(cam, cam, tm, params, None, big, None, abi.MT_RENDER_FULL)
    assert e.value.status == abi.MT_ERR_INVALID_ARG


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


@pytest.mark.parametrize("block", [32, 128])
def test_march_block_sizes_give_identical_frames(ctx, block):
    """The raymarch's CTA size (32, 128 or the default 256 threads) changes
    neither bits nor counters."""
    w, h = 300, 170
    cam, tm, params, _ = scenes.config_view(23, w, h)
    prev = to_dev(np.random.default_rng(4).random((h, w, 4), dtype=np.float32), torch)
    outs = []
    for b in (0, block):
        ctx.set_tuning(march_block=b)
        for flags in (abi.MT_RENDER_FULL, abi.MT_RENDER_CHECKERBOARD):
            cur = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
            mask = torch.full((h, w), float("nan"), dtype=torch.float32, device="cuda")
            ctx.render(cam, cam, tm, params, prev, cur, mask, flags | abi.MT_RENDER_COUNT)
            st = ctx.stats(reset=True)
            outs.append((cur.cpu().numpy(), mask.cpu().numpy(),
                         (st.primary_samples, st.light_samples, st.marched_rays, st.pixels)))
    ctx.set_tuning(march_block=0)
    for a, b in zip(outs[:2], outs[2:]):
        assert_bits_equal(a[0], b[0], f"block {block} rgba")
        assert_bits_equal(a[1], b[1], f"block {block} mask")
        assert a[2] == b[2]


@pytest.mark.parametrize("lanes", [1, 4, 16])
def test_march_lane_counts_give_identical_frames(ctx, lanes):
    """The step-parallel march is exact: any lane count gives the same bits and counters."""
    w, h = 320, 180
    cam, tm, params, _ = scenes.config_view(21, w, h)
    prev = to_dev(np.random.default_rng(1).random((h, w, 4), dtype=np.float32), torch)
    outs = []
    for g in (8, lanes):
        ctx.set_tuning(march_lanes=g)
        for flags in (abi.MT_RENDER_FULL, abi.MT_RENDER_CHECKERBOARD):
            cur = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
            mask = torch.full((h, w), float("nan"), dtype=torch.float32, device="cuda")
            ctx.render(cam, cam, tm, params, prev, cur, mask, flags | abi.MT_RENDER_COUNT)
            st = ctx.stats(reset=True)
            outs.append((cur.cpu().numpy(), mask.cpu().numpy(),
                         (st.primary_samples, st.light_samples, st.marched_rays, st.pixels)))
    ctx.set_tuning(march_lanes=0)
    for a, b in zip(outs[:2], outs[2:]):
        assert_bits_equal(a[0], b[0], f"lanes {lanes} rgba")
        assert_bits_equal(a[1], b[1], f"lanes {lanes} mask")
        assert a[2] == b[2]


@pytest.mark.parametrize("pitch", [-20.0, 0.0, 12.0, 45.0, 80.0])
def test_row_dispatch_order_gives_identical_frames(ctx, pitch):
    """Bottom-to-top ray-row order and top-to-bottom order give the same bits
    and counters, whatever the horizon's place in the image (or its absence)."""
    w, h = 256, 200
    cam = scenes.look((0.0, 100.0, 0.0), 30.0, pitch, 60.0, w, h)
    _, tm, params, _ = scenes.config_view(22, w, h)
    prev = to_dev(np.random.default_rng(2).random((h, w, 4), dtype=np.float32), torch)
    outs = []
    for order in (1, 0):
        ctx.set_tuning(march_order=order)
        for flags in (abi.MT_RENDER_FULL, abi.MT_RENDER_CHECKERBOARD):
            cur = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
            mask = torch.full((h, w), float("nan"), dtype=torch.float32, device="cuda")
            ctx.render(cam, cam, tm, params, prev, cur, mask, flags | abi.MT_RENDER_COUNT)
            st = ctx.stats(reset=True)
            outs.append((cur.cpu().numpy(), mask.cpu().numpy(),
                         (st.primary_samples, st.light_samples, st.marched_rays, st.pixels)))
    ctx.set_tuning(march_order=0)
    for a, b in zip(outs[:2], outs[2:]):
        assert_bits_equal(a[0], b[0], f"pitch {pitch} rgba")
        assert_bits_equal(a[1], b[1], f"pitch {pitch} mask")
        assert a[2] == b[2]


def test_reciprocal_division_is_ieee_exact(ctx):
    """The kernels divide by reused denominators through a correctly rounded
    reciprocal plus one correction step; it must equal IEEE division bit for bit."""
    rng = np.random.default_rng(123)
    n = 1 << 22
    ea = rng.integers(97, 157, n).astype(np.uint32)
    eb = rng.integers(97, 157, n).astype(np.uint32)
    ma = rng.integers(0, 1 << 23, n).astype(np.uint32)
    mb = rng.integers(0, 1 << 23, n).astype(np.uint32)
    mb[::4] = (1 << 23) - 1
    mb[1::4] = 0
    a = ((ea << 23) | ma).view(np.float32) * np.where(rng.random(n) < 0.5, -1, 1).astype(np.float32)
    b = ((eb << 23) | mb).view(np.float32) * np.where(rng.random(n) < 0.5, -1, 1).astype(np.float32)
    a[:64] = [0.0, -0.0, 1e-38, -1e-38, 3e38, np.inf, -np.inf, np.nan] * 8
    b[64:96] = [0.0, -0.0, np.inf, 1e-38] * 8
    for k in ((0.65, 0.3), (0.85, 0.3), (0.34, 0.07), (1.0, 0.6)):  # widths used by the kernels
        a[96:4096] = rng.random(4000).astype(np.float32)
        b[96:4096] = np.float32(k[0]) - np.float32(k[1])
    da, db = to_dev(a, torch), to_dev(b, torch)
    r, q = torch.empty_like(da), torch.empty_like(da)
    st = ctx.lib.mt_selftest_division(ctx.handle, da.data_ptr(), db.data_ptr(), r.data_ptr(), q.data_ptr(), n, None)
    assert st == abi.MT_OK
    r, q = r.cpu().numpy(), q.cpu().numpy()
    with np.errstate(all="ignore"):
        host = a / b
    assert_bits_equal(q[~np.isnan(host)], host[~np.isnan(host)], "device IEEE division vs host")
    assert_bits_equal(r, q, "reciprocal division vs IEEE")


@pytest.mark.parametrize("size", [(1, 1), (33, 9), (130, 18), (641, 361), (1920, 1080)])
def test_fused_frame_equals_render_then_txaa(ctx, size):
    """mt_render_frame (march + reprojection fused with TXAA) gives exactly the
    raw frame and the resolved frame of mt_render followed by mt_txaa."""
    w, h = size
    cam_old, tm, params, (yaw, pitch) = scenes.config_view(8, w, h)
    cam = scenes.look((0.0, 100.0, 0.0), yaw + 0.5, pitch, 60.0, w, h)
    rng = np.random.default_rng(w + h)
    prev = to_dev(rng.random((h, w, 4), dtype=np.float32), torch)
    hist = to_dev(rng.random((h, w, 4), dtype=np.float32), torch)
    for frame, flags in ((3, abi.MT_RENDER_CHECKERBOARD), (11, abi.MT_RENDER_CHECKERBOARD), (0, abi.MT_RENDER_FULL)):
        tm.frame_count_mod16 = frame
        cur_a = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
        out_a = torch.zeros_like(cur_a)
        ctx.render(cam, cam_old, tm, params, prev, cur_a, None, flags)
        ctx.txaa(cam, cam_old, tm, params, cur_a, hist, out_a)
        for fused, serial in ((False, False), (True, False), (False, True)):
            ctx.set_tuning(fused_resolve=fused, reproject_serial=serial)
            cur_b = torch.zeros_like(cur_a)
            out_b = torch.zeros_like(cur_a)
            ctx.render_frame(cam, cam_old, tm, params, prev, cur_b, hist, out_b, None, flags)
            what = f"{w}x{h} frame {frame} fused={fused} serial={serial}"
            assert_bits_equal(cur_b.cpu().numpy(), cur_a.cpu().numpy(), what + " raw")
            assert_bits_equal(out_b.cpu().numpy(), out_a.cpu().numpy(), what + " resolved")
            cur_c = torch.zeros_like(cur_a)
            ctx.render(cam, cam_old, tm, params, prev, cur_c, None, flags)
            assert_bits_equal(cur_c.cpu().numpy(), cur_a.cpu().numpy(), what + " mt_render")
        ctx.set_tuning(fused_resolve=False, reproject_serial=False)


@pytest.mark.parametrize("size", [(33, 9), (641, 361)])
def test_frame_counters_equal_render(ctx, size):
    """The executed-sample and pixel counters of mt_render_frame (the
    reprojection counted inside the history-taps + reprojection kernel, or the
    reprojection kernel when serialised) equal mt_render's for the same frame."""
    w, h = size
    cam_old, tm, params, (yaw, pitch) = scenes.config_view(9, w, h)
    cam = scenes.look((0.0, 100.0, 0.0), yaw + 0.5, pitch, 60.0, w, h)
    rng = np.random.default_rng(w * h)
    prev = to_dev(rng.random((h, w, 4), dtype=np.float32), torch)
    hist = to_dev(rng.random((h, w, 4), dtype=np.float32), torch)
    flags = abi.MT_RENDER_CHECKERBOARD | abi.MT_RENDER_COUNT
    tm.frame_count_mod16 = 6
    cur = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    out = torch.zeros_like(cur)
    ctx.stats(reset=True)
    ctx.render(cam, cam_old, tm, params, prev, cur, None, flags)
    ref = ctx.stats(reset=True)
    want = (ref.primary_samples, ref.light_samples, ref.marched_rays, ref.pixels)
    assert ref.pixels == w * h
    for serial in (False, True):
        ctx.set_tuning(reproject_serial=serial)
        ctx.render_frame(cam, cam_old, tm, params, prev, cur, hist, out, None, flags)
        st = ctx.stats(reset=True)
        assert (st.primary_samples, st.light_samples, st.marched_rays, st.pixels) == want, serial
    ctx.set_tuning(reproject_serial=False)


def test_config1_chain_16_frames(ctx, oracle, vol7):
    """A 16-frame config-1 sequence at 480x270 through Session (the
    reference's ping-pong, Renderer.cpp:131-136, 191): each frame reprojects
    the previous raw frame and TXAA resolves against the previous resolved
    frame, the GPU and the oracle each fed their own outputs, checked frame by
    frame (raw and resolved colour within the HDR bar, marched god-ray values
    bit-exact, executed-sample counters exact)."""
    from meteoros_gb300.renderer import FrameInputs, Session

    w, h = 480, 270
    seq = scenes.config_sequence(2017, w, h, frames=16)
    sess = Session(ctx, w, h, txaa=True)
    ctx.stats(reset=True)
    raw = out = None
    for k, (cam, old, tm, params) in enumerate(seq):
        sess.frame(FrameInputs(cam, old, tm, params), flags=abi.MT_RENDER_CHECKERBOARD | abi.MT_RENDER_COUNT)
        torch.cuda.synchronize()
        st = ctx.stats(reset=True)
        if k == 0:
            raw, mask, cnt = oracle.render(vol7, cam, old, tm, params, None, w, h, abi.MT_RENDER_FULL)
            out = oracle.txaa(cam, old, tm, params, raw, raw)
        else:
            raw, mask, cnt = oracle.render(vol7, cam, old, tm, params, raw, w, h, 0)
            out = oracle.txaa(cam, old, tm, params, raw, out)
        g_raw = sess.raw[sess.parity ^ 1].cpu().numpy()
        assert_hdr_close(g_raw, raw, f"frame {k} raw")
        assert_hdr_close(sess.output.cpu().numpy(), out, f"frame {k} resolved")
        m = ~np.isnan(mask)
        sx, sy = params.slot_x[tm.frame_count_mod16], params.slot_y[tm.frame_count_mod16]
        assert m.sum() == (w * h if k == 0 else ((w - sx + 3) // 4) * ((h - sy + 3) // 4))
        assert_bits_equal(sess.mask.cpu().numpy()[m], mask[m], f"frame {k} god-ray values")
        assert (st.primary_samples, st.light_samples, st.marched_rays) == (int(cnt[0]), int(cnt[1]), int(cnt[2])), k


@pytest.mark.parametrize("lanes", [1, 4])
def test_per_ray_control_flow_equals_oracle(ctx, oracle, vol7, lanes):
    """The exact FP32 form takes the same branch at every threshold as the
    oracle, ray by ray: the traced per-pixel step counts and control-flow
    signatures (jitter index, density > 0 and the six light samples' cbl > 0 of
    every executed step, in order) are equal for every pixel."""
    w, h = 160, 90
    cam, tm, params, _ = scenes.config_view(44, w, h)
    trace = torch.zeros((h, w, 4), dtype=torch.int32, device="cuda")
    cur = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    ctx.set_tuning(march_lanes=lanes)
    ctx.set_sample_trace(trace)
    try:
        ctx.render(cam, cam, tm, params, None, cur, None, abi.MT_RENDER_FULL)
        torch.cuda.synchronize()
    finally:
        ctx.set_sample_trace(None)
        ctx.set_tuning(march_lanes=0)
    got = trace.cpu().numpy().view(np.uint32).reshape(-1, 4)
    ys, xs = np.mgrid[0:h, 0:w]
    xy = np.stack([xs.ravel(), ys.ravel()], 1).astype(np.int32)
    _, _, want = oracle.march_pixels(vol7, cam, tm, params, w, h, xy, dtype=np.float32, counts=True)
    assert (want[:, 1] > 0).sum() > 100  # clouds in view
    bad = ~(got == want).all(1)
    assert not bad.any(), f"{int(bad.sum())} rays differ, first: {got[bad][:3].tolist()} vs {want[bad][:3].tolist()}"
