"""Batched form (config 3): one persistent, graph-captured launch over many
views equals one mt_render per view, bit for bit (GB300 only)."""
import numpy as np
import pytest

from meteoros_gb300 import abi, scenes
from tests.gpu_util import assert_bits_equal, to_dev

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SMALL = ((64, 64), (160, 90), (97, 55), (240, 135), (33, 17))


@pytest.fixture(scope="module")
def ctx(lib):
    from meteoros_gb300.renderer import Context

    c = Context(0)
    c.generate_volumes(7)
    for v in range(12):
        c.generate_weather(v, 7 + v)
    yield c
    c.close()


def build_views(storage=abi.MT_STORAGE_U8):
    specs = scenes.config3_views(5, n_views=12, resolutions=SMALL)
    rng = np.random.default_rng(0)
    views, bufs = [], []
    for i, (w, h, cam, tm, params) in enumerate(specs):
        params.storage = storage
        params.fp64_shells = 0 if storage == abi.MT_STORAGE_U8 else 1
        full = i % 3 != 0
        tm.frame_count_mod16 = i % 16
        prev = None if full else to_dev(rng.random((h, w, 4), dtype=np.float32), torch)
        cur = torch.full((h, w, 4), float("nan"), dtype=torch.float32, device="cuda")
        mask = torch.full((h, w), float("nan"), dtype=torch.float32, device="cuda")
        flags = abi.MT_RENDER_FULL if full else abi.MT_RENDER_CHECKERBOARD
        views.append(scenes.make_view(cam, cam, tm, params, cur, prev, mask, flags | abi.MT_RENDER_COUNT))
        bufs.append((cam, tm, params, prev, cur, mask, flags))
    return views, bufs


def per_view(ctx, bufs):
    outs = []
    for cam, tm, params, prev, cur, mask, flags in bufs:
        c = torch.full_like(cur, float("nan"))
        m = torch.full_like(mask, float("nan"))
        ctx.render(cam, cam, tm, params, prev, c, m, flags | abi.MT_RENDER_COUNT)
        outs.append((c.cpu().numpy(), m.cpu().numpy()))
    return outs, ctx.stats(reset=True)


@pytest.mark.parametrize("storage", [abi.MT_STORAGE_U8, abi.MT_STORAGE_F16])
def test_batch_equals_per_view(ctx, storage):
    views, bufs = build_views(storage)
    want, st_want = per_view(ctx, bufs)
    for tile, lanes, direct, order in (((16, 8), 1, False, 0), ((8, 8), 4, False, 1), ((32, 8), 8, False, 0),
                                       ((16, 8), 1, True, 1), ((16, 16), 4, True, 0)):
        ctx.set_tuning(batch_tile=tile, batch_lanes=lanes, batch_direct=direct, batch_order=order)
        for b in bufs:
            b[4].fill_(float("nan"))
            b[5].fill_(float("nan"))
        ctx.render_batch(views)
        st = ctx.stats(reset=True)
        for i, (b, (wc, wm)) in enumerate(zip(bufs, want)):
            assert_bits_equal(b[4].cpu().numpy(), wc, f"view {i} rgba, tile {tile} lanes {lanes}")
            assert_bits_equal(b[5].cpu().numpy(), wm, f"view {i} mask, tile {tile} lanes {lanes}")
        assert (st.primary_samples, st.light_samples, st.marched_rays, st.pixels) == (
            st_want.primary_samples, st_want.light_samples, st_want.marched_rays, st_want.pixels)
    ctx.set_tuning(batch_tile=(16, 8), batch_lanes=1, batch_direct=False, batch_order=0)


def test_autotune_keeps_results(ctx):
    views, bufs = build_views()
    want, _ = per_view(ctx, bufs)
    best = ctx.autotune_batch(views)
    assert (best.batch_tile_w, best.batch_tile_h) in ((8, 8), (16, 8), (16, 16), (32, 8))
    assert best.batch_lanes in (1, 4, 8) and best.batch_order in (0, 1)
    for b in bufs:
        b[4].fill_(float("nan"))
    ctx.render_batch(views)
    ctx.stats(reset=True)
    for i, (b, (wc, _)) in enumerate(zip(bufs, want)):
        assert_bits_equal(b[4].cpu().numpy(), wc, f"view {i} after autotune")
    ctx.set_tuning(batch_tile=(16, 8), batch_lanes=1, batch_order=0)


def test_batch_rejects_mixed_storage_and_bad_views(ctx):
    views, bufs = build_views()
    views[3].params.storage = abi.MT_STORAGE_F16
    with pytest.raises(abi.MeteorosError) as e:
        ctx.render_batch(views)
    assert e.value.status == abi.MT_ERR_INVALID_ARG
    views, bufs = build_views()
    views[2].width = 0
    with pytest.raises(abi.MeteorosError):
        ctx.render_batch(views)
    ctx.render_batch([])


@pytest.mark.parametrize("direct", [False, True])
def test_batches_overlap_on_two_streams(ctx, direct):
    """Three batches over disjoint images on two streams (the second overlaps
    the first on the device; the third reuses the first one's slot)."""
    ctx.set_tuning(batch_direct=direct)
    views, bufs = build_views()
    want, _ = per_view(ctx, bufs)
    for b in bufs:
        b[4].fill_(float("nan"))
        b[5].fill_(float("nan"))
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    s1.wait_stream(torch.cuda.current_stream())
    s2.wait_stream(torch.cuda.current_stream())
    ctx.render_batch(views[0:5], stream=s1)
    ctx.render_batch(views[5:9], stream=s2)
    ctx.render_batch(views[9:12], stream=s1)
    torch.cuda.synchronize()
    ctx.stats(reset=True)
    for i, (b, (wc, wm)) in enumerate(zip(bufs, want)):
        assert_bits_equal(b[4].cpu().numpy(), wc, f"view {i} rgba (two streams)")
        assert_bits_equal(b[5].cpu().numpy(), wm, f"view {i} mask (two streams)")
    ctx.set_tuning(batch_direct=False)
