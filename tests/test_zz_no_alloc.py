"""mt_render_batch_noalloc against mt_render_batch, through the C ABI (GB300 only).

The allocation-free entry point keeps its view table, tile list and work
counter in one fixed device array of the library, for callers that cannot
allocate device memory on their render path.  Two calls in a row (a
different batch each time, so the second runs over the first one's leftover
tables) must each give what mt_render_batch gives for the same views.  This
file is collected last so that it runs both after the other GPU tests and,
on its own, in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from meteoros_gb300 import abi, scenes
from tests.gpu_util import assert_bits_equal, to_dev

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SIZES = ((64, 64), (160, 90), (97, 55), (240, 135), (33, 17))


@pytest.fixture(scope="module")
def ctx(lib):
    from meteoros_gb300.renderer import Context

    c = Context(0)
    c.generate_volumes(7)
    for v in range(40):
        c.generate_weather(v, 7 + v)
    yield c
    c.close()


def make_batch(seed, n_views, storage):
    """Views over fresh images: every third view checkerboard (reprojecting a
    random previous frame), the rest full raymarch."""
    specs = scenes.config3_views(seed, n_views=n_views, resolutions=SIZES)
    rng = np.random.default_rng(seed)
    views, imgs = [], []
    for i, (w, h, cam, tm, params) in enumerate(specs):
        params.storage = storage
        params.fp64_shells = 0 if storage == abi.MT_STORAGE_U8 else 1
        tm.frame_count_mod16 = (seed + i) % 16
        full = i % 3 != 0
        prev = None if full else to_dev(rng.random((h, w, 4), dtype=np.float32), torch)
        cur = torch.full((h, w, 4), float("nan"), dtype=torch.float32, device="cuda")
        mask = torch.full((h, w), float("nan"), dtype=torch.float32, device="cuda")
        flags = (abi.MT_RENDER_FULL if full else abi.MT_RENDER_CHECKERBOARD) | abi.MT_RENDER_COUNT
        views.append(scenes.make_view(cam, cam, tm, params, cur, prev, mask, flags))
        imgs.append((cur, mask))
    return views, imgs


def call(ctx, name, views):
    arr = (abi.View * len(views))(*views)
    stream = torch.cuda.current_stream().cuda_stream
    return getattr(ctx.lib, name)(ctx.handle, arr, len(views), C.c_void_p(stream))


def run(ctx, name, views, imgs):
    for cur, mask in imgs:
        cur.fill_(float("nan"))
        mask.fill_(float("nan"))
    st = call(ctx, name, views)
    assert st == abi.MT_OK, ctx.lib.mt_last_error(ctx.handle).decode()
    torch.cuda.synchronize()
    s = ctx.stats(reset=True)
    return ([(c.cpu().numpy(), m.cpu().numpy()) for c, m in imgs],
            (s.primary_samples, s.light_samples, s.marched_rays, s.pixels))


def test_noalloc_equals_render_batch_on_two_calls_in_a_row(ctx):
    ctx.stats(reset=True)
    # 40 views: three store launches of the view tables; then 7 over their leftovers
    for seed, n_views, storage in ((11, 40, abi.MT_STORAGE_U8), (12, 7, abi.MT_STORAGE_F16)):
        views, imgs = make_batch(seed, n_views, storage)
        want, st_want = run(ctx, "mt_render_batch", views, imgs)
        got, st_got = run(ctx, "mt_render_batch_noalloc", views, imgs)
        for i, ((gc, gm), (wc, wm)) in enumerate(zip(got, want)):
            assert_bits_equal(gc, wc, f"seed {seed} view {i} rgba")
            assert_bits_equal(gm, wm, f"seed {seed} view {i} mask")
        assert st_got == st_want


def test_noalloc_rejects_batches_beyond_its_tables(ctx):
    views, _ = make_batch(13, 2, abi.MT_STORAGE_U8)
    too_many = [views[0]] * (abi.MT_NOALLOC_MAX_VIEWS + 1)
    assert call(ctx, "mt_render_batch_noalloc", too_many) == abi.MT_ERR_INVALID_ARG
    assert "views" in ctx.lib.mt_last_error(ctx.handle).decode()
    # one 1920x1080 full-raymarch view in 1x1 tiles: 2,073,600 tiles
    big = torch.zeros((1080, 1920, 4), dtype=torch.float32, device="cuda")
    cam, tm, params, _ = scenes.config_view(3, 1920, 1080)
    v = scenes.make_view(cam, cam, tm, params, big, None, None, abi.MT_RENDER_FULL)
    ctx.set_tuning(batch_tile=(1, 1), batch_lanes=1)
    try:
        assert call(ctx, "mt_render_batch_noalloc", [v]) == abi.MT_ERR_INVALID_ARG
        assert "tiles" in ctx.lib.mt_last_error(ctx.handle).decode()
    finally:
        ctx.set_tuning(batch_tile=(16, 8), batch_lanes=1)
    assert call(ctx, "mt_render_batch_noalloc", []) == abi.MT_OK
