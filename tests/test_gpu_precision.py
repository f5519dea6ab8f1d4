"""The precision form (config 2) against the FP64 oracle (GB300 only).

3840x2160, one full-raymarch frame, 128 primary + 6 light steps.  Forms:
  plain     RGBA8 volumes, exact FP32 (the parity form)
  fp16      IEEE-half volumes; primary density filtered in FP32, the cone-light
            samples' filtering and density math in half2; FP64 shell
            intersection
  bf16      bfloat16 volumes, filtered in FP32; FP64 shell intersection
Each is compared with the FP64 oracle fed the texel values that form stores,
on a 1/64 sample of the pixels (every 8th column and row).

The march has hard thresholds: density > 0 at each step, each light
sample's cbl > 0, the jitter index int(mod(frame + int(t), 16)) (which moves
the sample point by tens of metres when t crosses a whole metre) and the
early exit.  A pixel where any of them falls the other way than in FP64
moves by a whole step's contribution, whatever the precision.  Each ray's
control flow is traced (mt_set_sample_trace) and compared with the oracle's:
pixels that took the same branch everywhere carry only the continuous error
of the arithmetic and are held to the bar; the flipped pixels and the flip
fraction are reported.

The bar is 2e-3 relative to max(1, |value|): absolute below 1, relative above.
HDR cloud colours reach 40, where an absolute 2e-3 would be a 5e-5 relative
bar, finer than the reference's own RGBA16F images hold (a step of 2^-11
relative).
"""
import numpy as np
import pytest

from meteoros_gb300 import abi, scenes

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

W, H, STRIDE = 3840, 2160, 8
BAR = {"plain": 2e-3, "fp16": 2e-3, "bf16": 2e-3}


def split_stats(gpu_rgb, ref_rgb, same):
    d = np.abs(gpu_rgb.astype(np.float64) - ref_rgb.astype(np.float64)).max(-1)
    scale = np.maximum(1.0, np.abs(ref_rgb.astype(np.float64)).max(-1))
    r = d / scale
    k = same
    return {"flip_frac": float(1.0 - same.mean()), "same_pixels": int(k.sum()),
            "same_max_abs": float(d[k].max()), "same_mean_abs": float(d[k].mean()),
            "same_p999_abs": float(np.percentile(d[k], 99.9)), "same_max_rel": float(r[k].max()),
            "same_p999_rel": float(np.percentile(r[k], 99.9)), "same_frac_abs_le_2e-3": float((d[k] <= 2e-3).mean()),
            "all_max_rel": float(r.max()), "all_mean_abs": float(d.mean())}


@pytest.fixture(scope="module")
def ctx(lib):
    from meteoros_gb300.renderer import Context

    c = Context(0)
    c.generate_volumes(7)
    yield c
    c.close()


@pytest.fixture(scope="module")
def forms(ctx, oracle, volumes_seed7):
    """Per form: error statistics of one traced 4K frame against the FP64 oracle."""
    cam, tm, params, _ = scenes.config_view(31, W, H)
    ys, xs = np.mgrid[0:H:STRIDE, 0:W:STRIDE]
    xy = np.stack([xs.ravel(), ys.ravel()], 1).astype(np.int32)
    vols = {"plain": oracle.Volumes(volumes_seed7["base"], volumes_seed7["detail"], volumes_seed7["curl"],
                                    volumes_seed7["weather"]),
            "fp16": oracle.volumes_16(volumes_seed7, "h16"),
            "bf16": oracle.volumes_16(volumes_seed7, "b16")}
    storage = {"plain": abi.MT_STORAGE_U8, "fp16": abi.MT_STORAGE_F16, "bf16": abi.MT_STORAGE_BF16}
    out = {}
    for form in ("plain", "fp16", "bf16"):
        p = scenes.C_copy(abi.Params(), params)
        p.storage = storage[form]
        p.fp64_shells = 0 if form == "plain" else 1
        cur = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
        trace = torch.zeros((H, W, 4), dtype=torch.int32, device="cuda")
        ctx.set_sample_trace(trace)
        try:
            ctx.render(cam, cam, tm, p, None, cur, None, abi.MT_RENDER_FULL)
            torch.cuda.synchronize()
        finally:
            ctx.set_sample_trace(None)
        g = cur.cpu().numpy()[xy[:, 1], xy[:, 0], :3]
        gt = trace.cpu().numpy().view(np.uint32)[xy[:, 1], xy[:, 0]]
        ref, _, rt = oracle.march_pixels(vols[form], cam, tm, p, W, H, xy, dtype=np.float64, counts=True)
        out[form] = split_stats(g, ref[:, :3], (gt == rt).all(1))
        print(form, {k: round(v, 7) for k, v in out[form].items()})
    return out


@pytest.mark.parametrize("form", ["plain", "fp16", "bf16"])
def test_same_branch_pixels_within_the_bar(forms, form):
    s = forms[form]
    assert s["same_pixels"] > 10000  # a large part of the sample keeps the oracle's branches
    assert s["same_max_rel"] <= BAR[form], s


def test_precision_forms_flip_no_more_than_plain(forms):
    """FP64 shells remove the FP32 shell-intersection error, so the precision
    forms follow the FP64 control flow at least as often as exact FP32 does."""
    for form in ("fp16", "bf16"):
        assert forms[form]["flip_frac"] <= forms["plain"]["flip_frac"] + 0.02, (form, forms[form], forms["plain"])


def test_precision_storages_are_deterministic(ctx):
    cam, tm, params, _ = scenes.config_view(32, 320, 180)
    for st in (abi.MT_STORAGE_F16, abi.MT_STORAGE_BF16):
        p = scenes.C_copy(abi.Params(), params)
        p.storage = st
        p.fp64_shells = 1
        a = torch.zeros((180, 320, 4), dtype=torch.float32, device="cuda")
        b = torch.zeros_like(a)
        ctx.render(cam, cam, tm, p, None, a, None, abi.MT_RENDER_FULL)
        ctx.render(cam, cam, tm, p, None, b, None, abi.MT_RENDER_FULL)
        assert torch.equal(a, b)
        assert torch.isfinite(a).all()
