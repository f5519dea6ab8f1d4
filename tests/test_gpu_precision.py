"""The precision form (config 2) against the FP64 oracle (GB300 only).

3840x2160, one full-raymarch frame, 128 primary + 6 light steps.  Forms:
  plain     RGBA8 volumes, exact FP32 (the parity form)
  fp16      IEEE-half volumes, half2 interpolation, FP64 shell intersection
  bf16      bfloat16 volumes, bfloat16x2 interpolation, FP64 shell intersection
Each is compared with the FP64 oracle fed the texel values that form stores,
on a 1/64 sample of the pixels (every 8th column and row).

The march has hard thresholds (density > 0, the early exit, the step
recurrence t += stepSize), so even exact FP32 differs from FP64 by whole
samples in some pixels; the FP32-vs-FP64 distribution is printed beside the
precision forms' and the precision forms are held to it.
"""
import numpy as np
import pytest

from meteoros_gb300 import abi, scenes
from tests.gpu_util import to_dev

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

W, H, STRIDE = 3840, 2160, 8


def stats(gpu_rgb, ref_rgb):
    d = np.abs(gpu_rgb.astype(np.float64) - ref_rgb.astype(np.float64)).max(-1)
    return {"max": float(d.max()), "mean": float(d.mean()), "p99": float(np.percentile(d, 99)),
            "frac_gt_2e-3": float((d > 2e-3).mean())}


@pytest.fixture(scope="module")
def ctx(lib):
    from meteoros_gb300.renderer import Context

    c = Context(0)
    c.generate_volumes(7)
    yield c
    c.close()


def test_precision_form_vs_fp64_oracle(ctx, oracle, volumes_seed7):
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
        ctx.render(cam, cam, tm, p, None, cur, None, abi.MT_RENDER_FULL)
        g = cur.cpu().numpy()[xy[:, 1], xy[:, 0], :3]
        ref, _ = oracle.march_pixels(vols[form], cam, tm, p, W, H, xy, dtype=np.float64)
        out[form] = stats(g, ref[:, :3])
        print(form, {k: round(v, 6) for k, v in out[form].items()})
    for form in ("fp16", "bf16"):
        assert out[form]["mean"] <= 2.0 * out["plain"]["mean"] + 2e-3, form
        assert out[form]["p99"] <= 2.0 * out["plain"]["p99"] + 2e-2, form
        assert out[form]["max"] < 10.0, form


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
