"""Shared helpers of the GPU tests (parity tolerances, device buffers)."""
import numpy as np

# Parity bar for HDR colour against the FP32 oracle: max abs 1e-3, mean abs
# 1e-5.  The two sides run the same IEEE FP32 operations in the same order on
# the density path (the god-ray mask and the sample counters are exact); what
# differs feeds colour only: the sky (acos/cos with CUDA libdevice vs host
# libm, a few ulp; exp/pow in the special-function unit's forms), the phase
# function, and the cone-light samples and light energy (fused multiply-adds,
# reciprocal products, the special-function unit's exp2/log2).  For the rare pixels brighter than
# 4096 (the Preetham sun disk reaches ~1e6), 1e-3 is below 8 ulp of the value,
# so those are held to 1e-6 relative instead.
MAX_ABS = 1e-3
MEAN_ABS = 1e-5
BRIGHT = 4096.0
BRIGHT_REL = 1e-6


def to_dev(a, torch):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def hdr_error(gpu: np.ndarray, ref: np.ndarray):
    """(max abs over pixels <= BRIGHT, mean abs, max rel over bright pixels)."""
    gpu = np.asarray(gpu, np.float64)
    ref = np.asarray(ref, np.float64)
    written = ~np.isnan(ref)
    assert np.array_equal(written, ~np.isnan(gpu)), "written-pixel pattern differs"
    d = np.abs(np.where(written, gpu - ref, 0.0))
    bright = np.abs(np.where(written, ref, 0.0)) > BRIGHT
    max_abs = float(d[~bright].max()) if (~bright).any() else 0.0
    mean_abs = float(d[written].mean()) if written.any() else 0.0
    rel = float((d[bright] / np.abs(ref[bright])).max()) if bright.any() else 0.0
    return max_abs, mean_abs, rel


def assert_hdr_close(gpu, ref, what=""):
    max_abs, mean_abs, rel = hdr_error(gpu, ref)
    assert max_abs <= MAX_ABS, f"{what}: max abs error {max_abs}"
    assert mean_abs <= MEAN_ABS, f"{what}: mean abs error {mean_abs}"
    assert rel <= BRIGHT_REL, f"{what}: relative error on bright pixels {rel}"
    return max_abs, mean_abs, rel


def assert_bits_equal(a, b, what=""):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    na, nb = np.isnan(a), np.isnan(b)
    assert np.array_equal(na, nb), f"{what}: written-pixel pattern differs"
    diff = np.where(na, 0, a).view(np.uint32) != np.where(nb, 0, b).view(np.uint32)
    assert not diff.any(), f"{what}: {int(diff.sum())} values differ (max {np.nanmax(np.abs(a - b))})"
