"""TGA slice stacks decoded on the device (mt_decode_tga_volume) against the
CPU restatement of the reference's decoder, through the C ABI (GB300 only).
The slices are written by the tests (run-length and raw, 24/32 bits, both
row origins, truncated files)."""
import ctypes as C

import numpy as np
import pytest

from meteoros_gb300 import abi
from tests.tga_util import encode_tga, runs_image

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def ctx(lib):
    from meteoros_gb300.renderer import Context

    c = Context(0)
    c.generate_volumes(7)
    yield c
    c.close()


def decode(ctx, volume, files):
    arr = (C.c_void_p * len(files))(*[C.cast(C.c_char_p(f), C.c_void_p) for f in files])
    sizes = (C.c_size_t * len(files))(*[len(f) for f in files])
    return ctx.lib.mt_decode_tga_volume(ctx.handle, volume, arr, sizes, len(files), None)


def slice_files(n, seed):
    files, want = [], []
    for z in range(n):
        rng = np.random.default_rng(seed * 1000 + z)
        img = runs_image(n, n, seed * 1000 + z)
        rle, bpp, top = bool(z % 3), (24, 32)[z % 2], bool(z % 5 == 0)
        if bpp == 24:
            img[..., 3] = 255
        data = encode_tga(img, rle=rle, bpp=bpp, top_left=top, seed=z, image_id=b"x" * (z % 4))
        if z % 7 == 3:  # truncated: the missing bytes read as 0
            data = data[: int(rng.integers(18, len(data)))]
        files.append(data)
    return files


def test_decode_volumes_equal_restatement(ctx, oracle):
    for volume, n, seed in ((abi.MT_VOLUME_DETAIL, abi.MT_DETAIL_N, 1), (abi.MT_VOLUME_BASE, abi.MT_BASE_N, 2)):
        files = slice_files(n, seed)
        want = np.stack([oracle.decode_tga(f) for f in files])
        assert decode(ctx, volume, files) == abi.MT_OK, ctx.lib.mt_last_error(ctx.handle).decode()
        key = "base" if volume == abi.MT_VOLUME_BASE else "detail"
        got = ctx.download_volumes()[key]
        assert np.array_equal(got, want), f"volume {volume}"
        # the FP16 / BF16 copies are the decoded bytes / 255, rounded to nearest even
        unorm = want.astype(np.float32) / np.float32(255.0)
        h16 = ctx.download_volumes_16(abi.MT_STORAGE_F16)[key]
        assert np.array_equal(h16, unorm.astype(np.float16).view(np.uint16))
        b16 = ctx.download_volumes_16(abi.MT_STORAGE_BF16)[key]
        bits = unorm.view(np.uint32).astype(np.uint64)
        bf = ((bits + 0x7FFF + ((bits >> 16) & 1)) >> 16).astype(np.uint16)  # finite values, nearest even
        assert np.array_equal(b16, bf)


def test_decode_rejects_bad_stacks(ctx):
    files = slice_files(abi.MT_DETAIL_N, 3)
    assert decode(ctx, abi.MT_VOLUME_DETAIL, files[:-1]) == abi.MT_ERR_INVALID_ARG
    assert decode(ctx, abi.MT_VOLUME_BASE, files) == abi.MT_ERR_INVALID_ARG
    bad = list(files)
    b = bytearray(bad[4])
    b[2] = 3  # greyscale
    bad[4] = bytes(b)
    assert decode(ctx, abi.MT_VOLUME_DETAIL, bad) == abi.MT_ERR_INVALID_ARG
    assert "slice 4" in ctx.lib.mt_last_error(ctx.handle).decode()
    assert decode(ctx, 7, files) == abi.MT_ERR_INVALID_ARG
