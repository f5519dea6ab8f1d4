"""Small, self-contained launches of each kernel, for profiling one kernel at a
time under a profiler (a few launches, a few hundred MB on the device).

  python -m meteoros_gb300.profile_cases <case> [--reps N]

cases:
  march_full      960x540 full-raymarch frame (march_kernel<1>), config 0 view
  march_cb        1920x1080 checkerboard frame (march_kernel<4> + reprojection)
  frame           1920x1080 reprojected frame through mt_render_frame (raymarch, reprojection
                  and TXAA history beside it, then the TXAA resolve)
  txaa            1920x1080 TXAA resolve
  batch           64-view batched raymarch (march_batch_kernel), RGBA8 volumes
  batch_fp16      the same with FP16 volumes
  precision       3840x2160 full frame, FP16 volumes (march_kernel<1>, half2 path)
  precision_bf16  the same frame with bfloat16 volumes (filtered in FP32)
  upload          host RGBA8 volumes uploaded: the 16-bit copies (u8_to_16_kernel) and the
                  samplers' layouts (quads3_kernel, quads16_kernel, cells2_kernel)
  batch_noalloc   16 views through the allocation-free batch entry (noalloc_store_kernel,
                  noalloc_tiles_kernel, march_batch_kernel)
  godrays         1920x1080 god-ray radial blur
  tonemap         1920x1080 tone map + dither to RGBA8
  generate        noise-volume generation (gen_* kernels)
  frame_fused     the 1080p reprojected frame with the reprojection fused into the TXAA
                  resolve (resolve_kernel)
  tga             a 128-slice stack of 128x128 run-length TGA files decoded on the device
                  (tga_decode_kernel)

Each case renders its frame `reps` times (default 2) so a profiler can skip
the first launch and capture the next.
"""
from __future__ import annotations

import argparse
import sys

SEED = 2017


def _rle_tga(img) -> bytes:
    """A 32-bit run-length TGA (image type 10, bottom-left origin) of an
    (H, W, 4) RGBA8 image: runs of equal pixels as run packets, the rest as
    raw packets of up to 128 pixels."""
    h, w = img.shape[:2]
    header = bytes([0, 0, 10, 0, 0, 0, 0, 0, 0, 0, 0, 0, w & 255, w >> 8, h & 255, h >> 8, 32, 8])
    px = img[::-1].reshape(-1, 4)[:, [2, 1, 0, 3]]  # bottom row first, BGRA
    out, i, n = [header], 0, len(px)
    while i < n:
        j = i + 1
        while j < n and j - i < 128 and (px[j] == px[i]).all():
            j += 1
        if j - i > 1:
            out.append(bytes([0x80 | (j - i - 1)]) + px[i].tobytes())
        else:
            j = i + 1
            while j < n and j - i < 128 and not (j + 1 < n and (px[j] == px[j + 1]).all()):
                j += 1
            out.append(bytes([j - i - 1]) + px[i:j].tobytes())
        i = j
    return b"".join(out)


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("case")
    ap.add_argument("--reps", type=int, default=2)
    a = ap.parse_args(argv)

    import torch

    from . import abi, scenes
    from .renderer import Context

    ctx = Context(0)
    ctx.generate_volumes(SEED)
    dev = "cuda"
    if a.case == "march_full":
        cam, tm, params, _ = scenes.config_view(11, 960, 540)
        cur = torch.zeros((540, 960, 4), device=dev)
        for _ in range(a.reps):
            ctx.render(cam, cam, tm, params, None, cur, None, abi.MT_RENDER_FULL)
    elif a.case in ("march_cb", "txaa"):
        W, H = 1920, 1080
        cam, old, tm, params = scenes.config_sequence(SEED, W, H, frames=3)[2]
        prev = torch.rand((H, W, 4), device=dev)
        cur = torch.zeros_like(prev)
        out = torch.zeros_like(prev)
        for _ in range(a.reps):
            if a.case == "march_cb":
                ctx.render(cam, old, tm, params, prev, cur, None, abi.MT_RENDER_CHECKERBOARD)
            else:
                ctx.txaa(cam, old, tm, params, prev, cur, out)
    elif a.case in ("frame", "frame_fused"):
        if a.case == "frame_fused":
            ctx.set_tuning(fused_resolve=True)
        W, H = 1920, 1080
        seq = scenes.config_sequence(SEED, W, H, frames=a.reps)
        prev = torch.rand((H, W, 4), device=dev)
        hist = torch.rand((H, W, 4), device=dev)
        cur = torch.zeros_like(prev)
        out = torch.zeros_like(prev)
        mask = torch.zeros((H, W), device=dev)
        for cam, old, tm, params in seq:
            ctx.render_frame(cam, old, tm, params, prev, cur, hist, out, mask)
    elif a.case in ("batch", "batch_fp16"):
        storage = abi.MT_STORAGE_F16 if a.case == "batch_fp16" else abi.MT_STORAGE_U8
        specs = scenes.config3_views(SEED, n_views=64)
        for v in range(64):
            ctx.generate_weather(v, SEED + v)
        views = []
        keep = []
        for w, h, cam, tm, params in specs:
            params.storage = storage
            params.fp64_shells = 0 if storage == abi.MT_STORAGE_U8 else 1
            cur = torch.empty((h, w, 4), device=dev)
            keep.append(cur)
            views.append(scenes.make_view(cam, cam, tm, params, cur, None, None, abi.MT_RENDER_FULL))
        for _ in range(a.reps):
            ctx.render_batch(views)
    elif a.case in ("precision", "precision_bf16"):
        W, H = 3840, 2160
        cam, tm, params, _ = scenes.config_view(SEED + 2, W, H)
        params.storage = abi.MT_STORAGE_BF16 if a.case == "precision_bf16" else abi.MT_STORAGE_F16
        params.fp64_shells = 1
        cur = torch.empty((H, W, 4), device=dev)
        for _ in range(a.reps):
            ctx.render(cam, cam, tm, params, None, cur, None, abi.MT_RENDER_FULL)
    elif a.case in ("godrays", "tonemap"):
        W, H = 1920, 1080
        img = torch.rand((H, W, 4), device=dev) * 2.0
        mask = torch.rand((H, W), device=dev)
        out = torch.empty_like(img)
        out8 = torch.empty((H, W, 4), dtype=torch.uint8, device=dev)
        cam = scenes.look((0.0, 0.0, 2.0), 5.0, 12.0, 45.0, W, H)
        tm = abi.time_init()
        tm.time[1] = 2.75
        for _ in range(a.reps):
            if a.case == "godrays":
                ctx.godrays(cam, (1.0, 1.0, 0.57, 1.0), mask, img, out)
            else:
                ctx.tonemap(tm, img, out8, abi.MT_LDR_RGBA8)
    elif a.case == "upload":
        # host RGBA8 volumes in: the 16-bit copies and the samplers' layouts rebuilt
        vols = ctx.download_volumes()
        for _ in range(a.reps):
            ctx.upload_volumes(vols["base"], vols["detail"], vols["curl"], vols["weather"])
    elif a.case == "batch_noalloc":
        import ctypes as C

        # 16 views at the two smaller config-3 sizes: within the entry's fixed tile table
        specs = scenes.config3_views(SEED, n_views=16, resolutions=((256, 256), (640, 360)))
        for v in range(16):
            ctx.generate_weather(v, SEED + v)
        views, keep = [], []
        for w, h, cam, tm, params in specs:
            cur = torch.empty((h, w, 4), device=dev)
            keep.append(cur)
            views.append(scenes.make_view(cam, cam, tm, params, cur, None, None, abi.MT_RENDER_FULL))
        arr = (abi.View * len(views))(*views)
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        for _ in range(a.reps):
            st = ctx.lib.mt_render_batch_noalloc(ctx.handle, arr, len(views), stream)
            if st != abi.MT_OK:
                print(ctx.lib.mt_last_error(ctx.handle).decode(), file=sys.stderr)
                return 1
    elif a.case == "generate":
        for r in range(a.reps):
            ctx.generate_volumes(SEED + r)
    elif a.case == "tga":
        import ctypes as C

        base = ctx.download_volumes()["base"]
        files = [_rle_tga(base[z]) for z in range(abi.MT_BASE_N)]
        arr = (C.c_void_p * len(files))(*[C.cast(C.c_char_p(f), C.c_void_p) for f in files])
        sizes = (C.c_size_t * len(files))(*[len(f) for f in files])
        for _ in range(a.reps):
            st = ctx.lib.mt_decode_tga_volume(ctx.handle, abi.MT_VOLUME_BASE, arr, sizes, len(files), None)
            if st != abi.MT_OK:
                print(ctx.lib.mt_last_error(ctx.handle).decode(), file=sys.stderr)
                return 1
    else:
        print(f"unknown case {a.case}", file=sys.stderr)
        return 2
    torch.cuda.synchronize()
    ctx.close()
    print("ok")
    return 0


if __name__ == "__main__":
    sys.exit(main())
