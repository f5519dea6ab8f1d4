"""A TGA writer for the tests (image types 2 and 10, 24/32 bits per pixel,
either row origin), so that decoder tests need no asset files."""
import numpy as np


def encode_tga(rgba: np.ndarray, rle: bool = True, bpp: int = 32, top_left: bool = False, seed: int = 0,
               image_id: bytes = b"") -> bytes:
    """(H, W, 4) uint8 RGBA (top row first) -> TGA bytes.  Run-length packets
    are split at random lengths (1..128) and may cross scanlines."""
    h, w = rgba.shape[:2]
    rows = rgba if top_left else rgba[::-1]
    px = rows.reshape(-1, 4)
    comp = bpp // 8
    bgra = np.stack([px[:, 2], px[:, 1], px[:, 0], px[:, 3]], 1)[:, :comp].astype(np.uint8)
    hdr = bytearray(18)
    hdr[0] = len(image_id)
    hdr[2] = 10 if rle else 2
    hdr[12], hdr[13], hdr[14], hdr[15] = w & 255, w >> 8, h & 255, h >> 8
    hdr[16] = bpp
    hdr[17] = 32 if top_left else 0
    out = bytearray(hdr) + image_id
    if not rle:
        return bytes(out + bgra.tobytes())
    rng = np.random.default_rng(seed)
    i, n = 0, len(bgra)
    while i < n:
        j = i + 1
        while j < n and j - i < 128 and np.array_equal(bgra[j], bgra[i]):
            j += 1
        if j - i >= 2:
            out.append(0x80 | (j - i - 1))
            out += bgra[i].tobytes()
            i = j
            continue
        k = min(n - i, int(rng.integers(1, 129)))
        out.append(k - 1)
        out += bgra[i:i + k].tobytes()
        i += k
    return bytes(out)


def runs_image(h: int, w: int, seed: int) -> np.ndarray:
    """An RGBA image with runs of equal pixels (so run packets appear) and noise."""
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    flat = img.reshape(-1, 4)
    i = 0
    while i < len(flat):
        L = int(rng.integers(1, 300))
        if rng.random() < 0.5:
            flat[i:i + L] = flat[i]
        i += L
    return img
