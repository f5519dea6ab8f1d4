"""The CPU noise generator (oracle side of the generator kernels): number
formats, determinism, ranges and tiling.  CPU only."""
import numpy as np
import pytest


def test_half_conversion_is_ieee_round_to_nearest_even(oracle):
    rng = np.random.default_rng(5)
    vals = np.concatenate([
        rng.random(4000, dtype=np.float32),
        rng.random(1000, dtype=np.float32) * np.float32(1e-4),  # subnormal halves
        np.array([0.0, 1.0, 1.0 / 3.0, 65504.0, 65519.0, 65520.0, 5.9604645e-08, 2.9802322e-08,
                  0.00048828125 + 2.0 ** -22], np.float32),
    ])
    got = np.array([oracle.lib().orc_f2h(float(v)) for v in vals], np.uint16)
    want = vals.astype(np.float16).view(np.uint16)
    assert np.array_equal(got, want)


def test_bfloat16_conversion_is_round_to_nearest_even(oracle):
    rng = np.random.default_rng(6)
    vals = rng.random(5000, dtype=np.float32) * np.float32(7.0)
    got = np.array([oracle.lib().orc_f2bf(float(v)) for v in vals], np.uint16)
    u = vals.view(np.uint32).astype(np.uint64)
    want = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    assert np.array_equal(got, want)
    # ties go to even
    tie = np.array([0x3F808000, 0x3F818000], np.uint32).view(np.float32)
    assert [oracle.lib().orc_f2bf(float(t)) for t in tie] == [0x3F80, 0x3F82]


def test_generator_is_deterministic_and_seeded(oracle, volumes_seed7):
    again = oracle.generate_volumes(7)
    other = oracle.generate_volumes(8)
    for k in ("base", "detail", "curl", "weather"):
        assert np.array_equal(again[k], volumes_seed7[k])
        assert not np.array_equal(other[k], volumes_seed7[k])


def test_generator_ranges(volumes_seed7):
    v = volumes_seed7
    base = v["base"].reshape(-1, 4).astype(np.float64) / 255.0
    assert base.min() >= 0.0 and base.max() <= 1.0
    assert 0.3 < base[:, 1].mean() < 0.7  # Worley fBm
    assert (v["detail"][..., 3] == 255).all()
    w = v["weather"].reshape(-1, 4)
    assert set(np.unique(w[:, 2])) <= {0, 128, 255}  # cloud type in {0, 0.5, 1}
    assert len(np.unique(w[:, 2])) >= 2
    assert 0.4 < w[:, 1].mean() / 255.0 < 0.6  # precipitation uniform on [0,1)
    cov = w[:, 0] / 255.0
    assert cov.min() >= 0.0 and cov.max() <= 1.0 and cov.std() > 0.03


@pytest.mark.parametrize("key,axes", [("base", (0, 1, 2)), ("detail", (0, 1, 2)), ("curl", (0, 1)),
                                      ("weather", (0, 1))])
def test_generator_tiles_seamlessly(volumes_seed7, key, axes):
    """Across the wrap the continuous channels change no more than inside."""
    vol = volumes_seed7[key].astype(np.int32)
    chans = [0, 1] if key == "weather" else [0, 1, 2]
    for ax in axes:
        inner = np.abs(np.diff(vol, axis=ax)).mean(axis=tuple(range(vol.ndim - 1)))
        first = np.take(vol, 0, axis=ax)
        last = np.take(vol, -1, axis=ax)
        wrap = np.abs(first - last).mean(axis=tuple(range(first.ndim - 1)))
        for c in chans:
            if key == "weather" and c == 1:
                continue  # white-noise precipitation
            assert wrap[c] <= 1.5 * inner[c] + 1.0, (key, ax, c, wrap[c], inner[c])


def test_half_copies_track_rgba8(volumes_seed7):
    v = volumes_seed7
    for k in ("base", "detail", "curl", "weather"):
        h = v[k + "_h16"].view(np.float16).astype(np.float32)
        q = v[k].astype(np.float32) / 255.0
        assert np.abs(h - q).max() <= 0.5 / 255.0 + 1e-3
