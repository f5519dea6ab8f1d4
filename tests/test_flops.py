"""The raymarch's FLOP constants in bench.py are the op-counting oracle's fit
(oracle/count_flops.py), and the fit explains every counted pixel."""
import importlib.util
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]


def test_bench_flop_constants_match_the_counting_oracle(oracle):
    from oracle import count_flops

    coef, d, A = count_flops.fit()
    spec = importlib.util.spec_from_file_location("bench_consts", ROOT / "bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    consts = np.array([bench.FLOPS_PER_PIXEL, bench.FLOPS_PER_RAY, bench.FLOPS_PER_PRIMARY, bench.FLOPS_PER_LIGHT])
    np.testing.assert_allclose(consts, coef, rtol=2e-3)
    # the linear model reproduces the total count of the sample
    assert abs((A @ consts).sum() - d[:, 0].sum()) / d[:, 0].sum() < 1e-3
