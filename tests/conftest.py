import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU and the built CUDA library")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle

    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def lib():
    """The product's C-ABI library (built in-tree)."""
    from meteoros_gb300 import abi, build

    build.build()
    return abi.load_library()


@pytest.fixture(scope="session")
def volumes_seed7(oracle):
    """Generator output for seed 7 (the golden fixtures' inputs)."""
    return oracle.generate_volumes(7)


@pytest.fixture(scope="session")
def vol7(oracle, volumes_seed7):
    v = volumes_seed7
    return oracle.Volumes(v["base"], v["detail"], v["curl"], v["weather"])


@pytest.fixture(scope="session")
def golden():
    path = GOLDEN / "golden.npz"
    if not path.exists():
        pytest.fail(f"{path} is missing; run tests/golden/make_golden.py")
    return dict(np.load(path))
