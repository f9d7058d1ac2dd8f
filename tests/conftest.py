import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


def _load(name):
    with np.load(os.path.join(GOLDEN, name)) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def soundings():
    """13 soundings x 108 levels (level 0 = surface): the reference's
    ``dataset_soundings`` fixture (test/fixtures.py:1166-3441)."""
    return _load("soundings.npz")


@pytest.fixture(scope="session")
def era5():
    """17 ERA5 columns x 37 pressure levels: the reference's
    ``dataset_ERA5pressurelevel`` fixture (test/fixtures.py:29-1162).
    Keys are prefixed ``lev_`` (3-D) and ``sfc_`` (surface)."""
    return _load("era5_pressure.npz")


def cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
