import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = Path(__file__).resolve().parent / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libsarbp.so")
    config.addinivalue_line("markers", "slow: full-size parity check (tens of seconds)")


@pytest.fixture(scope="session")
def golden():
    cache = {}

    def load(name):
        if name not in cache:
            with np.load(GOLDEN / f"{name}.npz") as z:
                cache[name] = {k: z[k] for k in z.files}
        return cache[name]

    return load


def rel_err(reference, estimate):
    """Relative complex L2 error ||est - ref|| / ||ref|| (gpu_baseline.py:53-55)."""
    a = np.asarray(reference, np.complex128).ravel()
    b = np.asarray(estimate, np.complex128).ravel()
    return float(np.linalg.norm(b - a) / np.linalg.norm(a))
