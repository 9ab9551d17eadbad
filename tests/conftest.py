import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
VARIANTS = ("kMD", "k1", "k31")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


def relerr(a, b):
    """Norm-wise relative error max|a-b| / max|b| (absolute when b == 0)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = float(np.max(np.abs(a - b))) if a.size else 0.0
    s = float(np.max(np.abs(b))) if b.size else 0.0
    return d / s if s > 0 else d


@pytest.fixture(scope="session", params=VARIANTS)
def golden(request):
    g = np.load(os.path.join(GOLDEN, f"golden_{request.param}.npz"))
    d = {k: g[k] for k in g.files}
    d["variant"] = request.param
    return d
