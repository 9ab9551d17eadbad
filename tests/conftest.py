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


SHIPPED_MESHES = ("disk_20um_diam_edited", "disk_20um_diam_N1025", "disk_20um_diam_N2944")
SHIPPED_STATE = ("x", "V", "A", "ea", "cA", "cC", "fau")
SHIPPED_FINAL = ("x", "V", "ea", "cC", "fau")


@pytest.fixture(scope="session", params=VARIANTS)
def shipped(request):
    """Trajectories of the reference's own step loop on its shipped meshes
    (tests/golden/make_golden.py, make_shipped)."""
    g = np.load(os.path.join(GOLDEN, f"shipped_{request.param}.npz"))
    d = {k: g[k] for k in g.files}
    d["variant"] = request.param
    return d


def shipped_runs(g):
    """(mesh index, run kind, start state, start time, start AP call, steps) of a shipped fixture."""
    from wholecellfe_gb300 import synth
    runs = []
    for m in range(len(SHIPPED_MESHES)):
        st = tuple(g[f"m{m}_mov0_{k}"] for k in SHIPPED_STATE)
        runs.append((m, "mov", st, 0.7, 7, 20))
        if f"m{m}_rest_x" in g:
            runs.append((m, "rest", synth.initial_state(g[f"m{m}_x0"]), 0.0, 0, 200))
    return runs
