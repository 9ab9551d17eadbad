"""VTK frames (cellBP/iomesh.cpp:690-1047, the reference's write_vtk): the library's
formatter reproduces the reference's own writers byte for byte, on the golden frames that
tests/golden/make_golden.py wrote with them (every format; the concentration frame in the
kMD variant with the MD table and with a linear kint, and in the k1 and k31 variants).
Host only: no device."""
import os

import numpy as np
import pytest

from wholecellfe_gb300 import capi
from wholecellfe_gb300.params import default_params

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "vtk")
CASES = [("kMD", 0, -1.0), ("kMD", 1, -1.0), ("kMD", 2, -1.0), ("kMD", 2, 1000.0), ("k1", 2, -1.0),
         ("k31", 2, -1.0)]


def golden_name(variant, fmt, kint):
    return f"{variant}_f{fmt}" + ("_kint%g" % kint if kint >= 0 else "") + ".vtk"


def golden_state():
    return dict(np.load(os.path.join(GOLD, "state.npz")))


@pytest.mark.parametrize("variant,fmt,kint", CASES)
def test_format_matches_reference_writer(variant, fmt, kint):
    st = golden_state()
    p = default_params(variant)
    got = capi.vtk_format(fmt, st["x"], st["tri"], st["cA"], st["cC"], st["fau"], st["ea"], float(st["time"]), kint,
                          p.force_law, p.k_lin)
    with open(os.path.join(GOLD, golden_name(variant, fmt, kint)), "rb") as f:
        want = f.read()
    assert got == want


def test_format_edge_cases():
    """An empty mesh, and a zero strain (theta exactly 1) with zero bond vectors."""
    empty = capi.vtk_format(0, np.zeros((0, 3)), np.zeros((0, 3), np.int32), time=0.0)
    assert empty == b"# vtk DataFile Version 2.0\nCellBP Time: 0\nASCII\nDATASET UNSTRUCTURED_GRID\nPOINTS 0 double\n" \
                    b"CELLS 0 0\nCELL_TYPES 0\n"
    x = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])
    z = np.zeros((3, 3))
    t = capi.vtk_format(1, x, np.array([[0, 1, 2]]), None, None, z, np.zeros((3, 6)), time=1.5)
    assert b"SCALARS theta_e float 1\nLOOKUP_TABLE default\n1.000000\n1.000000\n1.000000\n" in t
    assert t.endswith(b"VECTORS fa_u float\n" + b"0.000000 0.000000 0.000000\n" * 3)
