"""GPU: asynchronous VTK frames (include/wcfe.h wcfe_frames_*) from engine state.  A frame
of the golden state equals the reference writer's own output (tests/golden/vtk) byte for
byte, from FP64 and mixed engines; frames written between steps, without synchronising,
hold the state of the moment they were queued."""
import math
import os

import numpy as np
import pytest

from wholecellfe_gb300 import capi, synth
from wholecellfe_gb300.params import default_params
from test_vtk_cpu import CASES, GOLD, golden_name, golden_state

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
def test_frames_match_reference_writer(tmp_path, prec):
    """FP64: the golden state's frames equal the reference writer's files.  Mixed (planar
    membranes only): the same state with z = 0, against the formatter that the CPU test pins
    to the reference."""
    st = golden_state()
    n = len(st["x"])
    zeros3 = np.zeros((n, 3))
    if prec == capi.PREC_MIXED:
        st["x"] = st["x"].copy()
        st["x"][:, 2] = 0.0   # +0: a float-float pair decodes -0.0 as +0.0 (hi + lo)
    e = capi.Engine(prec)
    fr = capi.Frames(e, slots=2, threads=2)
    cells = {}
    for variant in ("kMD", "k1", "k31"):
        cells[variant] = e.add_cell(st["x"], st["tri"], default_params(variant),
                                    state=(st["x"], zeros3, zeros3, st["ea"], st["cA"], st["cC"], st["fau"]))
    for variant, fmt, kint in CASES:
        fr.write(cells[variant], fmt, tmp_path / golden_name(variant, fmt, kint), time=float(st["time"]), kint=kint)
    fr.flush()
    fr.close()
    e.close()
    for variant, fmt, kint in CASES:
        if prec == capi.PREC_FP64:
            with open(os.path.join(GOLD, golden_name(variant, fmt, kint)), "rb") as f:
                want = f.read()
        else:
            p = default_params(variant)
            want = capi.vtk_format(fmt, st["x"], st["tri"], st["cA"], st["cC"], st["fau"], st["ea"],
                                   float(st["time"]), kint, p.force_law, p.k_lin)
        assert (tmp_path / golden_name(variant, fmt, kint)).read_bytes() == want, (variant, fmt, kint)


def test_frames_between_steps_hold_their_moment(tmp_path):
    x0, tri = synth.disk_mesh(800, seed=17)
    p = default_params("kMD")
    e = capi.Engine(capi.PREC_FP64)
    h = e.add_cell(x0, tri, p, state=synth.initial_state(x0, perturb=1.0, seed=17), t=0.2)
    fr = capi.Frames(e, slots=3)
    expect = []
    for k in range(5):
        e.step(7, 5e-5)
        fr.write(h, 2, tmp_path / f"f{k}.vtk")          # header time: the cell's clock
        fr.write(h, 1, tmp_path / f"s{k}.vtk", time=0.5)
        x, V, A, ea, cA, cC, fau = h.get_state()
        t, _ = h.clock()
        expect.append((capi.vtk_format(2, x, tri, cA, cC, fau, ea, t, -1.0, p.force_law, p.k_lin),
                       capi.vtk_format(1, x, tri, cA, cC, fau, ea, 0.5)))
    e.step(7, 5e-5)   # more steps queued behind the last frames
    fr.flush()
    fr.close()
    e.close()
    for k, (a, b) in enumerate(expect):
        assert (tmp_path / f"f{k}.vtk").read_bytes() == a
        assert (tmp_path / f"s{k}.vtk").read_bytes() == b
    assert math.isclose(float((tmp_path / "f0.vtk").read_bytes().split(b"\n")[1].split()[-1]), 0.2 + 7 * 5e-5,
                        rel_tol=1e-5)


def test_frames_report_write_errors(tmp_path):
    x0, tri = synth.disk_mesh(100, seed=2)
    e = capi.Engine(capi.PREC_FP64)
    h = e.add_cell(x0, tri, default_params("k1"))
    fr = capi.Frames(e)
    fr.write(h, 0, tmp_path / "missing_dir" / "a.vtk")
    with pytest.raises(capi.WcfeError):
        fr.flush()
    fr.write(h, 0, tmp_path / "ok.vtk")
    fr.flush()
    assert (tmp_path / "ok.vtk").read_bytes().startswith(b"# vtk DataFile Version 2.0")
    with pytest.raises(capi.WcfeError):
        fr.write(h, 3, tmp_path / "bad.vtk")
    fr.close()
    e.close()
