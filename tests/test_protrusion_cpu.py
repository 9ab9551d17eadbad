"""The radial protrusion driver of the oracle (wcfe_params.protrude_v): from rest, one
step moves every boundary vertex exactly one step's travel radially outward and leaves
the interior in place.  CPU only."""
import numpy as np

from oracle import oracle_py as O
from wholecellfe_gb300 import synth


def test_first_step_moves_boundary_radially():
    x0, tri, p, rho = synth.protruding_cell()
    bnd = synth.boundary_flags(len(x0), tri).astype(bool)
    c = O.OCell(O.OMesh(tri, len(x0)), synth.initial_state(x0), p, rho_w=rho)
    dt = 5e-5
    c.steps(1, dt)
    d = c.state()[0] - x0
    assert np.all(d[~bnd] == 0.0)
    r = x0[bnd, :2] / np.linalg.norm(x0[bnd, :2], axis=1)[:, None]
    np.testing.assert_allclose(d[bnd, :2], 0.010 * r, rtol=0, atol=1e-15)
    assert np.all(d[:, 2] == 0.0)


def test_protrusion_off_is_the_reference_driver():
    x0, tri, p, rho = synth.protruding_cell(n_target=400)
    st = synth.initial_state(x0, perturb=1.0, seed=3)
    q = p.copy()
    q.protrude_v = 0.0
    a = O.OCell(O.OMesh(tri, len(x0)), st, q, rho_w=rho)
    a.steps(3, 5e-5)
    b = O.OCell(O.OMesh(tri, len(x0)), st, p, rho_w=rho)
    b.steps(3, 5e-5)
    bnd = synth.boundary_flags(len(x0), tri).astype(bool)
    assert not np.array_equal(a.state()[0][bnd], b.state()[0][bnd])
