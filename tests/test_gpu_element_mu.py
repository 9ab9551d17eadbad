"""Per-element shear modulus (config 2's log-normal E per element; an extension,
the reference has one mu per material, UL:721-728): the FP64 engine against the
oracle carrying the same per-element moduli, the mixed form against the FP64
form, and None restoring the uniform modulus."""
import numpy as np
import pytest

from oracle import oracle_py as O
from wholecellfe_gb300 import capi, synth
from wholecellfe_gb300.params import default_params

pytestmark = pytest.mark.gpu
DT = 5e-5


def _lognormal_mu(nt, median, sigma, seed):
    return median * np.exp(sigma * np.random.default_rng(seed).standard_normal(nt))


def test_fp64_per_element_mu_matches_oracle():
    x0, tri = synth.disk_mesh(1500, seed=41)
    p = default_params("k31")
    p.force_law, p.poly_k0, p.poly_x0, p.linear_norm2d = 2, 31000.0, 0.005, 0
    st = synth.initial_state(x0, perturb=1.0, seed=41)
    mu = _lognormal_mu(len(tri), p.mu, 0.3, 5)
    e = capi.Engine(capi.PREC_FP64)
    h = e.add_cell(x0, tri, p, state=st, t=0.3)
    h.set_element_mu(mu)
    e.step(20, DT)
    got = h.get_state()
    e.close()
    oc = O.OCell(O.OMesh(tri, len(x0), mu_e=mu), st, p, t=0.3)
    oc.steps(20, DT)
    ref = oc.state()
    u = ref[0] - st[0]
    assert np.max(np.abs(got[0] - ref[0])) / np.max(np.abs(u)) < 1e-9
    for k in (1, 3, 5, 6):
        assert np.max(np.abs(got[k] - ref[k])) <= 1e-9 * max(np.max(np.abs(ref[k])), 1e-12), k
    # a different modulus field changes the result
    oc2 = O.OCell(O.OMesh(tri, len(x0)), st, p, t=0.3)
    oc2.steps(20, DT)
    assert np.max(np.abs(oc2.state()[0] - ref[0])) > 1e-6 * np.max(np.abs(u))


def test_mixed_per_element_mu_matches_fp64_and_reset():
    x0, tri = synth.disk_mesh(3000, seed=42)
    p = default_params("k1")
    mu = _lognormal_mu(len(tri), p.mu, 0.3, 6)
    st = synth.initial_state(x0)
    out = {}
    for prec in (capi.PREC_FP64, capi.PREC_MIXED):
        e = capi.Engine(prec)
        h = e.add_cell(x0, tri, p, state=st, t=0.3)
        h.set_element_mu(mu)
        e.step(300, DT)
        out[prec] = h.get_state()
        assert h.status() == 0
        e.close()
    u = out[capi.PREC_FP64][0] - x0
    err = np.max(np.abs(out[capi.PREC_MIXED][0] - out[capi.PREC_FP64][0])) / np.max(np.abs(u))
    assert err <= 1e-6, err
    # None restores the uniform modulus: bit-identical to a cell that never had one
    res = []
    for with_reset in (False, True):
        e = capi.Engine(capi.PREC_FP64)
        h = e.add_cell(x0, tri, p, state=st, t=0.3)
        if with_reset:
            h.set_element_mu(mu)
            h.set_element_mu(None)
        e.step(10, DT)
        res.append(h.get_state()[0])
        e.close()
    assert np.array_equal(res[0], res[1])
