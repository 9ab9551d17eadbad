"""GPU: a cell coupled to a deformable substrate simulated by the same engine (A10:
calculateForce_FA_subs UL:1305-1475 and the substrate overload of
updateForces_Explicit UL:429-504, with updateFA UL:2026-2174 on the moving
substrate) against the oracle's coupled step, FP64, 1e-9."""
import numpy as np
import pytest

from oracle import oracle_py as O
from wholecellfe_gb300 import capi, synth
from wholecellfe_gb300.params import default_params

pytestmark = pytest.mark.gpu
DT = 5e-5


def _oracle_coupled(xc0, tric, stc, p, rho, xs0, tris, sts, nsteps, t0):
    mc = O.OMesh(tric, len(xc0))
    ms = O.OMesh(tris, len(xs0))
    Xc, Vc, Ac, eac, cA, cC, fau = (np.array(a, dtype=np.float64) for a in stc)
    Xs, Vs, As, eas = (np.array(a, dtype=np.float64) for a in (sts[0], sts[1], sts[2], sts[3]))
    t, call = t0, 0
    for _ in range(nsteps):
        Vhs, xs = O.predict(Xs, Vs, As, DT)
        Vh, xc = O.predict(Xc, Vc, Ac, DT)
        cA, cC, fau, _ = O.update_fa(cA, cC, fau, DT, Xc, xc, p, sub=ms, Xs=Xs, xs=xs)
        Vc, Ac, eac, _ = O.update_forces(mc, Xc, xc, Vc, Vh, Ac, eac, cA, cC, fau, DT, DT, t, p, call, rho)
        Vs, As, eas = O.update_forces_subs(ms, Xs, xs, Vs, Vhs, As, eas, DT, DT, t, fau, cC, xc, mc, p, rho)
        Xc, Xs = xc, xs
        t += DT
        call += 1
    return (Xc, Vc, Ac, eac, cA, cC, fau), (Xs, Vs, As, eas)


def _rel(a, b, floor=1e-300):
    return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), floor))


@pytest.mark.parametrize("sub_perturb", [0.0, 1.0])
def test_coupled_substrate_matches_oracle(sub_perturb):
    xc0, tric = synth.disk_mesh(600, seed=61)
    p = default_params("k31")
    stc = synth.initial_state(xc0, perturb=1.0, seed=61)
    rho = np.where(np.random.default_rng(1).random(len(xc0)) < 0.4, p.rho_i_max, 0.0)
    xs0, tris = synth.square_substrate(30.0, 20)
    sts = synth.initial_state(xs0, perturb=sub_perturb, seed=62)
    sts = (sts[0], sts[1] * 1e-3, sts[2] * 1e-3, sts[3] * 1e-3) + tuple(sts[4:])
    ps = default_params("k31")
    ps.mu = 1e6
    e = capi.Engine(capi.PREC_FP64)
    hc = e.add_cell(xc0, tric, p, state=stc, t=0.3)
    hc.set_integrins(rho)
    hs = e.add_cell(xs0, tris, ps, state=sts, t=0.3)
    hc.couple_substrate(hs, margin=1.0)
    nsteps = 30
    e.step(nsteps, DT)
    gc, gs = hc.get_state(), hs.get_state()
    assert hc.status() == 0 and hs.status() == 0
    e.close()
    rc, rs = _oracle_coupled(xc0, tric, stc, p, rho, xs0, tris, sts, nsteps, 0.3)
    assert _rel(gc[0] - stc[0], rc[0] - stc[0]) < 1e-9
    for k in (1, 3, 5, 6):
        assert _rel(gc[k], rc[k], 1e-12) < 1e-9, k
    # the substrate moved under the bond reactions, and matches
    us = rs[0] - xs0
    assert np.max(np.abs(us)) > 0
    assert _rel(gs[0] - xs0, us) < 1e-9
    assert _rel(gs[1], rs[1], 1e-12) < 1e-9
    assert _rel(gs[3], rs[3], 1e-12) < 1e-9


def test_coupling_refused_on_other_paths_and_uncouples():
    xc0, tric = synth.disk_mesh(200, seed=63)
    xs0, tris = synth.square_substrate(30.0, 10)
    p = default_params("k1")
    ps = default_params("k1")
    ps.mu = 1e6
    e = capi.Engine(capi.PREC_FP64)
    hc = e.add_cell(xc0, tric, p, state=synth.initial_state(xc0))
    hs = e.add_cell(xs0, tris, ps, state=synth.initial_state(xs0))
    hc.couple_substrate(hs)
    with pytest.raises(capi.WcfeError):
        e.step_implicit(1, DT)
    with pytest.raises(capi.WcfeError):
        e.predict_all(DT, np.zeros((e.total_vertices(), 3)))
    hc.couple_substrate(None)
    e.step_implicit(1, DT)
    e.close()
    m = capi.Engine(capi.PREC_MIXED)
    a = m.add_cell(xc0, tric, p, state=synth.initial_state(xc0))
    b = m.add_cell(xs0, tris, ps, state=synth.initial_state(xs0))
    with pytest.raises(capi.WcfeError):
        a.couple_substrate(b)
    m.close()
