"""The oracle against the reference compiled from its sources (oracle/_ref), on
fresh seeded inputs.  Runs only where oracle/build_ref.sh has built the
reference (the container that holds the reference sources); skipped elsewhere."""
import numpy as np
import pytest

from conftest import relerr
from oracle import oracle_py as O
from wholecellfe_gb300 import synth
from wholecellfe_gb300.params import default_params, kint_for


@pytest.mark.parametrize("variant", ["kMD", "k1", "k31"])
@pytest.mark.parametrize("seed", [21, 22])
def test_oracle_matches_reference_build(variant, seed):
    if not O.ref_available(variant):
        pytest.skip("reference not built here (oracle/build_ref.sh)")
    R = O.Ref(variant)
    p = default_params(variant)
    x0, tri = synth.disk_mesh(500, seed=seed)
    n = len(x0)
    hc = R.mesh(tri, n)
    ptr, idx, bnd = R.mesh_map(hc, n, len(tri))
    m = O.OMesh(tri, n, ptr, idx, bnd)
    Xs, tri_s = synth.square_substrate(40.0, 16)
    hs = R.mesh(tri_s, len(Xs))
    ms = O.OMesh(tri_s, len(Xs))
    st = synth.initial_state(x0, perturb=1.0, seed=seed)
    s_ref, t_ref, c_ref = R.steps(hc, st, hs, Xs, kint_for(variant), 5e-5, 25, 1.9, p.seed, p.stream, 3)
    c = O.OCell(m, st, p, t=1.9, ap_call=3, sub=ms, Xs=Xs)
    c.steps(25, 5e-5)
    for a, b, s0 in zip(c.state(), s_ref, st):
        assert relerr(a - s0, b - s0) <= 1e-12
    assert c.t == t_ref and c.ap_call == c_ref


@pytest.mark.parametrize("variant", ["kMD", "k31"])
def test_oracle_matches_reference_build_on_an_annulus(variant):
    """A mesh with two boundary loops (the inner one oriented the other way): the
    boundary scan, the actin push, bending and the area constraint of both loops."""
    if not O.ref_available(variant):
        pytest.skip("reference not built here (oracle/build_ref.sh)")
    R = O.Ref(variant)
    p = default_params(variant)
    x0, tri = synth.annulus_mesh(700, 0.35, seed=23)
    n = len(x0)
    hc = R.mesh(tri, n)
    ptr, idx, bnd = R.mesh_map(hc, n, len(tri))
    m = O.OMesh(tri, n, ptr, idx, bnd)
    r = np.hypot(x0[:, 0], x0[:, 1])
    assert bnd[r < 5.0].any() and bnd[r > 9.0].any()
    Xs, tri_s = synth.square_substrate(40.0, 16)
    hs = R.mesh(tri_s, len(Xs))
    ms = O.OMesh(tri_s, len(Xs))
    st = synth.initial_state(x0, perturb=1.0, seed=5)
    s_ref, t_ref, c_ref = R.steps(hc, st, hs, Xs, kint_for(variant), 5e-5, 25, 1.9, p.seed, p.stream, 3)
    c = O.OCell(m, st, p, t=1.9, ap_call=3, sub=ms, Xs=Xs)
    c.steps(25, 5e-5)
    for a, b, s0 in zip(c.state(), s_ref, st):
        assert relerr(a - s0, b - s0) <= 1e-12
    assert c.t == t_ref and c.ap_call == c_ref


@pytest.mark.parametrize("variant", ["kMD", "k1", "k31"])
@pytest.mark.parametrize("t0,dt", [(1.99940, 5e-5), (1.996, 2e-4)])
def test_oracle_matches_reference_across_the_active_stress_switch(variant, t0, dt):
    """Runs that cross t = 2 s, where the active stress stops ramping and holds
    (UL:744-757), at two time steps."""
    if not O.ref_available(variant):
        pytest.skip("reference not built here (oracle/build_ref.sh)")
    R = O.Ref(variant)
    p = default_params(variant)
    x0, tri = synth.disk_mesh(400, seed=29)
    n = len(x0)
    hc = R.mesh(tri, n)
    ptr, idx, bnd = R.mesh_map(hc, n, len(tri))
    m = O.OMesh(tri, n, ptr, idx, bnd)
    Xs, tri_s = synth.square_substrate(40.0, 16)
    hs = R.mesh(tri_s, len(Xs))
    ms = O.OMesh(tri_s, len(Xs))
    st = synth.initial_state(x0, perturb=1.0, seed=7)
    nsteps = 25
    assert t0 < 2.0 < t0 + nsteps * dt
    s_ref, t_ref, c_ref = R.steps(hc, st, hs, Xs, kint_for(variant), dt, nsteps, t0, p.seed, p.stream, 0)
    c = O.OCell(m, st, p, t=t0, ap_call=0, sub=ms, Xs=Xs)
    c.steps(nsteps, dt)
    for a, b, s0 in zip(c.state(), s_ref, st):
        assert relerr(a - s0, b - s0) <= 1e-12
    assert c.t == t_ref and c.ap_call == c_ref
