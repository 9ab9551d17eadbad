"""The oracle (oracle/wcfe_oracle.c) against golden vectors produced by the
reference's own functions (tests/golden/make_golden.py).  CPU only."""
import numpy as np

from conftest import relerr
from oracle import oracle_py as O
from wholecellfe_gb300.params import default_params

TOL = 1e-13   # the restatement follows the reference's operation order; the residual is rounding


def _setup(g):
    p = default_params(g["variant"])
    n = len(g["x0"])
    m = O.OMesh(g["tri"], n, g["vt_ptr"], g["vt_idx"], g["bnd"])
    ms = O.OMesh(g["tri_s"], len(g["Xs"]))
    return p, m, ms


def test_mesh_map_matches_reference(golden):
    from wholecellfe_gb300 import synth
    n = len(golden["x0"])
    ptr, idx = synth.vertex_triangle_map(n, golden["tri"])
    assert np.array_equal(ptr, golden["vt_ptr"]) and np.array_equal(idx, golden["vt_idx"])
    assert np.array_equal(synth.boundary_flags(n, golden["tri"]), golden["bnd"])


def test_predict(golden):
    Vh, xp = O.predict(golden["x"], golden["V"], golden["A"], float(golden["dt"]))
    assert relerr(Vh, golden["pred_Vh"]) <= TOL and relerr(xp, golden["pred_x"]) <= TOL


def test_area_tot(golden):
    p, m, _ = _setup(golden)
    assert relerr(O.area_tot(m, golden["pred_x"]), golden["area4"]) <= TOL


def test_calc_res_cell(golden):
    p, m, _ = _setup(golden)
    g = golden
    out = O.calc_res(m, g["x"], g["pred_x"], g["ea"], g["cA"], g["cC"], float(g["dt"]), 1, p, g["area4"][1:],
                     float(g["t_tot"]))
    for o, k in zip(out, ("res_Res", "res_Rea", "res_MM", "res_RA", "res_RC")):
        assert relerr(o, g[k]) <= TOL, k


def test_calc_res_substrate(golden):
    p, _, ms = _setup(golden)
    g = golden
    ps = p.copy()
    ps.mu = 1e6
    out = O.calc_res(ms, g["Xs"], g["xs_def"], np.zeros((len(g["Xs"]), 6)), None, None, float(g["dt"]), 2, ps, None,
                     float(g["t_tot"]))
    for o, k in zip(out[:3], ("sres_Res", "sres_Rea", "sres_MM")):
        assert relerr(o, g[k]) <= TOL, k


def test_boundary_forces(golden):
    p, m, _ = _setup(golden)
    g = golden
    assert relerr(O.force_fa(m, g["pred_x"], g["cC"], g["fau"], p), g["f_fa"]) <= TOL
    assert relerr(O.force_bending(m, g["pred_x"], p), g["f_bend"]) <= TOL
    assert relerr(O.force_area(m, g["pred_x"], g["area4"][0], p), g["f_area"]) <= TOL
    ap = O.force_ap(m, g["pred_x"], float(g["ap_dt"]), p, int(g["ap_call"]))
    assert np.count_nonzero(g["f_ap"]) > 0
    assert relerr(ap, g["f_ap"]) <= TOL


def test_update_fa_deformable_substrate(golden):
    p, m, ms = _setup(golden)
    g = golden
    cA, cC, fau, loc = O.update_fa(g["cA"], g["cC"], g["fau"], float(g["dt"]), g["x"], g["pred_x"], p, ms, g["Xs"],
                                   g["xs_def"])
    assert (loc >= 0).all()
    assert relerr(cC, g["ufa_cC"]) <= TOL and relerr(fau, g["ufa_fau"]) <= TOL and relerr(cA, g["ufa_cA"]) <= TOL


def test_update_forces(golden):
    p, m, _ = _setup(golden)
    g = golden
    for key, dtr in (("uf", float(g["dt"])), ("uf2", 0.4 * float(g["dt"]))):
        V, A, ea, _ = O.update_forces(m, g["x"], g["pred_x"], g["V"], g["pred_Vh"], g["A"], g["ea"], g["ufa_cA"],
                                      g["ufa_cC"], g["ufa_fau"], float(g["dt"]), dtr, float(g["t_tot"]), p,
                                      int(g["ap_call"]))
        assert relerr(V, g[key + "_V"]) <= TOL and relerr(A, g[key + "_A"]) <= TOL and relerr(ea, g[key + "_ea"]) <= TOL


def test_substrate_reaction(golden):
    p, m, ms = _setup(golden)
    g = golden
    F = O.force_fa_subs(ms, g["Xs"], g["xs_def"], g["ufa_cC"], g["pred_x"], g["ufa_fau"], m, p)
    assert relerr(F, g["fsub"]) <= TOL


def test_trajectories(golden):
    p, m, ms = _setup(golden)
    g = golden
    from wholecellfe_gb300 import synth
    starts = {"traj0": (synth.initial_state(g["x0"]), 0.0, 0),
              "traj1": ((g["x"], g["V"], g["A"], g["ea"], g["cA"], g["cC"], g["fau"]), float(g["t_tot"]),
                        int(g["ap_call"]))}
    for key, (st, t0, c0) in starts.items():
        c = O.OCell(m, st, p, t=t0, ap_call=c0, sub=ms, Xs=g["Xs"])
        c.steps(40, float(g["dt"]))
        out = c.state()
        for k, a, s0 in zip(("x", "V", "A", "ea", "cA", "cC", "fau"), out, st):
            # compare the change over the trajectory, so the large initial positions do not hide it
            assert relerr(a - s0, g[f"{key}_{k}"] - s0) <= 1e-12, (key, k)
        assert c.t == float(g[f"{key}_t"]) and c.ap_call == int(g[f"{key}_call"])


def test_philox_known_answers():
    """Philox4x32-10 known-answer vectors (Random123 kat_vectors)."""
    import ctypes as C
    L = O.lib()
    cases = [((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
             ((0xffffffff,) * 4, (0xffffffff, 0xffffffff), (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
             ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
              (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]
    for ctr, key, want in cases:
        c = (C.c_uint32 * 4)(*ctr)
        k = (C.c_uint32 * 2)(*key)
        o = (C.c_uint32 * 4)()
        L.wo_philox4x32_10(c, k, o)
        assert tuple(o) == want


def test_oracle_per_element_mu_uniform_equals_params_mu():
    """The per-element modulus of the oracle with every element at params.mu is the
    uniform-modulus oracle, bit for bit (the extension does not move the pinned path)."""
    from wholecellfe_gb300 import synth
    from wholecellfe_gb300.params import default_params
    x0, tri = synth.disk_mesh(300, seed=3)
    p = default_params("k1")
    st = synth.initial_state(x0, perturb=1.0, seed=3)
    a = O.OCell(O.OMesh(tri, len(x0)), st, p, t=0.3)
    b = O.OCell(O.OMesh(tri, len(x0), mu_e=np.full(len(tri), p.mu)), st, p, t=0.3)
    a.steps(5, 5e-5)
    b.steps(5, 5e-5)
    for u, w in zip(a.state(), b.state()):
        assert np.array_equal(u, w)


def test_shipped_meshes(shipped):
    """The oracle's step on the reference's own meshes and substrate (cellBP/scripts),
    against the reference's step loop: 20 steps from a moving state, 200 from rest."""
    from conftest import SHIPPED_FINAL, SHIPPED_STATE, shipped_runs
    g = shipped
    p = default_params(g["variant"])
    ms = O.OMesh(g["tri_s"], len(g["Xs"]))
    for m, kind, st, t0, c0, n in shipped_runs(g):
        mesh = O.OMesh(g[f"m{m}_tri"], len(g[f"m{m}_x0"]))
        c = O.OCell(mesh, st, p, t=t0, ap_call=c0, sub=ms, Xs=g["Xs"])
        c.steps(n, float(g["dt"]))
        out = dict(zip(SHIPPED_STATE, c.state()))
        s0 = dict(zip(SHIPPED_STATE, st))
        for k in SHIPPED_FINAL:
            assert relerr(out[k] - s0[k], g[f"m{m}_{kind}_{k}"] - s0[k]) <= 1e-12, (m, kind, k)
        assert c.t == float(g[f"m{m}_{kind}_t"]) and c.ap_call == int(g[f"m{m}_{kind}_call"])
