"""GPU parity: the sm_103a path through the C ABI against the reference's own
outputs (golden fixtures) and against the oracle on fresh seeded inputs.

Tolerance: 1e-9 norm-wise relative error (max|gpu - ref| / max|ref|), the bar
the plain FP64 form must meet; trajectories compare the change of each state
array over the run.  Integer bookkeeping is compared exactly elsewhere
(test_capi_cpu.py); here bit-identity is asserted where the arithmetic is the
same by construction (batched vs alone, graphs vs eager, repeated runs).
"""
import numpy as np
import pytest

from conftest import relerr
from oracle import oracle_py as O
from wholecellfe_gb300 import capi, synth
from wholecellfe_gb300.params import default_params

pytestmark = pytest.mark.gpu
TOL = 1e-9


@pytest.fixture(scope="module")
def eng():
    e = capi.Engine(capi.PREC_FP64)
    yield e
    e.close()


# Absolute floors per state array (x [um], V [um/s], A [um/s^2], ea, c_A, c_C, fa_u [um]):
# a change smaller than the floor is at the rounding-noise level of that quantity in the
# reference itself.  The strain increment of one step is 1/2 (I - be^-1) with be = I + O(1e-8),
# a cancellation that leaves ~1e-16 absolute noise per step in the reference's own formula,
# hence its floor 1e-4 (1e-13 absolute at the 1e-9 bar).  Above the floor the bar is relative.
FLOORS = (1e-5, 1e-5, 1e-3, 1e-4, 1e-6, 1e-6, 1e-6)
NAMES = ("x", "V", "A", "ea", "c_A", "c_C", "fa_u")


class TrajErr(float):
    """The worst relative error, remembering which array it came from (shown on failure)."""
    where = ""

    def __repr__(self):
        return f"{float(self):.3e} (worst array: {self.where})"


def traj_err(got, want, start):
    """max over arrays of max|gpu - ref| / max(max|ref - start|, floor)."""
    worst, where = 0.0, ""
    for a, b, s0, fl, nm in zip(got, want, start, FLOORS, NAMES):
        a = np.asarray(a, dtype=np.float64); b = np.asarray(b, dtype=np.float64)
        d = float(np.max(np.abs(a - b)))
        s = max(float(np.max(np.abs(b - s0))), fl)
        if d / s > worst:
            worst, where = d / s, nm
    r = TrajErr(worst)
    r.where = where
    return r


# ---------------------------------------------------------------- golden ----
def test_golden_drop_in_pieces(eng, golden):
    g = golden
    p = default_params(g["variant"])
    n = len(g["x0"])
    st = (g["x"], g["V"], g["A"], g["ea"], g["cA"], g["cC"], g["fau"])
    c = eng.add_cell(g["x"], g["tri"], p, vt_ptr=g["vt_ptr"], vt_idx=g["vt_idx"], bnd=g["bnd"], state=st,
                     t=0.0, ap_calls=int(g["ap_call"]))
    try:
        c.set_substrate(g["Xs"], g["tri_s"], g["xs_def"])
        # driverVelocities_Explicit + predict
        vh, xp = c.predict(float(g["dt"]))
        assert relerr(vh, g["pred_Vh"]) <= TOL and relerr(xp, g["pred_x"]) <= TOL
        # calculateRes (cell) with the reference's centroid
        out = c.eval_residual(g["x"], g["pred_x"], float(g["dt"]), g["area4"][1:], float(g["t_tot"]))
        for o, k in zip(out, ("res_Res", "res_Rea", "res_MM", "res_RA", "res_RC")):
            assert relerr(o, g[k]) <= TOL, k
        # forces at the predicted positions
        FFA, FAP, FB, FAR, a4 = c.eval_forces(g["pred_x"], float(g["dt"]))
        assert relerr(a4, g["area4"]) <= TOL
        assert relerr(FFA, g["f_fa"]) <= TOL and relerr(FB, g["f_bend"]) <= TOL and relerr(FAR, g["f_area"]) <= TOL
        FFA2, FAP2, _, _, _ = c.eval_forces(g["pred_x"], float(g["ap_dt"]))
        assert np.count_nonzero(g["f_ap"]) > 0 and relerr(FAP2, g["f_ap"]) <= TOL
        # updateFA against a deformable substrate, then updateForces_Explicit
        c.set_state(*st)
        c.predict(float(g["dt"]))
        c.update_fa(float(g["dt"]), g["pred_x"], X=g["x"], Xs=g["Xs"], xs=g["xs_def"])
        s = c.get_state()
        assert relerr(s[5], g["ufa_cC"]) <= TOL and relerr(s[6], g["ufa_fau"]) <= TOL
        c.update_forces(float(g["dt"]), float(g["dt"]), float(g["t_tot"]))
        s = c.get_state()
        assert relerr(s[0], g["pred_x"]) == 0.0
        assert relerr(s[1], g["uf_V"]) <= TOL and relerr(s[2], g["uf_A"]) <= TOL
        assert relerr(s[3] - g["ea"], g["uf_ea"] - g["ea"]) <= TOL
        assert c.status() == 0
    finally:
        c.destroy()


def test_golden_dt_real_below_half_dt(eng, golden):
    """updateForces_Explicit's second velocity branch (dt_real <= dt/2, UL:625-626)."""
    g = golden
    p = default_params(g["variant"])
    st = (g["x"], g["V"], g["A"], g["ea"], g["ufa_cA"], g["ufa_cC"], g["ufa_fau"])
    c = eng.add_cell(g["x"], g["tri"], p, state=st, ap_calls=int(g["ap_call"]))
    try:
        c.predict(float(g["dt"]))   # V_hlf and x_pred stay on the device; x_pred is the golden x_new
        c.update_forces(float(g["dt"]), 0.4 * float(g["dt"]), float(g["t_tot"]))
        s = c.get_state()
        assert relerr(s[1], g["uf2_V"]) <= TOL and relerr(s[2], g["uf2_A"]) <= TOL
    finally:
        c.destroy()


def test_golden_trajectories(eng, golden):
    g = golden
    p = default_params(g["variant"])
    starts = {"traj0": (synth.initial_state(g["x0"]), 0.0, 0),
              "traj1": ((g["x"], g["V"], g["A"], g["ea"], g["cA"], g["cC"], g["fau"]), float(g["t_tot"]),
                        int(g["ap_call"]))}
    for key, (st, t0, c0) in starts.items():
        c = eng.add_cell(st[0], g["tri"], p, vt_ptr=g["vt_ptr"], vt_idx=g["vt_idx"], bnd=g["bnd"], state=st, t=t0,
                         ap_calls=c0)
        c.set_substrate(g["Xs"], g["tri_s"])
        eng.step_cells([c], 40, float(g["dt"]))
        got = c.get_state()
        want = [g[f"{key}_{k}"] for k in ("x", "V", "A", "ea", "cA", "cC", "fau")]
        # kMD from rest is the reference's noise-driven regime (the MD table jumps from 0 to
        # -7.2 pN at zero extension, so rounding-noise bond vectors decide forces): there the
        # bar is 1e-6; every other trajectory is held to 1e-9.
        tol = 1e-6 if (g["variant"] == "kMD" and key == "traj0") else TOL
        assert traj_err(got, want, st) <= tol, key
        t, calls = c.clock()
        assert calls == int(g[f"{key}_call"])
        assert abs(t - float(g[f"{key}_t"])) <= 1e-15 * max(1.0, abs(t))
        c.destroy()


def test_shipped_meshes(eng, shipped):
    """The FP64 engine on the reference's own meshes (the three COMSOL-edited disks of
    cellBP/scripts over the shipped 100 um substrate, read as read_ecomsol reads them)
    against the reference's step loop: 20 steps from a moving state (every variant) and
    200 steps from rest (k1, k31).  The change of each state array over the run is held
    to 1e-9 relative with no absolute floor; the FP64 form's own rounding noise on these
    runs (the same runs on rigidly translated meshes) is at most 7e-11 of the change."""
    from conftest import SHIPPED_FINAL, SHIPPED_STATE, shipped_runs
    g = shipped
    p = default_params(g["variant"])
    for m, kind, st, t0, c0, n in shipped_runs(g):
        c = eng.add_cell(st[0], g[f"m{m}_tri"], p, state=st, t=t0, ap_calls=c0)
        c.set_substrate(g["Xs"], g["tri_s"])
        eng.step_cells([c], n, float(g["dt"]))
        got = dict(zip(SHIPPED_STATE, c.get_state()))
        s0 = dict(zip(SHIPPED_STATE, st))
        for k in SHIPPED_FINAL:
            err = relerr(got[k] - s0[k], g[f"m{m}_{kind}_{k}"] - s0[k])
            assert err <= TOL, (m, kind, k, err)
        t, calls = c.clock()
        assert calls == int(g[f"m{m}_{kind}_call"])
        assert abs(t - float(g[f"m{m}_{kind}_t"])) <= 1e-15 * max(1.0, abs(t))
        c.destroy()


def test_protruding_cell_against_oracle(eng):
    """The single-cell workload with a protruding edge (2,044 vertices, E = 1 kPa and
    nu = 0.45 mapped to mu, 0.1 um thickness, 600 integrins of 1 pN/nm with a 20 nm rest
    length, boundary driven outward 10 nm per step) over 200 steps: the FP64 engine against
    the oracle's restatement (the driver and the rest length are extensions, so this parity
    is to the oracle only), 1e-9 of each array's change, no floor."""
    x0, tri, p, rho = synth.protruding_cell()
    st = synth.initial_state(x0)
    c = eng.add_cell(x0, tri, p, state=st)
    c.set_integrins(rho)
    eng.step_cells([c], 200, 5e-5)
    got = c.get_state()
    oc = O.OCell(O.OMesh(tri, len(x0)), st, p, rho_w=rho)
    oc.steps(200, 5e-5)
    want = oc.state()
    for k, (a, b, s0) in enumerate(zip(got, want, st)):
        if np.max(np.abs(b - s0)) == 0:
            assert np.array_equal(a, b), k
            continue
        assert relerr(a - s0, b - s0) <= TOL, (k, relerr(a - s0, b - s0))
    c.destroy()


# ---------------------------------------------------------------- oracle ----
@pytest.mark.parametrize("variant", ["kMD", "k1", "k31"])
@pytest.mark.parametrize("n", [120, 2000])
def test_steps_match_oracle(eng, variant, n):
    """From a moving, pre-strained state with bonds already formed.  (From rest, the
    MD table's jump at zero extension -- force 0 at D = 0 but py[0] = -7.2 pN as
    D -> 0+, UL:1258-1264 -- turns rounding noise in the interior bond vectors into
    O(1) forces, in the reference as much as here; kMD is therefore compared from
    moving states, see test_md_law_from_rest_is_noise_driven.)"""
    x0, tri = synth.disk_mesh(n, seed=n + 1)
    p = default_params(variant)
    st = synth.initial_state(x0, perturb=1.0, seed=n)
    c = eng.add_cell(x0, tri, p, state=st, t=1.99, ap_calls=5)
    eng.step_cells([c], 60, 5e-5)
    got = c.get_state()
    oc = O.OCell(O.OMesh(tri, len(x0)), st, p, t=1.99, ap_call=5)
    oc.steps(60, 5e-5)
    assert traj_err(got, oc.state(), st) <= TOL
    c.destroy()


def test_long_trajectory_200_steps(eng):
    """The plain form over a config-1-sized cell (about 2000 vertices) for 200 steps."""
    x0, tri = synth.disk_mesh(2000, seed=1)
    p = default_params("k1")
    st = synth.initial_state(x0)
    c = eng.add_cell(x0, tri, p, state=st)
    eng.step_cells([c], 200, 5e-5)
    oc = O.OCell(O.OMesh(tri, len(x0)), st, p)
    oc.steps(200, 5e-5)
    assert traj_err(c.get_state(), oc.state(), st) <= TOL
    c.destroy()


def test_extension_laws_match_oracle(eng):
    """Polynomial stiffening law, rest length and AP off: the config extensions."""
    x0, tri = synth.disk_mesh(700, seed=9)
    for law, rest in ((2, 0.0), (2, 0.002), (0, 0.02)):
        p = default_params("k31")
        p.force_law, p.rest_len, p.ap_enable, p.linear_norm2d = law, rest, 0, 0
        st = synth.initial_state(x0, perturb=1.0, seed=law)
        c = eng.add_cell(x0, tri, p, state=st)
        eng.step_cells([c], 30, 5e-5)
        oc = O.OCell(O.OMesh(tri, len(x0)), st, p)
        oc.steps(30, 5e-5)
        assert traj_err(c.get_state(), oc.state(), st) <= TOL, (law, rest)
        c.destroy()


def test_custom_one_ring_order_and_small_patches(eng):
    """A vertex->triangle map in non-ascending order (as El Topo's incremental edits leave it)
    and tiny patches: results still match the oracle fed the same map."""
    x0, tri = synth.disk_mesh(300, seed=2)
    n = len(x0)
    vt_ptr, vt_idx = synth.vertex_triangle_map(n, tri)
    rng = np.random.default_rng(0)
    vt_idx = vt_idx.copy()
    for v in range(n):
        seg = vt_idx[vt_ptr[v]:vt_ptr[v + 1]]
        rng.shuffle(seg)
        vt_idx[vt_ptr[v]:vt_ptr[v + 1]] = seg
    p = default_params("kMD")
    st = synth.initial_state(x0, perturb=1.0, seed=1)
    e2 = capi.Engine(capi.PREC_FP64)
    e2.set_shape(64, 32)
    c = e2.add_cell(x0, tri, p, vt_ptr=vt_ptr, vt_idx=vt_idx, state=st)
    e2.step(25, 5e-5)
    oc = O.OCell(O.OMesh(tri, n, vt_ptr, vt_idx), st, p)
    oc.steps(25, 5e-5)
    assert traj_err(c.get_state(), oc.state(), st) <= TOL
    e2.close()


def test_two_triangle_cell(eng):
    """Smallest well-posed mesh: a quad of two triangles, every vertex on the boundary.
    (A single triangle puts its centroid on the cell centroid, where the reference's
    active-stress direction a0 is 0/0, UL:875-877.)"""
    x = np.array([[0.0, 0, 0], [1.0, 0, 0], [1.1, 0.9, 0], [0.0, 1.0, 0]])
    tri = np.array([[0, 1, 2], [0, 2, 3]], np.int32)
    p = default_params("k1")
    st = synth.initial_state(x, perturb=1.0, seed=3)
    c = eng.add_cell(x, tri, p, state=st)
    eng.step_cells([c], 5, 5e-5)
    oc = O.OCell(O.OMesh(tri, 4), st, p)
    oc.steps(5, 5e-5)
    assert traj_err(c.get_state(), oc.state(), st) <= TOL
    c.destroy()


# ------------------------------------------------------- batching / systems ----
def test_batched_uneven_cells_equal_alone():
    """Cells of different sizes and force laws in one launch give bit-identical
    results to each cell stepped alone."""
    rng = np.random.default_rng(5)
    sizes = [150, 900, 60, 2500, 400]
    cells = []
    for i, n in enumerate(sizes):
        x0, tri = synth.disk_mesh(n, seed=100 + i)
        p = default_params(["kMD", "k1", "k31"][i % 3])
        p.stream = i
        cells.append((x0, tri, p, synth.initial_state(x0, perturb=1.0, seed=i)))
    eb = capi.Engine(capi.PREC_FP64)
    hs = [eb.add_cell(x, t, p, state=s, t=0.1, ap_calls=3) for x, t, p, s in cells]
    eb.step(20, 5e-5)
    batched = [h.get_state() for h in hs]
    eb.close()
    for (x, t, p, s), b in zip(cells, batched):
        ea = capi.Engine(capi.PREC_FP64)
        h = ea.add_cell(x, t, p, state=s, t=0.1, ap_calls=3)
        ea.step(20, 5e-5)
        alone = h.get_state()
        ea.close()
        for u, w in zip(b, alone):
            assert np.array_equal(u, w)
    assert rng is not None


def test_graphs_equal_eager_and_deterministic():
    x0, tri = synth.disk_mesh(1500, seed=11)
    p = default_params("kMD")
    st = synth.initial_state(x0, perturb=1.0, seed=11)
    outs = []
    for graphs in (False, True, True):
        e = capi.Engine(capi.PREC_FP64)
        e.set_graphs(graphs)
        h = e.add_cell(x0, tri, p, state=st)
        e.step(21, 5e-5)
        outs.append(h.get_state())
        e.close()
    for o in outs[1:]:
        for u, w in zip(o, outs[0]):
            assert np.array_equal(u, w)


def test_nan_flag_isolated_to_its_cell():
    """A NaN injected into one cell's host state sets that cell's status bit only;
    the other cell in the same launches is unaffected (bit-identical)."""
    x0, tri = synth.disk_mesh(400, seed=12)
    p = default_params("k1")
    st = synth.initial_state(x0, perturb=1.0, seed=12)
    bad = list(st)
    bad[1] = st[1].copy()
    bad[1][7, 0] = np.nan
    e = capi.Engine(capi.PREC_FP64)
    good = e.add_cell(x0, tri, p, state=st)
    sick = e.add_cell(x0, tri, p, state=tuple(bad))
    e.step(3, 5e-5)
    assert good.status() == 0 and sick.status() == 1
    ref = capi.Engine(capi.PREC_FP64)
    alone = ref.add_cell(x0, tri, p, state=st)
    ref.step(3, 5e-5)
    for u, w in zip(good.get_state(), alone.get_state()):
        assert np.array_equal(u, w)
    e.close()
    ref.close()


def test_autotune_keeps_state_and_results():
    x0, tri = synth.disk_mesh(3000, seed=13)
    p = default_params("kMD")
    st = synth.initial_state(x0, perturb=1.0, seed=13)
    e = capi.Engine(capi.PREC_FP64)
    h = e.add_cell(x0, tri, p, state=st)
    e.autotune(5e-5, 2)
    s0 = h.get_state()
    for u, w in zip(s0, st):
        assert np.array_equal(u, np.asarray(w, dtype=np.float64))
    e.step(10, 5e-5)
    oc = O.OCell(O.OMesh(tri, len(x0)), st, p)
    oc.steps(10, 5e-5)
    assert traj_err(h.get_state(), oc.state(), st) <= TOL
    e.close()


def test_large_cell_properties():
    """A config-2-sized cell (20k vertices, the polynomial stiffening law k0 = 31 pN/nm,
    x0 = 5 nm, from rest): the state stays finite, positions keep z = 0, the run is
    repeatable bit for bit, and 5 steps match the oracle."""
    x0, tri = synth.disk_mesh(20000, seed=2)
    p = default_params("k31")
    p.force_law, p.linear_norm2d = 2, 0
    st = synth.initial_state(x0)
    res = []
    for _ in range(2):
        e = capi.Engine(capi.PREC_FP64)
        h = e.add_cell(x0, tri, p, state=st)
        e.step(5, 5e-5)
        res.append(h.get_state())
        assert h.status() == 0
        e.close()
    for u, w in zip(*res):
        assert np.array_equal(u, w)
    assert np.all(res[0][0][:, 2] == 0)
    oc = O.OCell(O.OMesh(tri, len(x0)), st, p)
    oc.steps(5, 5e-5)
    assert traj_err(res[0], oc.state(), st) <= TOL


def test_md_law_from_rest_is_noise_driven():
    """Documents the reference's discontinuity: from rest, kMD interior bond vectors
    are rounding noise after the first step (|fa_u| ~ 1e-17 um), yet each such bond
    pulls with the table's 7.2 pN.  The GPU and the oracle agree on every vertex whose
    bond is not noise-sized; the k1 law, continuous at zero, matches everywhere."""
    x0, tri = synth.disk_mesh(3000, seed=2)
    st = synth.initial_state(x0)
    for variant in ("k1", "kMD"):
        p = default_params(variant)
        e = capi.Engine(capi.PREC_FP64)
        h = e.add_cell(x0, tri, p, state=st)
        e.step(3, 5e-5)
        got = h.get_state()
        e.close()
        oc = O.OCell(O.OMesh(tri, len(x0)), st, p)
        oc.steps(3, 5e-5)
        want = oc.state()
        if variant == "k1":
            assert traj_err(got, want, st) <= TOL
        else:
            noisy = (np.linalg.norm(want[6], axis=1) < 1e-12) | (np.linalg.norm(got[6], axis=1) < 1e-12)
            assert noisy.any()
            assert np.max(np.abs(got[5] - want[5])) <= 1e-9 * np.max(np.abs(want[5]))
