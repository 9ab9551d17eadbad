"""GPU: the implicit (Newton) step of FP64 engines (include/wcfe.h,
wcfe_engine_step_implicit) against an FP64 CPU Newton oracle built on the
oracle's own residual and force functions (oracle/oracle_py.py): the element
tangent against central finite differences of the FP64 residual, and one
backward-Euler step against the oracle's converged root.

The implicit step has no counterpart in the reference; the oracle here restates
its definition: G(x) = m (x - X)/dt^2 - m V/dt + (drag + damp m)(x - X)/dt - F_ext
+ Res(X, x, ea) = 0 in the plane, F_ext = F_FA + F_AP + F_bend + F_area at the
predicted positions after the bond kinetics."""
import numpy as np
import pytest

from oracle import oracle_py as O
from wholecellfe_gb300 import capi, synth
from wholecellfe_gb300.params import default_params

pytestmark = pytest.mark.gpu
DT = 5e-5


def _cell(n, seed, t=0.3):
    x0, tri = synth.disk_mesh(n, seed=seed)
    st = synth.initial_state(x0, perturb=1.0, seed=seed)
    p = default_params("k1")
    return x0, tri, st, p, t


def _residual_inplane(m, X, x, st, p, cen, t, dt=DT):
    Res, Rea, MM, _, _ = O.calc_res(m, X, x, st[3], st[4], st[5], dt, 1, p, cen, t)
    return Res[:, :2].reshape(-1), MM


def test_tangent_matches_finite_differences():
    """FP32 element tangents against central differences of the FP64 residual.  A long
    step (dt = 1e-2) keeps the mass term m/dt^2 comparable to the stiffness, so that the
    FP32 diagonal still resolves the membrane part (at dt = 5e-5 it is 1e6 times larger)."""
    dt = 1e-2
    x0, tri, st, p, t = _cell(90, 11)
    rng = np.random.default_rng(2)
    x = x0.copy()
    x[:, :2] += 2e-3 * rng.standard_normal((len(x0), 2))
    e = capi.Engine(capi.PREC_FP64)
    h = e.add_cell(x0, tri, p, state=st, t=t)
    J, diag = h.newton_tangent(x, dt)
    e.close()
    m = O.OMesh(tri, len(x0))
    cen = O.area_tot(m, x)[1:]
    n = len(x0)
    K = np.zeros((2 * n, 2 * n))
    hstep = 1e-6
    for j in range(2 * n):
        xp, xm = x.copy(), x.copy()
        xp[j // 2, j % 2] += hstep
        xm[j // 2, j % 2] -= hstep
        K[:, j] = (_residual_inplane(m, x0, xp, st, p, cen, t, dt)[0] -
                   _residual_inplane(m, x0, xm, st, p, cen, t, dt)[0]) / (2 * hstep)
    _, MM = _residual_inplane(m, x0, x, st, p, cen, t, dt)
    mass = MM * p.rho
    dg = mass / dt ** 2 + (p.drag + p.damp * mass) / dt
    assert np.allclose(diag, dg, rtol=1e-12, atol=0)
    Kg = J.astype(np.float64) - np.diag(np.repeat(dg, 2))
    err = np.max(np.abs(Kg - K)) / np.max(np.abs(K))
    assert err < 5e-3, err
    # structure: couplings only within one-rings
    assert np.all((np.abs(K) > 0) | (Kg == 0))


def _oracle_implicit_step(x0, tri, st, p, t, call=0):
    """FP64 Newton with a finite-difference Jacobian of the oracle residual."""
    m = O.OMesh(tri, len(x0))
    X, V, A, ea, cA, cC, fau = (np.array(a, dtype=np.float64) for a in st)
    n = len(X)
    _, xpred = O.predict(X, V, A, DT)
    cA, cC, fau, _ = O.update_fa(cA, cC, fau, DT, X, xpred, p)
    a4 = O.area_tot(m, xpred)
    Fext = (O.force_fa(m, xpred, cC, fau, p) + O.force_ap(m, xpred, DT, p, call) + O.force_bending(m, xpred, p) +
            O.force_area(m, xpred, a4[0], p))
    cen = a4[1:]
    stn = (X, V, A, ea, cA, cC, fau)

    def G(x):
        R, MM = _residual_inplane(m, X, x, stn, p, cen, t)
        mass = np.repeat(MM * p.rho, 2)
        d = (x - X)[:, :2].reshape(-1)
        inert, mom = mass * d / DT ** 2, mass * V[:, :2].reshape(-1) / DT
        g = inert - mom + (p.drag + p.damp * mass) * d / DT
        scale = max(np.max(np.abs(Fext[:, :2])), np.max(np.abs(R)), np.max(np.abs(inert)), np.max(np.abs(mom)))
        return g - Fext[:, :2].reshape(-1) + R, scale

    x = xpred.copy()
    for _ in range(12):
        g, scale = G(x)
        if np.max(np.abs(g)) <= 1e-14 * scale:
            break
        Jm = np.zeros((2 * n, 2 * n))
        hstep = 1e-7
        for j in range(2 * n):
            xp, xm = x.copy(), x.copy()
            xp[j // 2, j % 2] += hstep
            xm[j // 2, j % 2] -= hstep
            Jm[:, j] = (G(xp)[0] - G(xm)[0]) / (2 * hstep)
        x[:, :2] -= np.linalg.solve(Jm, g).reshape(n, 2)
    Rea = O.calc_res(m, X, x, stn[3], cA, cC, DT, 1, p, cen, t)[1]
    MM = O.calc_res(m, X, x, stn[3], cA, cC, DT, 1, p, cen, t)[2]
    Vn = (x - X) / DT
    return x, Vn, ea + Rea / MM[:, None], cC, fau


def test_implicit_step_matches_fp64_newton_oracle():
    x0, tri, st, p, t = _cell(150, 12)
    e = capi.Engine(capi.PREC_FP64)
    h = e.add_cell(x0, tri, p, state=st, t=t)
    stats = e.step_implicit(1, DT, rtol=1e-12, max_newton=8)
    got = h.get_state()
    assert h.status() == 0
    assert stats["unconverged"] == 0 and stats["max_rel_residual"] <= 1e-12, stats
    assert stats["max_refine_rel_residual"] <= 1e-10, stats
    e.close()
    x, Vn, ea, cC, fau = _oracle_implicit_step(x0, tri, st, p, t)
    u = x - st[0]
    assert np.max(np.abs(got[0] - x)) / np.max(np.abs(u)) < 1e-9
    assert np.max(np.abs(got[1][:, :2] - Vn[:, :2])) / np.max(np.abs(Vn[:, :2])) < 1e-9
    assert np.max(np.abs(got[3] - ea)) / np.max(np.abs(ea)) < 1e-9
    assert np.max(np.abs(got[5] - cC)) <= 1e-12 * max(np.max(np.abs(cC)), 1.0)


def test_implicit_steps_batched_uneven_cells():
    """Several uneven cells in one call: each converges, and equals the cell stepped alone."""
    cells = [_cell(n, 20 + i) for i, n in enumerate((120, 400, 260))]
    e = capi.Engine(capi.PREC_FP64)
    hs = [e.add_cell(x0, tri, p, state=st, t=t) for x0, tri, st, p, t in cells]
    stats = e.step_implicit(3, DT, rtol=1e-11, max_newton=8)
    assert stats["unconverged"] == 0, stats
    batched = [h.get_state() for h in hs]
    assert all(h.status() == 0 for h in hs)
    e.close()
    for (x0, tri, st, p, t), b in zip(cells, batched):
        e1 = capi.Engine(capi.PREC_FP64)
        h = e1.add_cell(x0, tri, p, state=st, t=t)
        e1.step_implicit(3, DT, rtol=1e-11, max_newton=8)
        a = h.get_state()
        e1.close()
        u = a[0] - st[0]
        assert np.max(np.abs(a[0] - b[0])) / np.max(np.abs(u)) < 1e-9


def test_implicit_refuses_mixed_engine():
    x0, tri, st, p, t = _cell(80, 3)
    e = capi.Engine(capi.PREC_MIXED)
    e.add_cell(x0, tri, p, state=st)
    with pytest.raises(capi.WcfeError):
        e.step_implicit(1, DT)
    e.close()


# (outer block, kind): tcgen05 two-level, tcgen05, mma.sync, then wider two-level blocks
LU_VARIANTS = [(256, 0), (64, 0), (64, 1), (384, 0), (512, 0), (1024, 0)]


@pytest.mark.parametrize("block,kind", LU_VARIANTS)
@pytest.mark.parametrize("m", [2, 64, 130, 512, 2050])
def test_dense_lu_solve(m, block, kind):
    """The LU factorisation on its own (no refinement): A = m I + U(-1, 1) has off-diagonal
    weight comparable to the diagonal's, so every block, panel and tensor-core tile of the
    factorisation shows in x; the error is at the TF32 level of the trailing updates."""
    rng = np.random.default_rng(m)
    A = rng.uniform(-1.0, 1.0, (m, m)) + m * np.eye(m)
    A32 = A.astype(np.float32)
    b = rng.uniform(-1.0, 1.0, m)
    x = capi.debug_lu_solve(A32, b, block, kind).astype(np.float64)
    ref = np.linalg.solve(A32.astype(np.float64), b)
    assert np.max(np.abs(x - ref)) / np.max(np.abs(ref)) < 3e-3
    # the off-diagonal part matters: dropping it is far off
    diag_only = b / np.diag(A32)
    assert np.max(np.abs(diag_only - ref)) / np.max(np.abs(ref)) > 1e-2


@pytest.mark.parametrize("m", [258, 770])
def test_dense_lu_tcgen05_matches_mma_sync(m):
    """The tcgen05 updates (two-level, K = 256) and the mma.sync updates (K = 64) factor the
    same matrix to the same solution within TF32 rounding; a matrix whose off-diagonal part
    dominates x makes a wrong tile visible."""
    rng = np.random.default_rng(m + 1)
    A = (rng.uniform(-1.0, 1.0, (m, m)) + 0.25 * m * np.eye(m)).astype(np.float32)
    b = rng.uniform(-1.0, 1.0, m)
    ref = np.linalg.solve(A.astype(np.float64), b)
    xs = [capi.debug_lu_solve(A, b, blk, kind).astype(np.float64) for blk, kind in LU_VARIANTS]
    for x in xs:
        assert np.max(np.abs(x - ref)) / np.max(np.abs(ref)) < 1e-2
    assert np.max(np.abs(xs[0] - xs[2])) / np.max(np.abs(ref)) < 1e-2


def test_implicit_step_lu_variants_agree():
    """The implicit step with each LU variant: the refinement takes every solve to 1e-10, so
    the converged states agree to the Newton tolerance."""
    x0, tri, st, p, t = _cell(300, 31)
    out = []
    for block, kind in LU_VARIANTS:
        e = capi.Engine(capi.PREC_FP64)
        e.set_lu(block, kind)
        h = e.add_cell(x0, tri, p, state=st, t=t)
        stats = e.step_implicit(2, DT, rtol=1e-11, max_newton=8)
        assert stats["unconverged"] == 0 and h.status() == 0, stats
        out.append(h.get_state()[0])
        e.close()
    u = out[0] - st[0]
    for x in out[1:]:
        assert np.max(np.abs(x - out[0])) / np.max(np.abs(u)) < 1e-9


def test_set_lu_rejects_bad_blocks():
    """Outer blocks are multiples of 64 up to 1024; the mma.sync updates take 64 only."""
    e = capi.Engine(capi.PREC_FP64)
    for block, kind in [(0, 0), (32, 0), (96, 0), (1088, 0), (256, 1), (64, 2), (64, -1)]:
        with pytest.raises(capi.WcfeError):
            e.set_lu(block, kind)
    e.set_lu(448, 0)
    e.close()
    A = np.eye(4, dtype=np.float32)
    with pytest.raises(capi.WcfeError):
        capi.debug_lu_solve(A, np.ones(4), 1088, 0)


def test_implicit_step_factor_reuse_agrees():
    """One factorisation per step (default) against a fresh one every Newton iteration: the
    refinement restores the exact correction, so the converged states agree."""
    x0, tri, st, p, t = _cell(400, 33)
    out = []
    for reuse in (True, False):
        e = capi.Engine(capi.PREC_FP64)
        e.set_lu_reuse(reuse)
        h = e.add_cell(x0, tri, p, state=st, t=t)
        stats = e.step_implicit(3, DT, rtol=1e-11, max_newton=8)
        assert stats["unconverged"] == 0 and h.status() == 0, stats
        assert stats["max_refine_rel_residual"] <= 1e-10, stats
        out.append(h.get_state()[0])
        e.close()
    u = out[1] - st[0]
    assert np.max(np.abs(out[0] - out[1])) / np.max(np.abs(u)) < 1e-9


def test_trsv_sweep_wait_times_out_cleanly():
    """The triangular sweep's failure path, with no GPU fault: block 0's solution is never
    published, so the next block's wait runs out (after 2e6 SM clocks, about 1 ms) and
    raises the sweep's abort word, which ends every other wait.  The call reports the
    timeout and returns promptly, and the context stays usable: a normal factorisation and
    solve right after it are correct."""
    import time
    m = 640
    rng = np.random.default_rng(5)
    A = (rng.uniform(-1.0, 1.0, (m, m)) + m * np.eye(m)).astype(np.float32)
    b = rng.uniform(-1.0, 1.0, m)
    t0 = time.perf_counter()
    rc, msg = capi.debug_trsv_withheld(A, b, 0, 2_000_000)
    assert rc != 0 and "timed out" in msg, (rc, msg)
    assert time.perf_counter() - t0 < 10.0
    x = capi.debug_lu_solve(A, b, 1024, 0).astype(np.float64)
    ref = np.linalg.solve(A.astype(np.float64), b)
    assert np.max(np.abs(x - ref)) / np.max(np.abs(ref)) < 3e-3


def test_implicit_workspace_kept_between_calls():
    """The implicit step keeps its workspace from one call to the next: three calls of one
    step give exactly the state of one call of three steps; after a cell is added the
    workspace is rebuilt, and the new cell steps as it does alone (to the Newton
    tolerance: in a batch a cell may take one more refinement pass than alone)."""
    x0, tri, st, p, t = _cell(220, 41)
    out = []
    for calls in ([1, 1, 1], [3]):
        e = capi.Engine(capi.PREC_FP64)
        h = e.add_cell(x0, tri, p, state=st, t=t)
        for n in calls:
            stats = e.step_implicit(n, DT, rtol=1e-11, max_newton=8)
            assert stats["unconverged"] == 0 and h.status() == 0, stats
        out.append(h.get_state())
        if len(calls) == 3:   # grow the cell set: the kept workspace must be rebuilt
            x1, tri1, st1, p1, t1 = _cell(160, 42)
            h1 = e.add_cell(x1, tri1, p1, state=st1, t=t1)
            e.step_implicit(1, DT, rtol=1e-11, max_newton=8)
            grown = h1.get_state()[0]
            a = capi.Engine(capi.PREC_FP64)
            ha = a.add_cell(x1, tri1, p1, state=st1, t=t1)
            a.step_implicit(1, DT, rtol=1e-11, max_newton=8)
            alone = ha.get_state()[0]
            a.close()
            assert np.max(np.abs(grown - alone)) <= 1e-9 * np.max(np.abs(alone - st1[0]))
        e.close()
    for u, w in zip(out[0], out[1]):
        assert np.array_equal(u, w)
