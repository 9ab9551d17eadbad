"""GPU: the mixed-precision form (FP32 increment-form assembly and forces,
float-float state and accumulation) against the FP64 form, and the batched
drop-in exchange path.

Mixed-form tolerance: relative displacement error <= 1e-6 against the FP64 form
after 300 steps (max|x_mixed - x_fp64| / max|x_fp64 - x0| per cell)."""
import numpy as np
import pytest

from wholecellfe_gb300 import capi, synth
from wholecellfe_gb300.params import default_params

pytestmark = pytest.mark.gpu
MIXED_TOL = 1e-6


def _law(p, k):
    if k == 2:
        p.force_law, p.poly_k0, p.poly_x0, p.linear_norm2d = 2, 31000.0, 0.005, 0
    return p


@pytest.mark.parametrize("variant,law", [("k1", 0), ("k31", 0), ("k31", 2)])
def test_mixed_matches_fp64_300_steps(variant, law):
    x0, tri = synth.disk_mesh(3000, seed=31)
    p = _law(default_params(variant), law)
    st = synth.initial_state(x0)
    out = {}
    for prec in (capi.PREC_FP64, capi.PREC_MIXED):
        e = capi.Engine(prec)
        h = e.add_cell(x0, tri, p, state=st)
        e.step(300, 5e-5)
        out[prec] = h.get_state()
        assert h.status() == 0
        e.close()
    u = out[capi.PREC_FP64][0] - x0
    err = np.max(np.abs(out[capi.PREC_MIXED][0] - out[capi.PREC_FP64][0])) / np.max(np.abs(u))
    assert np.max(np.abs(u)) > 0
    assert err <= MIXED_TOL, err


@pytest.mark.parametrize("variant,law", [("k1", 0), ("k31", 0), ("k31", 2)])
def test_mixed_moving_state_matches_fp64(variant, law):
    """From a moving, pre-strained state (strain ~1e-2, bonds formed, some bonds
    stretched far enough that the Bell off-rate exceeds the FP32 range)."""
    x0, tri = synth.disk_mesh(2000, seed=32)
    p = _law(default_params(variant), law)
    st = synth.initial_state(x0, perturb=1.0, seed=4)
    out = {}
    for prec in (capi.PREC_FP64, capi.PREC_MIXED):
        e = capi.Engine(prec)
        h = e.add_cell(x0, tri, p, state=st, t=0.3)
        e.step(100, 5e-5)
        out[prec] = h.get_state()
        e.close()
    u = out[capi.PREC_FP64][0] - st[0]
    err = np.max(np.abs(out[capi.PREC_MIXED][0] - out[capi.PREC_FP64][0])) / np.max(np.abs(u))
    assert err <= MIXED_TOL, err


def test_mixed_batched_equals_alone():
    sizes = [700, 2500, 180]
    cells = []
    for i, n in enumerate(sizes):
        x0, tri = synth.disk_mesh(n, seed=200 + i)
        p = _law(default_params(["k1", "k31", "k31"][i]), [0, 0, 2][i])
        p.stream = i
        cells.append((x0, tri, p))
    eb = capi.Engine(capi.PREC_MIXED)
    hs = [eb.add_cell(x, t, p, state=synth.initial_state(x)) for x, t, p in cells]
    eb.step(40, 5e-5)
    batched = [h.get_state() for h in hs]
    eb.close()
    for (x, t, p), b in zip(cells, batched):
        ea = capi.Engine(capi.PREC_MIXED)
        h = ea.add_cell(x, t, p, state=synth.initial_state(x))
        ea.step(40, 5e-5)
        for u, w in zip(b, h.get_state()):
            assert np.array_equal(u, w)
        ea.close()


@pytest.mark.parametrize("pinned", [False, True])
@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
def test_exchange_path_equals_internal_steps(prec, pinned):
    """wcfe_engine_predict / wcfe_engine_update with the host returning the predicted
    positions unchanged is the same computation as wcfe_engine_step: bit-identical for
    the FP64 form.  The mixed form keeps positions as float-float pairs (about 48
    bits) and the exchange carries them as binary64, which can round a pair's low
    part; its results agree to 1e-9 of each array's magnitude.  Both a pageable and
    a page-locked host buffer."""
    cells = [synth.disk_mesh(n, seed=300 + n) for n in (400, 1300)]
    res = []
    for mode in ("internal", "exchange"):
        e = capi.Engine(prec)
        hs = []
        for i, (x0, tri) in enumerate(cells):
            p = default_params("k31")
            p.stream = i
            hs.append(e.add_cell(x0, tri, p, state=synth.initial_state(x0, perturb=1.0, seed=i)))
        if mode == "internal":
            e.step(15, 5e-5)
        else:
            if pinned:
                import torch
                pin = torch.zeros((e.total_vertices(), 3), dtype=torch.float64, pin_memory=True)
                buf = pin.numpy()
            else:
                buf = np.zeros((e.total_vertices(), 3))
            for _ in range(15):
                e.predict_all(5e-5, buf)
                e.update_all(5e-5, 5e-5, buf)
            e.sync()
        res.append([h.get_state() for h in hs])
        e.close()
    for a, b in zip(*res):
        for u, w in zip(a, b):
            if prec == capi.PREC_FP64:
                assert np.array_equal(u, w)
            else:
                assert np.max(np.abs(u - w)) <= 1e-9 * max(np.max(np.abs(w)), 1e-12)


@pytest.mark.parametrize("host", ["pageable", "pinned", "alternating"])
@pytest.mark.parametrize("groups", [1, 3, 8])
@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
def test_exchange_groups_equal_internal_steps(prec, groups, host):
    """The exchange path with the cells split into groups on their own streams, with calls
    on the main stream in between (state reads, a regrouping, a status read), is the same
    computation as wcfe_engine_step: bit-identical for the FP64 form, 1e-9 of each array's
    magnitude for the mixed form (the binary64 exchange of float-float positions).  The
    host array is pageable, page-locked (copied asynchronously), or page-locked on odd
    steps only."""
    sizes = (300, 900, 500, 1200, 400, 700)
    cells = [synth.disk_mesh(n, seed=500 + n) for n in sizes]
    res = []
    for mode in ("internal", "exchange"):
        e = capi.Engine(prec)
        hs = []
        for i, (x0, tri) in enumerate(cells):
            p = default_params(["k1", "k31"][i % 2])
            p.stream = i
            hs.append(e.add_cell(x0, tri, p, state=synth.initial_state(x0, perturb=1.0, seed=i)))
        if mode == "internal":
            e.step(12, 5e-5)
        else:
            e.set_exchange_groups(groups)
            pageable = np.zeros((e.total_vertices(), 3))
            pinned = None
            if host != "pageable":
                import torch
                pinned = torch.zeros((e.total_vertices(), 3), dtype=torch.float64, pin_memory=True).numpy()
            for k in range(12):
                buf = pinned if host == "pinned" or (host == "alternating" and k % 2) else pageable
                e.predict_all(5e-5, buf)
                if k == 4:
                    hs[2].get_state()            # a main-stream read between predict and update
                e.update_all(5e-5, 5e-5, buf)
                if k == 6:
                    e.set_exchange_groups(1 + groups % 4)
                if k == 8:
                    assert hs[5].status() == 0   # and between update and predict
            e.sync()
        res.append([h.get_state() for h in hs])
        e.close()
    for a, b in zip(*res):
        for u, w in zip(a, b):
            if prec == capi.PREC_FP64:
                assert np.array_equal(u, w)
            else:
                assert np.max(np.abs(u - w)) <= 1e-9 * max(np.max(np.abs(w)), 1e-12)


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
def test_exchange_pinned_equals_pageable_with_host_moves(prec):
    """A host integrator that moves the predicted positions (as El Topo's collision
    handling does) before the update: a page-locked array (asynchronous copies) gives the
    same states bit for bit as a pageable one, for any grouping."""
    sizes = (500, 1100, 700)
    cells = [synth.disk_mesh(n, seed=700 + n) for n in sizes]
    res = []
    for host, groups in (("pageable", 1), ("pinned", 1), ("pinned", 3)):
        e = capi.Engine(prec)
        hs = []
        for i, (x0, tri) in enumerate(cells):
            p = default_params("k31")
            p.stream = i
            hs.append(e.add_cell(x0, tri, p, state=synth.initial_state(x0, perturb=1.0, seed=i)))
        e.set_exchange_groups(groups)
        n = e.total_vertices()
        if host == "pinned":
            import torch
            buf = torch.zeros((n, 3), dtype=torch.float64, pin_memory=True).numpy()
        else:
            buf = np.zeros((n, 3))
        shift = 1e-7 * np.sin(np.arange(n, dtype=np.float64))[:, None] * np.array([1.0, -0.5, 0.0])
        for k in range(10):
            e.predict_all(5e-5, buf)
            buf += shift * (k % 3)
            e.update_all(5e-5, 5e-5, buf)
            e.sync()
        res.append([h.get_state() for h in hs])
        e.close()
    for other in res[1:]:
        for a, b in zip(res[0], other):
            for u, w in zip(a, b):
                assert np.array_equal(u, w)


def test_exchange_groups_argument():
    e = capi.Engine(capi.PREC_MIXED)
    for g in (0, 9, -1):
        with pytest.raises(capi.WcfeError):
            e.set_exchange_groups(g)
    e.set_exchange_groups(8)
    e.close()


def test_mixed_engine_refuses_per_function_entry_points():
    """The reference-function mirrors run on FP64 engines; a mixed engine says so."""
    x0, tri = synth.disk_mesh(300, seed=8)
    e = capi.Engine(capi.PREC_MIXED)
    h = e.add_cell(x0, tri, default_params("k1"), state=synth.initial_state(x0))
    with pytest.raises(capi.WcfeError):
        h.predict(5e-5)
    with pytest.raises(capi.WcfeError):
        h.eval_forces(x0, 5e-5)
    e.close()


def test_mixed_state_round_trip():
    """set_state / get_state of a mixed engine: positions (triple-float) come back bit for
    bit, float-float storage keeps 48 bits, the acceleration is FP32."""
    x0, tri = synth.disk_mesh(500, seed=9)
    st = synth.initial_state(x0, perturb=1.0, seed=3)
    e = capi.Engine(capi.PREC_MIXED)
    h = e.add_cell(x0, tri, default_params("k31"), state=st)
    got = h.get_state()
    assert np.array_equal(got[0], st[0])
    for k, (a, b) in enumerate(zip(got, st)):
        tol = 2.0 ** -23 if k == 2 else 2.0 ** -47   # the acceleration is stored in FP32
        assert np.all(np.abs(a - b) <= tol * np.abs(b) + 1e-300), k
    e.close()


def _horizon_errors(cells, horizons, shift=(0.5, -0.25, 0.0)):
    """Per cell and horizon: (mixed error, FP64 noise, displacement), the errors as
    max|x_mixed - x_fp64| and max|(x_fp64' - shift) - x_fp64| with x_fp64' the FP64 form on
    the rigidly translated cell (the same physics, other roundings)."""
    shift = np.asarray(shift)
    runs = {}
    for name, prec, sh in (("m", capi.PREC_MIXED, 0.0), ("d", capi.PREC_FP64, 0.0), ("s", capi.PREC_FP64, 1.0)):
        e = capi.Engine(prec)
        hs = []
        for x0, tri, p, st, rho in cells:
            s0 = (st[0] + sh * shift,) + tuple(st[1:])
            h = e.add_cell(x0 + sh * shift, tri, p, state=s0)
            if rho is not None:
                h.set_integrins(rho)
            hs.append(h)
        done, runs[name] = 0, {}
        for n in horizons:
            e.step(n - done, 5e-5)
            done = n
            runs[name][n] = [h.get_state()[0] - sh * shift for h in hs]
            assert all(h.status() == 0 for h in hs)
        e.close()
    out = {}
    for n in horizons:
        out[n] = []
        for i, (x0, tri, p, st, rho) in enumerate(cells):
            xd = runs["d"][n][i]
            out[n].append((float(np.max(np.abs(runs["m"][n][i] - xd))), float(np.max(np.abs(runs["s"][n][i] - xd))),
                           float(np.max(np.abs(xd - st[0])))))
    return out


def test_mixed_error_every_horizon_bench_subset():
    """The 256-cell benchmark workload's smallest and largest cells and one cell of each
    stiffness model, from rest, after 1, 5, 20 and 300 steps.  After one step from rest
    nothing has moved and the mixed positions equal the FP64 ones exactly; at every
    horizon each cell's mixed error is <= 1e-6 of its displacement or within twice the
    FP64 form's own rounding noise (a 20-step-old cell of the workload has moved ~1e-9 um,
    where binary64 positions near 10 um carry ~1e-15 um of rounding per step); at the
    workload's 300-step horizon every cell is <= 1e-6."""
    import bench
    specs = bench.workload_specs(1000, 256)
    ns = [s["n"] for s in specs]
    pick = {int(np.argmin(ns)), int(np.argmax(ns))}
    for m in range(3):
        pick.add(next(s["index"] for s in specs if s["model"] == m))
    cells = []
    for i in sorted(pick):
        c = bench.build_cell(1000, specs[i])
        cells.append((c["x0"], c["tri"], c["p"], synth.initial_state(c["x0"]), c["rho"]))
    res = _horizon_errors(cells, (1, 5, 20, 300))
    for a, b, u in res[1]:
        assert u == 0.0 and a == 0.0
    for n in (5, 20):
        for a, b, u in res[n]:
            assert u > 0 and a <= max(MIXED_TOL * u, 2.0 * b), (n, a, b, u)
    for a, b, u in res[300]:
        assert a <= MIXED_TOL * u, (a, u)


@pytest.mark.parametrize("variant,law", [("kMD", 1), ("k1", 0), ("k31", 2)])
def test_mixed_error_every_horizon_moving_state(variant, law):
    """From a moving, pre-strained state (every law, the MD table included) the mixed
    displacement error stays <= 1e-6 at 1, 5, 20 and 300 steps."""
    x0, tri = synth.disk_mesh(2500, seed=33)
    p = default_params(variant)
    if law == 2:
        _law(p, 2)
    st = synth.initial_state(x0, perturb=1.0, seed=6)
    res = _horizon_errors([(x0, tri, p, st, None)], (1, 5, 20, 300))
    for n, rows in res.items():
        for a, b, u in rows:
            assert u > 0 and a <= MIXED_TOL * u, (n, a, b, u)


def test_integrin_density_mask():
    """Per-vertex integrin density: zero density removes the integrin force exactly;
    uniform rho_i_max reproduces the default."""
    x0, tri = synth.disk_mesh(900, seed=5)
    p = default_params("k1")
    st = synth.initial_state(x0, perturb=1.0, seed=5)
    outs = []
    for rho in (None, np.full(len(x0), 100.0)):
        e = capi.Engine(capi.PREC_FP64)
        h = e.add_cell(x0, tri, p, state=st)
        if rho is not None:
            h.set_integrins(rho)
        e.step(5, 5e-5)
        outs.append(h.get_state())
        e.close()
    for u, w in zip(*outs):
        assert np.array_equal(u, w)
    e = capi.Engine(capi.PREC_FP64)
    h = e.add_cell(x0, tri, p, state=st)
    h.set_integrins(np.zeros(len(x0)))
    F = h.eval_forces(st[0], 5e-5)[0]
    assert np.all(F == 0)
    e.close()


def test_staged_patch_kernel_equals_plain():
    """The staged patch kernel (bulk copies into shared memory) computes exactly what
    the plain kernel computes: bit-identical state after 30 steps, several cells and
    patch shapes, with integrin masks."""
    cells = []
    for i, n in enumerate([250, 1700, 5200]):
        x0, tri = synth.disk_mesh(n, seed=400 + i)
        p = _law(default_params(["k1", "k31", "k31"][i]), [0, 0, 2][i])
        p.stream = i
        rho = np.where(np.random.default_rng(i).random(len(x0)) < 0.4, p.rho_i_max, 0.0)
        cells.append((x0, tri, p, rho))
    for emax in (96, 512):
        res = []
        for kind in (0, 1):
            e = capi.Engine(capi.PREC_MIXED)
            e.set_shape(128, emax)
            e.set_patch_kernel(kind)
            hs = []
            for x0, tri, p, rho in cells:
                h = e.add_cell(x0, tri, p, state=synth.initial_state(x0, perturb=1.0, seed=7))
                h.set_integrins(rho)
                hs.append(h)
            e.step(30, 5e-5)
            res.append([h.get_state() for h in hs])
            assert all(h.status() == 0 for h in hs)
            e.close()
        for a, b in zip(*res):
            for u, w in zip(a, b):
                assert np.array_equal(u, w)


def test_mixed_protruding_cell():
    """The protruding single-cell workload (boundary driven 10 nm per step, 600 integrins
    with a 20 nm rest length, thin soft membrane) over 200 steps: mixed within 1e-6 of FP64."""
    x0, tri, p, rho = synth.protruding_cell()
    out = {}
    for prec in (capi.PREC_FP64, capi.PREC_MIXED):
        e = capi.Engine(prec)
        h = e.add_cell(x0, tri, p, state=synth.initial_state(x0))
        h.set_integrins(rho)
        e.step(200, 5e-5)
        out[prec] = h.get_state()[0]
        assert h.status() == 0
        e.close()
    u = out[capi.PREC_FP64] - x0
    err = np.max(np.abs(out[capi.PREC_MIXED] - out[capi.PREC_FP64])) / np.max(np.abs(u))
    assert err <= MIXED_TOL, err


def _fused_cells():
    """Cells that reach every branch of the fused step: small and large meshes, the
    three laws and the MD table, an integrin mask, a protruding edge, a moving state."""
    cells = []
    for i, (n, var, law) in enumerate([(180, "k1", 0), (900, "kMD", 0), (2600, "k31", 2), (5200, "k31", 0)]):
        x0, tri = synth.disk_mesh(n, seed=500 + i)
        p = _law(default_params(var), law)
        p.stream = i
        st = synth.initial_state(x0, perturb=1.0 if i % 2 else 0.0, seed=i)
        rho = np.where(np.random.default_rng(i).random(len(x0)) < 0.5, p.rho_i_max, 0.0) if i == 2 else None
        cells.append((x0, tri, p, st, rho, 0.2 * i))
    x0, tri, p, rho = synth.protruding_cell(n_target=1200)
    cells.append((x0, tri, p, synth.initial_state(x0), rho, 0.0))
    return cells


def _run_mixed(cells, calls, fused, graphs=False, shape=None, kind=1):
    e = capi.Engine(capi.PREC_MIXED)
    if shape:
        e.set_shape(*shape)
    e.set_patch_kernel(kind)
    e.set_fused(fused)
    e.set_graphs(graphs)
    hs = []
    for x0, tri, p, st, rho, t in cells:
        h = e.add_cell(x0, tri, p, state=st, t=t)
        if rho is not None:
            h.set_integrins(rho)
        hs.append(h)
    assert e.fused() == (fused and kind != 0)
    snaps = []
    for n in calls:
        e.step(n, 5e-5)
        snaps.append([h.get_state() for h in hs] + [[h.clock() for h in hs]])
    assert all(h.status() == 0 for h in hs)
    e.close()
    return snaps


@pytest.mark.parametrize("graphs", [False, True])
def test_fused_steps_equal_unfused(graphs):
    """A fused run of steps (each next vertex phase inside the patch phase) is the unfused
    computation bit for bit, in the state left after every call: calls of 1, 2, 3, 17 and 9
    steps, eager and from captured graphs (whose middle steps replay as one graph)."""
    cells = _fused_cells()
    calls = [1, 2, 3, 17, 9]
    ref = _run_mixed(cells, calls, fused=False)
    got = _run_mixed(cells, calls, fused=True, graphs=graphs)
    for a, b in zip(ref, got):
        for u, w in zip(a, b):
            for x, y in zip(u, w):
                assert np.array_equal(np.asarray(x), np.asarray(y))


@pytest.mark.parametrize("shape,kind", [((32, 128), 1), ((64, 256), 1), ((128, 768), 1), ((128, 512), 2),
                                        ((128, 192), 4)])
def test_fused_steps_equal_unfused_shapes(shape, kind):
    """The fused area sum has one order whatever the patch block size (32, 64 or 128
    threads) and register cap: bit-identical to the unfused steps."""
    cells = _fused_cells()[1:4]
    ref = _run_mixed(cells, [12], fused=False, shape=shape, kind=kind)
    got = _run_mixed(cells, [12], fused=True, shape=shape, kind=kind)
    for u, w in zip(ref[0], got[0]):
        for x, y in zip(u, w):
            assert np.array_equal(np.asarray(x), np.asarray(y))


def test_fused_flag():
    """Fused runs are off by default, apply to the plain patch kernels of a mixed engine,
    and never to the staged patch kernel or the FP64 form."""
    x0, tri = synth.disk_mesh(300, seed=1)
    e = capi.Engine(capi.PREC_MIXED)
    e.add_cell(x0, tri, default_params("k1"))
    assert not e.fused()
    e.set_fused(True)
    assert e.fused()
    e.set_patch_kernel(0)
    assert not e.fused()
    e.set_patch_kernel(1)
    e.set_fused(False)
    assert not e.fused()
    with pytest.raises(capi.WcfeError):
        e.set_shape(256, 512)   # the mixed patch kernels run at most 128 threads
    e.close()
    f = capi.Engine(capi.PREC_FP64)
    f.add_cell(x0, tri, default_params("k1"))
    f.set_fused(True)
    assert not f.fused()
    f.close()


def test_vertex_kernel_kinds_equal():
    """The vertex phase compiled for 5, 4, 6 and 8 blocks per SM computes the same bits."""
    cells = _fused_cells()[:3]
    ref = None
    for kind in range(4):
        e = capi.Engine(capi.PREC_MIXED)
        e.set_vertex_kernel(kind)
        hs = []
        for x0, tri, p, st, rho, t in cells:
            h = e.add_cell(x0, tri, p, state=st, t=t)
            if rho is not None:
                h.set_integrins(rho)
            hs.append(h)
        e.step(15, 5e-5)
        got = [h.get_state() for h in hs]
        e.close()
        if ref is None:
            ref = got
        for a, b in zip(ref, got):
            for u, w in zip(a, b):
                assert np.array_equal(u, w)


def _config2_cell(seed=2):
    """Config 2: one 20,000-vertex disk, 8,000 integrins on the polynomial law, a log-normal
    shear modulus per element (sigma 0.3)."""
    rng = np.random.default_rng(seed)
    x0, tri = synth.disk_mesh(20000, seed=seed)
    p = default_params("k31")
    p.force_law, p.poly_k0, p.poly_x0, p.linear_norm2d = 2, 31000.0, 0.005, 0
    rho = np.zeros(len(x0))
    rho[rng.choice(len(x0), size=8000, replace=False)] = p.rho_i_max
    mu = p.mu * np.exp(0.3 * rng.standard_normal(len(tri)))
    return x0, tri, p, rho, mu


def test_ff_element_config2_within_gate():
    """The mixed form with the float-float element (wcfe_engine_set_element_precision 1) on
    config 2 over its 500 steps: displacement within 1e-6 of the FP64 form (per-vertex max
    over the largest displacement), where the FP32 element reaches about 1.06e-6; the
    float-float element's error is below the FP32 element's."""
    x0, tri, p, rho, mu = _config2_cell()
    xs = {}
    for name, prec, ff in (("fp64", capi.PREC_FP64, 0), ("fp32", capi.PREC_MIXED, 0), ("ff", capi.PREC_MIXED, 1)):
        e = capi.Engine(prec)
        e.set_element_precision(ff)
        assert e.element_precision() == ff
        h = e.add_cell(x0, tri, p, state=synth.initial_state(x0))
        h.set_integrins(rho)
        h.set_element_mu(mu)
        e.step(500, 5e-5)
        assert h.status() == 0
        xs[name] = h.get_state()[0]
        e.close()
    u = np.max(np.abs(xs["fp64"] - x0))
    err32 = np.max(np.abs(xs["fp32"] - xs["fp64"])) / u
    errff = np.max(np.abs(xs["ff"] - xs["fp64"])) / u
    assert errff <= 1e-6, (errff, err32)
    assert errff < err32, (errff, err32)


def test_element_precision_flag():
    """Mode 1 is the mixed form's only; it is neither fused nor staged; it keeps the
    step's results within the mixed form's own bound of the FP32 element's."""
    e = capi.Engine(capi.PREC_FP64)
    with pytest.raises(capi.WcfeError):
        e.set_element_precision(1)
    e.set_element_precision(0)
    e.close()
    m = capi.Engine(capi.PREC_MIXED)
    for bad in (-1, 2):
        with pytest.raises(capi.WcfeError):
            m.set_element_precision(bad)
    m.set_element_precision(1)
    m.set_fused(True)
    x0, tri = synth.disk_mesh(900, seed=41)
    h = m.add_cell(x0, tri, default_params("kMD"), state=synth.initial_state(x0, perturb=1.0, seed=4))
    assert not m.fused()
    m.set_patch_kernel(0)
    m.step(20, 5e-5)
    a = h.get_state()
    m.close()
    r = capi.Engine(capi.PREC_MIXED)
    h2 = r.add_cell(x0, tri, default_params("kMD"), state=synth.initial_state(x0, perturb=1.0, seed=4))
    r.step(20, 5e-5)
    b = h2.get_state()
    r.close()
    d = np.max(np.abs(a[0] - b[0])) / max(np.max(np.abs(b[0] - x0)), 1e-30)
    assert d <= 1e-5, d
