"""GPU: the serving loop (wcfe_server_*) — continuous batching of whole cell
simulations under an HBM budget.  Requests that arrive while others run are
admitted as memory frees up.  Each result equals the same request run alone
bit for bit, because a cell's arithmetic does not depend on its neighbours in
the launch."""
import ctypes as C

import numpy as np
import pytest

from wholecellfe_gb300 import capi, synth
from wholecellfe_gb300.params import default_params

pytestmark = pytest.mark.gpu
DT = 5e-5


def _requests():
    reqs = []
    for i, (n, law, steps) in enumerate([(900, 0, 12), (3000, 1, 5), (400, 2, 20), (1800, 0, 9), (2500, 2, 7),
                                          (700, 1, 15)]):
        x0, tri = synth.disk_mesh(n, seed=500 + i)
        p = default_params("k31" if law else "k1")
        if law == 2:
            p.force_law, p.poly_k0, p.poly_x0, p.linear_norm2d = 2, 31000.0, 0.005, 0
        p.stream = i
        reqs.append((x0, tri, p, steps))
    return reqs


def _alone(x0, tri, p, steps, prec):
    e = capi.Engine(prec)
    h = e.add_cell(x0, tri, p, state=synth.initial_state(x0))
    e.step(steps, DT)
    x = h.get_state()[0]
    e.close()
    return x


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
@pytest.mark.parametrize("iter_ms", [1e-6, 8.0])
def test_server_results_equal_alone(prec, iter_ms):
    """iter_ms 1e-6: one step per iteration, so cells stay resident across iterations and
    the overlap shows in n_active; 8.0 (the default): many steps per iteration, cells
    finishing inside an iteration stopped by their device-side step budget."""
    reqs = _requests()
    L = capi.load()
    # a budget that holds only a few cells at once, so admissions wait for retirements
    budget = int(sum(L.wcfe_cell_bytes(len(x), len(t)) for x, t, _, _ in reqs[:3]) * 1.1)
    eng = capi.Engine(prec, budget_bytes=budget)
    srv = C.c_void_p()
    capi.check(L.wcfe_server_create(eng.h, DT, C.byref(srv)), "wcfe_server_create")
    capi.check(L.wcfe_server_set_iteration_ms(srv, iter_ms), "wcfe_server_set_iteration_ms")
    keep = []
    ids = []
    for k, (x0, tri, p, steps) in enumerate(reqs):
        tri32 = np.ascontiguousarray(tri, np.int32)
        x = np.ascontiguousarray(x0, np.float64)
        keep.append((tri32, x, p))
        rq = capi.Request(len(x), len(tri32), capi.ip(tri32), capi.dp(x), C.pointer(p), steps, None, None, 0, 0)
        rid = C.c_int64()
        capi.check(L.wcfe_server_submit(srv, C.byref(rq), C.byref(rid)), "submit")
        ids.append(rid.value)
        if k == 2:   # later requests arrive while the first ones are already running
            na, nq = C.c_int32(), C.c_int32()
            for _ in range(3):
                capi.check(L.wcfe_server_iterate(srv, C.byref(na), C.byref(nq)), "iterate")
    na, nq = C.c_int32(), C.c_int32()
    max_active = 0
    for _ in range(1000):
        capi.check(L.wcfe_server_iterate(srv, C.byref(na), C.byref(nq)), "iterate")
        max_active = max(max_active, na.value)
        if na.value == 0 and nq.value == 0:
            break
    assert na.value == 0 and nq.value == 0
    if iter_ms < 1e-3:
        assert max_active >= 2      # requests overlapped on the device
    assert L.wcfe_server_cell_steps(srv) == sum(r[3] for r in reqs)
    for rid, (x0, tri, p, steps) in zip(ids, reqs):
        out = np.zeros((len(x0), 3))
        lat = C.c_double()
        capi.check(L.wcfe_server_result(srv, rid, capi.dp(out), C.byref(lat)), "result")
        assert lat.value > 0
        assert np.array_equal(out, _alone(x0, tri, p, steps, prec))
    n = L.wcfe_server_step_times(srv, None, 0)
    assert n > 0
    L.wcfe_server_destroy(srv)
    eng.close()


def test_budget_rejects_oversized_cell():
    L = capi.load()
    x0, tri = synth.disk_mesh(4000, seed=1)
    eng = capi.Engine(capi.PREC_FP64, budget_bytes=L.wcfe_cell_bytes(len(x0), len(tri)) // 4)
    with pytest.raises(capi.WcfeError):
        eng.add_cell(x0, tri, default_params("k1"))
    eng.close()


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
def test_step_budget_stops_cell_exactly(prec):
    """A cell with a step budget of n runs exactly n steps and then stays put while later
    steps run the other cells (the serving loop's stop rule); the budget reads -1 after."""
    x0, tri = synth.disk_mesh(900, seed=71)
    x1, tri1 = synth.disk_mesh(1500, seed=72)
    p = default_params("k31")
    e = capi.Engine(prec)
    a = e.add_cell(x0, tri, p, state=synth.initial_state(x0))
    b = e.add_cell(x1, tri1, p, state=synth.initial_state(x1))
    a.set_step_budget(5)
    assert a.step_budget() == 5 and b.step_budget() == 0
    e.step(12, DT)
    got_a, got_b = a.get_state()[0], b.get_state()[0]
    assert a.step_budget() == -1 and b.step_budget() == 0
    assert a.clock()[0] == pytest.approx(5 * DT, rel=1e-12)
    e.close()
    assert np.array_equal(got_a, _alone(x0, tri, p, 5, prec))
    assert np.array_equal(got_b, _alone(x1, tri1, p, 12, prec))
