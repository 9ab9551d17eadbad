"""GPU: engine and cell entry points of include/wcfe.h beyond the step itself: changing a
cell's parameters between steps, re-uploading its topology, its sizes, the engine's
precision and its HBM budget."""
import numpy as np
import pytest

from wholecellfe_gb300 import capi, synth
from wholecellfe_gb300.params import default_params

pytestmark = pytest.mark.gpu
DT = 5e-5


def test_set_params_between_steps_equals_a_fresh_cell():
    x0, tri = synth.disk_mesh(500, seed=51)
    p1, p2 = default_params("k1"), default_params("k31")
    p2.mu = 1500.0
    st0 = synth.initial_state(x0, perturb=1.0, seed=51)
    e = capi.Engine(capi.PREC_FP64)
    h = e.add_cell(x0, tri, p1, state=st0, t=0.2)
    e.step(5, DT)
    mid = h.get_state()
    t, calls = h.clock()
    h.set_params(p2)
    e.step(5, DT)
    a = h.get_state()
    e.close()
    f = capi.Engine(capi.PREC_FP64)
    g = f.add_cell(x0, tri, p2, state=mid, t=t, ap_calls=calls)
    f.step(5, DT)
    b = g.get_state()
    f.close()
    for u, w in zip(a, b):
        np.testing.assert_array_equal(u, w)


def test_set_topology_and_state_continue_the_trajectory():
    x0, tri = synth.disk_mesh(400, seed=52)
    p = default_params("kMD")
    st0 = synth.initial_state(x0, perturb=1.0, seed=52)
    runs = []
    for reupload in (False, True):
        e = capi.Engine(capi.PREC_FP64)
        h = e.add_cell(x0, tri, p, state=st0, t=0.3)
        e.step(6, DT)
        if reupload:   # the topology again (as after a remeshing that changed nothing), then state and clock
            mid = h.get_state()
            t, calls = h.clock()
            h.set_topology(tri)
            h.set_state(*mid)
            h.set_clock(t, calls)
        e.step(6, DT)
        runs.append(h.get_state())
        e.close()
    for u, w in zip(*runs):
        np.testing.assert_array_equal(u, w)


def test_sizes_precision_and_budget():
    x0, tri = synth.disk_mesh(700, seed=53)
    bnd = synth.boundary_flags(len(x0), tri)
    for prec in (capi.PREC_FP64, capi.PREC_MIXED):
        e = capi.Engine(prec)
        assert e.engine_precision() == prec
        assert e.free_bytes() == 0   # no budget
        h = e.add_cell(x0, tri, default_params("k1"), state=synth.initial_state(x0))
        nv, nt, nb, npatch = h.sizes()
        assert (nv, nt, nb) == (len(x0), len(tri), int(np.sum(bnd)))
        assert npatch >= 1
        e.close()
    budget = 64 << 20
    e = capi.Engine(capi.PREC_MIXED, budget_bytes=budget)
    assert e.free_bytes() == budget
    e.add_cell(x0, tri, default_params("k1"), state=synth.initial_state(x0))
    left = e.free_bytes()
    assert 0 < left < budget
    big, btri = synth.disk_mesh(200000, seed=54)
    with pytest.raises(capi.WcfeError):   # more than the budget has left
        e.add_cell(big, btri, default_params("k1"))
    e.close()
