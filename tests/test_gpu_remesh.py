"""GPU: El Topo co-residency (include/wcfe.h wcfe_cell_remesh).  A host-side emulation of
El Topo's remeshing (edge splits that average every state field, eltopo3d/edgesplitter.cpp:
564-577, chained splits included; edge collapses that keep the survivor's state; defrag_mesh's
ordered compaction, eltopo3d/surftrack.cpp:487-593) gives the change list and the state El
Topo would hold.  The device remesh must reproduce that state bit for bit, keep the cell's
clock, and step on exactly like a cell freshly loaded with it."""
import numpy as np
import pytest

from wholecellfe_gb300 import capi, synth
from wholecellfe_gb300.params import default_params

pytestmark = pytest.mark.gpu
DT = 5e-5
FIELDS = ("V", "A", "ea", "cA", "cC", "fau", "rho")


def _ccw_ok(x, tris):
    t = np.asarray(tris)
    a, b, c = x[t[:, 0]], x[t[:, 1]], x[t[:, 2]]
    return np.all((b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0]) > 1e-6)


def _edges(tris):
    m = {}
    for ti, t in enumerate(tris):
        for k in range(3):
            a, b = t[k], t[(k + 1) % 3]
            m.setdefault((min(a, b), max(a, b)), []).append(ti)
    return m


def eltopo_remesh(x, tri, st, n_split, n_collapse, seed):
    """El Topo's state semantics on host arrays; returns (split_ab, keep, tri_new, x_new, state_new)."""
    rng = np.random.default_rng(seed)
    X = [p.copy() for p in x]
    tris = [list(t) for t in tri]
    ext = {k: [np.array(v, dtype=np.float64) for v in st[k]] for k in FIELDS}
    alive = [True] * len(x)
    splits = []
    for _ in range(n_split):
        em = _edges(tris)
        interior = [e for e, ts in em.items() if len(ts) == 2]
        if len(splits) >= 2 and rng.random() < 0.5:   # split an edge of an earlier split vertex (a chain)
            interior = [e for e in interior if max(e) >= len(x)] or interior
        a, b = interior[rng.integers(len(interior))]
        t0, t1 = em[(a, b)]
        if tris[t0].index(a) != (tris[t0].index(b) - 1) % 3:   # orient t0 as (a, b, c)
            t0, t1 = t1, t0
        c = [v for v in tris[t0] if v not in (a, b)][0]
        d = [v for v in tris[t1] if v not in (a, b)][0]
        e = len(X)
        X.append(0.5 * (X[a] + X[b]))
        for k in FIELDS:
            ext[k].append(0.5 * (ext[k][a] + ext[k][b]))
        alive.append(True)
        splits.append((a, b))
        for t in sorted((t0, t1), reverse=True):
            tris.pop(t)
        tris += [[a, e, c], [e, b, c], [b, e, d], [e, a, d]]
    done = 0
    for _ in range(50 * max(n_collapse, 1)):
        if done == n_collapse:
            break
        em = _edges(tris)
        interior = [e for e, ts in em.items() if len(ts) == 2]
        u, v = interior[rng.integers(len(interior))]
        bnd = {w for e2, ts in em.items() if len(ts) == 1 for w in e2}
        if u in bnd or v in bnd:
            continue
        new = [[u if w == v else w for w in t] for t in tris if not (u in t and v in t)]
        Xn = list(X)
        Xn[u] = 0.5 * (X[u] + X[v])
        if not _ccw_ok(np.array(Xn), new):
            continue
        tris, X = new, Xn
        alive[v] = False
        done += 1
    assert done == n_collapse
    keep = np.array([i for i, a in enumerate(alive) if a], np.int32)
    remap = -np.ones(len(alive), np.int64)
    remap[keep] = np.arange(len(keep))
    tri_new = remap[np.array(tris)].astype(np.int32)
    x_new = np.array(X)[keep]
    state = {k: np.array(ext[k])[keep] for k in FIELDS}
    return np.array(splits, np.int32).reshape(-1, 2), keep, tri_new, x_new, state


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
def test_remesh_carries_state_like_eltopo(prec):
    x0, tri = synth.disk_mesh(400, seed=41)
    p = default_params("k31")
    n = len(x0)
    rho = np.where(np.random.default_rng(3).random(n) < 0.5, p.rho_i_max, 0.3 * p.rho_i_max)
    e = capi.Engine(prec)
    h = e.add_cell(x0, tri, p, state=synth.initial_state(x0, perturb=1.0, seed=41), t=0.1)
    h.set_integrins(rho)
    e.step(7, DT)   # an odd number of steps: the state sits in the second ping-pong buffer
    x, V, A, ea, cA, cC, fau = h.get_state()
    t_before = h.clock()
    st = dict(V=V, A=A, ea=ea, cA=cA, cC=cC, fau=fau, rho=rho)
    sab, keep, tri2, x2, want = eltopo_remesh(x, tri, st, n_split=12, n_collapse=4, seed=5)
    assert len(sab) == 12 and len(keep) == n + 12 - 4
    h.remesh(sab, keep, tri2, x2)
    got = h.get_state()
    assert h.clock() == t_before and h.status() == 0
    if prec == capi.PREC_FP64:
        np.testing.assert_array_equal(got[0], x2)
    else:   # positions as float-float pairs (about 48 bits)
        assert np.max(np.abs(got[0] - x2)) <= 1e-13 * np.max(np.abs(x2))
    for i, k in enumerate(("V", "A", "ea", "cA", "cC", "fau"), start=1):
        if prec == capi.PREC_FP64:
            np.testing.assert_array_equal(got[i], want[k], err_msg=k)
        else:   # float-float state (A in FP32): the mixed layout's rounding of the same values
            tol = 1e-6 if k == "A" else 1e-13
            assert np.max(np.abs(got[i] - want[k])) <= tol * max(1.0, np.max(np.abs(want[k]))), k
    # stepping on equals a cell freshly loaded with the state El Topo would hold
    e.step(20, DT)
    a = h.get_state()
    f = capi.Engine(prec)
    g = f.add_cell(x2, tri2, p, state=(x2, want["V"], want["A"], want["ea"], want["cA"], want["cC"], want["fau"]),
                   t=t_before[0], ap_calls=t_before[1])
    g.set_integrins(want["rho"])
    f.step(20, DT)
    b = g.get_state()
    e.close()
    f.close()
    for i in range(7):
        np.testing.assert_array_equal(a[i], b[i])


def test_remesh_rejects_bad_change_lists():
    x0, tri = synth.disk_mesh(100, seed=2)
    e = capi.Engine(capi.PREC_FP64)
    h = e.add_cell(x0, tri, default_params("k1"))
    n = len(x0)
    with pytest.raises(capi.WcfeError):   # split endpoint not yet created
        h.remesh(np.array([[0, n]]), np.arange(n + 1), tri, np.vstack([x0, x0[:1]]))
    with pytest.raises(capi.WcfeError):   # map not ascending
        h.remesh(None, np.arange(n)[::-1], tri, x0)
    h.remesh(None, np.arange(n), tri, x0)   # identity: accepted
    e.close()
