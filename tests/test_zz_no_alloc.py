"""The allocation-free area reduction (wcfe_area_tot_noalloc) through the C ABI.

It serves host codes that cannot allocate device memory while they run (all of it
reserved up front, or no implicit synchronisation from cudaMalloc/cudaFree allowed
mid-loop): the caller passes its own device buffers and the scratch lives in a
file-scope device array.  Its output must equal the engine's own area/centroid
(wcfe_cell_eval_forces) within the parity tolerance, on two calls in a row, the
second on different positions so stale scratch would show.  This file is named to
run last."""
import numpy as np
import pytest

from conftest import relerr
from wholecellfe_gb300 import capi, synth
from wholecellfe_gb300.params import default_params

pytestmark = pytest.mark.gpu
TOL = 1e-9


def test_area_tot_noalloc_matches_engine_twice():
    import torch
    x0, tri = synth.disk_mesh(6000, seed=41)
    st = synth.initial_state(x0, perturb=1.0, seed=41)
    eng = capi.Engine(capi.PREC_FP64)
    cell = eng.add_cell(x0, tri, default_params("k1"), state=st)
    lib = capi.load()
    td = torch.tensor(np.asarray(tri, np.int32), device="cuda")
    out = torch.empty(4, dtype=torch.float64, device="cuda")
    rng = np.random.default_rng(7)
    for call in range(2):
        x = x0 + (0.0 if call == 0 else 1.0) * np.c_[rng.normal(0, 0.02, (len(x0), 2)), np.zeros(len(x0))]
        want = cell.eval_forces(x, 5e-5)[4]
        xd = torch.tensor(x, dtype=torch.float64, device="cuda")
        out.fill_(float("nan"))
        stream = torch.cuda.current_stream()
        rc = lib.wcfe_area_tot_noalloc(xd.data_ptr(), len(x0), td.data_ptr(), len(tri), out.data_ptr(),
                                       stream.cuda_stream)
        assert rc == 0
        stream.synchronize()
        got = out.cpu().numpy()
        assert relerr(got, want) <= TOL, (call, got, want)
    eng.close()


def test_area_tot_noalloc_rejects_oversize_without_launching():
    import torch
    lib = capi.load()
    x = torch.zeros((3, 3), dtype=torch.float64, device="cuda")
    t = torch.zeros((1, 3), dtype=torch.int32, device="cuda")
    out = torch.full((4,), 7.0, dtype=torch.float64, device="cuda")
    rc = lib.wcfe_area_tot_noalloc(x.data_ptr(), 3, t.data_ptr(), 4096 * 1024 + 1, out.data_ptr(), None)
    assert rc == 8  # WCFE_ERR_LIMIT
    torch.cuda.synchronize()
    assert bool((out == 7.0).all())
