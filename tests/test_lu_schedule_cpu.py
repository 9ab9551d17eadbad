"""The implicit step's LU schedule (host logic, no GPU): replayed in numpy, the exported
op list factors a matrix into L U = A for every outer block width and for orders that do
and do not divide into 64-wide steps."""
import numpy as np
import pytest

from wholecellfe_gb300 import capi

B = 64


def replay(A, ops):
    """Apply the schedule in float64: type 0 factors the diagonal block, type 1 forms the
    step's panels from its inverses, type 2 subtracts J[rows, ka:ka+K] J[ka:ka+K, cols] on
    each region (a bound of -1 is the order)."""
    J = A.copy()
    m = len(J)
    for op in ops:
        typ, k0, nreg, ka, kb, K = (int(v) for v in op[:6])
        if typ == 0:
            e = min(B, m - k0)
            D = J[k0:k0 + e, k0:k0 + e]
            for j in range(e):
                D[j + 1:, j] /= D[j, j]
                D[j + 1:, j + 1:] -= np.outer(D[j + 1:, j], D[j, j + 1:])
        elif typ == 1:
            e = min(B, m - k0)
            D = J[k0:k0 + e, k0:k0 + e]
            L = np.tril(D, -1) + np.eye(e)
            U = np.triu(D)
            J[k0 + e:, k0:k0 + e] = J[k0 + e:, k0:k0 + e] @ np.linalg.inv(U)
            J[k0:k0 + e, k0 + e:] = np.linalg.inv(L) @ J[k0:k0 + e, k0 + e:]
        else:
            for r in range(nreg):
                rlo, rhi, clo, chi = (int(v) for v in op[6 + 4 * r:10 + 4 * r])
                rhi = m if rhi < 0 else min(rhi, m)
                chi = m if chi < 0 else min(chi, m)
                if rlo >= rhi or clo >= chi:
                    continue
                J[rlo:rhi, clo:chi] -= J[rlo:rhi, ka:ka + K] @ J[ka:ka + K, clo:chi]
    return J


@pytest.mark.parametrize("m", [2, 64, 130, 520, 1000, 2050])
@pytest.mark.parametrize("block", [64, 128, 192, 256, 384, 448, 512, 768, 1024])
def test_schedule_factors(m, block):
    rng = np.random.default_rng(m + block)
    A = rng.uniform(-1.0, 1.0, (m, m)) + m * np.eye(m)
    ops = capi.debug_lu_schedule(m, block)
    J = replay(A, ops)
    L = np.tril(J, -1) + np.eye(m)
    U = np.triu(J)
    assert np.max(np.abs(L @ U - A)) <= 1e-10 * np.max(np.abs(A))
    # every 64-wide step is factored once, in order
    diag = [int(o[1]) for o in ops if o[0] == 0]
    assert diag == list(range(0, m, B))
    # updates use whole 64-column steps of one outer block
    for o in ops[ops[:, 0] == 2]:
        K, ka, kb = int(o[5]), int(o[3]), int(o[4])
        assert K % B == 0 and 0 < K <= block
        assert kb == ka - (ka // block) * block and kb + K <= block


def test_strips_run_at_growing_k():
    """Outer block 512: the strip updates inside a block run at K = 64, 128 and 256 and
    the trailing matrix at 512, so most strip flops run at K >= 128."""
    m = 5000
    ops = capi.debug_lu_schedule(m, 512)
    flops = {}
    for o in ops[ops[:, 0] == 2]:
        K = int(o[5])
        for r in range(int(o[2])):
            rlo, rhi, clo, chi = (int(v) for v in o[6 + 4 * r:10 + 4 * r])
            rhi = m if rhi < 0 else min(rhi, m)
            chi = m if chi < 0 else min(chi, m)
            if rlo < rhi and clo < chi:
                flops[K] = flops.get(K, 0) + 2 * (rhi - rlo) * (chi - clo) * K
    assert sorted(flops) == [64, 128, 256, 512]
    assert flops[64] < flops[128] < flops[256] < flops[512]


def test_schedule_arguments():
    for m, block in [(0, 512), (100, 96), (100, 1088), (100, 0)]:
        with pytest.raises(capi.WcfeError):
            capi.debug_lu_schedule(m, block)
