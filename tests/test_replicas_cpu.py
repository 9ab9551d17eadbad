"""The multi-GPU host logic on CPU: cells sharded over ranks with no data-path
collective.  Two gloo ranks each advance their shard of a small population with
the oracle; the union of the shards' results equals the one-process result bit
for bit, and the timing reductions (max over ranks, sum over ranks) agree."""
import os
import socket
import tempfile

import numpy as np
import pytest

from wholecellfe_gb300.replicas import partition_cells, rank_env, shard_loads

DT = 5e-5
SIZES = [120, 400, 60, 250, 250, 90]   # vertex targets of the population
STEPS = 4


def test_partition_covers_once_and_is_deterministic():
    rng = np.random.default_rng(3)
    costs = [int(c) for c in rng.integers(500, 20000, size=257)]
    for world in (1, 2, 3, 8):
        a = partition_cells(costs, world)
        b = partition_cells(list(costs), world)
        assert a == b
        flat = sorted(i for s in a for i in s)
        assert flat == list(range(len(costs)))
        loads = shard_loads(costs, a)
        # LPT bound: max load <= mean load + the largest single cost
        assert max(loads) <= sum(costs) / world + max(costs)
    assert partition_cells([], 4) == [[], [], [], []]
    assert partition_cells([5, 5, 5], 1) == [[0, 1, 2]]
    # equal costs go round-robin by index
    assert partition_cells([1, 1, 1, 1], 2) == [[0, 2], [1, 3]]


def test_partition_rejects_bad_arguments():
    with pytest.raises(ValueError):
        partition_cells([1, 2], 0)
    with pytest.raises(ValueError):
        partition_cells([1, -2], 2)


def test_rank_env():
    assert rank_env({}) == rank_env({"WORLD_SIZE": "1", "RANK": "0"})
    e = rank_env({"WORLD_SIZE": "4", "RANK": "3", "LOCAL_RANK": "3"})
    assert (e.rank, e.world, e.local) == (3, 4, 3)
    with pytest.raises(ValueError):
        rank_env({"WORLD_SIZE": "2", "RANK": "2"})


def _population():
    from wholecellfe_gb300 import synth
    from wholecellfe_gb300.params import default_params
    cells = []
    for i, n in enumerate(SIZES):
        x0, tri = synth.disk_mesh(n, seed=70 + i)
        p = default_params("k31" if i % 2 else "k1")
        p.stream = i
        cells.append((x0, tri, p, synth.initial_state(x0, perturb=1e-3, seed=i)))
    return cells


def _advance(cells, idx):
    from oracle import oracle_py as O
    out = {}
    for i in idx:
        x0, tri, p, st = cells[i]
        oc = O.OCell(O.OMesh(tri, len(x0)), st, p)
        oc.steps(STEPS, DT)
        out[i] = oc.state()
    return out


def _rank_main(rank, world, port, outdir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    from wholecellfe_gb300.replicas import max_over_ranks, sum_over_ranks
    env = rank_env()
    dist.init_process_group("gloo", rank=env.rank, world_size=env.world)
    cells = _population()
    shards = partition_cells([len(c[0]) for c in cells], env.world)
    mine = _advance(cells, shards[env.rank])
    # host-side reductions only: job time and units processed
    tmax = max_over_ranks(1.0 + env.rank, dist)
    units = sum_over_ranks(len(shards[env.rank]), dist)
    dist.barrier()
    dist.destroy_process_group()
    np.savez(os.path.join(outdir, f"rank{rank}.npz"), idx=np.array(sorted(mine)), tmax=tmax, units=units,
             **{f"c{i}_{k}": a for i, s in mine.items() for k, a in enumerate(s)})


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_match_one_process():
    import torch.multiprocessing as mp
    from oracle import oracle_py as O
    O.build()
    world = 2
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_rank_main, args=(world, _free_port(), d), nprocs=world, join=True, start_method="spawn")
        got = {}
        for r in range(world):
            z = np.load(os.path.join(d, f"rank{r}.npz"))
            assert float(z["tmax"]) == float(world)
            assert float(z["units"]) == float(len(SIZES))
            for i in z["idx"]:
                got[int(i)] = [z[f"c{int(i)}_{k}"] for k in range(7)]
    assert sorted(got) == list(range(len(SIZES)))
    ref = _advance(_population(), range(len(SIZES)))
    for i in range(len(SIZES)):
        for a, b in zip(got[i], ref[i]):
            assert np.array_equal(a, b)
