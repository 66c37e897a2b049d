"""Multi-process ensemble path on the CPU: two gloo ranks each advance their
share of the cells (the CPU oracle stands in for the GPU simulator), and the
gathered per-cell results equal a single-process run, cell for cell."""
import os
import socket

import numpy as np
import pytest

from ryr_hyperactivity_gb300.ensemble import cell_work, partition, run_sharded
from ryr_hyperactivity_gb300.workloads import config3_cells

NSTEPS = 120


def _cells():
    cells = config3_cells(5, nbeats=1)
    for p in cells:  # tiny lattices so the oracle finishes in a blink
        p.nx, p.ny, p.nz = 6 + p.cell_id, 5, 4
    return cells


def oracle_runner(shard, nsteps):
    from oracle import oracle as O

    out = []
    for p in shard:
        o = O.Oracle(p)
        _, wc, _ = o.run(nsteps)
        m = o.get_membrane()
        out.append((np.asarray(wc), m.v, m.xnai))
    return out


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, path):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        res = run_sharded(_cells(), NSTEPS, oracle_runner)
        if rank == 0:
            np.save(path, np.array(res, dtype=object), allow_pickle=True)
        else:
            assert res is None
    finally:
        dist.destroy_process_group()


def test_partition_balances_work_and_keeps_order():
    cells = config3_cells(40)
    work = [cell_work(p, 10_000) for p in cells]
    parts = partition(work, 4)
    assert [i for r in parts for i in r] == list(range(40))
    shares = [sum(work[i] for i in r) / sum(work) for r in parts]
    assert max(shares) < 0.25 + max(work) / sum(work)
    assert partition(work, 1) == [range(0, 40)]
    assert [len(r) for r in partition([1.0, 1.0], 4)].count(0) == 2


def test_two_gloo_ranks_match_single_process(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    path = str(tmp_path / "res.npy")
    mp.spawn(_worker, args=(2, _free_port(), path), nprocs=2, join=True)
    got = list(np.load(path, allow_pickle=True))
    ref = run_sharded(_cells(), NSTEPS, oracle_runner)  # no process group: one process
    assert len(got) == len(ref) == 5
    for (wc, v, na), (wc0, v0, na0) in zip(got, ref):
        np.testing.assert_array_equal(wc, wc0)
        assert v == v0 and na == na0
