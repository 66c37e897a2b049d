"""Ensembles of independent cells over several GPUs.

One process per GPU (launched with torchrun).  The cells are split into
contiguous ranges of about equal work (interior CRUs x simulated steps), each
process advances its range with the batched simulator, and nothing is
exchanged while the cells run: the only collective is one gather of the
per-cell results to rank 0 at the end.  A single cell is never split across
GPUs (its halo exchange every 0.025 ms would be latency-bound), so a run of
fewer cells than GPUs leaves GPUs idle.

    from ryr_hyperactivity_gb300.ensemble import run_sharded, gpu_runner
    results = run_sharded(cells, nsteps, gpu_runner("mixed"))   # list on rank 0, None elsewhere
"""
from __future__ import annotations

from typing import Callable, Sequence

from .abi import CellParams
from .workloads import interior

DT = 0.025


def cell_work(p: CellParams, nsteps: int) -> float:
    """Work of one cell: interior CRUs x steps it is active (the protocol
    ends at nbeats * PCL + 2100 ms)."""
    active = min(nsteps, int((p.nbeats * p.pcl_ms + 2100.0) / DT) + 1)
    return float(interior(p)) * active


def partition(work: Sequence[float], world: int) -> list[range]:
    """Contiguous ranges of cells, one per rank, of about equal total work:
    rank r takes the cells whose work prefix midpoint falls in
    [r/world, (r+1)/world) of the total."""
    n = len(work)
    total = float(sum(work))
    if world <= 1 or n == 0 or total <= 0:
        return [range(0, n)] + [range(n, n)] * max(world - 1, 0)
    bounds = [0]
    acc = 0.0
    r = 1
    for i, w in enumerate(work):
        mid = acc + 0.5 * w
        while r < world and mid >= total * r / world:
            bounds.append(i)
            r += 1
        acc += w
    while len(bounds) < world:
        bounds.append(n)
    bounds.append(n)
    return [range(bounds[k], bounds[k + 1]) for k in range(world)]


def _dist():
    try:
        import torch.distributed as dist
    except ImportError:  # pragma: no cover
        return None
    return dist if dist.is_available() and dist.is_initialized() else None


def run_sharded(cells: Sequence[CellParams], nsteps: int,
                run_shard: Callable[[list, int], list], group=None):
    """Runs `cells` for `nsteps` steps split over the ranks of the default
    process group (or `group`); `run_shard(cells, nsteps)` returns one result
    per cell.  Rank 0 returns the results of all cells in the input order,
    the other ranks None.  Without an initialised process group this is a
    single-process run."""
    dist = _dist()
    rank = dist.get_rank(group) if dist else 0
    world = dist.get_world_size(group) if dist else 1
    parts = partition([cell_work(p, nsteps) for p in cells], world)
    mine = parts[rank]
    local = run_shard([cells[i] for i in mine], nsteps) if len(mine) else []
    if world == 1:
        return list(local)
    gathered = [None] * world if rank == 0 else None
    dist.gather_object(list(local), gathered, dst=0, group=group)
    if rank != 0:
        return None
    out = []
    for r in range(world):
        out.extend(gathered[r])
    return out


def gpu_runner(precision: str = "mixed", device: int | None = None, **opts):
    """run_shard for the batched GPU simulator: per cell, the wholecell
    records and the per-beat statistics."""

    def run(shard: list, nsteps: int) -> list:
        import numpy as np

        from .sim import Simulator

        dev = device
        if dev is None:
            import os

            dev = int(os.environ.get("LOCAL_RANK", "0"))
        n = len(shard)
        recs = [[] for _ in range(n)]
        stats = [[] for _ in range(n)]
        kw = dict(window_steps=100, output_capacity=64, record_linescan=0, track_stats=1,
                  stats_capacity=64)
        kw.update(opts)
        with Simulator(shard, precision=precision, device=dev, **kw) as sim:
            done = 0
            while done < nsteps:
                k = min(4000, nsteps - done)
                sim.run_steps(k)
                done += k
                for c in range(n):
                    recs[c].append(sim.drain_wholecell(c, 64))
                    stats[c].extend(sim.drain_stats(c, 64))
        return [(np.concatenate(r), s) for r, s in zip(recs, stats)]

    return run
