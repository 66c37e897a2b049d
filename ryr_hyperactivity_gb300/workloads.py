"""Synthetic workloads (no dataset is involved: every input is a seeded set of
cell parameters).  Parameter bases follow run.sh:7-9: "stab" uses a6 = 10,
a8 = 1.0, "hyper" a6 = 3.333, a8 = 18; the other arguments are a3 = 1.0,
a4 = 740, a5 = 1.0, a7 = 0, a9 = 0.7, a10 = 1."""
from __future__ import annotations

import numpy as np

from .abi import CellParams, cell_params

STAB = dict(clamp_mv=1.0, cjsr_basal=740.0, ncx_scale=1.0, ku=10.0, r1=0.0, kb=1.0,
            ica_scale=0.7, ku2=1.0)
HYPER = dict(STAB, ku=3.333, kb=18.0)


def config1_cell(seed: int = 1) -> CellParams:
    """20x10x5 lattice, control build (IKr on, no iso), PCL 400 ms, 2 beats."""
    return cell_params(nx=20, ny=10, nz=5, nbeats=2, pcl_ms=400.0, lqt=0, iso2=0, seed=seed,
                       cell_id=0, **STAB)


def config2_cell(seed: int = 1) -> CellParams:
    """Full cell 100x20x10, LQT2-like (IKr x0: the lqt build), RyR CU->OU
    rate x2 (Ku2 = 2), iso2 build, PCL 2000 ms, 10 beats."""
    d = dict(STAB)
    d["ku2"] = 2.0
    return cell_params(nx=100, ny=20, nz=10, nbeats=10, pcl_ms=2000.0, lqt=1, iso2=1, seed=seed,
                       cell_id=0, **d)


def config3_cells(n: int = 512, param_seed: int = 12345, philox_seed: int = 1,
                  first_id: int = 0, nbeats: int = 20) -> list[CellParams]:
    """Heterogeneous ensemble: nx~U{60..100}, ny~U{12..20}, nz~U{6..10},
    RyR open-rate scale Ku2~U[1,3], IKr scale~U[0,1], PCL~U[500,3000] ms;
    the RyR-hyperactive parameter base of run.sh:9, iso2 build with IKr
    scaled (lqt off); Philox key = (seed, cell id)."""
    rng = np.random.default_rng(param_seed)
    nx = rng.integers(60, 101, n)
    ny = rng.integers(12, 21, n)
    nz = rng.integers(6, 11, n)
    ku2 = rng.uniform(1.0, 3.0, n)
    ikr = rng.uniform(0.0, 1.0, n)
    pcl = rng.uniform(500.0, 3000.0, n)
    cells = []
    for c in range(n):
        d = dict(HYPER)
        d["ku2"] = float(ku2[c])
        cells.append(cell_params(nx=int(nx[c]), ny=int(ny[c]), nz=int(nz[c]), nbeats=nbeats,
                                 pcl_ms=float(pcl[c]), lqt=0, iso2=1, ikr_scale=float(ikr[c]),
                                 seed=philox_seed, cell_id=first_id + c, **d))
    return cells


def interior(p: CellParams) -> int:
    return (p.nx - 2) * (p.ny - 2) * (p.nz - 2)
