"""Bulk-copy staging (bulk_staging 1) and tensor-copy staging (2, the tile's
own pair planes and real planes as 2-D tensor tiles) of the FP32 lattice
update against per-thread cp.async staging (0): the same arithmetic on the
same data, so they must agree bit for bit.  The lattices cover every alignment of the halo rows the bulk copies move
(x extent odd and even, x*y extent 0..3 modulo 4, so rows start 0..3 values
before a 16-byte boundary), tiles shorter than one x-row, and the arena's
first and last cells (rows that begin before the arena or end after it are
clamped to it)."""
import numpy as np
import pytest

from ryr_hyperactivity_gb300.sim import Simulator
from ryr_hyperactivity_gb300.workloads import config3_cells

from tests.gpu_helpers import c1_params

pytestmark = pytest.mark.gpu


def _cells():
    dims = [(13, 9, 6), (14, 8, 5), (15, 8, 7), (13, 11, 5), (12, 9, 6)]  # lx*ly mod 4: 1 0 2 3 2
    cells = [c1_params(nx=nx, ny=ny, nz=nz, seed=6, cell_id=i, ku2=1.0 + 0.3 * i)
             for i, (nx, ny, nz) in enumerate(dims)]
    ens = config3_cells(512)
    return [ens[124]] + cells + [ens[8]]  # 98-CRU rows first and last


def _run(bulk, tile, steps):
    cells = _cells()
    with Simulator(cells, precision="mixed") as sim:
        sim.set_launch_shape(0, tile, 0, 3, bulk)
        assert sim.launch_shape()["bulk_staging"] == bulk
        sim.run_steps(steps)
        return ([sim.get_state(c).snapshot() for c in range(len(cells))],
                [sim.get_membrane(c).as_dict() for c in range(len(cells))],
                [sim.drain_wholecell(c) for c in range(len(cells))],
                [sim.status(c) for c in range(len(cells))])


@pytest.mark.parametrize("staging", [1, 2])
@pytest.mark.parametrize("tile", [64, 128, 256])
def test_bulk_staging_equals_per_thread_staging(tile, staging):
    steps = 4400  # through the first upstroke, 44 output steps
    a = _run(0, tile, steps)
    b = _run(staging, tile, steps)
    assert b[3] == a[3]
    for c in range(len(a[0])):
        assert b[1][c] == a[1][c], c
        for k in a[0][c]:
            np.testing.assert_array_equal(b[0][c][k], a[0][c][k], err_msg=f"cell {c} {k}")
        np.testing.assert_array_equal(b[2][c], a[2][c])
