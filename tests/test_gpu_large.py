"""Parity at the benchmark lattice sizes and every compiled tile length.

The batched benchmark runs lattices of 60..100 CRUs along x, so most tiles
(64, 128 or 256 consecutive CRUs, x fastest) are shorter than one x-y plane,
and at 64-CRU tiles shorter than one x-row: their +-y and +-z neighbours all
come from the halo copies and the +-x ends of a row from the tile's x halo
(the stencil across CRU boundaries, cuda_Cell_Detailed.cu:1320-1355).  These
tests run the full 100x20x10 cell (LQT2-like, RyR CU->OU rate x2) and four
ensemble cells spanning nx 60..100 in one heterogeneous batch, at each tile
length, against one oracle per cell.

Bars: FP64, one lattice step from an identical rich state gives bit-identical
RyR/LCC counts and concentrations within 1e-10 relative; mixed precision
(FP32 lattice): concentrations within 1e-5 of the larger of their values
before and after the step (the fraction of values beyond 1e-5 of the new value
alone is printed), the per-CRU fluxes within 1e-5 of each flux's largest
magnitude, on the CRUs whose channel draws
did not fall on the other side of an FP32-rounded rate (their fraction is
reported and bounded); an FP64 run of 4400 steps through the first upstroke of a
98-CRU-long lattice at 64-CRU tiles follows the oracle's wholecell and
linescan records to 1e-9.
"""
import numpy as np
import pytest

from oracle import oracle as O
from ryr_hyperactivity_gb300.abi import HostState
from ryr_hyperactivity_gb300.sim import Simulator
from ryr_hyperactivity_gb300.workloads import config2_cell, config3_cells

from tests.gpu_helpers import (FLOAT_FIELDS, count_mismatch, field_errors, flux_errors,
                               rich_state, step_errors)

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10
FP32_RTOL = 1e-5
TILES = (64, 128, 256)
# ensemble cells: 60x12x7 (lx 58), 80x18x9 (lx 78), 100x16x9 and 100x19x6 (lx 98)
ENSEMBLE_IDS = (97, 77, 124, 8)


def _cells():
    ens = config3_cells(512)
    return [config2_cell()] + [ens[i] for i in ENSEMBLE_IDS]


def _oracle_lattice_step(p, st, m):
    o = O.Oracle(p)
    o.set_state(st)
    o.set_membrane(m)
    o.lattice_step()
    return o.get_state()


@pytest.fixture(scope="module")
def base_states():
    """Each cell's rich oracle state after 4200 steps (the oracle run is the
    costly part, done once for both precisions)."""
    return [(p,) + rich_state(p) for p in _cells()]


def _with_reference(base, to_float32):
    out = []
    for p, st, m in base:
        st0 = st
        st = HostState(st0.n)
        st.copy_from(st0)
        if to_float32:
            for f in FLOAT_FIELDS:
                st[f][...] = st[f].astype(np.float32).astype(np.float64)
        out.append((p, st, m, _oracle_lattice_step(p, st, m)))
    return out


@pytest.fixture(scope="module")
def fp64_states(base_states):
    return _with_reference(base_states, False)


@pytest.fixture(scope="module")
def f32_states(base_states):
    return _with_reference(base_states, True)


def _gpu_step(states, precision, tile):
    cells = [s[0] for s in states]
    with Simulator(cells, precision=precision, block_size=tile) as sim:
        assert sim.tile_size() == tile
        for c, (_, st, m, _) in enumerate(states):
            sim.set_state(c, st)
            sim.set_membrane(c, m)
        sim.lattice_step()
        return [sim.get_state(c) for c in range(len(cells))]


@pytest.mark.parametrize("tile", TILES)
def test_fp64_single_step_large_lattices(fp64_states, tile):
    got = _gpu_step(fp64_states, "fp64", tile)
    for c, ((p, _, _, ref), g) in enumerate(zip(fp64_states, got)):
        bad = count_mismatch(g, ref)
        assert not bad.any(), (tile, c, p.nx, p.ny, p.nz, int(bad.sum()))
        errs = field_errors(g, ref)
        worst = max(errs.items(), key=lambda kv: kv[1])
        assert worst[1] <= FP64_RTOL, (tile, c, worst)


@pytest.mark.parametrize("tile", TILES)
def test_mixed_single_step_large_lattices(f32_states, tile):
    got = _gpu_step(f32_states, "mixed", tile)
    for c, ((p, st, _, ref), g) in enumerate(zip(f32_states, got)):
        bad = count_mismatch(g, ref)
        frac = float(bad.mean())
        print(f"tile {tile} cell {c} ({p.nx}x{p.ny}x{p.nz}): count mismatch fraction {frac:.2e}")
        assert frac <= 0.01, (tile, c, frac)
        serrs = step_errors(g, ref, st, mask=~bad)
        ferrs = flux_errors(g, ref, mask=~bad)
        print({k: f"{e[0]:.1e} ({e[1]:.1e} of values above 1e-5 per value)"
               for k, e in serrs.items()}, {k: f"{e:.1e}" for k, e in ferrs.items()})
        worst = max(serrs.items(), key=lambda kv: kv[1][0])
        assert worst[1][0] <= FP32_RTOL, (tile, c, worst)
        worst = max(ferrs.items(), key=lambda kv: kv[1])
        assert worst[1] <= FP32_RTOL, (tile, c, worst)


def test_fp64_run_at_tiles_shorter_than_a_row():
    """4400 steps (through the first upstroke at t = 100 ms) of a 100x16x9
    ensemble cell (rows of 98 CRUs) at 64-CRU tiles."""
    p = config3_cells(512)[124]
    assert p.nx - 2 > 64
    nsteps = 4400
    o = O.Oracle(p)
    _, wc_ref, ls_ref = o.run(nsteps)
    with Simulator(p, precision="fp64", block_size=64) as sim:
        sim.run_steps(nsteps)
        wc = sim.drain_wholecell(0)
        ls = sim.drain_linescan(0)
        st = sim.get_state(0)
        m = sim.get_membrane(0)
    assert wc.shape == wc_ref.shape and ls.shape == ls_ref.shape
    np.testing.assert_allclose(wc, wc_ref, rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(ls, ls_ref, rtol=1e-9, atol=1e-9)
    m_ref = o.get_membrane()
    assert abs(m.v - m_ref.v) <= 1e-9 * (1 + abs(m_ref.v))
    ref = o.get_state()
    assert not count_mismatch(st, ref).any()
    errs = field_errors(st, ref, fields=FLOAT_FIELDS)
    assert max(errs.values()) <= 1e-8, errs
