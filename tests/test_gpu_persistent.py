"""The persistent window launch (run option persistent = 1) against the
two-launch path (persistent = 0), and the launch-shape autotuner.

Both launch paths run the same tile and cell-update code, and the whole-cell
sums are exact, so they must agree bit for bit: lattice state, membrane
state, output records, beat statistics and status, through full windows,
partial windows, output steps and cells that finish their protocol part-way
through a window.  The bounded waits are checked by a readiness target that
no cell ever publishes: every wait runs out, rh_run_steps reports
RH_ERR_TIMEOUT, the cells carry RH_STATUS_TIMEOUT and the GPU context stays
usable.
"""
import numpy as np
import pytest

from ryr_hyperactivity_gb300.native import NativeError
from ryr_hyperactivity_gb300.sim import Simulator
from ryr_hyperactivity_gb300.workloads import config3_cells

from tests.gpu_helpers import c1_params

pytestmark = pytest.mark.gpu

RH_STATUS_TIMEOUT = 0x20


def _cells():
    # uneven lattices and protocols; cell 2 is moved close to the end of its
    # protocol (2100 + 60 ms) before the run and finishes after 120 steps
    return [c1_params(nx=14, ny=9, nz=6, seed=2, cell_id=0, ku2=1.5),
            c1_params(nx=31, ny=8, nz=5, seed=2, cell_id=1, pcl_ms=300.0, lqt=0, iso2=0),
            c1_params(nx=6, ny=5, nz=4, seed=2, cell_id=2, nbeats=1, pcl_ms=60.0),
            c1_params(nx=23, ny=12, nz=7, seed=2, cell_id=3, cao_mM=2.2, ikr_scale=0.4)]


def _run(cells, precision, persistent, chunks, **opts):
    out = {}
    with Simulator(cells, precision=precision, persistent=persistent, **opts) as sim:
        if len(cells) > 2:
            m = sim.get_membrane(2)
            m.t = 2160.0 - 3.0
            sim.set_membrane(2, m)
        launches0, mode = sim.kernel_launches()
        assert mode == bool(persistent)
        wc = [[] for _ in cells]
        st = [[] for _ in cells]
        for k in chunks:
            sim.run_steps(k)
            for c in range(len(cells)):
                wc[c].append(sim.drain_wholecell(c))
                st[c].extend(sim.drain_stats(c))
        out["launches"] = sim.kernel_launches()[0] - launches0
        out["groups"] = sim.num_groups()
        out["state"] = [sim.get_state(c).snapshot() for c in range(len(cells))]
        out["membrane"] = [sim.get_membrane(c).as_dict() for c in range(len(cells))]
        out["wc"] = [np.concatenate(w) for w in wc]
        out["stats"] = st
        out["status"] = [sim.status(c) for c in range(len(cells))]
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("tile", [64, 128])
def test_persistent_windows_equal_two_launch_path(precision, tile):
    cells = _cells()
    # full windows, a partial one, steps across the end of cell 2's protocol
    chunks = [250, 100, 37, 4000, 263]
    a = _run(cells, precision, 0, chunks, block_size=tile, cell_groups=2)
    b = _run(cells, precision, 1, chunks, block_size=tile)
    assert b["status"] == a["status"]
    assert b["status"][2] & 0x8  # cell 2 finished inside a window
    for c in range(len(cells)):
        assert b["membrane"][c] == a["membrane"][c], c
        for k in a["state"][c]:
            np.testing.assert_array_equal(b["state"][c][k], a["state"][c][k], err_msg=f"{c} {k}")
        np.testing.assert_array_equal(b["wc"][c], a["wc"][c])
        assert b["stats"][c] == a["stats"][c]
    # one launch per window (or partial window) against two per step and group
    assert b["launches"] == sum((k + 99) // 100 for k in chunks)
    assert a["launches"] == 2 * a["groups"] * sum(chunks)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_persistent_with_fewer_ctas_per_sm_equals_two_launch_path(precision):
    """The persistent kernel compiled for one resident CTA per SM fewer (more
    registers per thread) runs the same arithmetic."""
    cells = [c1_params(nx=14, ny=9, nz=6, seed=2, cell_id=0, ku2=1.5),
             c1_params(nx=31, ny=8, nz=5, seed=2, cell_id=1, pcl_ms=300.0, lqt=0, iso2=0)]
    chunks = [250, 37, 413]
    a = _run(cells, precision, 0, chunks)
    out = {}
    with Simulator(cells, precision=precision) as sim:
        sim.set_launch_shape(persistent=1, tile_crus=128, fewer_ctas=1)
        assert sim.launch_shape() == {"persistent": 1, "tile_crus": 128, "fewer_ctas": 1,
                                      "cell_groups": sim.num_groups(), "bulk_staging": 0}
        for k in chunks:
            sim.run_steps(k)
        out["membrane"] = [sim.get_membrane(c).as_dict() for c in range(2)]
        out["state"] = [sim.get_state(c).snapshot() for c in range(2)]
    for c in range(2):
        assert out["membrane"][c] == a["membrane"][c]
        for k in ("ci", "cnsr", "cp", "cs", "nou", "ncb", "lcc", "camyo"):
            np.testing.assert_array_equal(out["state"][c][k], a["state"][c][k], err_msg=k)


def test_shape_autotuner_restores_state_and_caches_its_choice():
    cells = config3_cells(512)[:6]
    with Simulator(cells, precision="mixed", record_linescan=0) as a, \
            Simulator(cells, precision="mixed", record_linescan=0) as b:
        a.run_steps(150)
        b.run_steps(150)
        best, tried = a.autotune_shapes(8)
        # 4 persistent shapes; 3 tile lengths at one group count (6 cells cap
        # it), with each of the three stagings
        assert len(tried) == 13 and all(ms > 0 for _, ms in tried)
        assert {t["bulk_staging"] for t, _ in tried} == {0, 1, 2}
        assert {t["persistent"] for t, _ in tried} == {0, 1}
        assert a.launch_shape()["tile_crus"] == best["tile_crus"]
        assert a.get_membrane(0).step == 150
        a.run_steps(120)
        b.run_steps(120)
        for c in range(len(cells)):
            assert a.get_membrane(c).as_dict() == b.get_membrane(c).as_dict()
        # the same workload again: the cached choice, nothing timed
        best2, tried2 = b.autotune_shapes(8)
        assert tried2 == [] and best2 == best


def test_persistent_ensemble_cells_equal_two_launch_path():
    """Twelve cells of the benchmark ensemble (nx 60..100, mixed precision,
    128-CRU tiles) through two windows and an output step."""
    cells = config3_cells(512)[:12]
    a = _run(cells, "mixed", 0, [200], record_linescan=0)
    b = _run(cells, "mixed", 1, [200], record_linescan=0)
    for c in range(len(cells)):
        assert b["membrane"][c] == a["membrane"][c], c
        for k in ("ci", "cnsr", "cp", "cjsr", "nou", "nob", "lcc"):
            np.testing.assert_array_equal(b["state"][c][k], a["state"][c][k], err_msg=f"{c} {k}")
        np.testing.assert_array_equal(b["wc"][c], a["wc"][c])


def test_wait_that_never_completes_times_out_and_leaves_the_gpu_usable():
    cells = _cells()[:2]
    with Simulator(cells, precision="mixed", persistent=1) as sim:
        assert sim.kernel_launches()[1]
        sim.run_steps(20)
        sim.set_wait_limit(polls=2000, target_offset=1 << 20)  # a step no cell reaches
        with pytest.raises(NativeError, match="librh error -5"):
            sim.run_steps(100)
        assert any(sim.status(c) & RH_STATUS_TIMEOUT for c in range(len(cells)))
        sim.set_wait_limit(0, 0)
    # a new simulator on the same device runs and matches the two-launch path
    a = _run(cells, "fp64", 0, [120])
    b = _run(cells, "fp64", 1, [120])
    for c in range(len(cells)):
        assert b["membrane"][c] == a["membrane"][c]


def test_shape_choice_persists_across_processes(tmp_path):
    """With RH_SHAPE_CACHE set, the autotuner's choice is written to that file
    and a new process takes it from there without timing."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys; sys.path.insert(0, %r)\n"
            "from ryr_hyperactivity_gb300.sim import Simulator\n"
            "from ryr_hyperactivity_gb300.workloads import config3_cells\n"
            "sim = Simulator(config3_cells(512)[:4], precision='mixed', record_linescan=0)\n"
            "sim.run_steps(20)\n"
            "best, tried = sim.autotune_shapes(4)\n"
            "print(len(tried), best['persistent'], best['tile_crus'], best['cell_groups'],"
            " best['bulk_staging'])\n" % root)
    env = dict(os.environ, RH_SHAPE_CACHE=str(tmp_path / "shapes.txt"))
    first = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                           check=True).stdout.split()
    assert int(first[0]) > 0 and (tmp_path / "shapes.txt").exists()
    second = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True,
                            text=True, check=True).stdout.split()
    assert second[0] == "0" and second[1:] == first[1:]
