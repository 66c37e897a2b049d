"""Bulk state transfer (rh_export_state / rh_import_state) and the pipelined
run with host state (rh_run_steps_host): an exported state imported into a
fresh simulator continues bit for bit, and rh_run_steps_host gives the same
host image and output records as import + run + export, whether its copies
ride in the windows' graph branches per cell group (pinned buffers), run
around the steps (pageable buffers, persistent launch) or share one buffer
for both directions."""
import numpy as np
import pytest

from ryr_hyperactivity_gb300.native import NativeError
from ryr_hyperactivity_gb300.sim import Simulator
from ryr_hyperactivity_gb300.workloads import config3_cells

from tests.gpu_helpers import c1_params

pytestmark = pytest.mark.gpu


def _cells():
    ens = config3_cells(512)
    return [ens[3], c1_params(nx=14, ny=9, nz=6, seed=4, cell_id=1, ku2=1.5), ens[40],
            c1_params(nx=31, ny=8, nz=5, seed=4, cell_id=3, pcl_ms=300.0), ens[200], ens[77]]


def _pinned(nb):
    import torch
    return torch.empty(nb, dtype=torch.uint8, pin_memory=True)


def _ptr(buf):
    return buf.data_ptr() if hasattr(buf, "data_ptr") else buf.ctypes.data


def _bytes(buf):
    return buf.numpy().copy() if hasattr(buf, "numpy") else buf.copy()


def _same_records(got, want, msg=""):
    assert len(got) == len(want), msg
    for c, (g, w) in enumerate(zip(got, want)):
        np.testing.assert_array_equal(g, w, err_msg=f"{msg} cell {c}")


def _sim(**kw):
    kw.setdefault("cell_groups", 3)
    return Simulator(_cells(), precision="mixed", record_linescan=0, **kw)


def _start(sim, alloc):
    """Runs the common prefix and exports it."""
    sim.run_steps(130)
    nb = sim.state_bytes()
    h0 = alloc(nb)
    sim.export_state(_ptr(h0), nb)
    sim.drain_wholecell_all()
    return nb, h0


def _reference(nsteps, alloc=_pinned):
    """import + run + export, the three calls."""
    with _sim() as sim:
        nb, h0 = _start(sim, alloc)
        out = alloc(nb)
        sim.import_state(_ptr(h0), nb)
        sim.run_steps(nsteps)
        sim.export_state(_ptr(out), nb)
        return _bytes(h0), _bytes(out), sim.drain_wholecell_all()


@pytest.mark.parametrize("nsteps", [250, 300])
def test_run_steps_host_equals_import_run_export(nsteps):
    """250 steps: the import rides in the first (captured) window and the
    export in the last, partial window; 300: both in captured windows."""
    h0_ref, want, rec_ref = _reference(nsteps)
    with _sim() as sim:
        nb, h0 = _start(sim, _pinned)
        np.testing.assert_array_equal(_bytes(h0), h0_ref)
        out = _pinned(nb)
        sim.run_steps_host(nsteps, _ptr(h0), _ptr(out), nb)
        np.testing.assert_array_equal(_bytes(out), want)
        _same_records(sim.drain_wholecell_all(), rec_ref)
        # the device holds the same state as the exported image
        again = _pinned(nb)
        sim.export_state(_ptr(again), nb)
        np.testing.assert_array_equal(_bytes(again), want)


def test_run_steps_host_variants_agree():
    h0_ref, want, rec_ref = _reference(250)
    # pageable buffers: the copies run around the steps
    with _sim() as sim:
        nb, h0 = _start(sim, lambda n: np.empty(n, np.uint8))
        out = np.empty(nb, np.uint8)
        sim.run_steps_host(250, _ptr(h0), _ptr(out), nb)
        np.testing.assert_array_equal(out, want)
        _same_records(sim.drain_wholecell_all(), rec_ref)
    # one pinned buffer for both directions
    with _sim() as sim:
        nb, h = _start(sim, _pinned)
        sim.run_steps_host(250, _ptr(h), _ptr(h), nb)
        np.testing.assert_array_equal(_bytes(h), want)
    # import only, then export only
    with _sim() as sim:
        nb, h0 = _start(sim, _pinned)
        sim.run_steps_host(100, _ptr(h0), None, nb)
        out = _pinned(nb)
        sim.run_steps_host(150, None, _ptr(out), nb)
        np.testing.assert_array_equal(_bytes(out), want)
        _same_records(sim.drain_wholecell_all(), rec_ref)
    # one cell group (the copies run in the group's stream), and the
    # persistent launch (around the window); both are bit-identical to the
    # grouped two-launch path
    for kw in (dict(cell_groups=1), dict(persistent=1)):
        with _sim(**kw) as sim:
            nb, h0 = _start(sim, _pinned)
            out = _pinned(nb)
            sim.run_steps_host(250, _ptr(h0), _ptr(out), nb)
            np.testing.assert_array_equal(_bytes(out), want, err_msg=str(kw))
            _same_records(sim.drain_wholecell_all(), rec_ref, str(kw))


def test_exported_state_continues_in_a_fresh_simulator():
    with _sim() as a:
        nb, h0 = _start(a, _pinned)
        a.run_steps(170)
        want = _pinned(nb)
        a.export_state(_ptr(want), nb)
    with _sim() as b:
        b.import_state(_ptr(h0), nb)
        b.run_steps(170)
        got = _pinned(nb)
        b.export_state(_ptr(got), nb)
    np.testing.assert_array_equal(_bytes(got), _bytes(want))


def test_state_buffers_of_the_wrong_size_are_refused():
    with _sim() as sim:
        nb = sim.state_bytes()
        buf = np.zeros(nb + 8, np.uint8)
        with pytest.raises(NativeError):
            sim.run_steps_host(10, _ptr(buf), None, nb + 8)
        with pytest.raises(NativeError):
            sim.export_state(_ptr(buf), nb - 8)
        sim.run_steps_host(10, None, None, 0)  # no buffers: a plain run
