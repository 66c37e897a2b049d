"""Failure detection, with every failure made on the host (no GPU fault).

- rh_restore refuses a snapshot of another simulator: a corrupted header,
  another lattice, another precision, other cell parameters, a truncated
  file; each refusal is RH_ERR_IO and leaves the live state untouched.
- A NaN written into one CRU's state with rh_set_state is reported as
  RH_STATUS_NAN by rh_cell_status after one step, for that cell only.
- An RyR transition probability above 1 per step (the OB->OU probability pbu
  of subroutine_cuda.c:443 is not capped, so a large Ku2/Kb ratio drives it
  past 1) makes the Gaussian draw NaN; the draw is repeated until the
  200-try cap of subroutine_cuda.c:358-361 and counts 0, and the step sets
  RH_STATUS_RATE_CAP and RH_STATUS_GAUSS_RETRY, as the oracle does.
"""
import os
import tempfile

import numpy as np
import pytest

from oracle import oracle as O
from ryr_hyperactivity_gb300.native import NativeError
from ryr_hyperactivity_gb300.sim import Simulator

from tests.gpu_helpers import FLOAT_FIELDS, c1_params, count_mismatch, field_errors, rich_state

pytestmark = pytest.mark.gpu

RH_STATUS_NAN = 0x1
RH_STATUS_GAUSS_RETRY = 0x2
RH_STATUS_RATE_CAP = 0x10


def _cells(**kw):
    return [c1_params(nx=12, ny=8, nz=5, seed=4, cell_id=0, **kw),
            c1_params(nx=9, ny=7, nz=6, seed=4, cell_id=1, **kw)]


def _snapshot(sim):
    return [(sim.get_state(c).snapshot(), sim.get_membrane(c).as_dict()) for c in range(sim.ncells)]


def _assert_same(a, b):
    for (sa, ma), (sb, mb) in zip(a, b):
        assert ma == mb
        for k in sa:
            np.testing.assert_array_equal(sa[k], sb[k], err_msg=k)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_restore_refuses_foreign_snapshots(precision):
    with tempfile.TemporaryDirectory() as d:
        good = os.path.join(d, "good.bin")
        with Simulator(_cells(), precision=precision) as sim:
            sim.run_steps(150)
            sim.checkpoint(good)
        blob = open(good, "rb").read()
        bad = {}
        # header: magic
        bad["magic"] = b"X" + blob[1:]
        # truncated inside the lattice arena, and just before the last byte
        bad["truncated"] = blob[: len(blob) // 2]
        bad["last byte"] = blob[:-1]
        for name, data in bad.items():
            with open(os.path.join(d, name), "wb") as f:
                f.write(data)
        # another lattice, another precision, other cell parameters (same layout)
        other = {"lattice": (_cells()[:1] + [c1_params(nx=14, ny=7, nz=6, seed=4, cell_id=1)],
                             precision),
                 "precision": (_cells(), "mixed" if precision == "fp64" else "fp64"),
                 "parameters": (_cells(ku2=2.0), precision)}
        for name, (cells, prec) in other.items():
            with Simulator(cells, precision=prec) as s2:
                s2.run_steps(50)
                s2.checkpoint(os.path.join(d, name))
        with Simulator(_cells(), precision=precision) as sim:
            sim.run_steps(100)
            before = _snapshot(sim)
            want = {"magic": "not a snapshot", "truncated": "truncated", "last byte": "truncated",
                    "lattice": "not a snapshot", "precision": "not a snapshot",
                    "parameters": "different cell parameters"}
            for name, text in want.items():
                with pytest.raises(NativeError, match=r"librh error -6: .*" + text):
                    sim.restore(os.path.join(d, name))
                _assert_same(_snapshot(sim), before)
            with pytest.raises(NativeError, match="librh error -6"):
                sim.restore(os.path.join(d, "missing.bin"))
            # the refused restores left a working simulator; the good one resumes it
            sim.run_steps(10)
            sim.restore(good)
            assert sim.get_membrane(0).step == 150


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("field", ["cp", "ci"])
def test_nan_written_into_state_is_reported(precision, field):
    with Simulator(_cells(), precision=precision) as sim:
        sim.run_steps(20)
        assert sim.status(0) & RH_STATUS_NAN == 0 and sim.status(1) & RH_STATUS_NAN == 0
        st = sim.get_state(0)
        st[field][st.n // 3] = np.nan
        sim.set_state(0, st)
        sim.run_steps(1)
        assert sim.status(0) & RH_STATUS_NAN
        assert sim.status(1) & RH_STATUS_NAN == 0  # the other cell is clean


def test_rate_above_one_sets_rate_cap_and_retry_bits():
    ku, ku2, kb = 1.0, 3.0, 0.01  # pbu = dt/220 * 36*Ku2/Kb = 1.23 per step
    p = c1_params(ku=ku, ku2=ku2, kb=kb)
    st, m = rich_state(p, seed=7)
    rng = np.random.default_rng(8)
    idx = rng.choice(st.n, st.n // 10, replace=False)
    nob = rng.integers(2, 20, idx.size)  # n > 1 with p > 1: the Gaussian branch
    st["nob"][idx] = nob
    st["ncb"][idx] = np.minimum(st["ncb"][idx], 100 - st["nou"][idx] - nob)
    st["ncu"][idx] = 100 - st["nou"][idx] - nob - st["ncb"][idx]
    o = O.Oracle(p)
    o.set_state(st)
    o.set_membrane(m)
    o.lattice_step()
    ref = o.get_state()
    want = RH_STATUS_RATE_CAP | RH_STATUS_GAUSS_RETRY
    assert o.status & want == want
    with Simulator(p, precision="fp64") as sim:
        sim.set_state(0, st)
        sim.set_membrane(0, m)
        assert sim.status(0) & want == 0
        sim.lattice_step()
        got = sim.get_state(0)
        assert sim.status(0) & want == want
    assert not count_mismatch(got, ref).any()
    errs = field_errors(got, ref, fields=FLOAT_FIELDS)
    assert max(errs.values()) <= 1e-10, errs
