"""Per-beat statistics (APD90, EAD, peak [Ca]i, SR load, sparks): the
detectors the simulator runs on the GPU against the same detectors applied
(rh_analyze_trace) to the CPU oracle's trace of the same cell."""
import numpy as np
import pytest

from oracle import oracle as O
from ryr_hyperactivity_gb300.sim import Simulator, analyze_trace
from ryr_hyperactivity_gb300.workloads import config1_cell

pytestmark = pytest.mark.gpu


def test_beat_stats_match_oracle_trace_fp64():
    p = config1_cell()
    nsteps = 4 * 16000 + 4000  # through four beats at PCL 400 ms
    o = O.Oracle(p)
    t, v, wc = o.run_traced(nsteps)
    want = analyze_trace(p.pcl_ms, t, v, wc)
    with Simulator(p, precision="fp64") as sim:
        sim.run_steps(nsteps)
        got = sim.drain_stats(0)
    assert len(want) >= 3 and len(got) == len(want)
    for g, w in zip(got, want):
        assert g["beat"] == w["beat"] and g["ead"] == w["ead"] and g["sparks"] == w["sparks"]
        for k in ("apd90_ms", "v_peak", "ci_peak", "sr_load"):
            assert g[k] == pytest.approx(w[k], rel=1e-9, abs=1e-9), k
    # the detectors see real action potentials
    assert all(b["apd90_ms"] > 10 and b["v_peak"] > 20 for b in got)


def test_beat_stats_mixed_close_to_fp64():
    p = config1_cell()
    nsteps = 3 * 16000 + 4000
    out = {}
    for prec in ("fp64", "mixed"):
        with Simulator(p, precision=prec) as sim:
            sim.run_steps(nsteps)
            out[prec] = sim.drain_stats(0)
    a, b = out["fp64"], out["mixed"]
    assert len(a) == len(b) >= 2
    for x, y in zip(a, b):
        assert y["apd90_ms"] == pytest.approx(x["apd90_ms"], rel=0.05)
        assert y["v_peak"] == pytest.approx(x["v_peak"], abs=1.0)
        assert y["sr_load"] == pytest.approx(x["sr_load"], rel=0.02)
