"""Mixed precision against FP64 on identical Philox streams: per-output
trace errors while the trajectories share their channel decisions, and the
per-beat ensemble statistics (APD90, peak [Ca]i, SR load, sparks, EAD
incidence) of each parameter point within their confidence intervals."""
import math

import numpy as np
import pytest

from ryr_hyperactivity_gb300 import precision as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def res():
    # 100 seeds per parameter point (the seed count of the mixed-precision
    # ensemble study), beats after the first of 3
    return P.compare(points=2, seeds=100, nx=20, ny=10, nz=5, beats=3)


def test_mixed_traces_follow_fp64_until_a_draw_flips(res):
    te = res["trace"]
    # the first upstroke shares every channel decision in most cells
    assert np.median([e["max_dv_first_beat"] for e in te]) < 1.0
    # before the trajectories part, the FP32 lattice tracks the FP64 one
    for k in ("rel_ci", "rel_cjsr", "rel_total_ca"):
        v = np.array([e[k] for e in te])
        v = v[np.isfinite(v)]
        assert np.median(v) < 1e-3, (k, np.median(v))


def test_mixed_ensemble_statistics_within_ci_of_fp64(res):
    bad = []
    for p, row in zip(res["points"], res["agreement"]):
        for k, r in row.items():
            if not np.isfinite(r["tol95"]):
                continue
            # the 95% confidence interval of the difference of the two means:
            # 1.96 standard errors, sqrt(h64^2 + hmx^2) with h = 1.96 SE each
            if abs(r["diff"]) > r["tol95"] + 1e-12:
                bad.append((p, k, r))
    assert not bad, bad
    # every point produced beats with an action potential in both precisions
    for row in res["agreement"]:
        assert row["apd90_ms"]["n"][0] > 10 and row["apd90_ms"]["n"][1] > 10
