"""Host-side logic that needs no GPU: the synthetic ensemble's parameters, the
surrogate's input and target scaling and its screening split, and the
mixed-vs-FP64 report's statistics."""
import math

import numpy as np
import pytest

from ryr_hyperactivity_gb300 import precision as P
from ryr_hyperactivity_gb300 import surrogate as S
from ryr_hyperactivity_gb300.workloads import config2_cell, config3_cells, interior


def test_heterogeneous_ensemble_is_seeded_and_in_range():
    a, b = config3_cells(64), config3_cells(64)
    for p, q in zip(a, b):
        assert (p.nx, p.ny, p.nz, p.ku2, p.pcl_ms, p.ikr_scale) == \
            (q.nx, q.ny, q.nz, q.ku2, q.pcl_ms, q.ikr_scale)
    assert [p.cell_id for p in a] == list(range(64))
    assert all(60 <= p.nx <= 100 and 12 <= p.ny <= 20 and 6 <= p.nz <= 10 for p in a)
    assert all(1.0 <= p.ku2 <= 3.0 and 0.0 <= p.ikr_scale <= 1.0 for p in a)
    assert all(500.0 <= p.pcl_ms <= 3000.0 for p in a)
    # another parameter seed draws another ensemble; the first ids shift with first_id
    assert [p.nx for p in config3_cells(64, param_seed=7)] != [p.nx for p in a]
    assert config3_cells(4, first_id=100)[0].cell_id == 100
    # the full cell of the single-cell configuration: 98 x 18 x 8 interior CRUs
    assert interior(config2_cell()) == 98 * 18 * 8


def test_surrogate_scaling():
    pts = np.stack([S.LO, S.HI, 0.5 * (S.LO + S.HI)])
    x = S.normalise(pts)
    assert x.dtype == np.float32
    np.testing.assert_allclose(x, [[0, 0, 0, 0], [1, 1, 1, 1], [0.5] * 4], atol=1e-7)
    stats = np.array([[0.25, 300.0, 400.0, 8.0], [0.0, 0.0, 0.0, 0.0]])
    t = S.targets(stats)
    np.testing.assert_allclose(t, [[0.25, 300.0 / S.APD_SCALE, 400.0 / S.APD_VAR_SCALE],
                                   [0.0, 0.0, 0.0]], rtol=1e-7)


class _FakeModel:
    """Predicts an EAD probability equal to the normalised first input."""

    def predict(self, x):
        x = np.asarray(x)
        return np.stack([x[:, 0], np.zeros(len(x)), np.zeros(len(x))], axis=1)


def test_screen_flags_by_threshold_and_draws_the_holdout_from_the_rest():
    rng = np.random.default_rng(3)
    pts = S.LO + rng.random((1000, 4)) * (S.HI - S.LO)
    flagged, holdout, pred = S.screen(_FakeModel(), pts, threshold=0.7, holdout_frac=0.05,
                                      seed=11)
    np.testing.assert_array_equal(flagged, np.flatnonzero(pred[:, 0] > 0.7))
    assert len(holdout) == 50 and len(set(holdout)) == 50
    assert not set(holdout) & set(flagged)
    again = S.screen(_FakeModel(), pts, threshold=0.7, holdout_frac=0.05, seed=11)[1]
    np.testing.assert_array_equal(holdout, again)
    # no holdout asked for
    assert len(S.screen(_FakeModel(), pts, holdout_frac=0.0)[1]) == 0


def test_confidence_interval_and_paired_beat_errors():
    m, h, n = P._ci95([1.0, 2.0, 3.0, float("nan")])
    assert n == 3 and m == pytest.approx(2.0)
    assert h == pytest.approx(1.96 * 1.0 / math.sqrt(3))
    assert math.isnan(P._ci95([1.0])[1])

    def beat(b, apd, ead):
        return {"beat": b, "apd90_ms": apd, "ead": ead}

    s64 = [[beat(0, 200.0, 0), beat(1, 210.0, 0), beat(2, 220.0, 1)],
           [beat(1, -1.0, 0), beat(2, 230.0, 0)]]
    smx = [[beat(0, 100.0, 1), beat(1, 210.5, 0), beat(2, 219.0, 0)],
           [beat(1, 250.0, 0)]]
    r = P.beat_pair_errors(s64, smx, first_beat=1)
    # beats 1 and 2 of cell 0 and beat 1 of cell 1 pair up; cell 1's beat 1
    # did not repolarise in FP64, so only two APD90 differences count
    assert r["beats"] == 3
    assert r["apd90_abs_max"] == pytest.approx(1.0)
    assert r["apd90_abs_median"] == pytest.approx(0.75)
    assert r["ead_flag_differs"] == pytest.approx(1 / 3)
    assert r["ead_beats_either"] == 1
