"""The surrogate's CPU reference (oracle/mlp_oracle.py) checked on its own:
with its BF16 rounding points turned off, its analytic gradients of the mean
loss equal central finite differences of that loss.  This pins the checker
that tests/test_gpu_mlp.py holds the GPU gradients against."""
import numpy as np
import pytest

from oracle import mlp_oracle as MO


def _valid_params_mask():
    """Parameters the network uses (the padded input columns and output rows
    are masked out by the model)."""
    ws = [np.ones((n, k), np.float32) for n, k in MO.SHAPES]
    bs = [np.ones(n, np.float32) for n, _ in MO.SHAPES]
    ws = MO.mask(ws)
    bs[3][MO.NO:] = 0
    return MO.pack(ws, bs) > 0


def test_gradients_match_finite_differences(monkeypatch):
    monkeypatch.setattr(MO, "bf16", lambda x: np.asarray(x, np.float32))
    rng = np.random.default_rng(7)
    n_params = sum(n * k + n for n, k in MO.SHAPES)
    params = (rng.standard_normal(n_params) * 0.15).astype(np.float32)
    x = rng.uniform(-1, 1, (64, MO.NIN)).astype(np.float32)
    t = np.stack([rng.uniform(0, 1, 64), rng.normal(0, 1, 64), rng.uniform(0.1, 1, 64)], axis=1)
    loss, grad = MO.loss_and_grads(params, x, t)
    assert np.isfinite(loss)
    valid = _valid_params_mask()
    assert np.all(grad[~valid] == 0)  # masked parameters get no gradient
    cand = np.flatnonzero(valid & (np.abs(grad) > 1e-2))
    assert len(cand) > 50
    checked = 0
    for i in rng.choice(cand, 40, replace=False):
        eps = 1e-3
        p1, p2 = params.copy(), params.copy()
        p1[i] += eps
        p2[i] -= eps
        fd = (MO.loss_and_grads(p1, x, t)[0] - MO.loss_and_grads(p2, x, t)[0]) / (2 * eps)
        assert fd == pytest.approx(float(grad[i]), rel=3e-2, abs=1e-3), i
        checked += 1
    assert checked == 40
