"""The surrogate network's CUDA kernels: forward and hand-written backward
against the CPU reference (oracle/mlp_oracle.py, same BF16 rounding points),
training convergence, and the screening gain on a simulated ensemble."""
import os

import numpy as np
import pytest

from oracle import mlp_oracle as MO
from ryr_hyperactivity_gb300.surrogate import (Surrogate, init_params, normalise, screen,
                                               targets)

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _batch(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.random((n, 4)).astype(np.float32)
    t = np.stack([rng.random(n), rng.random(n) * 0.5, rng.random(n) * 0.2], 1).astype(np.float32)
    return x, t


def test_forward_matches_cpu_reference():
    m = Surrogate(batch_max=512, seed=1)
    p = init_params(1)
    x, _ = _batch(300, 2)
    y = m.predict(x)
    y_ref = MO.forward(p, x)[0]
    np.testing.assert_allclose(y, y_ref, rtol=2e-3, atol=2e-3)


def test_backward_gradients_match_cpu_reference():
    """Hand-written backward pass vs the CPU oracle's gradients (BF16 operands,
    FP32 accumulation): every layer's weight and bias gradient."""
    m = Surrogate(batch_max=512, seed=3)
    p = init_params(3)
    x, t = _batch(256, 4)
    loss, g = m.gradients(x, t)
    loss_ref, g_ref = MO.loss_and_grads(p, x, t)
    assert loss == pytest.approx(loss_ref, rel=2e-3)
    o = 0
    for (n, k) in MO.SHAPES:
        for size in (n * k, n):
            a, b = g[o:o + size], g_ref[o:o + size]
            scale = np.max(np.abs(b)) + 1e-12
            assert np.max(np.abs(a - b)) <= 2e-2 * scale, (n, k, size)
            assert np.linalg.norm(a - b) <= 1e-2 * (np.linalg.norm(b) + 1e-12)
            o += size


def test_training_reduces_loss_on_smooth_targets():
    rng = np.random.default_rng(5)
    x = rng.random((2048, 4)).astype(np.float32)
    # a smooth map of the same kind as the physiology targets
    p = 1 / (1 + np.exp(-(8 * x[:, 0] - 6 * x[:, 1] + 2 * x[:, 2] - 3)))
    mu = 0.2 + 0.3 * x[:, 2] - 0.1 * x[:, 1] + 0.05 * x[:, 3]
    var = 0.05 * p
    t = np.stack([p, mu, var], 1).astype(np.float32)
    m = Surrogate(batch_max=1024, seed=0)
    losses = m.fit(x, t, epochs=60, batch=256, lr=3e-3)
    y = m.predict(x)
    assert losses[-1] < 0.7 * losses[0]
    assert np.mean(np.abs(y[:, 0] - p)) < 0.05
    assert np.mean(np.abs(y[:, 1] - mu)) < 0.03


@pytest.mark.skipif(not os.path.exists(os.path.join(GOLD, "surrogate_ensemble.npz")),
                    reason="simulated ensemble fixture not generated")
def test_screening_gain_on_simulated_ensemble():
    """Train on 80% of the simulated parameter points, screen the other 20%:
    the full model only needs the flagged points plus a 2% holdout, and the
    flagged set must catch most of the EAD-positive points."""
    d = np.load(os.path.join(GOLD, "surrogate_ensemble.npz"))
    keep = d["stats"][:, 3] > 0  # points with at least one recorded beat
    pts, stats = d["points"][keep], d["stats"][keep]
    rng = np.random.default_rng(0)
    order = rng.permutation(len(pts))
    ntr = int(0.8 * len(pts))
    tr, te = order[:ntr], order[ntr:]
    m = Surrogate(seed=0)
    m.fit(normalise(pts[tr]), targets(stats[tr]), epochs=300, batch=128, lr=2e-3)
    flagged, holdout, pred = screen(m, pts[te], threshold=0.1, holdout_frac=0.02)
    positive = stats[te, 0] > 0.1
    caught = positive[flagged].sum() if len(flagged) else 0
    run_fraction = (len(flagged) + len(holdout)) / len(te)
    recall = caught / max(positive.sum(), 1)
    # the screen must skip work and still find the EAD region
    if positive.any():
        assert recall >= 0.7, (recall, positive.sum())
    assert run_fraction < 0.9
    # APD90 prediction error on unseen points
    apd_err = np.median(np.abs(pred[:, 1] * 1000.0 - stats[te, 1]))
    assert apd_err < 0.25 * np.median(stats[te, 1])


@pytest.mark.parametrize("shape", [
    # (M, N, K, a_k_major, b_k_major): the network's forward, dW and dA products
    (300, 128, 128, True, True),
    (77, 8, 16, True, True),
    (128, 16, 1000, False, False),
    (8, 128, 300, False, True),
    (4096, 128, 128, True, False),
])
def test_tcgen05_gemm_matches_exact_product(shape):
    """The tcgen05 GEMM (BF16 operands staged in shared memory, FP32
    accumulator in tensor memory) against the float64 product of the same
    BF16 values, and against the mma.sync kernel, for the operand layouts the
    network's forward and backward passes use."""
    import ctypes as C
    import torch
    from ryr_hyperactivity_gb300 import native
    M, N, K, ak, bk = shape
    L = native.load()
    L.rh_mlp_gemm_check.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_int32,
                                    C.c_int32, C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                    C.c_int32, C.c_int32]
    g = torch.Generator().manual_seed(M * 7 + N + K)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16)
    B = torch.randn(K, N, generator=g).to(torch.bfloat16)
    want = A.double().numpy() @ B.double().numpy()
    # device layouts: A row-major (k fastest) or column-major (m fastest), B likewise
    Ad = (A if ak else A.t().contiguous()).cuda()
    Bd = (B.t().contiguous() if bk else B).cuda()
    sam, sak = (K, 1) if ak else (1, M)
    sbk, sbn = (1, K) if bk else (N, 1)
    out = {}
    for tcores in (1, 0):
        Cd = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
        rc = L.rh_mlp_gemm_check(Ad.data_ptr(), sam, sak, Bd.data_ptr(), sbk, sbn, Cd.data_ptr(),
                                 N, M, N, K, tcores)
        assert rc == 0, rc
        out[tcores] = Cd.cpu().double().numpy()
    scale = np.abs(want).max()
    np.testing.assert_allclose(out[1], want, rtol=1e-5, atol=1e-5 * scale)
    np.testing.assert_allclose(out[1], out[0], rtol=1e-5, atol=1e-5 * scale)
