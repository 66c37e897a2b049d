"""rh_mlp_forward_noalloc, the surrogate forward pass that allocates nothing
(its intermediates live in a fixed device array inside the library), against
rh_mlp_forward, the handle-based forward, on the same parameters and inputs:
two calls in a row with different parameters and batch sizes, so that
anything the first call leaves in the shared array would show in the second.
Device buffers come from torch, standing in for a caller's own allocator."""
import ctypes as C

import numpy as np
import pytest

from ryr_hyperactivity_gb300 import native
from ryr_hyperactivity_gb300.surrogate import Surrogate, init_params

pytestmark = pytest.mark.gpu

MAX_BATCH = 4096  # RH_MLP_NOALLOC_MAX_BATCH
RTOL = ATOL = 2e-3  # the surrogate forward tolerance of the other network tests


def _entry():
    f = native.load().rh_mlp_forward_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_char_p,
                  C.c_size_t]
    f.restype = C.c_int
    return f


def _case(seed, n):
    rng = np.random.default_rng(seed)
    p = init_params(seed)
    p = (p * rng.uniform(0.8, 1.2, p.shape)).astype(np.float32)
    x = rng.random((n, 4)).astype(np.float32)
    return p, x


def _reference(p, x):
    m = Surrogate(batch_max=512, seed=0)
    try:
        m.set_params(p)
        return m.predict(x)
    finally:
        m.close()


def _noalloc(f, p, x):
    import torch

    dp = torch.from_numpy(p).cuda()
    dx = torch.from_numpy(x).cuda()
    dy = torch.full((x.shape[0], 3), float("nan"), dtype=torch.float32, device="cuda")
    err = C.create_string_buffer(256)
    torch.cuda.synchronize()
    rc = f(dp.data_ptr(), dx.data_ptr(), x.shape[0], dy.data_ptr(), None, err, 256)
    assert rc == 0, err.value.decode()
    torch.cuda.synchronize()
    return dy.cpu().numpy()


def test_noalloc_forward_matches_handle_forward_on_two_calls():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    f = _entry()
    for seed, n in ((11, MAX_BATCH), (12, 37)):
        p, x = _case(seed, n)
        y_ref = _reference(p, x)
        y = _noalloc(f, p, x)
        assert np.isfinite(y).all()
        np.testing.assert_allclose(y, y_ref, rtol=RTOL, atol=ATOL)


def test_noalloc_forward_rejects_what_it_cannot_hold():
    torch = pytest.importorskip("torch")
    f = _entry()
    p, x = _case(13, 8)
    dp = torch.from_numpy(p).cuda()
    big = torch.zeros((MAX_BATCH + 1, 4), dtype=torch.float32, device="cuda")
    dy = torch.zeros((MAX_BATCH + 1, 3), dtype=torch.float32, device="cuda")
    err = C.create_string_buffer(256)
    rc = f(dp.data_ptr(), big.data_ptr(), MAX_BATCH + 1, dy.data_ptr(), None, err, 256)
    assert rc == -1  # RH_ERR_ARG
    assert str(MAX_BATCH) in err.value.decode()
    assert f(dp.data_ptr(), big.data_ptr(), 0, dy.data_ptr(), None, err, 256) == -1
    # a host buffer is refused on the host before any GPU work
    assert f(dp.data_ptr(), x.ctypes.data, 8, dy.data_ptr(), None, err, 256) == -1
    assert "device memory" in err.value.decode()
    torch.cuda.synchronize()
    assert float(dy.abs().sum()) == 0.0
