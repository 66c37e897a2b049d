"""CPU reference of the surrogate network's forward and backward passes.

TEST INFRASTRUCTURE ONLY: the checker for the CUDA kernels of
ryr_hyperactivity_gb300/csrc/mlp.cu.  Same parameter layout (include/rh_mlp.h),
same BF16 rounding points (weights, inputs, hidden activations, back-propagated
dZ), accumulation in float64.
"""
from __future__ import annotations

import numpy as np

H, KIN, NOUT, NIN, NO = 128, 16, 8, 4, 3
SHAPES = [(H, KIN), (H, H), (H, H), (NOUT, H)]


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 to bfloat16 (nearest, ties to even), returned as float32."""
    x = np.ascontiguousarray(x, np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def unpack(params: np.ndarray):
    ws, bs, o = [], [], 0
    for n, k in SHAPES:
        ws.append(params[o:o + n * k].reshape(n, k).astype(np.float32))
        o += n * k
        bs.append(params[o:o + n].astype(np.float32))
        o += n
    return ws, bs


def pack(ws, bs) -> np.ndarray:
    return np.concatenate([np.concatenate([w.ravel(), b]) for w, b in zip(ws, bs)]).astype(np.float32)


def mask(ws):
    ws = [w.copy() for w in ws]
    ws[0][:, NIN:] = 0
    ws[3][NO:, :] = 0
    return ws


def sigmoid(z):
    return 1.0 / (1.0 + np.exp(-z))


def softplus(z):
    return np.where(z > 20, z, np.log1p(np.exp(np.minimum(z, 20))))


def forward(params, x):
    ws, bs = unpack(params)
    ws = mask(ws)
    wb = [bf16(w).astype(np.float64) for w in ws]
    n = x.shape[0]
    x0 = np.zeros((n, KIN), np.float32)
    x0[:, :NIN] = x
    a = bf16(x0).astype(np.float64)
    acts, zs = [a], []
    for l in range(3):
        z = (a @ wb[l].T).astype(np.float32) + bs[l]
        zs.append(z)
        a = bf16(np.maximum(z, 0)).astype(np.float64)
        acts.append(a)
    z4 = (a @ wb[3].T).astype(np.float32)
    zo = z4[:, :NO] + bs[3][:NO]
    y = np.stack([sigmoid(zo[:, 0]), zo[:, 1], softplus(zo[:, 2])], axis=1)
    return y, zo, zs, acts, wb


def loss_and_grads(params, x, t):
    n = x.shape[0]
    y, zo, zs, acts, wb = forward(params, x)
    e = 1e-7
    p, m, s = t[:, 0], t[:, 1], t[:, 2]
    loss = (-(p * np.log(np.maximum(y[:, 0], e)) + (1 - p) * np.log(np.maximum(1 - y[:, 0], e)))
            + (y[:, 1] - m) ** 2 + (y[:, 2] - s) ** 2)
    dz = np.zeros((n, NOUT), np.float32)
    dz[:, 0] = (y[:, 0] - p) / n
    dz[:, 1] = 2 * (y[:, 1] - m) / n
    dz[:, 2] = 2 * (y[:, 2] - s) * sigmoid(zo[:, 2]) / n
    gws, gbs = [None] * 4, [None] * 4
    dzb = bf16(dz).astype(np.float64)
    dzf = dz.astype(np.float64)
    for l in (3, 2, 1, 0):
        gws[l] = (dzb.T @ acts[l]).astype(np.float32)
        gbs[l] = dzf.sum(axis=0).astype(np.float32)
        if l == 0:
            break
        da = (dzb @ wb[l]).astype(np.float32)
        d = np.where(zs[l - 1] > 0, da, 0).astype(np.float32)
        dzf = d.astype(np.float64)
        dzb = bf16(d).astype(np.float64)
    return float(loss.mean()), pack(gws, gbs)
