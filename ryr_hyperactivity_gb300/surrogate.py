"""Surrogate screening of parameter sweeps.

A small network (include/rh_mlp.h) maps a cell's parameters -- RyR open-rate
scale Ku2, IKr scale, pacing cycle length and [Ca]o -- to its EAD probability
and APD90 mean/variance.  It is trained with the library's own CUDA forward,
backward and Adam kernels on ensembles simulated by the batched stochastic
model, and is only used to decide which sweep points the full model must run:
every point it flags (EAD probability above a threshold) plus a random holdout
is re-simulated, and the holdout measures what the screen misses.

    python -m ryr_hyperactivity_gb300.surrogate generate --points 512 --out data.npz
    python -m ryr_hyperactivity_gb300.surrogate screen --data data.npz --sweep 65536
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import time

import numpy as np

from . import native
from .abi import cell_params

N_IN, N_OUT = 4, 3
H, KIN, NOUT = 128, 16, 8
SHAPES = [(H, KIN), (H, H), (H, H), (NOUT, H)]
# parameter box of the sweep (config 5): Ku2, IKr scale, PCL (ms), [Ca]o (mM)
LO = np.array([1.0, 0.0, 500.0, 1.0])
HI = np.array([3.0, 1.0, 3000.0, 2.5])
APD_SCALE = 1000.0       # ms: APD90 mean target = mean / APD_SCALE
APD_VAR_SCALE = 1.0e4    # ms^2: variance target = var / APD_VAR_SCALE


def normalise(points: np.ndarray) -> np.ndarray:
    return ((np.asarray(points, np.float64) - LO) / (HI - LO)).astype(np.float32)


def _lib():
    L = native.load()
    vp = C.c_void_p
    fp = C.POINTER(C.c_float)
    L.rh_mlp_create.argtypes = [C.c_int32, C.c_int32, C.POINTER(vp)]
    L.rh_mlp_destroy.argtypes = [vp]
    L.rh_mlp_param_count.argtypes = [vp, C.POINTER(C.c_int32)]
    L.rh_mlp_set_params.argtypes = [vp, fp]
    L.rh_mlp_get_params.argtypes = [vp, fp]
    L.rh_mlp_forward.argtypes = [vp, fp, C.c_int32, fp]
    L.rh_mlp_gradients.argtypes = [vp, fp, fp, C.c_int32, fp, fp]
    L.rh_mlp_train_step.argtypes = [vp, fp, fp, C.c_int32, C.c_float, fp]
    L.rh_mlp_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
    return L


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def init_params(seed: int = 0) -> np.ndarray:
    """He-uniform weights, zero biases, padding zeroed (parameter layout of
    include/rh_mlp.h)."""
    rng = np.random.default_rng(seed)
    parts = []
    fan_in = [N_IN, H, H, H]
    for l, (n, k) in enumerate(SHAPES):
        lim = np.sqrt(6.0 / fan_in[l]) if l < 3 else np.sqrt(3.0 / fan_in[l])
        w = rng.uniform(-lim, lim, (n, k)).astype(np.float32)
        if l == 0:
            w[:, N_IN:] = 0
        if l == 3:
            w[N_OUT:, :] = 0
        parts += [w.ravel(), np.zeros(n, np.float32)]
    return np.concatenate(parts)


class Surrogate:
    def __init__(self, batch_max: int = 4096, seed: int = 0, device: int = 0):
        self.L = _lib()
        h = C.c_void_p()
        rc = self.L.rh_mlp_create(batch_max, device, C.byref(h))
        if rc != 0:
            raise native.NativeError(f"rh_mlp_create failed ({rc})")
        self.h = h
        self.batch_max = batch_max
        n = C.c_int32()
        self.L.rh_mlp_param_count(self.h, C.byref(n))
        self.nparams = n.value
        self.set_params(init_params(seed))

    def _ck(self, rc):
        if rc != 0:
            buf = C.create_string_buffer(512)
            self.L.rh_mlp_last_error(self.h, buf, 512)
            raise native.NativeError(f"rh_mlp error {rc}: {buf.value.decode()}")

    def close(self):
        if getattr(self, "h", None):
            self.L.rh_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.nparams
        self._ck(self.L.rh_mlp_set_params(self.h, _fptr(p)))

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.nparams, np.float32)
        self._ck(self.L.rh_mlp_get_params(self.h, _fptr(p)))
        return p

    def predict(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros((x.shape[0], N_OUT), np.float32)
        self._ck(self.L.rh_mlp_forward(self.h, _fptr(x), x.shape[0], _fptr(y)))
        return y

    def gradients(self, x: np.ndarray, t: np.ndarray):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        g = np.zeros(self.nparams, np.float32)
        loss = C.c_float()
        self._ck(self.L.rh_mlp_gradients(self.h, _fptr(x), _fptr(t), x.shape[0], _fptr(g),
                                         C.byref(loss)))
        return loss.value, g

    def fit(self, x: np.ndarray, t: np.ndarray, epochs: int = 300, batch: int = 256,
            lr: float = 2e-3, seed: int = 0) -> list[float]:
        rng = np.random.default_rng(seed)
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        n = x.shape[0]
        batch = min(batch, n, self.batch_max)
        losses = []
        for ep in range(epochs):
            order = rng.permutation(n)
            tot, cnt = 0.0, 0
            for s in range(0, n - batch + 1, batch):
                idx = order[s:s + batch]
                xb = np.ascontiguousarray(x[idx])
                tb = np.ascontiguousarray(t[idx])
                loss = C.c_float()
                step_lr = lr * (0.5 * (1 + np.cos(np.pi * ep / epochs)))  # cosine schedule
                self._ck(self.L.rh_mlp_train_step(self.h, _fptr(xb), _fptr(tb), batch,
                                                  float(step_lr), C.byref(loss)))
                tot += loss.value
                cnt += 1
            losses.append(tot / max(cnt, 1))
        return losses


# ------------------------------------------------------------ full-model data

def simulate_points(points: np.ndarray, cells_per_point: int = 1, duration_ms: float = 6000.0,
                    lattice=(82, 18, 10), precision: str = "mixed", philox_seed: int = 7,
                    first_id: int = 0, skip_beats: int = 1, beats_per_cell: int = 0,
                    chunk_steps: int = 4000):
    """Runs the full stochastic model for every parameter point (Ku2, IKr scale,
    PCL, [Ca]o) and returns per point: EAD probability (fraction of recorded
    beats with an EAD), APD90 mean and variance (ms) over the recorded beats,
    and the number of beats.  All points run in one batched simulation for at
    most `duration_ms` of simulated time; the first `skip_beats` beats of each
    cell are discarded as transient.  With beats_per_cell > 0 (the shortened
    protocol) a cell is retired, its protocol ended, as soon as it has
    recorded skip_beats + beats_per_cell beats, so a short-PCL cell stops
    long before a long-PCL one."""
    from .sim import Simulator
    from .workloads import HYPER

    pts = np.asarray(points, np.float64)
    cells = []
    for i, (ku2, ikr, pcl, cao) in enumerate(pts):
        for r in range(cells_per_point):
            d = dict(HYPER)
            d["ku2"] = float(ku2)
            cells.append(cell_params(nx=lattice[0], ny=lattice[1], nz=lattice[2], nbeats=1000,
                                     pcl_ms=float(pcl), lqt=0, iso2=1, ikr_scale=float(ikr),
                                     cao_mM=float(cao), seed=philox_seed,
                                     cell_id=first_id + i * cells_per_point + r, **d))
    nsteps = int(duration_ms / 0.025)
    out = np.zeros((len(pts), 4))
    ncell = len(cells)
    beats = [[] for _ in range(ncell)]
    with Simulator(cells, precision=precision, window_steps=100, output_capacity=8,
                   record_linescan=0, track_stats=1, stats_capacity=64) as sim:
        if beats_per_cell <= 0:
            sim.run_steps(nsteps)
            for c in range(ncell):
                beats[c] = sim.drain_stats(c)
        else:
            want = skip_beats + beats_per_cell
            live = np.ones(ncell, bool)
            done = 0
            while done < nsteps and live.any():
                k = min(chunk_steps, nsteps - done)
                sim.run_steps(k)
                done += k
                for c in np.flatnonzero(live):
                    beats[c].extend(sim.drain_stats(c))
                    if len(beats[c]) >= want:  # retire: end the cell's protocol now
                        m = sim.get_membrane(c)
                        m.t = 1e12
                        sim.set_membrane(c, m)
                        live[c] = False
            for c in np.flatnonzero(live):
                beats[c].extend(sim.drain_stats(c))
        for i in range(len(pts)):
            apd, ead = [], []
            for r in range(cells_per_point):
                st = beats[i * cells_per_point + r]
                if beats_per_cell > 0:
                    st = st[:skip_beats + beats_per_cell]
                for b in st[skip_beats:]:
                    ead.append(b["ead"])
                    if b["apd90_ms"] > 0:
                        apd.append(b["apd90_ms"])
                    else:  # did not repolarise within the beat: count the full cycle
                        apd.append(pts[i, 2])
            nb = len(ead)
            out[i] = [np.mean(ead) if nb else 0.0, np.mean(apd) if apd else 0.0,
                      np.var(apd) if apd else 0.0, nb]
    return out


def targets(stats: np.ndarray) -> np.ndarray:
    return np.stack([stats[:, 0], stats[:, 1] / APD_SCALE, stats[:, 2] / APD_VAR_SCALE],
                    axis=1).astype(np.float32)


def screen(model: Surrogate, sweep_points: np.ndarray, threshold: float = 0.1,
           holdout_frac: float = 0.02, seed: int = 0):
    """Predicts every sweep point; returns (flagged indices, holdout indices,
    predictions).  The holdout is drawn from the unflagged points."""
    rng = np.random.default_rng(seed)
    pred = model.predict(normalise(sweep_points))
    flagged = np.flatnonzero(pred[:, 0] > threshold)
    rest = np.setdiff1d(np.arange(len(sweep_points)), flagged)
    nh = int(round(holdout_frac * len(sweep_points)))
    holdout = rng.choice(rest, min(nh, len(rest)), replace=False) if nh else np.array([], int)
    return flagged, holdout, pred


def _cmd_generate(a):
    rng = np.random.default_rng(a.seed)
    pts = LO + (HI - LO) * rng.random((a.points, 4))
    t0 = time.time()
    stats = simulate_points(pts, a.cells, a.duration, tuple(a.lattice), a.precision,
                            beats_per_cell=a.beats_per_cell)
    np.savez(a.out, points=pts, stats=stats, duration_ms=a.duration, cells_per_point=a.cells,
             lattice=np.array(a.lattice), precision=a.precision,
             beats_per_cell=a.beats_per_cell)
    print(json.dumps({"points": a.points, "cells": a.cells, "seconds": time.time() - t0,
                      "ead_points": int((stats[:, 0] > 0).sum())}))


def _cmd_screen(a):
    d = np.load(a.data)
    keep = d["stats"][:, 3] > 0  # points with at least one recorded beat
    pts, stats = d["points"][keep], d["stats"][keep]
    n = len(pts)
    rng = np.random.default_rng(a.seed)
    order = rng.permutation(n)
    ntr = int(0.8 * n)
    tr, te = order[:ntr], order[ntr:]
    model = Surrogate(seed=a.seed)
    losses = model.fit(normalise(pts[tr]), targets(stats[tr]), epochs=a.epochs)
    pred_te = model.predict(normalise(pts[te]))
    sweep = LO + (HI - LO) * rng.random((a.sweep, 4))
    flagged, holdout, _ = screen(model, sweep, a.threshold, 0.02, a.seed)
    res = {"train_points": int(ntr), "train_loss": losses[-1], "test_points": int(len(te)),
           "test_ead_mae": float(np.mean(np.abs(pred_te[:, 0] - stats[te, 0]))),
           "test_apd_mae_ms": float(np.mean(np.abs(pred_te[:, 1] * APD_SCALE - stats[te, 1]))),
           "sweep": a.sweep, "flagged": int(len(flagged)), "holdout": int(len(holdout)),
           "full_model_fraction": float((len(flagged) + len(holdout)) / a.sweep)}
    if a.verify > 0:
        res.update(verify(model, sweep, flagged, holdout, a.verify, a.threshold, d, rng))
    print(json.dumps(res))


def verify(model: Surrogate, sweep, flagged, holdout, cap: int, threshold: float, data, rng):
    """Re-runs up to `cap` flagged points and `cap` holdout points with the
    full stochastic model (the training data's lattice, duration and cells per
    point) and reports what the surrogate got right: the fraction of flagged
    points that do show EADs, the fraction of holdout (unflagged) points that
    show EADs the screen missed, and the prediction errors."""
    fl = rng.choice(flagged, min(cap, len(flagged)), replace=False) if len(flagged) else flagged
    ho = rng.choice(holdout, min(cap, len(holdout)), replace=False) if len(holdout) else holdout
    idx = np.concatenate([fl, ho]).astype(int)
    t0 = time.time()
    full = simulate_points(sweep[idx], int(data["cells_per_point"]), float(data["duration_ms"]),
                           tuple(int(x) for x in data["lattice"]), str(data["precision"]),
                           philox_seed=11,
                           beats_per_cell=int(data["beats_per_cell"]) if "beats_per_cell" in data
                           else 0)
    pred = model.predict(normalise(sweep[idx]))
    ok = full[:, 3] > 0
    ead_true = full[:, 0] > 0
    nf = len(fl)
    return {
        "verify_seconds": time.time() - t0,
        "verified_flagged": int(nf), "verified_holdout": int(len(ho)),
        "flagged_with_ead": float(np.mean(ead_true[:nf][ok[:nf]])) if np.any(ok[:nf]) else None,
        "holdout_with_ead": float(np.mean(ead_true[nf:][ok[nf:]])) if np.any(ok[nf:]) else None,
        "sweep_ead_points_est": None if not np.any(ok[nf:]) or not np.any(ok[:nf]) else float(
            len(flagged) * np.mean(ead_true[:nf][ok[:nf]]) +
            (len(sweep) - len(flagged)) * np.mean(ead_true[nf:][ok[nf:]])),
        "verify_ead_prob_mae": float(np.mean(np.abs(pred[ok, 0] - full[ok, 0]))),
        "verify_apd_mae_ms": float(np.mean(np.abs(pred[ok, 1] * APD_SCALE - full[ok, 1]))),
        "threshold": threshold,
    }


def main(argv=None):
    ap = argparse.ArgumentParser(prog="ryr_hyperactivity_gb300.surrogate")
    sub = ap.add_subparsers(dest="cmd", required=True)
    g = sub.add_parser("generate")
    g.add_argument("--points", type=int, default=512)
    g.add_argument("--cells", type=int, default=1)
    g.add_argument("--duration", type=float, default=6000.0)
    g.add_argument("--lattice", type=int, nargs=3, default=[82, 18, 10])
    g.add_argument("--precision", default="mixed")
    g.add_argument("--seed", type=int, default=12345)
    g.add_argument("--beats-per-cell", type=int, default=0,
                   help="shortened protocol: retire a cell after the first beat plus this many "
                        "recorded beats (0 = run every cell for --duration)")
    g.add_argument("--out", required=True)
    s = sub.add_parser("screen")
    s.add_argument("--data", required=True)
    s.add_argument("--sweep", type=int, default=65536)
    s.add_argument("--threshold", type=float, default=0.1)
    s.add_argument("--epochs", type=int, default=400)
    s.add_argument("--seed", type=int, default=0)
    s.add_argument("--verify", type=int, default=0,
                   help="re-run up to this many flagged and holdout points with the full model")
    a = ap.parse_args(argv)
    {"generate": _cmd_generate, "screen": _cmd_screen}[a.cmd](a)


if __name__ == "__main__":
    main()
