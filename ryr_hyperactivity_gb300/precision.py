"""Mixed-precision error report.

The same cells (identical parameters and Philox streams) run once in FP64 and
once in mixed precision (FP32 lattice; FP64 voltage, [Na]i, whole-cell sums
and Total-Ca accounting).  The report gives, per output, the error of the
mixed run against the FP64 run, and per parameter point the agreement of the
ensemble statistics (mean with its 95% confidence interval in each precision).

    python -m ryr_hyperactivity_gb300.precision [--points 4] [--seeds 64]
        [--nx 20 --ny 10 --nz 6] [--beats 3] [--pcl-max 1500] [--out report.md]

Parameter points follow the heterogeneous ensemble (RyR-hyperactive base,
Ku2 ~ U[1,3], IKr scale ~ U[0,1], PCL ~ U[500, pcl_max] ms); every seed of a
point is one cell with its own Philox key (seed, cell id).  Only the paced
beats are simulated (not the 2100 ms tail of the protocol).
"""
from __future__ import annotations

import argparse
import math
import time

import numpy as np

from .abi import cell_params
from .sim import Simulator
from .workloads import HYPER

DT = 0.025
CHUNK = 4000  # steps between drains (40 output records, below the default capacity)

# wholecell record columns (0-based) compared per output
COLS = {"V": 2, "ci": 1, "cjsr": 7, "total_ca": 44}
BEAT_STATS = ["apd90_ms", "ci_peak", "sr_load", "sparks", "ead"]


def ensemble(points: int, seeds: int, nx: int, ny: int, nz: int, beats: int,
             param_seed: int = 2024, pcl_max: float = 1500.0):
    rng = np.random.default_rng(param_seed)
    ku2 = rng.uniform(1.0, 3.0, points)
    ikr = rng.uniform(0.0, 1.0, points)
    pcl = rng.uniform(500.0, pcl_max, points)
    cells, meta = [], []
    for p in range(points):
        for s in range(seeds):
            d = dict(HYPER)
            d["ku2"] = float(ku2[p])
            cells.append(cell_params(nx=nx, ny=ny, nz=nz, nbeats=beats, pcl_ms=float(pcl[p]),
                                     lqt=0, iso2=1, ikr_scale=float(ikr[p]), seed=1 + s,
                                     cell_id=p, **d))
            meta.append((p, s))
    pts = [dict(ku2=float(ku2[p]), ikr_scale=float(ikr[p]), pcl_ms=float(pcl[p]))
           for p in range(points)]
    return cells, meta, pts


def run(cells, precision: str, nsteps: int):
    """Wholecell records and beat statistics of every cell."""
    n = len(cells)
    recs = [[] for _ in range(n)]
    stats = [[] for _ in range(n)]
    with Simulator(cells, precision=precision, window_steps=100, output_capacity=64,
                   record_linescan=0, track_stats=1, stats_capacity=64) as sim:
        t0 = time.perf_counter()
        done = 0
        while done < nsteps:
            k = min(CHUNK, nsteps - done)
            sim.run_steps(k)
            done += k
            for c in range(n):
                recs[c].append(sim.drain_wholecell(c, 64))
                stats[c].extend(sim.drain_stats(c, 64))
        el = time.perf_counter() - t0
    return [np.concatenate(r) if r else np.zeros((0, 45)) for r in recs], stats, el


def _ci95(x):
    x = np.asarray(x, dtype=float)
    x = x[np.isfinite(x)]
    if len(x) < 2:
        return float("nan"), float("nan"), len(x)
    return float(x.mean()), 1.96 * float(x.std(ddof=1)) / math.sqrt(len(x)), len(x)


def beat_table(stats, meta, points, first_beat: int = 1):
    """Per point and statistic, the values over seeds and beats >= first_beat
    (the first beat starts from rest and is left out)."""
    out = [{k: [] for k in BEAT_STATS} for _ in range(points)]
    for c, st in enumerate(stats):
        p = meta[c][0]
        for b in st:
            if b["beat"] < first_beat:
                continue
            apd = b["apd90_ms"]
            out[p]["apd90_ms"].append(apd if apd >= 0 else float("nan"))
            out[p]["ci_peak"].append(b["ci_peak"])
            out[p]["sr_load"].append(b["sr_load"] if b["sr_load"] >= 0 else float("nan"))
            out[p]["sparks"].append(b["sparks"])
            out[p]["ead"].append(float(b["ead"]))
    return out


def beat_pair_errors(s64, smx, first_beat: int = 1):
    """Per-beat errors of the mixed run against the FP64 run of the same cell
    and beat (identical Philox streams): |dAPD90| over the beats where both
    repolarised, and the fraction of beats whose EAD flag differs."""
    dapd, ead_diff, ead_any, n = [], 0, 0, 0
    for a, b in zip(s64, smx):
        bb = {r["beat"]: r for r in b}
        for r in a:
            if r["beat"] < first_beat or r["beat"] not in bb:
                continue
            q = bb[r["beat"]]
            n += 1
            if r["apd90_ms"] >= 0 and q["apd90_ms"] >= 0:
                dapd.append(abs(q["apd90_ms"] - r["apd90_ms"]))
            ead_diff += int(bool(r["ead"]) != bool(q["ead"]))
            ead_any += int(bool(r["ead"]) or bool(q["ead"]))
    dapd = np.array(dapd)
    return dict(beats=n,
                apd90_abs_median=float(np.median(dapd)) if len(dapd) else float("nan"),
                apd90_abs_p95=float(np.quantile(dapd, 0.95)) if len(dapd) else float("nan"),
                apd90_abs_max=float(dapd.max()) if len(dapd) else float("nan"),
                ead_flag_differs=ead_diff / n if n else float("nan"),
                ead_beats_either=ead_any)


def trace_errors(r64, rmx):
    """Per cell: max |dV| in the first 100 ms after the first stimulus and
    over the run, time of first |dV| > 1 mV, median relative errors of the
    other outputs over the records before that time."""
    res = []
    for a, b in zip(r64, rmx):
        m = min(len(a), len(b))
        a, b = a[:m], b[:m]
        t = a[:, 0]
        dv = np.abs(a[:, COLS["V"]] - b[:, COLS["V"]])
        div = np.nonzero(dv > 1.0)[0]
        t_div = float(t[div[0]]) if len(div) else float("inf")
        pre = t < t_div if len(div) else np.ones(m, bool)
        e = {"t_diverge_ms": t_div,
             "max_dv_first_beat": float(dv[(t >= 100) & (t < 200)].max()) if np.any((t >= 100) & (t < 200)) else float("nan"),
             "max_dv": float(dv.max()) if m else float("nan")}
        for k in ("ci", "cjsr", "total_ca"):
            x, y = a[pre, COLS[k]], b[pre, COLS[k]]
            rel = np.abs(y - x) / np.maximum(np.abs(x), 1e-30)
            e[f"rel_{k}"] = float(np.median(rel)) if len(rel) else float("nan")
        res.append(e)
    return res


def compare(points=4, seeds=64, nx=20, ny=10, nz=6, beats=3, pcl_max=1500.0):
    cells, meta, pts = ensemble(points, seeds, nx, ny, nz, beats, pcl_max=pcl_max)
    nsteps = int(round(max(beats * p["pcl_ms"] for p in pts) / DT))
    r64, s64, t64 = run(cells, "fp64", nsteps)
    rmx, smx, tmx = run(cells, "mixed", nsteps)
    b64 = beat_table(s64, meta, points)
    bmx = beat_table(smx, meta, points)
    agree = []
    for p in range(points):
        row = {}
        for k in BEAT_STATS:
            m1, h1, n1 = _ci95(b64[p][k])
            m2, h2, n2 = _ci95(bmx[p][k])
            tol = math.sqrt(h1 * h1 + h2 * h2) if np.isfinite(h1) and np.isfinite(h2) else float("nan")
            row[k] = dict(fp64=m1, fp64_ci=h1, mixed=m2, mixed_ci=h2, n=(n1, n2),
                          diff=m2 - m1, tol95=tol,
                          within=bool(abs(m2 - m1) <= tol) if np.isfinite(tol) else (m1 == m2))
        agree.append(row)
    te = trace_errors(r64, rmx)
    return dict(points=pts, seeds=seeds, lattice=(nx, ny, nz), beats=beats, nsteps=nsteps,
                seconds=dict(fp64=t64, mixed=tmx), agreement=agree, trace=te,
                beat_pairs=beat_pair_errors(s64, smx))


def markdown(res) -> str:
    nx, ny, nz = res["lattice"]
    L = []
    L.append("# Mixed precision against FP64 on identical Philox streams\n")
    L.append(f"{len(res['points'])} parameter points x {res['seeds']} seeds, lattice {nx}x{ny}x{nz}, "
             f"{res['beats']} beats ({res['nsteps']} steps); run time FP64 "
             f"{res['seconds']['fp64']:.0f} s, mixed {res['seconds']['mixed']:.0f} s.\n")
    L.append("## Per-output error of the mixed run (per cell, over all cells)\n")
    te = res["trace"]
    def q(key, f=np.median):
        v = np.array([e[key] for e in te], float)
        v = v[np.isfinite(v)]
        return f(v) if len(v) else float("nan")
    L.append("| output | median over cells | max over cells |")
    L.append("|---|---:|---:|")
    L.append(f"| max abs V error, first 100 ms after the first stimulus (mV) | {q('max_dv_first_beat'):.3g} | {q('max_dv_first_beat', np.max):.3g} |")
    tdv = np.array([e["t_diverge_ms"] for e in te], float)
    ndv = int(np.isfinite(tdv).sum())
    if ndv:
        L.append(f"| time until abs V error first exceeds 1 mV, {ndv} of {len(te)} cells (ms) | "
                 f"{np.median(tdv[np.isfinite(tdv)]):.0f} | {np.max(tdv[np.isfinite(tdv)]):.0f} |")
    else:
        L.append(f"| cells whose V error ever exceeds 1 mV | 0 of {len(te)} | |")
    L.append(f"| max abs V error over the run (mV) | {q('max_dv'):.3g} | {q('max_dv', np.max):.3g} |")
    for k, name in (("rel_ci", "[Ca]i"), ("rel_cjsr", "JSR load"), ("rel_total_ca", "Total Ca")):
        L.append(f"| median relative error of {name} (records before any 1 mV V error) | {q(k):.2e} | {q(k, np.max):.2e} |")
    bp = res.get("beat_pairs")
    if bp:
        L.append(f"| APD90 error per beat, same cell and beat ({bp['beats']} beats after the first; "
                 f"median / 95th percentile, ms) | {bp['apd90_abs_median']:.3g} | "
                 f"{bp['apd90_abs_p95']:.3g} (max {bp['apd90_abs_max']:.3g}) |")
        L.append(f"| EAD flag differing, same cell and beat (fraction of beats; beats with an EAD "
                 f"in either run: {bp['ead_beats_either']}) | {bp['ead_flag_differs']:.3g} | |")
    L.append("")
    L.append("The stochastic trajectories share their random numbers, so they stay together until a")
    L.append("channel draw lands on the other side of an FP32-rounded rate; after that they are two")
    L.append("independent samples of the same process, and agreement is judged on ensemble statistics.\n")
    L.append("## Ensemble statistics per parameter point (beats after the first; mean and 95% CI)\n")
    L.append("| point (Ku2, IKr scale, PCL ms) | statistic | FP64 | mixed | difference | within 95% CI |")
    L.append("|---|---|---:|---:|---:|---|")
    for p, row in zip(res["points"], res["agreement"]):
        lab = f"({p['ku2']:.2f}, {p['ikr_scale']:.2f}, {p['pcl_ms']:.0f})"
        for k, r in row.items():
            L.append(f"| {lab} | {k} | {r['fp64']:.4g} ± {r['fp64_ci']:.2g} | {r['mixed']:.4g} ± "
                     f"{r['mixed_ci']:.2g} | {r['diff']:+.3g} | {'yes' if r['within'] else 'NO'} |")
    L.append("")
    return "\n".join(L)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--points", type=int, default=4)
    ap.add_argument("--seeds", type=int, default=64)
    ap.add_argument("--nx", type=int, default=20)
    ap.add_argument("--ny", type=int, default=10)
    ap.add_argument("--nz", type=int, default=6)
    ap.add_argument("--beats", type=int, default=3)
    ap.add_argument("--pcl-max", type=float, default=1500.0,
                    help="upper end of the PCL draw (ms); the lower end is 500")
    ap.add_argument("--out", default="")
    ap.add_argument("--json", default="", help="also write the raw result as JSON")
    a = ap.parse_args(argv)
    res = compare(a.points, a.seeds, a.nx, a.ny, a.nz, a.beats, a.pcl_max)
    if a.json:
        import json
        with open(a.json, "w") as f:
            json.dump(res, f, default=float)
    md = markdown(res)
    if a.out:
        with open(a.out, "w") as f:
            f.write(md)
    print(md)


if __name__ == "__main__":
    main()
