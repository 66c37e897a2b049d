"""Benchmark of the per-time-step myocyte update on one GB300 (or N, one
process per GPU, cells sharded with no collective on the data path).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload: the heterogeneous ensemble (512 cells, nx~U{60..100},
ny~U{12..20}, nz~U{6..10}, Ku2~U[1,3], IKr scale~U[0,1], PCL~U[500,3000]) in
mixed precision (FP32 lattice, FP64 V/[Na]i/reductions), per GPU.  One bench
step = one output window = 100 lattice updates (2.5 ms of simulated time) of
every cell.  The state (~1 GB) is far larger than L2, so no flush is needed.

Printed (rank 0, one JSON line): CRU-updates/s (value), cell-beats/s, the
step kernel's HBM roofline, the plain FP64 single-cell path (100x20x10) for
the 10x target, the end-to-end number through the C ABI with host buffers,
and the CPU baseline (the reference's routines built for the host, or the
oracle port where that build is absent).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WINDOW = 100  # lattice updates per bench step
DT = 0.025


def _env_rank():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.samples = []
        self._stop = threading.Event()
        self._t = threading.Thread(target=self._run, daemon=True)

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True,
                                     text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        import statistics
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 5 + i and s[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def _peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def _fp64_profile():
    """FP64-pipe utilisation of the FP64 lattice kernel from its committed ncu
    summary (profiles/step_kernel_fp64.json)."""
    try:
        return json.load(open(os.path.join(ROOT, "profiles", "step_kernel_fp64.json")))
    except Exception:
        return None


def _traffic_profile():
    try:
        return json.load(open(os.path.join(ROOT, "profiles", "step_kernel_traffic.json")))
    except Exception:
        return None


# The CPU baseline: the reference's own update routines compiled for the host
# (oracle/build_ref.sh, variant bench_mean: Compute, the host ODE and the
# writers of cuda_Cell_Detailed.cu, OpenMP over the lattice sites) on the mean
# lattice of the ensemble, 80x16x8 (6552 interior CRUs), PCL 1750 ms, with the
# RyR-hyperactive argv of run.sh:9 and Ku2 = 2 (the ensemble's mean).  Where
# that build is absent the oracle port (the same update restated in C, pinned
# byte for byte to the reference build) runs instead.
MEAN_CELL = dict(nx=80, ny=16, nz=8, pcl_ms=1750.0)
MEAN_ARGS = [1.0, 740, 1.0, 3.333, 0.0, 18.0, 0.7, 2.0]
REF_SAMPLE_STEPS = 1000  # lattice updates per reference sample (one process run)


def _mean_interior() -> int:
    return (MEAN_CELL["nx"] - 2) * (MEAN_CELL["ny"] - 2) * (MEAN_CELL["nz"] - 2)


def _reference_exe():
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_bench_mean")
    return exe if os.access(exe, os.X_OK) else None


class CpuSampler:
    """Runs bounded samples of the mean-size cell on the host cores: the
    reference build when present ("reference"), else the oracle port."""

    def __init__(self, threads: int | None = None):
        self.threads = threads or os.cpu_count() or 1
        self.exe = _reference_exe()
        self.kind = "reference" if self.exe else "port"
        self.n = _mean_interior()
        self._o = None
        self._dir = None

    def sample(self, steps: int) -> float:
        """Runs `steps` lattice updates; returns the elapsed seconds."""
        if self.exe:
            import tempfile
            if self._dir is None:
                self._dir = tempfile.mkdtemp(prefix="rh_ref_")
            env = dict(os.environ, REF_MAX_STEPS=str(int(steps)),
                       OMP_NUM_THREADS=str(self.threads))
            t0 = time.perf_counter()
            subprocess.run([self.exe, "0", "b"] + [str(a) for a in MEAN_ARGS], cwd=self._dir,
                           env=env, check=True, stdout=subprocess.DEVNULL)
            return time.perf_counter() - t0
        if self._o is None:
            from oracle import oracle as O
            from ryr_hyperactivity_gb300.abi import cell_params
            from ryr_hyperactivity_gb300.workloads import HYPER
            d = dict(HYPER, ku2=2.0)
            p = cell_params(nbeats=20, lqt=0, iso2=1, seed=1, cell_id=0, **MEAN_CELL, **d)
            self._o = O.Oracle(p, threads=self.threads)
        t0 = time.perf_counter()
        self._o.run(steps)
        return time.perf_counter() - t0

    def describe(self, steps: int, seconds: float) -> str:
        what = ("the reference's host build (oracle/_ref/ref_bench_mean), one process run per "
                "sample" if self.kind == "reference" else "the oracle port")
        return (f"{what}: one 80x16x8 cell ({self.n} interior CRUs), {steps} steps in "
                f"{REF_SAMPLE_STEPS}-step samples, {seconds:.1f} s")


def cpu_baseline(seconds: float = 12.0, threads: int | None = None) -> dict:
    """The CPU baseline on the mean-size ensemble cell for about `seconds`."""
    cs = CpuSampler(threads)
    cs.sample(100)  # warm
    el, steps = 0.0, 0
    while el < seconds:
        el += cs.sample(REF_SAMPLE_STEPS)
        steps += REF_SAMPLE_STEPS
    return {"value": cs.n * steps / el, "unit": "CRU-updates/s", "cores": cs.threads,
            "kind": cs.kind, "sample": cs.describe(steps, el),
            "cell_beats_per_s": steps * DT / MEAN_CELL["pcl_ms"] / el}


def run_reference(args, rank, world):
    """Reference arm: the reference's update routines on the host cores, same
    metric and unit as the GPU arm; each bench step is one bounded sample of
    the ensemble's mean-size cell (REF_SAMPLE_STEPS lattice updates)."""
    if rank != 0:
        return
    cs = CpuSampler()
    for _ in range(args.warmup):
        cs.sample(REF_SAMPLE_STEPS // 10)
    el = 0.0
    for _ in range(args.steps):
        el += cs.sample(REF_SAMPLE_STEPS)
    steps = REF_SAMPLE_STEPS * args.steps
    val = cs.n * steps / el
    cb = steps * DT / MEAN_CELL["pcl_ms"] / el
    line = {"impl": "reference", "metric": "CRU-updates/s", "value": val, "unit": "CRU-updates/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "cell_beats_per_s": cb,
            "config": {"workload": "heterogeneous ensemble, 512 cells/GPU", "precision": "fp64",
                       "sample": "the ensemble's mean-size cell (80x16x8), %d lattice updates "
                                 "per bench step, host CPU" % REF_SAMPLE_STEPS,
                       "window_steps": REF_SAMPLE_STEPS},
            "cpu_baseline": {"value": val, "unit": "CRU-updates/s", "cores": cs.threads,
                             "kind": cs.kind, "sample": cs.describe(steps, el)},
            "e2e": {"value": val, "unit": "CRU-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cells", type=int, default=512)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--tile", type=int, default=0,
                    help="CRUs per CTA (64, 128, 256); 0 = pick with the autotuner")
    ap.add_argument("--groups", type=int, default=0,
                    help="cell groups on concurrent streams (0 = library default)")
    ap.add_argument("--persistent", type=int, default=0, choices=[0, 1],
                    help="with --tile: 1 = one persistent launch per window, 0 = two "
                         "launches per step and cell group")
    ap.add_argument("--bulk", type=int, default=0, choices=[0, 1, 2],
                    help="with --tile, two-launch path, mixed precision: 1 = staging by bulk "
                         "asynchronous copies, 2 = by tensor copies")
    args = ap.parse_args()
    rank, world, local = _env_rank()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()

    from ryr_hyperactivity_gb300.sim import Simulator
    from ryr_hyperactivity_gb300.workloads import config2_cell, config3_cells, interior

    cells = config3_cells(args.cells, first_id=rank * args.cells)
    n_in = sum(interior(p) for p in cells)
    # the per-beat detectors (APD90, EAD, peak [Ca]i, SR load, sparks) run in
    # the timed region, as an ensemble study needs them
    sim = Simulator(cells, precision=args.precision, device=local, window_steps=WINDOW,
                    track_stats=1, stats_capacity=64, block_size=args.tile,
                    cell_groups=args.groups)
    bpc = sim.bytes_per_cru_step()
    for _ in range(args.warmup):
        sim.run_steps(WINDOW)
    if args.tile:
        sim.set_launch_shape(args.persistent, args.tile, 0, args.groups, args.bulk)
        tune = []
    else:  # launch shape for this workload (the simulation state is unchanged)
        _, tune = sim.autotune_shapes(40)
    shape = sim.launch_shape()
    tile = shape["tile_crus"]
    sim.kernel_timing()  # reset
    sim.drain_wholecell_all()
    kernels0, persistent = sim.kernel_launches()
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            sim.run_steps(WINDOW)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    barrier()
    launches, kms = sim.kernel_timing()  # lattice updates; CUDA events on the sim's stream
    kernels = sim.kernel_launches()[0] - kernels0
    el = kms / 1e3
    if dist is not None:
        t = torch.tensor([el], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        el = float(t.item())
    upd = n_in * WINDOW * args.steps * world
    value = upd / el
    cell_beats = sum(WINDOW * DT / p.pcl_ms for p in cells) * args.steps * world / el
    avg_launch_s = kms / 1e3 / max(launches, 1)
    achieved = bpc * n_in / avg_launch_s / 1e9
    peaks = _peaks()
    peak = peaks.get("hbm_gbs")
    prof = _traffic_profile()
    traffic = None
    if prof and prof.get("precision") == args.precision:
        traffic = prof["dram_bytes_per_cru_update"] * n_in
    result = {
        "metric": "CRU-updates/s", "value": value, "unit": "CRU-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if args.precision == "mixed" else "f64", "data": "synthetic",
        "cell_beats_per_s": cell_beats,
        "config": {"workload": f"heterogeneous ensemble, {args.cells} cells/GPU",
                   "precision": args.precision, "cells": args.cells, "interior_crus": n_in,
                   "window_steps": WINDOW,
                   "step": "one output window = 100 lattice updates of every cell",
                   "l2": f"state {sim.state_bytes() / 1e9:.2f} GB > 129 MB L2, no flush",
                   "parallelism": f"cells sharded, {world} GPU(s)",
                   "launch_shape": shape,
                   "launch": ("one persistent cooperative launch per window, %d CTAs of %d "
                              "threads" % (sim.window_ctas(), tile) if persistent else
                              "two launches per step and cell group, %d groups, %d-CRU tiles"
                              % (sim.num_groups(), tile)),
                   "autotune_ms_per_update": [
                       {"persistent": t["persistent"], "tile": t["tile_crus"],
                        "fewer_ctas": t["fewer_ctas"], "groups": t["cell_groups"],
                        "bulk_staging": t["bulk_staging"], "ms": round(m, 4)}
                       for t, m in tune]},
        "gpu_launches": kernels,  # counted by the library
        "timed_wall_s": wall,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if peak else None, "traffic": traffic,
                     "bytes_per_cru_update": bpc, "kernel_ms": avg_launch_s * 1e3,
                     "kernel_ms_is": "one lattice update of every cell (lattice and whole-cell "
                                     "updates): the window launch's time per step" if persistent
                                     else "one lattice update of every cell: per cell group one "
                                     "step-kernel launch and one cell-update launch, the groups "
                                     "running concurrently",
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peak else None},
        "clocks": clk.summary(),
    }
    # end to end through the C ABI with host buffers: every window imports
    # the whole state from pinned host memory, runs, exports the state and
    # drains the output records (rh_run_steps_host: each cell group's copies
    # overlap the other groups' steps)
    if not args.no_e2e:
        nb = sim.state_bytes()
        host = torch.empty(nb, dtype=torch.uint8, pin_memory=True)
        sim.export_state(host.data_ptr(), nb)
        sim.drain_wholecell_all()
        reps = max(4, args.steps)  # the host copies' rate varies from run to run
        ring = sim.ncells * (sim.opts.output_capacity or 64) * 45 * 8  # the batched drain's copy
        sim.run_steps_host(WINDOW, host.data_ptr(), host.data_ptr(), nb)  # its graphs, untimed
        sim.drain_wholecell_all()
        t0 = time.perf_counter()
        for _ in range(reps):
            sim.run_steps_host(WINDOW, host.data_ptr(), host.data_ptr(), nb)
            sim.drain_wholecell_all()
        e2e_el = time.perf_counter() - t0
        # the sequential form (import, run, export) beside it
        t0 = time.perf_counter()
        for _ in range(reps):
            sim.import_state(host.data_ptr(), nb)
            sim.run_steps(WINDOW)
            sim.export_state(host.data_ptr(), nb)
            sim.drain_wholecell_all()
        seq_el = time.perf_counter() - t0
        result["e2e"] = {"value": n_in * WINDOW * reps / e2e_el, "unit": "CRU-updates/s",
                         "h2d_bytes_per_step": nb, "d2h_bytes_per_step": nb + ring,
                         "api": "rh_run_steps_host(100, state image in and out, pinned) + "
                                "rh_drain_wholecell_all",
                         "sequential_value": n_in * WINDOW * reps / seq_el,
                         "sequential_api": "rh_import_state + rh_run_steps(100) + "
                                           "rh_export_state + rh_drain_wholecell_all"}
    sim.close()
    # plain FP64 single-cell path (the 10x target's denominator)
    if not args.no_fp64 and rank == 0:
        p2 = config2_cell()
        s64 = Simulator(p2, precision="fp64", window_steps=WINDOW, track_stats=0)
        s64.run_steps(WINDOW)
        s64.kernel_timing()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        nw = 5
        for _ in range(nw):
            s64.run_steps(WINDOW)
        torch.cuda.synchronize()
        e64 = time.perf_counter() - t0
        l64, k64 = s64.kernel_timing()
        s64.close()
        v64 = interior(p2) * WINDOW * nw / e64
        cb64 = WINDOW * DT / p2.pcl_ms * nw / e64
        result["fp64_single_cell"] = {
            "workload": "100x20x10 single cell, FP64", "cru_updates_per_s": v64,
            "cell_beats_per_s": cb64, "kernel_ms": k64 / max(l64, 1),
            "mixed_batched_over_fp64_single_cell_cell_beats": cell_beats / world / cb64}
    # the same 512-cell ensemble with every field and operation in FP64
    # (batched FP64): its lattice kernel is bound by the FP64 pipe
    if not args.no_fp64 and rank == 0 and args.precision == "mixed":
        sb = Simulator(cells, precision="fp64", device=local, window_steps=WINDOW, track_stats=1,
                       stats_capacity=64, block_size=args.tile, cell_groups=args.groups)
        sb.run_steps(WINDOW)
        _, tune64 = sb.autotune_shapes(10)
        shape64 = sb.launch_shape()
        sb.kernel_timing()
        torch.cuda.synchronize()
        nwb = 2
        for _ in range(nwb):
            sb.run_steps(WINDOW)
        torch.cuda.synchronize()
        lb, kb = sb.kernel_timing()
        bpc64 = sb.bytes_per_cru_step()
        sb.close()
        vb = n_in * WINDOW * nwb / (kb / 1e3)
        cbb = sum(WINDOW * DT / p.pcl_ms for p in cells) * nwb / (kb / 1e3)
        ach64 = bpc64 * n_in / (kb / 1e3 / max(lb, 1)) / 1e9
        fp64_prof = _fp64_profile()
        result["fp64_batched"] = {
            "workload": f"heterogeneous ensemble, {args.cells} cells, FP64",
            "cru_updates_per_s": vb, "cell_beats_per_s": cbb, "kernel_ms": kb / max(lb, 1),
            "launch_shape": shape64,
            "autotune_ms_per_update": [
                {"persistent": t["persistent"], "tile": t["tile_crus"], "fewer_ctas": t["fewer_ctas"],
                 "groups": t["cell_groups"], "ms": round(m, 3)} for t, m in tune64],
            "roofline": {"bound": "fp64", "hbm_achieved": ach64, "hbm_peak": peak,
                         "hbm_frac": (ach64 / peak) if peak else None,
                         "bytes_per_cru_update": bpc64,
                         "fp64_pipe_pct_of_peak_ncu": fp64_prof.get("fp64_pipe_pct") if fp64_prof
                         else None,
                         "fp64_evidence": fp64_prof.get("source") if fp64_prof else None},
            "mixed_over_fp64_batched_cell_beats": cell_beats / world / cbb}
    if rank == 0 and not args.no_cpu:
        result["cpu_baseline"] = cpu_baseline()
    if rank == 0:
        print(json.dumps(result), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
