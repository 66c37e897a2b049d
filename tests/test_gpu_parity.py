"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Bars: from identical state, one lattice step gives bit-identical RyR/LCC
counts and concentrations within 1e-10 relative in FP64; in the mixed (FP32
lattice) path concentrations within 1e-5 relative and the per-CRU fluxes
within 1e-5 of each flux's largest magnitude (a flux is a difference of larger
terms, so FP32 rounding scales with the terms).
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from oracle import oracle as O
from ryr_hyperactivity_gb300.abi import cell_params
from ryr_hyperactivity_gb300.sim import Simulator

from tests.gpu_helpers import (COUNT_FIELDS, DIAG, FLOAT_FIELDS, assert_text_files_match,
                               c1_params, count_mismatch, field_errors, flux_errors, rich_state)

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10
FP32_RTOL = 1e-5


def _oracle_lattice_step(p, st, m):
    o = O.Oracle(p)
    o.set_state(st)
    o.set_membrane(m)
    o.lattice_step()
    return o.get_state()


def _gpu_lattice_step(p, st, m, precision):
    with Simulator(p, precision=precision) as sim:
        sim.set_state(0, st)
        sim.set_membrane(0, m)
        sim.lattice_step()
        return sim.get_state(0)


@pytest.mark.parametrize("variant", [dict(), dict(lqt=0, iso2=0, ku2=2.0, ikr_scale=0.3),
                                     dict(ku=10.0, kb=1.0, tapsi=1)])
def test_fp64_single_step_bitexact_counts(variant):
    p = c1_params(**variant)
    st, m = rich_state(p)
    ref = _oracle_lattice_step(p, st, m)
    got = _gpu_lattice_step(p, st, m, "fp64")
    bad = count_mismatch(got, ref)
    assert not bad.any(), f"{bad.sum()} CRUs with differing counts: {np.flatnonzero(bad)[:10]}"
    errs = field_errors(got, ref)
    worst = max(errs.items(), key=lambda kv: kv[1])
    assert worst[1] <= FP64_RTOL, errs


def _gaussian_branch_crus(st, ku, ku2, kb, dt=0.025):
    """CRUs whose CU->OU (pkum) or OB->OU (pbu) transition takes the Gaussian
    branch of subroutine_cuda.c:336/447 (n > 5 and p >= 0.3, or n > 1 and
    p >= 0.2 ... evaluated as the reference does)."""
    cp, cj = st["cp"], st["cjsr"]
    common = 1 / ((1 + (5000 / cj) ** 2) * (1 + (ku / cp) ** 2))
    pku = np.minimum(4.5 * 1.5 * ku2 * common, 1 / dt)
    pkb = np.minimum(4.5 * 1.5 / 36 * kb * common, 1 / dt)
    pkum = pku * dt
    pbu = (1 / 220.0) * dt * (pku / pkb)

    def gauss(n, p):
        return ~((n <= 1) | (p < 0.2) | ((n <= 5) & (p < 0.3)))
    return gauss(st["ncu"], pkum) | gauss(st["nob"], pbu)


def test_fp64_single_step_gaussian_branches_exercised():
    """Gaussian RyR draws (Box-Muller with a dither bit) are reached when the
    bound-RyR reopening rate dominates (Ku2/Kb large) or the JSR is
    overloaded; build such CRUs, check on the oracle's inputs that the branch
    is taken, then require parity."""
    ku, ku2, kb = 1.0, 3.0, 0.01
    p = c1_params(ku=ku, ku2=ku2, kb=kb)
    st, m = rich_state(p, hot_frac=0.5, seed=3)
    rng = np.random.default_rng(4)
    over = rng.choice(st.n, st.n // 5, replace=False)
    st["cjsr"][over] = rng.uniform(5000.0, 9000.0, over.size)
    g = _gaussian_branch_crus(st, ku, ku2, kb)
    assert g.sum() > 20, g.sum()
    ref = _oracle_lattice_step(p, st, m)
    got = _gpu_lattice_step(p, st, m, "fp64")
    assert not count_mismatch(got, ref).any()
    errs = field_errors(got, ref)
    assert max(errs.values()) <= FP64_RTOL, errs


def test_mixed_single_step_within_fp32_tolerance():
    p = c1_params()
    st, m = rich_state(p, to_float32=True)
    ref = _oracle_lattice_step(p, st, m)
    got = _gpu_lattice_step(p, st, m, "mixed")
    bad = count_mismatch(got, ref)
    # float uniforms (24 bit) decide a Poisson/LCC comparison differently only
    # when the two sides are within ~6e-8 of each other
    assert bad.mean() <= 0.01, f"{bad.sum()} of {bad.size} CRUs differ in counts"
    errs = field_errors(got, ref, mask=~bad, fields=FLOAT_FIELDS)
    assert max(errs.values()) <= FP32_RTOL, errs
    ferrs = flux_errors(got, ref, mask=~bad)
    assert max(ferrs.values()) <= FP32_RTOL, ferrs


@pytest.mark.parametrize("v", [-85.0, -40.0, -5e-5, 0.3, 20.0])
def test_mixed_two_full_steps_fp32_coefficients(v):
    """The mixed cell update computes the next step's coefficients in FP32
    (gating rates, GHK and NCX factors).  From an identical state at voltage v
    (including |v| < 1e-4 mV, where taudin and the GHK factor take their
    limiting forms), two full steps, the second on those coefficients, stay
    within the FP32 tolerance of the FP64 oracle."""
    p = c1_params()
    st, m = rich_state(p, to_float32=True)
    m.v = v
    o = O.Oracle(p)
    o.set_state(st)
    o.set_membrane(m)
    for _ in range(2):
        o.step()
    ref, mref = o.get_state(), o.get_membrane()
    with Simulator(p, precision="mixed") as sim:
        sim.set_state(0, st)
        sim.set_membrane(0, m)
        sim.run_steps(2)
        got, mgot = sim.get_state(0), sim.get_membrane(0)
    bad = count_mismatch(got, ref)
    print(f"v {v}: count mismatch fraction {bad.mean():.2e}")
    assert bad.mean() <= 0.02, f"{bad.sum()} of {bad.size} CRUs differ in counts"
    errs = field_errors(got, ref, mask=~bad, fields=FLOAT_FIELDS)
    print({k: f"{e:.2e}" for k, e in errs.items()})
    assert max(errs.values()) <= FP32_RTOL, errs
    assert abs(mgot.v - mref.v) <= 1e-3, (mgot.v, mref.v)
    assert abs(mgot.xnai - mref.xnai) <= 1e-6 * abs(mref.xnai)


def test_fp64_full_steps_match_oracle_outputs():
    p = c1_params()
    nsteps = 4400  # through the first upstroke (stimulus at t = 100 ms)
    o = O.Oracle(p)
    _, wc_ref, ls_ref = o.run(nsteps)
    with Simulator(p, precision="fp64") as sim:
        sim.run_steps(nsteps)
        wc = sim.drain_wholecell(0)
        ls = sim.drain_linescan(0)
        m = sim.get_membrane(0)
        st = sim.get_state(0)
    m_ref = o.get_membrane()
    assert wc.shape == wc_ref.shape and ls.shape == ls_ref.shape
    np.testing.assert_allclose(wc, wc_ref, rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(ls, ls_ref, rtol=1e-9, atol=1e-9)
    for k in ("v", "xnai", "xm", "xh", "xj", "xr", "xs1", "qks", "xtos", "ytos", "xtof", "ytof"):
        assert abs(getattr(m, k) - getattr(m_ref, k)) <= 1e-9 * (1 + abs(getattr(m_ref, k))), k
    assert m.step == m_ref.step and m.t == m_ref.t
    ref = o.get_state()
    assert not count_mismatch(st, ref).any()
    errs = field_errors(st, ref, fields=FLOAT_FIELDS)
    assert max(errs.values()) <= 1e-8, errs


def test_batched_heterogeneous_cells_match_their_oracles():
    cells = [c1_params(nx=12, ny=9, nz=7, seed=5, cell_id=0),
             c1_params(nx=23, ny=6, nz=4, seed=5, cell_id=1, ku2=2.5, lqt=0, iso2=0),
             c1_params(nx=3, ny=3, nz=3, seed=9, cell_id=2),  # a single interior CRU
             c1_params(nx=40, ny=7, nz=6, seed=5, cell_id=3, pcl_ms=300.0, cao_mM=2.2)]
    nsteps = 4300
    with Simulator(cells, precision="fp64") as sim:
        sim.run_steps(nsteps)
        for c, p in enumerate(cells):
            o = O.Oracle(p)
            _, wc_ref, _ = o.run(nsteps)
            wc = sim.drain_wholecell(c)
            np.testing.assert_allclose(wc, wc_ref, rtol=1e-9, atol=1e-9, err_msg=f"cell {c}")
            assert not count_mismatch(sim.get_state(c), o.get_state()).any(), c


def test_runs_are_deterministic_and_resume_bit_identically():
    p = [c1_params(seed=3), c1_params(seed=3, cell_id=7, nx=17)]
    with tempfile.TemporaryDirectory() as d:
        snap = os.path.join(d, "s.bin")
        with Simulator(p, precision="mixed") as a:
            a.run_steps(700)
            a.checkpoint(snap)
            a.run_steps(650)
            sa = [a.get_state(c).snapshot() for c in range(2)]
            ma = [a.get_membrane(c).as_dict() for c in range(2)]
        with Simulator(p, precision="mixed") as b:
            b.run_steps(1350)
            sb = [b.get_state(c).snapshot() for c in range(2)]
        with Simulator(p, precision="mixed") as r:
            r.restore(snap)
            r.run_steps(650)
            sr = [r.get_state(c).snapshot() for c in range(2)]
            mr = [r.get_membrane(c).as_dict() for c in range(2)]
    for c in range(2):
        for k in sa[c]:
            if k in DIAG:
                continue
            np.testing.assert_array_equal(sa[c][k], sb[c][k], err_msg=k)
            np.testing.assert_array_equal(sa[c][k], sr[c][k], err_msg=k)
        assert ma[c] == mr[c]


def test_protocol_end_and_status():
    p = c1_params(nx=6, ny=5, nz=4, nbeats=0, pcl_ms=100.0)  # runs 2100 ms
    with Simulator(p, precision="mixed") as sim:
        sim.run_to_end()
        m = sim.get_membrane(0)
        assert not (m.t < 2100.0)
        assert sim.status(0) & 0x8
        step = m.step
        sim.run_steps(10)  # finished cells do not advance
        assert sim.get_membrane(0).step == step
        assert len(sim.drain_wholecell(0, max_rec=10000)) > 0


def test_cli_dropin_matches_oracle_files():
    exe = os.path.join(os.path.dirname(os.path.dirname(__file__)), "ryr_hyperactivity_gb300",
                       "bin", "cuda_Cell_Detailed")
    args = [1.0, 740, 1.0, 3.333, 0.00, 18.0, 0.7, 1]
    steps = 3000
    p = cell_params(nx=20, ny=10, nz=5, nbeats=2, pcl_ms=400.0, lqt=0, iso2=0)
    o = O.Oracle(p)
    _, wc_ref, ls_ref = o.run(steps)
    with tempfile.TemporaryDirectory() as d:
        subprocess.run([exe, "0", "x"] + [str(a) for a in args] +
                       ["--nx", "20", "--ny", "10", "--nz", "5", "--nbeats", "2", "--pcl", "400",
                        "--lqt", "0", "--iso2", "0", "--max-steps", str(steps)],
                       cwd=d, check=True, capture_output=True)
        wt = open(os.path.join(d, "wholetest_x")).read()
        lst = open(os.path.join(d, "linescan_x")).read()
        assert os.path.exists(os.path.join(d, "cadist_x"))
    assert_text_files_match(wt, O.wholecell_text(wc_ref))
    assert_text_files_match(lst, O.linescan_text(ls_ref))


def test_tile_sizes_agree_and_autotune_leaves_state_unchanged():
    cells = [c1_params(nx=30, ny=12, nz=6, seed=2, cell_id=0),
             c1_params(nx=17, ny=9, nz=5, seed=2, cell_id=1, ku2=2.0)]
    ref = None
    for tile in (64, 128, 256):
        with Simulator(cells, precision="fp64", block_size=tile) as sim:
            assert sim.tile_size() == tile
            sim.run_steps(600)
            st = [sim.get_state(c).snapshot() for c in range(2)]
            mv = [sim.get_membrane(c).v for c in range(2)]
        if ref is None:
            ref = (st, mv)
            continue
        for c in range(2):
            for k in ("nou", "ncu", "nob", "ncb", "lcc"):
                np.testing.assert_array_equal(st[c][k], ref[0][c][k])
            np.testing.assert_allclose(st[c]["ci"], ref[0][c]["ci"], rtol=1e-12)
            assert abs(mv[c] - ref[1][c]) < 1e-10
    with Simulator(cells, precision="mixed") as a, Simulator(cells, precision="mixed") as b:
        a.run_steps(300)
        b.run_steps(300)
        tile, ms = a.autotune(20)
        assert tile in (64, 128, 256) and all(m > 0 for m in ms)
        assert a.get_membrane(0).step == b.get_membrane(0).step == 300
        a.run_steps(200)
        b.run_steps(200)
        for c in range(2):
            for k in ("nou", "ncb", "lcc"):
                np.testing.assert_array_equal(a.get_state(c)[k], b.get_state(c)[k])


def test_cell_groups_give_identical_results():
    """Cells advance independently and the whole-cell sums are exact, so how
    the cells are grouped onto concurrent streams changes no bit of the
    state, the membrane or the output records."""
    cells = [c1_params(nx=14 + 3 * i, ny=8 + i, nz=5, seed=3, cell_id=i, ku2=1.0 + 0.4 * i)
             for i in range(5)]
    for precision in ("mixed", "fp64"):
        runs = []
        for groups in (1, 2, 5):
            with Simulator(cells, precision=precision, cell_groups=groups) as sim:
                assert (sim.num_groups() == 1) == (groups == 1)  # about equal CRU counts
                sim.run_steps(450)  # four output windows and a partial one
                runs.append(([sim.get_state(c).snapshot() for c in range(5)],
                             [sim.get_membrane(c) for c in range(5)],
                             [sim.drain_wholecell(c) for c in range(5)],
                             [sim.status(c) for c in range(5)]))
        st0, m0, wc0, s0 = runs[0]
        for st, m, wc, s in runs[1:]:
            assert s == s0
            for c in range(5):
                for k in st0[c]:
                    np.testing.assert_array_equal(st[c][k], st0[c][k], err_msg=f"{precision} {k}")
                assert m[c].v == m0[c].v and m[c].xnai == m0[c].xnai and m[c].t == m0[c].t
                np.testing.assert_array_equal(wc[c], wc0[c])


def test_batched_drain_matches_per_cell_drain():
    """rh_drain_wholecell_all returns, for every cell, the records
    rh_drain_wholecell returns, and honours max_rec and the ring wrap-around
    the same way (records beyond max_rec stay queued)."""
    cells = [c1_params(nx=12 + 2 * i, ny=7 + i, nz=5, seed=5, cell_id=i) for i in range(4)]
    out = []
    for batched in (False, True):
        with Simulator(cells, precision="mixed", output_capacity=8) as sim:
            got = [[] for _ in cells]
            for steps, max_rec in ((250, 64), (1100, 3), (100, 64)):
                sim.run_steps(steps)  # 2, then 11 (3 drained, 8 left of which the ring keeps 8), then 1
                if batched:
                    for c, rows in enumerate(sim.drain_wholecell_all(max_rec)):
                        got[c].append(rows)
                else:
                    for c in range(len(cells)):
                        got[c].append(sim.drain_wholecell(c, max_rec))
            out.append(got)
    per_cell, batched = out
    for c in range(len(cells)):
        for a, b in zip(per_cell[c], batched[c]):
            assert a.shape == b.shape and a.shape[0] > 0
            np.testing.assert_array_equal(a, b)


def _small_il():
    """The reference's small_il fixture cell (12x9x7, PCL 1000 ms, lqt/iso2
    build, curand seed 18) and its recorded cadist run."""
    import json
    gold = os.path.join(os.path.dirname(__file__), "golden")
    spec = json.load(open(os.path.join(gold, "ref_full_runs.json")))["small_il_cd"]
    a = spec["args"]
    p = cell_params(clamp_mv=a[0], cjsr_basal=a[1], ncx_scale=a[2], ku=a[3], r1=a[4], kb=a[5],
                    ica_scale=a[6], ku2=a[7], seed=spec["seed"], **spec["cell"])
    return p, spec, a


def test_fp64_cadist_matches_reference_file():
    """cadist records (the outputcadist build, cuda_Cell_Detailed.cu:1001-1013)
    through the C ABI: equal to the oracle's within 1e-9 and, printed as the
    reference prints them, the same bytes as the reference program's own
    cadist_ file (sha256 of the fixture run)."""
    import hashlib
    p, spec, _ = _small_il()
    ref = O.Oracle(p).run_cadist(spec["steps"])
    recs = []
    with Simulator(p, precision="fp64", record_cadist=1, cadist_capacity=4) as sim:
        done = 0
        while done < spec["steps"]:  # drained every 500 steps (at most 3 records)
            k = min(500, spec["steps"] - done)
            sim.run_steps(k)
            done += k
            recs.extend(sim.drain_cadist(0))
    assert len(recs) == len(ref) == spec["cadist_records"]
    for r, w in zip(recs, ref):
        assert r[0] == w[0]  # the same clock, bit for bit
        np.testing.assert_allclose(r, w, rtol=1e-9, atol=1e-12)
    text = O.cadist_text(recs)
    assert hashlib.sha256(text.encode()).hexdigest() == spec["cadist_sha256"]


def test_cadist_batched_cells_groups_and_period_gap():
    """Each cell's cadist records land in its own ring: two cells of different
    size on two streams, one with PCL 520 ms so the 500 ms recording window
    closes (no records in 500..515 ms) and reopens at the next period."""
    p0, _, _ = _small_il()
    cells = [p0, cell_params(nx=5, ny=4, nz=4, nbeats=2, pcl_ms=520.0, seed=5, cell_id=1)]
    nsteps = 21000
    refs = [O.Oracle(p).run_cadist(nsteps) for p in cells]
    got = [[], []]
    with Simulator(cells, precision="fp64", record_cadist=1, cadist_capacity=16,
                   cell_groups=2) as sim:
        assert sim.num_groups() == 2
        done = 0
        while done < nsteps:
            k = min(2000, nsteps - done)  # at most 10 records per cell between drains
            sim.run_steps(k)
            done += k
            for c in range(2):
                got[c].extend(sim.drain_cadist(c))
    for c in range(2):
        assert len(got[c]) == len(refs[c]), c
        np.testing.assert_allclose(np.array(got[c]), np.array(refs[c]), rtol=1e-9, atol=1e-12)
    t1 = np.array([r[0] for r in got[1]])
    assert not np.any((t1 > 496) & (t1 < 519)) and np.any(t1 > 519)


def test_cadist_mixed_precision_records():
    """The mixed path writes the same records at the same times; its lattice
    values are the FP32 state (ci, cs, cjsr within 1e-4 relative of FP64
    before the first stimulus)."""
    p, spec, _ = _small_il()
    out = {}
    for precision in ("fp64", "mixed"):
        with Simulator(p, precision=precision, record_cadist=1, cadist_capacity=16) as sim:
            sim.run_steps(spec["steps"])
            out[precision] = sim.drain_cadist(0)
    a, b = out["fp64"], out["mixed"]
    assert a.shape == b.shape == (spec["cadist_records"], 2 + 6 * sim.n[0])
    np.testing.assert_array_equal(a[:, 0], b[:, 0])
    ra = a[:, 2:].reshape(len(a), -1, 6)
    rb = b[:, 2:].reshape(len(b), -1, 6)
    for col in (0, 1, 3):
        np.testing.assert_allclose(rb[:, :, col], ra[:, :, col], rtol=1e-4)


def test_cli_cadist_file_is_the_reference_file():
    """The drop-in program with --cadist writes the reference's cadist_ file:
    the same sha256 as the reference program built with outputcadist."""
    import hashlib
    exe = os.path.join(os.path.dirname(os.path.dirname(__file__)), "ryr_hyperactivity_gb300",
                       "bin", "cuda_Cell_Detailed")
    p, spec, a = _small_il()
    c = spec["cell"]
    with tempfile.TemporaryDirectory() as d:
        subprocess.run([exe, "0", "cd"] + [str(x) for x in a] +
                       ["--nx", str(c["nx"]), "--ny", str(c["ny"]), "--nz", str(c["nz"]),
                        "--nbeats", str(c["nbeats"]), "--pcl", str(c["pcl_ms"]),
                        "--lqt", str(c["lqt"]), "--iso2", str(c["iso2"]), "--cadist",
                        "--max-steps", str(spec["steps"])],
                       cwd=d, check=True, capture_output=True)
        text = open(os.path.join(d, "cadist_cd")).read()
    assert text.count("header") == spec["cadist_records"]
    assert hashlib.sha256(text.encode()).hexdigest() == spec["cadist_sha256"]


def test_linescan_off_changes_nothing_else():
    """record_linescan = 0 (the reference built without outputlinescan, :46)
    drains no linescan rows and leaves every other output bit-identical."""
    p = c1_params(nx=12, ny=8, nz=5)
    out = []
    for ls in (1, 0):
        with Simulator(p, precision="mixed", record_linescan=ls) as sim:
            sim.run_steps(1000)
            out.append((sim.drain_wholecell(0), sim.drain_linescan(0)))
    assert len(out[0][1]) == 10 and len(out[1][1]) == 0
    np.testing.assert_array_equal(out[0][0], out[1][0])
