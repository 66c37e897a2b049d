"""The voltage protocols and the permeabilised cell on the GPU (through the C
ABI) against the oracle, which tests/test_oracle.py pins to the reference
built with each switch (cuda_Cell_Detailed.cu:34-35, :54-61, :383-396,
:694-773, :1249-1300, :1409-1411, :1603-1689)."""
import json
import os
import subprocess
import tempfile

import numpy as np
import pytest

from oracle import oracle as O
from ryr_hyperactivity_gb300.native import NativeError
from ryr_hyperactivity_gb300.sim import Simulator

from tests.gpu_helpers import ap_waveform, assert_text_files_match, c1_params, variant_params

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")
META = json.load(open(os.path.join(GOLD, "ref_full_runs.json")))
VARIANTS = ["vclamp", "brownvclamp", "apclamp", "linearapclamp", "nopacing", "perm", "iso",
            "iso_il", "slowncxchange", "oldncx", "ncx_noallo"]
EXE = os.path.join(os.path.dirname(os.path.dirname(__file__)), "ryr_hyperactivity_gb300", "bin",
                   "cuda_Cell_Detailed")


def _oracle_run(p, steps):
    o = O.Oracle(p)
    if p.protocol == 4:
        o.set_ap_clamp(ap_waveform(p.pcl_ms))
    _, wc, ls = o.run(steps, max_rec=steps // 100 + 2)
    return o, wc, ls


@pytest.mark.parametrize("variant", VARIANTS)
def test_fp64_protocol_matches_oracle(variant):
    """FP64 records follow the oracle to 1e-9 over the recorded run, and the
    membrane state ends where the oracle's does."""
    spec = META[variant]
    p = variant_params(spec)
    steps = spec["steps"]
    o, wc_ref, ls_ref = _oracle_run(p, steps)
    wc, ls = [], []
    with Simulator(p, precision="fp64") as sim:
        if variant == "apclamp":
            sim.set_ap_clamp(0, ap_waveform(p.pcl_ms))
        done = 0
        while done < steps:
            k = min(5000, steps - done)  # 50 records between drains
            sim.run_steps(k)
            done += k
            wc.append(sim.drain_wholecell(0, 64))
            ls.append(sim.drain_linescan(0, 64))
        m = sim.get_membrane(0)
    wc, ls = np.concatenate(wc), np.concatenate(ls)
    assert wc.shape == wc_ref.shape and ls.shape == ls_ref.shape
    np.testing.assert_allclose(wc, wc_ref, rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(ls, ls_ref, rtol=1e-9, atol=1e-9)
    m_ref = o.get_membrane()
    assert m.t == m_ref.t and m.step == m_ref.step
    assert abs(m.v - m_ref.v) <= 1e-9 * (1 + abs(m_ref.v))


def test_protocols_in_one_batch():
    """Cells of every protocol advance together in one batch (the same
    launches per step), each with its own voltage source, and each matches
    its own oracle."""
    cells = [c1_params(nx=9, ny=6, nz=5, seed=4, cell_id=i, pcl_ms=200.0, nbeats=2, protocol=pr,
                       clamp_mv=-20.0, perm=int(pr == "paced" and i == 6))
             for i, pr in enumerate(["paced", "nopacing", "vclamp", "brownvclamp", "apclamp",
                                     "linearapclamp", "paced"])]
    steps = 6000
    with Simulator(cells, precision="fp64", cell_groups=3) as sim:
        sim.set_ap_clamp(4, ap_waveform(200.0))
        sim.run_steps(steps)
        for c, p in enumerate(cells):
            _, wc_ref, _ = _oracle_run(p, steps)
            np.testing.assert_allclose(sim.drain_wholecell(c), wc_ref, rtol=1e-9, atol=1e-9,
                                       err_msg=f"cell {c}")


def test_randomlcc_cells_match_their_oracles():
    """randomlcc: every CRU starts with 0..8 LCCs from one Philox draw (the
    reference's own draw reads an uninitialised curand state, :1150 runs
    before setup_kernel, so this draw is defined here).  GPU and oracle give
    the same channel layout and follow each other; all nine counts occur."""
    cells = [c1_params(nx=14, ny=9, nz=6, seed=11, cell_id=i, randomlcc=1, iso=i, pcl_ms=100.0,
                       nbeats=13) for i in range(2)]
    steps = 4000
    with Simulator(cells, precision="fp64") as sim:
        st0 = [sim.get_state(c) for c in range(2)]
        sim.run_steps(steps)
        for c, p in enumerate(cells):
            o = O.Oracle(p)
            ref0 = o.get_state()
            np.testing.assert_array_equal(st0[c]["lcc"], ref0["lcc"])
            n = (st0[c]["lcc"].reshape(8, -1) < 16).sum(axis=0)
            assert set(np.unique(n)) == set(range(9))
            _, wc_ref, _ = o.run(steps)
            np.testing.assert_allclose(sim.drain_wholecell(c), wc_ref, rtol=1e-9, atol=1e-9)
            np.testing.assert_array_equal(sim.get_state(c)["lcc"], o.get_state()["lcc"])


def test_mixed_precision_protocols_run():
    """The mixed path runs the protocols too: a voltage clamp holds V exactly,
    and the records are finite where the FP64 ones are (two wholecell ratio
    columns of the reference divide by zero under a long clamp) and close to
    FP64."""
    ps = [variant_params(META["vclamp"]), variant_params(META["perm"])]
    for p in ps:
        out = {}
        for precision in ("fp64", "mixed"):
            with Simulator(p, precision=precision) as sim:
                sim.run_steps(5000)
                out[precision] = sim.drain_wholecell(0)
        a, b = out["fp64"], out["mixed"]
        assert a.shape == b.shape
        np.testing.assert_array_equal(np.isfinite(b), np.isfinite(a))
        if p.protocol == 2:  # the clamp sets V itself: the same value in both paths
            np.testing.assert_array_equal(a[:, 2], b[:, 2])
        np.testing.assert_allclose(b[:, 7], a[:, 7], rtol=2e-2)  # mean JSR load


def test_ap_clamp_waveform_is_required_and_checked():
    p = variant_params(META["apclamp"])
    with Simulator(p, precision="mixed") as sim:
        with pytest.raises(NativeError, match="waveform not set"):
            sim.run_steps(10)
        with pytest.raises(NativeError, match="samples"):
            sim.set_ap_clamp(0, np.zeros(10))
        sim.set_ap_clamp(0, ap_waveform(p.pcl_ms))
        sim.run_steps(10)
    with Simulator(c1_params(), precision="mixed") as sim:
        with pytest.raises(NativeError, match="not RH_PROTO_AP_CLAMP"):
            sim.set_ap_clamp(0, ap_waveform(400.0))


@pytest.mark.parametrize("variant", ["vclamp", "apclamp", "perm", "iso", "slowncxchange", "oldncx"])
def test_cli_protocol_builds(variant):
    """The drop-in program's --protocol / --perm options write the files the
    reference's protocol builds write (numerically equal to the oracle's;
    apclamp reads v_1000.txt from the working directory as the reference
    does)."""
    spec = META[variant]
    p = variant_params(spec)
    c = spec["cell"]
    steps = min(spec["steps"], 6000)
    _, wc_ref, ls_ref = _oracle_run(p, steps)
    flags = ["--nx", str(c["nx"]), "--ny", str(c["ny"]), "--nz", str(c["nz"]),
             "--nbeats", str(c["nbeats"]), "--pcl", str(c["pcl_ms"]), "--lqt", str(c["lqt"]),
             "--iso2", str(c["iso2"]), "--max-steps", str(steps)]
    if "protocol" in c:
        flags += ["--protocol", c["protocol"]]
    if c.get("perm"):
        flags += ["--perm"]
    if c.get("iso"):
        flags += ["--iso"]
    if c.get("slowncx"):
        flags += ["--slowncxchange"]
    if "ncx_form" in c:
        flags += ["--ncx", c["ncx_form"]]
    with tempfile.TemporaryDirectory() as d:
        if variant == "apclamp":
            with open(os.path.join(d, "v_1000.txt"), "w") as f:
                f.write("".join("%.17g\n" % x for x in ap_waveform(p.pcl_ms)))
        subprocess.run([EXE, "0", "x"] + [str(a) for a in spec["args"]] + flags, cwd=d,
                       check=True, capture_output=True)
        wt = open(os.path.join(d, "wholetest_x")).read()
        lst = open(os.path.join(d, "linescan_x")).read()
    got = np.array([[float(v) for v in line.split()] for line in wt.splitlines()])
    np.testing.assert_allclose(got, wc_ref, rtol=1e-5, atol=2e-6)
    assert_text_files_match(wt, O.wholecell_text(wc_ref))
    assert_text_files_match(lst, O.linescan_text(ls_ref))
