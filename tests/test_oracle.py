"""The CPU oracle against the reference's own outputs.

The fixtures in tests/golden were produced by the reference program itself,
compiled for the host (oracle/build_ref.sh, tests/golden/make_golden.py).  The
oracle restatement must reproduce them byte for byte.
"""
import hashlib
import json
import os
import tempfile

import numpy as np
import pytest

from oracle import oracle as O
from ryr_hyperactivity_gb300.abi import cell_params

GOLD = os.path.join(os.path.dirname(__file__), "golden")
META = json.load(open(os.path.join(GOLD, "ref_full_runs.json")))


def _params(variant):
    spec = META[variant]
    a = spec["args"]
    return cell_params(clamp_mv=a[0], cjsr_basal=a[1], ncx_scale=a[2], ku=a[3], r1=a[4], kb=a[5],
                       ica_scale=a[6], ku2=a[7], seed=spec["seed"], **spec["cell"]), spec


@pytest.mark.parametrize("variant", ["c1", "c1_il", "small_il"])
def test_oracle_matches_reference_head(variant):
    p, spec = _params(variant)
    want_wt = open(os.path.join(GOLD, f"ref_{variant}_wholetest_head.txt")).read()
    want_ls = open(os.path.join(GOLD, f"ref_{variant}_linescan_head.txt")).read()
    nrec = len(want_wt.splitlines())
    o = O.Oracle(p)
    _, wc, ls = o.run(nrec * 100 - 99)
    assert len(wc) == nrec
    assert O.wholecell_text(wc) == want_wt
    nblk = want_ls.count("\n\n")
    assert O.linescan_text(ls[:nblk]) == want_ls


def test_oracle_cadist_matches_reference():
    """The cadist_ writer (cuda_Cell_Detailed.cu:1001-1013, built with
    outputcadist): first record byte for byte, all records by sha256."""
    p, _ = _params("small_il")
    spec = META["small_il_cd"]
    o = O.Oracle(p)
    recs = o.run_cadist(spec["steps"])
    text = O.cadist_text(recs)
    assert len(recs) == spec["cadist_records"]
    want = open(os.path.join(GOLD, "ref_small_il_cd_cadist_head.txt")).read()
    assert O.cadist_text(recs[:1]) == want
    assert hashlib.sha256(text.encode()).hexdigest() == spec["cadist_sha256"]


# wholecell columns of the window accumulators out_ncx, out_ica, out_ina
# (:1044-1045, :1058): the reference leaves them uninitialised before the first
# output window (:332-334), the oracle starts them at 0
WINDOW_COLS = (3, 4, 17)
PROTOCOL_VARIANTS = ["vclamp", "brownvclamp", "apclamp", "linearapclamp", "nopacing", "perm",
                     "iso", "iso_il", "slowncxchange", "oldncx", "ncx_noallo"]


@pytest.mark.parametrize("variant", PROTOCOL_VARIANTS)
def test_oracle_matches_reference_protocol_build(variant):
    """The voltage protocols, the permeabilised cell, isoproterenol,
    slowncxchange and the two unused NCX forms against the reference built
    with the matching switch: every wholetest_ and linescan_ byte, except the
    first record's uninitialised window accumulators."""
    from tests.gpu_helpers import ap_waveform, variant_params
    spec = META[variant]
    p = variant_params(spec)
    o = O.Oracle(p)
    if variant == "apclamp":
        o.set_ap_clamp(ap_waveform(p.pcl_ms))
    _, wc, ls = o.run(spec["steps"], max_rec=spec["wholetest_lines"] + 1)
    wt = O.wholecell_text(wc)
    assert len(wc) == spec["wholetest_lines"]
    first, rest = wt.split("\n", 1)
    got, want = first.split(), spec["wholetest_first_line"].split()
    assert len(got) == len(want) == 45
    assert [g for k, g in enumerate(got) if k not in WINDOW_COLS] == \
        [w for k, w in enumerate(want) if k not in WINDOW_COLS]
    assert hashlib.sha256(rest.encode()).hexdigest() == spec["wholetest_rest_sha256"]
    lst = O.linescan_text(ls)
    assert hashlib.sha256(lst.encode()).hexdigest() == spec["linescan_sha256"]


@pytest.mark.slow
def test_oracle_matches_reference_full_run():
    p, spec = _params("c1")
    o = O.Oracle(p)
    _, wc, ls = o.run(10 ** 7, max_rec=spec["wholetest_lines"] + 1)
    wt = O.wholecell_text(wc)
    lst = O.linescan_text(ls)
    assert len(wc) == spec["wholetest_lines"]
    assert hashlib.sha256(wt.encode()).hexdigest() == spec["wholetest_sha256"]
    assert hashlib.sha256(lst.encode()).hexdigest() == spec["linescan_sha256"]
    assert o.done


@pytest.mark.skipif(O.ref_binary("small_il") is None, reason="oracle/_ref not built here")
def test_oracle_matches_reference_build_live():
    p, spec = _params("small_il")
    o = O.Oracle(p)
    _, wc, ls = o.run(3000)
    with tempfile.TemporaryDirectory() as d:
        wt, lst = O.run_ref("small_il", spec["args"], d, max_steps=3000)
    assert O.wholecell_text(wc) == wt
    assert O.linescan_text(ls) == lst


def test_state_roundtrip_and_determinism():
    p, _ = _params("c1")
    a = O.Oracle(p)
    a.run(500)
    s = a.get_state()
    m = a.get_membrane()
    b = O.Oracle(p)
    b.set_state(s)
    b.set_membrane(m)
    a.run(300)
    b.run(300)
    sa, sb = a.get_state(), b.get_state()
    for k in sa.arrays:
        np.testing.assert_array_equal(sa[k], sb[k], err_msg=k)


def test_thread_count_does_not_change_results():
    p, _ = _params("c1_il")
    outs = []
    for nt in (1, 4):
        o = O.Oracle(p, threads=nt)
        _, wc, _ = o.run(400)
        outs.append(wc)
    O.lib().orc_set_threads(0)
    np.testing.assert_array_equal(outs[0], outs[1])


def test_closed_cell_conserves_total_ca():
    """With ICaL and NCX off (ica_scale = ncx_scale = 0) no Ca crosses the
    sarcolemma, so the Total_Ca column (col 45, :1031-1039, every compartment
    weighted by its volume) stays constant.  The model holds it to a few 1e-8
    relative through an action potential and its Ca transient (release,
    uptake, buffering and diffusion exchange Ca between compartments only);
    after the transient it is constant to rounding.  The FP64 GPU path follows
    these records to 1e-9 (tests/test_gpu_parity.py)."""
    from tests.gpu_helpers import c1_params
    p = c1_params(ica_scale=0.0, ncx_scale=0.0)
    o = O.Oracle(p)
    n, wc, _ = o.run(8000)
    assert n == 8000 and len(wc) == 80
    assert wc[:, 2].max() > 0  # an action potential ran
    tc = wc[:, 44]
    assert np.max(np.abs(tc - tc[0])) <= 1e-7 * tc[0]
    assert np.max(np.abs(tc[60:] - tc[60])) <= 1e-12 * tc[0]
