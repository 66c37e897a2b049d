"""Generates the golden fixtures in this directory from the reference program
compiled for the host (oracle/_ref, built by oracle/build_ref.sh from the
reference sources).  Run where the reference sources exist, REF_SRC naming
their directory:

    REF_SRC=<reference sources> bash oracle/build_ref.sh && python tests/golden/make_golden.py

Fixtures (all produced by running the reference's own code):
  ref_<variant>_wholetest_head.txt   first wholetest_ lines of the run
  ref_<variant>_linescan_head.txt    first linescan_ blocks of the run
  ref_full_runs.json                 sha256 and line counts of the complete
                                     wholetest_/linescan_ files of each run
  ref_small_il_cd_cadist_head.txt    first record of the cadist_ file of the
                                     small_il build with outputcadist defined,
                                     run for CADIST_STEPS steps (its sha256 is in
                                     ref_full_runs.json under "small_il_cd")

The protocol and option builds (vclamp, brownvclamp, apclamp, linearapclamp,
nopacing, perm, iso, iso_il, slowncxchange, oldncx, ncx_noallo) are recorded
in ref_full_runs.json only: the first wholetest_ line as
text (in some of these builds it carries the reference's uninitialised
window accumulators, cuda_Cell_Detailed.cu:332-334), the sha256 of the rest
of the file and of the linescan_ file.  The apclamp build reads the waveform
tests.gpu_helpers.ap_waveform writes into its v_1000.txt.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from tests.gpu_helpers import ap_waveform  # noqa: E402

# (variant, reference argv a3..a10, lattice/protocol the variant was built with)
RUNS = {
    "c1": dict(args=[1.0, 740, 1.0, 3.333, 0.00, 18.0, 0.7, 1],
               cell=dict(nx=20, ny=10, nz=5, nbeats=2, pcl_ms=400.0, lqt=0, iso2=0,
                         linescan_jz=-1)),
    "c1_il": dict(args=[1.0, 740, 1.0, 3.333, 0.00, 18.0, 0.7, 1],
                  cell=dict(nx=20, ny=10, nz=5, nbeats=2, pcl_ms=400.0, lqt=1, iso2=1,
                            linescan_jz=-1)),
    "small_il": dict(args=[1.0, 740, 1.0, 10, 0.00, 1.0, 0.7, 1],
                     cell=dict(nx=12, ny=9, nz=7, nbeats=1, pcl_ms=1000.0, lqt=1, iso2=1,
                               linescan_jz=-1)),
}
# protocol builds: (reference argv a3..a10, cell, steps); each cell's lattice,
# PCL and build modes are those oracle/build_ref.sh compiles the variant with
CONTROL = [1.0, 740, 1.0, 3.333, 0.00, 18.0, 0.7, 1]
PROTOCOL_RUNS = {
    "vclamp": dict(args=[-10.0] + CONTROL[1:],
                   cell=dict(nx=12, ny=8, nz=5, nbeats=1, pcl_ms=400.0, lqt=0, iso2=0,
                             linescan_jz=-1, protocol="vclamp"), steps=6000),
    "brownvclamp": dict(args=CONTROL,
                        cell=dict(nx=6, ny=5, nz=4, nbeats=2, pcl_ms=3000.0, lqt=0, iso2=0,
                                  linescan_jz=-1, protocol="brownvclamp"), steps=300000),
    "apclamp": dict(args=CONTROL,
                    cell=dict(nx=10, ny=6, nz=5, nbeats=2, pcl_ms=200.0, lqt=1, iso2=1,
                              linescan_jz=-1, protocol="apclamp"), steps=20000),
    "linearapclamp": dict(args=CONTROL,
                          cell=dict(nx=12, ny=8, nz=5, nbeats=1, pcl_ms=1000.0, lqt=0, iso2=0,
                                    linescan_jz=-1, protocol="linearapclamp"), steps=16500),
    "nopacing": dict(args=CONTROL,
                     cell=dict(nx=12, ny=8, nz=5, nbeats=1, pcl_ms=400.0, lqt=1, iso2=1,
                               linescan_jz=-1, protocol="nopacing"), steps=5000),
    "perm": dict(args=CONTROL[:7] + [2],
                 cell=dict(nx=12, ny=9, nz=6, nbeats=1, pcl_ms=1000.0, lqt=0, iso2=0,
                           linescan_jz=-1, perm=1), steps=6000),
    # iso through the LCC insertion and SERCA boost at 5.5 PCL and the end of
    # pacing at 11.9 PCL
    "iso": dict(args=CONTROL,
                cell=dict(nx=8, ny=6, nz=5, nbeats=13, pcl_ms=100.0, lqt=0, iso2=0,
                          linescan_jz=-1, iso=1), steps=52000),
    "iso_il": dict(args=CONTROL,
                   cell=dict(nx=8, ny=6, nz=5, nbeats=13, pcl_ms=100.0, lqt=1, iso2=1,
                             linescan_jz=-1, iso=1), steps=30000),
    "slowncxchange": dict(args=CONTROL,
                          cell=dict(nx=12, ny=8, nz=5, nbeats=1, pcl_ms=400.0, lqt=0, iso2=0,
                                    linescan_jz=-1, slowncx=1), steps=12000),
    "oldncx": dict(args=CONTROL,
                   cell=dict(nx=12, ny=8, nz=5, nbeats=1, pcl_ms=400.0, lqt=0, iso2=0,
                             linescan_jz=-1, ncx_form="oldncx"), steps=12000),
    "ncx_noallo": dict(args=CONTROL,
                       cell=dict(nx=12, ny=8, nz=5, nbeats=1, pcl_ms=400.0, lqt=0, iso2=0,
                                 linescan_jz=-1, ncx_form="ncx_noallo"), steps=12000),
}
CADIST_VARIANT = "small_il_cd"  # small_il with the cadist_ writer enabled
CADIST_STEPS = 1700
HEAD_WHOLETEST_LINES = 40
HEAD_LINESCAN_BLOCKS = 6


def sha(text: str) -> str:
    return hashlib.sha256(text.encode()).hexdigest()


def main() -> None:
    meta = {}
    for variant, spec in RUNS.items():
        with tempfile.TemporaryDirectory() as d:
            wt, ls = O.run_ref(variant, spec["args"], d)
        wt_lines = wt.splitlines(keepends=True)
        blocks = ls.split("\n\n")
        with open(os.path.join(HERE, f"ref_{variant}_wholetest_head.txt"), "w") as f:
            f.write("".join(wt_lines[:HEAD_WHOLETEST_LINES]))
        with open(os.path.join(HERE, f"ref_{variant}_linescan_head.txt"), "w") as f:
            f.write("\n\n".join(blocks[:HEAD_LINESCAN_BLOCKS]) + "\n\n")
        meta[variant] = dict(args=spec["args"], cell=spec["cell"], seed=18,
                             wholetest_sha256=sha(wt), wholetest_lines=len(wt_lines),
                             linescan_sha256=sha(ls), linescan_lines=len(ls.splitlines()))
        print(variant, meta[variant]["wholetest_lines"], "wholetest lines")
    spec = RUNS["small_il"]
    with tempfile.TemporaryDirectory() as d:
        O.run_ref(CADIST_VARIANT, spec["args"], d, max_steps=CADIST_STEPS)
        cd = O.ref_cadist(d)
    first = cd.split("0 header")[1]
    with open(os.path.join(HERE, f"ref_{CADIST_VARIANT}_cadist_head.txt"), "w") as f:
        f.write("0 header" + first)
    meta[CADIST_VARIANT] = dict(args=spec["args"], cell=spec["cell"], seed=18, steps=CADIST_STEPS,
                                cadist_sha256=sha(cd), cadist_records=cd.count("0 header"))
    print(CADIST_VARIANT, meta[CADIST_VARIANT]["cadist_records"], "cadist records")
    for variant, spec in PROTOCOL_RUNS.items():
        with tempfile.TemporaryDirectory() as d:
            if spec["cell"].get("protocol") == "apclamp":
                with open(os.path.join(d, "v_1000.txt"), "w") as f:
                    f.write("".join("%.17g\n" % x for x in ap_waveform(spec["cell"]["pcl_ms"])))
            wt, ls = O.run_ref(variant, spec["args"], d, max_steps=spec["steps"])
        first, rest = wt.split("\n", 1)
        meta[variant] = dict(args=spec["args"], cell=spec["cell"], seed=18, steps=spec["steps"],
                             wholetest_first_line=first, wholetest_rest_sha256=sha(rest),
                             wholetest_lines=len(wt.splitlines()), linescan_sha256=sha(ls),
                             linescan_lines=len(ls.splitlines()))
        print(variant, meta[variant]["wholetest_lines"], "wholetest lines")
    with open(os.path.join(HERE, "ref_full_runs.json"), "w") as f:
        json.dump(meta, f, indent=1)


if __name__ == "__main__":
    main()
