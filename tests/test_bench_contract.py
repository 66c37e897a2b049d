"""The reference arm of bench.py (the reference's host build, or the oracle
port where that build is absent, on the host cores) prints one JSON line with
the fields and units of the GPU arm; runs on CPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "1"], check=True, capture_output=True,
                         text=True, timeout=600).stdout
    lines = [ln for ln in out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "CRU-updates/s" and d["unit"] == "CRU-updates/s"
    assert d["higher_is_better"] is True and d["value"] > 0
    assert d["config"]["workload"] == "heterogeneous ensemble, 512 cells/GPU"
    assert d["cpu_baseline"]["kind"] in ("reference", "port") and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"]
