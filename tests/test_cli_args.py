"""The drop-in program's argument handling, on the host: malformed command
lines are rejected with the usage text and exit code 2 before any device work,
and parameters the simulator rejects end the run with exit code 1 and the
library's error text (host-side fault injection; no GPU is touched)."""
import os
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "ryr_hyperactivity_gb300", "bin", "cuda_Cell_Detailed")
ARGS = ["0", "t", "1.0", "740", "1.0", "3.333", "0", "18", "0.7", "1"]  # run.sh:9


def _run(args):
    if not os.path.exists(CLI):
        pytest.skip("drop-in program not built")
    with tempfile.TemporaryDirectory() as d:
        r = subprocess.run([CLI] + args, cwd=d, capture_output=True, text=True, timeout=60)
    return r.returncode, r.stderr


@pytest.mark.parametrize("args", [
    [],
    ARGS[:9],
    ARGS + ["--bogus"],
    ARGS + ["--protocol", "sideways"],
    ARGS + ["--ncx", "reverse"],
    ARGS + ["--nx"],
])
def test_malformed_command_lines_exit_2_with_usage(args):
    rc, err = _run(args)
    assert rc == 2
    assert "usage: cuda_Cell_Detailed" in err


def test_rejected_lattice_exits_1_with_the_library_error():
    rc, err = _run(ARGS + ["--nx", "2"])
    assert rc == 1
    assert "rh_create failed" in err and "lattice" in err
