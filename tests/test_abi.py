"""C ABI boundary checks that need no GPU: the library loads, exports every
function include/rh.h declares, and formats records exactly as the
reference's fprintf calls (checked against the oracle's restatement)."""
import os
import re

import numpy as np
import pytest

from ryr_hyperactivity_gb300 import native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for hdr in os.listdir(os.path.join(ROOT, "include")):
        if not hdr.endswith(".h") or hdr == "rh_philox.h":
            continue
        txt = open(os.path.join(ROOT, "include", hdr)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names |= set(re.findall(r"^\s*(?:int|void)\s+(rh_\w+)\s*\(", txt, flags=re.M))
    return names


def test_library_exports_every_declared_symbol():
    L = native.load()
    declared = _declared()
    assert "rh_create" in declared and len(declared) >= 20
    for name in sorted(declared):
        assert hasattr(L, name), name
    assert declared <= set(native.EXPORTS) | declared


def test_defaults_match_reference_build():
    import ctypes as C
    from ryr_hyperactivity_gb300.abi import CellParams, RunOpts
    L = native.load()
    p = CellParams()
    L.rh_default_cell_params(C.byref(p))
    assert (p.nx, p.ny, p.nz, p.nbeats, p.pcl_ms) == (64, 28, 12, 7, 4000.0)
    assert (p.lqt, p.iso2, p.tapsi, p.seed) == (1, 1, 0, 18)
    o = RunOpts()
    L.rh_default_run_opts(C.byref(o))
    assert o.dt_ms == 0.025 and o.precision == 0


def test_create_rejects_bad_arguments_without_gpu_work():
    import ctypes as C
    from ryr_hyperactivity_gb300.abi import cell_params
    L = native.load()
    h = C.c_void_p()
    p = cell_params(nx=2)
    rc = L.rh_create(C.byref(p), 1, None, C.byref(h))
    assert rc == -1 and not h.value
    buf = C.create_string_buffer(256)
    L.rh_last_error(None, buf, 256)
    assert b"lattice" in buf.value


def test_calls_on_a_null_handle_are_rejected():
    """Every per-simulator entry point returns RH_ERR_ARG for a NULL handle
    (no device work is attempted)."""
    import ctypes as C
    L = native.load()
    n = C.c_int32()
    rows = (C.c_double * 45)()
    assert L.rh_run_steps(None, 10) == -1
    assert L.rh_drain_wholecell(None, 0, rows, 1, C.byref(n)) == -1
    assert L.rh_drain_wholecell_all(None, rows, 1, C.byref(n)) == -1
    assert L.rh_num_cells(None, C.byref(n)) == -1
    assert L.rh_num_groups(None, C.byref(n)) == -1


def test_record_formats_match_reference():
    from oracle import oracle as O
    from ryr_hyperactivity_gb300.sim import format_linescan, format_wholecell
    rng = np.random.default_rng(0)
    for _ in range(50):
        w = rng.normal(size=45) * 10.0 ** rng.integers(-3, 4, size=45)
        w[[26, 27, 28, 29, 30, 31, 32, 33, 34, 35, 36, 40]] = rng.integers(0, 30000, size=12)
        assert format_wholecell(w) == O.format_wholecell(w)
        r = rng.normal(size=22) * 100
        r[[3, 4, 5, 6, 7]] = rng.integers(0, 100, size=5)
        assert format_linescan(r) == O.format_linescan(r)
