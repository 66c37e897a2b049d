"""ctypes binding of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  The oracle restates the
reference's per-step update in FP64 C (see rh_oracle.c for the line-by-line
citations).  Build it with ``make -C oracle``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_HERE)
if _ROOT not in sys.path:
    sys.path.insert(0, _ROOT)

from ryr_hyperactivity_gb300.abi import (  # noqa: E402
    LINESCAN_COLS, WHOLECELL_COLS, CellParams, HostState, Membrane, StateF64)

LIB_PATH = os.path.join(_HERE, "liboracle.so")
REF_DIR = os.path.join(_HERE, "_ref")

_lib = None


def build() -> None:
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(CellParams), C.c_double]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_get_threads.restype = C.c_int
        L.orc_step.argtypes = [C.c_void_p]
        L.orc_step.restype = C.c_int
        L.orc_run.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_double), C.c_int32,
                              C.POINTER(C.c_int32), C.POINTER(C.c_double), C.c_int32,
                              C.POINTER(C.c_int32)]
        L.orc_run.restype = C.c_int64
        L.orc_lattice_step.argtypes = [C.c_void_p]
        L.orc_run_traced.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_double),
                                     C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int32,
                                     C.POINTER(C.c_int32)]
        L.orc_run_traced.restype = C.c_int64
        L.orc_get_state.argtypes = [C.c_void_p, C.POINTER(StateF64)]
        L.orc_set_state.argtypes = [C.c_void_p, C.POINTER(StateF64)]
        L.orc_get_membrane.argtypes = [C.c_void_p, C.POINTER(Membrane)]
        L.orc_set_membrane.argtypes = [C.c_void_p, C.POINTER(Membrane)]
        L.orc_last_wholecell.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.orc_last_linescan.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.orc_last_linescan.restype = C.c_int32
        L.orc_last_cadist.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.orc_last_cadist.restype = C.c_int32
        L.orc_set_ap_clamp.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_int64]
        L.orc_set_ap_clamp.restype = C.c_int32
        L.orc_protocol_done.argtypes = [C.c_void_p]
        L.orc_protocol_done.restype = C.c_int32
        L.orc_status.argtypes = [C.c_void_p]
        L.orc_status.restype = C.c_uint32
        L.orc_interior.argtypes = [C.c_void_p]
        L.orc_interior.restype = C.c_int32
        L.orc_format_wholecell.argtypes = [C.POINTER(C.c_double), C.c_char_p, C.c_size_t]
        L.orc_format_linescan.argtypes = [C.POINTER(C.c_double), C.c_char_p, C.c_size_t]
        _lib = L
    return _lib


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def format_wholecell(row) -> str:
    a = np.ascontiguousarray(row, np.float64)
    buf = C.create_string_buffer(4096)
    lib().orc_format_wholecell(_dptr(a), buf, 4096)
    return buf.value.decode()


def format_linescan(row) -> str:
    a = np.ascontiguousarray(row, np.float64)
    buf = C.create_string_buffer(1024)
    lib().orc_format_linescan(_dptr(a), buf, 1024)
    return buf.value.decode()


class Oracle:
    """One cell simulated by the CPU oracle."""

    def __init__(self, params: CellParams, dt: float = 0.025, threads: int | None = None):
        self.L = lib()
        if threads is not None:
            self.L.orc_set_threads(int(threads))
        self.params = params
        self.h = self.L.orc_create(C.byref(params), float(dt))
        if not self.h:
            raise ValueError("orc_create rejected the parameters")
        self.n = self.L.orc_interior(self.h)
        self.lx = params.nx - 2

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.L.orc_destroy(h)
            self.h = None

    def step(self) -> bool:
        r = self.L.orc_step(self.h)
        if r < 0:
            raise RuntimeError("AP-clamp waveform not set")
        return bool(r)

    def set_ap_clamp(self, v) -> None:
        """Waveform of an AP-clamp cell: (int)(pcl/dt + 0.1) voltages (mV)."""
        a = np.ascontiguousarray(v, np.float64)
        if self.L.orc_set_ap_clamp(self.h, _dptr(a), len(a)) != 0:
            raise ValueError("orc_set_ap_clamp rejected the waveform")

    def lattice_step(self) -> None:
        self.L.orc_lattice_step(self.h)

    def run(self, nsteps: int, max_rec: int | None = None):
        """Runs nsteps; returns (steps_run, wholecell[nrec,45], linescan[nrec,lx,22])."""
        if max_rec is None:
            max_rec = nsteps // 100 + 2
        wc = np.zeros((max_rec, WHOLECELL_COLS))
        ls = np.zeros((max_rec, self.lx, LINESCAN_COLS))
        nrec = C.c_int32(0)
        nbl = C.c_int32(0)
        done = self.L.orc_run(self.h, int(nsteps), _dptr(wc), max_rec, C.byref(nrec), _dptr(ls),
                              max_rec, C.byref(nbl))
        return done, wc[: nrec.value].copy(), ls[: nbl.value].copy()

    def run_traced(self, nsteps: int):
        """Runs nsteps; returns (t[n], v[n], wholecell[nrec,45]) where t is each
        step's time before the step and v the voltage after it."""
        t = np.zeros(nsteps)
        v = np.zeros(nsteps)
        max_rec = nsteps // 100 + 2
        wc = np.zeros((max_rec, WHOLECELL_COLS))
        nrec = C.c_int32(0)
        done = self.L.orc_run_traced(self.h, int(nsteps), _dptr(t), _dptr(v), _dptr(wc), max_rec,
                                     C.byref(nrec))
        return t[:done].copy(), v[:done].copy(), wc[: nrec.value].copy()

    def run_cadist(self, nsteps: int) -> list[np.ndarray]:
        """Runs nsteps and returns the cadist records written on the way
        (each: t, v, then 6 values per interior CRU, reference order)."""
        recs = []
        buf = np.zeros(2 + 6 * self.n)
        for _ in range(int(nsteps)):
            if self.done:
                break
            if self.L.orc_step(self.h) < 0:
                raise RuntimeError("AP-clamp waveform not set")
            if self.L.orc_last_cadist(self.h, _dptr(buf)):
                recs.append(buf.copy())
        return recs

    def get_state(self) -> HostState:
        hs = HostState(self.n)
        self.L.orc_get_state(self.h, C.byref(hs.view))
        return hs

    def set_state(self, hs: HostState) -> None:
        self.L.orc_set_state(self.h, C.byref(hs.view))

    def get_membrane(self) -> Membrane:
        m = Membrane()
        self.L.orc_get_membrane(self.h, C.byref(m))
        return m

    def set_membrane(self, m: Membrane) -> None:
        self.L.orc_set_membrane(self.h, C.byref(m))

    def last_wholecell(self) -> np.ndarray:
        a = np.zeros(WHOLECELL_COLS)
        self.L.orc_last_wholecell(self.h, _dptr(a))
        return a

    def last_linescan(self) -> np.ndarray:
        a = np.zeros((self.lx, LINESCAN_COLS))
        self.L.orc_last_linescan(self.h, _dptr(a))
        return a

    @property
    def done(self) -> bool:
        return bool(self.L.orc_protocol_done(self.h))

    @property
    def status(self) -> int:
        return int(self.L.orc_status(self.h))


def wholecell_text(rows) -> str:
    return "".join(format_wholecell(r) for r in rows)


def cadist_text(records) -> str:
    """The reference's cadist_ file for these records (:1005, :1009)."""
    out = []
    for r in records:
        out.append("0 header %f %f\n" % (r[0], r[1]))
        rows = np.asarray(r[2:]).reshape(-1, 6)
        out.extend("%f %f %f %f %f %f\n" % tuple(x) for x in rows)
    return "".join(out)


def linescan_text(blocks) -> str:
    out = []
    for b in blocks:
        out.extend(format_linescan(r) for r in b)
        out.append("\n")
    return "".join(out)


# ---- the reference compiled for the host (oracle/_ref), when built here ----

def ref_binary(variant: str) -> str | None:
    p = os.path.join(REF_DIR, f"ref_{variant}")
    return p if os.path.exists(p) else None


def run_ref(variant: str, args, workdir: str, max_steps: int | None = None,
            threads: int | None = None) -> tuple[str, str]:
    """Runs oracle/_ref/ref_<variant> with reference argv a3..a10 and returns
    the text of its wholetest_ and linescan_ files."""
    exe = ref_binary(variant)
    if exe is None:
        raise FileNotFoundError(f"oracle/_ref/ref_{variant} not built")
    env = dict(os.environ)
    if max_steps is not None:
        env["REF_MAX_STEPS"] = str(int(max_steps))
    if threads is not None:
        env["OMP_NUM_THREADS"] = str(int(threads))
    name = "ref"
    subprocess.run([exe, "0", name] + [str(a) for a in args], cwd=workdir, env=env, check=True,
                   stdout=subprocess.DEVNULL)
    with open(os.path.join(workdir, f"wholetest_{name}")) as f:
        wt = f.read()
    with open(os.path.join(workdir, f"linescan_{name}")) as f:
        ls = f.read()
    return wt, ls


def ref_cadist(workdir: str) -> str:
    """Text of the cadist_ file of the last run_ref in workdir."""
    with open(os.path.join(workdir, "cadist_ref")) as f:
        return f.read()
