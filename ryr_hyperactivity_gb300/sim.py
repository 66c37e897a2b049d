"""Python mirror of the C ABI (include/rh.h): a batch of independent cells
advanced on one GPU.  Every call goes through librh.so; failures raise
NativeError with the library's error text."""
from __future__ import annotations

import ctypes as C
from typing import Iterable

import numpy as np

from . import native
from .abi import (LINESCAN_COLS, RH_FP64, RH_MIXED, WHOLECELL_COLS, BeatStats, CellParams,
                  HostState, LaunchShape, Membrane, RunOpts)

PRECISIONS = {"fp64": RH_FP64, "mixed": RH_MIXED}


def run_opts(precision: str = "fp64", **kw) -> RunOpts:
    L = native.load()
    o = RunOpts()
    L.rh_default_run_opts(C.byref(o))
    o.precision = PRECISIONS[precision]
    names = {f[0] for f in RunOpts._fields_}
    for k, v in kw.items():
        if k not in names:
            raise TypeError(f"unknown run option {k!r}")
        setattr(o, k, v)
    return o


class Simulator:
    def __init__(self, cells: CellParams | Iterable[CellParams], precision: str = "fp64",
                 **opts):
        self.L = native.load()
        if isinstance(cells, CellParams):
            cells = [cells]
        cells = list(cells)
        self.params = cells
        self.ncells = len(cells)
        arr = (CellParams * self.ncells)(*cells)
        self.opts = run_opts(precision, **opts)
        h = C.c_void_p()
        rc = self.L.rh_create(arr, self.ncells, C.byref(self.opts), C.byref(h))
        if rc != 0:
            raise native.NativeError(f"rh_create failed ({rc}): {self._err(None)}")
        self.h = h
        self.n = []
        for c in range(self.ncells):
            n = C.c_int32()
            self._ck(self.L.rh_cell_size(self.h, c, C.byref(n)))
            self.n.append(n.value)

    # -- helpers
    def _err(self, h) -> str:
        buf = C.create_string_buffer(1024)
        self.L.rh_last_error(h, buf, 1024)
        return buf.value.decode(errors="replace")

    def _ck(self, rc: int) -> None:
        if rc != 0:
            raise native.NativeError(f"librh error {rc}: {self._err(self.h)}")

    def close(self) -> None:
        if getattr(self, "h", None):
            self.L.rh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- stepping
    def run_steps(self, n: int) -> None:
        self._ck(self.L.rh_run_steps(self.h, int(n)))

    def run_to_end(self) -> None:
        self._ck(self.L.rh_run_to_end(self.h))

    def lattice_step(self) -> None:
        self._ck(self.L.rh_lattice_step(self.h))

    def set_ap_clamp(self, cell: int, v_mV) -> None:
        """Waveform of an AP-clamp cell (protocol "apclamp"): one voltage per
        step of one PCL, (int)(pcl/dt + 0.1) samples."""
        a = np.ascontiguousarray(v_mV, np.float64)
        self._ck(self.L.rh_set_ap_clamp(self.h, cell, a.ctypes.data_as(C.POINTER(C.c_double)),
                                        len(a)))

    # -- state
    def get_state(self, cell: int = 0) -> HostState:
        hs = HostState(self.n[cell])
        self._ck(self.L.rh_get_state(self.h, cell, C.byref(hs.view)))
        return hs

    def set_state(self, cell: int, hs: HostState) -> None:
        self._ck(self.L.rh_set_state(self.h, cell, C.byref(hs.view)))

    def get_membrane(self, cell: int = 0) -> Membrane:
        m = Membrane()
        self._ck(self.L.rh_get_membrane(self.h, cell, C.byref(m)))
        return m

    def set_membrane(self, cell: int, m: Membrane) -> None:
        self._ck(self.L.rh_set_membrane(self.h, cell, C.byref(m)))

    # -- outputs
    def drain_wholecell(self, cell: int = 0, max_rec: int = 4096) -> np.ndarray:
        a = np.zeros((max_rec, WHOLECELL_COLS))
        n = C.c_int32()
        self._ck(self.L.rh_drain_wholecell(self.h, cell, a.ctypes.data_as(C.POINTER(C.c_double)),
                                           max_rec, C.byref(n)))
        return a[: n.value].copy()

    def drain_wholecell_all(self, max_rec: int = 64) -> list[np.ndarray]:
        """drain_wholecell of every cell in one library call."""
        a = np.empty((self.ncells, max_rec, WHOLECELL_COLS))
        n = np.zeros(self.ncells, dtype=np.int32)
        self._ck(self.L.rh_drain_wholecell_all(self.h, a.ctypes.data_as(C.POINTER(C.c_double)),
                                               max_rec, n.ctypes.data_as(C.POINTER(C.c_int32))))
        return [a[c, : n[c]].copy() for c in range(self.ncells)]

    def drain_linescan(self, cell: int = 0, max_rec: int = 4096) -> np.ndarray:
        lx = self.params[cell].nx - 2
        a = np.zeros((max_rec, lx, LINESCAN_COLS))
        n = C.c_int32()
        self._ck(self.L.rh_drain_linescan(self.h, cell, a.ctypes.data_as(C.POINTER(C.c_double)),
                                          max_rec, C.byref(n)))
        return a[: n.value].copy()

    def drain_cadist(self, cell: int = 0, max_rec: int = 64) -> np.ndarray:
        """cadist records (run option record_cadist=1), one row each: t, V,
        then 6 values per interior CRU in the reference's order."""
        a = np.zeros((max_rec, 2 + 6 * self.n[cell]))
        n = C.c_int32()
        self._ck(self.L.rh_drain_cadist(self.h, cell, a.ctypes.data_as(C.POINTER(C.c_double)),
                                        max_rec, C.byref(n)))
        return a[: n.value].copy()

    def drain_stats(self, cell: int = 0, max_rec: int = 256) -> list[dict]:
        arr = (BeatStats * max_rec)()
        n = C.c_int32()
        self._ck(self.L.rh_drain_stats(self.h, cell, arr, max_rec, C.byref(n)))
        return [{k: getattr(arr[i], k) for k, _ in BeatStats._fields_ if k != "pad"}
                for i in range(n.value)]

    def status(self, cell: int = 0) -> int:
        s = C.c_uint32()
        self._ck(self.L.rh_cell_status(self.h, cell, C.byref(s)))
        return s.value

    def checkpoint(self, path: str) -> None:
        self._ck(self.L.rh_checkpoint(self.h, path.encode()))

    def restore(self, path: str) -> None:
        self._ck(self.L.rh_restore(self.h, path.encode()))

    def state_bytes(self) -> int:
        b = C.c_size_t()
        self._ck(self.L.rh_state_bytes(self.h, C.byref(b)))
        return b.value

    def export_state(self, ptr: int, nbytes: int) -> None:
        """Copies the whole batch's state into host memory at address ptr."""
        self._ck(self.L.rh_export_state(self.h, C.c_void_p(ptr), nbytes))

    def import_state(self, ptr: int, nbytes: int) -> None:
        self._ck(self.L.rh_import_state(self.h, C.c_void_p(ptr), nbytes))

    def run_steps_host(self, n: int, in_ptr: int | None, out_ptr: int | None, nbytes: int) -> None:
        """import_state(in_ptr) + run_steps(n) + export_state(out_ptr) in one
        call (rh_run_steps_host); with pinned buffers the copies of each cell
        group overlap the other groups' steps.  Either address may be None."""
        self._ck(self.L.rh_run_steps_host(self.h, int(n), C.c_void_p(in_ptr or 0),
                                          C.c_void_p(out_ptr or 0), nbytes))

    def autotune(self, steps: int = 50) -> tuple[int, list[float]]:
        """Picks the fastest tile length for this workload; returns it and the
        measured ms per step of each candidate (64, 128, 256 CRUs)."""
        tile = C.c_int32()
        ms = (C.c_double * 3)()
        self._ck(self.L.rh_autotune(self.h, int(steps), C.byref(tile), ms))
        return tile.value, list(ms)

    def tile_size(self) -> int:
        t = C.c_int32()
        self._ck(self.L.rh_tile_size(self.h, C.byref(t)))
        return t.value

    def bytes_per_cru_step(self) -> float:
        b = C.c_double()
        self._ck(self.L.rh_bytes_per_cru_step(self.h, C.byref(b)))
        return b.value

    def num_groups(self) -> int:
        """Cell groups advanced on concurrent streams (per group and time
        step, a lattice launch and a cell-update launch)."""
        n = C.c_int32()
        self._ck(self.L.rh_num_groups(self.h, C.byref(n)))
        return n.value

    def kernel_launches(self) -> tuple[int, bool]:
        """Kernel launches issued for time steps since creation, and whether
        windows run as persistent launches."""
        n, p = C.c_int64(), C.c_int32()
        self._ck(self.L.rh_kernel_launches(self.h, C.byref(n), C.byref(p)))
        return n.value, bool(p.value)

    def window_ctas(self) -> int:
        """CTAs of the persistent window launch (0 when windows are not persistent)."""
        n = C.c_int32()
        self._ck(self.L.rh_window_ctas(self.h, C.byref(n)))
        return n.value

    def set_wait_limit(self, polls: int = 0, target_offset: int = 0) -> None:
        """Testing hook of the persistent launch's bounded waits (rh.h)."""
        self._ck(self.L.rh_set_wait_limit(self.h, int(polls), int(target_offset)))

    def launch_shape(self) -> dict:
        sh = LaunchShape()
        self._ck(self.L.rh_get_launch_shape(self.h, C.byref(sh)))
        return sh.as_dict()

    def set_launch_shape(self, persistent: int, tile_crus: int, fewer_ctas: int = 0,
                         cell_groups: int = 0, bulk_staging: int = 0) -> None:
        sh = LaunchShape(persistent, tile_crus, fewer_ctas, cell_groups, bulk_staging)
        self._ck(self.L.rh_set_launch_shape(self.h, C.byref(sh)))

    def autotune_shapes(self, steps: int = 40) -> tuple[dict, list[tuple[dict, float]]]:
        """Launch-shape autotuner (rh_autotune_shapes): the chosen shape and
        every candidate timed with its ms per lattice update (empty when the
        process-wide cache held this workload's choice)."""
        best = LaunchShape()
        tried = (LaunchShape * 64)()
        ms = (C.c_double * 64)()
        n = C.c_int32()
        self._ck(self.L.rh_autotune_shapes(self.h, int(steps), C.byref(best), tried, ms, 64,
                                           C.byref(n)))
        return best.as_dict(), [(tried[i].as_dict(), float(ms[i])) for i in range(n.value)]

    def kernel_timing(self) -> tuple[int, float]:
        n = C.c_int64()
        ms = C.c_double()
        self._ck(self.L.rh_kernel_timing(self.h, C.byref(n), C.byref(ms)))
        return n.value, ms.value


def analyze_trace(pcl_ms: float, t, v, wholecell, max_beats: int = 4096) -> list[dict]:
    """Per-beat statistics of a (t, V) trace and its output records, computed
    by the same detectors the simulator runs on the GPU."""
    L = native.load()
    t = np.ascontiguousarray(t, np.float64)
    v = np.ascontiguousarray(v, np.float64)
    wc = np.ascontiguousarray(wholecell, np.float64).reshape(-1, WHOLECELL_COLS)
    arr = (BeatStats * max_beats)()
    n = C.c_int32()
    dp = C.POINTER(C.c_double)
    rc = L.rh_analyze_trace(float(pcl_ms), t.ctypes.data_as(dp), v.ctypes.data_as(dp), len(t),
                            wc.ctypes.data_as(dp), len(wc), arr, max_beats, C.byref(n))
    if rc != 0:
        raise native.NativeError(f"rh_analyze_trace failed ({rc})")
    return [{k: getattr(arr[i], k) for k, _ in BeatStats._fields_ if k != "pad"}
            for i in range(n.value)]


def format_wholecell(row) -> str:
    L = native.load()
    a = np.ascontiguousarray(row, np.float64)
    buf = C.create_string_buffer(4096)
    L.rh_format_wholecell(a.ctypes.data_as(C.POINTER(C.c_double)), buf, 4096)
    return buf.value.decode()


def format_linescan(row) -> str:
    L = native.load()
    a = np.ascontiguousarray(row, np.float64)
    buf = C.create_string_buffer(1024)
    L.rh_format_linescan(a.ctypes.data_as(C.POINTER(C.c_double)), buf, 1024)
    return buf.value.decode()
