"""Loader and prototypes of librh.so, the CUDA simulator behind include/rh.h.

There is no fallback: if the library is missing or cannot be loaded, every
simulator call raises.  Build it with ``python -m ryr_hyperactivity_gb300.build``.
"""
from __future__ import annotations

import ctypes as C
import os

from .abi import BeatStats, CellParams, LaunchShape, Membrane, RunOpts, StateF64

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "librh.so")

# every symbol include/rh.h declares
EXPORTS = [
    "rh_default_cell_params", "rh_default_run_opts", "rh_create", "rh_destroy", "rh_run_steps",
    "rh_run_to_end", "rh_lattice_step", "rh_set_ap_clamp", "rh_num_cells", "rh_cell_size", "rh_get_state",
    "rh_set_state", "rh_get_membrane", "rh_set_membrane", "rh_drain_wholecell", "rh_drain_wholecell_all",
    "rh_drain_linescan", "rh_drain_cadist", "rh_drain_stats", "rh_cell_status", "rh_checkpoint", "rh_restore",
    "rh_bytes_per_cru_step", "rh_kernel_timing", "rh_num_groups", "rh_last_error", "rh_format_wholecell",
    "rh_format_linescan", "rh_state_bytes", "rh_export_state", "rh_import_state",
    "rh_analyze_trace", "rh_autotune", "rh_tile_size", "rh_kernel_launches", "rh_set_wait_limit",
    "rh_window_ctas", "rh_get_launch_shape", "rh_set_launch_shape", "rh_autotune_shapes",
    "rh_run_steps_host",
]

_lib = None


class NativeError(RuntimeError):
    pass


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise NativeError(f"{LIB_PATH} is not built; run python -m ryr_hyperactivity_gb300.build")
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    dp = C.POINTER(C.c_double)
    L.rh_default_cell_params.argtypes = [C.POINTER(CellParams)]
    L.rh_default_cell_params.restype = None
    L.rh_default_run_opts.argtypes = [C.POINTER(RunOpts)]
    L.rh_default_run_opts.restype = None
    L.rh_create.argtypes = [C.POINTER(CellParams), C.c_int32, C.POINTER(RunOpts), C.POINTER(vp)]
    L.rh_destroy.argtypes = [vp]
    L.rh_run_steps.argtypes = [vp, C.c_int64]
    L.rh_run_steps_host.argtypes = [vp, C.c_int64, vp, vp, C.c_size_t]
    L.rh_run_to_end.argtypes = [vp]
    L.rh_lattice_step.argtypes = [vp]
    L.rh_num_cells.argtypes = [vp, C.POINTER(C.c_int32)]
    L.rh_cell_size.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32)]
    L.rh_get_state.argtypes = [vp, C.c_int32, C.POINTER(StateF64)]
    L.rh_set_state.argtypes = [vp, C.c_int32, C.POINTER(StateF64)]
    L.rh_get_membrane.argtypes = [vp, C.c_int32, C.POINTER(Membrane)]
    L.rh_set_membrane.argtypes = [vp, C.c_int32, C.POINTER(Membrane)]
    L.rh_drain_wholecell.argtypes = [vp, C.c_int32, dp, C.c_int32, C.POINTER(C.c_int32)]
    L.rh_drain_wholecell_all.argtypes = [vp, dp, C.c_int32, C.POINTER(C.c_int32)]
    L.rh_drain_linescan.argtypes = [vp, C.c_int32, dp, C.c_int32, C.POINTER(C.c_int32)]
    L.rh_set_ap_clamp.argtypes = [vp, C.c_int32, dp, C.c_int64]
    L.rh_drain_cadist.argtypes = [vp, C.c_int32, dp, C.c_int32, C.POINTER(C.c_int32)]
    L.rh_drain_stats.argtypes = [vp, C.c_int32, C.POINTER(BeatStats), C.c_int32,
                                 C.POINTER(C.c_int32)]
    L.rh_cell_status.argtypes = [vp, C.c_int32, C.POINTER(C.c_uint32)]
    L.rh_analyze_trace.argtypes = [C.c_double, dp, dp, C.c_int64, dp, C.c_int32,
                                   C.POINTER(BeatStats), C.c_int32, C.POINTER(C.c_int32)]
    L.rh_checkpoint.argtypes = [vp, C.c_char_p]
    L.rh_restore.argtypes = [vp, C.c_char_p]
    L.rh_bytes_per_cru_step.argtypes = [vp, dp]
    L.rh_state_bytes.argtypes = [vp, C.POINTER(C.c_size_t)]
    L.rh_export_state.argtypes = [vp, vp, C.c_size_t]
    L.rh_import_state.argtypes = [vp, vp, C.c_size_t]
    L.rh_kernel_timing.argtypes = [vp, C.POINTER(C.c_int64), dp]
    L.rh_num_groups.argtypes = [vp, C.POINTER(C.c_int32)]
    L.rh_autotune.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32), dp]
    L.rh_tile_size.argtypes = [vp, C.POINTER(C.c_int32)]
    L.rh_kernel_launches.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int32)]
    L.rh_set_wait_limit.argtypes = [vp, C.c_int64, C.c_uint32]
    L.rh_window_ctas.argtypes = [vp, C.POINTER(C.c_int32)]
    L.rh_get_launch_shape.argtypes = [vp, C.POINTER(LaunchShape)]
    L.rh_set_launch_shape.argtypes = [vp, C.POINTER(LaunchShape)]
    L.rh_autotune_shapes.argtypes = [vp, C.c_int32, C.POINTER(LaunchShape), C.POINTER(LaunchShape),
                                     dp, C.c_int32, C.POINTER(C.c_int32)]
    L.rh_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
    L.rh_format_wholecell.argtypes = [dp, C.c_char_p, C.c_size_t]
    L.rh_format_linescan.argtypes = [dp, C.c_char_p, C.c_size_t]
    for name in EXPORTS:
        fn = getattr(L, name)
        if fn.restype is C.c_int or fn.restype is None and name not in (
                "rh_default_cell_params", "rh_default_run_opts"):
            fn.restype = C.c_int
    _lib = L
    return L
