"""ctypes mirror of the C ABI types in include/rh.h.

These structures describe cells, run options and host-side state views for
``librh.so``.  Field meanings and reference citations are in include/rh.h.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

RH_OK = 0
RH_FP64 = 0
RH_MIXED = 1
RH_STATUS_NAN = 0x1
RH_STATUS_GAUSS_RETRY = 0x2
RH_STATUS_CI_HIGH = 0x4
RH_STATUS_DONE = 0x8
RH_STATUS_RATE_CAP = 0x10
RH_STATUS_TIMEOUT = 0x20
WHOLECELL_COLS = 45
LINESCAN_COLS = 22
CADIST_COLS = 6
RH_PROTO_PACED = 0
RH_PROTO_NOPACING = 1
RH_PROTO_VCLAMP = 2
RH_PROTO_BROWN_VCLAMP = 3
RH_PROTO_AP_CLAMP = 4
RH_PROTO_LINEAR_AP_CLAMP = 5
RH_NCX_ALLOSTERIC = 0
RH_NCX_OLD = 1
RH_NCX_NOALLO = 2
# protocol names as the reference's build switches spell them
PROTOCOLS = {"paced": RH_PROTO_PACED, "nopacing": RH_PROTO_NOPACING, "vclamp": RH_PROTO_VCLAMP,
             "brownvclamp": RH_PROTO_BROWN_VCLAMP, "apclamp": RH_PROTO_AP_CLAMP,
             "linearapclamp": RH_PROTO_LINEAR_AP_CLAMP}
NCX_FORMS = {"ncx": RH_NCX_ALLOSTERIC, "oldncx": RH_NCX_OLD, "ncx_noallo": RH_NCX_NOALLO}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class CellParams(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("nbeats", C.c_int32),
        ("pcl_ms", C.c_double),
        ("clamp_mv", C.c_double),
        ("cjsr_basal", C.c_double),
        ("ncx_scale", C.c_double),
        ("ku", C.c_double),
        ("r1", C.c_double),
        ("kb", C.c_double),
        ("ica_scale", C.c_double),
        ("ku2", C.c_double),
        ("ikr_scale", C.c_double),
        ("cao_mM", C.c_double),
        ("lqt", C.c_int32), ("iso2", C.c_int32), ("tapsi", C.c_int32),
        ("seed", C.c_uint32),
        ("cell_id", C.c_uint32),
        ("linescan_jz", C.c_int32),
        ("protocol", C.c_int32),
        ("perm", C.c_int32),
        ("iso", C.c_int32),
        ("randomlcc", C.c_int32),
        ("slowncx", C.c_int32),
        ("ncx_form", C.c_int32),
    ]


class LaunchShape(C.Structure):
    """rh_launch_shape: how a simulator's time steps are launched."""
    _fields_ = [
        ("persistent", C.c_int32),
        ("tile_crus", C.c_int32),
        ("fewer_ctas", C.c_int32),
        ("cell_groups", C.c_int32),
        ("bulk_staging", C.c_int32),
    ]

    def as_dict(self) -> dict:
        return {f: int(getattr(self, f)) for f, _ in self._fields_}


class RunOpts(C.Structure):
    _fields_ = [
        ("precision", C.c_int32),
        ("device", C.c_int32),
        ("dt_ms", C.c_double),
        ("block_size", C.c_int32),
        ("output_capacity", C.c_int32),
        ("record_linescan", C.c_int32),
        ("track_stats", C.c_int32),
        ("stats_capacity", C.c_int32),
        ("keep_diagnostics", C.c_int32),
        ("window_steps", C.c_int32),
        ("cell_groups", C.c_int32),
        ("record_cadist", C.c_int32),
        ("cadist_capacity", C.c_int32),
        ("persistent", C.c_int32),
    ]


STATE_F64_FIELDS = ["cp", "cs", "cjsr", "cjsrb", "ancx", "casar", "casarh", "casarj", "casarhj"]
STATE_SUB_FIELDS = ["ci", "cnsr", "catf", "cats", "cacal", "casr", "camyo", "mgmyo"]
STATE_INT_FIELDS = ["nou", "ncu", "nob", "ncb", "nl", "nspark"]
DIAG_FIELDS = ["xire", "po", "xinaca", "xicat"]
DIAG_SUB_FIELDS = ["xiup", "xileak"]


class StateF64(C.Structure):
    _fields_ = (
        [("n", C.c_int32)]
        + [(f, _dp) for f in STATE_F64_FIELDS]
        + [(f, _dp) for f in STATE_SUB_FIELDS]
        + [(f, _ip) for f in STATE_INT_FIELDS]
        + [("lcc", _ip)]
        + [(f, _dp) for f in DIAG_FIELDS]
        + [(f, _dp) for f in DIAG_SUB_FIELDS]
    )


class Membrane(C.Structure):
    _fields_ = [
        ("t", C.c_double), ("step", C.c_int64),
        ("v", C.c_double), ("xnai", C.c_double), ("xm", C.c_double), ("xh", C.c_double),
        ("xj", C.c_double), ("xr", C.c_double), ("xs1", C.c_double), ("xs2", C.c_double),
        ("qks", C.c_double), ("xtos", C.c_double), ("ytos", C.c_double), ("xtof", C.c_double),
        ("ytof", C.c_double),
        ("out_ica", C.c_double), ("out_ncx", C.c_double), ("out_ina", C.c_double),
        ("sparksum", C.c_int64),
        ("csubt", C.c_double), ("xicatto", C.c_double), ("xinacato", C.c_double),
        ("xina", C.c_double), ("xiks", C.c_double), ("xikr", C.c_double), ("xik1", C.c_double),
        ("xinak", C.c_double), ("xitos", C.c_double), ("xitof", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class BeatStats(C.Structure):
    _fields_ = [
        ("beat", C.c_int32), ("ead", C.c_int32),
        ("apd90_ms", C.c_double), ("v_peak", C.c_double), ("ci_peak", C.c_double),
        ("sr_load", C.c_double), ("sparks", C.c_int32), ("pad", C.c_int32),
    ]


def cell_params(**kw) -> CellParams:
    """Reference defaults (the run.sh "hyper" line on the shipped 64x28x12
    lattice, make-il build) overridden by keyword arguments."""
    d = dict(nx=64, ny=28, nz=12, nbeats=7, pcl_ms=4000.0, clamp_mv=1.0, cjsr_basal=740.0,
             ncx_scale=1.0, ku=3.333, r1=0.0, kb=18.0, ica_scale=0.7, ku2=1.0, ikr_scale=1.0,
             cao_mM=1.8, lqt=1, iso2=1, tapsi=0, seed=18, cell_id=0, linescan_jz=-1,
             protocol=RH_PROTO_PACED, perm=0, iso=0, randomlcc=0, slowncx=0,
             ncx_form=RH_NCX_ALLOSTERIC)
    d.update(kw)
    if isinstance(d["protocol"], str):  # a build-switch name, e.g. "vclamp"
        d["protocol"] = PROTOCOLS[d["protocol"]]
    if isinstance(d["ncx_form"], str):  # the reference's function name
        d["ncx_form"] = NCX_FORMS[d["ncx_form"]]
    p = CellParams()
    for k, v in d.items():
        setattr(p, k, v)
    return p


class HostState:
    """numpy-backed host arrays bound to an ``StateF64`` view (interior CRUs
    only, x fastest; sub-voxel fields are 8 planes of n)."""

    def __init__(self, n: int):
        self.n = n
        self.arrays: dict[str, np.ndarray] = {}
        for f in STATE_F64_FIELDS + DIAG_FIELDS:
            self.arrays[f] = np.zeros(n, np.float64)
        for f in STATE_SUB_FIELDS + DIAG_SUB_FIELDS:
            self.arrays[f] = np.zeros(8 * n, np.float64)
        for f in STATE_INT_FIELDS:
            self.arrays[f] = np.zeros(n, np.int32)
        self.arrays["lcc"] = np.zeros(8 * n, np.int32)
        self.view = StateF64()
        self.view.n = n
        for f, a in self.arrays.items():
            ptype = _ip if a.dtype == np.int32 else _dp
            setattr(self.view, f, a.ctypes.data_as(ptype))

    def __getitem__(self, k: str) -> np.ndarray:
        return self.arrays[k]

    def copy_from(self, other: "HostState") -> None:
        for k, a in other.arrays.items():
            self.arrays[k][...] = a

    def snapshot(self) -> dict[str, np.ndarray]:
        return {k: a.copy() for k, a in self.arrays.items()}
