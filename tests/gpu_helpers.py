"""Shared helpers of the GPU parity tests: building rich lattice states with
the oracle and comparing simulator state against it."""
from __future__ import annotations

import numpy as np

from oracle import oracle as O
from ryr_hyperactivity_gb300.abi import (DIAG_FIELDS, DIAG_SUB_FIELDS, STATE_F64_FIELDS,
                                         STATE_INT_FIELDS, STATE_SUB_FIELDS, HostState, cell_params)

COUNT_FIELDS = ["nou", "ncu", "nob", "ncb"]
FLOAT_FIELDS = STATE_F64_FIELDS + STATE_SUB_FIELDS
DIAG = DIAG_FIELDS + DIAG_SUB_FIELDS


def c1_params(**kw):
    """20x10x5 lattice (432 interior CRUs), PCL 400 ms, 2 beats."""
    d = dict(nx=20, ny=10, nz=5, nbeats=2, pcl_ms=400.0, seed=1, cell_id=0)
    d.update(kw)
    return cell_params(**d)


def rich_state(p, steps=4200, seed=0, hot_frac=0.15, to_float32=False):
    """Oracle state after `steps` full steps (through the first beat's upstroke
    and Ca release), with a fraction of CRUs pushed into high-cp / many-open
    configurations so that the Gaussian RyR branches and long Poisson loops
    run.  Returns (HostState, Membrane)."""
    o = O.Oracle(p)
    o.run(steps)
    st = o.get_state()
    m = o.get_membrane()
    rng = np.random.default_rng(seed)
    n = st.n
    k = int(n * hot_frac)
    idx = rng.choice(n, k, replace=False)
    st["cp"][idx] = rng.uniform(15.0, 400.0, k)
    half = idx[: k // 2]
    nou = rng.integers(3, 45, len(half))
    nob = rng.integers(0, 30, len(half))
    ncb = np.minimum(st["ncb"][half], 100 - nou - nob)
    st["nou"][half] = nou
    st["nob"][half] = nob
    st["ncb"][half] = ncb
    st["ncu"][half] = 100 - nou - nob - ncb
    if to_float32:
        for f in FLOAT_FIELDS:
            st[f][...] = st[f].astype(np.float32).astype(np.float64)
    return st, m


def rel_err(a, b, floor_frac=1e-9):
    """max |a-b| / max(|b|, floor), floor = floor_frac * max|b| (per field)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.size == 0:
        return 0.0
    scale = np.maximum(np.abs(b), floor_frac * max(np.max(np.abs(b)), 1e-300))
    return float(np.max(np.abs(a - b) / scale))


def count_mismatch(got: HostState, ref: HostState) -> np.ndarray:
    """Boolean mask of CRUs whose RyR counts, window counters or LCC states differ."""
    n = ref.n
    bad = np.zeros(n, bool)
    for f in COUNT_FIELDS + ["nl", "nspark"]:
        bad |= got[f] != ref[f]
    bad |= (got["lcc"] != ref["lcc"]).reshape(8, n).any(axis=0)
    return bad


def field_errors(got: HostState, ref: HostState, mask=None, fields=None):
    """Per-field relative error over CRUs in `mask` (all if None)."""
    n = ref.n
    out = {}
    for f in fields or (FLOAT_FIELDS + DIAG):
        g = got[f]
        r = ref[f]
        if g.size == 8 * n:
            g = g.reshape(8, n)
            r = r.reshape(8, n)
            if mask is not None:
                g, r = g[:, mask], r[:, mask]
        elif mask is not None:
            g, r = g[mask], r[mask]
        out[f] = rel_err(g, r)
    return out


def ap_waveform(pcl_ms: float, dt: float = 0.025) -> np.ndarray:
    """Synthetic action-potential clamp waveform, one sample per step of one
    PCL ((int)(pcl/dt + 0.1) samples, the length the reference reads from
    v_1000.txt, cuda_Cell_Detailed.cu:383-395): rest at -86 mV, a 2 ms
    upstroke to +40 mV at 10 ms, then a quadratic repolarisation over 140 ms.
    Values are rounded to 1e-6 mV so that their decimal text parses back to
    the same doubles."""
    n = int(pcl_ms / dt + 0.1)
    t = np.arange(n) * dt
    v = np.full(n, -86.0)
    up = (t >= 10) & (t < 12)
    v[up] = -86 + (t[up] - 10) / 2 * 126
    pl = t >= 12
    v[pl] = 40 - 126 * np.clip((t[pl] - 12) / 140, 0, 1) ** 2
    return np.round(v, 6)


def variant_params(spec: dict):
    """Cell parameters of a recorded reference run (tests/golden/ref_full_runs.json)."""
    from ryr_hyperactivity_gb300.abi import cell_params
    a = spec["args"]
    return cell_params(clamp_mv=a[0], cjsr_basal=a[1], ncx_scale=a[2], ku=a[3], r1=a[4], kb=a[5],
                       ica_scale=a[6], ku2=a[7], seed=spec["seed"], **spec["cell"])


def assert_text_files_match(got: str, want: str, rtol: float = 1e-5, atol: float = 2e-6):
    """Output files printed as the reference prints them (wholetest_,
    linescan_): the same lines, blank lines included, each with the same
    fields in the same places (the same single and double spaces), and the
    numbers equal within rtol/atol (atol covers the last printed digit of a
    %f field)."""
    a_lines, b_lines = got.splitlines(), want.splitlines()
    assert len(a_lines) == len(b_lines), (len(a_lines), len(b_lines))
    for k, (a, b) in enumerate(zip(a_lines, b_lines)):
        fa, fb = a.split(" "), b.split(" ")
        assert len(fa) == len(fb), (k, a, b)
        for x, y in zip(fa, fb):
            assert (x == "") == (y == ""), (k, a, b)
        va = np.array([float(x) for x in fa if x])
        vb = np.array([float(x) for x in fb if x])
        np.testing.assert_allclose(va, vb, rtol=rtol, atol=atol, err_msg=f"line {k}")


def flux_errors(got: HostState, ref: HostState, mask=None):
    """Per-flux (diagnostic) error relative to that flux's largest magnitude
    in the cell.  A flux is a difference of larger terms (the GHK LCC current
    lcc_k (cpx e2z - cao) crosses zero near its reversal, SERCA is uptake
    minus back-flux), so in FP32 its rounding error scales with those terms,
    not with the difference; what reaches the concentrations is that error
    against the flux's scale."""
    n = ref.n
    out = {}
    for f in DIAG:
        g, r = got[f], ref[f]
        if g.size == 8 * n:
            g, r = g.reshape(8, n), r.reshape(8, n)
            if mask is not None:
                g, r = g[:, mask], r[:, mask]
        elif mask is not None:
            g, r = g[mask], r[mask]
        scale = max(float(np.max(np.abs(r))) if r.size else 0.0, 1e-300)
        out[f] = float(np.max(np.abs(g - r))) / scale if r.size else 0.0
    return out



def step_errors(got: HostState, ref: HostState, before: HostState, mask=None, fields=None):
    """Per-field error of a one-step FP32 update against the FP64 oracle,
    relative to the larger of each value before and after the step.  An FP32
    update x + dx rounds at the scale of max(|x|, |dx|): where a concentration
    falls by orders of magnitude within one step (the dyadic space emptying
    once release stops), its error relative to the small new value says
    nothing about the arithmetic.  Returns {field: (scaled error, fraction of
    values whose plain relative error exceeds 1e-5)}."""
    n = ref.n
    out = {}
    for f in fields or FLOAT_FIELDS:
        g, r, b = got[f], ref[f], before[f]
        if g.size == 8 * n:
            g, r, b = g.reshape(8, n), r.reshape(8, n), b.reshape(8, n)
            if mask is not None:
                g, r, b = g[:, mask], r[:, mask], b[:, mask]
        elif mask is not None:
            g, r, b = g[mask], r[mask], b[mask]
        if r.size == 0:
            out[f] = (0.0, 0.0)
            continue
        floor = 1e-9 * max(float(np.max(np.abs(r))), 1e-300)
        d = np.abs(g - r)
        scaled = d / np.maximum(np.maximum(np.abs(r), np.abs(b)), floor)
        plain = d / np.maximum(np.abs(r), floor)
        out[f] = (float(scaled.max()), float((plain > 1e-5).mean()))
    return out
