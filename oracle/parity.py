"""Comparison helpers of the GPU path against the FP64 oracle -- TEST
INFRASTRUCTURE ONLY (used by tests/ and by bench.py's parity leg, never by the
seidart_gb300 package).

Every function here runs the oracle as the checker: the GPU results it is
given are produced by the caller through the C ABI.
"""
from __future__ import annotations

import numpy as np

from . import run as _run


def rel_l2(a, b) -> float:
    """||a - b|| / ||b|| in FP64 (||a|| when b is zero)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = float(np.linalg.norm(b))
    if den == 0.0:
        return float(np.linalg.norm(a))
    return float(np.linalg.norm(a - b) / den)


def case_options(case) -> dict:
    """The physics options of ``case`` as oracle.run keywords."""
    return {"legacy": bool(getattr(case, "legacy", False)), "density": getattr(case, "density", "arithmetic"),
            "stress_src": getattr(case, "stress_srcfn", None)}


def oracle_case(case, nsteps=None, packed=None, **kw):
    """Run ``case`` (a seidart_gb300.synthetic.Case) on the FP64 oracle from
    rest for ``nsteps`` steps (all by default), with the case's physics
    options.  Returns (state, traces)."""
    from seidart_gb300 import cpml as cp
    n = case.nstep if nsteps is None else int(nsteps)
    prof = cp.pack_profiles(case.profiles) if packed is None else packed
    opts = case_options(case)
    opts.update(kw)
    st, tr, _, blew = _run(case.grid.kind, case.grid, case.planes, prof, case.src_ijk, case.srcfn, case.rec_ijk, n,
                           **opts)
    if blew:
        raise RuntimeError(f"oracle blew up on {case.name}")
    return st, tr


def oracle_case_peaks(case, nsteps=None, chunk=200):
    """As oracle_case, run in chunks of ``chunk`` steps, also returning the
    largest L2 norm each field reached at a chunk boundary (the peak the
    final-field error is set against once the wave has left the grid)."""
    from seidart_gb300 import cpml as cp
    n = case.nstep if nsteps is None else int(nsteps)
    prof = cp.pack_profiles(case.profiles)
    st, parts, peaks, done = None, [], None, 0
    while done < n:
        m = min(chunk, n - done)
        st, tr, _, blew = _run(case.grid.kind, case.grid, case.planes, prof, case.src_ijk, case.srcfn, case.rec_ijk,
                               m, state=st, **case_options(case))
        if blew:
            raise RuntimeError(f"oracle blew up on {case.name}")
        parts.append(tr)
        norms = np.array([np.linalg.norm(f) for f in st.fields])
        peaks = norms if peaks is None else np.maximum(peaks, norms)
        done += m
    return st, np.concatenate(parts, axis=0), peaks


def compare_run(gpu_traces, gpu_fields, ref_state, ref_traces, field_names, peaks=None):
    """Relative L2 of the traces and of each final field (GPU FP32 against the
    oracle FP64), the largest of the field errors, and, given each field's
    peak norm over the run, the final-field errors relative to that peak."""
    out = {"rel_l2_traces": rel_l2(gpu_traces, ref_traces)}
    errs, vs_peak = {}, {}
    for q, name in enumerate(field_names):
        errs[name] = rel_l2(gpu_fields[q], ref_state.fields[q])
        if peaks is not None and peaks[q] > 0:
            d = np.asarray(gpu_fields[q], dtype=np.float64) - ref_state.fields[q]
            vs_peak[name] = float(np.linalg.norm(d) / peaks[q])
    out["rel_l2_fields"] = errs
    out["rel_l2_fields_max"] = max(errs.values()) if errs else None
    if vs_peak:
        out["fields_err_vs_peak_norm"] = vs_peak
        out["fields_err_vs_peak_norm_max"] = max(vs_peak.values())
    return out


def misfit(traces, d_obs) -> float:
    r = np.asarray(traces, dtype=np.float64) - np.asarray(d_obs, dtype=np.float64)
    return 0.5 * float(np.sum(r * r))


def fd_cells(shape, npml, n=20, seed=7):
    """``n`` seeded interior cells (k, i) of an (NZ, NX) grid, outside the CPML."""
    rng = np.random.default_rng(seed)
    NZ, NX = shape
    ks = rng.integers(npml, NZ - npml, n)
    iss = rng.integers(npml, NX - npml, n)
    return [(int(k), int(i)) for k, i in zip(ks, iss)]
