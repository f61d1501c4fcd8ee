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


def oracle_case(case, nsteps=None, packed=None, **kw):
    """Run ``case`` (a seidart_gb300.synthetic.Case) on the FP64 oracle from
    rest for ``nsteps`` steps (all by default).  Returns (state, traces)."""
    from seidart_gb300 import cpml as cp
    n = case.nstep if nsteps is None else int(nsteps)
    prof = cp.pack_profiles(case.profiles) if packed is None else packed
    st, tr, _, blew = _run(case.grid.kind, case.grid, case.planes, prof, case.src_ijk, case.srcfn, case.rec_ijk, n,
                           **kw)
    if blew:
        raise RuntimeError(f"oracle blew up on {case.name}")
    return st, tr


def compare_run(gpu_traces, gpu_fields, ref_state, ref_traces, field_names):
    """Relative L2 of the traces and of each final field (GPU FP32 against the
    oracle FP64), and the largest of the field errors."""
    out = {"rel_l2_traces": rel_l2(gpu_traces, ref_traces)}
    errs = {}
    for q, name in enumerate(field_names):
        errs[name] = rel_l2(gpu_fields[q], ref_state.fields[q])
    out["rel_l2_fields"] = errs
    out["rel_l2_fields_max"] = max(errs.values()) if errs else None
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
