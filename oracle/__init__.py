"""FP64 CPU oracle of the FDTD path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
use this package, and only as the reference results or the timed CPU baseline.  The
product (seidart_gb300) never imports it.

``liboracle.so`` (built from fdtd_oracle.cpp by the Makefile here) restates the
reference's legacy Fortran loops in double precision; see the header of
fdtd_oracle.cpp for the file:line of every loop.  Parity status: unpinned
(the reference has no tests or golden vectors for this path, and its Fortran
cannot be compiled on these machines).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
LIB_NATIVE = HERE / "liboracle_native.so"
# compiler flags of liboracle_native.so (the timed CPU baseline's build)
NATIVE_FLAGS = "g++ -O3 -fopenmp " + ("-mcpu=native" if os.uname().machine == "aarch64" else "-march=native")
SEISMIC2, SEISMIC25, ELECTROMAG2, ELECTROMAG25, ELECTROMAG2C = 1, 2, 3, 4, 5
NFIELDS = {SEISMIC2: 5, SEISMIC25: 9, ELECTROMAG2: 3, ELECTROMAG25: 6, ELECTROMAG2C: 6}
NMEM = {SEISMIC2: 12, SEISMIC25: 18, ELECTROMAG2: 4, ELECTROMAG25: 12, ELECTROMAG2C: 8}
# density_method values of the driver (src/seidart/routines/classes.py:311) -> oracle option bits
DENSITY = {"arithmetic": 0, "none": 1, "geometric": 2, "harmonic": 3}
NSTRESS = {SEISMIC2: 3, SEISMIC25: 6}  # stress source components (xx zz xz | xx yy zz xy xz yz)
NCH = {SEISMIC2: 2, SEISMIC25: 3, ELECTROMAG2: 2, ELECTROMAG25: 3, ELECTROMAG2C: 4}

_lock = threading.Lock()
_libs = {}


def build(force: bool = False, native: bool = False) -> Path:
    """Compile liboracle.so (or the host-tuned liboracle_native.so) with the
    Makefile in this directory."""
    src = HERE / "fdtd_oracle.cpp"
    out = LIB_NATIVE if native else LIB
    if force or not out.exists() or out.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE), out.name] + (["-B"] if force else []), check=True)
    return out


def lib(native: bool = False):
    with _lock:
        if native not in _libs:
            L = C.CDLL(str(build(native=native)))
            dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
            i, d = C.c_int, C.c_double
            common_tail = [dp, dp, i, i, dp, i, i, i, dp, dp, i, ip, dp, dp, ip]
            L.orc_electromag2.argtypes = [i, i, d, d, d] + common_tail + [dp]
            L.orc_electromag2c.argtypes = [i, i, d, d, d] + common_tail
            L.orc_seismic2.argtypes = [i, i, d, d, d] + common_tail + [i, dp, dp]
            tail3 = [dp, dp, i, i, i, dp, i, i, i, dp, dp, i, ip, dp, dp, ip]
            L.orc_seismic25.argtypes = [i, i, i, d, d, d, d] + tail3 + [i, dp]
            L.orc_electromag25.argtypes = [i, i, i, d, d, d, d] + tail3
            for f in (L.orc_electromag2, L.orc_electromag2c, L.orc_seismic2, L.orc_seismic25, L.orc_electromag25):
                f.restype = C.c_int
            L.orc_num_threads.restype = C.c_int
            _libs[native] = L
        return _libs[native]


@dataclass
class OracleState:
    kind: int
    shape: tuple          # (NZ, NX) or (NZ, NY, NX)
    fields: np.ndarray    # (nfields, *shape)
    memory: np.ndarray    # (nmem, *shape)
    step: int = 0

    @classmethod
    def zeros(cls, kind, shape):
        return cls(kind, tuple(shape), np.zeros((NFIELDS[kind],) + tuple(shape)),
                   np.zeros((NMEM[kind],) + tuple(shape)))


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def run(kind, grid, planes, packed_profiles, src_ijk, srcfn, rec_ijk, nsteps, state: OracleState = None,
        native: bool = False, legacy: bool = False, density: str = "arithmetic", stress_src=None, cpml2d=None):
    """Advance ``nsteps`` steps of the FP64 oracle.  Returns (state, traces,
    maxnorm, blew_up); traces is (nsteps, nch, nrec).  ``native`` runs the
    host-tuned build (timing only).  Seismic kinds: ``legacy`` keeps the
    legacy Fortran's quirks (default: corrected physics), ``density`` is the
    density method ('arithmetic', 'none', 'geometric', 'harmonic') and
    ``stress_src`` the stress source time functions (NSTRESS[kind] x nstep,
    same cell as the force source) or None.  ``cpml2d``: electromag2 and
    seismic2 only, the driver's 2-D CPML fields (6, NZ, NX): K, a, b,
    K_half, a_half, b_half, used for every derivative direction in place of
    the per-axis profiles (which are then ignored)."""
    L = lib(native)
    opts = (1 if legacy else 0) | (DENSITY[density] << 1)
    f2 = None
    if cpml2d is not None:
        if kind not in (ELECTROMAG2, SEISMIC2):
            raise ValueError("2-D CPML fields apply to electromag2 and seismic2")
        if legacy:
            raise ValueError("the legacy loops read 1-D CPML profiles")
        f2 = np.ascontiguousarray(cpml2d, dtype=np.float64)
        if f2.shape != (6, grid.nz, grid.nx):
            raise ValueError("cpml2d must be (6, NZ, NX)")
    ssrc = None
    if stress_src is not None:
        ssrc = np.ascontiguousarray(stress_src, dtype=np.float64)
        if kind not in NSTRESS or ssrc.shape != (NSTRESS[kind], np.asarray(srcfn).shape[1]):
            raise ValueError("stress_src must be (3 | 6, nstep) for seismic2 | seismic25")
    three = kind in (SEISMIC25, ELECTROMAG25)
    shape = (grid.nz, grid.ny, grid.nx) if three else (grid.nz, grid.nx)
    if state is None:
        state = OracleState.zeros(kind, shape)
    planes = np.ascontiguousarray(planes, dtype=np.float64)
    prof = np.ascontiguousarray(packed_profiles, dtype=np.float64)
    srcfn = np.ascontiguousarray(srcfn, dtype=np.float64)
    rec = np.ascontiguousarray(np.asarray(rec_ijk, dtype=np.int32).reshape(-1, 3))
    nrec = rec.shape[0]
    traces = np.zeros((nsteps, NCH[kind], max(nrec, 1)))
    maxnorm = C.c_double(0.0)
    blew = C.c_int(0)
    i, j, k = (int(v) for v in src_ijk)
    recp = rec.ctypes.data_as(C.POINTER(C.c_int)) if nrec else None
    if kind == ELECTROMAG2:
        n = L.orc_electromag2(grid.nx, grid.nz, grid.dx, grid.dz, grid.dt, _d(prof), _d(planes), i, k, _d(srcfn),
                              srcfn.shape[1], state.step, nsteps, _d(state.fields), _d(state.memory), nrec, recp,
                              _d(traces), C.byref(maxnorm), C.byref(blew), _d(f2) if f2 is not None else None)
    elif kind == ELECTROMAG2C:
        n = L.orc_electromag2c(grid.nx, grid.nz, grid.dx, grid.dz, grid.dt, _d(prof), _d(planes), i, k, _d(srcfn),
                               srcfn.shape[1], state.step, nsteps, _d(state.fields), _d(state.memory), nrec, recp,
                               _d(traces), C.byref(maxnorm), C.byref(blew))
    elif kind == SEISMIC2:
        n = L.orc_seismic2(grid.nx, grid.nz, grid.dx, grid.dz, grid.dt, _d(prof), _d(planes), i, k, _d(srcfn),
                           srcfn.shape[1], state.step, nsteps, _d(state.fields), _d(state.memory), nrec, recp,
                           _d(traces), C.byref(maxnorm), C.byref(blew), opts,
                           _d(ssrc) if ssrc is not None else None, _d(f2) if f2 is not None else None)
    elif kind == SEISMIC25:
        n = L.orc_seismic25(grid.nx, grid.ny, grid.nz, grid.dx, grid.dy, grid.dz, grid.dt, _d(prof), _d(planes),
                            i, j, k, _d(srcfn), srcfn.shape[1], state.step, nsteps, _d(state.fields),
                            _d(state.memory), nrec, recp, _d(traces), C.byref(maxnorm), C.byref(blew), opts,
                            _d(ssrc) if ssrc is not None else None)
    elif kind == ELECTROMAG25:
        n = L.orc_electromag25(grid.nx, grid.ny, grid.nz, grid.dx, grid.dy, grid.dz, grid.dt, _d(prof), _d(planes),
                               i, j, k, _d(srcfn), srcfn.shape[1], state.step, nsteps, _d(state.fields),
                               _d(state.memory), nrec, recp, _d(traces), C.byref(maxnorm), C.byref(blew))
    else:
        raise ValueError(kind)
    state.step += n
    return state, traces[:n, :, :nrec], float(maxnorm.value), bool(blew.value)


def num_threads() -> int:
    return int(lib().orc_num_threads())


def set_threads(n: int) -> None:
    os.environ["OMP_NUM_THREADS"] = str(n)
