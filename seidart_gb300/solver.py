"""Python host side of the FDTD backend: one :class:`FDTDSolver` per model/shot.

This mirrors the in-process solver calls of the reference (the f2py
subroutines ``seismic2``, ``seismic25``, ``electromag2``, ``electromag25`` of
``legacy/fortran/seismicfdtd.f95`` and ``legacy/fortran/electromagfdtd.f95``,
called from ``legacy/prjrun_101424.py:691-808``), with the inputs they read
from ``.dat`` files passed as arrays.  The device state is one torch uint8
tensor per solver; the kernels are the CUDA library's (no CPU path exists).

Array conventions: materials are float64 arrays ``(planes, NZ, NX)`` (x
fastest, the Fortran order of the reference's ``.dat`` records); fields are
``(NZ, NX)`` in 2-D and ``(NZ, NY, NX)`` in 2.5-D; traces are
``(nstep, channel, receiver)``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import ELECTROMAG2, ELECTROMAG25, ELECTROMAG2C, SEISMIC2, SEISMIC25, SfdConfig, check

MODEL_PLANES = {
    SEISMIC2: ["c11", "c13", "c15", "c33", "c35", "c55", "rho", "gamma_x", "gamma_z"],
    SEISMIC25: ["c11", "c12", "c13", "c14", "c15", "c16", "c22", "c23", "c24", "c25", "c26", "c33", "c34",
                "c35", "c36", "c44", "c45", "c46", "c55", "c56", "c66", "rho", "gamma_x", "gamma_y", "gamma_z"],
    ELECTROMAG2: ["eps11", "eps13", "eps33", "sig11", "sig13", "sig33"],
    ELECTROMAG25: ["eps11", "eps12", "eps13", "eps22", "eps23", "eps33",
                   "sig11", "sig12", "sig13", "sig22", "sig23", "sig33"],
    # complex permittivities as (real, imaginary) plane pairs
    ELECTROMAG2C: ["eps11_re", "eps11_im", "eps13_re", "eps13_im", "eps33_re", "eps33_im", "sig11", "sig13", "sig33"],
}
FIELDS = {
    SEISMIC2: ["vx", "vz", "sigmaxx", "sigmazz", "sigmaxz"],
    SEISMIC25: ["vx", "vy", "vz", "sigmaxx", "sigmayy", "sigmazz", "sigmaxy", "sigmaxz", "sigmayz"],
    ELECTROMAG2: ["Ex", "Ez", "Hy"],
    ELECTROMAG25: ["Ex", "Ey", "Ez", "Hx", "Hy", "Hz"],
    ELECTROMAG2C: ["Ex_re", "Ex_im", "Ez_re", "Ez_im", "Hy_re", "Hy_im"],
}
CHANNELS = {SEISMIC2: ["vx", "vz"], SEISMIC25: ["vx", "vy", "vz"],
            ELECTROMAG2: ["Ex", "Ez"], ELECTROMAG25: ["Ex", "Ey", "Ez"],
            ELECTROMAG2C: ["Ex_re", "Ex_im", "Ez_re", "Ez_im"]}
MEMORY = {
    ELECTROMAG2: ["dEx_dz", "dEz_dx", "dHy_dz", "dHy_dx"],
    # the last four: the sigmaxz loop's own velocity-gradient memory (corrected physics)
    SEISMIC2: ["dvx_dx", "dvz_dz", "dvx_dz", "dvz_dx", "dsigmaxx_dx", "dsigmazz_dz", "dsigmaxz_dx", "dsigmaxz_dz",
               "dvx_dx_sxz", "dvz_dz_sxz", "dvx_dz_sxz", "dvz_dx_sxz"],
    SEISMIC25: ["dvx_dx", "dvx_dy", "dvx_dz", "dvy_dx", "dvy_dy", "dvy_dz", "dvz_dx", "dvz_dy", "dvz_dz",
                "dsigmaxx_dx", "dsigmayy_dy", "dsigmazz_dz", "dsigmaxy_dx", "dsigmaxy_dy", "dsigmaxz_dx",
                "dsigmaxz_dz", "dsigmayz_dy", "dsigmayz_dz"],
    ELECTROMAG25: ["dEz_dy", "dEy_dz", "dEx_dz", "dEz_dx", "dEx_dy", "dEy_dx",
                   "dHz_dy", "dHy_dz", "dHz_dx", "dHx_dz", "dHx_dy", "dHy_dx"],
    ELECTROMAG2C: ["dEx_dz_re", "dEx_dz_im", "dEz_dx_re", "dEz_dx_im", "dHy_dz_re", "dHy_dz_im", "dHy_dx_re",
                   "dHy_dx_im"],
}


FLAG_TWO_PASS = 1
FLAG_STREAMING = 2
FLAG_LEGACY_QUIRKS = 4
FLAG_CPML_2D = 32  # electromag2, seismic2: CPML from the driver's 2-D fields (set_cpml2d)
# density_method (the driver's argument, src/seidart/routines/classes.py:311) -> flag bits
DENSITY_FLAGS = {"arithmetic": 0, "none": 8, "geometric": 16, "harmonic": 24}


def physics_flags(legacy: bool = False, density: str = "arithmetic") -> int:
    """sfd_config flag bits of the seismic physics options: ``legacy`` keeps
    the legacy Fortran loops' quirks (default: corrected physics), ``density``
    is the density averaging method."""
    if density not in DENSITY_FLAGS:
        raise ValueError(f"density must be one of {sorted(DENSITY_FLAGS)}, got {density!r}")
    return (FLAG_LEGACY_QUIRKS if legacy else 0) | DENSITY_FLAGS[density]


def is_25d(kind: int) -> bool:
    return kind in (SEISMIC25, ELECTROMAG25)


@dataclass
class GridSpec:
    """Full grid (CPML included) of one model."""
    kind: int
    nx: int
    nz: int
    dx: float
    dz: float
    dt: float
    npml: int
    ny: int = 1
    dy: float = 1.0

    @property
    def shape(self):
        return (self.nz, self.ny, self.nx) if is_25d(self.kind) else (self.nz, self.nx)

    @property
    def cells(self) -> int:
        return self.nx * self.ny * self.nz


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class FDTDSolver:
    """One FDTD model on the GPU, driven through the C ABI.

    ``flags`` = ``FLAG_TWO_PASS`` selects, for the 2-D kinds, the two-kernel
    step (fields updated in place) instead of the default single-pass step.
    ``FLAG_STREAMING`` keeps one launch per step even where the grid would
    fit on chip (by default an electromag2 grid that fits in the SMs' shared
    memory runs a whole ``run`` in one launch with the state held on chip).

    ``nstep`` is the number of source samples (the run length); ``nrec`` the
    number of receivers.  The device state is allocated with torch on
    ``device`` and bound to the current torch stream of that device.

    Seismic kinds: ``legacy`` reproduces the legacy Fortran loops' quirks
    (shared CPML memory of the two seismic2 stress loops, b_x_half(j), vx
    over the cell's own density; the seismic25 c16/c45 pairs) instead of the
    default corrected physics; ``density`` is the density averaging method
    ('arithmetic', 'none', 'geometric', 'harmonic').
    """

    def __init__(self, grid: GridSpec, nstep: int, nrec: int, device="cuda", stream=None, flags: int = 0,
                 legacy: bool = False, density: str = "arithmetic"):
        import torch
        if grid.kind in (SEISMIC2, SEISMIC25):
            flags = int(flags) | physics_flags(legacy, density)
        elif legacy or density != "arithmetic":
            raise ValueError("legacy and density apply to the seismic kinds only")

        self.grid = grid
        self.kind = grid.kind
        self.nstep = int(nstep)
        self.nrec = int(nrec)
        L = _lib.lib()
        self._L = L
        self.cfg = SfdConfig(kind=grid.kind, nx=grid.nx, ny=grid.ny if is_25d(grid.kind) else 1, nz=grid.nz,
                             npml=grid.npml, nstep=self.nstep, nrec=self.nrec, flags=int(flags),
                             dx=grid.dx, dy=grid.dy, dz=grid.dz, dt=grid.dt)
        nbytes = C.c_size_t(0)
        check(L.sfd_state_bytes(C.byref(self.cfg), C.byref(nbytes)))
        self.device = torch.device(device)
        self.state = torch.empty(int(nbytes.value), dtype=torch.uint8, device=self.device)
        if stream is None:
            stream = torch.cuda.current_stream(self.device)
        self.stream = stream
        h = C.c_void_p()
        check(L.sfd_create(C.byref(self.cfg), C.c_void_p(self.state.data_ptr()), C.c_size_t(self.state.numel()),
                           C.c_void_p(stream.cuda_stream), C.byref(h)))
        self._h = h
        self.nch = L.sfd_num_channels(grid.kind)

    # -- inputs ------------------------------------------------------------
    def set_model(self, planes) -> None:
        """Material planes: array (planes, NZ, NX) or dict name -> (NZ, NX)."""
        names = MODEL_PLANES[self.kind]
        if isinstance(planes, dict):
            zero = np.zeros((self.grid.nz, self.grid.nx))
            arr = np.stack([np.asarray(planes.get(n, zero), dtype=np.float64) for n in names])
        else:
            arr = np.asarray(planes, dtype=np.float64)
        arr = np.ascontiguousarray(arr)
        check(self._L.sfd_set_model(self._h, _dptr(arr), arr.size))

    def set_model_ids(self, ids, table) -> None:
        """The model as a material-id map: ids (NZ, NX) integers in [0, nmat)
        (numpy, or a torch tensor on this solver's device) and table (nmat,
        planes) in ``MODEL_PLANES`` order.  The coefficients are formed on the
        GPU; the id map is kept on the device with the solver."""
        import torch
        names = MODEL_PLANES[self.kind]
        tab = np.ascontiguousarray(np.asarray(table, dtype=np.float64))
        if tab.ndim != 2 or tab.shape[1] != len(names):
            raise ValueError(f"table must be (nmat, {len(names)}) in the order {names}")
        if isinstance(ids, torch.Tensor):
            dev = ids.to(device=self.device, dtype=torch.int32).contiguous()
        else:
            dev = torch.as_tensor(np.ascontiguousarray(np.asarray(ids, dtype=np.int32))).to(self.device)
        if tuple(dev.shape) != (self.grid.nz, self.grid.nx):
            raise ValueError(f"ids must be ({self.grid.nz}, {self.grid.nx}), got {tuple(dev.shape)}")
        check(self._L.sfd_set_model_ids(self._h, C.c_void_p(dev.data_ptr()), tab.shape[0], _dptr(tab), tab.size))
        self._ids = dev  # read again by set_source and the adjoint

    def set_cpml(self, profiles) -> None:
        """Per-axis CPML profiles: list of cpml.AxisProfile or the packed FP64 vector."""
        if isinstance(profiles, (list, tuple)):
            from .cpml import pack_profiles
            arr = pack_profiles(profiles)
        else:
            arr = np.ascontiguousarray(profiles, dtype=np.float64)
        check(self._L.sfd_set_cpml(self._h, _dptr(arr), arr.size))

    def set_cpml2d(self, fields) -> None:
        """The driver's 2-D CPML fields (solver created with ``FLAG_CPML_2D``):
        array (6, NZ, NX) of K, a, b, K_half, a_half, b_half, or a dict of
        those names."""
        names = ("K", "a", "b", "K_half", "a_half", "b_half")
        if isinstance(fields, dict):
            fields = np.stack([np.asarray(fields[n], dtype=np.float64) for n in names])
        arr = np.ascontiguousarray(fields, dtype=np.float64)
        if arr.shape != (6, self.grid.nz, self.grid.nx):
            raise ValueError(f"2-D CPML fields must be (6, {self.grid.nz}, {self.grid.nx})")
        check(self._L.sfd_set_cpml2d(self._h, _dptr(arr), arr.size))

    def set_cpml_params(self, sig_max, alpha_max, kappa_max=5.0, NP=2.0, NPA=2.0, mode="driver") -> None:
        """CPML profiles computed on the device (``sfd_set_cpml_params``):
        ``sig_max`` per axis (x, z) or (x, y, z), as ``cpml.sigma_alpha_max``
        gives them; the other parameters as ``cpml.axis_profile``."""
        sm = [float(v) for v in sig_max]
        if len(sm) == 2:
            sm = [sm[0], 0.0, sm[1]]
        if len(sm) != 3:
            raise ValueError("sig_max needs one value per axis")
        if mode not in ("driver", "legacy"):
            raise ValueError(f"unknown CPML mode {mode!r}")
        prm = _lib.SfdCpmlParams((C.c_double * 3)(*sm), float(alpha_max), float(kappa_max), float(NP), float(NPA),
                                 0 if mode == "driver" else 1)
        check(self._L.sfd_set_cpml_params(self._h, C.byref(prm)))

    def set_source_wavelet(self, ijk, f0, amp=1.0, comp=None, stype="gaus1", stress=False) -> None:
        """Source time functions formed on the device (``sfd_set_source_wavelet``):
        component c is ``comp[c] * amp * w(t)`` with ``w`` the driver's
        peak-normalised wavelet ``stype`` of centre frequency ``f0`` on the
        time vector ``arange(nstep) * dt``.  ``stress`` sets the stress source
        (moment-tensor factors in ``comp``) instead of the force source."""
        if stype not in _lib.WAVELETS:
            raise ValueError(f"unknown wavelet {stype!r}")
        c = np.ascontiguousarray(comp if comp is not None else [1.0], dtype=np.float64)
        i, j, k = (int(v) for v in ijk)
        check(self._L.sfd_set_source_wavelet(self._h, int(bool(stress)), i, j, k, _lib.WAVELETS[stype], float(f0),
                                             float(amp), _dptr(c), c.size))

    def share_model(self, other: "FDTDSolver") -> None:
        """Read ``other``'s update coefficients instead of a copy (shots of one model)."""
        check(self._L.sfd_share_model(self._h, other._h))
        self._model_owner = other  # keeps the coefficients alive

    def set_source(self, ijk, srcfn) -> None:
        """Source cell (i, j, k) (j = 0 in 2-D) and time functions (ncomp, nstep)."""
        s = np.ascontiguousarray(srcfn, dtype=np.float64)
        if s.ndim != 2:
            raise ValueError("srcfn must be (ncomp, nstep)")
        i, j, k = (int(v) for v in ijk)
        check(self._L.sfd_set_source(self._h, i, j, k, _dptr(s), s.shape[0], s.shape[1]))

    def set_stress_source(self, ijk, srcfn) -> None:
        """Seismic kinds: moment-tensor source at cell (i, j, k) (the force
        source's cell) with time functions (ncomp, nstep): sigma xx, zz, xz in
        2-D, xx, yy, zz, xy, xz, yz in 2.5-D; sigma_ij += srcfn[ij][t] dt
        after each stress half-step.  None removes it."""
        i, j, k = (int(v) for v in ijk)
        if srcfn is None:
            check(self._L.sfd_set_stress_source(self._h, i, j, k, None, 0, 0))
            return
        s = np.ascontiguousarray(srcfn, dtype=np.float64)
        if s.ndim != 2:
            raise ValueError("srcfn must be (ncomp, nstep)")
        check(self._L.sfd_set_stress_source(self._h, i, j, k, _dptr(s), s.shape[0], s.shape[1]))

    def set_receivers(self, ijk) -> None:
        r = np.ascontiguousarray(np.asarray(ijk, dtype=np.int32).reshape(-1, 3))
        check(self._L.sfd_set_receivers(self._h, r.ctypes.data_as(C.POINTER(C.c_int32)), r.shape[0]))

    def set_field(self, name, values) -> None:
        q = FIELDS[self.kind].index(name) if isinstance(name, str) else int(name)
        v = np.ascontiguousarray(values, dtype=np.float32)
        check(self._L.sfd_set_field(self._h, q, _fptr(v), v.size))

    # -- time stepping -----------------------------------------------------
    def run(self, nsteps: int) -> None:
        check(self._L.sfd_run(self._h, int(nsteps)))

    def status(self):
        """(steps done, largest field norm of the last run); raises UnstableError."""
        step = C.c_int64(0)
        norm = C.c_double(0.0)
        check(self._L.sfd_status(self._h, C.byref(step), C.byref(norm)))
        return int(step.value), float(norm.value)

    def reset(self) -> None:
        check(self._L.sfd_reset(self._h))

    def launch_half(self, which: int, count: int) -> None:
        """Profiling aid: run one half-step kernel ``count`` times (state is
        invalid afterwards; reset before the next run)."""
        check(self._L.sfd_launch_half(self._h, int(which), int(count)))

    def set_wait_limit(self, ns: int) -> None:
        """Longest wait (ns) of an on-chip run for a neighbouring tile; 0 = the
        default 2 s.  A wait that runs out makes ``status`` raise SfdError
        with code SFD_ERR_TIMEOUT."""
        check(self._L.sfd_set_wait_limit(self._h, int(ns)))

    def on_chip(self):
        """(tiles, tile rows) when ``run`` keeps the whole state on chip (one
        launch per run, one CTA per tile), else None (one launch per step)."""
        tx, tz = C.c_int32(), C.c_int32()
        rc = self._L.sfd_on_chip(self._h, C.byref(tx), C.byref(tz))
        if rc < 0:
            check(rc)
        return (tx.value, tz.value) if rc == 1 else None

    # -- outputs -----------------------------------------------------------
    def field(self, name) -> np.ndarray:
        q = FIELDS[self.kind].index(name) if isinstance(name, str) else int(name)
        out = np.empty(self.grid.shape, dtype=np.float32)
        check(self._L.sfd_get_field(self._h, q, _fptr(out), out.size))
        return out

    def field_async(self, name, out) -> None:
        """Queue the copy of field ``name`` into ``out`` (a page-locked CPU
        float32 torch tensor of the grid's shape) on the solver's stream and
        return at once; ``out`` holds the field once the stream has passed
        this point (record a CUDA event on ``self.stream`` after the call)."""
        import torch
        q = FIELDS[self.kind].index(name) if isinstance(name, str) else int(name)
        if out.dtype != torch.float32 or out.device.type != "cpu" or not out.is_contiguous() or \
                out.numel() != int(np.prod(self.grid.shape)):
            raise ValueError("out must be a contiguous float32 CPU tensor of the grid's size")
        check(self._L.sfd_get_field_async(self._h, q, C.c_void_p(out.data_ptr()), out.numel()))

    def encode_i16(self, name, codes, minmax) -> None:
        """Queue the block-floating int16 encoding of field ``name`` on the
        solver's stream (``sfd_encode_field_i16``): ``minmax`` (device float32,
        2 values) gets the field's min and max, ``codes`` (device int16, one per
        cell, x fastest) the codes of ``seidart_gb300.em25block``."""
        import torch
        q = FIELDS[self.kind].index(name) if isinstance(name, str) else int(name)
        n = int(np.prod(self.grid.shape))
        if codes.dtype != torch.int16 or codes.numel() != n or codes.device.type != "cuda" or not codes.is_contiguous():
            raise ValueError("codes must be a contiguous int16 CUDA tensor with one value per cell")
        if minmax.dtype != torch.float32 or minmax.numel() != 2 or minmax.device.type != "cuda":
            raise ValueError("minmax must be a float32 CUDA tensor of 2 values")
        check(self._L.sfd_encode_field_i16(self._h, q, C.c_void_p(codes.data_ptr()), C.c_void_p(minmax.data_ptr())))

    def complex_field(self, name) -> np.ndarray:
        """Field ``name`` ('Ex', 'Ez', 'Hy') of a complex-permittivity solver
        (ELECTROMAG2C) as complex64, from its real and imaginary planes."""
        return (self.field(name + "_re") + 1j * self.field(name + "_im")).astype(np.complex64)

    def complex_traces(self) -> np.ndarray:
        """Traces (nstep, 2, nrec) of Ex, Ez of an ELECTROMAG2C solver, complex64."""
        t = self.traces()
        return (t[:, 0::2] + 1j * t[:, 1::2]).astype(np.complex64)

    def memory(self, name) -> np.ndarray:
        q = MEMORY[self.kind].index(name) if isinstance(name, str) else int(name)
        out = np.empty(self.grid.shape, dtype=np.float32)
        check(self._L.sfd_get_memory(self._h, q, _fptr(out), out.size))
        return out

    def traces(self) -> np.ndarray:
        out = np.empty((self.nstep, self.nch, self.nrec), dtype=np.float32)
        check(self._L.sfd_get_traces(self._h, _fptr(out), out.size))
        return out

    def field_tensor(self, name):
        """Device view (no copy) of field ``name`` of the current state:
        (NZ, NX) in 2-D, (NZ, NY, NX) in 2.5-D, a strided view into the state
        buffer (rows padded to the library's pitch).  The view holds until the
        next ``run``, ``reset`` or checkpoint load: single-pass 2-D solvers
        alternate between two copies of their fields."""
        import torch
        q = FIELDS[self.kind].index(name) if isinstance(name, str) else int(name)
        ptr, pitch = C.c_void_p(), C.c_int64()
        check(self._L.sfd_field_device(self._h, q, C.byref(ptr), C.byref(pitch)))
        off = (int(ptr.value) - self.state.data_ptr()) // 4
        g = self.grid
        rows = g.nz * (g.ny if is_25d(self.kind) else 1)
        flat = self.state.view(torch.float32)[off: off + rows * pitch.value].view(rows, pitch.value)[:, :g.nx]
        return flat.view(g.nz, g.ny, g.nx) if is_25d(self.kind) else flat

    def traces_tensor(self):
        """Device view (nstep, nch, nrec) of the trace buffer (no copy)."""
        import torch
        ptr = self._L.sfd_traces_device(self._h)
        off = int(ptr) - self.state.data_ptr()
        n = self.nstep * self.nch * self.nrec
        return self.state[off: off + 4 * n].view(torch.float32).view(self.nstep, self.nch, self.nrec)

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.sfd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def run_shot(grid: GridSpec, planes, profiles, src_ijk, srcfn, rec_ijk, nsteps=None, device="cuda", ids=None,
             table=None, stress_srcfn=None, legacy: bool = False, density: str = "arithmetic"):
    """One complete shot: model + CPML + source + receivers in, traces out
    (host arrays both ways).  The model is ``planes``, or, with ``ids`` and
    ``table`` (``planes`` may then be None), a material-id map whose
    coefficients are formed on the GPU.  Seismic kinds also take a stress
    source (``stress_srcfn``, at the force source's cell) and the physics
    options of :class:`FDTDSolver`.  Raises UnstableError like the Fortran
    stop."""
    srcfn = np.asarray(srcfn, dtype=np.float64)
    nstep = srcfn.shape[1]
    rec = np.asarray(rec_ijk, dtype=np.int32).reshape(-1, 3)
    opts = {"legacy": legacy, "density": density} if grid.kind in (SEISMIC2, SEISMIC25) else {}
    with FDTDSolver(grid, nstep, rec.shape[0], device=device, **opts) as s:
        if ids is not None:
            s.set_model_ids(ids, table)
        else:
            s.set_model(planes)
        s.set_cpml(profiles)
        s.set_source(src_ijk, srcfn)
        if stress_srcfn is not None:
            s.set_stress_source(src_ijk, stress_srcfn)
        s.set_receivers(rec)
        s.run(nstep if nsteps is None else nsteps)
        s.status()
        return s.traces()



class ShotPipeline:
    """Runs many shots through two handles on two streams in turn, so a
    shot's host work (the FP64 model folding) and its uploads run while the
    GPU is still stepping the shot before; the GPU runs the shots one after
    another.  The handles persist between :meth:`run` calls and are reused
    while the grid, the number of steps and of receivers stay the same (a
    long-running caller keeps them warm); :meth:`close` releases them."""

    def __init__(self, device="cuda", legacy: bool = False, density: str = "arithmetic"):
        import torch
        self.device = torch.device(device)
        self.streams = [torch.cuda.Stream(self.device), torch.cuda.Stream(self.device)]
        self.solvers = [None, None]
        self.opts = {"legacy": legacy, "density": density}

    def _solver(self, k, grid, nstep, nrec):
        s = self.solvers[k]
        if s is not None and s.grid == grid and s.nstep == nstep and s.nrec == nrec:
            return s
        if s is not None:
            s.close()
        opts = self.opts if grid.kind in (SEISMIC2, SEISMIC25) else {}
        s = self.solvers[k] = FDTDSolver(grid, nstep, nrec, device=self.device, stream=self.streams[k], **opts)
        return s

    def run(self, shots):
        """Each shot is a tuple (grid, planes, profiles, src_ijk, srcfn,
        rec_ijk), host arrays in as for :func:`run_shot`; yields each shot's
        host traces, in order, as soon as they are back (UnstableError like
        the Fortran stop)."""
        pending = None
        for n, (grid, planes, profiles, src_ijk, srcfn, rec_ijk) in enumerate(shots):
            srcfn = np.asarray(srcfn, dtype=np.float64)
            rec = np.asarray(rec_ijk, dtype=np.int32).reshape(-1, 3)
            s = self._solver(n & 1, grid, srcfn.shape[1], rec.shape[0])
            # the setters only copy (and wait for their own copies); the state
            # is cleared after them, because the clearing kernels cannot start
            # before the previous shot's run leaves the SMs
            s.set_model(planes)
            s.set_cpml(profiles)
            s.set_source(src_ijk, srcfn)
            s.set_receivers(rec)
            s.reset()
            s.run(srcfn.shape[1])  # queued behind the previous shot's run
            if pending is not None:
                pending.status()
                yield pending.traces()
            pending = s
        if pending is not None:
            pending.status()
            yield pending.traces()

    def close(self) -> None:
        for k, s in enumerate(self.solvers):
            if s is not None:
                s.close()
                self.solvers[k] = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def run_shots(shots, device="cuda", legacy: bool = False, density: str = "arithmetic"):
    """Traces of many shots, in order, through a :class:`ShotPipeline` made
    for the call: each shot is a tuple (grid, planes, profiles, src_ijk,
    srcfn, rec_ijk), host arrays in and host traces out as for
    :func:`run_shot`."""
    with ShotPipeline(device, legacy, density) as p:
        yield from p.run(shots)
