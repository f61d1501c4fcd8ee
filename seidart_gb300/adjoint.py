"""Gradients of a receiver-trace misfit with respect to the electromag2 and
seismic2 models.

``TraceModel`` owns one single-pass electromag2 solver and its checkpoints.
Its forward pass runs the whole shot, saving the dynamic state every
``ckpt_every`` steps.  Its backward pass walks the checkpoints from the last
to the first.  For each one it recomputes that segment's forward states on the
device and runs the hand-written discrete adjoint backwards over them: when
the grid runs on chip, one launch recomputes the segment and writes every
step's state (``csrc/resident2d.cu``) and one launch sweeps the adjoint over
it with its state on chip (``csrc/resident_adj.cu``); otherwise one launch per
step does each (``csrc/adjoint_em2.cu``).  ``flags`` are the solver's
(``FLAG_STREAMING`` selects the per-step form).  ``sfd_adjoint_gradient`` then
applies the FP64 chain rule from the update coefficients to the model planes.
With ``record=True`` the forward pass instead keeps every step's state in
device memory (``sfd_adjoint_record``; about 6.7 MB a step on a 1040 x 540
electromag2 grid, 2.5 MB on a 440 x 240 seismic2 one) and the backward pass
is the adjoint sweep alone, with no recompute.

``traces = TraceMisfit.apply(eps11, eps33, sigma, model)`` is differentiable
in torch: ``eps11``, ``eps33``, ``sigma`` (sig11 = sig33) are per-cell
(NZ, NX) FP64 tensors, and the traces are (nstep, 2, nrec) FP32 on the GPU.

``SeismicTraceModel`` does the same for a seismic2 shot (any of the solver's
step forms, the corrected physics with 1-D CPML profiles, any density
method): the backward pass recomputes each segment (in one on-chip launch
when the grid runs on chip, else by the solver's own steps) and runs the
transposed step (``csrc/adjoint_s2.cu``) over it, and the
gradient covers all nine model planes (c11 c13 c15 c33 c35 c55 rho gamma_x
gamma_z).  ``traces = SeismicTraceMisfit.apply(planes, model)`` is its torch
function for a (9, NZ, NX) FP64 tensor.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check
from .solver import FDTDSolver, GridSpec


def _declare(L):
    if getattr(L, "_adj_declared", False):
        return
    P, i32, i64, sz = C.c_void_p, C.c_int32, C.c_int64, C.c_size_t
    for name, res, args in [
        ("sfd_checkpoint_bytes", i32, [P, C.POINTER(sz)]),
        ("sfd_checkpoint_save", i32, [P, P]),
        ("sfd_checkpoint_load", i32, [P, P, i64]),
        ("sfd_run_checkpointed", i32, [P, i64, P, sz, i32]),
        ("sfd_adjoint_bytes", i32, [P, i32, C.POINTER(sz)]),
        ("sfd_adjoint_begin", i32, [P, P, sz, i32, P]),
        ("sfd_adjoint_segment", i32, [P, i64]),
        ("sfd_adjoint_record", i32, [P, i64]),
        ("sfd_adjoint_gradient", i32, [P, C.POINTER(C.c_double), i64]),
    ]:
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    L._adj_declared = True


class _Checkpointed:
    """One solver, its checkpoints and the adjoint workspace; ``_run(planes)``
    runs the shot saving a checkpoint per segment, ``_gradient(resid)`` runs
    the adjoint over the segments, last first, and returns the FP64 gradient
    planes of ``sfd_adjoint_gradient``."""

    nplanes = 0

    def __init__(self, grid: GridSpec, base_planes, profiles, src_ijk, srcfn, rec_ijk, ckpt_every, device, flags,
                 record=False, **solver_kw):
        import torch

        self.grid = grid
        self.base = np.ascontiguousarray(base_planes, dtype=np.float64)
        self.src_ijk = src_ijk
        self.srcfn = np.asarray(srcfn, dtype=np.float64)
        self.nstep = self.srcfn.shape[1]
        self.record = bool(record)
        self._recorded = False
        self.ckpt_every = self.nstep if self.record else int(ckpt_every)
        self.solver = FDTDSolver(grid, self.nstep, len(rec_ijk), device=device, flags=flags, **solver_kw)
        self.solver.set_model(self.base)
        self.solver.set_cpml(profiles)
        self.solver.set_source(src_ijk, self.srcfn)
        self.solver.set_receivers(rec_ijk)
        L = _lib.lib()
        _declare(L)
        self._L = L
        h = self.solver._h
        nb = C.c_size_t()
        check(L.sfd_checkpoint_bytes(h, C.byref(nb)))
        self.nseg = (self.nstep + self.ckpt_every - 1) // self.ckpt_every
        self.ckpt = torch.empty((0 if self.record else self.nseg, int(nb.value)), dtype=torch.uint8,
                                device=self.solver.device)
        self.resid = torch.zeros((self.nstep, 2, len(rec_ijk)), dtype=torch.float32, device=self.solver.device)
        nb2 = C.c_size_t()
        check(L.sfd_adjoint_bytes(h, self.ckpt_every, C.byref(nb2)))
        self.work = torch.empty(int(nb2.value), dtype=torch.uint8, device=self.solver.device)

    def _run(self, planes):
        s = self.solver
        s.set_model(planes)
        s.set_source(self.src_ijk, self.srcfn)  # the amplitude is divided by the model at the source
        s.reset()
        if self.record:  # every state kept: the backward pass only sweeps
            check(self._L.sfd_adjoint_begin(s._h, C.c_void_p(self.work.data_ptr()), C.c_size_t(self.work.numel()),
                                            self.nstep, C.c_void_p(self.resid.data_ptr())))
            check(self._L.sfd_adjoint_record(s._h, self.nstep))
            self._recorded = True
        else:
            check(self._L.sfd_run_checkpointed(s._h, self.nstep, C.c_void_p(self.ckpt.data_ptr()),
                                               C.c_size_t(self.ckpt.stride(0)), self.ckpt_every))
        s.status()
        return s.traces_tensor().clone()

    def _gradient(self, resid):
        h = self.solver._h
        self.resid.copy_(resid.detach().reshape(self.resid.shape))
        if self.record:
            if not self._recorded:
                raise RuntimeError("a recorded backward pass needs the forward pass right before it")
            self._recorded = False
            check(self._L.sfd_adjoint_segment(h, self.nstep))
            return self._planes()
        check(self._L.sfd_adjoint_begin(h, C.c_void_p(self.work.data_ptr()), C.c_size_t(self.work.numel()),
                                        self.ckpt_every, C.c_void_p(self.resid.data_ptr())))
        for q in reversed(range(self.nseg)):
            start = q * self.ckpt_every
            n = min(self.ckpt_every, self.nstep - start)
            check(self._L.sfd_checkpoint_load(h, C.c_void_p(self.ckpt[q].data_ptr()), start))
            check(self._L.sfd_adjoint_segment(h, n))
        return self._planes()

    def _planes(self):
        import torch

        g = np.empty((self.nplanes, self.grid.nz, self.grid.nx))
        check(self._L.sfd_adjoint_gradient(self.solver._h, g.ctypes.data_as(C.POINTER(C.c_double)), g.size))
        torch.cuda.synchronize(self.solver.device)
        return g

    def close(self):
        self.solver.close()


class TraceModel(_Checkpointed):
    """An electromag2 shot whose eps11, eps33 and sigma can be differentiated.

    ``base_planes``: (6, NZ, NX) FP64 model (eps11 eps13 eps33 sig11 sig13 sig33);
    eps13 and sig13 stay fixed, the other planes are replaced by the inputs.
    ``flags`` are the solver's; the handle must be single-pass.  ``record``
    keeps every step's state from the forward pass (the grid must run on
    chip) so that ``backward`` needs no recompute; each ``backward`` then
    follows its own ``forward``.
    """

    nplanes = 6

    def __init__(self, grid: GridSpec, base_planes, profiles, src_ijk, srcfn, rec_ijk, ckpt_every=200,
                 device="cuda", flags=0, record=False):
        super().__init__(grid, base_planes, profiles, src_ijk, srcfn, rec_ijk, ckpt_every, device, flags,
                         record=record)

    def planes_for(self, eps11, eps33, sigma):
        p = self.base.copy()
        p[0] = np.asarray(eps11, dtype=np.float64)
        p[2] = np.asarray(eps33, dtype=np.float64)
        p[3] = np.asarray(sigma, dtype=np.float64)
        p[5] = np.asarray(sigma, dtype=np.float64)
        return p

    def forward(self, eps11, eps33, sigma):
        """Run the shot; returns the device trace tensor (nstep, 2, nrec)."""
        return self._run(self.planes_for(eps11, eps33, sigma))

    def backward(self, resid):
        """dJ/d(eps11, eps33, sigma) for dJ/d(traces) = resid (device FP32)."""
        g = self._gradient(resid)
        return g[0], g[2], g[3] + g[5], g


class SeismicTraceModel(_Checkpointed):
    """A seismic2 shot whose nine model planes (c11 c13 c15 c33 c35 c55 rho
    gamma_x gamma_z) can be differentiated.

    ``base_planes``: (9, NZ, NX) FP64, the model before the first ``forward``.
    ``density`` is the density averaging method; ``stress_srcfn`` (3, nstep)
    adds the moment-tensor source at the force source's cell.  ``flags`` are
    the solver's (any step form).  ``record`` keeps every step's state from
    the forward pass, as for ``TraceModel`` (the grid must run on chip).
    """

    nplanes = 9

    def __init__(self, grid: GridSpec, base_planes, profiles, src_ijk, srcfn, rec_ijk, ckpt_every=200,
                 device="cuda", flags=0, density="arithmetic", stress_srcfn=None, record=False):
        super().__init__(grid, base_planes, profiles, src_ijk, srcfn, rec_ijk, ckpt_every, device, flags,
                         record=record, density=density)
        if stress_srcfn is not None:
            self.solver.set_stress_source(src_ijk, stress_srcfn)

    def forward(self, planes):
        """Run the shot with the (9, NZ, NX) model; returns the device trace
        tensor (nstep, 2, nrec)."""
        return self._run(np.ascontiguousarray(planes, dtype=np.float64))

    def backward(self, resid):
        """dJ/d(planes) (9, NZ, NX) FP64 for dJ/d(traces) = resid (device FP32)."""
        return self._gradient(resid)


def _make_function():
    import torch

    class TraceMisfit(torch.autograd.Function):
        """traces = TraceMisfit.apply(eps11, eps33, sigma, model)."""

        @staticmethod
        def forward(ctx, eps11, eps33, sigma, model):
            ctx.model = model
            ctx.like = (eps11, eps33, sigma)
            return model.forward(eps11.detach().cpu().numpy(), eps33.detach().cpu().numpy(),
                                 sigma.detach().cpu().numpy())

        @staticmethod
        def backward(ctx, grad):
            g11, g33, gs, _ = ctx.model.backward(grad)
            outs = []
            for g, like in zip((g11, g33, gs), ctx.like):
                outs.append(torch.as_tensor(g, dtype=like.dtype, device=like.device))
            return outs[0], outs[1], outs[2], None

    return TraceMisfit


def _make_seismic_function():
    import torch

    class SeismicTraceMisfit(torch.autograd.Function):
        """traces = SeismicTraceMisfit.apply(planes, model), planes (9, NZ, NX)."""

        @staticmethod
        def forward(ctx, planes, model):
            ctx.model = model
            ctx.like = planes
            return model.forward(planes.detach().cpu().numpy())

        @staticmethod
        def backward(ctx, grad):
            g = ctx.model.backward(grad)
            return torch.as_tensor(g, dtype=ctx.like.dtype, device=ctx.like.device), None

    return SeismicTraceMisfit


class _Lazy:
    """The torch function, made on first use (torch is imported then)."""

    def __init__(self, make):
        self._make = make
        self._fn = None

    def __getattr__(self, name):
        if self._fn is None:
            self._fn = self._make()
        return getattr(self._fn, name)


TraceMisfit = _Lazy(_make_function)
SeismicTraceMisfit = _Lazy(_make_seismic_function)
