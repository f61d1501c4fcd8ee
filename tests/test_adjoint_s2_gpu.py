"""GPU tests of the seismic2 discrete adjoint (checkpointed, recomputing).

The misfit is J = 1/2 sum (d(theta) - d_obs)^2 over all receivers and steps.
The GPU gradient of all nine planes (c11 c13 c15 c33 c35 c55 rho gamma_x
gamma_z) is checked cell by cell against the FP64 numpy adjoint of the same
scheme, and along smooth directions against central finite differences of
the FP64 oracle's J, for the solver's step forms and density methods, with
attenuation and a moment-tensor source.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from seidart_gb300 import SEISMIC2, cpml as cp, synthetic as sy
from seidart_gb300.adjoint import SeismicTraceMisfit, SeismicTraceModel
from seidart_gb300.solver import FLAG_CPML_2D, FLAG_STREAMING, FLAG_TWO_PASS, FDTDSolver

pytestmark = pytest.mark.gpu


def _blob(shape, rng, amp, width=6.0):
    z, x = np.meshgrid(np.arange(shape[0]), np.arange(shape[1]), indexing="ij")
    cz, cx = rng.uniform(0.3, 0.7) * shape[0], rng.uniform(0.3, 0.7) * shape[1]
    return amp * np.exp(-((z - cz) ** 2 + (x - cx) ** 2) / (2 * width ** 2))


def _setup(density, seed=17):
    case = sy.small_case(SEISMIC2, seed=seed, nx=46, nz=40, npml=5, nstep=160, nrec=10)
    rng = np.random.default_rng(seed)
    t = np.arange(case.nstep)
    ssrc = 2e5 * rng.standard_normal((3, 1)) * np.exp(-((t - 25) / 8.0) ** 2)[None, :]
    prof = cp.pack_profiles(case.profiles)
    _, d_obs, _, blew = oracle.run(SEISMIC2, case.grid, case.planes, prof, case.src_ijk, case.srcfn, case.rec_ijk,
                                   case.nstep, density=density, stress_src=ssrc)
    assert not blew
    cur = case.planes.copy()
    for q, a in ((0, 0.04), (3, -0.04), (5, 0.05), (6, -0.03)):
        cur[q] = case.planes[q] * (1 + _blob(cur[0].shape, rng, a))
    return case, prof, ssrc, cur, d_obs, rng


def _model(case, cur, ssrc, density, flags=0, ckpt=40):
    return SeismicTraceModel(case.grid, cur, case.profiles, case.src_ijk, case.srcfn, case.rec_ijk, ckpt_every=ckpt,
                             flags=flags, density=density, stress_srcfn=ssrc)


def _gpu_gradient(case, cur, ssrc, d_obs, density, flags=0, ckpt=40):
    import torch
    m = _model(case, cur, ssrc, density, flags, ckpt)
    try:
        tr = m.forward(cur)
        g = m.backward(tr - torch.as_tensor(d_obs, dtype=torch.float32, device=tr.device))
        return tr.cpu().numpy(), g
    finally:
        m.close()


@pytest.mark.parametrize("density,flags,ckpt", [("arithmetic", 0, 40), ("harmonic", FLAG_TWO_PASS, 160),
                                                ("geometric", FLAG_STREAMING, 33)])
def test_gradient_matches_fp64_discrete_adjoint(gpu, density, flags, ckpt):
    """Every cell of the nine GPU gradient planes against the FP64 numpy adjoint."""
    from oracle import numpy_adjoint as na
    case, prof, ssrc, cur, d_obs, _ = _setup(density)
    g = case.grid
    src = (case.src_ijk[0], case.src_ijk[2])
    tr64, states, _ = na.seismic2_forward(g.nx, g.nz, g.dx, g.dz, g.dt, prof, cur, src, case.srcfn, case.nstep,
                                          case.rec_ijk, density=density, stress_src=ssrc)
    ref = na.seismic2_gradient(g.nx, g.nz, g.dx, g.dz, g.dt, prof, cur, src, case.srcfn, case.rec_ijk, states,
                               tr64 - d_obs, density=density, stress_src=ssrc)
    tr, g9 = _gpu_gradient(case, cur, ssrc, d_obs, density, flags, ckpt)
    assert np.linalg.norm(tr - tr64) <= 1e-5 * np.linalg.norm(tr64)
    for q in range(9):
        err = np.linalg.norm(g9[q] - ref[q]) / np.linalg.norm(ref[q])
        assert err <= 3e-3, f"plane {q}: relative L2 {err:.3e}"


def test_directional_derivative_matches_fd(gpu):
    """<dJ/dtheta, d> against central differences of the FP64 oracle's J."""
    density = "arithmetic"
    case, prof, ssrc, cur, d_obs, rng = _setup(density)
    _, g9 = _gpu_gradient(case, cur, ssrc, d_obs, density)

    def J(p):
        _, tr, _, _ = oracle.run(SEISMIC2, case.grid, p, prof, case.src_ijk, case.srcfn, case.rec_ijk, case.nstep,
                                 density=density, stress_src=ssrc)
        return 0.5 * float(np.sum((tr - d_obs) ** 2))

    for q in range(9):
        direction = np.zeros_like(cur)
        scale = 1e-3 if q >= 7 else float(np.abs(cur[q]).mean())
        direction[q] = _blob(cur[0].shape, rng, scale)
        eps = 1e-4
        fd = (J(cur + eps * direction) - J(cur - eps * direction)) / (2 * eps)
        ad = float(np.sum(g9[q] * direction[q]))
        assert abs(ad - fd) <= 3e-3 * abs(fd) + 1e-30, f"plane {q}: adjoint {ad:.6e} vs FD {fd:.6e}"


def test_step_forms_agree_and_autograd(gpu):
    """The single-pass and two-pass handles give the same gradient, and the
    torch function returns it."""
    import torch
    density = "arithmetic"
    case, prof, ssrc, cur, d_obs, _ = _setup(density, seed=23)
    _, ga = _gpu_gradient(case, cur, ssrc, d_obs, density, 0, 50)
    _, gb = _gpu_gradient(case, cur, ssrc, d_obs, density, FLAG_TWO_PASS, 50)
    for q in range(9):
        assert np.linalg.norm(ga[q] - gb[q]) <= 1e-4 * np.linalg.norm(ga[q]), q
    m = _model(case, cur, ssrc, density, 0, 50)
    try:
        planes = torch.tensor(cur, requires_grad=True)
        tr = SeismicTraceMisfit.apply(planes, m)
        J = 0.5 * ((tr - torch.as_tensor(d_obs, dtype=torch.float32, device=tr.device)) ** 2).sum()
        J.backward()
        gt = planes.grad.numpy()
    finally:
        m.close()
    for q in range(9):
        assert np.linalg.norm(gt[q] - ga[q]) <= 1e-4 * np.linalg.norm(ga[q]), q


@pytest.mark.parametrize("opts", [dict(legacy=True), dict(flags=FLAG_CPML_2D)])
def test_unsupported_physics_is_refused(gpu, opts):
    from seidart_gb300 import _lib
    from seidart_gb300.adjoint import _declare
    case = sy.small_case(SEISMIC2, seed=1, nx=24, nz=20, npml=4, nstep=10, nrec=2)
    s = FDTDSolver(case.grid, case.nstep, 2, **opts)
    try:
        L = _lib.lib()
        _declare(L)
        nb = C.c_size_t()
        assert L.sfd_adjoint_bytes(s._h, 10, C.byref(nb)) != 0
        assert "corrected physics" in L.sfd_last_error().decode()
    finally:
        s.close()


def test_shared_and_boundary_receivers(gpu):
    """Receivers that share a cell add their residuals there, and a receiver
    on a Dirichlet plane (whose trace is zero) adds none: the GPU gradient
    against the FP64 numpy adjoint with such a receiver set."""
    import dataclasses
    from oracle import numpy_adjoint as na
    density = "arithmetic"
    case, prof, ssrc, cur, _, _ = _setup(density, seed=31)
    g = case.grid
    rec = np.array(case.rec_ijk, dtype=np.int32).copy()
    rec[1] = rec[0]                      # two receivers at one cell
    rec[2] = (0, 0, g.nz // 2)           # on the x = 0 plane
    rec[3] = rec[5]
    case = dataclasses.replace(case, rec_ijk=rec)
    src = (case.src_ijk[0], case.src_ijk[2])
    _, d_obs, _, _ = oracle.run(SEISMIC2, g, case.planes, prof, case.src_ijk, case.srcfn, rec, case.nstep,
                                density=density, stress_src=ssrc)
    tr64, states, _ = na.seismic2_forward(g.nx, g.nz, g.dx, g.dz, g.dt, prof, cur, src, case.srcfn, case.nstep, rec,
                                          density=density, stress_src=ssrc)
    ref = na.seismic2_gradient(g.nx, g.nz, g.dx, g.dz, g.dt, prof, cur, src, case.srcfn, rec, states, tr64 - d_obs,
                               density=density, stress_src=ssrc)
    _, g9 = _gpu_gradient(case, cur, ssrc, d_obs, density, 0, 50)
    for q in range(9):
        err = np.linalg.norm(g9[q] - ref[q]) / np.linalg.norm(ref[q])
        assert err <= 3e-3, f"plane {q}: relative L2 {err:.3e}"


def test_recorded_adjoint_matches_checkpointed(gpu):
    """sfd_adjoint_record on a seismic2 handle: the forward pass keeps every
    step's state (traces and final state as a plain run's), the backward pass
    only sweeps, and the gradient equals the checkpointed one to rounding."""
    import torch
    density = "harmonic"
    case, prof, ssrc, cur, d_obs, _ = _setup(density, seed=37)
    out = []
    for record in (False, True):
        m = SeismicTraceModel(case.grid, cur, case.profiles, case.src_ijk, case.srcfn, case.rec_ijk, ckpt_every=45,
                              density=density, stress_srcfn=ssrc, record=record)
        try:
            assert m.solver.on_chip() is not None
            tr = m.forward(cur)
            vx = m.solver.field("vx")
            g = m.backward(tr - torch.as_tensor(d_obs, dtype=torch.float32, device=tr.device))
            out.append((tr.cpu().numpy(), vx, g))
        finally:
            m.close()
    (ta, va, ga), (tb, vb, gb) = out
    assert np.array_equal(ta, tb) and np.array_equal(va, vb)
    for q in range(9):
        err = np.linalg.norm(ga[q] - gb[q]) / np.linalg.norm(ga[q])
        assert err <= 1e-6, f"plane {q}: relative L2 {err:.3e}"
