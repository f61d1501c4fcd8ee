"""GPU tests of the electromag2 discrete adjoint (checkpointed, recomputing).

The misfit is J = 1/2 sum (d(theta) - d_obs)^2 over all receivers and steps.
The GPU gradient (FP32 adjoint kernels) is checked against central finite
differences of the FP64 oracle's J: along random smooth directions (which
tests every cell at once) and at single cells.
"""
import numpy as np
import pytest

import oracle
from seidart_gb300 import ELECTROMAG2, cpml as cp, synthetic as sy
from seidart_gb300.adjoint import TraceModel, TraceMisfit

pytestmark = pytest.mark.gpu


def _case():
    return sy.small_case(ELECTROMAG2, seed=41, nx=44, nz=38, npml=5, nstep=130, nrec=10)


def _oracle_traces(case, planes):
    _, tr, _, blew = oracle.run(ELECTROMAG2, case.grid, planes, cp.pack_profiles(case.profiles), case.src_ijk,
                                case.srcfn, case.rec_ijk, case.nstep)
    assert not blew
    return tr


def _blob(shape, rng, amp):
    z, x = np.meshgrid(np.arange(shape[0]), np.arange(shape[1]), indexing="ij")
    cz, cx = rng.uniform(0.3, 0.7) * shape[0], rng.uniform(0.3, 0.7) * shape[1]
    return amp * np.exp(-((z - cz) ** 2 + (x - cx) ** 2) / (2 * 6.0 ** 2))


def _setup():
    case = _case()
    rng = np.random.default_rng(5)
    case.planes[5] = case.planes[3]  # the differentiable model ties sig33 = sig11 = sigma
    base = case.planes.copy()
    d_obs = _oracle_traces(case, base)
    true = base.copy()
    true[0] = base[0] * (1 + _blob(base[0].shape, rng, 0.05))
    true[2] = base[2] * (1 + _blob(base[0].shape, rng, -0.05))
    # current model = perturbed; data = unperturbed
    return case, true, d_obs, rng


def _J(case, planes, d_obs):
    tr = _oracle_traces(case, planes)
    return 0.5 * float(np.sum((tr - d_obs) ** 2))


@pytest.mark.parametrize("ckpt", [25, 130])
def test_directional_derivative_matches_fd(gpu, ckpt):
    case, cur, d_obs, rng = _setup()
    m = TraceModel(case.grid, cur, case.profiles, case.src_ijk, case.srcfn, case.rec_ijk, ckpt_every=ckpt)
    import torch
    tr = m.forward(cur[0], cur[2], cur[3])
    resid = tr - torch.as_tensor(d_obs, dtype=torch.float32, device=tr.device)
    g11, g33, gs, g6 = m.backward(resid)
    m.close()
    for q, scale in ((0, 1.0), (2, 1.0), (3, 1e-3)):
        direction = np.zeros_like(cur)
        direction[q] = _blob(cur[0].shape, rng, scale)
        if q == 3:
            direction[5] = direction[3]
        eps = 1e-4
        jp = _J(case, cur + eps * direction, d_obs)
        jm = _J(case, cur - eps * direction, d_obs)
        fd = (jp - jm) / (2 * eps)
        ad = float(np.sum(g6 * direction))
        assert abs(ad - fd) <= 2e-3 * abs(fd) + 1e-30, f"plane {q}: adjoint {ad:.6e} vs FD {fd:.6e}"


def test_gradient_matches_fp64_discrete_adjoint(gpu):
    """Every cell of the GPU gradient against the FP64 numpy adjoint of the same scheme."""
    import torch
    from oracle import numpy_adjoint as na
    case, cur, d_obs, rng = _setup()
    g = case.grid
    prof = cp.pack_profiles(case.profiles)
    src = (case.src_ijk[0], case.src_ijk[2])
    tr64, states = na.forward(g.nx, g.nz, g.dx, g.dz, g.dt, prof, cur, src, case.srcfn, case.nstep, case.rec_ijk)
    ref = na.gradient(g.nx, g.nz, g.dx, g.dz, g.dt, prof, cur, src, case.srcfn, case.rec_ijk, states, tr64 - d_obs)
    m = TraceModel(g, cur, case.profiles, case.src_ijk, case.srcfn, case.rec_ijk, ckpt_every=32)
    tr = m.forward(cur[0], cur[2], cur[3])
    _, _, _, g6 = m.backward(tr - torch.as_tensor(d_obs, dtype=torch.float32, device=tr.device))
    m.close()
    for q in range(6):
        err = np.linalg.norm(g6[q] - ref[q]) / np.linalg.norm(ref[q])
        assert err <= 2e-3, f"plane {q}: relative L2 {err:.3e}"


def test_pointwise_gradient_and_autograd(gpu):
    import torch
    case, cur, d_obs, rng = _setup()
    m = TraceModel(case.grid, cur, case.profiles, case.src_ijk, case.srcfn, case.rec_ijk, ckpt_every=40)
    e11 = torch.tensor(cur[0], requires_grad=True)
    e33 = torch.tensor(cur[2], requires_grad=True)
    sig = torch.tensor(cur[3], requires_grad=True)
    tr = TraceMisfit.apply(e11, e33, sig, m)
    J = 0.5 * ((tr - torch.as_tensor(d_obs, dtype=torch.float32, device=tr.device)) ** 2).sum()
    J.backward()
    g11 = e11.grad.numpy()
    m.close()
    # FD at the cells with the largest gradient (plus the source cell)
    flat = np.argsort(np.abs(g11).ravel())[::-1][:4]
    cells = [np.unravel_index(f, g11.shape) for f in flat] + [(case.src_ijk[2], case.src_ijk[0])]
    for (k, i) in cells:
        h = 1e-4 * cur[0][k, i]
        p, q = cur.copy(), cur.copy()
        p[0][k, i] += h
        q[0][k, i] -= h
        fd = (_J(case, p, d_obs) - _J(case, q, d_obs)) / (2 * h)
        assert abs(g11[k, i] - fd) <= 5e-3 * abs(fd) + 1e-3 * np.abs(g11).max(), (k, i, g11[k, i], fd)


def _grads(case, planes, d_obs_t, flags, ckpt):
    m = TraceModel(case.grid, planes, case.profiles, case.src_ijk, case.srcfn, case.rec_ijk, ckpt_every=ckpt,
                   flags=flags)
    try:
        on_chip = m.solver.on_chip()
        tr = m.forward(planes[0], planes[2], planes[3])
        _, _, _, g6 = m.backward(tr - d_obs_t(tr))
        return on_chip, tr.cpu().numpy(), g6
    finally:
        m.close()


@pytest.mark.parametrize("grid", ["small", "layered"])
def test_on_chip_adjoint_matches_per_step_adjoint(gpu, grid):
    """The on-chip sweep (one recompute launch and one adjoint launch per
    checkpoint segment) against the per-step kernels, on a small grid of many
    tiles and on the 1040 x 540 layered model (152 tiles) with uneven
    segments.  The two forms do the same FP32 arithmetic per cell in a
    different order, so the gradients agree to rounding, not bit for bit."""
    import torch
    from seidart_gb300.solver import FLAG_STREAMING
    if grid == "small":
        case, cur, d_obs, _ = _setup()
        ckpt = 40
        d_obs_t = lambda tr: torch.as_tensor(d_obs, dtype=torch.float32, device=tr.device)
    else:
        case = sy.electromag2_layers(nstep=300)
        case.planes[5] = case.planes[3]
        cur = case.planes.copy()
        cur[0] = cur[0] * 1.02
        ckpt = 110
        d_obs_t = lambda tr: torch.zeros_like(tr)
    on_a, tr_a, ga = _grads(case, cur, d_obs_t, 0, ckpt)
    on_b, tr_b, gb = _grads(case, cur, d_obs_t, FLAG_STREAMING, ckpt)
    assert on_a is not None and on_b is None
    assert np.linalg.norm(tr_a - tr_b) <= 1e-5 * np.linalg.norm(tr_b)
    for q in (0, 2, 3, 5):
        err = np.linalg.norm(ga[q] - gb[q]) / np.linalg.norm(gb[q])
        assert err <= 1e-4, f"plane {q}: relative L2 {err:.3e}"


@pytest.mark.parametrize("flags", [0, "streaming"])
def test_run_checkpointed_matches_save_and_run(gpu, flags):
    """sfd_run_checkpointed (on chip: checkpoints written from the one launch
    of the run) saves the same states as a save / run loop, and leaves the
    same final state and traces."""
    import ctypes as C
    import torch
    from seidart_gb300 import _lib
    from seidart_gb300.adjoint import _declare
    from seidart_gb300.solver import FLAG_STREAMING
    from helpers import make_solver
    case = sy.electromag2_layers(nstep=230)
    fl = FLAG_STREAMING if flags == "streaming" else 0
    L = _lib.lib()
    _declare(L)
    out = []
    for mode in ("checkpointed", "loop"):
        s = make_solver(case, gpu, fl)
        try:
            assert (s.on_chip() is not None) == (fl == 0)
            nb = C.c_size_t()
            assert L.sfd_checkpoint_bytes(s._h, C.byref(nb)) == 0
            every = 50
            nseg = (case.nstep + every - 1) // every
            ck = torch.zeros((nseg, nb.value + 12), dtype=torch.uint8, device=gpu)  # padded rows: stride > size
            if mode == "checkpointed":
                assert L.sfd_run_checkpointed(s._h, case.nstep, C.c_void_p(ck.data_ptr()), C.c_size_t(ck.stride(0)),
                                              every) == 0, L.sfd_last_error()
            else:
                for q in range(nseg):
                    assert L.sfd_checkpoint_save(s._h, C.c_void_p(ck[q].data_ptr())) == 0
                    s.run(min(every, case.nstep - q * every))
            s.status()
            out.append((ck.cpu().numpy()[:, :nb.value], s.traces(), s.field("Ex")))
        finally:
            s.close()
    (ca, ta, ea), (cb, tb, eb) = out
    assert np.array_equal(ca, cb)
    assert np.array_equal(ta, tb) and np.array_equal(ea, eb)


@pytest.mark.parametrize("grid", ["small", "layered"])
def test_recorded_adjoint_matches_checkpointed(gpu, grid):
    """sfd_adjoint_record keeps every forward state so that the backward pass
    is the sweep alone.  Its forward pass is the same on-chip kernel as a run
    (traces and final state bit for bit) and its states are the ones the
    checkpointed form recomputes, so the gradients agree to rounding."""
    import torch
    if grid == "small":
        case, cur, d_obs, _ = _setup()
        d_obs_t = lambda tr: torch.as_tensor(d_obs, dtype=torch.float32, device=tr.device)
    else:
        case = sy.electromag2_layers(nstep=300)
        case.planes[5] = case.planes[3]
        cur = case.planes.copy()
        cur[0] = cur[0] * 1.02
        d_obs_t = lambda tr: torch.zeros_like(tr)
    out = []
    for record in (False, True):
        m = TraceModel(case.grid, cur, case.profiles, case.src_ijk, case.srcfn, case.rec_ijk, ckpt_every=70,
                       record=record)
        try:
            assert m.solver.on_chip() is not None
            tr = m.forward(cur[0], cur[2], cur[3])
            ex = m.solver.field("Ex")
            _, _, _, g6 = m.backward(tr - d_obs_t(tr))
            if record:
                with pytest.raises(RuntimeError):
                    m.backward(tr - d_obs_t(tr))
            out.append((tr.cpu().numpy(), ex, g6))
        finally:
            m.close()
    (ta, ea, ga), (tb, eb, gb) = out
    assert np.array_equal(ta, tb) and np.array_equal(ea, eb)
    # The recorded form sweeps the whole run at once, the checkpointed form
    # one segment at a time, so each cell's per-step products are summed in
    # a different grouping; the conductivity plane's sums cancel the most
    # (measured: 1e-7 for the permittivity planes, 4e-7 to 1.3e-6 for it,
    # depending on the forward tiling's rounding).
    for q, tol in ((0, 1e-6), (2, 1e-6), (3, 3e-6), (5, 1e-6)):
        err = np.linalg.norm(ga[q] - gb[q]) / np.linalg.norm(ga[q])
        assert err <= tol, f"plane {q}: relative L2 {err:.3e}"


def test_record_refused_off_chip(gpu):
    """A handle whose runs are not on chip cannot record: the C call says so."""
    from seidart_gb300._lib import SfdError
    from seidart_gb300.solver import FLAG_STREAMING
    case, cur, _, _ = _setup()
    m = TraceModel(case.grid, cur, case.profiles, case.src_ijk, case.srcfn, case.rec_ijk, flags=FLAG_STREAMING,
                   record=True)
    try:
        with pytest.raises(SfdError, match="on chip"):
            m.forward(cur[0], cur[2], cur[3])
    finally:
        m.close()
