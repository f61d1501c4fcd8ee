"""GPU: models given as a material-id map and a table (sfd_set_model_ids),
with the update coefficients formed on the device, against the same models
given as full FP64 planes (sfd_set_model).

Both paths evaluate the same FP64 formulas and round once to FP32, so the
runs are compared bit for bit; the adjoint gradient of an id-map model
(whose FP64 planes the host expands from the ids on demand) is compared
likewise.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import make_solver
from seidart_gb300 import ELECTROMAG2, ELECTROMAG25, SEISMIC2, SEISMIC25
from seidart_gb300 import synthetic as sy
from seidart_gb300._lib import SfdError

pytestmark = pytest.mark.gpu


def _id_model(kind, nx, nz, nmat, seed):
    """A random block-structured id map and a table of plausible materials."""
    rng = np.random.default_rng(seed)
    coarse = rng.integers(0, nmat, size=(nz // 6 + 1, nx // 6 + 1))
    ids = np.kron(coarse, np.ones((6, 6), dtype=np.int64))[:nz, :nx].astype(np.int32)
    if kind == ELECTROMAG2:  # eps11 eps13 eps33 sig11 sig13 sig33
        table = np.column_stack([rng.uniform(1.5, 3.2, nmat), rng.uniform(0, 0.05, nmat), rng.uniform(1.5, 3.2, nmat),
                                 10 ** rng.uniform(-6, -3, nmat), np.zeros(nmat), 10 ** rng.uniform(-6, -3, nmat)])
    else:  # c11 c13 c15 c33 c35 c55 rho gamma_x gamma_z (wave speeds within small_case's time step)
        c11 = rng.uniform(8e9, 12e9, nmat)
        table = np.column_stack([c11, 0.4 * c11, rng.uniform(0, 1e8, nmat), rng.uniform(8e9, 12e9, nmat),
                                 rng.uniform(0, 1e8, nmat), rng.uniform(1.5e9, 3e9, nmat), rng.uniform(850, 950, nmat),
                                 rng.uniform(0, 0.002, nmat) * (np.arange(nmat) % 2), np.zeros(nmat)])
    planes = np.ascontiguousarray(np.transpose(table[ids], (2, 0, 1)))
    return ids, table, planes


def _pair(kind, seed, nx=70, nz=56, nmat=4, nstep=120):
    case = sy.small_case(kind, seed=seed, nx=nx, nz=nz, npml=6, nstep=nstep)
    if kind in (SEISMIC25, ELECTROMAG25):  # materials drawn from the case's own cells (its time step fits them)
        rng = np.random.default_rng(seed)
        ids, _, _ = _id_model(ELECTROMAG2, nx, nz, nmat, seed)
        cells = rng.integers(0, nx * nz, nmat)
        table = np.ascontiguousarray(case.planes.reshape(case.planes.shape[0], -1)[:, cells].T)
        planes = np.ascontiguousarray(np.transpose(table[ids], (2, 0, 1)))
    else:
        ids, table, planes = _id_model(kind, nx, nz, nmat, seed)
    case.planes = planes
    a = make_solver(case)
    b = make_solver(case)
    b.set_model_ids(ids, table)
    b.set_source(case.src_ijk, case.srcfn)  # the amplitude divides by the model at the source cell
    return case, a, b, ids, table


@pytest.mark.parametrize("kind,seed", [(ELECTROMAG2, 1), (ELECTROMAG2, 2), (SEISMIC2, 3), (SEISMIC2, 4),
                                       (ELECTROMAG25, 5), (SEISMIC25, 6)])
def test_id_map_matches_planes(gpu, kind, seed):
    three = kind in (SEISMIC25, ELECTROMAG25)
    case, a, b, _, _ = _pair(kind, seed, nx=40 if three else 70, nz=34 if three else 56, nstep=60 if three else 120)
    with a, b:
        for s in (a, b):
            s.run(47)
            s.run(case.nstep - 47)
            s.status()
        assert np.array_equal(a.traces(), b.traces())
        from seidart_gb300.solver import FIELDS
        for name in FIELDS[kind]:
            assert np.array_equal(a.field(name), b.field(name)), name


@pytest.mark.parametrize("kind,density,legacy", [(SEISMIC2, "geometric", False), (SEISMIC2, "harmonic", True),
                                                  (SEISMIC2, "none", False), (SEISMIC25, "harmonic", False),
                                                  (SEISMIC25, "geometric", True)])
def test_id_map_matches_planes_with_physics_options(gpu, kind, density, legacy):
    """The density methods and the legacy/corrected density of vx, formed on
    the device from the ids and on the host from the planes.  Both evaluate
    the same FP64 expression; the 2.5-D geometric mean goes through cbrt,
    whose host and device results may differ in the last bit, so that case
    is compared to 1e-6 instead of bit for bit."""
    from helpers import rel_l2
    from seidart_gb300.solver import FIELDS
    three = kind == SEISMIC25
    case, a, b, ids, table = _pair(kind, 7, nx=40 if three else 64, nz=34 if three else 52, nstep=60 if three else 100)
    a.close()
    b.close()
    case.density, case.legacy = density, legacy
    a = make_solver(case)
    b = make_solver(case)
    b.set_model_ids(ids, table)
    b.set_source(case.src_ijk, case.srcfn)
    exact = not (three and density == "geometric")
    with a, b:
        for s in (a, b):
            s.run(case.nstep)
            s.status()
        if exact:
            assert np.array_equal(a.traces(), b.traces())
        else:
            assert rel_l2(b.traces(), a.traces()) <= 1e-6
        for name in FIELDS[kind]:
            if exact:
                assert np.array_equal(a.field(name), b.field(name)), name
            else:
                assert rel_l2(b.field(name), a.field(name)) <= 1e-6, name


def test_bad_ids_and_tables_are_rejected(gpu):
    case, a, b, ids, table = _pair(SEISMIC2, 5, nstep=10)
    with a, b:
        bad = ids.copy()
        bad[3, 4] = table.shape[0]
        with pytest.raises(SfdError):
            b.set_model_ids(bad, table)
        neg = table.copy()
        neg[1, 6] = -1.0  # density
        with pytest.raises(SfdError):
            b.set_model_ids(ids, neg)
        with pytest.raises(ValueError):
            b.set_model_ids(ids, table[:, :5])


def test_adjoint_gradient_of_an_id_map_model(gpu):
    """The chain rule reads the FP64 planes, expanded from the ids on demand."""
    import torch
    from seidart_gb300 import adjoint as adj
    nx, nz = 64, 52
    case = sy.small_case(ELECTROMAG2, seed=8, nx=nx, nz=nz, npml=6, nstep=90)
    ids, table, planes = _id_model(ELECTROMAG2, nx, nz, 3, 8)
    table[:, 5] = table[:, 3]  # TraceModel's sigma is sig11 = sig33
    planes[5] = planes[3]
    tm = adj.TraceModel(case.grid, planes, case.profiles, case.src_ijk, case.srcfn, case.rec_ijk, ckpt_every=30)
    try:
        tr = tm.forward(planes[0], planes[2], planes[3])
        resid = torch.randn_like(tr)
        want = tm.backward(resid)[3]
        # the same model as ids: forward with checkpoints and the adjoint, as TraceModel does
        s, L, h = tm.solver, tm._L, tm.solver._h
        s.set_model_ids(ids, table)
        s.set_source(case.src_ijk, case.srcfn)
        s.reset()
        for q in range(tm.nseg):
            L.sfd_checkpoint_save(h, C.c_void_p(tm.ckpt[q].data_ptr()))
            s.run(min(tm.ckpt_every, tm.nstep - q * tm.ckpt_every))
        s.status()
        assert torch.equal(s.traces_tensor(), tr)
        got = tm.backward(resid)[3]
        assert np.array_equal(got, want)
    finally:
        tm.close()


def test_run_shot_of_the_layered_model_by_ids(gpu):
    """The 1040 x 540 layered model (three materials) through run_shot, as
    planes and as its id map: the same traces."""
    from seidart_gb300.solver import run_shot
    case = sy.electromag2_layers(nstep=60)
    g, m = case.grid, case.meta
    assert m["ids"].shape == (g.nz, g.nx) and m["table"].shape == (3, 6)
    assert np.array_equal(np.transpose(m["table"][m["ids"]], (2, 0, 1)), case.planes)
    a = run_shot(g, case.planes, case.profiles, case.src_ijk, case.srcfn, case.rec_ijk)
    b = run_shot(g, None, case.profiles, case.src_ijk, case.srcfn, case.rec_ijk, ids=m["ids"], table=m["table"])
    assert np.array_equal(a, b)
