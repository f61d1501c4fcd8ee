"""GPU edge cases against the FP64 oracle: the smallest grid a CPML width
allows, receivers on the outer Dirichlet planes and corners and several at
one cell, no receivers at all, sources at the extreme cells the library
accepts, zero-step runs and runs past the source length.  Every step form
of the 2-D kinds (on chip, one launch per step, two-pass) is covered where
it applies."""
import dataclasses

import numpy as np
import pytest

from helpers import make_solver, rel_l2, run_oracle
from seidart_gb300 import ELECTROMAG2, ELECTROMAG25, SEISMIC2, SEISMIC25, synthetic as sy
from seidart_gb300._lib import SfdError
from seidart_gb300.solver import FIELDS, FLAG_STREAMING, FLAG_TWO_PASS

pytestmark = pytest.mark.gpu

TOL = 1e-5
KINDS = [ELECTROMAG2, SEISMIC2, SEISMIC25, ELECTROMAG25]
FORMS = {ELECTROMAG2: [0, FLAG_STREAMING, FLAG_TWO_PASS], SEISMIC2: [0, FLAG_STREAMING, FLAG_TWO_PASS],
         SEISMIC25: [0], ELECTROMAG25: [0]}


def _three(kind):
    return kind in (SEISMIC25, ELECTROMAG25)


def _check(case, flags=0, tol_field=TOL):
    st, ref, _, blew = run_oracle(case)
    assert not blew
    with make_solver(case, flags=flags) as s:
        s.run(case.nstep)
        s.status()
        tr = s.traces()
        if case.rec_ijk.shape[0]:
            assert rel_l2(tr, ref) <= TOL, rel_l2(tr, ref)
        for q, name in enumerate(FIELDS[case.grid.kind]):
            assert rel_l2(s.field(name), st.fields[q]) <= tol_field, name


@pytest.mark.parametrize("kind", KINDS)
def test_smallest_grid(gpu, kind):
    """nx = nz (= ny) = 2 npml + 2, the smallest grid sfd_create accepts."""
    npml = 5
    n = 2 * npml + 2
    case = sy.small_case(kind, seed=11, nx=n, nz=n, ny=n, npml=npml, nstep=60, nrec=4)
    for flags in FORMS[kind]:
        _check(case, flags)


@pytest.mark.parametrize("kind", KINDS)
def test_receivers_on_planes_corners_and_shared_cells(gpu, kind):
    case = sy.small_case(kind, seed=13, nx=40, nz=34, ny=18, npml=5, nstep=80, nrec=4)
    g = case.grid
    j = g.ny // 2 if _three(kind) else 0
    jm = g.ny - 1 if _three(kind) else 0
    cells = [(0, 0, 0), (g.nx - 1, jm, g.nz - 1), (0, j, g.nz - 1), (g.nx - 1, 0, 0), (g.nx // 2, j, 0),
             (5, j, 7), (5, j, 7), (g.nx - 2, j, g.nz - 2)]
    case = dataclasses.replace(case, rec_ijk=np.array(cells, dtype=np.int32))
    for flags in FORMS[kind]:
        _check(case, flags)


@pytest.mark.parametrize("kind", KINDS)
def test_no_receivers(gpu, kind):
    case = sy.small_case(kind, seed=17, nx=36, nz=30, ny=16, npml=5, nstep=50, nrec=0)
    assert case.rec_ijk.shape[0] == 0
    for flags in FORMS[kind]:
        _check(case, flags)
        with make_solver(case, flags=flags) as s:
            s.run(case.nstep)
            s.status()
            assert s.traces().shape == (case.nstep, 3 if _three(kind) else 2, 0)


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("corner", ["low", "high"])
def test_source_at_extreme_cells(gpu, kind, corner):
    """The source may sit at i, k (and j) = 1 up to n - 3 (two planes off
    the far edge); the near edge's cell 1 is inside the CPML strip."""
    case = sy.small_case(kind, seed=19, nx=38, nz=32, ny=16, npml=5, nstep=70, nrec=6)
    g = case.grid
    if corner == "low":
        src = (1, 1 if _three(kind) else 0, 1)
    else:
        src = (g.nx - 3, g.ny - 3 if _three(kind) else 0, g.nz - 3)
    case = dataclasses.replace(case, src_ijk=src)
    for flags in FORMS[kind]:
        # a source in the CPML corner leaves a field whose norm is a small
        # fraction of its peak: FP32 rounding relative to it reaches 1.5e-5
        _check(case, flags, tol_field=5e-5)


@pytest.mark.parametrize("kind", KINDS)
def test_zero_step_and_overlong_runs(gpu, kind):
    case = sy.small_case(kind, seed=23, nx=30, nz=28, ny=14, npml=4, nstep=20, nrec=3)
    with make_solver(case) as s:
        s.run(0)
        assert s.status()[0] == 0
        s.run(case.nstep)
        assert s.status()[0] == case.nstep
        with pytest.raises(SfdError, match="exceeds"):
            s.run(1)
        with pytest.raises(SfdError):
            s.set_source((0, 0, 0), case.srcfn)  # outside the accepted cells
