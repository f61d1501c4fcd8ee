"""GPU parity of the seismic physics options against the FP64 oracle.

The options, each a flag of the C ABI that the oracle takes too:

* legacy quirks (SFD_FLAG_LEGACY_QUIRKS) or, by default, corrected physics:
  seismic2's second stress loop with its own CPML memory, b_x_half(i), vx over
  the averaged density; seismic25's Voigt coefficient pairs of c16 and c45;
* the density method (arithmetic, none, geometric, harmonic: the driver's
  density_method, src/seidart/routines/classes.py:311);
* a moment-tensor (stress) source, sigma_ij += f_ij(t) dt at the source cell
  (the driver's seismicsource{xx,..,yz}.dat, sourcefunction.py:354-372).

Every execution form runs them: seismic2 on chip, one launch per step, two
kernels per step and in a batch; seismic25 y-marching.  Tolerances as in
test_parity_gpu.py: relative L2 <= 1e-5 on traces and fields, 1e-4 on the
CPML memory variables.
"""
import dataclasses

import numpy as np
import pytest

from golden.make_golden import stress_source
from helpers import make_solver, rel_l2, run_oracle
from seidart_gb300 import SEISMIC2, SEISMIC25
from seidart_gb300 import synthetic as sy
from seidart_gb300.batch import Batch
from seidart_gb300.solver import FIELDS, FLAG_STREAMING, FLAG_TWO_PASS, MEMORY

pytestmark = pytest.mark.gpu

OPTIONS = [  # legacy, density, stress source
    (False, "arithmetic", False),
    (True, "arithmetic", False),
    (False, "none", True),
    (False, "geometric", False),
    (False, "harmonic", True),
    (True, "geometric", True),
]
FORMS = {"onchip": 0, "streaming": FLAG_STREAMING, "twopass": FLAG_TWO_PASS}


def _case(kind, seed, legacy, density, stress, **kw):
    c = sy.small_case(kind, seed=seed, **kw)
    c.legacy, c.density = legacy, density
    if stress:
        c.stress_srcfn = stress_source(kind, 1e6 * c.srcfn[0])
    return c


def _check(case, s, mem=True):
    st, ref, _, blew = run_oracle(case)
    assert not blew
    e = rel_l2(s.traces(), ref)
    assert e <= 1e-5, f"traces rel L2 {e:.2e}"
    for q, name in enumerate(FIELDS[case.grid.kind]):
        e = rel_l2(s.field(name), st.fields[q])
        assert e <= 1e-5, f"{name}: rel L2 {e:.2e}"
    if mem:
        for q, name in enumerate(MEMORY[case.grid.kind]):
            ref_m = st.memory[q]
            if np.linalg.norm(ref_m) == 0.0:
                assert np.linalg.norm(s.memory(name)) == 0.0, name
                continue
            e = rel_l2(s.memory(name), ref_m)
            assert e <= 1e-4, f"{name}: rel L2 {e:.2e}"


@pytest.mark.parametrize("form", list(FORMS))
@pytest.mark.parametrize("legacy,density,stress", OPTIONS,
                         ids=[f"{'legacy' if o[0] else 'corrected'}-{o[1]}{'-stress' if o[2] else ''}" for o in OPTIONS])
def test_seismic2_options(gpu, form, legacy, density, stress):
    case = _case(SEISMIC2, 21, legacy, density, stress, nx=53, nz=47, npml=6, nstep=150)
    with make_solver(case, flags=FORMS[form]) as s:
        assert (s.on_chip() is not None) == (form == "onchip")
        s.run(61)
        s.run(case.nstep - 61)
        s.status()
        _check(case, s)


def test_seismic2_nz_above_nx_corrected(gpu):
    """NZ > NX: legacy loop 1 reads b_x_half past the x axis; the corrected
    loop reads b_x_half(i) -- on chip and in two-pass form."""
    for flags in (0, FLAG_TWO_PASS):
        case = _case(SEISMIC2, 22, False, "arithmetic", True, nx=30, nz=46, npml=5, nstep=120)
        with make_solver(case, flags=flags) as s:
            s.run(case.nstep)
            s.status()
            _check(case, s)


@pytest.mark.parametrize("legacy,density,stress", OPTIONS[:5],
                         ids=[f"{'legacy' if o[0] else 'corrected'}-{o[1]}{'-stress' if o[2] else ''}" for o in OPTIONS[:5]])
def test_seismic25_options(gpu, legacy, density, stress):
    case = _case(SEISMIC25, 23, legacy, density, stress, nx=37, nz=31, ny=23, npml=5, nstep=80)
    with make_solver(case) as s:
        s.run(33)
        s.run(case.nstep - 33)
        s.status()
        _check(case, s)


def test_batch_with_options(gpu):
    """A batch of seismic2 models with different options (each handle keeps
    its own) and an electromag2 shot, against the oracle."""
    cases = [_case(SEISMIC2, 24 + q, *OPTIONS[q], nx=41 + 6 * q, nz=50 - 3 * q, npml=6, nstep=100)
             for q in range(len(OPTIONS))]
    cases.append(sy.small_case(sy.ELECTROMAG2, seed=30, nx=46, nz=38, npml=5, nstep=100))
    solvers = [make_solver(c) for c in cases]
    b = Batch(solvers)
    try:
        b.run(41)
        b.run(59)
        b.status()
        for c, s in zip(cases, solvers):
            _check(c, s, mem=False)
    finally:
        b.close()
        for s in solvers:
            s.close()


def test_config2_explosive_source_short(gpu):
    """The seismic25 workload's explosive source (equal normal stresses) on a
    reduced grid of the same model generator, against the oracle."""
    case = sy.seismic25_ice(nstep=120, nx=60, ny=20, nz=40, c=6)
    assert case.stress_srcfn is not None and not case.srcfn.any()
    with make_solver(case) as s:
        s.run(case.nstep)
        s.status()
        st, ref, _, _ = run_oracle(case)
        assert rel_l2(s.traces(), ref) <= 1e-5
        assert np.abs(ref).max() > 0


def test_stress_source_must_share_the_force_source_cell(gpu):
    from seidart_gb300._lib import SfdError
    case = _case(SEISMIC2, 25, False, "arithmetic", True, nx=40, nz=36, npml=5, nstep=30)
    with make_solver(case) as s:
        i, j, k = case.src_ijk
        with pytest.raises(SfdError):
            s.set_stress_source((i + 1, j, k), case.stress_srcfn)
        with pytest.raises(SfdError):
            s.set_source((i, j, k + 1), case.srcfn)
        s.set_stress_source(case.src_ijk, None)  # removed: the force source may move
        s.set_source((i, j, k + 1), case.srcfn)
        s.run(case.nstep)
        s.status()
        moved = dataclasses.replace(case, src_ijk=(i, j, k + 1), stress_srcfn=None)
        _, ref, _, _ = run_oracle(moved)
        assert rel_l2(s.traces(), ref) <= 1e-5


def test_options_rejected_for_em_kinds(gpu):
    from seidart_gb300.solver import FDTDSolver
    case = sy.small_case(sy.ELECTROMAG2, seed=31, nx=40, nz=36, npml=5, nstep=20)
    with pytest.raises(ValueError):
        FDTDSolver(case.grid, case.nstep, 3, legacy=True)
    from seidart_gb300._lib import SfdError
    with pytest.raises(SfdError):
        FDTDSolver(case.grid, case.nstep, 3, flags=4)
