"""GPU parity: the CUDA kernels (through the C ABI) against the FP64 oracle.

Every case runs the same seeded model, CPML profiles, source and receivers on
both sides and compares receiver traces, final fields and the CPML memory
variables.  Tolerance (FP32 kernels vs FP64 oracle): relative L2 <= 1e-5 on
traces and fields, 1e-4 on memory variables (which are small differences of
nearly equal numbers at the strip edges).
"""
import numpy as np
import pytest

from helpers import make_solver, rel_l2, run_oracle
from oracle import OracleState
from seidart_gb300 import ELECTROMAG2, ELECTROMAG25, SEISMIC2, SEISMIC25, KIND_NAMES
from seidart_gb300 import synthetic as sy
from seidart_gb300.solver import FIELDS, MEMORY

pytestmark = pytest.mark.gpu

TOL_TRACE = 1e-5
TOL_FIELD = 1e-5
TOL_MEM = 1e-4

CASES = [
    # kind, seed, nx, nz, ny, npml, nstep, flags (1 = two-pass form of the 2-D
    # kinds, 2 = one launch per step; electromag2 with 0 runs on chip)
    (ELECTROMAG2, 0, 45, 37, 1, 5, 160, 0),
    (ELECTROMAG2, 0, 45, 37, 1, 5, 160, 1),
    (ELECTROMAG2, 0, 45, 37, 1, 5, 160, 2),
    (ELECTROMAG2, 1, 70, 52, 1, 8, 100, 0),
    (ELECTROMAG2, 1, 70, 52, 1, 8, 100, 1),
    (ELECTROMAG2, 1, 70, 52, 1, 8, 100, 2),
    (ELECTROMAG2, 3, 97, 67, 1, 9, 75, 0),
    (ELECTROMAG2, 4, 301, 203, 1, 12, 260, 0),  # odd sizes: partial float4 groups, ragged last tiles
    (ELECTROMAG2, 4, 301, 203, 1, 12, 260, 2),
    (SEISMIC2, 0, 45, 37, 1, 5, 160, 0),
    (SEISMIC2, 0, 45, 37, 1, 5, 160, 1),
    (SEISMIC2, 1, 70, 52, 1, 8, 100, 0),
    (SEISMIC2, 1, 70, 52, 1, 8, 100, 1),
    (SEISMIC2, 2, 30, 44, 1, 5, 120, 0),   # NZ > NX: b_x_half read past the x axis
    (SEISMIC2, 2, 30, 44, 1, 5, 120, 1),
    (SEISMIC2, 3, 97, 67, 1, 9, 75, 0),
    (SEISMIC25, 0, 37, 29, 21, 5, 90, 0),
    (SEISMIC25, 1, 50, 34, 26, 7, 70, 0),
    (ELECTROMAG25, 0, 37, 29, 21, 5, 90, 0),
    (ELECTROMAG25, 1, 50, 34, 26, 7, 70, 0),
    (SEISMIC25, 2, 100, 30, 20, 5, 60, 0),     # wide enough for blocks of interior columns only
    (ELECTROMAG25, 2, 100, 30, 20, 5, 60, 0),
]


def _ids(c):
    return f"{KIND_NAMES[c[0]]}-s{c[1]}-{c[2]}x{c[3]}" + (f"x{c[4]}" if c[4] > 1 else "") + \
        {0: "", 1: "-twopass", 2: "-streaming"}[c[7]]


@pytest.mark.parametrize("spec", CASES, ids=[_ids(c) for c in CASES])
def test_parity_against_oracle(gpu, spec):
    kind, seed, nx, nz, ny, npml, nstep, flags = spec
    case = sy.small_case(kind, seed=seed, nx=nx, nz=nz, ny=max(ny, 2) if ny > 1 else 24, npml=npml, nstep=nstep)
    st, tr_ref, _, blew = run_oracle(case)
    assert not blew
    with make_solver(case, flags=flags) as s:
        # uneven chunks: graph-captured 32-step blocks plus remainders
        done = 0
        for n in (37, 64, nstep):
            n = min(n, nstep - done)
            if n > 0:
                s.run(n)
                done += n
        step, norm = s.status()
        assert step == nstep
        tr = s.traces()
        assert np.all(np.isfinite(tr))
        e_tr = rel_l2(tr, tr_ref)
        assert e_tr <= TOL_TRACE, f"traces rel L2 {e_tr:.3e}"
        for q, name in enumerate(FIELDS[kind]):
            e = rel_l2(s.field(name), st.fields[q])
            assert e <= TOL_FIELD, f"field {name} rel L2 {e:.3e}"
        for q, name in enumerate(MEMORY[kind]):
            ref = st.memory[q]
            e = rel_l2(s.memory(name), ref, floor=1e-30)
            assert e <= TOL_MEM, f"memory {name} rel L2 {e:.3e}"
        # the device norm monitor sees the same magnitude as the oracle's
        assert norm > 0


@pytest.mark.parametrize("kind", [ELECTROMAG2, SEISMIC2])
def test_initial_conditions(gpu, kind):
    """A nonzero initial field (the initialcondition*.dat inputs) evolves like the oracle's."""
    case = sy.small_case(kind, seed=7, nx=41, nz=33, npml=5, nstep=80)
    rng = np.random.default_rng(3)
    st = OracleState.zeros(kind, case.grid.shape)
    init = np.zeros(case.grid.shape)
    init[8:-8, 8:-8] = rng.standard_normal((case.grid.nz - 16, case.grid.nx - 16))
    init *= 1e-6
    st.fields[0] = init.astype(np.float32).astype(np.float64)
    st, tr_ref, _, _ = run_oracle(case, state=st)
    with make_solver(case) as s:
        s.set_field(FIELDS[kind][0], init.astype(np.float32))
        s.run(case.nstep)
        s.status()
        assert rel_l2(s.traces(), tr_ref) <= TOL_TRACE
        assert rel_l2(s.field(0), st.fields[0]) <= TOL_FIELD


def test_reset_reproduces(gpu):
    case = sy.small_case(ELECTROMAG2, seed=4, nx=40, nz=36, npml=5, nstep=70)
    with make_solver(case) as s:
        s.run(case.nstep)
        a = s.traces().copy()
        s.reset()
        s.run(case.nstep)
        b = s.traces()
        assert np.array_equal(a, b)


def test_unstable_reported(gpu):
    """dt far above the CFL limit: the run completes and the status reports the
    blow-up instead of stopping the process (host-made bad input; no fault)."""
    from seidart_gb300 import UnstableError
    case = sy.small_case(SEISMIC2, seed=5, nx=40, nz=36, npml=5, nstep=400)
    case.grid.dt *= 4.0
    with make_solver(case) as s:
        s.run(case.nstep)
        with pytest.raises(UnstableError):
            s.status()


def test_run_past_source_length_rejected(gpu):
    from seidart_gb300 import SfdError
    case = sy.small_case(ELECTROMAG2, seed=6, nx=40, nz=36, npml=5, nstep=20)
    with make_solver(case) as s:
        s.run(20)
        with pytest.raises(SfdError):
            s.run(1)
