"""GPU: electromag2c (complex permittivities, electromagfdtd.f95:329-616)
against the FP64 oracle, and against electromag2 when the imaginary parts
vanish.  FP32 on the GPU: relative L2 <= 1e-5 on traces and fields, <= 1e-4
on the CPML memory variables (as for the real solvers)."""
import numpy as np
import pytest

from helpers import make_solver, rel_l2, run_oracle
from seidart_gb300 import ELECTROMAG2, ELECTROMAG2C
from seidart_gb300 import synthetic as sy
from seidart_gb300.solver import FIELDS, FLAG_TWO_PASS, MEMORY, GridSpec

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed,nx,nz,nstep,chunks", [(1, 61, 47, 150, (150,)), (2, 37, 83, 140, (33, 70, 37)),
                                                     (3, 130, 64, 200, (1, 199))])
def test_matches_oracle(gpu, seed, nx, nz, nstep, chunks):
    case = sy.small_case(ELECTROMAG2C, seed=seed, nx=nx, nz=nz, npml=6, nstep=nstep)
    st, tr, _, blew = run_oracle(case)
    assert not blew
    assert np.abs(tr[:, 1::2]).max() > 1e-3 * np.abs(tr[:, 0::2]).max()  # the imaginary parts matter
    with make_solver(case) as s:
        for n in chunks:
            s.run(n)
        s.status()
        e = rel_l2(s.traces(), tr)
        assert e <= 1e-5, f"traces rel L2 {e:.3e}"
        for q, name in enumerate(FIELDS[ELECTROMAG2C]):
            e = rel_l2(s.field(name), st.fields[q])
            assert e <= 1e-5, f"{name} rel L2 {e:.3e}"
        for q, name in enumerate(MEMORY[ELECTROMAG2C]):
            e = rel_l2(s.memory(name), st.memory[q], floor=1e-30)
            assert e <= 1e-4, f"{name} rel L2 {e:.3e}"
        c = s.complex_traces()
        assert c.shape == (nstep, 2, len(case.rec_ijk))
        assert np.array_equal(c.real, s.traces()[:, 0::2])


def test_real_permittivity_is_electromag2(gpu):
    """Zero imaginary parts: the real parts follow the two-pass electromag2
    kernels.  The complex multiply-adds round (and fuse) differently from the
    real ones, so the two agree to the oracle bar, not bit for bit."""
    c = sy.small_case(ELECTROMAG2C, seed=4, nx=50, nz=44, npml=5, nstep=120)
    c.planes[[1, 3, 5]] = 0.0
    r = sy.small_case(ELECTROMAG2, seed=4, nx=50, nz=44, npml=5, nstep=120)
    g = c.grid
    r.grid = GridSpec(ELECTROMAG2, g.nx, g.nz, g.dx, g.dz, g.dt, g.npml)
    r.planes = np.ascontiguousarray(c.planes[[0, 2, 4, 6, 7, 8]])
    r.profiles, r.srcfn, r.src_ijk, r.rec_ijk = c.profiles, c.srcfn, c.src_ijk, c.rec_ijk
    with make_solver(c) as a, make_solver(r, flags=FLAG_TWO_PASS) as b:
        a.run(120)
        b.run(120)
        a.status()
        b.status()
        tr_a, tr_b = a.traces(), b.traces()
        assert not tr_a[:, 1::2].any()
        assert rel_l2(tr_a[:, 0::2], tr_b) <= 1e-5
        for name in ("Ex", "Ez", "Hy"):
            assert rel_l2(a.field(name + "_re"), b.field(name)) <= 1e-5
            assert not a.field(name + "_im").any()


def test_bad_inputs_are_rejected(gpu):
    from seidart_gb300._lib import SfdError
    case = sy.small_case(ELECTROMAG2C, seed=5, nx=30, nz=30, npml=4, nstep=10)
    with make_solver(case) as s:
        bad = case.planes.copy()
        bad[0, 3, 3] = -1.0  # eps11 real part
        bad[2, 3, 3] = 0.0
        with pytest.raises(SfdError):
            s.set_model(bad)
        with pytest.raises(SfdError):
            s.set_source(case.src_ijk, np.zeros((4, 10)))  # two components (x, z)
