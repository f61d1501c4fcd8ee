"""GPU: seismic2 runs that keep the whole state on chip (one launch per run,
one CTA per tile, halo exchange through tagged edge words) against the same
runs with one launch per step, and against the FP64 oracle.

The per-cell arithmetic is the same in both forms; the compiler may fuse
multiply-adds differently in the two kernels, so they are compared to
relative L2 <= 1e-5 (the oracle bar), not bit for bit.
"""
import numpy as np
import pytest

from helpers import make_solver, rel_l2, run_oracle
from seidart_gb300 import SEISMIC2
from seidart_gb300 import synthetic as sy
from seidart_gb300.solver import FIELDS, FLAG_STREAMING, FLAG_TWO_PASS, MEMORY

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _compare(case, chunks):
    with make_solver(case) as a, make_solver(case, flags=FLAG_STREAMING) as b:
        assert a.on_chip() is not None, "grid expected to fit on chip"
        assert b.on_chip() is None
        for n in chunks:
            a.run(n)
            b.run(n)
        sa, sb = a.status(), b.status()
        assert sa[0] == sb[0]
        assert abs(sa[1] - sb[1]) <= 1e-5 * max(sb[1], 1e-30)
        e = rel_l2(a.traces(), b.traces())
        assert e <= TOL, f"traces rel L2 {e:.3e}"
        for name in FIELDS[SEISMIC2]:
            e = rel_l2(a.field(name), b.field(name))
            assert e <= TOL, f"{name} rel L2 {e:.3e}"
        for name in MEMORY[SEISMIC2]:
            e = rel_l2(a.memory(name), b.memory(name), floor=1e-30)
            assert e <= 10 * TOL, f"{name} rel L2 {e:.3e}"
        return a.on_chip()


def test_config0_grid_on_chip_matches_streaming(gpu):
    """The 440 x 240 firn/ice model (config 0), uneven chunks (a 1-step run included)."""
    case = sy.seismic2_firn_ice(nstep=150)
    tiles = _compare(case, (1, 40, 61, 48))
    assert tiles[0] > 100 and tiles[1] > 1


@pytest.mark.parametrize("seed,nx,nz,npml", [(2, 61, 47, 6), (3, 37, 90, 5), (4, 130, 33, 8)])
def test_small_grids_with_attenuation(gpu, seed, nx, nz, npml):
    """Odd sizes, NZ > NX, per-cell material noise and attenuation (small_case)."""
    case = sy.small_case(SEISMIC2, seed=seed, nx=nx, nz=nz, npml=npml, nstep=120)
    _compare(case, (57, 63))


def test_matches_oracle(gpu):
    case = sy.small_case(SEISMIC2, seed=9, nx=72, nz=58, npml=7, nstep=160)
    st, tr, _, blew = run_oracle(case)
    assert not blew
    with make_solver(case) as s:
        assert s.on_chip() is not None
        s.run(90)
        s.run(70)
        s.status()
        assert rel_l2(s.traces(), tr) <= TOL
        for q, name in enumerate(FIELDS[SEISMIC2]):
            assert rel_l2(s.field(name), st.fields[q]) <= TOL, name
        for q, name in enumerate(MEMORY[SEISMIC2]):
            assert rel_l2(s.memory(name), st.memory[q], floor=1e-30) <= 1e-4, name


def test_receivers_on_every_tile_edge(gpu):
    """Receivers along whole rows and columns cross every tile edge; the source
    sits next to the domain edge."""
    case = sy.small_case(SEISMIC2, seed=7, nx=150, nz=96, npml=8, nstep=80)
    NX, NZ = case.grid.nx, case.grid.nz
    rows = [0, 1, 17, 48, NZ - 2, NZ - 1]
    cols = [0, 3, 4, 75, NX - 2, NX - 1]
    rec = [(x, 0, z) for z in rows for x in range(NX)] + [(x, 0, z) for x in cols for z in range(NZ)]
    case.rec_ijk = np.array(rec, dtype=np.int32)
    case.src_ijk = (2, 0, NZ // 2)
    _compare(case, (80,))


def test_two_pass_handle_never_on_chip(gpu):
    case = sy.small_case(SEISMIC2, seed=5, nx=61, nz=47, npml=6, nstep=10)
    with make_solver(case, flags=FLAG_TWO_PASS) as s:
        assert s.on_chip() is None
