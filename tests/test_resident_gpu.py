"""GPU: electromag2 runs that keep the whole state on chip (one launch per
run, one CTA per tile) against the same runs with one launch per step.

Both forms perform the same FP32 arithmetic per cell; the compiler may fuse
multiply-adds differently in the two kernels, so they are compared to
relative L2 <= 1e-5, the bar both meet against the FP64 oracle, rather than
bit for bit.  Parity of the on-chip form with
the FP64 oracle is in test_parity_gpu (flags 0).
"""
import numpy as np
import pytest

from helpers import make_solver, rel_l2
from seidart_gb300 import ELECTROMAG2
from seidart_gb300 import synthetic as sy
from seidart_gb300.solver import FIELDS, FLAG_STREAMING, MEMORY, FLAG_TWO_PASS

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
        for name in FIELDS[ELECTROMAG2]:
            e = rel_l2(a.field(name), b.field(name))
            assert e <= TOL, f"{name} rel L2 {e:.3e}"
        for name in MEMORY[ELECTROMAG2]:
            e = rel_l2(a.memory(name), b.memory(name), floor=1e-30)
            assert e <= 10 * TOL, f"{name} rel L2 {e:.3e}"
        return a.on_chip()


def test_headline_grid_on_chip_matches_streaming(gpu):
    """The 1040 x 540 layered model, uneven chunks (1-step run included)."""
    case = sy.electromag2_layers(nstep=120)
    tiles = _compare(case, (1, 31, 50, 38))
    assert tiles[0] * tiles[1] > 1


def test_many_small_tiles(gpu):
    """A small odd-sized grid cut into many tiles of a few cells each."""
    case = sy.small_case(ELECTROMAG2, seed=5, nx=61, nz=47, npml=6, nstep=140)
    _compare(case, (70, 70))


def test_two_pass_handle_never_on_chip(gpu):
    case = sy.small_case(ELECTROMAG2, seed=5, nx=61, nz=47, npml=6, nstep=10)
    with make_solver(case, flags=FLAG_TWO_PASS) as s:
        assert s.on_chip() is None


def test_receivers_on_every_tile_edge(gpu):
    """Receivers along whole rows and columns cross every tile edge; the source
    sits next to the domain edge."""
    case = sy.small_case(ELECTROMAG2, seed=7, nx=150, nz=96, npml=8, nstep=80)
    NX, NZ = case.grid.nx, case.grid.nz
    rows = [0, 1, 17, 48, NZ - 2, NZ - 1]
    cols = [0, 3, 4, 75, NX - 2, NX - 1]
    rec = [(x, 0, z) for z in rows for x in range(NX)] + [(x, 0, z) for x in cols for z in range(NZ)]
    case.rec_ijk = np.array(rec, dtype=np.int32)
    case.src_ijk = (2, 0, NZ // 2)
    _compare(case, (80,))


def test_many_receivers_in_one_tile(gpu):
    """400 receivers in a 20 x 20 block, more than a tile lists in shared memory."""
    case = sy.electromag2_layers(nstep=60)
    block = [(x, 0, z) for z in range(200, 220) for x in range(500, 520)]
    case.rec_ijk = np.array(block + [(30, 0, 30), (500, 0, 200)], dtype=np.int32)
    _compare(case, (60,))


@pytest.mark.parametrize("src", [(520, 0, 270), (37 * 4 + 2, 0, 300), (800, 0, 22 + 3 * 30)])
def test_source_inside_interior_tiles(gpu, src):
    """The headline grid's interior tiles hold three rows per thread and take
    the short update only; the source cell in one of them (mid-grid, and near
    the top and the right of the interior) is injected there, and receivers
    around it and on its row read the same fields as the per-step kernels."""
    case = sy.electromag2_layers(nstep=90)
    x, _, z = src
    rec = [(x + dx, 0, z + dz) for dx in (-5, 0, 3) for dz in (-4, 0, 2)] + [(q, 0, z) for q in range(30, 1000, 37)]
    case.rec_ijk = np.array(rec, dtype=np.int32)
    case.src_ijk = src
    _compare(case, (45, 45))
