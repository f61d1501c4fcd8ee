"""run_shots: many shots through two handles in turn (host work of one shot
overlapping the previous shot's run) give each shot the traces run_shot
gives it alone, bit for bit -- also across a change of grid, of step count
and of the kind, where the handles are replaced."""
import numpy as np
import pytest

from seidart_gb300 import ELECTROMAG2, SEISMIC2, synthetic as sy
from seidart_gb300.solver import run_shot, run_shots

pytestmark = pytest.mark.gpu


def _shot(case, src=None):
    return (case.grid, case.planes, case.profiles, src or case.src_ijk, case.srcfn, case.rec_ijk)


def test_run_shots_matches_run_shot(gpu):
    a = sy.small_case(ELECTROMAG2, seed=3, nx=60, nz=44, npml=6, nstep=90, nrec=6)
    b = sy.small_case(ELECTROMAG2, seed=4, nx=72, nz=40, npml=6, nstep=70, nrec=5)
    c = sy.small_case(SEISMIC2, seed=5, nx=56, nz=48, npml=6, nstep=80, nrec=7)
    i, j, k = a.src_ijk
    shots = [_shot(a), _shot(a, (i + 3, j, k)), _shot(a, (i - 4, j, k + 2)), _shot(b), _shot(c), _shot(c),
             _shot(a)]
    got = list(run_shots(shots))
    assert len(got) == len(shots)
    for q, (sh, tr) in enumerate(zip(shots, got)):
        ref = run_shot(*sh)
        assert tr.shape == ref.shape and np.array_equal(tr, ref), q
    assert not np.array_equal(got[0], got[1])  # the sources differ


def test_pipeline_keeps_its_handles_between_runs(gpu):
    from seidart_gb300.solver import ShotPipeline
    a = sy.small_case(ELECTROMAG2, seed=6, nx=52, nz=40, npml=5, nstep=60, nrec=4)
    i, j, k = a.src_ijk
    shots = [_shot(a, (i + d, j, k)) for d in range(-2, 3)]
    with ShotPipeline() as p:
        first = list(p.run(shots[:2]))
        handles = list(p.solvers)
        second = list(p.run(shots[2:]))
        assert p.solvers[0] is handles[0] and p.solvers[1] is handles[1]
    for sh, tr in zip(shots, first + second):
        assert np.array_equal(tr, run_shot(*sh))
