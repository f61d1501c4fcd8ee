"""GPU tests of the batched persistent launch: every model of a mixed batch
(electromag2 shots and seismic2 models of uneven sizes) gives the same traces
and fields as its own single run, and as the FP64 oracle.

The batch runs the tile bodies of the one-launch-per-step kernels, so the
arithmetic per cell is the same; the compiler may still fuse multiply-adds
differently in the two kernels, so batch and single runs are compared to
relative L2 <= 1e-6 (ten times tighter than the bar against the oracle)
rather than bit for bit."""
import numpy as np
import pytest

from helpers import make_solver, rel_l2, run_oracle
from seidart_gb300 import ELECTROMAG2, SEISMIC2
from seidart_gb300 import synthetic as sy
from seidart_gb300.batch import Batch, autotune
from seidart_gb300.solver import FLAG_STREAMING

pytestmark = pytest.mark.gpu


def _mixed_cases():
    cases = [sy.small_case(ELECTROMAG2, seed=20 + q, nx=45 + 7 * q, nz=37 + 3 * q, npml=5, nstep=90) for q in range(3)]
    cases += [sy.small_case(SEISMIC2, seed=30 + q, nx=38 + 11 * q, nz=52 - 5 * q, npml=6, nstep=90) for q in range(3)]
    return cases


@pytest.mark.parametrize("zb,bps", [(1, 3), (2, 3), (4, 2)])
def test_batch_matches_oracle_and_single_runs(gpu, zb, bps):
    cases = _mixed_cases()
    solvers = [make_solver(c) for c in cases]
    b = Batch(solvers)
    b.set_tiling(zb, bps)
    b.run(37)   # odd: the ping-pong parity differs between the two runs
    b.run(53)
    b.status()
    for c, s in zip(cases, solvers):
        _, ref, _, _ = run_oracle(c)
        tr = s.traces()
        assert rel_l2(tr, ref) <= 1e-5
        # the batch runs the tiles of the one-launch-per-step form
        with make_solver(c, flags=FLAG_STREAMING) as one:
            one.run(c.nstep)
            one.status()
            e = rel_l2(tr, one.traces())
            assert e <= 1e-6, f"traces: batched vs single rel L2 {e:.2e}"
            for name in ("Ex", "Ez", "Hy") if c.grid.kind == ELECTROMAG2 else ("vx", "vz", "sigmaxz"):
                e = rel_l2(s.field(name), one.field(name))
                assert e <= 1e-6, f"{name}: batched vs single rel L2 {e:.2e}"
    b.close()
    for s in solvers:
        s.close()


def test_autotune_picks_a_candidate(gpu, tmp_path, monkeypatch):
    monkeypatch.setenv("SEIDART_GB300_TUNING", str(tmp_path / "tuning.json"))
    cases = _mixed_cases()[:4]
    solvers = [make_solver(c) for c in cases]
    b = Batch(solvers)
    res = autotune(b, steps=4)
    from seidart_gb300.batch import CANDIDATES
    assert res["timings"] and res["tiling"] in CANDIDATES
    again = autotune(b, steps=4)
    assert again["cached"] and again["tiling"] == res["tiling"]
    # after autotuning the models are back at step 0 and run correctly
    b.run(cases[0].nstep)
    b.status()
    _, ref, _, _ = run_oracle(cases[0])
    assert rel_l2(solvers[0].traces(), ref) <= 1e-5
    b.close()


def test_shared_model_batch_matches_separate_models(gpu):
    """Shots that share one model's coefficients (interleaved batch tiles) give
    the same traces as shots with their own copies."""
    from seidart_gb300.solver import FDTDSolver
    base = sy.small_case(ELECTROMAG2, seed=70, nx=70, nz=44, npml=6, nstep=64)
    srcs = [(10 + 9 * q, 0, 12) for q in range(5)]
    own, shared = [], []
    for q, src in enumerate(srcs):
        a = FDTDSolver(base.grid, base.nstep, len(base.rec_ijk))
        a.set_model(base.planes)
        b = FDTDSolver(base.grid, base.nstep, len(base.rec_ijk))
        if shared:
            b.share_model(shared[0])
        else:
            b.set_model(base.planes)
        for s in (a, b):
            s.set_cpml(base.profiles)
            s.set_source(src, base.srcfn)
            s.set_receivers(base.rec_ijk)
        own.append(a)
        shared.append(b)
    for group in (own, shared):
        bt = Batch(group)
        bt.run(base.nstep)
        bt.status()
        bt.close()
    for a, b in zip(own, shared):
        assert np.array_equal(a.traces(), b.traces())
    for s in own + shared:
        s.close()
