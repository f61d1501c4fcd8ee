"""seismic2 one launch per step (the single-pass tiles) on grids too large to
run on chip, against the FP64 oracle: the default physics, the legacy
quirks, a density method with a moment-tensor source, NZ > NX, and
attenuation; and against the two-pass form of the same handle."""
import numpy as np
import pytest

from helpers import make_solver, rel_l2, run_oracle
from seidart_gb300 import SEISMIC2, synthetic as sy
from seidart_gb300.solver import FLAG_STREAMING, FLAG_TWO_PASS

pytestmark = pytest.mark.gpu


def _case(seed=21, nx=1310, nz=530, **kw):
    c = sy.small_case(SEISMIC2, seed=seed, nx=nx, nz=nz, npml=10, nstep=110, nrec=12)
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def _run(case, flags):
    with make_solver(case, flags=flags) as s:
        assert s.on_chip() is None
        s.run(case.nstep)
        s.status()
        return s.traces(), [s.field(n) for n in ("vx", "vz", "sigmaxx", "sigmazz", "sigmaxz")]


@pytest.mark.parametrize("variant", ["default", "legacy", "harmonic+stress", "nz>nx"])
def test_large_grid_matches_oracle(gpu, variant):
    if variant == "legacy":
        case = _case(legacy=True)
    elif variant == "harmonic+stress":
        t = np.arange(110)
        w = 3e5 * np.exp(-((t - 20) / 6.0) ** 2)
        case = _case(seed=22, density="harmonic", stress_srcfn=np.stack([w, 0.5 * w, 0.2 * w]))
    elif variant == "nz>nx":
        case = _case(seed=23, nx=700, nz=1200)
    else:
        case = _case()
    tr, fields = _run(case, FLAG_STREAMING)
    st, ref, _, blew = run_oracle(case)
    assert not blew
    assert rel_l2(tr, ref) <= 1e-5
    for q, f in enumerate(fields):
        assert rel_l2(f, st.fields[q]) <= 1e-5, q


def test_large_grid_agrees_with_two_pass(gpu):
    case = _case(seed=24)
    ta, fa = _run(case, FLAG_STREAMING)
    tb, fb = _run(case, FLAG_TWO_PASS)
    assert rel_l2(ta, tb) <= 1e-6
    for a, b in zip(fa, fb):
        assert rel_l2(a, b) <= 1e-6


def test_large_grid_graph_chunks_and_split_runs(gpu):
    """Runs split across the 32-step graph chunks and odd lengths."""
    case = _case(seed=25)
    with make_solver(case, flags=FLAG_STREAMING) as s:
        for n in (1, 33, 7, 64, 5):
            s.run(n)
        s.status()
        tr = s.traces()
    _, ref, _, _ = run_oracle(case)
    assert rel_l2(tr, ref) <= 1e-5
