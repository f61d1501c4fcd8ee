"""GPU tests of the input assembly on the device (sfd_set_source_wavelet,
sfd_set_cpml_params).

Each device-built input is checked against the host path it replaces: the
same model run with the source time functions of ``synthetic.wavelet`` (the
driver's wavelet, sourcefunction.py:25-57, pinned by the reference fixtures)
passed through ``set_source``, or with the profiles of ``cpml.axis_profile``
passed through ``set_cpml``.  The FP64 values differ only where the device's
exp and pow round differently from the host's, so after the FP32 cast the
inputs agree to an ulp and the runs to rounding.
"""
import numpy as np
import pytest

from helpers import make_solver, rel_l2
from seidart_gb300 import ELECTROMAG2, ELECTROMAG25, SEISMIC2, SEISMIC25, cpml as cp, synthetic as sy
from seidart_gb300._lib import SfdError
from seidart_gb300.solver import FLAG_LEGACY_QUIRKS, FIELDS

pytestmark = pytest.mark.gpu

TOL = 1e-6


def _case(kind, seed=3):
    three = kind in (SEISMIC25, ELECTROMAG25)
    return sy.small_case(kind, seed=seed, nx=44, nz=36, ny=20 if three else 1, npml=6, nstep=120, nrec=8)


def _run(s, case):
    s.run(case.nstep)
    s.status()
    return s.traces(), [s.field(f) for f in FIELDS[case.grid.kind]]


def _compare(a, b):
    (ta, fa), (tb, fb) = a, b
    assert np.abs(ta).max() > 0
    assert rel_l2(tb, ta) <= TOL, rel_l2(tb, ta)
    for x, y in zip(fa, fb):
        assert rel_l2(y, x, floor=1e-30) <= TOL


@pytest.mark.parametrize("kind", [ELECTROMAG2, SEISMIC2, SEISMIC25, ELECTROMAG25])
@pytest.mark.parametrize("stype", ["gaus0", "gaus1", "gaus2"])
def test_source_wavelet_matches_host_source(gpu, kind, stype):
    case = _case(kind)
    ncomp = case.srcfn.shape[0]
    comp = np.linspace(0.4, 1.0, ncomp) * np.where(np.arange(ncomp) % 2, -1.0, 1.0)
    amp, f0 = 2.5, 1.0 / (25 * case.grid.dt)
    t = np.arange(case.nstep) * case.grid.dt
    host = comp[:, None] * (amp * sy.wavelet(t, f0, stype))[None, :]
    out = []
    for device in (False, True):
        with make_solver(case) as s:
            if device:
                s.set_source_wavelet(case.src_ijk, f0, amp, comp, stype)
            else:
                s.set_source(case.src_ijk, host)
            out.append(_run(s, case))
    _compare(*out)


@pytest.mark.parametrize("kind", [SEISMIC2, SEISMIC25])
def test_stress_source_wavelet_matches_host(gpu, kind):
    case = _case(kind, seed=5)
    ns = 3 if kind == SEISMIC2 else 6
    mt = np.array([1.0, -0.5, 0.8, 0.3, -0.2, 0.6][:ns])
    f0 = 1.0 / (20 * case.grid.dt)
    t = np.arange(case.nstep) * case.grid.dt
    host = mt[:, None] * (1e3 * sy.wavelet(t, f0, "gaus1"))[None, :]
    out = []
    for device in (False, True):
        with make_solver(case) as s:
            if device:
                s.set_source_wavelet(case.src_ijk, f0, 1e3, mt, "gaus1", stress=True)
            else:
                s.set_stress_source(case.src_ijk, host)
            out.append(_run(s, case))
    _compare(*out)


@pytest.mark.parametrize("kind,mode,flags", [(ELECTROMAG2, "driver", 0), (ELECTROMAG2, "legacy", 0),
                                             (SEISMIC2, "driver", 0), (SEISMIC2, "legacy", FLAG_LEGACY_QUIRKS),
                                             (SEISMIC25, "driver", 0), (ELECTROMAG25, "legacy", 0)])
def test_cpml_params_match_host_profiles(gpu, kind, mode, flags):
    case = _case(kind, seed=7)
    g = case.grid
    seismic = kind in (SEISMIC2, SEISMIC25)
    three = kind in (SEISMIC25, ELECTROMAG25)
    shape = (g.nx, g.ny, g.nz) if three else (g.nx, g.nz)
    deltas = (g.dx, g.dy, g.dz) if three else (g.dx, g.dz)
    f0 = 1.0 / (25 * g.dt)
    vmax = 3500.0 if seismic else 1.5e8
    sig = [cp.sigma_alpha_max(seismic, g.npml, min(deltas), f0, vmax * (1 + 0.1 * a), dt=g.dt, mode=mode)[0]
           for a in range(len(shape))]
    alpha = cp.sigma_alpha_max(seismic, g.npml, min(deltas), f0, vmax, dt=g.dt, mode=mode)[1]
    prm = dict(kappa_max=4.0, NP=2.0, NPA=1.5)
    profiles = [cp.axis_profile(n, g.npml, d, g.dt, sm, alpha, seismic=seismic, mode=mode, **prm)
                for n, d, sm in zip(shape, deltas, sig)]
    out = []
    for device in (False, True):
        with make_solver(case, flags=flags) as s:
            if device:
                s.set_cpml_params(sig, alpha, mode=mode, **prm)
            else:
                s.set_cpml(profiles)
            out.append(_run(s, case))
    _compare(*out)


def test_refusals(gpu):
    from seidart_gb300 import ELECTROMAG2C
    case = _case(ELECTROMAG2)
    with make_solver(case) as s:
        with pytest.raises(SfdError, match="wavelet"):
            s.set_source_wavelet(case.src_ijk, 0.0, 1.0, [1.0, 1.0])
        with pytest.raises(SfdError, match="stress sources"):
            s.set_source_wavelet(case.src_ijk, 1e8, 1.0, [1.0, 1.0, 1.0], stress=True)
        with pytest.raises(SfdError, match="components"):
            s.set_source_wavelet(case.src_ijk, 1e8, 1.0, [1.0])
        with pytest.raises(SfdError, match="finite"):
            s.set_cpml_params([np.nan, 1.0], 1.0)
    c2 = sy.small_case(ELECTROMAG2C, seed=1, nx=30, nz=26, npml=5, nstep=20, nrec=2)
    with make_solver(c2) as s:
        with pytest.raises(SfdError, match="electromag2c"):
            s.set_source_wavelet(c2.src_ijk, 1e8, 1.0, [1.0, 1.0])
