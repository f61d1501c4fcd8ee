"""CPU tests of the FP64 CPML profile builder and the time step."""
import math

import numpy as np
import pytest

from seidart_gb300 import cpml as cp


@pytest.mark.parametrize("mode", ["driver", "legacy"])
@pytest.mark.parametrize("seismic", [True, False])
@pytest.mark.parametrize("half", [False, True])
def test_profile_matches_formulas(seismic, half, mode):
    n, c, d, dt = 60, 10, 0.5, 1e-5 if seismic else 1e-11
    sig, alp = 1234.0 if seismic else 0.05, 300.0 if seismic else 1e-9
    p = cp.axis_profile(n, c, d, dt, sig, alp, kappa_max=5.0, NP=2.0, NPA=2.0, seismic=seismic, mode=mode)
    K = p.K_half if half else p.K
    a = p.a_half if half else p.a
    b = p.b_half if half else p.b
    for ind in range(c):
        dist = (d * c - (d * ind + (d / 2 if half else 0.0))) / (d * c)
        if mode == "driver" and half:  # the driver rescales the half-offset distances to a largest value of 1
            dist /= (c - 0.5) / c
        s = sig * dist ** 2
        k = 1.0 + 4.0 * dist ** 2
        al = alp * (1 - dist) ** 2
        bb = math.exp(-(s / k + al) * (dt if seismic else dt / cp.EPS0))
        aa = s * (bb - 1) / (k * s + k * al)
        for pos in (ind, n - 1 - ind):
            assert K[pos] == pytest.approx(k, rel=1e-14)
            assert b[pos] == pytest.approx(bb, rel=1e-14)
            assert a[pos] == pytest.approx(aa, rel=1e-12)
    # interior: K = 1, a = 0; b = 0 (legacy/prjrun_101424.py:260-266) or exp(0) = 1 (the driver's fields)
    assert np.all(K[c:n - c] == 1.0) and np.all(a[c:n - c] == 0.0)
    assert np.all(b[c:n - c] == (1.0 if mode == "driver" else 0.0))


def test_packed_layout():
    prof = cp.build_profiles((30, 20), (1.0, 1.0), 5, 1e-4, 100.0, 3000.0, seismic=True)
    v = cp.pack_profiles(prof)
    assert v.shape == (6 * 30 + 6 * 20,)
    assert np.array_equal(v[:30], prof[0].K)
    assert np.array_equal(v[6 * 30 + 2 * 20: 6 * 30 + 3 * 20], prof[1].b)


def test_time_step_and_velocity():
    C6 = np.zeros((6, 6))
    lam, mu, rho = 4e9, 3e9, 1000.0
    C6[:3, :3] = lam
    for q in range(3):
        C6[q, q] = lam + 2 * mu
        C6[q + 3, q + 3] = mu
    assert cp.max_velocity(C6, rho, 2) == pytest.approx(math.sqrt((lam + 2 * mu) / rho))
    assert cp.time_step(0.5, 2000.0, (0.5, 0.5)) == pytest.approx(0.5 / (2000.0 * math.sqrt(8.0)))
