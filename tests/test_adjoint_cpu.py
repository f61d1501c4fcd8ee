"""CPU checks of the FP64 discrete-adjoint references (oracle/numpy_adjoint.py),
electromag2 and seismic2: their forward passes reproduce the oracle's traces
and their gradients match central finite differences of the oracle's misfit."""
import numpy as np
import pytest

import oracle
from oracle import numpy_adjoint as na
from seidart_gb300 import ELECTROMAG2, SEISMIC2, cpml as cp, synthetic as sy


def test_numpy_adjoint_matches_oracle_fd():
    c = sy.small_case(ELECTROMAG2, seed=41, nx=34, nz=30, npml=4, nstep=90, nrec=8)
    g = c.grid
    prof = cp.pack_profiles(c.profiles)
    src = (c.src_ijk[0], c.src_ijk[2])
    base = c.planes.copy()
    _, d_obs, _, _ = oracle.run(ELECTROMAG2, g, base, prof, c.src_ijk, c.srcfn, c.rec_ijk, c.nstep)
    rng = np.random.default_rng(1)
    cur = base * (1 + 0.03 * rng.standard_normal(base.shape) * (np.arange(6) < 3)[:, None, None])
    tr, states = na.forward(g.nx, g.nz, g.dx, g.dz, g.dt, prof, cur, src, c.srcfn, c.nstep, c.rec_ijk)
    _, tr_o, _, _ = oracle.run(ELECTROMAG2, g, cur, prof, c.src_ijk, c.srcfn, c.rec_ijk, c.nstep)
    assert np.allclose(tr, tr_o, rtol=1e-12, atol=1e-30)
    G = na.gradient(g.nx, g.nz, g.dx, g.dz, g.dt, prof, cur, src, c.srcfn, c.rec_ijk, states, tr - d_obs)

    def J(p):
        _, t, _, _ = oracle.run(ELECTROMAG2, g, p, prof, c.src_ijk, c.srcfn, c.rec_ijk, c.nstep)
        return 0.5 * np.sum((t - d_obs) ** 2)

    for q, scale in ((0, 1.0), (1, 0.01), (2, 1.0), (3, 1e-3), (4, 1e-4), (5, 1e-3)):
        d = np.zeros_like(cur)
        d[q] = scale * rng.standard_normal(cur[0].shape)
        eps = 1e-4
        fd = (J(cur + eps * d) - J(cur - eps * d)) / (2 * eps)
        ad = float(np.sum(G * d))
        assert abs(ad - fd) <= 1e-6 * abs(fd), (q, ad, fd)


def _s2_setup(density, seed=3):
    c = sy.small_case(SEISMIC2, seed=seed, nx=30, nz=26, npml=4, nstep=110, nrec=8)
    g = c.grid
    prof = cp.pack_profiles(c.profiles)
    rng = np.random.default_rng(seed)
    ssrc = 1e6 * rng.standard_normal((3, c.nstep)) * np.exp(-((np.arange(c.nstep) - 20) / 8.0) ** 2)
    _, d_obs, _, _ = oracle.run(SEISMIC2, g, c.planes, prof, c.src_ijk, c.srcfn, c.rec_ijk, c.nstep,
                                density=density, stress_src=ssrc)
    cur = c.planes * (1 + 0.03 * rng.standard_normal(c.planes.shape) * (np.arange(9) < 7)[:, None, None])
    return c, g, prof, ssrc, d_obs, cur, rng


@pytest.mark.parametrize("density", ["arithmetic", "harmonic", "geometric", "none"])
def test_numpy_seismic2_adjoint_matches_oracle_fd(density):
    """The FP64 seismic2 adjoint: its forward reproduces the oracle's traces
    (corrected physics, attenuation, force and stress sources), and its
    gradient of all nine planes matches central differences of the oracle."""
    c, g, prof, ssrc, d_obs, cur, rng = _s2_setup(density)
    src = (c.src_ijk[0], c.src_ijk[2])
    tr, states, _ = na.seismic2_forward(g.nx, g.nz, g.dx, g.dz, g.dt, prof, cur, src, c.srcfn, c.nstep, c.rec_ijk,
                                        density=density, stress_src=ssrc)
    _, tr_o, _, _ = oracle.run(SEISMIC2, g, cur, prof, c.src_ijk, c.srcfn, c.rec_ijk, c.nstep, density=density,
                               stress_src=ssrc)
    assert np.allclose(tr, tr_o, rtol=1e-11, atol=1e-14 * np.abs(tr_o).max())
    G = na.seismic2_gradient(g.nx, g.nz, g.dx, g.dz, g.dt, prof, cur, src, c.srcfn, c.rec_ijk, states, tr - d_obs,
                             density=density, stress_src=ssrc)

    def J(p):
        _, t, _, _ = oracle.run(SEISMIC2, g, p, prof, c.src_ijk, c.srcfn, c.rec_ijk, c.nstep, density=density,
                                stress_src=ssrc)
        return 0.5 * np.sum((t - d_obs) ** 2)

    for q in range(9):
        d = np.zeros_like(cur)
        scale = 1e-3 if q >= 7 else np.abs(cur[q]).mean()
        d[q] = scale * rng.standard_normal(cur[0].shape)
        eps = 1e-5  # per-cell random directions: the FD truncation error, ~eps^2, stays below 1e-7
        fd = (J(cur + eps * d) - J(cur - eps * d)) / (2 * eps)
        ad = float(np.sum(G[q] * d[q]))
        assert abs(ad - fd) <= 3e-7 * abs(fd), (q, ad, fd)
