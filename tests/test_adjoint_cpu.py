"""CPU checks of the FP64 discrete-adjoint reference (oracle/numpy_adjoint.py):
its gradient matches central finite differences of the FP64 oracle forward."""
import numpy as np

import oracle
from oracle import numpy_adjoint as na
from seidart_gb300 import ELECTROMAG2, cpml as cp, synthetic as sy


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
