"""CPU tests of the FP64 oracle: agreement of two independent restatements,
physical known-answer checks, and the blow-up detector."""
import math

import numpy as np
import pytest

import oracle
from oracle import numpy_ref
from helpers import rel_l2, run_oracle
from seidart_gb300 import ELECTROMAG2, ELECTROMAG25, ELECTROMAG2C, SEISMIC2, SEISMIC25
from seidart_gb300 import cpml as cp
from seidart_gb300 import synthetic as sy
from seidart_gb300.solver import GridSpec


@pytest.mark.parametrize("kind,fn", [(ELECTROMAG2, numpy_ref.electromag2), (SEISMIC2, numpy_ref.seismic2)])
@pytest.mark.parametrize("seed,nx,nz", [(1, 37, 29), (2, 26, 41)])
def test_loop_and_slice_restatements_agree(kind, fn, seed, nx, nz):
    c = sy.small_case(kind, seed=seed, nx=nx, nz=nz, npml=5, nstep=120)
    g = c.grid
    prof = cp.pack_profiles(c.profiles)
    st, tr, _, blew = run_oracle(c)
    assert not blew
    F, M, T = fn(g.nx, g.nz, g.dx, g.dz, g.dt, prof, c.planes, (c.src_ijk[0], c.src_ijk[2]), c.srcfn, c.nstep,
                 rec=c.rec_ijk)
    # identical operation order in FP64: agreement to rounding
    assert rel_l2(st.fields, F) < 1e-13
    assert rel_l2(st.memory, M, floor=1e-300) < 1e-13
    assert rel_l2(tr, T) < 1e-13


@pytest.mark.parametrize("legacy,density,stress", [(True, "arithmetic", False), (False, "geometric", True),
                                                    (False, "harmonic", False), (False, "none", True)])
@pytest.mark.parametrize("seed,nx,nz", [(3, 33, 28), (4, 24, 39)])
def test_seismic2_physics_options_agree(legacy, density, stress, seed, nx, nz):
    """The seismic2 physics options (legacy quirks or corrected physics,
    density method, moment-tensor source) in the C++ loops and the numpy
    slices."""
    c = sy.small_case(SEISMIC2, seed=seed, nx=nx, nz=nz, npml=5, nstep=110)
    c.legacy, c.density = legacy, density
    if stress:
        w = 1e6 * c.srcfn[0]
        c.stress_srcfn = np.stack([w, 0.7 * w, -0.4 * w])
    g = c.grid
    st, tr, _, blew = run_oracle(c)
    assert not blew
    F, M, T = numpy_ref.seismic2(g.nx, g.nz, g.dx, g.dz, g.dt, cp.pack_profiles(c.profiles), c.planes,
                                 (c.src_ijk[0], c.src_ijk[2]), c.srcfn, c.nstep, rec=c.rec_ijk, legacy=legacy,
                                 density=density, stress_src=c.stress_srcfn)
    assert rel_l2(st.fields, F) < 1e-12
    assert rel_l2(st.memory, M, floor=1e-300) < 1e-12
    assert rel_l2(tr, T) < 1e-12


def test_seismic_physics_options_change_the_result():
    """Each option changes the traces (so the tests above compare something):
    the corrected physics against the legacy loops, each density method
    against the others, and the stress source against none."""
    base = sy.small_case(SEISMIC2, seed=5, nx=36, nz=30, npml=5, nstep=120)
    _, ref, _, _ = run_oracle(base)
    for legacy, density in [(True, "arithmetic"), (False, "none"), (False, "geometric"), (False, "harmonic")]:
        c = sy.small_case(SEISMIC2, seed=5, nx=36, nz=30, npml=5, nstep=120)
        c.legacy, c.density = legacy, density
        assert rel_l2(run_oracle(c)[1], ref) > 1e-6, (legacy, density)
    c = sy.small_case(SEISMIC2, seed=5, nx=36, nz=30, npml=5, nstep=120)
    w = 1e6 * c.srcfn[0]
    c.stress_srcfn = np.stack([w, w, 0 * w])
    assert rel_l2(run_oracle(c)[1], ref) > 1e-3


@pytest.mark.parametrize("seed,nx,nz", [(1, 37, 29), (2, 26, 41)])
def test_complex_em_restatements_agree(seed, nx, nz):
    """electromag2c (complex permittivities): the C++ loops against the numpy
    slices; complex values travel as (real, imaginary) plane pairs."""
    c = sy.small_case(ELECTROMAG2C, seed=seed, nx=nx, nz=nz, npml=5, nstep=120)
    g = c.grid
    prof = cp.pack_profiles(c.profiles)
    st, tr, _, blew = run_oracle(c)
    assert not blew
    F, M, T = numpy_ref.electromag2c(g.nx, g.nz, g.dx, g.dz, g.dt, prof, c.planes, (c.src_ijk[0], c.src_ijk[2]),
                                     c.srcfn, c.nstep, rec=c.rec_ijk)
    split = lambda a: np.stack([v for z in a for v in (z.real, z.imag)])
    assert np.abs(F.imag).max() > 1e-3 * np.abs(F.real).max()  # the imaginary parts matter
    assert rel_l2(st.fields, split(F)) < 1e-13
    assert rel_l2(st.memory, split(M), floor=1e-300) < 1e-13
    assert rel_l2(tr, np.stack([T[:, 0].real, T[:, 0].imag, T[:, 1].real, T[:, 1].imag], axis=1)) < 1e-13


def test_complex_em_with_real_permittivity_is_electromag2():
    c = sy.small_case(ELECTROMAG2C, seed=4, nx=30, nz=28, npml=5, nstep=80)
    c.planes[[1, 3, 5]] = 0.0
    st, tr, _, _ = run_oracle(c)
    r = sy.small_case(ELECTROMAG2, seed=4, nx=30, nz=28, npml=5, nstep=80)
    r.planes = np.ascontiguousarray(c.planes[[0, 2, 4, 6, 7, 8]])
    g = c.grid
    r.grid = GridSpec(ELECTROMAG2, g.nx, g.nz, g.dx, g.dz, g.dt, g.npml)
    r.profiles, r.srcfn, r.src_ijk, r.rec_ijk = c.profiles, c.srcfn, c.src_ijk, c.rec_ijk
    st_r, tr_r, _, _ = run_oracle(r)
    assert np.array_equal(st.fields[[0, 2, 4]], st_r.fields) and not st.fields[[1, 3, 5]].any()
    assert np.array_equal(tr[:, [0, 2]], tr_r)


@pytest.mark.parametrize("kind", [ELECTROMAG2, SEISMIC2, SEISMIC25, ELECTROMAG25, ELECTROMAG2C])
def test_split_runs_equal_one_run(kind):
    c = sy.small_case(kind, seed=3, nx=30, nz=26, ny=18, npml=4, nstep=60)
    st1, tr1, _, _ = run_oracle(c)
    st2, a, _, _ = run_oracle(c, nsteps=25)
    st2, b, _, _ = run_oracle(c, nsteps=35, state=st2)
    assert np.array_equal(st1.fields, st2.fields)
    assert np.array_equal(tr1, np.concatenate([a, b]))


def _homogeneous_em(nx=260, nz=120, eps=4.0, npml=20, nstep=900):
    d = 0.02
    v = cp.CLIGHT / math.sqrt(eps)
    dt = cp.time_step(0.5, v, (d, d))
    planes = np.stack([np.full((nz, nx), eps), np.zeros((nz, nx)), np.full((nz, nx), eps),
                       np.zeros((nz, nx)), np.zeros((nz, nx)), np.zeros((nz, nx))])
    f0 = 600e6
    prof = cp.build_profiles((nx, nz), (d, d), npml, dt, f0, v, seismic=False)
    g = GridSpec(ELECTROMAG2, nx, nz, d, d, dt, npml)
    src = np.zeros((2, nstep))
    src[1] = sy.ricker(nstep, dt, f0)
    return g, planes, prof, src, v


def test_em_arrival_speed_matches_medium():
    """Ez pulse in a homogeneous eps_r = 4 medium travels at c/2."""
    g, planes, prof, src, v = _homogeneous_em()
    sx, sz = 60, 60
    rec = np.array([[sx + 40, 0, sz], [sx + 140, 0, sz]], dtype=np.int32)
    st, tr, _, _ = oracle.run(ELECTROMAG2, g, planes, cp.pack_profiles(prof), (sx, 0, sz), src, rec, src.shape[1])
    ez = tr[:, 1, :]
    t1, t2 = (np.argmax(np.abs(ez[:, r])) for r in range(2))
    vel = (100 * g.dx) / ((t2 - t1) * g.dt)
    assert abs(vel / v - 1.0) < 0.03


def test_elastic_p_arrival_speed_matches_medium():
    """vz pulse in a homogeneous isotropic solid travels at the P velocity along z."""
    nx, nz, npml, d = 120, 260, 20, 0.5
    lam, mu, rho = 4e9, 3e9, 1000.0
    vp = math.sqrt((lam + 2 * mu) / rho)
    dt = cp.time_step(0.5, vp, (d, d))
    nstep = 700
    f0 = 250.0
    z = np.zeros((nz, nx))
    planes = np.stack([z + lam + 2 * mu, z + lam, z, z + lam + 2 * mu, z, z + mu, z + rho, z, z])
    prof = cp.build_profiles((nx, nz), (d, d), npml, dt, f0, vp, seismic=True)
    g = GridSpec(SEISMIC2, nx, nz, d, d, dt, npml)
    src = np.zeros((2, nstep))
    src[1] = sy.ricker(nstep, dt, f0)
    rec = np.array([[60, 0, 100], [60, 0, 200]], dtype=np.int32)
    st, tr, _, _ = oracle.run(SEISMIC2, g, planes, cp.pack_profiles(prof), (60, 0, 60), src, rec, nstep)
    vz = tr[:, 1, :]
    t1, t2 = (np.argmax(np.abs(vz[:, r])) for r in range(2))
    vel = (100 * d) / ((t2 - t1) * dt)
    assert abs(vel / vp - 1.0) < 0.03


def test_em_cpml_absorbs():
    """After the pulse has left the interior, the CPML has removed almost all of
    its energy; with the CPML coefficients switched off (a = 0) the Dirichlet
    box keeps it."""
    g, planes, prof, src, v = _homogeneous_em(nx=140, nz=140, nstep=1600)
    packed = cp.pack_profiles(prof)
    rec = np.zeros((0, 3), dtype=np.int32)

    def energy_after(p):
        st, _, _, _ = oracle.run(ELECTROMAG2, g, planes, p, (70, 0, 70), src, rec, src.shape[1])
        return float(np.sum(st.fields[0] ** 2 + st.fields[1] ** 2))

    off = packed.copy()
    nx, nz = g.nx, g.nz
    for base, n in ((0, nx), (6 * nx, nz)):
        for q in (1, 4):  # a, a_half
            off[base + q * n: base + (q + 1) * n] = 0.0
        for q in (0, 3):  # K, K_half
            off[base + q * n: base + (q + 1) * n] = 1.0
    assert energy_after(packed) < 1e-3 * energy_after(off)


def test_blow_up_detected():
    """dt far above the stability limit: the norm check of seismicfdtd.f95:378-379 fires."""
    c = sy.small_case(SEISMIC2, seed=5, nx=40, nz=36, npml=5, nstep=400)
    c.grid.dt *= 4.0
    _, _, norm, blew = run_oracle(c)
    assert blew and norm > 1e25


def _planes2d(c):
    g = c.grid
    seismic = g.kind == SEISMIC2
    return cp.driver_cpml_planes(g.nx, g.nz, g.npml, g.dx, g.dz, g.dt, c.f0, c.meta["vmax"], seismic)


@pytest.mark.parametrize("kind", [ELECTROMAG2, SEISMIC2])
@pytest.mark.parametrize("seed,nx,nz", [(7, 38, 31), (8, 27, 40)])
def test_cpml2d_restatements_agree(kind, seed, nx, nz):
    """The driver's 2-D CPML fields in place of the axis profiles: C++ loops
    against the numpy slices, and different from the 1-D run."""
    c = sy.small_case(kind, seed=seed, nx=nx, nz=nz, npml=6, nstep=110)
    g = c.grid
    F = _planes2d(c)
    prof = cp.pack_profiles(c.profiles)
    st, tr, _, blew = oracle.run(kind, g, c.planes, prof, c.src_ijk, c.srcfn, c.rec_ijk, c.nstep, cpml2d=F)
    assert not blew
    fn = numpy_ref.electromag2 if kind == ELECTROMAG2 else numpy_ref.seismic2
    Fn, Mn, Tn = fn(g.nx, g.nz, g.dx, g.dz, g.dt, prof, c.planes, (c.src_ijk[0], c.src_ijk[2]), c.srcfn, c.nstep,
                    rec=c.rec_ijk, cpml2d=F)
    assert rel_l2(st.fields, Fn) < 1e-12
    assert rel_l2(st.memory, Mn, floor=1e-300) < 1e-12
    assert rel_l2(tr, Tn) < 1e-12
    _, tr1, _, _ = run_oracle(c)
    assert rel_l2(tr, tr1) > 1e-6
