"""GPU: the driver's 2-D CPML fields (SFD_FLAG_CPML_2D, sfd_set_cpml2d)
against the FP64 oracle given the same fields, for electromag2 and seismic2
(with a moment-tensor source and each density method), and the
seidartfdtd --cpml-mode 2d run of a project whose CPML files are written as
the driver writes them (the layout tests/test_reference_fixtures.py pins to
the reference's cpmlcompute).  Tolerances as in test_parity_gpu.py."""
import numpy as np
import pytest

from golden.make_golden import stress_source
from helpers import rel_l2
from project_helpers import write_project
from seidart_gb300 import ELECTROMAG2, SEISMIC2, cli, cpml as cp, fortran_io as fio
from seidart_gb300 import synthetic as sy
from seidart_gb300.solver import FIELDS, FLAG_CPML_2D, MEMORY, FDTDSolver

pytestmark = pytest.mark.gpu


def _fields(c):
    g = c.grid
    return cp.driver_cpml_planes(g.nx, g.nz, g.npml, g.dx, g.dz, g.dt, c.f0, c.meta["vmax"], g.kind == SEISMIC2)


@pytest.mark.parametrize("kind,density,stress", [(ELECTROMAG2, "arithmetic", False), (SEISMIC2, "arithmetic", False),
                                                 (SEISMIC2, "harmonic", True), (SEISMIC2, "geometric", True)])
def test_cpml2d_matches_oracle(gpu, kind, density, stress):
    import oracle
    c = sy.small_case(kind, seed=51, nx=58, nz=47, npml=7, nstep=140)
    opts = {}
    if kind == SEISMIC2:
        c.density = density
        opts = {"density": density}
        if stress:
            c.stress_srcfn = stress_source(kind, 1e6 * c.srcfn[0])
    F = _fields(c)
    with FDTDSolver(c.grid, c.nstep, len(c.rec_ijk), flags=FLAG_CPML_2D, **opts) as s:
        assert s.on_chip() is None
        s.set_model(c.planes)
        s.set_cpml2d(F)
        s.set_source(c.src_ijk, c.srcfn)
        if c.stress_srcfn is not None:
            s.set_stress_source(c.src_ijk, c.stress_srcfn)
        s.set_receivers(c.rec_ijk)
        s.run(53)
        s.run(c.nstep - 53)
        s.status()
        st, ref, _, blew = oracle.run(kind, c.grid, c.planes, cp.pack_profiles(c.profiles), c.src_ijk, c.srcfn,
                                      c.rec_ijk, c.nstep, density=c.density, stress_src=c.stress_srcfn, cpml2d=F)
        assert not blew
        assert rel_l2(s.traces(), ref) <= 1e-5
        for q, name in enumerate(FIELDS[kind]):
            assert rel_l2(s.field(name), st.fields[q]) <= 1e-5, name
        for q, name in enumerate(MEMORY[kind]):
            if np.linalg.norm(st.memory[q]) > 0:
                assert rel_l2(s.memory(name), st.memory[q]) <= 1e-4, name


def test_cpml2d_handle_rules(gpu):
    from seidart_gb300._lib import SfdError
    c = sy.small_case(SEISMIC2, seed=52, nx=40, nz=36, npml=5, nstep=20)
    with pytest.raises(SfdError):  # the legacy loops read 1-D profiles
        FDTDSolver(c.grid, c.nstep, 2, flags=FLAG_CPML_2D, legacy=True)
    with FDTDSolver(c.grid, c.nstep, 2, flags=FLAG_CPML_2D) as s:
        with pytest.raises(SfdError):
            s.set_cpml(c.profiles)  # a 2-D handle takes sfd_set_cpml2d
    e = sy.small_case(sy.SEISMIC25, seed=53, nx=30, nz=28, ny=20, npml=5, nstep=10)
    with pytest.raises(SfdError):
        FDTDSolver(e.grid, e.nstep, 2, flags=FLAG_CPML_2D)


@pytest.mark.parametrize("kind", [ELECTROMAG2, SEISMIC2])
def test_cli_cpml_mode_2d(gpu, tmp_path, kind):
    import oracle
    c = sy.small_case(kind, seed=54, nx=44, nz=38, npml=5, nstep=80)
    g = c.grid
    F = _fields(c)
    rec_m = [((i - g.npml + 0.25) * g.dx, 0.0, (k - g.npml + 0.25) * g.dz) for i, k in ((10, 12), (30, 20), (18, 9))]
    path, _ = write_project(c, tmp_path, receivers_m=rec_m)
    for q, name in enumerate(["kappa_cpml", "acoef_cpml", "bcoef_cpml", "kappa_half_cpml", "acoef_half_cpml",
                              "bcoef_half_cpml"]):
        fio.write_record(tmp_path / f"{name}.dat", F[q], np.float64)  # (NX, NZ) x fastest, as _write2d does
    seismic = kind == SEISMIC2
    args = [path, f"seismic={str(seismic).lower()}", "density_method=arithmetic", "--workdir", str(tmp_path),
            "--snapshot-every", "0", "--receivers", str(tmp_path / "receivers.csv"),
            "--traces", str(tmp_path / "traces.npy"), "--cpml-mode", "2d"]
    assert cli.run(args) == 0
    p = cli.load_project(path, seismic, tmp_path)
    rec = cli.read_receivers(tmp_path / "receivers.csv", g)
    _, tr, _, _ = oracle.run(kind, g, p["planes"], cp.pack_profiles(p["profiles"]), p["src_ijk"], p["srcfn"], rec,
                             c.nstep, cpml2d=cli.read_cpml2d(tmp_path, g))
    assert rel_l2(np.load(tmp_path / "traces.npy"), tr) <= 1e-5
    if seismic:
        assert cli.run(args + ["--legacy-quirks"]) == 1
