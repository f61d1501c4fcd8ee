"""The seidartfdtd drop-in: file formats, project loading (CPU) and a full
run against the oracle (GPU)."""
import glob
import os

import numpy as np
import pytest

from helpers import rel_l2, run_oracle
from project_helpers import write_project
from seidart_gb300 import ELECTROMAG2, SEISMIC2, cli, cpml as cp, fortran_io as fio
from seidart_gb300 import synthetic as sy


def test_record_roundtrip_and_scipy_compat(tmp_path):
    scipy_io = pytest.importorskip("scipy.io")
    a = np.arange(12, dtype=np.float64).reshape(3, 4)
    fio.write_record(tmp_path / "a.dat", a, np.float64)
    with scipy_io.FortranFile(tmp_path / "a.dat", "r") as f:
        assert np.array_equal(f.read_reals(np.float64), a.ravel())
    with scipy_io.FortranFile(tmp_path / "b.dat", "w") as f:
        f.write_record(a.T.astype(np.float32))
    assert np.array_equal(fio.read_record(tmp_path / "b.dat", np.float32), a.T.ravel().astype(np.float32))
    (tmp_path / "c.dat").write_bytes(b"\x10\x00\x00\x00abc")
    with pytest.raises(ValueError):
        fio.read_record(tmp_path / "c.dat")


@pytest.mark.parametrize("kind", [ELECTROMAG2, SEISMIC2])
def test_load_project(tmp_path, kind):
    case = sy.small_case(kind, seed=2, nx=40, nz=34, npml=5, nstep=60)
    path, (xi, yi, zi) = write_project(case, tmp_path)
    p = cli.load_project(path, seismic=(kind == SEISMIC2), workdir=tmp_path)
    assert p["kind"] == kind
    assert (p["grid"].nx, p["grid"].nz, p["grid"].npml) == (40, 34, 5)
    assert p["src_ijk"] == case.src_ijk
    assert np.array_equal(p["planes"], case.planes)
    assert np.array_equal(p["srcfn"], case.srcfn)
    assert p["vmax"] > 0
    packed = cp.pack_profiles(p["profiles"])
    assert packed.shape == (6 * (40 + 34),)


def test_missing_file_is_an_input_error(tmp_path):
    case = sy.small_case(ELECTROMAG2, seed=2, nx=40, nz=34, npml=5, nstep=60)
    path, _ = write_project(case, tmp_path)
    os.remove(tmp_path / "e33.dat")
    assert cli.run([path, "seismic=false", "--workdir", str(tmp_path)]) == 1


@pytest.mark.gpu
@pytest.mark.parametrize("kind", [ELECTROMAG2, SEISMIC2])
def test_cli_run_matches_oracle(gpu, tmp_path, kind):
    case = sy.small_case(kind, seed=3, nx=40, nz=34, npml=5, nstep=60)
    g = case.grid
    rec_m = [((i - g.npml + 0.25) * g.dx, 0.0, (k - g.npml + 0.25) * g.dz) for i, k in ((10, 12), (25, 20), (18, 9))]
    path, (xi, yi, zi) = write_project(case, tmp_path, receivers_m=rec_m)
    seismic = kind == SEISMIC2
    rc = cli.run([path, f"seismic={str(seismic).lower()}", "density_method=arithmetic", "--workdir", str(tmp_path),
                  "--snapshot-every", "20", "--receivers", str(tmp_path / "receivers.csv"),
                  "--traces", str(tmp_path / "traces.npy")])
    assert rc == 0
    p = cli.load_project(path, seismic, tmp_path)
    rec = cli.read_receivers(tmp_path / "receivers.csv", g)
    from oracle import run as orun
    st, tr, _, _ = orun(kind, g, p["planes"], cp.pack_profiles(p["profiles"]), p["src_ijk"], p["srcfn"], rec, 60)
    assert rel_l2(np.load(tmp_path / "traces.npy"), tr) <= 1e-5
    ch = "Vx" if seismic else "Ex"
    files = sorted(glob.glob(str(tmp_path / f"{ch}.*.{xi}.{zi}.dat")))
    assert [os.path.basename(f).split(".")[1] for f in files] == ["000020", "000040", "000060"]
    last = fio.read_record(files[-1], np.float32).reshape(g.nz, g.nx)
    assert rel_l2(last, st.fields[0]) <= 1e-5


def _gradient(case):
    """An air-surface style taper: 0.15 and 0.575 in the top two interior rows."""
    c = case.grid.npml
    ni, nk = case.grid.nx - 2 * c, case.grid.nz - 2 * c
    g = np.ones((ni, nk))
    g[:, 0], g[:, 1] = 0.15, 0.575
    return g


def test_load_project_density_gradient_and_stress(tmp_path):
    case = sy.small_case(SEISMIC2, seed=4, nx=40, nz=34, npml=5, nstep=60)
    w = case.srcfn[1]
    path, _ = write_project(case, tmp_path, stress={"xx": w, "yy": 2 * w, "zz": 3 * w, "xz": 0.5 * w},
                            density_gradient=_gradient(case))
    p = cli.load_project(path, seismic=True, workdir=tmp_path)
    rho = case.planes[6].copy()
    rho[:6, :] *= 0.15  # CPML rows take the edge row's factor
    rho[6, :] *= 0.575
    assert np.allclose(p["planes"][6], rho, rtol=0, atol=0)
    assert np.array_equal(p["stress_srcfn"], np.stack([w, 3 * w, 0.5 * w]))  # xx zz xz in 2-D
    q = cli.load_project(path, seismic=True, workdir=tmp_path, density_gradient=False)
    assert np.array_equal(q["planes"][6], case.planes[6])


def test_unknown_density_method_is_an_input_error(tmp_path):
    case = sy.small_case(SEISMIC2, seed=2, nx=40, nz=34, npml=5, nstep=60)
    path, _ = write_project(case, tmp_path)
    assert cli.run([path, "seismic=true", "density_method=cubic", "--workdir", str(tmp_path)]) == 1


@pytest.mark.gpu
@pytest.mark.parametrize("density,legacy", [("geometric", False), ("harmonic", True), ("none", False),
                                            ("arithmetic", False)])
def test_cli_seismic_options_match_oracle(gpu, tmp_path, density, legacy):
    """A default SeidarT seismic project: density_method, density_gradient.dat
    and a moment-tensor source, with and without --legacy-quirks."""
    case = sy.small_case(SEISMIC2, seed=5, nx=44, nz=38, npml=5, nstep=80)
    g = case.grid
    w = 1e6 * case.srcfn[1]
    rec_m = [((i - g.npml + 0.25) * g.dx, 0.0, (k - g.npml + 0.25) * g.dz) for i, k in ((10, 12), (30, 20), (18, 9))]
    path, _ = write_project(case, tmp_path, receivers_m=rec_m, stress={"xx": w, "zz": w, "yy": w},
                            density_gradient=_gradient(case))
    args = [path, "seismic=true", f"density_method={density}", "--workdir", str(tmp_path), "--snapshot-every", "0",
            "--receivers", str(tmp_path / "receivers.csv"), "--traces", str(tmp_path / "traces.npy")]
    assert cli.run(args + (["--legacy-quirks"] if legacy else [])) == 0
    p = cli.load_project(path, True, tmp_path)
    rec = cli.read_receivers(tmp_path / "receivers.csv", g)
    from oracle import run as orun
    _, tr, _, _ = orun(SEISMIC2, g, p["planes"], cp.pack_profiles(p["profiles"]), p["src_ijk"], p["srcfn"], rec,
                       case.nstep, legacy=legacy, density=density, stress_src=p["stress_srcfn"])
    assert rel_l2(np.load(tmp_path / "traces.npy"), tr) <= 1e-5


def test_cpml_mode_2d_refused_where_it_cannot_be_honoured(tmp_path):
    """--cpml-mode 2d: a 2.5-D model (the driver writes no y fields) and a
    project without the CPML files end with exit status 1."""
    case = sy.small_case(SEISMIC2, seed=2, nx=40, nz=34, npml=5, nstep=20)
    path, _ = write_project(case, tmp_path)
    assert cli.run([path, "seismic=true", "--workdir", str(tmp_path), "--cpml-mode", "2d"]) == 1
    from seidart_gb300 import SEISMIC25
    d = tmp_path / "three"
    d.mkdir()
    case3 = sy.small_case(SEISMIC25, seed=3, nx=30, nz=28, ny=20, npml=5, nstep=20)
    path3, _ = write_project(case3, d)
    assert cli.run([path3, "seismic=true", "--workdir", str(d), "--cpml-mode", "2d"]) == 1
