"""This repository's host side against outputs of the reference's own Python
code (tests/golden/reference_inputs.npz, made by
tests/golden/make_ref_fixtures.py with the reference's Model.build,
cpmlcompute/cpml_parameters, pointsource, wavelet, read_dat and read_block):

* the CLI loader reads the per-cell material files, the source files (force
  and moment tensor) and density_gradient.dat the driver writes, in the
  right orientation;
* the time step and the Christoffel velocities behind it;
* the CPML profiles (1-D, along each edge) and the 2-D CPML fields;
* the Ricker (gaus1) wavelet;
* the reference's readers decode the snapshot records and EM25 block files
  written here.
"""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from seidart_gb300 import cli, cpml as cp, em25block, fortran_io as fio
from seidart_gb300 import synthetic as sy
from seidart_gb300.solver import MODEL_PLANES

FIX = Path(__file__).resolve().parent / "golden" / "reference_inputs.npz"
CASES = ["seismic2_tnt", "seismic2_ac", "seismic2_dc", "em2", "seismic25_tnt"]


@pytest.fixture(scope="module")
def ref():
    return np.load(FIX)


def _record(ref, case, name):
    """The values of one .dat file the driver wrote (one Fortran record)."""
    raw = ref[f"{case}/file/{name}"].tobytes()
    n = np.frombuffer(raw[:4], dtype="<i4")[0]
    return np.frombuffer(raw[4:4 + n], dtype="<f8")


def _project(ref, case, tmp_path):
    """The driver's files of ``case`` in a project directory, plus a JSON with
    the Domain and Source entries its save_to_json would write."""
    for name in ref[f"{case}/files"]:
        (tmp_path / str(name)).write_bytes(ref[f"{case}/file/{name}"].tobytes())
    dim, nx, ny, nz, dx, dy, dz, c, ams, kmax, NP, NPA, R = ref[f"{case}/domain"]
    f0, steps, x, y, z = ref[f"{case}/source"]
    seismic = case.startswith("seismic")
    prj = {"Domain": {"dim": dim, "nx": int(nx), "ny": int(ny), "nz": int(nz), "dx": dx, "dy": dy, "dz": dz,
                      "cpml": int(c), "alpha_max_scalar": ams, "kappa_max": kmax, "NP": NP, "NPA": NPA, "Rcoef": R},
           ("Seismic" if seismic else "Electromagnetic"): {
               "Source": {"dt": float(ref[f"{case}/dt"]), "time_steps": int(steps), "xind": int(x / dx),
                          "yind": int(y / dy), "zind": int(z / dz), "source_frequency": f0}}}
    (tmp_path / "project.json").write_text(json.dumps(prj))
    return tmp_path / "project.json", seismic


@pytest.mark.parametrize("case", CASES)
def test_loader_reads_the_driver_files(ref, case, tmp_path):
    path, seismic = _project(ref, case, tmp_path)
    p = cli.load_project(path, seismic, tmp_path, density_gradient=False)
    c = int(ref[f"{case}/domain"][7])
    geo = ref[f"{case}/geometry"]  # (nx, nz) material ids of the interior
    nx, nz = geo.shape
    assert p["planes"].shape[1:] == (nz + 2 * c, nx + 2 * c)
    # every plane is the material column spread over the geometry (x fastest
    # on disk) and extended into the CPML by edge replication
    for q, name in enumerate(MODEL_PLANES[p["kind"]]):
        fname = cli._FILE_OF.get(name, name) + ".dat"
        if fname not in ref[f"{case}/files"]:
            assert not p["planes"][q].any(), name
            continue
        vals = _record(ref, case, fname)
        per_mat = {int(m): vals.reshape(nz + 2 * c, nx + 2 * c)[c + k, c + i]
                   for (i, k), m in np.ndenumerate(geo)}
        want = np.pad(np.vectorize(per_mat.get)(geo).T, c, mode="edge")
        assert np.array_equal(p["planes"][q], want), name
    # sources: force components and, for seismic, the moment tensor
    comps = ["x", "y", "z"] if p["kind"] in (2, 4) else ["x", "z"]
    stem = "seismicsource" if seismic else "electromagneticsource"
    for q, comp in enumerate(comps):
        assert np.array_equal(p["srcfn"][q], _record(ref, case, f"{stem}{comp}.dat"))
    if seismic:
        names = ["xx", "yy", "zz", "xy", "xz", "yz"] if p["kind"] == 2 else ["xx", "zz", "xz"]
        recs = np.stack([_record(ref, case, f"seismicsource{n}.dat") for n in names])
        if not recs.any():  # 'ac': a force source only
            assert case.endswith("ac") and p["stress_srcfn"] is None
        else:
            assert np.array_equal(p["stress_srcfn"], recs)
    if case.endswith("tnt"):  # explosive: equal normal stresses, no force, no shear
        s = p["stress_srcfn"]
        assert not p["srcfn"].any() and s[0].any()
        assert np.array_equal(s[0], s[1])


@pytest.mark.parametrize("case", ["seismic2_tnt", "seismic25_tnt"])
def test_density_gradient_orientation(ref, case, tmp_path):
    """density_gradient.dat (the driver's airsurf) multiplies the density: the
    factors below the air layer (material 1, the top rows of the geometry)
    vary with depth, and the loader lays them out that way."""
    path, _ = _project(ref, case, tmp_path)
    p0 = cli.load_project(path, True, tmp_path, density_gradient=False)
    p1 = cli.load_project(path, True, tmp_path)
    q = MODEL_PLANES[p0["kind"]].index("rho")
    c = int(ref[f"{case}/domain"][7])
    fac = (p1["planes"][q] / p0["planes"][q])[c:-c, c:-c]  # (nz, nx) interior
    g = _record(ref, case, "density_gradient.dat")
    geo = ref[f"{case}/geometry"]
    assert np.array_equal(fac, g.reshape(geo.shape).T)
    # below the air (rows 0-3) the first two rows of firn are tapered, then 1
    col = fac[:, 1]
    assert col[4] == pytest.approx(0.15) and 0.15 < col[5] < 1.0 and np.all(fac[7:, :] == 1.0)
    assert np.all(fac[4] == fac[4, 0])  # a row is uniform along x: the z axis is the taper's axis


@pytest.mark.parametrize("case", CASES)
def test_time_step_and_velocities(ref, case):
    """dt = CFL / (vmax sqrt(sum 1/delta^2)) (classes.py:469-485) with the
    Christoffel velocities of each material (classes.py:1070-1121)."""
    dim, nx, ny, nz, dx, dy, dz = ref[f"{case}/domain"][:7]
    vm = ref[f"{case}/vmax_all"]
    if case == "em2":
        # the driver's EM branch: clight / sqrt(min eps_ii) (classes.py:472-474)
        vmax = cp.CLIGHT / np.sqrt(1.0)  # air (eps = 1) is the fastest material
    else:
        lam, mu = 6.0e9, 3.0e9  # the fixture's ice: isotropic (6, 3) GPa with c11, c33, c13, c55 overridden
        C = np.zeros((6, 6))
        C[:3, :3] = lam
        for k in range(3):
            C[k, k] = lam + 2 * mu
            C[k + 3, k + 3] = mu
        C[0, 0], C[2, 2], C[0, 2], C[2, 0], C[4, 4] = 13.9e9, 15.0e9, 5.8e9, 5.8e9, 3.0e9
        v_ice = cp.max_velocity(C, 917.0, 2.5 if dim == 2.5 else 2)
        assert v_ice == pytest.approx(vm[0], rel=1e-12)
        assert cp.axis_velocity(C, 917.0, "x") == pytest.approx(ref[f"{case}/vmax_x"][0], rel=1e-12)
        assert cp.axis_velocity(C, 917.0, "z") == pytest.approx(ref[f"{case}/vmax_z"][0], rel=1e-12)
        vmax = max(vm)
    deltas = (dx, dy, dz) if dim == 2.5 else (dx, dz)
    dt = cp.time_step(float(ref[f"{case}/cfl"]), vmax, deltas)
    assert dt == pytest.approx(float(ref[f"{case}/dt"]), rel=1e-14)


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("half", [False, True])
def test_cpml_profiles_match_driver_fields(ref, case, half):
    """The 1-D profiles the kernels take equal the driver's 2-D CPML fields
    along each edge (outside the corners), and driver_fields_2d rebuilds the
    whole fields, corners included (definitions.py:560-998)."""
    dim, nx, ny, nz, dx, dy, dz, c, ams, kmax, NP, NPA, R = ref[f"{case}/domain"]
    c, nx, ny, nz = int(c), int(nx), int(ny), int(nz)
    NX, NZ = nx + 2 * c, nz + 2 * c
    seismic = case.startswith("seismic")
    f0 = float(ref[f"{case}/source"][0])
    dt = float(ref[f"{case}/dt"])
    vx = float(max(ref[f"{case}/vmax_x"])) if seismic else 0.0  # per-axis speeds of the seismic sigma_max
    vz = float(max(ref[f"{case}/vmax_z"])) if seismic else 0.0
    params = dict(alpha_max_scalar=ams, kappa_max=kmax, NP=NP, NPA=NPA, Rcoef=R)
    deltas = (dx, dy, dz) if dim == 2.5 else (dx, dz)
    suffix = "_half_cpml.dat" if half else "_cpml.dat"
    drv = {n: _record(ref, case, n + suffix).reshape(NZ, NX) for n in ("sigma", "kappa", "alpha", "acoef", "bcoef")}
    mine = cp.driver_fields_2d(NX, NZ, c, dx, dz, dt, f0, vx, seismic, params, half=half, deltamin=min(deltas),
                               vmax_z=vz)
    for n in drv:
        assert np.allclose(mine[n], drv[n], rtol=1e-12, atol=1e-300), n
    shape = (NX, ny + 2 * c, NZ) if dim == 2.5 else (NX, NZ)
    speeds = (vx, vz, vz) if dim == 2.5 else (vx, vz)
    prof = cp.build_profiles(shape, deltas, c, dt, f0, max(vx, vz), seismic, params, axis_vmax=speeds)
    px, pz = prof[0], prof[-1]
    K = (px.K_half, pz.K_half) if half else (px.K, pz.K)
    a = (px.a_half, pz.a_half) if half else (px.a, pz.a)
    b = (px.b_half, pz.b_half) if half else (px.b, pz.b)
    row, col = NZ // 2, NX // 2  # an interior row (the x profile) and column (the z profile)
    assert np.allclose(K[0], drv["kappa"][row], rtol=1e-12)
    assert np.allclose(a[0], drv["acoef"][row], rtol=1e-12, atol=1e-300)
    assert np.allclose(b[0], drv["bcoef"][row], rtol=1e-12)
    assert np.allclose(K[1], drv["kappa"][:, col], rtol=1e-12)
    assert np.allclose(a[1], drv["acoef"][:, col], rtol=1e-12, atol=1e-300)
    assert np.allclose(b[1], drv["bcoef"][:, col], rtol=1e-12)


def test_wavelets(ref):
    t = ref["wavelet/t"]
    dt = t[1] - t[0]
    assert np.allclose(sy.ricker(len(t), dt, 200.0), ref["wavelet/gaus1"], rtol=1e-12, atol=1e-15)
    for stype in ("gaus0", "gaus1", "gaus2"):
        assert np.allclose(sy.wavelet(t, 200.0, stype), ref[f"wavelet/{stype}"], rtol=1e-12, atol=1e-15)


def test_snapshot_records_read_by_the_reference_reader(ref, tmp_path):
    """read_dat (definitions.py:77-137) on a record written by the snapshot
    writer returns the (NZ, NX) field."""
    snap = ref["read_dat/written"]
    fio.write_record(tmp_path / "s.dat", snap, np.float32)
    assert (tmp_path / "s.dat").read_bytes() == ref["read_dat/bytes"].tobytes()
    assert np.array_equal(ref["read_dat/read"], snap)


def test_block_files_read_by_the_reference_reader(ref, tmp_path):
    """read_block (definitions.py:140-212) on an EM25 block file written by
    em25block.BlockWriter decodes the same fields as em25block.read."""
    raw = ref["read_block/bytes"].tobytes()
    (tmp_path / "b.blk").write_bytes(raw)
    mine = em25block.read(tmp_path / "b.blk")
    meta = ref["read_block/meta"]
    assert mine["metadata"]["first_step"] == meta[4] and mine["metadata"]["step_count"] == meta[5]
    for ch in ("Ex", "Ey", "Ez"):
        theirs = ref[f"read_block/{ch}"]  # (nt, nx, ny, nz)
        assert np.allclose(np.transpose(mine["fields"][ch], (0, 3, 2, 1)), theirs, rtol=0, atol=1e-6)
    assert hashlib.sha256(raw).hexdigest() == hashlib.sha256(ref["read_block/bytes"].tobytes()).hexdigest()
