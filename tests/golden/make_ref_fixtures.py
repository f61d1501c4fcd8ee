"""Fixtures made by the reference's own Python code -- pins for the inputs,
formats and host-side formulas of the solver path.

The reference's solver (the Fortran backend) cannot be built or run here, but
the Python driver that prepares its inputs and reads its outputs can be
imported once a few plotting/IO dependencies it imports at module level
(pandas, matplotlib, glob2, zstandard, pyevtk, trimesh, PIL) are replaced by
stubs; none of them is used on the code paths called here (the material
tables are given as a minimal stand-in of the pandas.DataFrame API those
paths touch).  numpy 2 dropped np.row_stack, an alias of np.vstack that
airsurf calls; the alias is restored.  read_block calls a helper,
_open_binary_maybe_gzip, that the reference's source never defines; the
script supplies one that does what the name says (gzip.open for .gz files,
open otherwise).  This script runs,
in a scratch directory:

* ``Model.build`` (src/seidart/routines/classes.py:393-547) of small seismic
  2-D, electromagnetic 2-D and seismic 2.5-D models: the time step
  (classes.py:469-485 with the Christoffel velocities of :1070-1121), the
  source files (sourcefunction.py:239-383, with the 'ac', 'tnt' and 'dc'
  source types), the 2-D CPML fields (definitions.py:560-998), the per-cell
  material files (classes.py:608-750) and density_gradient.dat
  (definitions.py:475-557);
* ``wavelet`` (sourcefunction.py:25-57) for the three Gaussian wavelets;
* ``read_dat`` and ``read_block`` (definitions.py:77-212) on a snapshot record
  and an EM25 block file written by this repository's writers.

It stores every file the driver wrote (raw bytes) and the values it computed
in tests/golden/reference_inputs.npz, which tests/test_reference_fixtures.py
compares with this repository's CLI loader, CPML builder, time step,
wavelet, snapshot writer and block reader.  Only this script reads the
reference tree; the tests read the fixture file.

Usage:  python tests/golden/make_ref_fixtures.py [reference root (default /root/reference)]
"""
from __future__ import annotations

import io
import os
import sys
import tempfile
import types
from contextlib import redirect_stdout
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
OUT = HERE / "reference_inputs.npz"


# ---------------------------------------------------------------------------
# stand-ins for the modules the reference imports but these paths never use

class _Row(dict):
    """One material row (pandas.Series stand-in): string keys to numbers."""


class _Col:
    def __init__(self, values):
        self.values = np.asarray(values)

    def min(self):
        return float(np.min(self.values))


class _Frame:
    """The part of pandas.DataFrame the build path uses: columns, index,
    .loc[row], frame[col].values, frame[[cols]].min().min(), frame * scalar."""

    def __init__(self, data: dict):
        self.data = {k: np.asarray(v, dtype=np.float64) for k, v in data.items()}
        self.columns = list(self.data)
        self.index = list(range(len(next(iter(self.data.values())))))
        frame = self

        class _Loc:
            def __getitem__(self, i):
                return _Row({k: float(v[i]) for k, v in frame.data.items()})

        self.loc = _Loc()

    def __getitem__(self, key):
        if isinstance(key, list):
            return _Frame({k: self.data[k] for k in key})
        return _Col(self.data[key])

    def min(self):
        return _Col([float(np.min(v)) for v in self.data.values()])

    def __mul__(self, s):
        return _Frame({k: v * s for k, v in self.data.items()})


class _AnyModule(types.ModuleType):
    def __getattr__(self, k):
        if k.startswith("__"):
            raise AttributeError(k)
        return type(k, (), {})


def import_reference(root: Path):
    names = ["pandas", "glob2", "zstandard", "matplotlib", "matplotlib.pyplot", "matplotlib.image",
             "matplotlib.animation", "matplotlib.figure", "matplotlib.axes", "matplotlib.colors", "matplotlib.cm",
             "mpl_toolkits", "mpl_toolkits.mplot3d", "pyevtk", "pyevtk.hl", "trimesh", "PIL", "PIL.Image"]
    for n in names:
        sys.modules.setdefault(n, _AnyModule(n))
    for n in names:
        if "." in n:
            parent, child = n.rsplit(".", 1)
            setattr(sys.modules[parent], child, sys.modules[n])
    pd = sys.modules["pandas"]
    pd.Series, pd.DataFrame = _Row, _Frame
    pd.concat = lambda rows: _Row({k: v for r in rows for k, v in r.items()})
    if not hasattr(np, "row_stack"):  # removed from numpy 2; it was an alias of vstack, which airsurf uses
        np.row_stack = np.vstack
    sys.path.insert(0, str(root / "src"))
    import seidart.routines.classes as classes
    import seidart.routines.definitions as definitions
    import seidart.routines.sourcefunction as sourcefunction
    if not hasattr(definitions, "_open_binary_maybe_gzip"):
        # read_block (definitions.py:154) calls this helper, which the
        # reference's source never defines; supply what its name says
        import gzip

        def _open_binary_maybe_gzip(fn):
            return gzip.open(fn, "rb") if str(fn).endswith(".gz") else open(fn, "rb")

        definitions._open_binary_maybe_gzip = _open_binary_maybe_gzip
    return classes, definitions, sourcefunction


# ---------------------------------------------------------------------------

VOIGT = ["c11", "c12", "c13", "c14", "c15", "c16", "c22", "c23", "c24", "c25", "c26", "c33", "c34", "c35",
         "c36", "c44", "c45", "c46", "c55", "c56", "c66"]


def _iso(lam, mu):
    c = dict.fromkeys(VOIGT, 0.0)
    c["c11"] = c["c22"] = c["c33"] = lam + 2 * mu
    c["c12"] = c["c13"] = c["c23"] = lam
    c["c44"] = c["c55"] = c["c66"] = mu
    return c


def _geometry(nx, nz):
    """(nx, nz) material ids: material 1 (air) over the top rows, 2 (firn), 0 (ice)."""
    g = np.zeros((nx, nz), dtype=int)
    g[:, :4] = 1
    g[:, 4:9] = 2
    g[nx // 2:, 9:12] = 2
    return g


class Domain:
    def __init__(self, dim, nx, nz, ny=1, d=(0.5, 0.5, 0.5), cpml=5):
        self.dim = float(dim)
        self.nx, self.ny, self.nz = nx, ny, nz
        self.dx, self.dy, self.dz = d
        self.cpml = cpml
        self.geometry = _geometry(nx, nz)
        self.nmats = 3
        self.alpha_max_scalar, self.kappa_max, self.NP, self.NPA, self.Rcoef = 1.0, 5.0, 2.0, 2.0, 0.001


class Material:
    material = np.array(["ice", "air", "firn"])


def seismic_model(classes, source_type, f0=200.0, steps=120, angles=(0.0, 0.0, 0.0)):
    m = classes.Model()
    m.is_seismic = True
    m.f0, m.time_steps = f0, steps
    m.x, m.y, m.z = 10.0, 0.0, 6.0
    m.phi, m.theta, m.psi = angles  # strike, dip, rake of a double couple
    m.source_amplitude, m.source_wavelet, m.source_type = 1.0, "gaus1", source_type
    ice = dict(_iso(6.0e9, 3.0e9), c33=15.0e9, c13=5.8e9, c11=13.9e9, c55=3.0e9, rho=917.0)
    air = dict(_iso(1.42e5, 0.0), rho=1.2)
    firn = dict(_iso(1.0e9, 1.5e9), rho=500.0)
    m.stiffness_coefficients = _Frame({k: [ice[k], air[k], firn[k]] for k in VOIGT + ["rho"]})
    m.attenuation_coefficients = _Frame({"gamma_x": [1e-5, 0.0, 2e-5], "gamma_y": [0.0, 0.0, 0.0],
                                         "gamma_z": [3e-5, 0.0, 1e-5], "reference_frequency": [f0, f0, f0]})
    return m


def em_model(classes, f0=100e6, steps=120):
    m = classes.Model()
    m.is_seismic = False
    m.f0, m.time_steps = f0, steps
    m.x, m.y, m.z = 10.0, 0.0, 6.0
    m.theta, m.phi, m.psi = 0.0, 0.0, 0.0
    m.source_amplitude, m.source_wavelet, m.source_type = 1.0, "gaus1", "ac"
    eps = {"e11": [3.2, 1.0, 1.8], "e12": [0.0, 0.0, 0.0], "e13": [0.02, 0.0, 0.01], "e22": [3.2, 1.0, 1.8],
           "e23": [0.0, 0.0, 0.0], "e33": [3.15, 1.0, 1.9]}
    sig = {"s11": [1e-5, 0.0, 1e-6], "s12": [0.0, 0.0, 0.0], "s13": [0.0, 0.0, 0.0], "s22": [1e-5, 0.0, 1e-6],
           "s23": [0.0, 0.0, 0.0], "s33": [2e-5, 0.0, 1e-6]}
    m.permittivity_coefficients = _Frame(eps)
    m.conductivity_coefficients = _Frame(sig)
    return m


def _files(wd: Path):
    return {p.name: p.read_bytes() for p in sorted(wd.glob("*.dat"))}


def build_case(classes, model, domain):
    """Run Model.build in a scratch directory; return (dt, {file: bytes},
    velocities) with the per-material maximum velocities over all directions
    (the time step's) and along x and along z (the CPML's, definitions.py:
    613-620)."""
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as td:
        os.chdir(td)
        try:
            with redirect_stdout(io.StringIO()):
                model.build(Material(), domain, recompute_tensors=False, write_tensor=True)
            files = _files(Path(td))
        finally:
            os.chdir(cwd)
    vel = {}
    for key, dirs in (("all", None), ("x", "x"), ("z", "z")):
        model.compute_max_velocities(dim=domain.dim, directions=dirs)
        vel[key] = dict(model.max_velocity_per_material)
    return model.dt, files, vel


def main():
    root = Path(sys.argv[1]) if len(sys.argv) > 1 else Path("/root/reference")
    classes, definitions, sourcefunction = import_reference(root)
    out = {}

    cases = {
        "seismic2_tnt": (seismic_model(classes, "tnt"), Domain(2, 40, 30)),
        "seismic2_ac": (seismic_model(classes, "ac"), Domain(2, 40, 30)),
        "seismic2_dc": (seismic_model(classes, "dc", angles=(30.0, 60.0, 45.0)), Domain(2, 40, 30)),
        "em2": (em_model(classes), Domain(2, 40, 30, d=(0.05, 0.05, 0.05))),
        "seismic25_tnt": (seismic_model(classes, "tnt"), Domain(2.5, 32, 24, ny=12, d=(1.0, 1.0, 1.0), cpml=4)),
    }
    for name, (model, dom) in cases.items():
        dt, files, vel = build_case(classes, model, dom)
        out[f"{name}/dt"] = np.float64(dt)
        out[f"{name}/cfl"] = np.float64(model.CFL)
        for key, v in vel.items():  # [material] maximum velocity (EM: its inverse, as the driver keeps it)
            out[f"{name}/vmax_{key}"] = np.array([v[k] for k in sorted(v)], dtype=np.float64)
        out[f"{name}/geometry"] = dom.geometry
        out[f"{name}/domain"] = np.array([dom.dim, dom.nx, dom.ny, dom.nz, dom.dx, dom.dy, dom.dz, dom.cpml,
                                          dom.alpha_max_scalar, dom.kappa_max, dom.NP, dom.NPA, dom.Rcoef])
        out[f"{name}/source"] = np.array([model.f0, model.time_steps, model.x, model.y, model.z])
        out[f"{name}/files"] = np.array(sorted(files))
        for fn, data in files.items():
            out[f"{name}/file/{fn}"] = np.frombuffer(data, dtype=np.uint8)

    # the Gaussian wavelets
    t = np.arange(400) * 2.5e-5
    for stype in ("gaus0", "gaus1", "gaus2"):
        out[f"wavelet/{stype}"] = sourcefunction.wavelet(t, 200.0, stype)
    out["wavelet/t"] = t

    # the reference's readers on files written by this repository
    sys.path.insert(0, str(ROOT))
    from seidart_gb300 import em25block
    from seidart_gb300 import fortran_io as fio
    rng = np.random.default_rng(9)
    snap = rng.standard_normal((30, 40)).astype(np.float32)  # (NZ, NX), x fastest on disk
    blk_fields = {ch: rng.standard_normal((3, 6, 5, 4)).astype(np.float32) for ch in ("Ex", "Ey", "Ez")}
    with tempfile.TemporaryDirectory() as td:
        fn = Path(td) / "Vx.000001.10.12.dat"
        fio.write_record(fn, snap, np.float32)
        dom = types.SimpleNamespace(dim=2, nx=40, ny=1, nz=30)
        out["read_dat/written"] = snap
        out["read_dat/read"] = definitions.read_dat(str(fn), dom, single=True)
        out["read_dat/bytes"] = np.frombuffer(fn.read_bytes(), dtype=np.uint8)
        bn = Path(td) / "block.blk"
        w = em25block.BlockWriter(bn, 4, 5, 6, 7, ["Ex", "Ey", "Ez"])  # nx, ny, nz, first step, channels
        for s in range(3):
            for ch in ("Ex", "Ey", "Ez"):
                f = blk_fields[ch][s]  # (nz, ny, nx)
                lo, hi = float(f.min()), float(f.max())
                codes = np.rint((f - lo) / (hi - lo) * 65534.0 - 32767.0).astype(np.int16)
                w.add(7 + s, ch, lo, hi, codes.ravel())
        w.close()
        blk = definitions.read_block(str(bn))
        out["read_block/bytes"] = np.frombuffer(bn.read_bytes(), dtype=np.uint8)
        for ch, v in blk["fields"].items():
            out[f"read_block/{ch}"] = v  # (nt, nx, ny, nz) as the reference returns them
        out["read_block/meta"] = np.array([blk["metadata"][k] for k in
                                           ("version", "nx", "ny", "nz", "first_step", "step_count",
                                            "component_count")])
    np.savez_compressed(OUT, **out)
    print(OUT, len(out), "arrays")


if __name__ == "__main__":
    main()
