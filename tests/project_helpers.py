"""Write a SeidarT-style project directory (JSON + Fortran-record .dat files)
from a synthetic case, the way the driver's Model.build / Model.run do
(src/seidart/routines/classes.py:608-750, 787-924)."""
import json

import numpy as np

from seidart_gb300 import fortran_io as fio
from seidart_gb300.solver import MODEL_PLANES, is_25d
from seidart_gb300._lib import SEISMIC2, SEISMIC25

FILE_OF = {"eps11": "e11", "eps12": "e12", "eps13": "e13", "eps22": "e22", "eps23": "e23", "eps33": "e33",
           "sig11": "s11", "sig12": "s12", "sig13": "s13", "sig22": "s22", "sig23": "s23", "sig33": "s33"}


def write_project(case, workdir, receivers_m=None, stress=None, density_gradient=None):
    """``stress``: dict of seismicsource{xx,yy,zz,xy,xz,yz}.dat time series to
    write; ``density_gradient``: the interior (nx, nz) factors the driver's
    airsurf writes (definitions.py:475-557), saved the way it saves them."""
    g = case.grid
    c = g.npml
    seismic = g.kind in (SEISMIC2, SEISMIC25)
    three = is_25d(g.kind)
    xind, yind, zind = case.src_ijk[0] - c, (case.src_ijk[1] - c) if three else 0, case.src_ijk[2] - c
    prj = {
        "Domain": {"dim": 2.5 if three else 2, "nx": g.nx - 2 * c, "ny": (g.ny - 2 * c) if three else 1,
                   "nz": g.nz - 2 * c, "dx": g.dx, "dy": g.dy, "dz": g.dz, "cpml": c, "nmats": 1,
                   "alpha_max_scalar": 1.0, "kappa_max": 5, "NP": 2, "NPA": 2, "Rcoef": 0.001},
        ("Seismic" if seismic else "Electromagnetic"): {
            "Source": {"dt": g.dt, "time_steps": case.nstep, "xind": xind, "yind": yind, "zind": zind,
                       "source_frequency": case.f0}},
    }
    with open(f"{workdir}/project.json", "w") as f:
        json.dump(prj, f)
    for name, plane in zip(MODEL_PLANES[g.kind], case.planes):
        fio.write_record(f"{workdir}/{FILE_OF.get(name, name)}.dat", plane, np.float64)
    stem = "seismicsource" if seismic else "electromagneticsource"
    comps = ["x", "y", "z"] if three else ["x", "z"]
    for q, s in zip(comps, case.srcfn):
        fio.write_record(f"{workdir}/{stem}{q}.dat", s, np.float64)
    for name, series in (stress or {}).items():
        fio.write_record(f"{workdir}/seismicsource{name}.dat", np.asarray(series), np.float64)
    if density_gradient is not None:  # a C-order (nx, nz) record, no transpose (definitions.py:554-556)
        g = np.ascontiguousarray(density_gradient, dtype=np.float64)
        with open(f"{workdir}/density_gradient.dat", "wb") as f:
            n = np.array([g.nbytes], dtype=np.int32).tobytes()
            f.write(n + g.tobytes() + n)
    if receivers_m is not None:
        with open(f"{workdir}/receivers.csv", "w") as f:
            f.write("X,Y,Z\n")
            for x, y, z in receivers_m:
                f.write(f"{x},{y},{z}\n")
    return f"{workdir}/project.json", (xind, yind, zind)
