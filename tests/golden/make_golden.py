"""Regenerate the golden fixtures of tests/golden/ from the FP64 oracle.

The reference publishes no golden vectors for its solvers and its Fortran
cannot be compiled here, so these fixtures pin the oracle's own output for a
few seeded small models (regression anchors for the oracle and parity targets
for the GPU kernels), in the default corrected physics and in the seismic
physics variants (legacy quirks; harmonic and geometric density with a
moment-tensor source).  Each .npz stores the case spec, the receiver traces and
the L2 norm of every final field.

Usage:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from helpers import run_oracle  # noqa: E402
from seidart_gb300 import ELECTROMAG2, ELECTROMAG25, SEISMIC2, SEISMIC25, KIND_NAMES  # noqa: E402
from seidart_gb300 import synthetic as sy  # noqa: E402

SPECS = [
    # kind, seed, nx, nz, ny, npml, nstep, physics variant (VARIANTS)
    (ELECTROMAG2, 11, 41, 35, 1, 6, 150, 0),
    (SEISMIC2, 11, 41, 35, 1, 6, 150, 0),
    (SEISMIC25, 11, 33, 27, 19, 5, 80, 0),
    (ELECTROMAG25, 11, 33, 27, 19, 5, 80, 0),
    (SEISMIC2, 11, 41, 35, 1, 6, 150, 1),
    (SEISMIC25, 11, 33, 27, 19, 5, 80, 1),
    (SEISMIC2, 12, 37, 44, 1, 6, 150, 2),
    (SEISMIC25, 12, 29, 31, 21, 5, 80, 3),
]
# seismic physics options: (name, legacy quirks, density method, stress source)
VARIANTS = {0: ("", False, "arithmetic", False), 1: ("_legacy", True, "arithmetic", False),
            2: ("_harmonic_stress", False, "harmonic", True), 3: ("_geometric_stress", False, "geometric", True)}


def stress_source(kind, w):
    """A moment-tensor source with every component nonzero: sigma xx, zz, xz
    (2-D) or xx, yy, zz, xy, xz, yz (2.5-D), scaled copies of the wavelet w."""
    f = (1.0, 0.8, 0.3) if kind == SEISMIC2 else (1.0, 0.8, 1.2, 0.3, -0.2, 0.1)
    return np.stack([a * w for a in f])


def case_of(spec):
    kind, seed, nx, nz, ny, npml, nstep, var = spec
    case = sy.small_case(kind, seed=seed, nx=nx, nz=nz, ny=ny if ny > 1 else 24, npml=npml, nstep=nstep)
    _, legacy, density, stress = VARIANTS[var]
    case.legacy, case.density = legacy, density
    if stress:
        case.stress_srcfn = stress_source(kind, 1e6 * case.srcfn[0])
    return case


def path_of(spec):
    return os.path.join(HERE, f"{KIND_NAMES[spec[0]]}_s{spec[1]}{VARIANTS[spec[7]][0]}.npz")


def main():
    for spec in SPECS:
        case = case_of(spec)
        st, tr, norm, blew = run_oracle(case)
        assert not blew
        np.savez_compressed(path_of(spec), spec=np.array(spec, dtype=np.int64), traces=tr,
                            field_norms=np.array([np.linalg.norm(f) for f in st.fields]), maxnorm=norm)
        print(path_of(spec), tr.shape)


if __name__ == "__main__":
    main()
