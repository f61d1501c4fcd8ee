"""Helpers shared by the tests: run one case on the oracle and on the GPU."""
import numpy as np

import oracle
from seidart_gb300 import cpml as cp


def rel_l2(a, b, floor=0.0):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = max(np.linalg.norm(b), floor)
    if den == 0.0:
        return float(np.linalg.norm(a))
    return float(np.linalg.norm(a - b) / den)


def run_oracle(case, nsteps=None, state=None):
    n = case.nstep if nsteps is None else nsteps
    return oracle.run(case.grid.kind, case.grid, case.planes, cp.pack_profiles(case.profiles), case.src_ijk,
                      case.srcfn, case.rec_ijk, n, state=state)


def make_solver(case, device="cuda", flags=0):
    from seidart_gb300.solver import FDTDSolver
    s = FDTDSolver(case.grid, case.nstep, len(case.rec_ijk), device=device, flags=flags)
    s.set_model(case.planes)
    s.set_cpml(case.profiles)
    s.set_source(case.src_ijk, case.srcfn)
    s.set_receivers(case.rec_ijk)
    return s
