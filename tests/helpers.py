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
    """The FP64 oracle on ``case`` with its physics options (stress source,
    legacy quirks, density method)."""
    from oracle.parity import case_options
    n = case.nstep if nsteps is None else nsteps
    return oracle.run(case.grid.kind, case.grid, case.planes, cp.pack_profiles(case.profiles), case.src_ijk,
                      case.srcfn, case.rec_ijk, n, state=state, **case_options(case))


def make_solver(case, device="cuda", flags=0):
    from seidart_gb300.solver import FDTDSolver
    s = FDTDSolver(case.grid, case.nstep, len(case.rec_ijk), device=device, flags=flags, **case.solver_options())
    s.set_model(case.planes)
    s.set_cpml(case.profiles)
    s.set_source(case.src_ijk, case.srcfn)
    if getattr(case, "stress_srcfn", None) is not None:
        s.set_stress_source(case.src_ijk, case.stress_srcfn)
    s.set_receivers(case.rec_ijk)
    return s
