"""The timed workloads at their full size against the FP64 oracle.

seismic2 on the 400 x 200 firn/ice model (105,600 cells with the CPML,
2000 steps) and electromag2 on the 1000 x 500 layered model (561,600 cells,
6000 steps, 100 receivers), each through its default GPU form (the whole run
on chip) and through one launch per step.  FP32 drift over the full step
count is what these measure: traces within relative L2 1e-5 of the oracle,
final fields within 1e-4 of the largest norm each reached during the run
(by the end of the electromag2 run its fields have decayed to ~1e-4 of
that peak, so their own relative error measures cancellation, not drift).
"""
import numpy as np
import pytest

from oracle import parity as par
from seidart_gb300 import synthetic as sy
from seidart_gb300.solver import FIELDS, FLAG_STREAMING

from helpers import make_solver

pytestmark = pytest.mark.gpu

TRACE_TOL = 1e-5
FIELD_VS_PEAK_TOL = 1e-4

_REF = {}


def _oracle(name, make):
    if name not in _REF:
        case = make()
        _REF[name] = (case,) + par.oracle_case_peaks(case)
    return _REF[name]


@pytest.mark.parametrize("flags", [0, FLAG_STREAMING], ids=["default", "per-step"])
@pytest.mark.parametrize("name,make", [("seismic2_firn_ice", lambda: sy.seismic2_firn_ice(nstep=2000)),
                                       ("electromag2_layers", lambda: sy.electromag2_layers(nstep=6000))])
def test_full_size_workload_matches_oracle(gpu, name, make, flags):
    case, st, ref, peaks = _oracle(name, make)
    s = make_solver(case, gpu, flags)
    try:
        on_chip = s.on_chip()
        assert bool(on_chip) == (flags == 0), "the default form of these grids runs on chip"
        s.run(case.nstep)
        s.status()
        tr = s.traces()
        names = FIELDS[case.grid.kind]
        fields = [s.field(nm) for nm in names]
    finally:
        s.close()
    r = par.compare_run(tr, fields, st, ref, names, peaks)
    assert np.abs(ref).max() > 0
    assert r["rel_l2_traces"] <= TRACE_TOL, r
    assert r["fields_err_vs_peak_norm_max"] <= FIELD_VS_PEAK_TOL, r
