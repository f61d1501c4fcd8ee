"""Golden fixtures (tests/golden/*.npz, made by make_golden.py from the oracle):
the oracle must reproduce them exactly (CPU) and the GPU kernels within the
parity tolerance (GPU)."""
import numpy as np
import pytest

from golden.make_golden import SPECS, VARIANTS, case_of, path_of
from helpers import make_solver, rel_l2, run_oracle
from seidart_gb300 import KIND_NAMES

IDS = [f"{KIND_NAMES[s[0]]}_s{s[1]}{VARIANTS[s[7]][0]}" for s in SPECS]


@pytest.mark.parametrize("spec", SPECS, ids=IDS)
def test_oracle_reproduces_golden(spec):
    g = np.load(path_of(spec))
    assert tuple(g["spec"]) == tuple(spec)
    st, tr, norm, _ = run_oracle(case_of(spec))
    assert rel_l2(tr, g["traces"]) < 1e-12
    assert np.allclose([np.linalg.norm(f) for f in st.fields], g["field_norms"], rtol=1e-12, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("spec", SPECS, ids=IDS)
def test_gpu_matches_golden(gpu, spec):
    g = np.load(path_of(spec))
    case = case_of(spec)
    with make_solver(case) as s:
        s.run(case.nstep)
        s.status()
        assert rel_l2(s.traces(), g["traces"]) <= 1e-5
        norms = [np.linalg.norm(s.field(q).astype(np.float64)) for q in range(len(g["field_norms"]))]
        assert np.allclose(norms, g["field_norms"], rtol=1e-5, atol=0)
