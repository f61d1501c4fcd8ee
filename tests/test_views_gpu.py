"""Zero-copy torch views of the fields (FDTDSolver.field_tensor, through
sfd_field_device) against the host copies (sfd_get_field), for every form:
single-pass 2-D handles alternate between two copies of their fields, so
the view follows the current one after odd and even runs."""
import numpy as np
import pytest

from helpers import make_solver
from seidart_gb300 import ELECTROMAG2, ELECTROMAG25, SEISMIC2, SEISMIC25
from seidart_gb300 import synthetic as sy
from seidart_gb300.solver import FIELDS, FLAG_STREAMING, FLAG_TWO_PASS

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,flags", [(ELECTROMAG2, 0), (ELECTROMAG2, FLAG_STREAMING), (ELECTROMAG2, FLAG_TWO_PASS),
                                        (SEISMIC2, 0), (SEISMIC2, FLAG_STREAMING), (SEISMIC25, 0),
                                        (ELECTROMAG25, 0)])
def test_field_views_match_host_copies(gpu, kind, flags):
    three = kind in (SEISMIC25, ELECTROMAG25)
    case = sy.small_case(kind, seed=41, nx=45, nz=39, ny=21, npml=5, nstep=60)
    with make_solver(case, flags=flags) as s:
        for n in (7, 16):  # odd, then odd + even steps
            s.run(n)
            s.status()
            for name in FIELDS[kind]:
                v = s.field_tensor(name)
                assert tuple(v.shape) == ((case.grid.nz, case.grid.ny, case.grid.nx) if three else
                                          (case.grid.nz, case.grid.nx))
                assert v.device.type == "cuda"
                assert np.array_equal(v.cpu().numpy(), s.field(name)), name
