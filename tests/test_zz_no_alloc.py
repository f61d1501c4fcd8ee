"""The electromag2 entry point for callers that cannot allocate device memory.

sfd_electromag2_run_static keeps the whole device state of a shot in a
fixed-size array inside the library, so a caller that has no way to call
cudaMalloc (an application that owns all device allocations, a plugin in a
process that forbids new ones) can still run a shot: it passes host inputs
and gets host traces back.  This test calls it through the C ABI twice in a
row (the second call must not see the first call's state) and compares both
against the ordinary handle-based entry point.  It sits in a file of its own,
collected last, and passes alone in a fresh process as well as after the
other tests.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import make_solver, rel_l2, run_oracle
from seidart_gb300 import ELECTROMAG2, _lib, cpml as cp, synthetic as sy
from seidart_gb300._lib import SfdConfig

pytestmark = pytest.mark.gpu


def _static_run(L, case, flags=0):
    g = case.grid
    cfg = SfdConfig(kind=ELECTROMAG2, nx=g.nx, ny=1, nz=g.nz, npml=g.npml, nstep=case.nstep,
                    nrec=len(case.rec_ijk), flags=flags, dx=g.dx, dy=g.dy, dz=g.dz, dt=g.dt)
    model = np.ascontiguousarray(case.planes, dtype=np.float64)
    prof = cp.pack_profiles(case.profiles)
    src = np.ascontiguousarray(case.srcfn, dtype=np.float64)
    rec = np.ascontiguousarray(case.rec_ijk, dtype=np.int32)
    out = np.full((case.nstep, 2, len(rec)), np.nan, dtype=np.float32)
    dp, fp, ip = C.POINTER(C.c_double), C.POINTER(C.c_float), C.POINTER(C.c_int32)
    rc = L.sfd_electromag2_run_static(C.byref(cfg), model.ctypes.data_as(dp), prof.ctypes.data_as(dp),
                                      case.src_ijk[0], case.src_ijk[2], src.ctypes.data_as(dp),
                                      rec.ctypes.data_as(ip), out.ctypes.data_as(fp), None)
    return rc, out


def test_static_entry_point_matches_handle_entry_point(gpu):
    import torch
    L = _lib.lib()
    cases = [sy.small_case(ELECTROMAG2, seed=61, nx=52, nz=44, npml=6, nstep=120, nrec=9),
             sy.small_case(ELECTROMAG2, seed=62, nx=47, nz=39, npml=5, nstep=100, nrec=7)]
    for case in cases:  # two calls in a row on the shared array
        torch.cuda.synchronize()
        rc, tr = _static_run(L, case)
        assert rc == 0, L.sfd_last_error().decode()
        with make_solver(case) as s:
            s.run(case.nstep)
            s.status()
            ref = s.traces()
        assert np.all(np.isfinite(tr))
        assert rel_l2(tr, ref) <= 1e-5
        assert rel_l2(tr, run_oracle(case)[1]) <= 1e-5


def test_static_entry_point_takes_no_device_memory(gpu):
    """After a first call (which loads the library's module and its array),
    a call leaves the device's free memory unchanged: it allocates nothing."""
    import torch
    L = _lib.lib()
    case = sy.small_case(ELECTROMAG2, seed=63, nx=50, nz=42, npml=6, nstep=80, nrec=5)
    rc, _ = _static_run(L, case)
    assert rc == 0, L.sfd_last_error().decode()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    rc, tr = _static_run(L, case)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert rc == 0, L.sfd_last_error().decode()
    assert free1 == free0
    assert rel_l2(tr, run_oracle(case)[1]) <= 1e-5


def test_static_entry_point_rejects_other_forms(gpu):
    L = _lib.lib()
    case = sy.small_case(ELECTROMAG2, seed=64, nx=40, nz=36, npml=5, nstep=20, nrec=3)
    for flags in (2, 4, 1 << 20):
        rc, _ = _static_run(L, case, flags=flags)
        assert rc == _lib.SFD_ERR_BAD_ARG
        assert "two-pass" in L.sfd_last_error().decode()
    rc, _ = _static_run(L, case, flags=1)  # the form it runs, named explicitly
    assert rc == 0, L.sfd_last_error().decode()


def test_static_entry_point_rejects_oversized_state(gpu):
    L = _lib.lib()
    n = 1200  # 3 fields + 4 coefficient planes of 1200 x 1216 floats alone exceed 32 MiB
    cfg = SfdConfig(kind=ELECTROMAG2, nx=n, ny=1, nz=n, npml=5, nstep=20, nrec=2, flags=0,
                    dx=0.05, dy=0.05, dz=0.05, dt=1e-11)
    dummy = np.zeros(6 * n * n)
    prof = np.zeros(6 * 2 * n)
    src = np.zeros(40)
    rec = np.zeros(6, dtype=np.int32)
    out = np.zeros(80, dtype=np.float32)
    dp, fp, ip = C.POINTER(C.c_double), C.POINTER(C.c_float), C.POINTER(C.c_int32)
    rc = L.sfd_electromag2_run_static(C.byref(cfg), dummy.ctypes.data_as(dp), prof.ctypes.data_as(dp), 10, 10,
                                      src.ctypes.data_as(dp), rec.ctypes.data_as(ip), out.ctypes.data_as(fp), None)
    assert rc == _lib.SFD_ERR_BAD_ARG
    assert "static scratch" in L.sfd_last_error().decode()
