"""Bounded device waits on the GPU.

The on-chip runs poll neighbouring tiles' edge values, the batched kernel
meets at a grid barrier every step, and the 2.5-D kernels wait for their
TMA-staged planes.  Each wait gives up after a limit
(sfd_set_wait_limit / sfd_batch_set_wait_limit, 2 s by default), records the
failure, and every tile or block leaves the kernel; the host reads
SFD_ERR_TIMEOUT.  These tests make the waits run out on purpose with the
library's test aid (the waits expect values that nothing writes), with a 1 ms
limit, and check the status.  Then they check that the context is still
usable: after a reset, a run at the default limit matches the FP64 oracle.
No kernel faults or hangs here: every wait is bounded by the limit.
"""
import pytest

from helpers import make_solver, rel_l2, run_oracle
from seidart_gb300 import ELECTROMAG2, ELECTROMAG25, SEISMIC2, SEISMIC25, _lib
from seidart_gb300 import synthetic as sy
from seidart_gb300._lib import SFD_ERR_TIMEOUT, SfdError
from seidart_gb300.batch import Batch

pytestmark = pytest.mark.gpu

LIMIT_NS = 1_000_000  # 1 ms


def _timeout_then_recover(case, steps):
    L = _lib.lib()
    with make_solver(case) as s:
        assert s.on_chip() is not None, "the case must run on chip"
        s.set_wait_limit(LIMIT_NS)
        assert L.sfd_test_stall_waits(s._h, 1) == 0
        s.run(steps)
        with pytest.raises(SfdError) as e:
            s.status()
        assert e.value.code == SFD_ERR_TIMEOUT
        assert "did not answer" in str(e.value)
        # the context and the handle stay usable
        assert L.sfd_test_stall_waits(s._h, 0) == 0
        s.set_wait_limit(0)
        s.reset()
        s.run(case.nstep)
        s.status()
        tr = s.traces()
    _, ref, _, _ = run_oracle(case)
    assert rel_l2(tr, ref) <= 1e-5


def test_electromag2_on_chip_exchange_times_out(gpu):
    _timeout_then_recover(sy.electromag2_layers(nstep=150), 60)


def test_seismic2_on_chip_exchange_times_out(gpu):
    _timeout_then_recover(sy.seismic2_firn_ice(nstep=150), 60)


def test_batch_grid_barrier_times_out(gpu):
    L = _lib.lib()
    cases = [sy.small_case(ELECTROMAG2, seed=70 + q, nx=45 + 5 * q, nz=39, npml=5, nstep=60) for q in range(2)]
    cases += [sy.small_case(SEISMIC2, seed=80, nx=41, nz=47, npml=6, nstep=60)]
    solvers = [make_solver(c) for c in cases]
    b = Batch(solvers)
    try:
        b.set_wait_limit(LIMIT_NS)
        assert L.sfd_batch_test_stall_waits(b._b, 1) == 0
        b.run(20)
        with pytest.raises(SfdError) as e:
            b.status()
        assert e.value.code == SFD_ERR_TIMEOUT
        assert L.sfd_batch_test_stall_waits(b._b, 0) == 0
        b.set_wait_limit(0)
        b.reset()
        b.run(60)
        b.status()
        for c, s in zip(cases, solvers):
            _, ref, _, _ = run_oracle(c)
            assert rel_l2(s.traces(), ref) <= 1e-5
    finally:
        b.close()
        for s in solvers:
            s.close()


@pytest.mark.parametrize("kind", [SEISMIC25, ELECTROMAG25], ids=["seismic25", "electromag25"])
def test_2p5d_staged_tiles_time_out(gpu, kind):
    """The 2.5-D kernels wait on mbarriers for their TMA-staged planes; with
    the test aid each stage expects 16 bytes that never arrive."""
    L = _lib.lib()
    case = sy.small_case(kind, seed=5, nx=70, nz=36, ny=30, npml=5, nstep=40)
    with make_solver(case) as s:
        s.set_wait_limit(LIMIT_NS)
        assert L.sfd_test_stall_waits(s._h, 1) == 0
        s.run(3)
        with pytest.raises(SfdError) as e:
            s.status()
        assert e.value.code == SFD_ERR_TIMEOUT
        assert "staged tile" in str(e.value)
        assert L.sfd_test_stall_waits(s._h, 0) == 0
        s.set_wait_limit(0)
        s.reset()
        s.run(case.nstep)
        s.status()
        tr = s.traces()
    _, ref, _, _ = run_oracle(case)
    assert rel_l2(tr, ref) <= 1e-5

