"""Surveys split over ranks: the balanced split of shots, the host-side
gather of their traces and the all-reduce of per-shot gradients.

The CPU tests run two gloo ranks (torch.multiprocessing, spawn) on
127.0.0.1 with the FP64 oracle as the shot runner and the FP64 numpy
adjoint for per-shot gradients, and check that the split run returns
exactly what one process computes.  The GPU tests check the batched shot
runner and the common-offset image against the oracle.
"""
import copy
import dataclasses
import os
import pickle
import socket

import numpy as np
import pytest

from helpers import rel_l2, run_oracle
from seidart_gb300 import ELECTROMAG2, SEISMIC2, cpml as cp, survey
from seidart_gb300 import synthetic as sy


def _shots(n=5, nstep=40):
    base = sy.small_case(ELECTROMAG2, seed=11, nx=40, nz=34, npml=5, nstep=nstep, nrec=3)
    shots = []
    for q in range(n):
        c = copy.copy(base)  # the shots share the model's planes
        c.src_ijk = (8 + 5 * q, 0, 12)
        shots.append(c)
    return shots


def _survey_cases():
    return _shots() + [sy.small_case(SEISMIC2, seed=12, nx=36, nz=30, npml=5, nstep=40, nrec=4)]


def _co_args():
    base = _shots(1)[0]
    src = np.array([[8 + 4 * q, 0, 10] for q in range(5)])
    rec = np.array([[10 + 4 * q, 0, 14] for q in range(5)])
    return base, src, rec


def oracle_runner(cases):
    return [run_oracle(c)[1] for c in cases]


def _numpy_grad(case, residual_fn, index, **kw):
    from oracle import numpy_adjoint as na
    g = case.grid
    prof = cp.pack_profiles(case.profiles)
    src = (case.src_ijk[0], case.src_ijk[2])
    tr, states = na.forward(g.nx, g.nz, g.dx, g.dz, g.dt, prof, case.planes, src, case.srcfn, case.nstep,
                            case.rec_ijk)
    return na.gradient(g.nx, g.nz, g.dx, g.dz, g.dt, prof, case.planes, src, case.srcfn, case.rec_ijk, states,
                       residual_fn(index, tr))


def _residual(index, traces):
    return (1.0 + 0.1 * index) * np.asarray(traces)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, outdir, what):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        if what == "survey":
            res = survey.run_survey(_survey_cases(), runner=oracle_runner)
        elif what == "co":
            base, src, rec = _co_args()
            res = survey.CommonOffset(base.grid, base.planes, base.profiles, base.srcfn, src, rec, "Ez",
                                      runner=oracle_runner).co_run()
        elif what == "device":
            # one process per GPU: each rank's default shot runner gets cuda:{LOCAL_RANK}
            os.environ["LOCAL_RANK"] = str(rank)
            seen = []
            survey.gpu_runner = lambda cases, device=None: (seen.append(device), oracle_runner(cases))[1]
            survey.run_survey(_survey_cases())
            res = (survey.default_device(), seen)
        else:
            res = survey.survey_gradient(_shots(3), _residual, grad_fn=_numpy_grad)
        with open(os.path.join(outdir, f"{what}_{rank}.pkl"), "wb") as f:
            pickle.dump(res, f)
    finally:
        dist.destroy_process_group()


def _spawn(what, tmp_path, world=2):
    import torch.multiprocessing as mp
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path), what), nprocs=world, join=True)
    out = []
    for r in range(world):
        with open(tmp_path / f"{what}_{r}.pkl", "rb") as f:
            out.append(pickle.load(f))
    return out


def test_partition_balances_and_covers():
    costs = [10, 3, 7, 7, 2, 9, 1, 5]
    for n in (1, 2, 3, 5):
        parts = survey.partition(costs, n)
        assert sorted(i for p in parts for i in p) == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs)
        assert parts == survey.partition(costs, n)  # the same split on every rank
    assert survey.partition([], 2) == [[], []]
    assert survey.partition([4, 4, 4, 4], 4) == [[0], [1], [2], [3]]
    with pytest.raises(ValueError):
        survey.partition([1], 0)


def test_channel_index():
    assert survey.channel_index(ELECTROMAG2, "Ez") == 1
    assert survey.channel_index(SEISMIC2, "Vx") == 0
    with pytest.raises(ValueError):
        survey.channel_index(SEISMIC2, "Ex")


def test_single_process_survey_is_the_runner_output():
    cases = _survey_cases()
    got = survey.run_survey(cases, runner=oracle_runner)
    for c, tr in zip(cases, got):
        assert np.array_equal(tr, run_oracle(c)[1])


def test_two_rank_survey_gathers_every_shot(tmp_path):
    res = _spawn("survey", tmp_path)
    assert res[1] is None
    cases = _survey_cases()
    assert len(res[0]) == len(cases)
    for c, tr in zip(cases, res[0]):
        assert np.array_equal(tr, run_oracle(c)[1])


def test_two_rank_common_offset_image(tmp_path):
    res = _spawn("co", tmp_path)
    assert res[1] is None
    base, src, rec = _co_args()
    want = np.stack([run_oracle(dataclasses.replace(base, src_ijk=tuple(s), rec_ijk=r.reshape(1, 3).astype(np.int32)))
                     [1][:, 1, 0] for s, r in zip(src, rec)], axis=1)
    assert res[0].shape == (base.nstep, len(src))
    assert np.array_equal(res[0], want)


def test_two_rank_default_device_follows_local_rank(tmp_path):
    res = _spawn("device", tmp_path)
    for rank, (dev, seen) in enumerate(res):
        assert dev == f"cuda:{rank}"
        assert seen == [f"cuda:{rank}"]


def test_single_process_default_device_is_the_current_one(monkeypatch):
    monkeypatch.setenv("LOCAL_RANK", "3")  # no process group: the current device
    assert survey.default_device() == "cuda"


def test_two_rank_gradient_is_the_sum_over_shots(tmp_path):
    res = _spawn("grad", tmp_path)
    shots = _shots(3)
    want = sum(_numpy_grad(c, _residual, q) for q, c in enumerate(shots))
    for g in res:  # the all-reduced sum is on every rank
        assert g.shape == want.shape
        assert np.abs(g - want).max() <= 1e-12 * np.abs(want).max()


@pytest.mark.gpu
@pytest.mark.parametrize("schedule", ["sequential", "batch"])
def test_gpu_runner_batches_shots_like_the_oracle(gpu, schedule):
    cases = _survey_cases()
    got = survey.run_survey(cases, runner=lambda cs: survey.gpu_runner(cs, schedule=schedule))
    for c, tr in zip(cases, got):
        e = rel_l2(tr, run_oracle(c)[1])
        assert e <= 1e-5, f"{c.name}: rel L2 {e:.2e}"


@pytest.mark.gpu
@pytest.mark.parametrize("schedule", ["sequential", "batch"])
def test_gpu_runner_with_a_model_too_large_for_chip(gpu, schedule):
    """A seismic2 grid too large for the on-chip form (700 x 600 cells) with
    shots and a small model that fit on chip (sequential: each alone in its
    default form; batch: all in one batched launch), all against the
    oracle."""
    from helpers import make_solver
    big = sy.small_case(SEISMIC2, seed=13, nx=700, nz=600, npml=10, nstep=40, nrec=6)
    cases = _survey_cases() + [big]
    with make_solver(big) as s:
        assert s.on_chip() is None
    with make_solver(cases[-2]) as s:
        assert s.on_chip() is not None
    got = survey.run_survey(cases, runner=lambda cs: survey.gpu_runner(cs, schedule=schedule))
    for c, tr in zip(cases, got):
        e = rel_l2(tr, run_oracle(c)[1])
        assert e <= 1e-5, f"{c.name}: rel L2 {e:.2e}"


@pytest.mark.gpu
def test_gpu_common_offset_image(gpu):
    base, src, rec = _co_args()
    co = survey.CommonOffset(base.grid, base.planes, base.profiles, base.srcfn, src, rec, "Ex").co_run()
    ref = survey.CommonOffset(base.grid, base.planes, base.profiles, base.srcfn, src, rec, "Ex",
                              runner=oracle_runner).co_run()
    assert co.shape == ref.shape == (base.nstep, len(src))
    e = rel_l2(co, ref)
    assert e <= 1e-5, f"co_image rel L2 {e:.2e}"
