"""Surveys: many shots (and models) advanced together, and split over GPUs.

The reference's common-offset survey runs one solver process per source
position and reads one receiver column back per shot
(``src/seidart/simulations/common_offset.py:143-284``: ``process_source``
builds and runs the model for source i and extracts receiver i;
``co_run`` stacks the columns into ``co_image[time step, source]``).

Here the shots a process owns run on the GPU one after another, each in its
fastest form (:func:`gpu_runner`; on chip where the grid fits), or, on
request, together in one batched launch (:mod:`seidart_gb300.batch`);
shots of one model share its coefficient planes on the device.  Shots are independent, so several GPUs -- one
process per GPU under ``torch.distributed`` -- split them with no exchange
on the data path:

* :func:`partition` assigns the shots to ranks, balancing cells x steps;
* each rank runs its own shots;
* rank 0 gathers the results on the host (:func:`gather_to_root`).

The gradient of a misfit summed over shots is the sum of the per-shot
gradients: each rank adds up its own shots', and one all-reduce
(:func:`allreduce_sum`) adds the ranks' sums.  Nothing here needs a GPU
except the default shot runners; the distribution logic runs on any
``torch.distributed`` backend (gloo on CPU, nccl on GPUs).
"""
from __future__ import annotations

from typing import Callable, Dict, List, Optional, Sequence

import numpy as np

from ._lib import ELECTROMAG2, ELECTROMAG25, SEISMIC2, SEISMIC25

# Receiver channels of each solver, in trace order.
CHANNELS = {
    SEISMIC2: ("Vx", "Vz"),
    ELECTROMAG2: ("Ex", "Ez"),
    SEISMIC25: ("Vx", "Vy", "Vz"),
    ELECTROMAG25: ("Ex", "Ey", "Ez"),
}


def channel_index(kind: int, channel: str) -> int:
    """Trace channel of ``channel`` ('Vx', 'Ez', ...) for a solver kind."""
    names = CHANNELS[kind]
    if channel not in names:
        raise ValueError(f"channel {channel!r} is not one of {names} for this solver")
    return names.index(channel)


def partition(costs: Sequence[float], nparts: int) -> List[List[int]]:
    """Split items of the given costs into ``nparts`` lists of indices with
    near-equal total cost.  Largest items go first, each to the currently
    least-loaded part; ties go to the lower index, so every rank computes the
    same split.  Each list is returned in ascending order."""
    if nparts < 1:
        raise ValueError("nparts must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    loads = [0.0] * nparts
    parts: List[List[int]] = [[] for _ in range(nparts)]
    for i in order:
        r = min(range(nparts), key=lambda p: (loads[p], p))
        parts[r].append(i)
        loads[r] += float(costs[i])
    return [sorted(p) for p in parts]


def _dist(group=None):
    """(rank, world size, torch.distributed module or None)."""
    try:
        import torch.distributed as dist
    except ImportError:  # pragma: no cover - torch always ships it
        return 0, 1, None
    if not (dist.is_available() and dist.is_initialized()):
        return 0, 1, None
    return dist.get_rank(group), dist.get_world_size(group), dist


def gather_to_root(local: Dict[int, object], group=None) -> Optional[Dict[int, object]]:
    """Merge every rank's {item index: result} on rank 0 (host-side gather of
    pickled objects).  Returns the merged dict on rank 0, None elsewhere; in a
    single process, the dict itself."""
    rank, world, dist = _dist(group)
    if world == 1:
        return dict(local)
    out = [None] * world if rank == 0 else None
    dist.gather_object(local, out, dst=0, group=group)
    if rank != 0:
        return None
    merged: Dict[int, object] = {}
    for part in out:
        merged.update(part)
    return merged


def allreduce_sum(a: np.ndarray, group=None) -> np.ndarray:
    """Elementwise sum of ``a`` over the ranks (FP64), returned on every rank."""
    rank, world, dist = _dist(group)
    a = np.asarray(a, dtype=np.float64)
    if world == 1:
        return a.copy()
    import torch
    t = torch.from_numpy(np.ascontiguousarray(a).copy())
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()


def _cost(case) -> float:
    return float(case.grid.cells) * float(case.nstep)


def default_device(group=None) -> str:
    """The GPU of this process: ``cuda:{LOCAL_RANK}`` when torch.distributed
    is initialised with more than one rank (one process per GPU, as torchrun
    starts them), else ``cuda`` (the current device)."""
    import os
    _, world, _ = _dist(group)
    if world > 1 and "LOCAL_RANK" in os.environ:
        return f"cuda:{int(os.environ['LOCAL_RANK'])}"
    return "cuda"


def gpu_runner(cases, device=None, schedule: str = "sequential") -> List[np.ndarray]:
    """Receiver traces (nstep, nch, nrec) of each case.  ``device`` defaults
    to :func:`default_device`.  2.5-D cases run one after another.  For the
    2-D single-pass kinds, ``schedule``:

    * ``"sequential"`` (default): every case alone, one after another, each
      in its own default form -- the whole run in one launch on chip where
      the grid fits, else one launch per step -- through a
      :class:`~seidart_gb300.solver.ShotPipeline` (two handles in turn, a
      case's host work overlapping the previous case's run);
    * ``"batch"``: all of them advancing together in one persistent launch
      per shot length (:mod:`seidart_gb300.batch`).

    On the 80-model survey of 64 electromag2 shots (1040 x 540) and 16
    seismic2 models (200-1200 x 100-600 cells), 4000 steps, the sequential
    schedule took 1.73 s and the batch 2.40 s (wall clock, set-up
    included): on chip a shot runs faster than a batch tile streaming from
    HBM, and a grid too large for the chip runs its own launches at least as
    fast as the batch kernel's register-capped tiles.  Running the models
    that fit on chip alone and batching the rest took 2.08 s.

    In the batch schedule, cases that hold the same model planes (the same
    array object) share one copy of the coefficients."""
    from .batch import Batch, autotune
    from .solver import FDTDSolver, ShotPipeline, run_shot
    if schedule not in ("sequential", "batch"):
        raise ValueError("schedule must be 'sequential' or 'batch'")
    device = default_device() if device is None else device
    if schedule == "sequential":
        with ShotPipeline(device) as p:
            return list(p.run((c.grid, c.planes, c.profiles, c.src_ijk, c.srcfn, c.rec_ijk) for c in cases))

    out: List[Optional[np.ndarray]] = [None] * len(cases)
    two_d = [q for q, c in enumerate(cases) if c.grid.kind in (SEISMIC2, ELECTROMAG2)]
    for q, c in enumerate(cases):
        if q not in two_d:
            out[q] = run_shot(c.grid, c.planes, c.profiles, c.src_ijk, c.srcfn, c.rec_ijk, device=device)
    if not two_d:
        return out
    solvers: Dict[int, FDTDSolver] = {}
    owner = {}
    try:
        for q in two_d:
            c = cases[q]
            s = FDTDSolver(c.grid, c.nstep, len(c.rec_ijk), device=device)
            solvers[q] = s
            if id(c.planes) in owner:
                s.share_model(owner[id(c.planes)])
            else:
                s.set_model(c.planes)
                owner[id(c.planes)] = s
            s.set_cpml(c.profiles)
            s.set_source(c.src_ijk, c.srcfn)
            s.set_receivers(c.rec_ijk)
        by_len: Dict[int, List[int]] = {}
        for q in two_d:  # one batch per shot length: a batch advances all its models together
            by_len.setdefault(cases[q].nstep, []).append(q)
        for nstep, qs in by_len.items():
            if len(qs) == 1:
                s = solvers[qs[0]]
                s.run(nstep)
                s.status()
                out[qs[0]] = s.traces()
                continue
            b = Batch([solvers[q] for q in qs])
            try:
                autotune(b, steps=4)
                b.run(nstep)
                b.status()
                for q in qs:
                    out[q] = solvers[q].traces()
            finally:
                b.close()
    finally:
        for s in solvers.values():
            s.close()
    return out


def run_survey(cases, runner: Optional[Callable] = None, group=None, device=None) -> Optional[List[np.ndarray]]:
    """Traces of every case of a survey (a list of
    :class:`seidart_gb300.synthetic.Case`-like objects: grid, planes, profiles,
    src_ijk, srcfn, rec_ijk).  Under ``torch.distributed`` each rank runs
    the cases :func:`partition` gives it.  ``runner(cases)`` returns their
    traces; the default is :func:`gpu_runner` on ``device`` (by default
    :func:`default_device`: each rank its own GPU).  Returns the traces in
    case order on rank 0, None on the other ranks."""
    rank, world, _ = _dist(group)
    device = default_device(group) if device is None else device
    mine = partition([_cost(c) for c in cases], world)[rank]
    run = runner or (lambda cs: gpu_runner(cs, device=device))
    traces = run([cases[q] for q in mine]) if mine else []
    merged = gather_to_root({q: np.asarray(tr) for q, tr in zip(mine, traces)}, group)
    if merged is None:
        return None
    return [merged[q] for q in range(len(cases))]


class _Shot:
    __slots__ = ("grid", "planes", "profiles", "src_ijk", "srcfn", "rec_ijk")

    def __init__(self, grid, planes, profiles, src_ijk, srcfn, rec_ijk):
        self.grid, self.planes, self.profiles = grid, planes, profiles
        self.src_ijk, self.srcfn, self.rec_ijk = src_ijk, srcfn, rec_ijk

    @property
    def nstep(self) -> int:
        return self.srcfn.shape[1]


class CommonOffset:
    """Common-offset survey over one model: source i is recorded by receiver
    i only (``common_offset.py:13-284``).  ``source_ijk`` and
    ``receiver_ijk`` are (n, 3) full-grid cell indices (CPML included);
    ``channel`` is one of the solver's channels ('Ex', 'Vz', ...).

    ``co_run()`` returns ``co_image`` of shape (time steps, sources), as the
    reference's ``co_run`` builds it, on rank 0 (None on other ranks).  The
    shots share the model's coefficient planes and run through
    :func:`gpu_runner`."""

    def __init__(self, grid, planes, profiles, srcfn, source_ijk, receiver_ijk, channel: str, device=None,
                 runner: Optional[Callable] = None, group=None):
        self.grid = grid
        self.planes = np.ascontiguousarray(planes, dtype=np.float64)
        self.profiles = profiles
        self.srcfn = np.asarray(srcfn, dtype=np.float64)
        self.source_xyz_all = np.asarray(source_ijk, dtype=np.int64).reshape(-1, 3)
        self.receiver_xyz_all = np.asarray(receiver_ijk, dtype=np.int64).reshape(-1, 3)
        if len(self.source_xyz_all) != len(self.receiver_xyz_all):
            raise ValueError("one receiver per source: the source and receiver lists differ in length")
        self.channel = channel
        self.ch = channel_index(grid.kind, channel)
        self.device = device
        self.runner = runner
        self.group = group
        self.co_image = None
        self.timeseries = None

    @property
    def time_steps(self) -> int:
        return self.srcfn.shape[1]

    def shots(self) -> List[_Shot]:
        return [_Shot(self.grid, self.planes, self.profiles, tuple(int(v) for v in s), self.srcfn,
                      np.asarray(r, dtype=np.int32).reshape(1, 3))
                for s, r in zip(self.source_xyz_all, self.receiver_xyz_all)]

    def co_run(self, parallel=None) -> Optional[np.ndarray]:
        """Run every shot and assemble the image; ``parallel`` is accepted for
        the reference's signature (the shots of a rank always run together)."""
        traces = run_survey(self.shots(), runner=self.runner, group=self.group, device=self.device)
        if traces is None:
            return None
        self.co_image = np.stack([tr[:, self.ch, 0] for tr in traces], axis=1).astype(np.float64)
        self.timeseries = self.co_image
        return self.co_image


def survey_gradient(cases, residual_fn: Callable, grad_fn: Optional[Callable] = None, group=None,
                    ckpt_every: int = 200, device=None) -> np.ndarray:
    """Gradient of a misfit summed over the shots of one model with respect
    to its six planes: the sum over shots of the per-shot gradients, on every
    rank.  ``residual_fn(index, traces)`` gives dJ/d(traces) of shot
    ``index`` from its traces; ``grad_fn(case, residual_fn, index)`` returns
    that shot's (6, NZ, NX) gradient -- the default runs the forward and the
    checkpointed adjoint of :class:`seidart_gb300.adjoint.TraceModel`
    (electromag2).  Each rank adds up its own shots; one all-reduce adds the
    ranks' sums.  ``device`` defaults to :func:`default_device`."""
    rank, world, _ = _dist(group)
    device = default_device(group) if device is None else device
    mine = partition([_cost(c) for c in cases], world)[rank]
    g = None
    for q in mine:
        gq = (grad_fn or _adjoint_gradient)(cases[q], residual_fn, q, ckpt_every=ckpt_every, device=device)
        g = np.array(gq, dtype=np.float64) if g is None else g + gq
    if g is None:
        nz, nx = cases[0].planes.shape[1:]
        g = np.zeros((6, nz, nx))
    return allreduce_sum(g, group)


def _adjoint_gradient(case, residual_fn, index, ckpt_every=200, device="cuda"):
    import torch
    from .adjoint import TraceModel
    p = case.planes
    if not np.array_equal(p[5], p[3]):
        raise ValueError("the differentiable electromag2 model ties sig33 = sig11 (planes 5 and 3 must be equal)")
    m = TraceModel(case.grid, p, case.profiles, case.src_ijk, case.srcfn, case.rec_ijk, ckpt_every=ckpt_every,
                   device=device)
    try:
        tr = m.forward(p[0], p[2], p[3])
        r = residual_fn(index, tr.cpu().numpy())
        _, _, _, g6 = m.backward(torch.as_tensor(r, dtype=torch.float32, device=tr.device))
        return g6
    finally:
        m.close()
