#!/usr/bin/env python
"""Throughput benchmark of the GB300 FDTD backend.

Headline workload (one bench "step" = one complete shot): the 2-D anisotropic
EM model, electromag2 on a 1000x500 interior + 20-cell CPML (1040x540 cells),
three seeded random layers, 100 MHz Ricker Ex source, 6000 time steps, 100
receivers, FP32 fields.  metric = Gcell-updates/s (full grid incl. CPML x
time steps / wall time).  Inputs are seeded synthetic models with the
workload's shapes and value ranges (the reference measures nothing public).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm on the host cores: the FP64
restatement of the legacy Fortran loops (oracle/, OpenMP, all host threads),
because the reference's own solver cannot be built or run on these machines.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Gcell-updates/s"
WORKLOAD = "electromag2 plain 1040x540 cells (1000x500 + 20-cell CPML) x 6000 steps, 100 receivers"
DATA = "synthetic (seeded layered permittivity/conductivity model)"


def cpu_model() -> str:
    """The host CPU's model name (lscpu), for the CPU baseline's record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
    except (OSError, subprocess.SubprocessError):
        return "unknown"
    for line in out.splitlines():
        if line.strip().lower().startswith("model name"):
            return line.split(":", 1)[1].strip()
    return "unknown"


def bench_config(nstep, cells, world):
    """The workload description both arms print (the reference arm times a
    bounded sample of it, described in its cpu_baseline.sample)."""
    return {"workload": WORKLOAD, "time_steps_per_bench_step": nstep, "cells": cells,
            "l2": "256 MiB buffer written between shots (flush)", "parallelism": f"replicas x{world}"}


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# clocks during the timed region

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.tmp = None

    def start(self):
        try:
            self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-i", str(self.idx), "-lms", "200"], stdout=self.tmp,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.tmp.flush()
        rows = [r.split(",") for r in Path(self.tmp.name).read_text().splitlines() if r.strip()]
        os.unlink(self.tmp.name)
        sm, mx, reasons = [], [], set()
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for name, val in zip(self.NAMES, r[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "samples": len(sm),
                "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
# algorithmic bytes (FP32 = 4 B), per kernel launch and per cell update

def strip_fractions(grid):
    W = grid.npml
    fx = min(1.0, 2 * W / grid.nx)
    fz = min(1.0, 2 * W / grid.nz)
    fy = min(1.0, 2 * W / grid.ny) if grid.ny > 1 else 0.0
    return fx, fy, fz


def em2_bytes(grid):
    """electromag2.  H kernel: read Ex Ez Hy, write Hy; psi dEx_dz (z-strip), dEz_dx (x-strip).
    E kernel: read Hy Ex Ez + caEx cbEx caEz cbEz, write Ex Ez; psi dHy_dz (z), dHy_dx (x).
    Step (each field read and written once, each coefficient read once): 40 B + strip psi."""
    fx, _, fz = strip_fractions(grid)
    cells = grid.nx * grid.nz
    psi = 8 * (fx + fz)
    h = (16 + psi) * cells
    e = (36 + psi) * cells
    step = (40 + 2 * psi) * cells
    return {"half1": h, "half2": e, "step": step, "per_cell_step": 40 + 2 * psi}


def seis2_bytes(grid, atten=False):
    """seismic2.  Stress kernel: read vx vz, read+write sxx szz sxz, 6 stiffness; 4 velocity-gradient psi
    (2 on each strip).  Velocity kernel: read 3 stresses, read+write vx vz, dt/rho x2 (+2 gamma); 4 stress
    psi.  Step: 5 fields read and written once + 8 (+2) coefficients + psi."""
    fx, _, fz = strip_fractions(grid)
    cells = grid.nx * grid.nz
    g = 8 if atten else 0
    psi = 16 * (fx + fz)
    h1 = (8 + 24 + 24 + psi) * cells
    h2 = (12 + 16 + 8 + g + psi) * cells
    step = (40 + 32 + g + 2 * psi) * cells
    return {"half1": h1, "half2": h2, "step": step, "per_cell_step": step / cells}


def em25_bytes(grid):
    """electromag25 with y-marching: H kernel reads Hx Hy Hz and Ex Ey Ez, writes H; E kernel reads all six,
    writes E; 6 coefficients per (x,z) column amortised over NY; psi: 12 on strips (2 per axis per kernel)."""
    fx, fy, fz = strip_fractions(grid)
    cells = grid.nx * grid.ny * grid.nz
    col = grid.nx * grid.nz
    psi = 2 * 8 * (fx + fy + fz)
    h1 = (6 * 4 + 3 * 4 + psi) * cells
    h2 = (6 * 4 + 3 * 4 + psi) * cells + 6 * 4 * col
    step = (6 * 8 + 2 * psi) * cells + 6 * 4 * col
    return {"half1": h1, "half2": h2, "step": step, "per_cell_step": step / cells}


def em2c_bytes(grid):
    """electromag2c: electromag2 with every field, coefficient and memory variable a (real, imaginary) pair."""
    b = em2_bytes(grid)
    return {k: 2 * v for k, v in b.items()}


def seis25_bytes(grid, atten=True):
    """seismic25 with y-marching: coefficients (21 stiffness, 3 dt/rho, 3 gamma) are read once per (x,z)
    column and amortised over NY.  Stress kernel: read 9 fields, write 6 stresses; velocity kernel: read
    9 fields, write 3 velocities.  psi: 9 velocity-gradient (3 per axis) and 9 stress-gradient."""
    fx, fy, fz = strip_fractions(grid)
    cells = grid.nx * grid.ny * grid.nz
    col = grid.nx * grid.nz
    psi_axis = 3 * 8 * (fx + fy + fz)
    h1 = (9 * 4 + 6 * 4 + psi_axis) * cells + 21 * 4 * col
    h2 = (9 * 4 + 3 * 4 + psi_axis) * cells + 6 * 4 * col
    step = (9 * 8 + 2 * psi_axis) * cells + 27 * 4 * col
    return {"half1": h1, "half2": h2, "step": step, "per_cell_step": step / cells}


# ---------------------------------------------------------------------------

def make_solver(case, device, flags=0):
    from seidart_gb300.solver import FDTDSolver
    s = FDTDSolver(case.grid, case.nstep, len(case.rec_ijk), device=device, flags=flags, **case.solver_options())
    s.set_model(case.planes)
    s.set_cpml(case.profiles)
    s.set_source(case.src_ijk, case.srcfn)
    if case.stress_srcfn is not None:
        s.set_stress_source(case.src_ijk, case.stress_srcfn)
    s.set_receivers(case.rec_ijk)
    return s


def launches_per_shot(kind, nstep, single_pass=True):
    from seidart_gb300 import ELECTROMAG25
    # begin + 1 (single-pass) or 2 kernels per step + one advance per 32-step graph + finalize
    # (+ H faces for EM25) + slot reduce
    per = 1 if single_pass else 2
    return per * nstep + nstep // 32 + 3 + (1 if kind == ELECTROMAG25 else 0)


def bench_plain(case, device, flush, stream, peak, bytes_fn, steps, warmup, flags=0):
    """One plain configuration: shots of `case`, kernel times, roofline fractions."""
    s = make_solver(case, device, flags)
    ms = time_shots(s, case.nstep, max(1, steps), warmup, flush, stream)
    kt = kernel_times(s, stream, n=20)
    b = bytes_fn(case.grid)
    r = case.grid.cells * case.nstep / (ms / 1e3) / 1e9
    tiles = s.on_chip()
    s.close()
    return {"workload": f"{case.name}: {case.grid.cells} cells x {case.nstep} steps", "value": round(r, 3),
            "unit": METRIC, "ms_per_shot": round(ms, 3),
            "form": (f"on chip, {tiles[0]} tiles in {tiles[1]} rows, one launch per run" if tiles
                     else "one launch per step"),
            "bytes_per_cell_update": round(b["per_cell_step"], 1),
            "hbm_frac": round(b["per_cell_step"] * r / peak, 4),
            # the one-launch-per-step kernels, timed alone (sfd_launch_half), whichever form the shot used
            "kernel_ms": [round(x, 4) for x in kt],
            "kernel_frac": [round(b[h] / (t / 1e3) / 1e9 / peak, 4) for h, t in zip(("half1", "half2"), kt)]}


def bench_batched(device, flush, stream, peak, plain_value, runs=2, nstep=4000, tiling=None, parity_models=()):
    """The batched survey: 64 electromag2 shots of the layered 1000x500 model (sources every 15
    cells) + 16 seeded seismic2 models of uneven size, 4000 steps, one persistent launch per run.
    ``parity_models``: indices of the models (shots first) whose batched traces and fields are
    compared with the FP64 oracle."""
    import torch
    from seidart_gb300 import ELECTROMAG2, synthetic as sy
    from seidart_gb300.batch import Batch, autotune
    from seidart_gb300.solver import FDTDSolver
    shots, models = sy.batched_survey(nshots=64, nelastic=16, nstep=nstep)
    cases = shots + models
    solvers, owner = [], {}
    for c in cases:  # the shots of one model read one copy of its coefficients
        s = FDTDSolver(c.grid, c.nstep, len(c.rec_ijk), device=device)
        if id(c.planes) in owner:
            s.share_model(owner[id(c.planes)])
        else:
            s.set_model(c.planes)
            owner[id(c.planes)] = s
        s.set_cpml(c.profiles)
        s.set_source(c.src_ijk, c.srcfn)
        s.set_receivers(c.rec_ijk)
        solvers.append(s)
    b = Batch(solvers)
    if tiling:  # a fixed (rows per thread, blocks per SM), e.g. for a profiler run
        b.set_tiling(*tiling)
        tune = {"tiling": tuple(tiling), "timings": {}}
    else:
        tune = autotune(b, steps=8, use_cache=False)
    nstep = cases[0].nstep
    b.reset()
    b.run(min(64, nstep))
    b.status()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    total_ms = 0.0
    for _ in range(runs):
        flush.zero_()
        b.reset()
        torch.cuda.synchronize()
        ev0.record(stream)
        b.run(nstep)
        ev1.record(stream)
        b.status()
        total_ms += ev0.elapsed_time(ev1)
    ms = total_ms / runs
    cells = sum(c.grid.cells for c in cases)
    # per model: its fields and memory variables; per distinct model: its coefficients (read once per step)
    step_bytes = 0.0
    seen = set()
    for c in cases:
        if c.grid.kind == ELECTROMAG2:
            b_ = em2_bytes(c.grid)
            coef = 16 * c.grid.cells
        else:
            b_ = seis2_bytes(c.grid)
            coef = 32 * c.grid.cells
        step_bytes += b_["step"] - coef
        if id(c.planes) not in seen:
            seen.add(id(c.planes))
            step_bytes += coef
    unshared = sum(em2_bytes(c.grid)["step"] if c.grid.kind == ELECTROMAG2 else seis2_bytes(c.grid)["step"]
                   for c in cases)
    value = cells * nstep / (ms / 1e3) / 1e9
    achieved = step_bytes * nstep / (ms / 1e3) / 1e9
    # The same survey through the plain single-shot path, one model after the
    # other (each handle's own run: the electromag2 shots on chip, the
    # seismic2 models one launch per step), against the batched traces.
    batched_traces = [s.traces() for s in solvers]
    parity = None
    if parity_models:
        # a few shots and models of the batch against the FP64 oracle (traces
        # and final fields of the batched run)
        from oracle import parity as par
        from seidart_gb300.solver import FIELDS
        picks = [q for q in parity_models if q < len(cases)]
        fields = {q: [solvers[q].field(nm) for nm in FIELDS[cases[q].grid.kind]] for q in picks}
        parity = {}
        t0 = time.perf_counter()
        for q in picks:
            st, ref, peaks = par.oracle_case_peaks(cases[q])
            r = par.compare_run(batched_traces[q], fields[q], st, ref, FIELDS[cases[q].grid.kind], peaks)
            parity[cases[q].name] = {k: r[k] for k in ("rel_l2_traces", "rel_l2_fields_max",
                                                        "fields_err_vs_peak_norm_max")}
        parity = {"models": parity, "steps": nstep,
                  "rel_l2_traces_max": max(v["rel_l2_traces"] for v in parity.values()),
                  "rel_l2_fields_max": max(v["rel_l2_fields_max"] for v in parity.values()),
                  "fields_err_vs_peak_norm_max": max(v["fields_err_vs_peak_norm_max"] for v in parity.values()),
                  "oracle_s": round(time.perf_counter() - t0, 1)}
    for s in solvers:
        s.reset()
    torch.cuda.synchronize()
    ev0.record(stream)
    for s in solvers:
        s.run(nstep)
    ev1.record(stream)
    for s in solvers:
        s.status()
    plain_ms = ev0.elapsed_time(ev1)
    num = den = 0.0
    for s, tb in zip(solvers, batched_traces):
        tp = s.traces().astype(np.float64)
        num += float(((tp - tb) ** 2).sum())
        den += float((tp ** 2).sum())
    plain_agg = cells * nstep / (plain_ms / 1e3) / 1e9
    # ... and through the one-launch-per-step kernels whose tile bodies the
    # batch runs (SFD_FLAG_STREAMING: no model runs on chip)
    from seidart_gb300.solver import FLAG_STREAMING
    step_solvers, owner2 = [], {}
    for c in cases:
        s = FDTDSolver(c.grid, c.nstep, len(c.rec_ijk), device=device, flags=FLAG_STREAMING)
        if id(c.planes) in owner2:
            s.share_model(owner2[id(c.planes)])
        else:
            s.set_model(c.planes)
            owner2[id(c.planes)] = s
        s.set_cpml(c.profiles)
        s.set_source(c.src_ijk, c.srcfn)
        s.set_receivers(c.rec_ijk)
        step_solvers.append(s)
    for s in step_solvers:
        s.run(8)
        s.reset()
    torch.cuda.synchronize()
    ev0.record(stream)
    for s in step_solvers:
        s.run(nstep)
    ev1.record(stream)
    for s in step_solvers:
        s.status()
    step_ms = ev0.elapsed_time(ev1)
    num2 = den2 = 0.0
    for s, tb in zip(step_solvers, batched_traces):
        tp = s.traces().astype(np.float64)
        num2 += float(((tp - tb) ** 2).sum())
        den2 += float((tp ** 2).sum())
    for s in step_solvers:
        s.close()
    step_agg = cells * nstep / (step_ms / 1e3) / 1e9
    # ... and the survey runner's default: every model in its default form,
    # through the two-handle shot pipeline (wall clock, set-up included)
    from seidart_gb300 import survey
    survey.gpu_runner(cases[:2] + cases[-2:], device=device)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    surv_traces = survey.gpu_runner(cases, device=device)
    torch.cuda.synchronize()
    surv_s = time.perf_counter() - t0
    num3 = sum(float(((tp.astype(np.float64) - tb) ** 2).sum()) for tp, tb in zip(surv_traces, batched_traces))
    den3 = sum(float((tp.astype(np.float64) ** 2).sum()) for tp in surv_traces)
    out = {"workload": f"64 electromag2 shots 1040x540 + 16 seismic2 models (nx 200-1200, nz 100-600) x {nstep} steps",
           "value": round(value, 3), "unit": METRIC, "ms_per_run": round(ms, 2), "cells": cells,
           "bytes_per_cell_update": round(step_bytes / cells, 2),
           "bytes_per_cell_update_unshared": round(unshared / cells, 2),
           "roofline": {"bound": "hbm", "kernel": "batch_kernel", "achieved": round(achieved, 1), "peak": peak,
                        "unit": "GB/s", "frac": round(achieved / peak, 4)},
           "vs_plain_single_shot": round(value / plain_value, 3) if plain_value else None,
           "plain_sequential": {"value": round(plain_agg, 3), "unit": METRIC, "ms_per_run": round(plain_ms, 2),
                                "traces_rel_l2_vs_batched": (num / den) ** 0.5 if den > 0 else None},
           "vs_plain_aggregate": round(value / plain_agg, 3),
           "per_step_sequential": {"value": round(step_agg, 3), "unit": METRIC, "ms_per_run": round(step_ms, 2),
                                   "form": "each model alone, one launch per step (SFD_FLAG_STREAMING)",
                                   "traces_rel_l2_vs_batched": (num2 / den2) ** 0.5 if den2 > 0 else None},
           "vs_per_step_aggregate": round(value / step_agg, 3),
           "survey_pipeline": {"value": round(cells * nstep / surv_s / 1e9, 3), "unit": METRIC,
                               "s": round(surv_s, 3),
                               "form": "survey.gpu_runner (default): each model in its default form through "
                                       "solver.ShotPipeline, wall clock with the set-up",
                               "traces_rel_l2_vs_batched": (num3 / den3) ** 0.5 if den3 > 0 else None},
           "tiling": {"rows_per_thread": tune["tiling"][0], "blocks_per_sm": tune["tiling"][1],
                      "candidates_ms_per_step": {k: round(v * 1e3, 4) for k, v in tune["timings"].items()}},
           "launches_per_run": 3}
    if parity is not None:
        out["parity"] = parity
    b.close()
    for s in solvers:
        s.close()
    return out


def bench_adjoint(device, ckpt_every=200, nstep=6000, fd_cells=0):
    """Adjoint gradient on the layered electromag2 model (6000 steps, 100 receivers): misfit against
    the unperturbed model's traces, current model with six +-5% Gaussian blobs in eps11 and eps33
    (seed 6), checkpoints every 200 steps with recompute.  Reports backward / forward wall time, and
    the same for the recompute-free form that keeps every forward state."""
    import torch
    from seidart_gb300 import synthetic as sy
    from seidart_gb300.adjoint import TraceModel
    case = sy.electromag2_layers(nstep=nstep)
    base = case.planes
    rng = np.random.default_rng(6)
    nz, nx = base.shape[1:]
    zz, xx = np.meshgrid(np.arange(nz), np.arange(nx), indexing="ij")
    pert = np.zeros((nz, nx))
    for _ in range(6):
        cz, cx = rng.uniform(0.2, 0.8) * nz, rng.uniform(0.2, 0.8) * nx
        pert += rng.choice([-1, 1]) * 0.05 * np.exp(-((zz - cz) ** 2 + (xx - cx) ** 2) / (2 * 25.0 ** 2))
    cur = base.copy()
    cur[0] = base[0] * (1 + pert)
    cur[2] = base[2] * (1 + pert)
    m = TraceModel(case.grid, base, case.profiles, case.src_ijk, case.srcfn, case.rec_ijk, ckpt_every=ckpt_every,
                   device=device)
    d_obs = m.forward(base[0], base[2], base[3])
    m.forward(cur[0], cur[2], cur[3])  # warm
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tr = m.forward(cur[0], cur[2], cur[3])
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t0
    resid = tr - d_obs
    m.backward(resid)  # warm
    t0 = time.perf_counter()
    g11, g33, gs, _ = m.backward(resid)
    t_bwd = time.perf_counter() - t0
    # plain forward (no checkpoints) for the ratio's denominator
    s = m.solver
    s.reset()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.run(case.nstep)
    s.status()
    t_plain = time.perf_counter() - t0
    m.close()
    # the recompute-free form: every forward state kept in HBM, the backward pass only sweeps
    mr = TraceModel(case.grid, base, case.profiles, case.src_ijk, case.srcfn, case.rec_ijk, device=device,
                    record=True)
    mr.backward(mr.forward(cur[0], cur[2], cur[3]) - d_obs)  # warm
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tr_r = mr.forward(cur[0], cur[2], cur[3])
    torch.cuda.synchronize()
    t_fwd_r = time.perf_counter() - t0
    t0 = time.perf_counter()
    r11, r33, rs, _ = mr.backward(tr_r - d_obs)
    t_bwd_r = time.perf_counter() - t0
    work_gb = mr.work.numel() / 1e9
    mr.close()
    rec_err = max(float(np.linalg.norm(a - b) / np.linalg.norm(a)) for a, b in ((g11, r11), (g33, r33), (gs, rs)))
    misfit = 0.5 * float((resid.double() ** 2).sum())
    out = {"workload": f"electromag2 1040x540 x {nstep} steps, gradient wrt eps11, eps33, sigma per cell",
           "forward_s": round(t_plain, 4), "forward_with_checkpoints_s": round(t_fwd, 4),
           "adjoint_s": round(t_bwd, 4), "adjoint_over_forward": round(t_bwd / t_plain, 3),
           "whole_gradient_over_forward": round((t_fwd + t_bwd) / t_plain, 3),
           "checkpoints_every": ckpt_every, "misfit": misfit,
           "grad_abs_max": [float(np.abs(g).max()) for g in (g11, g33, gs)],
           "recorded": {"form": "every forward state kept in device memory, no recompute (sfd_adjoint_record)",
                        "forward_recording_s": round(t_fwd_r, 4), "adjoint_s": round(t_bwd_r, 4),
                        "adjoint_over_forward": round(t_bwd_r / t_plain, 3),
                        "whole_gradient_over_forward": round((t_fwd_r + t_bwd_r) / t_plain, 3),
                        "workspace_gb": round(work_gb, 2), "grad_rel_l2_vs_checkpointed": rec_err}}
    if fd_cells:
        out["parity_fd"] = adjoint_fd_check(case, base, cur, (g11, g33, gs), fd_cells)
    return out


def bench_seismic2_adjoint(device, ckpt_every=200, fd_cells=0):
    """Adjoint gradient of all nine seismic2 planes on the firn/ice model (400 x 200 + CPML, 2000 steps,
    force source): misfit against the oracle's traces of the model, current model with +-4% Gaussian
    blobs in c11, c33, c55 and rho (seed 6), checkpoints every 200 steps with recompute.  Reports the
    wall times and, with ``fd_cells``, central differences of the FP64 oracle's misfit at seeded cells."""
    import torch
    import oracle
    from oracle import parity as par
    from seidart_gb300 import cpml as cp, synthetic as sy
    from seidart_gb300.adjoint import SeismicTraceModel
    case = sy.seismic2_firn_ice(nstep=2000)
    base = case.planes
    rng = np.random.default_rng(6)
    nz, nx = base.shape[1:]
    zz, xx = np.meshgrid(np.arange(nz), np.arange(nx), indexing="ij")
    cur = base.copy()
    for q in (0, 3, 5, 6):
        cz, cx = rng.uniform(0.3, 0.7) * nz, rng.uniform(0.3, 0.7) * nx
        cur[q] = base[q] * (1 + rng.choice([-1, 1]) * 0.04 * np.exp(-((zz - cz) ** 2 + (xx - cx) ** 2) / (2 * 12.0 ** 2)))
    prof = cp.pack_profiles(case.profiles)

    def traces(planes):
        _, tr, _, blew = oracle.run(case.grid.kind, case.grid, planes, prof, case.src_ijk, case.srcfn, case.rec_ijk,
                                    case.nstep)
        assert not blew
        return tr

    d_obs_np = traces(base)
    m = SeismicTraceModel(case.grid, cur, case.profiles, case.src_ijk, case.srcfn, case.rec_ijk,
                          ckpt_every=ckpt_every, device=device)
    d_obs = torch.as_tensor(d_obs_np, dtype=torch.float32, device=device)
    m.forward(cur)  # warm
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tr = m.forward(cur)
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t0
    resid = tr - d_obs
    m.backward(resid)  # warm
    t0 = time.perf_counter()
    g = m.backward(resid)
    t_bwd = time.perf_counter() - t0
    s = m.solver
    s.reset()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.run(case.nstep)
    s.status()
    t_plain = time.perf_counter() - t0
    on_chip = s.on_chip() is not None
    m.close()
    recorded = None
    if on_chip:  # the recompute-free form: every forward state kept in HBM, the backward pass only sweeps
        mr = SeismicTraceModel(case.grid, cur, case.profiles, case.src_ijk, case.srcfn, case.rec_ijk, device=device,
                               record=True)
        mr.backward(mr.forward(cur) - d_obs)  # warm
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tr_r = mr.forward(cur)
        torch.cuda.synchronize()
        t_fwd_r = time.perf_counter() - t0
        t0 = time.perf_counter()
        g_r = mr.backward(tr_r - d_obs)
        t_bwd_r = time.perf_counter() - t0
        work_gb = mr.work.numel() / 1e9
        mr.close()
        recorded = {"form": "every forward state kept in device memory, no recompute (sfd_adjoint_record)",
                    "forward_recording_s": round(t_fwd_r, 4), "adjoint_s": round(t_bwd_r, 4),
                    "adjoint_over_forward": round(t_bwd_r / t_plain, 2),
                    "whole_gradient_over_forward": round((t_fwd_r + t_bwd_r) / t_plain, 2),
                    "workspace_gb": round(work_gb, 2),
                    "grad_rel_l2_vs_checkpointed": max(float(np.linalg.norm(g_r[q] - g[q]) / np.linalg.norm(g[q]))
                                                       for q in range(9))}
    out = {"workload": "seismic2 firn/ice 400x200 x 2000 steps, gradient wrt c11 c13 c15 c33 c35 c55 rho gamma_x "
                       "gamma_z per cell",
           "forward_form": "on chip" if on_chip else "one launch per step",
           "forward_s": round(t_plain, 4), "forward_with_checkpoints_s": round(t_fwd, 4),
           "adjoint_s": round(t_bwd, 4), "adjoint_over_forward": round(t_bwd / t_plain, 2),
           "whole_gradient_over_forward": round((t_fwd + t_bwd) / t_plain, 2), "checkpoints_every": ckpt_every,
           "misfit": 0.5 * float((resid.double() ** 2).sum()), "recorded": recorded}
    if fd_cells:
        t0 = time.perf_counter()
        names = ("c11", "c13", "c15", "c33", "c35", "c55", "rho", "gamma_x", "gamma_z")
        floor = [1e-4 * float(np.abs(cur[0]).mean())] * 6 + [0.0, 1e-3, 1e-3]
        cells = par.fd_cells(base.shape[1:], case.grid.npml, fd_cells, 7)
        rows, ad, fd = [], [], []
        for n, (k, i) in enumerate(cells):
            q = n % 9
            h = 1e-4 * max(abs(float(cur[q][k, i])), floor[q])
            p_, m_ = cur.copy(), cur.copy()
            p_[q][k, i] += h
            m_[q][k, i] -= h
            d = (par.misfit(traces(p_), d_obs_np) - par.misfit(traces(m_), d_obs_np)) / (2 * h)
            a = float(g[q][k, i])
            ad.append(a)
            fd.append(d)
            rows.append({"cell": [k, i], "param": names[q], "adjoint": a, "fd": d,
                         "rel_err": abs(a - d) / abs(d) if d != 0 else None})
        ad, fd = np.array(ad), np.array(fd)
        rel = [r["rel_err"] for r in rows if r["rel_err"] is not None]
        out["parity_fd"] = {"cells": len(cells), "seed": 7, "h_rel": 1e-4, "steps": case.nstep,
                            "rel_l2": float(np.linalg.norm(ad - fd) / np.linalg.norm(fd)),
                            "rel_err_max": max(rel) if rel else None,
                            "rel_err_median": float(np.median(rel)) if rel else None,
                            "per_cell": rows, "oracle_s": round(time.perf_counter() - t0, 1)}
    return out


def adjoint_fd_check(case, base, cur, grads, ncells, seed=7, h_rel=1e-4):
    """Central finite differences of the FP64 oracle's misfit at ``ncells``
    seeded interior cells (seed 7), relative step h = 1e-4 of the cell's value,
    against the GPU adjoint gradient.  The parameter cycles through eps11,
    eps33 and sigma (= sig11 = sig33) from cell to cell.  d_obs = the oracle's
    traces of the unperturbed model; the misfit is evaluated at ``cur``."""
    from oracle import parity as par
    from seidart_gb300 import cpml as cp
    prof = cp.pack_profiles(case.profiles)
    t0 = time.perf_counter()
    import oracle

    def J(planes):
        _, tr, _, blew = oracle.run(case.grid.kind, case.grid, planes, prof, case.src_ijk, case.srcfn,
                                    case.rec_ijk, case.nstep)
        assert not blew
        return tr

    d_obs = J(base)
    cells = par.fd_cells(base.shape[1:], case.grid.npml, ncells, seed)
    names = ("eps11", "eps33", "sigma")
    planes_of = ((0,), (2,), (3, 5))
    ad, fd, rows = [], [], []
    for n, (k, i) in enumerate(cells):
        q = n % 3
        h = h_rel * cur[planes_of[q][0]][k, i]
        p, m_ = cur.copy(), cur.copy()
        for pl in planes_of[q]:
            p[pl][k, i] += h
            m_[pl][k, i] -= h
        d = (par.misfit(J(p), d_obs) - par.misfit(J(m_), d_obs)) / (2 * h)
        g = float(grads[q][k, i])
        ad.append(g)
        fd.append(d)
        rows.append({"cell": [k, i], "param": names[q], "adjoint": g, "fd": d,
                     "rel_err": abs(g - d) / abs(d) if d != 0 else None})
    ad, fd = np.array(ad), np.array(fd)
    rel = [r["rel_err"] for r in rows if r["rel_err"] is not None]
    return {"cells": len(cells), "seed": seed, "h_rel": h_rel, "steps": case.nstep,
            "rel_l2": float(np.linalg.norm(ad - fd) / np.linalg.norm(fd)),
            "rel_err_max": max(rel) if rel else None, "rel_err_median": float(np.median(rel)) if rel else None,
            "per_cell": rows, "oracle_s": round(time.perf_counter() - t0, 1)}


def parity_plain(case, device, nsteps=None):
    """The default GPU path of ``case`` (the form the bench times) against the
    FP64 oracle over ``nsteps`` steps from rest: traces and final fields."""
    from seidart_gb300 import SEISMIC2, SEISMIC25
    from oracle import parity as par
    from seidart_gb300.solver import FIELDS
    n = case.nstep if nsteps is None else int(nsteps)
    s = make_solver(case, device)
    tiles = s.on_chip()
    s.run(n)
    s.status()
    tr = s.traces()[:n]
    names = FIELDS[case.grid.kind]
    fields = [s.field(nm) for nm in names]
    s.close()
    t0 = time.perf_counter()
    st, ref, peaks = par.oracle_case_peaks(case, n)
    out = {"workload": f"{case.name}: {case.grid.cells} cells", "steps": n, "of_steps": case.nstep,
           "form": "on chip" if tiles else "one launch per step",
           "physics": {"legacy_quirks": case.legacy, "density": case.density,
                       "source": "stress (explosive)" if case.stress_srcfn is not None else "force"}
           if case.grid.kind in (SEISMIC2, SEISMIC25) else None}
    out.update(par.compare_run(tr, fields, st, ref, names, peaks))
    out["oracle_s"] = round(time.perf_counter() - t0, 1)
    return out


def time_shots(solver, nstep, K, W, flush, stream, sync_all=None):
    import torch
    for _ in range(W):
        flush.zero_()
        solver.reset()
        solver.run(nstep)
    solver.status()
    torch.cuda.synchronize()
    if sync_all:
        sync_all()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(K):
        flush.zero_()  # 256 MiB write: evicts the 129 MB L2 between shots
        solver.reset()
        solver.run(nstep)
    ev1.record(stream)
    torch.cuda.synchronize()
    if sync_all:
        sync_all()
    solver.status()
    return ev0.elapsed_time(ev1) / K


def kernel_times(solver, stream, n=200):
    """Average duration (ms) of each half-step kernel launched alone, CUDA events on its stream."""
    import torch
    out = []
    for which in (0, 1):
        solver.reset()
        solver.launch_half(which, 10)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        solver.launch_half(which, n)
        e1.record(stream)
        torch.cuda.synchronize()
        out.append(e0.elapsed_time(e1) / n)
    solver.reset()
    return out


def run_times(solver, nstep, stream, n=3):
    """Average duration (ms) of one whole run of `nstep` steps, CUDA events on its stream."""
    import torch
    tot = 0.0
    for _ in range(n):
        solver.reset()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        solver.run(nstep)
        e1.record(stream)
        torch.cuda.synchronize()
        tot += e0.elapsed_time(e1)
    solver.status()
    solver.reset()
    return tot / n


def profile_value(name, key):
    """A number recorded in profiles/<name>.md as a "key: N" line, else None."""
    p = ROOT / "profiles" / f"{name}.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.strip().startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


def profile_traffic(name):
    """dram bytes per launch recorded in profiles/<name>.md ("dram_bytes_per_launch: N"), else None."""
    p = ROOT / "profiles" / f"{name}.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.strip().startswith("dram_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


def cpu_baseline(case, seconds=10.0, chunk=100):
    """FP64 oracle (restated legacy Fortran loops) on all host threads, time-bounded sample, built
    for the host CPU (oracle.NATIVE_FLAGS)."""
    import oracle
    from seidart_gb300 import cpml as cp
    prof = cp.pack_profiles(case.profiles)
    st = None
    done = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds and done + chunk <= case.nstep:
        st, _, _, _ = oracle.run(case.grid.kind, case.grid, case.planes, prof, case.src_ijk, case.srcfn,
                                 case.rec_ijk, chunk, state=st, native=True)
        done += chunk
    el = time.perf_counter() - t0
    value = case.grid.cells * done / el / 1e9
    return {"value": round(value, 4), "unit": METRIC, "cores": oracle.num_threads(), "kind": "port",
            "cpu": cpu_model(), "build": oracle.NATIVE_FLAGS,
            "sample": f"{done} of {case.nstep} steps of the same workload, FP64, OpenMP ({el:.1f} s)"}


def cpu_baseline_snapshots(case, steps=100):
    """The FP64 oracle with the reference's per-step output: after every step
    one full-field FP32 record per channel (write_image2,
    readwrite_routines.f95:473-499, called each step at
    electromagfdtd.f95:323).  The two parts run one after the other in the
    reference, so each is timed on its own over ``steps`` steps of the
    workload and the times are added: the oracle advancing the steps in one
    call, and the records of every step written to a scratch directory."""
    import oracle
    from seidart_gb300 import cpml as cp, fortran_io as fio
    prof = cp.pack_profiles(case.profiles)
    oracle.lib(native=True)  # built before the timed region
    t0 = time.perf_counter()
    st, _, _, _ = oracle.run(case.grid.kind, case.grid, case.planes, prof, case.src_ijk, case.srcfn, case.rec_ijk,
                             steps, native=True)
    t_comp = time.perf_counter() - t0
    with tempfile.TemporaryDirectory() as td:
        t0 = time.perf_counter()
        for t in range(steps):
            for q, ch in enumerate(("Ex", "Ez")):
                fio.write_record(Path(td) / f"{ch}.{t + 1:06d}.500.25.dat", st.fields[q].astype(np.float32),
                                 np.float32)
        t_write = time.perf_counter() - t0
    value = case.grid.cells * steps / (t_comp + t_write) / 1e9
    return {"value": round(value, 4), "unit": METRIC, "cores": oracle.num_threads(), "kind": "port",
            "cpu": cpu_model(), "build": oracle.NATIVE_FLAGS,
            "sample": f"{steps} of {case.nstep} steps: compute {t_comp:.2f} s plus a full-field FP32 record of Ex "
                      f"and Ez per step, {t_write:.2f} s (timed apart, added)"}


def run_reference(args):
    """--impl reference: the reference algorithm (FP64 oracle port) on the host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import oracle
    from seidart_gb300 import cpml as cp, synthetic as sy
    oracle.build()
    case = sy.electromag2_layers(nstep=6000)
    prof = cp.pack_profiles(case.profiles)
    chunk = args.ref_chunk
    st = None

    def step():
        nonlocal st
        if st is not None and st.step + chunk > case.nstep:
            st = None
        st, _, _, _ = oracle.run(case.grid.kind, case.grid, case.planes, prof, case.src_ijk, case.srcfn,
                                 case.rec_ijk, chunk, state=st, native=True)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    el = time.perf_counter() - t0
    value = case.grid.cells * chunk * args.steps / el / 1e9
    sample = (f"{chunk} consecutive time steps of the workload per bench step (the shot restarts after its "
              f"{case.nstep} steps), FP64 restatement of the legacy loops")
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": METRIC, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * el / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA,
        "config": bench_config(case.nstep, case.grid.cells, args.gpus),
        "cpu_baseline": {"value": round(value, 4), "unit": METRIC, "cores": oracle.num_threads(), "kind": "port",
                         "cpu": cpu_model(), "build": oracle.NATIVE_FLAGS, "sample": sample},
        "e2e": {"value": round(value, 4), "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import torch
    from seidart_gb300 import ELECTROMAG2, SEISMIC2, SEISMIC25, synthetic as sy
    from seidart_gb300 import build as b
    from seidart_gb300.solver import ShotPipeline, run_shot

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    b.build()

    def sync_all():
        if dist is not None:
            dist.barrier()

    stream = torch.cuda.current_stream(device)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=device)
    peak, peak_kind = _peaks()

    if args.only:
        # one leg alone (profiler runs): prints that leg's record, not a bench line
        if args.only == "seismic2":
            rec = bench_plain(sy.seismic2_firn_ice(nstep=args.time_steps if args.time_steps != 6000 else 2000),
                              device, flush, stream, peak, seis2_bytes, args.steps, args.warmup)
        elif args.only == "seismic25":
            rec = bench_plain(sy.seismic25_ice(nstep=args.time_steps if args.time_steps != 6000 else 3000),
                              device, flush, stream, peak, seis25_bytes, args.steps, args.warmup)
        elif args.only == "electromag2_step":  # the workload with one launch per step (em2_step_kernel)
            from seidart_gb300.solver import FLAG_STREAMING
            rec = bench_plain(sy.electromag2_layers(nstep=args.time_steps), device, flush, stream, peak, em2_bytes,
                              args.steps, args.warmup, flags=FLAG_STREAMING)
        elif args.only == "electromag25":  # a 2.5-D EM model of the seismic25 workload's grid
            from seidart_gb300 import ELECTROMAG25
            c = sy.small_case(ELECTROMAG25, seed=3, nx=630, nz=330, ny=70, npml=15,
                              nstep=args.time_steps if args.time_steps != 6000 else 300)
            c.name = "electromag25 random 600x40x300"
            rec = bench_plain(c, device, flush, stream, peak, em25_bytes, args.steps, args.warmup)
        elif args.only == "electromag2c":  # complex permittivities, 2000 x 1500 cells
            from seidart_gb300 import ELECTROMAG2C
            c = sy.small_case(ELECTROMAG2C, seed=3, nx=2000, nz=1500, npml=20,
                              nstep=args.time_steps if args.time_steps != 6000 else 300)
            c.name = "electromag2c random 1960x1460"
            rec = bench_plain(c, device, flush, stream, peak, em2c_bytes, args.steps, args.warmup)
        elif args.only == "seismic2_large":  # a grid too large for the chip: one launch per step
            from seidart_gb300 import SEISMIC2
            c = sy.small_case(SEISMIC2, seed=3, nx=2040, nz=1540, npml=20,
                              nstep=args.time_steps if args.time_steps != 6000 else 100, nrec=10)
            c.name = "seismic2 random 2000x1500"
            rec = bench_plain(c, device, flush, stream, peak, seis2_bytes, args.steps, args.warmup)
        elif args.only == "batched":
            tiling = tuple(int(v) for v in args.batch_tiling.split("x")) if args.batch_tiling else None
            rec = bench_batched(device, flush, stream, peak, None, runs=args.steps,
                                nstep=args.time_steps if args.time_steps != 6000 else 4000, tiling=tiling)
        elif args.only == "seismic2_adjoint":
            rec = bench_seismic2_adjoint(device, fd_cells=9)
        else:
            rec = bench_adjoint(device, nstep=args.time_steps)
        print(json.dumps({"only": args.only, **rec}), flush=True)
        return 0

    # ---- headline: electromag2 plain, one shot per bench step --------------
    case = sy.electromag2_layers(nstep=args.time_steps)
    g = case.grid
    solver = make_solver(case, device)
    clocks = ClockSampler(local)
    clocks.start()
    ms = time_shots(solver, case.nstep, args.steps, args.warmup, flush, stream, sync_all)
    ck = clocks.stop()
    if dist is not None:
        t = torch.tensor([ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    cells = g.cells
    value = world * cells * case.nstep / (ms / 1e3) / 1e9
    byts = em2_bytes(g)
    step_ms = ms / case.nstep
    tiles = solver.on_chip()
    if tiles:
        # one launch per shot holds the whole state in shared memory: em2_resident_kernel
        dom_name = "em2_resident_kernel"
        kms = run_times(solver, case.nstep, stream) if not args.headline_only else ms
        per_launch = byts["step"] * case.nstep
        note = (f"state held on chip for the whole run ({tiles[0]} tiles in {tiles[1]} rows, one CTA per SM); "
                "HBM carries only the state's load and store per launch, so algorithmic bytes / time "
                "exceeds the HBM copy peak")
        launches = 3  # begin, the on-chip run, norm reduce
    else:
        # one kernel per step: em2_step_kernel, the whole step's bytes
        dom_name = "em2_step_kernel"
        kms = (kernel_times(solver, stream) if not args.headline_only else [1.0, 1.0])[0]
        per_launch = byts["step"]
        note = "state (23 MB) is L2-resident during a shot; fraction is against the HBM copy peak"
        launches = launches_per_shot(ELECTROMAG2, case.nstep)
    achieved = per_launch / (kms / 1e3) / 1e9
    traffic = profile_traffic(f"{dom_name}_1040x540")
    roofline = {"bound": "hbm", "kernel": dom_name, "achieved": round(achieved, 1), "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": int(per_launch),
                "kernel_ms": round(kms, 5),
                "note": note}
    issue = profile_value(f"{dom_name}_1040x540", "issue_active_pct")
    if issue is not None and dom_name == "em2_resident_kernel":
        # the on-chip kernel's own bound, from its ncu summary of the same workload: the
        # time per step if every SM sub-partition issued an instruction every cycle, and
        # the share of the warps' stalls spent at the block barriers
        bar = profile_value(f"{dom_name}_1040x540", "barrier_stall_per_issue")
        tot = profile_value(f"{dom_name}_1040x540", "total_stall_per_issue")
        us = kms * 1e3 / case.nstep
        roofline["on_chip"] = {"bound": "issue", "issue_active": round(issue / 100, 4),
                               "issue_bound_us_per_step": round(us * issue / 100, 3), "us_per_step": round(us, 3),
                               "barrier_share_of_stalls": round(bar / tot, 3) if bar and tot else None,
                               "source": f"profiles/{dom_name}_1040x540.md (ncu --set full)"}
    step_achieved = byts["step"] / (step_ms / 1e3) / 1e9
    roofline_step = {"bytes_per_cell_update": round(byts["per_cell_step"], 2),
                     "achieved": round(step_achieved, 1), "frac": round(step_achieved / peak, 4), "unit": "GB/s"}
    solver.close()

    line = {
        "metric": METRIC, "value": round(value, 3), "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": DATA,
        "config": bench_config(case.nstep, cells, world),
        "gpu_launches": args.steps * launches,
        "roofline": roofline, "roofline_step": roofline_step,
    }
    if args.headline_only:
        line.pop("roofline")
    if ck:
        line["clocks"] = ck

    # ---- e2e through the public API with host buffers ----------------------
    if args.e2e_steps > 0:
        n_e2e = max(1, min(args.steps, args.e2e_steps))
        shot = (g, case.planes, case.profiles, case.src_ijk, case.srcfn, case.rec_ijk)
        run_shot(*shot, device=device)
        pipe = ShotPipeline(device)  # its two handles made (and kept) before the timed shots
        for _ in pipe.run([shot, shot]):
            pass
        torch.cuda.synchronize()

        def max_rank(el):
            if dist is not None:
                t = torch.tensor([el], dtype=torch.float64)
                dist.all_reduce(t, op=dist.ReduceOp.MAX)
                el = float(t.item())
            return el

        sync_all()
        t0 = time.perf_counter()
        for tr in pipe.run([shot] * n_e2e):
            pass
        torch.cuda.synchronize()
        el = max_rank((time.perf_counter() - t0) / n_e2e)
        pipe.close()
        sync_all()
        t0 = time.perf_counter()
        for _ in range(n_e2e):
            tr1 = run_shot(*shot, device=device)
        torch.cuda.synchronize()
        el1 = max_rank((time.perf_counter() - t0) / n_e2e)
        h2d = 4 * (4 * g.nx * g.nz + 6 * (g.nx + g.nz) + g.nz + 2 * case.nstep + 3 * len(case.rec_ijk))
        d2h = tr.nbytes + 32
        line["e2e"] = {"value": round(world * cells * case.nstep / el / 1e9, 3), "unit": METRIC,
                       "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                       "ms_per_step": round(el * 1e3, 2),
                       "path": "seidart_gb300.solver.ShotPipeline.run (host arrays in, host traces out; two warm "
                               "handles in turn, a shot's host work and uploads overlapping the previous shot's run)",
                       "one_shot_at_a_time": {"value": round(world * cells * case.nstep / el1 / 1e9, 3),
                                              "ms_per_step": round(el1 * 1e3, 2),
                                              "path": "seidart_gb300.solver.run_shot, one call per shot",
                                              "traces_equal": bool(np.array_equal(tr, tr1))}}
        # the same shots with the model as its material-id map and table
        # (sfd_set_model_ids: coefficients formed on the GPU)
        ids, table = case.meta["ids"], case.meta["table"]
        sync_all()
        t0 = time.perf_counter()
        for _ in range(n_e2e):
            tr_ids = run_shot(g, None, case.profiles, case.src_ijk, case.srcfn, case.rec_ijk, device=device, ids=ids,
                              table=table)
        torch.cuda.synchronize()
        el_ids = (time.perf_counter() - t0) / n_e2e
        if dist is not None:
            t = torch.tensor([el_ids], dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            el_ids = float(t.item())
        h2d_ids = h2d - 4 * 4 * g.nx * g.nz + ids.nbytes + table.nbytes
        line["e2e_material_ids"] = {"value": round(world * cells * case.nstep / el_ids / 1e9, 3), "unit": METRIC,
                                    "h2d_bytes_per_step": int(h2d_ids), "d2h_bytes_per_step": int(d2h),
                                    "ms_per_step": round(el_ids * 1e3, 2),
                                    "traces_equal_to_planes_path": bool(np.array_equal(tr_ids, tr)),
                                    "path": "run_shot(ids=, table=): sfd_set_model_ids"}

    # ---- extra lines: the other plain configurations ------------------------
    if not args.skip_extras:
        extras = {}
        extras["seismic2_plain"] = bench_plain(sy.seismic2_firn_ice(nstep=2000), device, flush, stream, peak,
                                               seis2_bytes, 5, 2)
        extras["seismic25_plain"] = bench_plain(sy.seismic25_ice(nstep=3000), device, flush, stream, peak,
                                                seis25_bytes, 2, 1)
        line["extras"] = extras
    par_on = rank == 0 and not args.skip_parity
    if not args.skip_batched:
        picks = (0, 31, 63, 64, 69, 74, 79) if par_on else ()
        line.setdefault("extras", {})["batched"] = bench_batched(device, flush, stream, peak, value / world,
                                                                 parity_models=picks)
    if not args.skip_adjoint:
        line.setdefault("extras", {})["adjoint"] = bench_adjoint(device, fd_cells=args.parity_fd_cells if par_on else 0)
        line["extras"]["seismic2_adjoint"] = bench_seismic2_adjoint(device, fd_cells=9 if par_on else 0)

    # ---- parity: each workload's timed GPU form against the FP64 oracle ------
    if par_on:
        par = {"tolerance_rel_l2": 1e-5,
               "config0_seismic2": parity_plain(sy.seismic2_firn_ice(nstep=2000), device),
               "config1_electromag2": parity_plain(case, device),
               "config2_seismic25": parity_plain(sy.seismic25_ice(nstep=3000), device, nsteps=args.parity_s25_steps)}
        if par["config2_seismic25"]["steps"] < 3000:
            par["config2_seismic25"]["note"] = ("first steps of the 3000-step shot only: the FP64 oracle of the "
                                                "14.6 M-cell grid takes minutes per thousand steps on the host")
        ex = line.get("extras", {})
        if "parity" in ex.get("batched", {}):
            par["config3_batched"] = ex["batched"]["parity"]
        if "parity_fd" in ex.get("adjoint", {}):
            par["config4_adjoint_fd"] = {k: v for k, v in ex["adjoint"]["parity_fd"].items() if k != "per_cell"}
        if "parity_fd" in ex.get("seismic2_adjoint", {}):
            par["seismic2_adjoint_fd"] = {k: v for k, v in ex["seismic2_adjoint"]["parity_fd"].items()
                                          if k != "per_cell"}
        line["parity"] = par

    if rank == 0 and not args.skip_cpu:
        line["cpu_baseline"] = cpu_baseline(case, seconds=args.cpu_seconds)
        line["cpu_baseline"]["with_snapshot_writes"] = cpu_baseline_snapshots(case)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--ref-chunk", type=int, default=200, help="time steps per reference bench step")
    ap.add_argument("--skip-extras", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--time-steps", type=int, default=6000,
                    help="time steps per headline shot (6000 = the workload; smaller only for profiler runs)")
    ap.add_argument("--skip-batched", action="store_true")
    ap.add_argument("--only", choices=["seismic2", "seismic25", "batched", "adjoint", "seismic2_adjoint",
                                       "electromag2_step", "electromag25", "electromag2c", "seismic2_large"],
                    help="run one secondary leg alone and print its record (for profiler runs)")
    ap.add_argument("--skip-adjoint", action="store_true")
    ap.add_argument("--skip-parity", action="store_true",
                    help="skip the comparison of each workload's GPU form with the FP64 oracle (untimed)")
    ap.add_argument("--parity-s25-steps", type=int, default=1000,
                    help="time steps of the seismic25 workload compared with the oracle")
    ap.add_argument("--parity-fd-cells", type=int, default=20,
                    help="cells of the adjoint's finite-difference check (0 = none)")
    ap.add_argument("--batch-tiling", default=None,
                    help="with --only batched: fixed rows-per-thread x blocks-per-SM (e.g. 4x3) instead of the autotuner")
    ap.add_argument("--headline-only", action="store_true",
                    help="only the timed headline shots (for profiler runs): no e2e, extras or CPU leg")
    args = ap.parse_args(argv)
    if args.headline_only:
        args.skip_extras = args.skip_cpu = args.skip_batched = args.skip_adjoint = args.skip_parity = True
        args.e2e_steps = 0
    if args.warmup < 3:
        print("note: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
