"""Batched runs: many 2-D shots and models in one persistent launch.

The reference runs one ``seidartfdtd`` process per source position and
re-reads every snapshot afterwards (``src/seidart/simulations/common_offset.py:143-284``).
Here every shot/model is an :class:`~seidart_gb300.solver.FDTDSolver` and a
:class:`Batch` advances all of them together in one cooperative kernel launch
per run (``sfd_batch_run``), with per-model receivers gathered on the device.

:func:`autotune` picks the tile depth (rows per thread) and blocks per SM of
that launch by timing a few steps of each candidate on the batch itself, and
caches the choice per batch signature and GPU.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import time
from pathlib import Path

from . import _lib
from ._lib import check

CANDIDATES = [(1, 3), (2, 3), (4, 3), (1, 2), (2, 2), (4, 2), (2, 1)]


def _declare(L):
    if getattr(L, "_batch_declared", False):
        return
    P, i32, i64, sz = C.c_void_p, C.c_int32, C.c_int64, C.c_size_t
    for name, res, args in [
        ("sfd_batch_scratch_bytes", i32, [i32, C.POINTER(sz)]),
        ("sfd_batch_create", i32, [C.POINTER(P), i32, P, sz, C.POINTER(P)]),
        ("sfd_batch_set_tiling", i32, [P, i32, i32]),
        ("sfd_batch_run", i32, [P, i64]),
        ("sfd_batch_status", i32, [P, C.POINTER(i32)]),
        ("sfd_batch_set_wait_limit", i32, [P, i64]),
        ("sfd_batch_test_stall_waits", i32, [P, i32]),
        ("sfd_batch_destroy", i32, [P]),
    ]:
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    L._batch_declared = True


class Batch:
    """Advance a list of single-pass 2-D solvers together (same device and stream)."""

    def __init__(self, solvers):
        import torch

        if not solvers:
            raise ValueError("empty batch")
        self.solvers = list(solvers)
        L = _lib.lib()
        _declare(L)
        self._L = L
        n = len(self.solvers)
        nbytes = C.c_size_t()
        check(L.sfd_batch_scratch_bytes(n, C.byref(nbytes)))
        self.scratch = torch.empty(int(nbytes.value), dtype=torch.uint8, device=self.solvers[0].device)
        arr = (C.c_void_p * n)(*[s._h.value for s in self.solvers])
        b = C.c_void_p()
        check(L.sfd_batch_create(arr, n, C.c_void_p(self.scratch.data_ptr()), nbytes, C.byref(b)))
        self._b = b
        self.tiling = (2, 3)

    @property
    def cells(self) -> int:
        return sum(s.grid.cells for s in self.solvers)

    def set_tiling(self, zb: int, blocks_per_sm: int) -> None:
        check(self._L.sfd_batch_set_tiling(self._b, int(zb), int(blocks_per_sm)))
        self.tiling = (int(zb), int(blocks_per_sm))

    def run(self, nsteps: int) -> None:
        check(self._L.sfd_batch_run(self._b, int(nsteps)))

    def set_wait_limit(self, ns: int) -> None:
        """Longest wait (ns) at the kernel's grid barrier; 0 = the default 2 s."""
        check(self._L.sfd_batch_set_wait_limit(self._b, int(ns)))

    def status(self) -> None:
        """Synchronise; raise on a barrier timeout or a blown-up model."""
        m = C.c_int32(-1)
        rc = self._L.sfd_batch_status(self._b, C.byref(m))
        if rc != 0:
            msg = self._L.sfd_last_error().decode(errors="replace")
            cls = _lib.UnstableError if rc == _lib.SFD_ERR_UNSTABLE else _lib.SfdError
            raise cls(rc, f"{msg} (model {m.value})")

    def reset(self) -> None:
        for s in self.solvers:
            s.reset()

    def signature(self) -> str:
        import torch
        dev = torch.cuda.get_device_name(self.solvers[0].device)
        key = [dev] + [f"{s.kind}:{s.grid.nx}x{s.grid.nz}" for s in self.solvers]
        return hashlib.sha1("|".join(key).encode()).hexdigest()[:16]

    def close(self) -> None:
        if getattr(self, "_b", None):
            self._L.sfd_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _cache_path() -> Path:
    return Path(os.environ.get("SEIDART_GB300_TUNING", Path.home() / ".cache" / "seidart_gb300" / "tuning.json"))


def autotune(batch: Batch, steps: int = 16, candidates=CANDIDATES, use_cache: bool = True, verbose: bool = False):
    """Time each (rows per thread, blocks per SM) candidate for ``steps`` steps
    and keep the fastest.  The trial steps advance the models, so every
    solver is reset afterwards: call this before the real run."""
    import torch

    path = _cache_path()
    sig = batch.signature()
    cache = {}
    if use_cache and path.exists():
        try:
            cache = json.loads(path.read_text())
        except (OSError, ValueError):
            cache = {}
    if use_cache and sig in cache:
        zb, bps = cache[sig]["tiling"]
        batch.set_tiling(zb, bps)
        return {"tiling": (zb, bps), "cached": True, "timings": cache[sig].get("timings", {})}
    timings = {}
    best = None
    for zb, bps in candidates:
        try:
            batch.set_tiling(zb, bps)
        except _lib.SfdError:
            continue
        batch.reset()
        batch.run(2)
        batch.status()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        batch.run(steps)
        batch.status()
        el = (time.perf_counter() - t0) / steps
        timings[f"{zb}x{bps}"] = el
        if verbose:
            print(f"autotune zb={zb} blocks/SM={bps}: {el * 1e3:.3f} ms/step")
        if best is None or el < best[0]:
            best = (el, zb, bps)
    if best is None:
        raise RuntimeError("no tiling candidate could be launched")
    batch.set_tiling(best[1], best[2])
    batch.reset()
    if use_cache:
        cache[sig] = {"tiling": [best[1], best[2]], "timings": timings}
        try:
            path.parent.mkdir(parents=True, exist_ok=True)
            path.write_text(json.dumps(cache, indent=1))
        except OSError:
            pass
    return {"tiling": (best[1], best[2]), "cached": False, "timings": timings}
