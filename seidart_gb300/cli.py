"""``seidartfdtd`` drop-in: the process the SeidarT driver launches.

    python -m seidart_gb300.cli <project.json> seismic=<true|false> density_method=<m> [options]

Same argv and the same working-directory files as the backend that
``Model.run`` calls (``src/seidart/routines/classes.py:878-924``):

* project JSON: ``Domain`` (dim, nx, ny, nz, dx, dy, dz, cpml, alpha_max_scalar,
  kappa_max, NP, NPA, Rcoef) and ``Seismic``/``Electromagnetic`` ``Source``
  (dt, time_steps, xind, yind, zind, source_frequency), as saved by
  ``Model.save_to_json`` (``classes.py:787-836``);
* material planes ``c11.dat ... c66.dat rho.dat`` (+ ``gamma_x/y/z.dat``) or
  ``e11.dat ... e33.dat s11.dat ... s33.dat`` (``classes.py:608-750``);
* source time functions ``seismicsource{x,y,z}.dat`` /
  ``electromagneticsource{x,y,z}.dat`` and the moment-tensor (stress) source
  ``seismicsource{xx,yy,zz,xy,xz,yz}.dat`` (``sourcefunction.py:354-372``);
  a 2-D model takes the in-plane xx, zz, xz components (yy, xy and yz do not
  enter the x-z equations);
* ``density_gradient.dat`` (``definitions.py:475-557``, the air-surface
  density taper the driver writes, ``classes.py:525-533``): the interior
  (nx, nz) factors, extended into the CPML by edge replication, multiply the
  density of a seismic model;
* initial conditions ``initialcondition{V|E}{x,y,z}.dat`` (``classes.py:882-898``).

``density_method`` (``classes.py:311, 910-924``) selects the density
averaging at the staggered velocity points (none, arithmetic, geometric,
harmonic); ``--legacy-quirks`` reproduces the legacy Fortran loops' quirks
instead of the default corrected physics (``SFD_FLAG_LEGACY_QUIRKS``).
``--cpml-mode 2d`` (2-D models) takes the driver's 2-D CPML fields
``{kappa,acoef,bcoef}{,_half}_cpml.dat`` for every derivative direction
instead of per-axis profiles built from the project's CPML parameters.

All are Fortran records, x fastest, full grid (CPML included).  The CPML
profiles are computed from the project's CPML parameters in FP64
(``seidart_gb300.cpml``).  Outputs: one FP32 snapshot record per channel and
per step, named ``{Vx,Vy,Vz|Ex,Ey,Ez}.{step:06d}.{xind}.{[yind.]}{zind}.dat``
with 1-based steps, which is what ``Array.getrcx`` globs
(``src/seidart/routines/arraybuild.py:199-240``).  Snapshots leave the GPU
through page-locked buffers and are written on a background thread while
the GPU steps on.  ``--snapshot-every N``
thins the snapshots and ``--receivers FILE --traces OUT.npy`` records
receiver traces on the device instead.  The exit status is 0 on success, 2
when the run became unstable, and 1 on any input error.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys
import threading
import queue
from pathlib import Path

import numpy as np

from . import cpml as cp
from . import fortran_io as fio
from ._lib import ELECTROMAG2, ELECTROMAG25, SEISMIC2, SEISMIC25, SfdError, UnstableError
from .solver import CHANNELS, FIELDS, MODEL_PLANES, GridSpec, is_25d

# .dat file name of each model plane (the driver's column names, classes.py:608-679)
_FILE_OF = {
    "eps11": "e11", "eps12": "e12", "eps13": "e13", "eps22": "e22", "eps23": "e23", "eps33": "e33",
    "sig11": "s11", "sig12": "s12", "sig13": "s13", "sig22": "s22", "sig23": "s23", "sig33": "s33",
}
_OPTIONAL = {"gamma_x", "gamma_y", "gamma_z"}


class ProjectError(ValueError):
    pass


def parse_flag(args, name, default=None):
    for a in args:
        if a.startswith(name + "="):
            return a.split("=", 1)[1]
    return default


def load_project(json_path, seismic: bool, workdir=".", density_gradient: bool = True):
    """Everything one run needs, read from the project JSON and the .dat files."""
    with open(json_path) as f:
        prj = json.load(f)
    dom = prj["Domain"]
    sec = prj["Seismic" if seismic else "Electromagnetic"]
    src = sec["Source"]
    dim = float(dom["dim"])
    if dim not in (2.0, 2.5):
        raise ProjectError(f"Domain.dim = {dim}: this backend runs 2 and 2.5-D models")
    c = int(dom["cpml"])
    nx, nz = int(dom["nx"]) + 2 * c, int(dom["nz"]) + 2 * c
    ny = int(dom.get("ny", 1)) + 2 * c if dim == 2.5 else 1
    dx, dz = float(dom["dx"]), float(dom["dz"])
    dy = float(dom.get("dy", 1.0))
    kind = (SEISMIC25 if dim == 2.5 else SEISMIC2) if seismic else (ELECTROMAG25 if dim == 2.5 else ELECTROMAG2)
    dt = float(src["dt"])
    nstep = int(src["time_steps"])
    if nstep < 1 or not (dt > 0):
        raise ProjectError("Source.time_steps and Source.dt must be positive")
    grid = GridSpec(kind, nx, nz, dx, dz, dt, c, ny=ny, dy=dy)
    wd = Path(workdir)
    shape2 = (nz, nx)
    planes = []
    for name in MODEL_PLANES[kind]:
        fn = wd / (_FILE_OF.get(name, name) + ".dat")
        if not fn.exists():
            if name in _OPTIONAL:
                planes.append(np.zeros(shape2))
                continue
            raise ProjectError(f"missing model file {fn}")
        planes.append(fio.read_plane(fn, shape2))
    planes = np.stack(planes)
    comps = ["x", "y", "z"] if is_25d(kind) else ["x", "z"]
    stem = "seismicsource" if seismic else "electromagneticsource"
    srcfn = []
    for q in comps:
        fn = wd / f"{stem}{q}.dat"
        if fn.exists():
            s = fio.read_record(fn, np.float64)
            if s.size < nstep:
                raise ProjectError(f"{fn}: {s.size} samples, need {nstep}")
            srcfn.append(s[:nstep])
        else:
            srcfn.append(np.zeros(nstep))
    srcfn = np.stack(srcfn)
    stress = None
    if seismic:  # moment-tensor source: the components the solver carries
        names = ["xx", "yy", "zz", "xy", "xz", "yz"] if is_25d(kind) else ["xx", "zz", "xz"]
        comps_s = []
        for q in names:
            fn = wd / f"seismicsource{q}.dat"
            s = np.zeros(nstep)
            if fn.exists():
                v = fio.read_record(fn, np.float64)
                if v.size < nstep:
                    raise ProjectError(f"{fn}: {v.size} samples, need {nstep}")
                s = v[:nstep]
            comps_s.append(s)
        if any(np.any(s) for s in comps_s):
            stress = np.stack(comps_s)
        gfile = wd / "density_gradient.dat"
        if density_gradient and gfile.exists():
            g = fio.read_record(gfile, np.float64)
            ni, nk = nx - 2 * c, nz - 2 * c
            if g.size != ni * nk:
                raise ProjectError(f"{gfile}: {g.size} values, need {ni} x {nk}")
            if not np.all(np.isfinite(g)) or np.any(g <= 0):
                raise ProjectError(f"{gfile}: density factors must be positive")
            # the driver's (nx, nz) array (written without a transpose) -> (nz, nx), then the CPML
            fac = np.pad(g.reshape(ni, nk).T, c, mode="edge")
            planes[MODEL_PLANES[kind].index("rho")] *= fac
    xind, yind, zind = int(src.get("xind", 0)), int(src.get("yind", 0)), int(src.get("zind", 0))
    src_ijk = (xind + c, (yind + c) if is_25d(kind) else 0, zind + c)
    init = {}
    letter = "V" if seismic else "E"
    fshape = grid.shape
    for q, ch in zip(comps, CHANNELS[kind]):
        fn = wd / f"initialcondition{letter}{q}.dat"
        if fn.exists():
            a = fio.read_record(fn, np.float64)
            if a.size == int(np.prod(fshape)) and np.any(a):
                init[ch] = a.reshape(fshape)
    f0 = float(src.get("source_frequency", 1.0))
    params = {k: float(dom[k]) for k in ("alpha_max_scalar", "kappa_max", "NP", "NPA", "Rcoef") if k in dom}
    vmax, axis_v = max_speed(kind, planes, per_axis=True)
    deltas = (dx, dy, dz) if is_25d(kind) else (dx, dz)
    shape = (nx, ny, nz) if is_25d(kind) else (nx, nz)
    # the driver's seismic sigma_max of an axis takes the largest speed along it (definitions.py:613-661)
    profiles = cp.build_profiles(shape, deltas, c, dt, f0, vmax, seismic=seismic, params=params,
                                 axis_vmax=axis_v if seismic else None)
    return dict(kind=kind, grid=grid, planes=planes, profiles=profiles, srcfn=srcfn, src_ijk=src_ijk,
                init=init, nstep=nstep, xind=xind, yind=yind, zind=zind, seismic=seismic, vmax=vmax,
                stress_srcfn=stress)


def read_cpml2d(workdir, grid):
    """The driver's 2-D CPML fields (definitions.py:560-998): the records of
    {kappa,acoef,bcoef}{,_half}_cpml.dat, (NX, NZ) arrays x fastest, as
    (6, NZ, NX) K, a, b, K_half, a_half, b_half."""
    wd = Path(workdir)
    out = []
    for suffix in ("_cpml.dat", "_half_cpml.dat"):
        for name in ("kappa", "acoef", "bcoef"):
            fn = wd / f"{name}{suffix}"
            if not fn.exists():
                raise ProjectError(f"missing CPML file {fn} (--cpml-mode 2d)")
            out.append(fio.read_plane(fn, (grid.nz, grid.nx)))
    return np.stack(out)


def max_speed(kind, planes, per_axis=False):
    """Largest wave speed of the model over the driver's direction set, and
    with ``per_axis`` also the largest speed along each axis (x, [y,] z), the
    velocities the driver's seismic CPML takes (definitions.py:613-661)."""
    if kind in (ELECTROMAG2, ELECTROMAG25):
        eps = planes[[0, 2]] if kind == ELECTROMAG2 else planes[[0, 3, 5]]
        v = cp.CLIGHT / math.sqrt(max(float(eps.min()), 1e-30))
        return (v, None) if per_axis else v
    names = MODEL_PLANES[kind]
    idx = {n: q for q, n in enumerate(names)}
    rho = planes[idx["rho"]].ravel()
    voigt = {"c11": (0, 0), "c12": (0, 1), "c13": (0, 2), "c14": (0, 3), "c15": (0, 4), "c16": (0, 5),
             "c22": (1, 1), "c23": (1, 2), "c24": (1, 3), "c25": (1, 4), "c26": (1, 5), "c33": (2, 2),
             "c34": (2, 3), "c35": (2, 4), "c36": (2, 5), "c44": (3, 3), "c45": (3, 4), "c46": (3, 5),
             "c55": (4, 4), "c56": (4, 5), "c66": (5, 5)}
    cols = [n for n in names if n in voigt]
    stack = np.stack([planes[idx[n]].ravel() for n in cols] + [rho], axis=1)
    uniq = np.unique(stack, axis=0)
    if len(uniq) > 4096:  # per-cell random media: a strided sample bounds the cost
        uniq = uniq[:: max(1, len(uniq) // 4096)]
    dim = 2.5 if kind == SEISMIC25 else 2
    axes = ("x", "y", "z") if kind == SEISMIC25 else ("x", "z")
    best, along = 0.0, [0.0] * len(axes)
    for row in uniq:
        C6 = np.zeros((6, 6))
        for v, n in zip(row[:-1], cols):
            a, b = voigt[n]
            C6[a, b] = C6[b, a] = v
        if kind == SEISMIC2:  # the 2-D model carries the x-z plane only; fill y as a copy of x
            C6[1, 1], C6[0, 1], C6[1, 0] = C6[0, 0], C6[0, 2], C6[0, 2]
            C6[1, 2], C6[2, 1], C6[3, 3], C6[5, 5] = C6[0, 2], C6[0, 2], C6[4, 4], C6[4, 4]
        if row[-1] > 0:
            best = max(best, cp.max_velocity(C6, row[-1], dim))
            for q, ax in enumerate(axes):
                along[q] = max(along[q], cp.axis_velocity(C6, row[-1], ax))
    return (best, tuple(along)) if per_axis else best


def read_receivers(path, grid):
    """Receiver CSV with a header row and X, Y, Z columns in metres (the
    driver's receiver file, arraybuild.py:142-196) -> full-grid (i, j, k)."""
    rows = []
    with open(path) as f:
        lines = [ln.strip() for ln in f if ln.strip()]
    for ln in lines[1:]:
        vals = [float(v) for v in ln.replace(";", ",").split(",")]
        if len(vals) == 2:
            vals = [vals[0], 0.0, vals[1]]
        rows.append(vals[:3])
    xyz = np.asarray(rows, dtype=np.float64).reshape(-1, 3)
    c = grid.npml
    i = (xyz[:, 0] / grid.dx).astype(int) + c
    k = (xyz[:, 2] / grid.dz).astype(int) + c
    j = (xyz[:, 1] / grid.dy).astype(int) + c if is_25d(grid.kind) else np.zeros(len(xyz), int)
    return np.stack([i, j, k], axis=1).astype(np.int32)


class SnapshotWriter:
    """Drains snapshots through page-locked host buffers.  ``put`` queues the
    device-to-host copy of a field on the solver's stream and returns without
    waiting; background threads wait for that copy's event, write the record
    and hand the buffer back.  The GPU keeps stepping meanwhile; with every
    buffer in flight, ``put`` waits for one to be written."""

    def __init__(self, workdir, solver, nbuf=12, nthreads=4):
        import torch

        self.wd = Path(workdir)
        self.solver = solver
        self.err = None
        self.free = queue.Queue()
        for _ in range(nbuf):
            self.free.put(torch.empty(solver.grid.shape, dtype=torch.float32, pin_memory=True))
        self.q = queue.Queue()
        self.ts = [threading.Thread(target=self._loop, daemon=True) for _ in range(nthreads)]
        for t in self.ts:
            t.start()

    def _loop(self):
        while True:
            item = self.q.get()
            if item is None:
                return
            name, buf, ev = item
            try:
                ev.synchronize()
                fio.write_record(self.wd / name, buf.numpy(), np.float32)
            except (OSError, RuntimeError) as e:
                self.err = e
            finally:
                self.free.put(buf)

    def put(self, name, ch):
        import torch

        buf = self.free.get()
        self.solver.field_async(ch, buf)
        ev = torch.cuda.Event()
        ev.record(self.solver.stream)
        self.q.put((name, buf, ev))

    def close(self):
        for _ in self.ts:
            self.q.put(None)
        for t in self.ts:
            t.join()
        if self.err:
            raise self.err


class BlockDrain:
    """Electromag25 snapshots as SEIDART_EM25B1 block files of ``per_block``
    consecutive steps (``seidart_gb300.em25block``).  Each field is encoded
    to int16 on the GPU, copied into page-locked buffers without waiting,
    and appended to the current block file by one background thread."""

    def __init__(self, workdir, solver, p, per_block, nslots=8):
        import torch

        self.wd = Path(workdir)
        self.solver = solver
        self.p = p
        self.per_block = int(per_block)
        self.chans = CHANNELS[p["kind"]]
        n = int(np.prod(solver.grid.shape))
        self.free = queue.Queue()
        for _ in range(nslots):
            self.free.put({"dev": torch.empty(n, dtype=torch.int16, device=solver.device),
                           "dmm": torch.empty(2, dtype=torch.float32, device=solver.device),
                           "pin": torch.empty(n, dtype=torch.int16, pin_memory=True),
                           "pmm": torch.empty(2, dtype=torch.float32, pin_memory=True)})
        self.err = None
        self.q = queue.Queue()
        self.t = threading.Thread(target=self._loop, daemon=True)
        self.t.start()

    def put(self, step, ch):
        import torch

        slot = self.free.get()
        self.solver.encode_i16(ch, slot["dev"], slot["dmm"])
        with torch.cuda.stream(self.solver.stream):
            slot["pin"].copy_(slot["dev"], non_blocking=True)
            slot["pmm"].copy_(slot["dmm"], non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(self.solver.stream)
        self.q.put((step, ch, slot, ev))

    def _loop(self):
        from . import em25block

        g = self.solver.grid
        w = None
        while True:
            item = self.q.get()
            if item is None:
                break
            step, ch, slot, ev = item
            try:
                ev.synchronize()
                if self.err is None:
                    if w is None or (ch == self.chans[0] and w.steps >= self.per_block):
                        if w is not None:
                            w.close()
                        name = em25block.block_name(self.p["xind"], self.p["yind"], self.p["zind"], step)
                        w = em25block.BlockWriter(self.wd / name, g.nx, g.ny, g.nz, step, self.chans)
                    w.add(step, ch, float(slot["pmm"][0]), float(slot["pmm"][1]), slot["pin"].numpy())
            except (OSError, ValueError, RuntimeError) as e:
                self.err = e
            finally:
                self.free.put(slot)
        if w is not None and self.err is None:
            try:
                w.close()
            except (OSError, ValueError) as e:
                self.err = e

    def close(self):
        self.q.put(None)
        self.t.join()
        if self.err:
            raise self.err


def snapshot_name(ch, step, p):
    ch = ch[0].upper() + ch[1:]  # Vx Vy Vz / Ex Ey Ez, write_image2/3 (readwrite_routines.f95:486)
    if is_25d(p["kind"]):
        return f"{ch}.{step:06d}.{p['xind']}.{p['yind']}.{p['zind']}.dat"
    return f"{ch}.{step:06d}.{p['xind']}.{p['zind']}.dat"


def run(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="seidartfdtd", description=__doc__,
                                 formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("project")
    ap.add_argument("flags", nargs="*", help="seismic=<true|false> density_method=<none|arithmetic|...>")
    ap.add_argument("--workdir", default=".")
    ap.add_argument("--snapshot-every", type=int, default=1, help="write snapshots every N steps (0 = none)")
    ap.add_argument("--em25-blocks", type=int, default=0,
                    help="electromag25: write the snapshots as SEIDART_EM25B1 block files of N steps each "
                         "(int16 block-floating) instead of one FP32 record per channel and step")
    ap.add_argument("--receivers", help="receiver CSV (X,Y,Z in metres)")
    ap.add_argument("--traces", help="write receiver traces (nstep, channel, receiver) to this .npy")
    ap.add_argument("--device", default="cuda")
    ap.add_argument("--legacy-quirks", action="store_true",
                    help="seismic: reproduce the legacy Fortran loops' quirks instead of the corrected physics")
    ap.add_argument("--no-density-gradient", action="store_true",
                    help="seismic: ignore density_gradient.dat")
    ap.add_argument("--cpml-mode", choices=["1d", "2d"], default="1d",
                    help="1d: per-axis CPML profiles from the project's CPML parameters (default); 2d: the driver's "
                         "2-D fields {kappa,acoef,bcoef}{,_half}_cpml.dat for every derivative direction "
                         "(2-D models)")
    a = ap.parse_args(argv)
    seismic = str(parse_flag(a.flags, "seismic", "true")).lower() in ("true", "1", "yes")
    density = str(parse_flag(a.flags, "density_method", "arithmetic")).lower()
    from .solver import DENSITY_FLAGS, FDTDSolver
    if density not in DENSITY_FLAGS:
        print(f"seidartfdtd: density_method={density}: expected one of {', '.join(sorted(DENSITY_FLAGS))}",
              file=sys.stderr)
        return 1
    try:
        p = load_project(a.project, seismic, a.workdir, density_gradient=not a.no_density_gradient)
    except (ProjectError, ValueError, KeyError, OSError) as e:
        print(f"seidartfdtd: {e}", file=sys.stderr)
        return 1
    opts = {"legacy": a.legacy_quirks, "density": density} if seismic else {}
    fields2d = None
    if a.cpml_mode == "2d":
        if p["kind"] not in (ELECTROMAG2, SEISMIC2):
            print("seidartfdtd: --cpml-mode 2d applies to 2-D models (electromag2, seismic2)", file=sys.stderr)
            return 1
        if a.legacy_quirks:
            print("seidartfdtd: --cpml-mode 2d excludes --legacy-quirks (the legacy loops read 1-D profiles)",
                  file=sys.stderr)
            return 1
        try:
            fields2d = read_cpml2d(a.workdir, p["grid"])
        except (ProjectError, ValueError, OSError) as e:
            print(f"seidartfdtd: {e}", file=sys.stderr)
            return 1
    grid = p["grid"]
    rec = read_receivers(a.receivers, grid) if a.receivers else np.zeros((0, 3), np.int32)
    every = max(0, int(a.snapshot_every))
    blocks = max(0, int(a.em25_blocks))
    if blocks and (p["kind"] != ELECTROMAG25 or every != 1):
        print("seidartfdtd: --em25-blocks writes consecutive steps of electromag25 runs "
              "(seismic=false on a 2.5-D project, --snapshot-every 1)", file=sys.stderr)
        return 1
    try:
        from .solver import FLAG_CPML_2D
        with FDTDSolver(grid, p["nstep"], len(rec), device=a.device, flags=FLAG_CPML_2D if fields2d is not None else 0,
                        **opts) as s:
            s.set_model(p["planes"])
            if fields2d is not None:
                s.set_cpml2d(fields2d)
            else:
                s.set_cpml(p["profiles"])
            s.set_source(p["src_ijk"], p["srcfn"])
            if p["stress_srcfn"] is not None:
                s.set_stress_source(p["src_ijk"], p["stress_srcfn"])
            if len(rec):
                s.set_receivers(rec)
            for ch, v in p["init"].items():
                s.set_field(ch, v.astype(np.float32))
            chans = CHANNELS[p["kind"]]
            if blocks:
                writer = BlockDrain(a.workdir, s, p, blocks)
            else:
                writer = SnapshotWriter(a.workdir, s) if every else None
            done = 0
            while done < p["nstep"]:
                n = min(every, p["nstep"] - done) if every else p["nstep"]
                s.run(n)
                done += n
                if writer:
                    for ch in chans:
                        if blocks:
                            writer.put(done, ch)
                        else:
                            writer.put(snapshot_name(ch, done, p), ch)
            if writer:
                writer.close()
            s.status()
            if a.traces and len(rec):
                np.save(a.traces, s.traces())
    except UnstableError as e:
        print(f"seidartfdtd: {e}", file=sys.stderr)
        return 2
    except SfdError as e:
        print(f"seidartfdtd: {e}", file=sys.stderr)
        return 1
    return 0


def main():
    sys.exit(run())


if __name__ == "__main__":
    main()
