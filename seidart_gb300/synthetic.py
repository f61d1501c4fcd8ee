"""Seeded synthetic models with the shapes, sizes and value ranges of the
workloads the backend is measured on, plus small random models for parity
tests.  No dataset is involved: the reference measures nothing public, so
every input here is generated from a seed.

Index conventions follow the solver: full grid (CPML included), 0-based,
x fastest; an interior (driver) cell index ``ix`` is full-grid ``ix + npml``.
Source time functions use the reference's Ricker form ``gaus1``
(``src/seidart/routines/sourcefunction.py:35-38``, normalised to unit peak).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import cpml as cp
from ._lib import ELECTROMAG2, ELECTROMAG25, ELECTROMAG2C, SEISMIC2, SEISMIC25
from .solver import GridSpec, is_25d


@dataclass
class Case:
    name: str
    grid: GridSpec
    planes: np.ndarray          # (nplanes, NZ, NX) float64
    profiles: list              # cpml.AxisProfile per axis
    src_ijk: tuple
    srcfn: np.ndarray           # (ncomp, nstep) float64
    rec_ijk: np.ndarray         # (nrec, 3) int32
    f0: float
    meta: dict = field(default_factory=dict)
    # seismic kinds: stress source (3 | 6, nstep) at src_ijk, legacy quirks, density method
    stress_srcfn: Optional[np.ndarray] = None
    legacy: bool = False
    density: str = "arithmetic"

    @property
    def nstep(self) -> int:
        return self.srcfn.shape[1]

    def solver_options(self) -> dict:
        """FDTDSolver keywords of the case's physics options."""
        if self.grid.kind in (SEISMIC2, SEISMIC25):
            return {"legacy": self.legacy, "density": self.density}
        return {}


def ricker(nstep: int, dt: float, f0: float, amp: float = 1.0) -> np.ndarray:
    """gaus1 wavelet of sourcefunction.py:35-38 (peak-normalised), times amp."""
    t = np.arange(nstep) * dt
    a = np.pi * f0 * (t - 1.0 / f0)
    x = (1.0 - 2.0 * a * a) * np.exp(-a * a)
    return amp * x / np.max(np.abs(x))


def wavelet(t: np.ndarray, f: float, stype: str = "gaus1") -> np.ndarray:
    """The driver's Gaussian source wavelets at times t, peak-normalised
    (sourcefunction.py:25-57): 'gaus0' a Gaussian of width 0.2/(pi f),
    'gaus1' the Ricker wavelet, 'gaus2' the second derivative form; each
    centred on t0 = 1/f."""
    t0 = 1.0 / f
    if stype == "gaus0":
        a = (t - t0) / (0.2 / (math.pi * f))
        x = np.exp(-a * a)
    elif stype == "gaus1":
        a = math.pi * f * (t - t0)
        x = (1.0 - 2.0 * a * a) * np.exp(-a * a)
    elif stype == "gaus2":
        k = math.pi * math.pi * f * f
        d = t - t0
        x = 2.0 * k * d * (2.0 * k * d * d - 3.0) * np.exp(-k * d * d)
    else:
        raise ValueError(f"unknown wavelet {stype!r}")
    return x / np.max(np.abs(x))


def extend_cpml(interior: np.ndarray, npml: int) -> np.ndarray:
    """(nz, nx) interior -> (nz+2c, nx+2c) by edge replication (classes.py:660-674)."""
    return np.pad(interior, npml, mode="edge")


# ---------------------------------------------------------------------------
# Stiffness helpers

def iso_voigt(lam, mu):
    C = np.zeros(np.shape(lam) + (6, 6))
    C[..., 0, 0] = C[..., 1, 1] = C[..., 2, 2] = lam + 2 * mu
    C[..., 0, 1] = C[..., 0, 2] = C[..., 1, 2] = C[..., 1, 0] = C[..., 2, 0] = C[..., 2, 1] = lam
    C[..., 3, 3] = C[..., 4, 4] = C[..., 5, 5] = mu
    return C


def hex_voigt(C11, C33, C13, C12, C44):
    C = np.zeros((6, 6))
    C[0, 0] = C[1, 1] = C11
    C[2, 2] = C33
    C[0, 1] = C[1, 0] = C12
    C[0, 2] = C[2, 0] = C[1, 2] = C[2, 1] = C13
    C[3, 3] = C[4, 4] = C44
    C[5, 5] = 0.5 * (C11 - C12)
    return C


def bond_matrix(R: np.ndarray) -> np.ndarray:
    """6x6 Bond stress-transformation matrices for rotations R (..., 3, 3)."""
    R = np.asarray(R)
    M = np.zeros(R.shape[:-2] + (6, 6))
    pairs = [(0, 0), (1, 1), (2, 2), (1, 2), (0, 2), (0, 1)]
    for I, (i, j) in enumerate(pairs):
        for J, (k, l) in enumerate(pairs):
            if J < 3:
                M[..., I, J] = R[..., i, k] * R[..., j, l]
            else:
                M[..., I, J] = R[..., i, k] * R[..., j, l] + R[..., i, l] * R[..., j, k]
    return M


def rotation(tilt, azim):
    """c-axis tilted by ``tilt`` from z toward azimuth ``azim`` (radians): R = Rz(azim) Ry(tilt)."""
    ct, st, ca, sa = np.cos(tilt), np.sin(tilt), np.cos(azim), np.sin(azim)
    Ry = np.zeros(np.shape(tilt) + (3, 3))
    Ry[..., 0, 0] = ct; Ry[..., 0, 2] = st; Ry[..., 1, 1] = 1.0; Ry[..., 2, 0] = -st; Ry[..., 2, 2] = ct
    Rz = np.zeros(np.shape(azim) + (3, 3))
    Rz[..., 0, 0] = ca; Rz[..., 0, 1] = -sa; Rz[..., 1, 0] = sa; Rz[..., 1, 1] = ca; Rz[..., 2, 2] = 1.0
    return Rz @ Ry


VOIGT21 = [(0, 0), (0, 1), (0, 2), (0, 3), (0, 4), (0, 5), (1, 1), (1, 2), (1, 3), (1, 4), (1, 5),
           (2, 2), (2, 3), (2, 4), (2, 5), (3, 3), (3, 4), (3, 5), (4, 4), (4, 5), (5, 5)]


def max_velocity_batch(C6: np.ndarray, rho: np.ndarray, dim) -> float:
    """Largest Christoffel velocity over all cells and the driver's direction set."""
    s = 1.0 / math.sqrt(2.0)
    dirs = [(1, 0, 0), (0, 0, 1), (s, 0, s)] if dim == 2 else \
        [(1, 0, 0), (0, 1, 0), (0, 0, 1), (s, s, 0), (s, 0, s), (0, s, s)]
    flat = C6.reshape(-1, 6, 6)
    r = np.broadcast_to(rho, C6.shape[:-2]).reshape(-1)
    # unique tensors only (layered models repeat a handful)
    key = np.concatenate([flat.reshape(len(flat), -1), r[:, None]], axis=1)
    uniq, inv = np.unique(key, axis=0, return_index=True)
    best = 0.0
    for row in uniq:
        C = row[:36].reshape(6, 6)
        for d in dirs:
            best = max(best, float(cp.christoffel_velocities(C, row[36], np.array(d, float)).max()))
    return best


# ---------------------------------------------------------------------------
# The measured workloads

def seismic2_firn_ice(nstep: int = 2000) -> Case:
    """2-D anisotropic elastic, 400x200, dx=dz=0.5 m, 20-cell CPML, firn over ice,
    200 Hz Ricker Fz at (200, 45), Courant 0.5, 40 surface receivers every 10 cells."""
    nx, nz, c, d = 400, 200, 20, 0.5
    firn = dict(rho=500.0, c11=5e9, c33=5e9, c13=2e9, c55=1.5e9)
    ice = dict(rho=917.0, c11=13.9e9, c33=15.0e9, c13=5.8e9, c55=3.0e9)
    interior = {k: np.where(np.arange(nz)[:, None] < 40, firn[k], ice[k]) * np.ones((nz, nx))
                for k in firn}
    ext = {k: extend_cpml(v, c) for k, v in interior.items()}
    NX, NZ = nx + 2 * c, nz + 2 * c
    zero = np.zeros((NZ, NX))
    planes = np.stack([ext["c11"], ext["c13"], zero, ext["c33"], zero, ext["c55"], ext["rho"], zero, zero])
    vmax = 0.0
    for m in (firn, ice):
        C6 = np.zeros((6, 6))
        C6[0, 0], C6[2, 2], C6[0, 2], C6[2, 0], C6[4, 4] = m["c11"], m["c33"], m["c13"], m["c13"], m["c55"]
        C6[1, 1], C6[1, 2], C6[2, 1], C6[0, 1], C6[1, 0] = m["c11"], m["c13"], m["c13"], m["c13"], m["c13"]
        C6[3, 3] = C6[5, 5] = m["c55"]
        vmax = max(vmax, cp.max_velocity(C6, m["rho"], 2))
    dt = cp.time_step(0.5, vmax, (d, d))
    f0 = 200.0
    grid = GridSpec(SEISMIC2, NX, NZ, d, d, dt, c)
    profiles = cp.build_profiles((NX, NZ), (d, d), c, dt, f0, vmax, seismic=True)
    srcfn = np.zeros((2, nstep))
    srcfn[1] = ricker(nstep, dt, f0)
    rec = np.array([[10 * q + c, 0, c] for q in range(40)], dtype=np.int32)
    return Case("seismic2 firn/ice 400x200", grid, planes, profiles, (200 + c, 0, 45 + c), srcfn, rec, f0,
                dict(vmax=vmax))


def _random_interfaces(rng, nx, n_if=2, nvert=8, zmin=100, zmax=400):
    xs = np.linspace(0, nx - 1, nvert)
    lines = []
    for q in range(n_if):
        lo = zmin + q * (zmax - zmin) / n_if
        hi = zmin + (q + 1) * (zmax - zmin) / n_if
        zs = rng.uniform(lo, hi, nvert)
        lines.append(np.interp(np.arange(nx), xs, zs))
    return lines


def electromag2_layers(nstep: int = 6000, src_x: int = 500, nx: int = 1000, nz: int = 500) -> Case:
    """2-D anisotropic EM, 1000x500, dx=dz=0.05 m, 20-cell CPML, three layers with
    seeded polygonal interfaces, eps in [1.5, 3.2], sigma log-uniform in [1e-6, 1e-3],
    100 MHz Ricker Ex source at (src_x, 25), 100 receivers, CFL 1/sqrt(2)."""
    c, d = 20, 0.05
    rng_geo = np.random.default_rng(1)
    lines = _random_interfaces(rng_geo, nx, zmin=100 * nz / 500, zmax=400 * nz / 500)
    layer = np.zeros((nz, nx), dtype=np.int32)
    zz = np.arange(nz)[:, None]
    for q, ln in enumerate(lines):
        layer[zz >= ln[None, :]] = q + 1
    rng = np.random.default_rng(2)
    e11 = rng.uniform(1.5, 3.2, 3)
    e33 = rng.uniform(1.5, 3.2, 3)
    e13 = rng.uniform(0.0, 0.05, 3)
    s11 = 10 ** rng.uniform(-6, -3, 3)
    mats = dict(eps11=e11, eps13=e13, eps33=e33, sig11=s11, sig13=np.zeros(3), sig33=s11)
    NX, NZ = nx + 2 * c, nz + 2 * c
    planes = np.stack([extend_cpml(mats[k][layer], c) for k in ["eps11", "eps13", "eps33", "sig11", "sig13", "sig33"]])
    vmax = cp.CLIGHT / math.sqrt(min(e11.min(), e33.min()))
    dt = cp.time_step(1.0 / math.sqrt(2.0), vmax, (d, d))
    f0 = 100e6
    grid = GridSpec(ELECTROMAG2, NX, NZ, d, d, dt, c)
    profiles = cp.build_profiles((NX, NZ), (d, d), c, dt, f0, vmax, seismic=False)
    srcfn = np.zeros((2, nstep))
    srcfn[0] = ricker(nstep, dt, f0)
    nrec = 100
    rec = np.array([[min(nx - 1, 10 * q + 5) + c, 0, 25 + c] for q in range(nrec)], dtype=np.int32)
    # the same model as a material-id map (CPML cells take their edge's id) and its table
    ids = extend_cpml(layer, c).astype(np.int32)
    table = np.column_stack([mats[k] for k in ["eps11", "eps13", "eps33", "sig11", "sig13", "sig33"]])
    return Case(f"electromag2 layers {nx}x{nz}", grid, planes, profiles, (src_x + c, 0, 25 + c), srcfn, rec, f0,
                dict(vmax=vmax, layers=layer, ids=ids, table=table))


def seismic25_ice(nstep: int = 3000, nx: int = 600, ny: int = 40, nz: int = 300, c: int = 15,
                  explosive: bool = True) -> Case:
    """2.5-D anisotropic elastic, 600x40x300, 1 m cells, 15-cell CPML, per-(x,z)
    hexagonal ice rotated by tilt U[0,30] deg / azimuth U[0,360) (seed 3),
    gamma U[0,0.02] per axis (seed 4), 150 Hz Ricker explosive source at
    (300,20,150) (equal normal stress components, the driver's 'tnt' source,
    src/seidart/routines/sourcefunction.py:305-311), CFL 1/sqrt(3), 100
    receivers on the surface line y=20.  ``explosive=False`` applies the
    wavelet as equal x, y, z forces instead (the legacy seismic25 injects
    forces only)."""
    d = 1.0
    rng = np.random.default_rng(3)
    tilt = np.deg2rad(rng.uniform(0, 30, (nz, nx)))
    azim = np.deg2rad(rng.uniform(0, 360, (nz, nx)))
    H = hex_voigt(13.9e9, 15.0e9, 5.8e9, 7.1e9, 3.0e9)
    M = bond_matrix(rotation(tilt, azim))
    C = M @ H @ np.swapaxes(M, -1, -2)
    rng4 = np.random.default_rng(4)
    gam = rng4.uniform(0, 0.02, (3, nz, nx))
    NX, NY, NZ = nx + 2 * c, ny + 2 * c, nz + 2 * c
    planes = [extend_cpml(C[..., a, b], c) for a, b in VOIGT21]
    planes.append(extend_cpml(np.full((nz, nx), 917.0), c))
    planes += [extend_cpml(g, c) for g in gam]
    planes = np.stack(planes)
    vmax = max_velocity_batch(C[::7, ::7], 917.0, 2.5)
    vmax = max(vmax, cp.max_velocity(H, 917.0, 2.5))
    dt = cp.time_step(1.0 / math.sqrt(3.0), vmax, (d, d, d))
    f0 = 150.0
    grid = GridSpec(SEISMIC25, NX, NZ, d, d, dt, c, ny=NY, dy=d)
    profiles = cp.build_profiles((NX, NY, NZ), (d, d, d), c, dt, f0, vmax, seismic=True)
    rec = np.array([[min(nx - 1, 6 * q) + c, 20 + c, c] for q in range(100)], dtype=np.int32)
    src = (nx // 2 + c, 20 + c, nz // 2 + c)
    if explosive:
        w = ricker(nstep, dt, f0)
        z = np.zeros(nstep)
        return Case(f"seismic25 ice {nx}x{ny}x{nz}", grid, planes, profiles, src, np.zeros((3, nstep)), rec, f0,
                    dict(vmax=vmax), stress_srcfn=np.stack([w, w, w, z, z, z]))
    w = ricker(nstep, dt, f0) / math.sqrt(3.0)
    return Case(f"seismic25 ice {nx}x{ny}x{nz}", grid, planes, profiles, src, np.stack([w, w, w]), rec, f0,
                dict(vmax=vmax))


# ---------------------------------------------------------------------------
# Small random models (parity tests)

def small_case(kind: int, seed: int = 0, nx: int = 48, nz: int = 40, ny: int = 24, npml: int = 6,
               nstep: int = 200, nrec: int = 12, atten: bool = True) -> Case:
    """A small model with per-cell random material noise (every averaging index
    matters), a Ricker source near the centre and receivers spread over the
    grid, including inside the CPML strips.  Sizes are full-grid."""
    rng = np.random.default_rng(seed)
    three = is_25d(kind)
    NX, NZ, NY = nx, nz, (ny if three else 1)
    d = 0.5 if kind in (SEISMIC2, SEISMIC25) else 0.05
    shape2 = (NZ, NX)
    noise = lambda s=0.1: 1.0 + s * rng.uniform(-1, 1, shape2)
    if kind == SEISMIC2:
        rho = 900.0 * noise()
        lam, mu = 6e9 * noise(), 3e9 * noise()
        c11, c33 = (lam + 2 * mu) * noise(0.05), (lam + 2 * mu) * noise(0.05)
        c13, c55 = lam.copy(), mu.copy()
        c15, c35 = 0.05 * mu * rng.uniform(-1, 1, shape2), 0.05 * mu * rng.uniform(-1, 1, shape2)
        g = (lambda: 0.002 * rng.uniform(0, 1, shape2)) if atten else (lambda: np.zeros(shape2))
        planes = np.stack([c11, c13, c15, c33, c35, c55, rho, g(), g()])
        vmax = float(np.sqrt((np.maximum(c11, c33) / rho).max())) * 1.05
        cfl = 0.45
        seismic = True
        f0 = 400.0
    elif kind == SEISMIC25:
        rho = 917.0 * noise()
        H = hex_voigt(13.9e9, 15.0e9, 5.8e9, 7.1e9, 3.0e9)
        R = rotation(np.deg2rad(rng.uniform(0, 30, shape2)), np.deg2rad(rng.uniform(0, 360, shape2)))
        M = bond_matrix(R)
        C = (M @ H @ np.swapaxes(M, -1, -2)) * noise(0.05)[..., None, None]
        g = (lambda: 0.002 * rng.uniform(0, 1, shape2)) if atten else (lambda: np.zeros(shape2))
        planes = np.stack([C[..., a, b] for a, b in VOIGT21] + [rho, g(), g(), g()])
        vmax = float(np.sqrt(C[..., 2, 2].max() / rho.min())) * 1.15
        cfl = 0.4
        seismic = True
        f0 = 300.0
    elif kind == ELECTROMAG2C:  # complex permittivities with small loss (negative imaginary) parts
        e11, e33 = 2.0 * noise(0.3), 2.2 * noise(0.3)
        e13 = 0.03 * rng.uniform(0, 1, shape2)
        im = lambda e: -0.02 * e * rng.uniform(0, 1, shape2)
        s11 = 10 ** rng.uniform(-5, -2.5, shape2)
        s33 = 10 ** rng.uniform(-5, -2.5, shape2)
        s13 = 1e-4 * rng.uniform(0, 1, shape2)
        planes = np.stack([e11, im(e11), e13, 0.1 * im(e13), e33, im(e33), s11, s13, s33])
        vmax = cp.CLIGHT / math.sqrt(min(e11.min(), e33.min()))
        cfl = 0.6
        seismic = False
        f0 = 400e6
    elif kind == ELECTROMAG2:
        e11, e33 = 2.0 * noise(0.3), 2.2 * noise(0.3)
        e13 = 0.03 * rng.uniform(0, 1, shape2)
        s11 = 10 ** rng.uniform(-5, -2.5, shape2)
        s33 = 10 ** rng.uniform(-5, -2.5, shape2)
        s13 = 1e-4 * rng.uniform(0, 1, shape2)
        planes = np.stack([e11, e13, e33, s11, s13, s33])
        vmax = cp.CLIGHT / math.sqrt(min(e11.min(), e33.min()))
        cfl = 0.6
        seismic = False
        f0 = 400e6
    else:
        e = [2.0 * noise(0.3), 0.02 * rng.uniform(0, 1, shape2), 0.02 * rng.uniform(0, 1, shape2),
             2.1 * noise(0.3), 0.02 * rng.uniform(0, 1, shape2), 2.2 * noise(0.3)]
        s = [10 ** rng.uniform(-5, -2.5, shape2), 1e-5 * rng.uniform(0, 1, shape2), 1e-5 * rng.uniform(0, 1, shape2),
             10 ** rng.uniform(-5, -2.5, shape2), 1e-5 * rng.uniform(0, 1, shape2), 10 ** rng.uniform(-5, -2.5, shape2)]
        planes = np.stack(e + s)
        vmax = cp.CLIGHT / math.sqrt(min(e[0].min(), e[3].min(), e[5].min()))
        cfl = 0.5
        seismic = False
        f0 = 400e6
    deltas = (d, d, d) if three else (d, d)
    dt = cp.time_step(cfl, vmax, deltas)
    grid = GridSpec(kind, NX, NZ, d, d, dt, npml, ny=NY, dy=d)
    shape = (NX, NY, NZ) if three else (NX, NZ)
    profiles = cp.build_profiles(shape, deltas, npml, dt, f0, vmax, seismic=seismic)
    ncomp = 3 if three else 2
    w = ricker(nstep, dt, f0)
    srcfn = np.stack([w * (0.7 + 0.3 * q) * (-1) ** q for q in range(ncomp)])
    src = (NX // 2 + 1, NY // 2 if three else 0, NZ // 2 - 1)
    rec = np.stack([rng.integers(1, NX - 1, nrec), rng.integers(1, NY - 1, nrec) if three else np.zeros(nrec, int),
                    rng.integers(1, NZ - 1, nrec)], axis=1).astype(np.int32)
    return Case(f"small {kind} seed {seed}", grid, np.ascontiguousarray(planes), profiles, src, srcfn, rec, f0,
                dict(vmax=vmax))


def batched_survey(nshots: int = 64, nelastic: int = 16, nstep: int = 4000, em=None):
    """The batched workload: ``nshots`` EM shots of the layered 1000x500 model with
    sources every 15 cells along the surface, plus ``nelastic`` seeded 2-D elastic
    models of uneven size (nx in [200,1200], nz in [100,600]) built from the
    firn/ice materials with a seeded interface depth."""
    base = em or electromag2_layers(nstep=nstep)
    shots = []
    for q in range(nshots):
        c = base.grid.npml
        x = 12 + 15 * q
        shots.append(Case(f"em shot {q}", base.grid, base.planes, base.profiles, (x + c, 0, 25 + c), base.srcfn,
                          base.rec_ijk, base.f0, base.meta))
    rng = np.random.default_rng(5)
    models = []
    for q in range(nelastic):
        nx = int(rng.integers(200, 1201))
        nz = int(rng.integers(100, 601))
        cut = int(rng.uniform(0.1, 0.5) * nz)
        models.append(_elastic_two_layer(nx, nz, cut, nstep, name=f"elastic {q} {nx}x{nz}"))
    return shots, models


def _elastic_two_layer(nx, nz, cut, nstep, c=20, d=0.5, name="elastic"):
    firn = dict(rho=500.0, c11=5e9, c33=5e9, c13=2e9, c55=1.5e9)
    ice = dict(rho=917.0, c11=13.9e9, c33=15.0e9, c13=5.8e9, c55=3.0e9)
    interior = {k: np.where(np.arange(nz)[:, None] < cut, firn[k], ice[k]) * np.ones((nz, nx)) for k in firn}
    ext = {k: extend_cpml(v, c) for k, v in interior.items()}
    NX, NZ = nx + 2 * c, nz + 2 * c
    zero = np.zeros((NZ, NX))
    planes = np.stack([ext["c11"], ext["c13"], zero, ext["c33"], zero, ext["c55"], ext["rho"], zero, zero])
    vmax = math.sqrt(15.0e9 / 917.0) * 1.0001
    dt = cp.time_step(0.5, vmax, (d, d))
    f0 = 200.0
    grid = GridSpec(SEISMIC2, NX, NZ, d, d, dt, c)
    profiles = cp.build_profiles((NX, NZ), (d, d), c, dt, f0, vmax, seismic=True)
    srcfn = np.zeros((2, nstep))
    srcfn[1] = ricker(nstep, dt, f0)
    src = (nx // 2 + c, 0, min(45, nz - 10) + c)
    rec = np.array([[int(q * (nx - 1) / 39) + c, 0, c] for q in range(40)], dtype=np.int32)
    return Case(name, grid, planes, profiles, src, srcfn, rec, f0, dict(vmax=vmax))
