"""FP64 host computation of the CPML damping profiles, the time step and the
Christoffel velocities that set them.

The solvers consume one 1-D profile per axis and per grid offset (full node
and half node): ``K``, ``a`` and ``b`` (``alpha`` and ``sigma`` are returned
for inspection).  By default (``mode="driver"``) the profiles are those the
current driver's 2-D CPML fields hold along each edge, away from the corners
(``src/seidart/routines/definitions.py:560-998``; ``driver_fields_2d``
builds the whole fields).  The profile shape (as in the reference's 1-D
writer, ``legacy/prjrun_101424.py:174-303``): ``sigma = sigma_max d^NP``,
``kappa = 1 + (kappa_max - 1) d^NP``, ``alpha = alpha_max (1 - d)^NPA``,
``b = exp(-(sigma/kappa + alpha) dt)`` -- ``dt/eps0`` for EM -- and
``a = sigma (b - 1) / (kappa sigma + kappa alpha)`` where ``|sigma| > 1e-6``;
interior cells keep ``K = 1, a = 0, b = 0``).  ``sigma_max`` and
``alpha_max`` follow the current driver's "global" mode
(``src/seidart/routines/definitions.py:646-699``) or, with
``mode="legacy"``, the legacy writer (``legacy/prjrun_101424.py:226-244``).

Everything here is FP64 and runs once per model on the host.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

# src/seidart/routines/definitions.py:67-69
CLIGHT = 2.99792458e8
EPS0 = 8.85418782e-12
MU0 = 4.0 * np.pi * 1.0e-7

# Project-file defaults, src/seidart/routines/prjbuild.py:43-49
DEFAULT_CPML = dict(alpha_max_scalar=1.0, kappa_max=5.0, NP=2.0, NPA=2.0, Rcoef=0.001)


@dataclass
class AxisProfile:
    """CPML coefficients of one axis, full-node and half-node offsets."""
    K: np.ndarray
    a: np.ndarray
    b: np.ndarray
    K_half: np.ndarray
    a_half: np.ndarray
    b_half: np.ndarray
    alpha: np.ndarray
    alpha_half: np.ndarray
    sigma: np.ndarray
    sigma_half: np.ndarray

    def packed(self) -> np.ndarray:
        """K, a, b, K_half, a_half, b_half stacked (6, n): the solver layout."""
        return np.stack([self.K, self.a, self.b, self.K_half, self.a_half, self.b_half])


def _distance(npml, delta, half, mode):
    """Normalised distance into the layer of its npml cells, outermost first.
    The driver's cpml_parameters rescales it so that its largest value is 1
    (definitions.py:933-934, which moves the half-offset profile by half a
    cell); the legacy writer does not."""
    dist = delta * np.arange(npml, dtype=np.float64)
    if half:
        dist = dist + delta / 2.0
    dist = (delta * npml - dist) / (delta * npml)
    if mode == "driver":
        dist = dist / dist.max()
    return dist


def _profile_1d(n, npml, delta, dt, sig_max, alpha_max, kappa_max, NP, NPA, seismic, half, mode="driver"):
    """One offset of one axis: the profile the driver's cpml_parameters writes
    along an edge of its 2-D field away from the corners
    (src/seidart/routines/definitions.py:862-998; interior b = exp(0) = 1),
    or, with ``mode="legacy"``, legacy/prjrun_101424.py:174-303 (interior
    b = 0).  Where a = 0 a memory variable stays zero whatever b is."""
    kappa = np.ones(n)
    alpha = np.zeros(n)
    sigma = np.zeros(n)
    acoef = np.zeros(n)
    scale = dt if seismic else dt / EPS0
    bcoef = np.ones(n) if mode == "driver" else np.zeros(n)
    dist = _distance(npml, delta, half, mode)
    for ind in range(npml):
        for pos in (ind, n - 1 - ind):
            sigma[pos] = sig_max * dist[ind] ** NP
            kappa[pos] = 1.0 + (kappa_max - 1.0) * dist[ind] ** NP
            alpha[pos] = alpha_max * (1.0 - dist[ind]) ** NPA
            bcoef[pos] = math.exp(-(sigma[pos] / kappa[pos] + alpha[pos]) * scale)
    alpha[alpha < 0.0] = 0.0
    idx = np.abs(sigma) > 1.0e-6
    acoef[idx] = sigma[idx] * (bcoef[idx] - 1.0) / (kappa[idx] * sigma[idx] + kappa[idx] * alpha[idx])
    return kappa, acoef, bcoef, alpha, sigma


def sigma_alpha_max(seismic: bool, npml: int, deltamin: float, f0: float, vmax: float,
                    alpha_max_scalar=1.0, NP=2.0, Rcoef=0.001, dt=None, mode="driver",
                    velocity_scaling_factor=1.0):
    """Maximum CPML conductivity and alpha of one axis.

    ``vmax`` is the largest wave speed (m/s) in the model.  For ``mode="driver"``
    this is ``definitions.py:646-699`` ("global" smoothing); the EM branch is
    written there in terms of ``clight / sqrt(eps_r)``, which is ``vmax``.
    For ``mode="legacy"`` it is ``legacy/prjrun_101424.py:226-244``.
    """
    if mode == "driver":
        if seismic:
            s = -math.log(Rcoef) * (NP + 1) * velocity_scaling_factor * 0.7 * vmax / (2.0 * npml)
            a = alpha_max_scalar * math.pi * f0
        else:
            # definitions.py:688-693 takes clight / sqrt(max(map, 1)) of a
            # velocity map that, for EM, holds 1 / v_max of each material
            # (classes.py:1110-1112): the clamp turns it into 1, so the
            # driver's EM sigma_max uses the speed of light whatever vmax is
            s = -(NP + 1) * math.log(Rcoef) * EPS0 * CLIGHT / (2.0 * npml * deltamin)
            a = alpha_max_scalar * math.pi * EPS0 * f0
    elif mode == "legacy":
        if seismic:
            quasi_cp_max = 0.7 * deltamin / (2.0 * dt)
            s = -math.log(Rcoef) * (NP + 1) * quasi_cp_max / (2.0 * npml)
            a = math.pi * f0
        else:
            # sig_opt_scalar of the legacy script is 1.2 (legacy/prjrun_101424.py:23)
            s = 1.2 * ((NP + 1) / (deltamin * (MU0 / EPS0) ** 0.5))
            a = alpha_max_scalar * 2 * math.pi * EPS0 * f0
    else:
        raise ValueError(f"unknown CPML mode {mode!r}")
    return s, a


def axis_profile(n: int, npml: int, delta: float, dt: float, sig_max: float, alpha_max: float,
                 kappa_max=5.0, NP=2.0, NPA=2.0, seismic=True, mode="driver") -> AxisProfile:
    """Full- and half-offset profiles of one axis of ``n`` cells (CPML included)."""
    if npml < 1 or 2 * npml > n:
        raise ValueError(f"npml={npml} does not fit an axis of {n} cells")
    K, a, b, al, sg = _profile_1d(n, npml, delta, dt, sig_max, alpha_max, kappa_max, NP, NPA, seismic, False, mode)
    Kh, ah, bh, alh, sgh = _profile_1d(n, npml, delta, dt, sig_max, alpha_max, kappa_max, NP, NPA, seismic, True,
                                       mode)
    return AxisProfile(K, a, b, Kh, ah, bh, al, alh, sg, sgh)


def build_profiles(shape, deltas, npml, dt, f0, vmax, seismic, params=None, mode="driver", axis_vmax=None):
    """Profiles for every axis of a grid.

    ``shape``/``deltas`` are (NX, NZ) or (NX, NY, NZ) full-grid sizes and steps.
    ``vmax`` is the model's largest wave speed; ``axis_vmax`` (one value per
    axis), where given, the largest speed along each axis, which the driver's
    seismic sigma_max of that axis takes (definitions.py:613-661: the
    per-material velocities along x and along z).
    Returns the list of AxisProfile in axis order (x, [y,] z).
    """
    p = dict(DEFAULT_CPML)
    if params:
        p.update(params)
    deltamin = min(deltas)
    speeds = list(axis_vmax) if axis_vmax is not None else [vmax] * len(shape)
    out = []
    for n, d, v in zip(shape, deltas, speeds):
        sig, alp = sigma_alpha_max(seismic, npml, deltamin, f0, v, p["alpha_max_scalar"], p["NP"], p["Rcoef"], dt=dt,
                                   mode=mode)
        out.append(axis_profile(n, npml, d, dt, sig, alp, p["kappa_max"], p["NP"], p["NPA"], seismic, mode))
    return out


def driver_fields_2d(nx, nz, npml, dx, dz, dt, f0, vmax, seismic, params=None, half=False, deltamin=None,
                     vmax_z=None):
    """The 2-D sigma, kappa, alpha, acoef, bcoef fields (each (NZ, NX)) the
    current driver writes to ``{name}{,_half}_cpml.dat`` for 2 / 2.5-D
    models (definitions.py:560-998, "global" mode): the per-axis profiles in
    the strips; in the corners sigma is the sum of the two axes' values while
    kappa and alpha are the z axis' (the z-strip loop of cpml_parameters,
    :977-986, overwrites the corner products of :940-960); a and b follow
    from them cell by cell.  ``vmax``: the largest wave speed along x
    (seismic; ``vmax_z`` along z, default the same); ``deltamin``: the
    smallest grid step (default min(dx, dz))."""
    p = dict(DEFAULT_CPML)
    if params:
        p.update(params)
    dmin = min(dx, dz) if deltamin is None else deltamin
    sig_max, alpha_max = sigma_alpha_max(seismic, npml, dmin, f0, vmax, p["alpha_max_scalar"], p["NP"], p["Rcoef"])
    sig_max_z, _ = sigma_alpha_max(seismic, npml, dmin, f0, vmax if vmax_z is None else vmax_z, p["alpha_max_scalar"],
                                   p["NP"], p["Rcoef"])
    NP, NPA, kmax = p["NP"], p["NPA"], p["kappa_max"]
    dxn = _distance(npml, dx, half, "driver")
    dzn = _distance(npml, dz, half, "driver")
    sigma = np.zeros((nz, nx))
    kappa = np.ones((nz, nx))
    alpha = np.zeros((nz, nx))
    sx, sz = np.zeros(nx), np.zeros(nz)
    kx, kz, ax, az = np.ones(nx), np.ones(nz), np.zeros(nx), np.zeros(nz)
    inx, inz = np.zeros(nx, bool), np.zeros(nz, bool)
    for ind in range(npml):
        for pos in (ind, nx - 1 - ind):
            sx[pos] = sig_max * dxn[ind] ** NP
            kx[pos] = 1.0 + (kmax - 1.0) * dxn[ind] ** NP
            ax[pos] = alpha_max * (1.0 - dxn[ind]) ** NPA
            inx[pos] = True
        for pos in (ind, nz - 1 - ind):
            sz[pos] = sig_max_z * dzn[ind] ** NP
            kz[pos] = 1.0 + (kmax - 1.0) * dzn[ind] ** NP
            az[pos] = alpha_max * (1.0 - dzn[ind]) ** NPA
            inz[pos] = True
    sigma = sx[None, :] * np.ones((nz, 1)) * ~inz[:, None] + sz[:, None] * np.ones((1, nx)) * ~inx[None, :]
    corner = inz[:, None] & inx[None, :]
    sigma[corner] = (sx[None, :] + sz[:, None])[corner]
    kappa = np.where(inx[None, :], kx[None, :], 1.0) * np.ones((nz, 1))
    kappa = np.where(inz[:, None], kz[:, None] * np.ones((1, nx)), kappa)
    alpha = np.where(inx[None, :], ax[None, :], 0.0) * np.ones((nz, 1))
    alpha = np.where(inz[:, None], az[:, None] * np.ones((1, nx)), alpha)
    scale = dt if seismic else dt / EPS0
    bcoef = np.exp(-(sigma / kappa + alpha) * scale)
    alpha = np.maximum(alpha, 0.0)
    acoef = np.zeros((nz, nx))
    idx = np.abs(sigma) > 1.0e-6
    acoef[idx] = sigma[idx] * (bcoef[idx] - 1.0) / (kappa[idx] * sigma[idx] + kappa[idx] * alpha[idx])
    return {"sigma": sigma, "kappa": kappa, "alpha": alpha, "acoef": acoef, "bcoef": bcoef}


def driver_cpml_planes(nx, nz, npml, dx, dz, dt, f0, vmax_x, seismic, params=None, vmax_z=None, deltamin=None):
    """The (6, NZ, NX) planes K, a, b, K_half, a_half, b_half of the driver's
    2-D CPML fields (driver_fields_2d at both offsets), the input of
    FDTDSolver.set_cpml2d."""
    out = []
    for half in (False, True):
        f = driver_fields_2d(nx, nz, npml, dx, dz, dt, f0, vmax_x, seismic, params, half=half, deltamin=deltamin,
                             vmax_z=vmax_z)
        out += [f["kappa"], f["acoef"], f["bcoef"]]
    return np.ascontiguousarray(np.stack(out))


def pack_profiles(profiles) -> np.ndarray:
    """Concatenate K, a, b, K_half, a_half, b_half of every axis (x, [y,] z)."""
    return np.ascontiguousarray(np.concatenate([pr.packed().ravel() for pr in profiles]), dtype=np.float64)


# ---------------------------------------------------------------------------
# Christoffel velocities and the time step (src/seidart/routines/classes.py:469-492,
# classes.py:1070-1121).

_VOIGT = [[0, 5, 4], [5, 1, 3], [4, 3, 2]]


def voigt_full(C6: np.ndarray) -> np.ndarray:
    """6x6 Voigt stiffness -> 3x3x3x3 tensor."""
    C = np.zeros((3, 3, 3, 3))
    for i in range(3):
        for j in range(3):
            for k in range(3):
                for l in range(3):
                    C[i, j, k, l] = C6[_VOIGT[i][j], _VOIGT[k][l]]
    return C


def christoffel_velocities(C6: np.ndarray, rho: float, n: np.ndarray) -> np.ndarray:
    """Phase velocities (3,) along unit direction ``n``."""
    C = voigt_full(C6)
    G = np.einsum("ijkl,j,l->ik", C, n, n) / rho
    w = np.linalg.eigvalsh(G)
    return np.sqrt(np.maximum(w, 0.0))


def axis_velocity(C6: np.ndarray, rho: float, axis: str) -> float:
    """Largest Christoffel velocity along one coordinate axis ('x', 'y', 'z')."""
    n = {"x": (1.0, 0.0, 0.0), "y": (0.0, 1.0, 0.0), "z": (0.0, 0.0, 1.0)}[axis]
    return float(christoffel_velocities(C6, rho, np.array(n)).max())


def max_velocity(C6: np.ndarray, rho: float, dim: float) -> float:
    """Maximum Christoffel velocity over the driver's direction set
    (x, z, xz in 2-D; x, y, z, xy, xz, yz in 2.5-D; classes.py:1079-1083)."""
    s = 1.0 / math.sqrt(2.0)
    dirs = {"x": (1, 0, 0), "y": (0, 1, 0), "z": (0, 0, 1),
            "xy": (s, s, 0), "xz": (s, 0, s), "yz": (0, s, s)}
    keys = ["x", "z", "xz"] if dim == 2 else ["x", "y", "z", "xy", "xz", "yz"]
    return max(float(christoffel_velocities(C6, rho, np.array(dirs[k], float)).max()) for k in keys)


def time_step(cfl: float, vmax: float, deltas) -> float:
    """dt = CFL / (vmax * sqrt(sum 1/delta^2)), classes.py:480-485."""
    return cfl / (vmax * math.sqrt(sum(1.0 / d ** 2 for d in deltas)))
