"""Second, independent FP64 restatement of electromag2 (real and complex
permittivities) and seismic2 in vectorised numpy -- TEST INFRASTRUCTURE ONLY.

Written from the Fortran (legacy/fortran/electromagfdtd.f95:244-325, :519-612,
legacy/fortran/seismicfdtd.f95:243-384) with whole-array slices instead of
loops, so that an indexing slip in one restatement shows up as a mismatch
against the other (fdtd_oracle.cpp).  Arrays are (NZ, NX) = [k, i].
"""
from __future__ import annotations

import numpy as np

EPS0 = 8.85418782e-12
MU0 = 4.0 * np.pi * 1.0e-7


def _axes(prof, NX, NZ):
    p = np.asarray(prof, dtype=np.float64)
    x = p[:6 * NX].reshape(6, NX)
    z = p[6 * NX:6 * NX + 6 * NZ].reshape(6, NZ)
    return x, z  # rows: K, a, b, Kh, ah, bh


def electromag2(NX, NZ, dx, dz, dt, prof, mat, src_ik, srcfn, nsteps, rec=None, cpml2d=None):
    """cpml2d: the driver's 2-D CPML fields (6, NZ, NX), K a b K_half a_half
    b_half, for every derivative direction in place of the axis profiles."""
    eps11, eps13, eps33, sig11, sig13, sig33 = np.asarray(mat, dtype=np.float64)
    return _em2(NX, NZ, dx, dz, dt, prof, eps11, eps13, eps33, sig11, sig13, sig33, src_ik, srcfn, nsteps, rec,
                np.float64, cpml2d)


def electromag2c(NX, NZ, dx, dz, dt, prof, mat, src_ik, srcfn, nsteps, rec=None):
    """electromagfdtd.f95:329-616: electromag2 with complex permittivities.
    mat = eps11 re, im, eps13 re, im, eps33 re, im, sig11, sig13, sig33;
    the fields, memory variables and traces come back complex."""
    m = np.asarray(mat, dtype=np.float64)
    eps11, eps13, eps33 = m[0] + 1j * m[1], m[2] + 1j * m[3], m[4] + 1j * m[5]
    return _em2(NX, NZ, dx, dz, dt, prof, eps11, eps13, eps33, m[6], m[7], m[8], src_ik, srcfn, nsteps, rec,
                np.complex128)


def _coef_fields(X, Z, NX, NZ, cpml2d):
    """Every CPML coefficient as an (NZ, NX) array: the x profile spread over
    the rows and the z profile over the columns, or, with the driver's 2-D
    fields, the same field for both axes.  Returns (x tuple, z tuple), each
    K, a, b, K_half, a_half, b_half."""
    if cpml2d is not None:
        F = tuple(np.asarray(cpml2d, dtype=np.float64))
        return F, F
    xs = tuple(np.broadcast_to(X[q][None, :], (NZ, NX)) for q in range(6))
    zs = tuple(np.broadcast_to(Z[q][:, None], (NZ, NX)) for q in range(6))
    return xs, zs


def _em2(NX, NZ, dx, dz, dt, prof, eps11, eps13, eps33, sig11, sig13, sig33, src_ik, srcfn, nsteps, rec, dtype,
         cpml2d=None):
    X, Z = _axes(prof, NX, NZ)
    epsx, epsz = (eps11 + eps13) * EPS0, (eps13 + eps33) * EPS0
    sigx, sigz = sig11 + sig13, sig13 + sig33
    caEx = (1 - sigx * dt / (2 * epsx)) / (1 + sigx * dt / (2 * epsx))
    cbEx = (dt / epsx) / (1 + sigx * dt / (2 * epsx))
    caEz = (1 - sigz * dt / (2 * epsz)) / (1 + sigz * dt / (2 * epsz))
    cbEz = (dt / epsz) / (1 + sigz * dt / (2 * epsz))
    dbH = dt / MU0
    Ex, Ez, Hy = (np.zeros((NZ, NX), dtype=dtype) for _ in range(3))
    mExz, mEzx, mHyz, mHyx = (np.zeros((NZ, NX), dtype=dtype) for _ in range(4))
    si, sk = src_ik
    out = []
    (Kx, ax, bx, Kxh, axh, bxh), (Kz, az, bz, Kzh, azh, bzh) = _coef_fields(X, Z, NX, NZ, cpml2d)
    H, EX, EZ = np.s_[:-1, :-1], np.s_[1:-1, :-1], np.s_[:-1, 1:-1]
    for t in range(nsteps):
        # H: k in [0,NZ-2], i in [0,NX-2]
        dEx = (Ex[1:, :-1] - Ex[:-1, :-1]) / dz
        mExz[H] = bz[H] * mExz[H] + az[H] * dEx
        vz = dEx / Kz[H] + mExz[H]
        dEz = (Ez[:-1, 1:] - Ez[:-1, :-1]) / dx
        mEzx[H] = bx[H] * mEzx[H] + ax[H] * dEz
        vx = dEz / Kx[H] + mEzx[H]
        Hy[H] = Hy[H] + dbH * (vx + vz)
        # Ex: k in [1,NZ-2], i in [0,NX-2]
        d = (Hy[1:-1, :-1] - Hy[:-2, :-1]) / dz
        mHyz[EX] = bzh[EX] * mHyz[EX] + azh[EX] * d
        d = d / Kzh[EX] + mHyz[EX]
        Ex[EX] = ((caEx[1:-1, :-1] + caEx[:-2, :-1]) / 2) * Ex[EX] + ((cbEx[1:-1, :-1] + cbEx[:-2, :-1]) / 2) * d
        # Ez: k in [0,NZ-2], i in [1,NX-2]
        d = (Hy[:-1, 1:-1] - Hy[:-1, :-2]) / dx
        mHyx[EZ] = bxh[EZ] * mHyx[EZ] + axh[EZ] * d
        d = d / Kxh[EZ] + mHyx[EZ]
        Ez[EZ] = ((caEz[:-1, 1:-1] + caEz[:-1, :-2]) / 2) * Ez[EZ] + ((cbEz[:-1, 1:-1] + cbEz[:-1, :-2]) / 2) * d
        Ex[sk, si] += srcfn[0][t] * dt / eps11[sk, si]
        Ez[sk, si] += srcfn[1][t] * dt / eps33[sk, si]
        Ex[:, 0] = 0; Ex[:, NX - 2] = 0; Ex[0, :] = 0; Ex[NZ - 1, :] = 0
        Ez[:, 0] = 0; Ez[:, NX - 1] = 0; Ez[0, :] = 0; Ez[NZ - 2, :] = 0
        Hy[:, 0] = 0; Hy[:, NX - 2] = 0; Hy[0, :] = 0; Hy[NZ - 2, :] = 0
        if rec is not None:
            out.append(np.stack([Ex[rec[:, 2], rec[:, 0]], Ez[rec[:, 2], rec[:, 0]]]))
    return np.stack([Ex, Ez, Hy]), np.stack([mExz, mEzx, mHyz, mHyx]), (np.stack(out) if out else None)


def _rho_avg(method, w, r, a, b):
    """Density at a staggered point, weights (w, 1, 1) (as rho_avg of fdtd_oracle.cpp)."""
    if method == "none":
        return r
    if method == "geometric":
        return np.sqrt(np.sqrt(r * r * a * b)) if w == 2 else np.cbrt(np.sqrt(r * r * r * r * a * b))
    if method == "harmonic":
        return (w + 2.0) / (w / r + 1.0 / a + 1.0 / b)
    return (w * r + a + b) / (w + 2.0)


def seismic2(NX, NZ, dx, dz, dt, prof, mat, src_ik, srcfn, nsteps, rec=None, legacy=False, density="arithmetic",
             stress_src=None, cpml2d=None):
    """legacy: the legacy quirks (shared velocity-gradient memory of the two
    stress loops, b_x_half(j), vx over the cell's own rho); otherwise
    corrected physics.  stress_src: (3, nstep) sxx, szz, sxz or None."""
    X, Z = _axes(prof, NX, NZ)
    c11, c13, c15, c33, c35, c55, rho, gx, gz = np.asarray(mat, dtype=np.float64)
    vx, vz, sxx, szz, sxz = (np.zeros((NZ, NX)) for _ in range(5))
    m_vxx, m_vzz, m_vxz, m_vzx, m_sxx, m_szz, m_sxzx, m_sxzz = (np.zeros((NZ, NX)) for _ in range(8))
    n_vxx, n_vzz, n_vxz, n_vzx = (np.zeros((NZ, NX)) for _ in range(4))  # the sigmaxz loop's own
    if legacy:
        n_vxx, n_vzz, n_vxz, n_vzx = m_vxx, m_vzz, m_vxz, m_vzx
    si, sk = src_ik
    (Kx, ax, bx, Kxh, axh, bxh), (Kz, az, bz, Kzh, azh, bzh) = _coef_fields(X, Z, NX, NZ, cpml2d)
    if legacy:  # b_x_half read with the z index (seismicfdtd.f95:255); 0 past the x axis
        q3 = np.zeros(NZ)
        n = min(NX, NZ)
        q3[:n] = X[5][:n]
        q3 = np.broadcast_to(q3[:, None], (NZ, NX))
    else:
        q3 = bxh
    out = []
    for t in range(nsteps):
        # loop 1: k in [1, NZ-1], i in [0, NX-2]
        s1 = (slice(1, NZ), slice(0, NX - 1))
        dvx_dx = (vx[1:, 1:] - vx[1:, :-1]) / dx
        dvz_dz = (vz[1:, :-1] - vz[:-1, :-1]) / dz
        dvz_dx = (vz[1:, 1:] - vz[1:, :-1]) / dx
        dvx_dz = (vx[1:, :-1] - vx[:-1, :-1]) / dz
        m_vxx[s1] = q3[s1] * m_vxx[s1] + axh[s1] * dvx_dx
        m_vzz[s1] = bz[s1] * m_vzz[s1] + az[s1] * dvz_dz
        m_vxz[s1] = bzh[s1] * m_vxz[s1] + azh[s1] * dvx_dz
        m_vzx[s1] = bx[s1] * m_vzx[s1] + ax[s1] * dvz_dx
        dvx_dx = dvx_dx / Kxh[s1] + m_vxx[s1]
        dvz_dz = dvz_dz / Kz[s1] + m_vzz[s1]
        dvz_dx = dvz_dx / Kx[s1] + m_vzx[s1]
        dvx_dz = dvx_dz / Kzh[s1] + m_vxz[s1]
        av = lambda c: (c[1:, 1:] + 2 * c[1:, :-1] + c[:-1, :-1]) / 4
        sxx[s1] = sxx[s1] + (av(c11) * dvx_dx + av(c13) * dvz_dz + av(c15) * (dvz_dx + dvx_dz)) * dt
        szz[s1] = szz[s1] + (av(c13) * dvx_dx + av(c33) * dvz_dz + av(c35) * (dvz_dx + dvx_dz)) * dt
        # loop 2: k in [0, NZ-2], i in [1, NX-1]
        s2 = (slice(0, NZ - 1), slice(1, NX))
        dvx_dx = (vx[:-1, 1:] - vx[:-1, :-1]) / dx
        dvz_dz = (vz[1:, 1:] - vz[:-1, 1:]) / dz
        dvz_dx = (vz[:-1, 1:] - vz[:-1, :-1]) / dx
        dvx_dz = (vx[1:, 1:] - vx[:-1, 1:]) / dz
        n_vxx[s2] = bxh[s2] * n_vxx[s2] + axh[s2] * dvx_dx
        n_vzz[s2] = bz[s2] * n_vzz[s2] + az[s2] * dvz_dz
        n_vxz[s2] = bzh[s2] * n_vxz[s2] + azh[s2] * dvx_dz
        n_vzx[s2] = bx[s2] * n_vzx[s2] + ax[s2] * dvz_dx
        dvx_dx = dvx_dx / Kxh[s2] + n_vxx[s2]
        dvz_dz = dvz_dz / Kz[s2] + n_vzz[s2]
        dvz_dx = dvz_dx / Kx[s2] + n_vzx[s2]
        dvx_dz = dvx_dz / Kzh[s2] + n_vxz[s2]
        bv = lambda c: (c[1:, 1:] + 2 * c[:-1, 1:] + c[:-1, :-1]) / 4
        sxz[s2] = sxz[s2] + (bv(c15) * dvx_dx + bv(c35) * dvz_dz + bv(c55) * (dvz_dx + dvx_dz)) * dt
        if stress_src is not None:
            sxx[sk, si] += stress_src[0][t] * dt
            szz[sk, si] += stress_src[1][t] * dt
            sxz[sk, si] += stress_src[2][t] * dt
        # vx: k in [1, NZ-1], i in [1, NX-1]
        s3 = (slice(1, NZ), slice(1, NX))
        d1 = (sxx[1:, 1:] - sxx[1:, :-1]) / dx
        d2 = (sxz[1:, 1:] - sxz[:-1, 1:]) / dz
        m_sxx[s3] = bx[s3] * m_sxx[s3] + ax[s3] * d1
        m_sxzz[s3] = bz[s3] * m_sxzz[s3] + az[s3] * d2
        d1 = d1 / Kx[s3] + m_sxx[s3]
        d2 = d2 / Kz[s3] + m_sxzz[s3]
        rx = rho[s3] if legacy else _rho_avg(density, 2, rho[s3], rho[1:, :-1], rho[:-1, 1:])
        vx[s3] = vx[s3] * (1 - gx[s3]) + (d1 + d2) * dt / rx
        # vz: k in [0, NZ-2], i in [0, NX-2]
        s4 = (slice(0, NZ - 1), slice(0, NX - 1))
        rbar = _rho_avg(density, 2, rho[s4], rho[:-1, 1:], rho[1:, :-1])
        d1 = (sxz[:-1, 1:] - sxz[:-1, :-1]) / dx
        d2 = (szz[1:, :-1] - szz[:-1, :-1]) / dz
        m_sxzx[s4] = bxh[s4] * m_sxzx[s4] + axh[s4] * d1
        m_szz[s4] = bzh[s4] * m_szz[s4] + azh[s4] * d2
        d1 = d1 / Kxh[s4] + m_sxzx[s4]
        d2 = d2 / Kzh[s4] + m_szz[s4]
        vz[s4] = vz[s4] * (1 - gz[s4]) + (d1 + d2) * dt / rbar
        vx[sk, si] += srcfn[0][t] * dt / rho[sk, si]
        vz[sk, si] += srcfn[1][t] * dt / rho[sk, si]
        for f in (vx, vz):
            f[:, 0] = 0; f[:, NX - 1] = 0; f[0, :] = 0; f[NZ - 1, :] = 0
        if rec is not None:
            out.append(np.stack([vx[rec[:, 2], rec[:, 0]], vz[rec[:, 2], rec[:, 0]]]))
    zero = np.zeros((NZ, NX))
    second = [zero] * 4 if legacy else [n_vxx, n_vzz, n_vxz, n_vzx]
    mem = np.stack([m_vxx, m_vzz, m_vxz, m_vzx, m_sxx, m_szz, m_sxzx, m_sxzz] + second)
    return np.stack([vx, vz, sxx, szz, sxz]), mem, (np.stack(out) if out else None)
