"""FP64 discrete adjoint of electromag2 in numpy -- TEST INFRASTRUCTURE ONLY.

Forward: the legacy step (legacy/fortran/electromagfdtd.f95:249-321) as in
oracle/numpy_ref.py, keeping every per-step state.  Adjoint: the exact
transpose of that step in reverse order (masks, E half, H half), written the
same way as the CUDA kernels of seidart_gb300/csrc/adjoint_em2.cu, so the GPU
gradient can be compared with an FP64 gradient of the same discrete scheme.
Arrays are [k, i] = (NZ, NX).
"""
from __future__ import annotations

import numpy as np

EPS0 = 8.85418782e-12
MU0 = 4.0 * np.pi * 1.0e-7


def _axes(prof, NX, NZ):
    p = np.asarray(prof, dtype=np.float64)
    return p[:6 * NX].reshape(6, NX), p[6 * NX:6 * NX + 6 * NZ].reshape(6, NZ)


def coefficients(mat, dt):
    e11, e13, e33, s11, s13, s33 = np.asarray(mat, dtype=np.float64)
    ex, ez = (e11 + e13) * EPS0, (e13 + e33) * EPS0
    sx, sz = s11 + s13, s13 + s33
    caEx = (1 - sx * dt / (2 * ex)) / (1 + sx * dt / (2 * ex))
    cbEx = (dt / ex) / (1 + sx * dt / (2 * ex))
    caEz = (1 - sz * dt / (2 * ez)) / (1 + sz * dt / (2 * ez))
    cbEz = (dt / ez) / (1 + sz * dt / (2 * ez))
    return caEx, cbEx, caEz, cbEz


def _masks(NX, NZ):
    mex = np.ones((NZ, NX)); mex[:, 0] = 0; mex[:, NX - 2] = 0; mex[0, :] = 0; mex[NZ - 1, :] = 0
    mez = np.ones((NZ, NX)); mez[:, 0] = 0; mez[:, NX - 1] = 0; mez[0, :] = 0; mez[NZ - 2, :] = 0
    mhy = np.ones((NZ, NX)); mhy[:, 0] = 0; mhy[:, NX - 2] = 0; mhy[0, :] = 0; mhy[NZ - 2, :] = 0
    return mex, mez, mhy


def forward(NX, NZ, dx, dz, dt, prof, mat, src_ik, srcfn, nsteps, rec):
    """Returns (traces [nsteps,2,nrec], states) with states[t] = (Ex,Ez,Hy,A,B,C,D) before step t."""
    X, Z = _axes(prof, NX, NZ)
    caEx, cbEx, caEz, cbEz = coefficients(mat, dt)
    e11, e33 = mat[0], mat[2]
    dbH = dt / MU0
    Ex, Ez, Hy, A, B, C, D = (np.zeros((NZ, NX)) for _ in range(7))
    si, sk = src_ik
    mex, mez, mhy = _masks(NX, NZ)
    ikx, adx, bx = 1 / (dx * X[0]), X[1] / dx, X[2]
    ikxh, adxh, bxh = 1 / (dx * X[3]), X[4] / dx, X[5]
    ikz, adz, bz = (1 / (dz * Z[0]))[:, None], (Z[1] / dz)[:, None], Z[2][:, None]
    ikzh, adzh, bzh = (1 / (dz * Z[3]))[:, None], (Z[4] / dz)[:, None], Z[5][:, None]
    states, traces = [], []
    for t in range(nsteps):
        states.append(tuple(a.copy() for a in (Ex, Ez, Hy, A, B, C, D)))
        H = (slice(0, NZ - 1), slice(0, NX - 1))
        dEx = Ex[1:, :-1] - Ex[:-1, :-1]
        dEz = Ez[:-1, 1:] - Ez[:-1, :-1]
        A[H] = bz[:-1] * A[H] + adz[:-1] * dEx
        B[H] = bx[:-1] * B[H] + adx[:-1] * dEz
        Hy[H] = Hy[H] + dbH * (dEz * ikx[:-1] + B[H] + dEx * ikz[:-1] + A[H])
        E1 = (slice(1, NZ - 1), slice(0, NX - 1))
        dHz = Hy[1:-1, :-1] - Hy[:-2, :-1]
        C[E1] = bzh[1:-1] * C[E1] + adzh[1:-1] * dHz
        CA = 0.5 * (caEx[1:-1, :-1] + caEx[:-2, :-1])
        CB = 0.5 * (cbEx[1:-1, :-1] + cbEx[:-2, :-1])
        Ex[E1] = CA * Ex[E1] + CB * (dHz * ikzh[1:-1] + C[E1])
        E2 = (slice(0, NZ - 1), slice(1, NX - 1))
        dHx = Hy[:-1, 1:-1] - Hy[:-1, :-2]
        D[E2] = bxh[1:-1] * D[E2] + adxh[1:-1] * dHx
        CA = 0.5 * (caEz[:-1, 1:-1] + caEz[:-1, :-2])
        CB = 0.5 * (cbEz[:-1, 1:-1] + cbEz[:-1, :-2])
        Ez[E2] = CA * Ez[E2] + CB * (dHx * ikxh[1:-1] + D[E2])
        Ex[sk, si] += srcfn[0][t] * dt / e11[sk, si]
        Ez[sk, si] += srcfn[1][t] * dt / e33[sk, si]
        Ex *= mex; Ez *= mez; Hy *= mhy
        traces.append(np.stack([Ex[rec[:, 2], rec[:, 0]], Ez[rec[:, 2], rec[:, 0]]]))
    return np.stack(traces), states


def gradient(NX, NZ, dx, dz, dt, prof, mat, src_ik, srcfn, rec, states, resid):
    """dJ/d(eps11 eps13 eps33 sig11 sig13 sig33) for dJ/d(traces) = resid (FP64)."""
    X, Z = _axes(prof, NX, NZ)
    mat = np.asarray(mat, dtype=np.float64)
    caEx, cbEx, caEz, cbEz = coefficients(mat, dt)
    dbH = dt / MU0
    ikx, adx, bx = 1 / (dx * X[0]), X[1] / dx, X[2]
    ikxh, adxh, bxh = 1 / (dx * X[3]), X[4] / dx, X[5]
    ikz, adz, bz = (1 / (dz * Z[0]))[:, None], (Z[1] / dz)[:, None], Z[2][:, None]
    ikzh, adzh, bzh = (1 / (dz * Z[3]))[:, None], (Z[4] / dz)[:, None], Z[5][:, None]
    mex, mez, mhy = _masks(NX, NZ)
    si, sk = src_ik
    LEx, LEz, LHy, LA, LB, LC, LD = (np.zeros((NZ, NX)) for _ in range(7))
    gCAx, gCBx, gCAz, gCBz = (np.zeros((NZ, NX)) for _ in range(4))
    acc = np.zeros(2)
    nsteps = len(states)
    # Ex/Ez/H ranges as index slices
    E1 = (slice(1, NZ - 1), slice(0, NX - 1))
    E2 = (slice(0, NZ - 1), slice(1, NX - 1))
    H = (slice(0, NZ - 1), slice(0, NX - 1))
    CAx = np.zeros((NZ, NX)); CBx = np.zeros((NZ, NX)); CAz = np.zeros((NZ, NX)); CBz = np.zeros((NZ, NX))
    CAx[E1] = 0.5 * (caEx[1:-1, :-1] + caEx[:-2, :-1]); CBx[E1] = 0.5 * (cbEx[1:-1, :-1] + cbEx[:-2, :-1])
    CAz[E2] = 0.5 * (caEz[:-1, 1:-1] + caEz[:-1, :-2]); CBz[E2] = 0.5 * (cbEz[:-1, 1:-1] + cbEz[:-1, :-2])
    inEx = np.zeros((NZ, NX), bool); inEx[E1] = True
    inEz = np.zeros((NZ, NX), bool); inEz[E2] = True
    inH = np.zeros((NZ, NX), bool); inH[H] = True
    for t in range(nsteps - 1, -1, -1):
        Ex, Ez, Hy, A, B, C, D = states[t]
        np.add.at(LEx, (rec[:, 2], rec[:, 0]), resid[t, 0])
        np.add.at(LEz, (rec[:, 2], rec[:, 0]), resid[t, 1])
        lex, lez, lhy = LEx * mex, LEz * mez, LHy * mhy
        # forward recompute of the H half
        Hp = np.zeros((NZ, NX))
        dEx = Ex[1:, :-1] - Ex[:-1, :-1]
        dEz = Ez[:-1, 1:] - Ez[:-1, :-1]
        Ap = bz[:-1] * A[H] + adz[:-1] * dEx
        Bp = bx[:-1] * B[H] + adx[:-1] * dEz
        Hp[H] = Hy[H] * mhy[H] + dbH * (dEz * ikx[:-1] + Bp + dEx * ikz[:-1] + Ap)
        # E half transposed
        gx = np.zeros((NZ, NX)); gz = np.zeros((NZ, NX))
        gx[inEx] = (CBx * lex * (ikzh + adzh) + LC * adzh)[inEx]
        gz[inEz] = (CBz * lez * (ikxh + adxh)[None, :] + LD * adxh[None, :])[inEz]
        TH = lhy.copy()
        TH += gx; TH[:-1, :] -= gx[1:, :]
        TH += gz; TH[:, :-1] -= gz[:, 1:]
        dHz = np.zeros((NZ, NX)); dHz[1:, :] = Hp[1:, :] - Hp[:-1, :]
        dHx = np.zeros((NZ, NX)); dHx[:, 1:] = Hp[:, 1:] - Hp[:, :-1]
        Cp = bzh * C + adzh * dHz
        Dp = bxh[None, :] * D + adxh[None, :] * dHx
        gCAx[inEx] += (lex * Ex)[inEx]
        gCBx[inEx] += (lex * (dHz * ikzh + Cp))[inEx]
        gCAz[inEz] += (lez * Ez)[inEz]
        gCBz[inEz] += (lez * (dHx * ikxh[None, :] + Dp))[inEz]
        acc[0] += lex[sk, si] * srcfn[0][t] * dt / mat[0][sk, si]
        acc[1] += lez[sk, si] * srcfn[1][t] * dt / mat[2][sk, si]
        MEx = np.where(inEx, CAx * lex, lex)
        MEz = np.where(inEz, CAz * lez, lez)
        LCn = np.where(inEx, bzh * (CBx * lex + LC), LC)
        LDn = np.where(inEz, bxh[None, :] * (CBz * lez + LD), LD)
        # H half transposed
        hA = np.zeros((NZ, NX)); hB = np.zeros((NZ, NX))
        hA[inH] = (dbH * TH * (ikz + adz) + LA * adz)[inH]
        hB[inH] = (dbH * TH * (ikx + adx)[None, :] + LB * adx[None, :])[inH]
        LEx = MEx - hA; LEx[1:, :] += hA[:-1, :]
        LEz = MEz - hB; LEz[:, 1:] += hB[:, :-1]
        LHy = np.where(inH & (mhy == 0), 0.0, TH)
        LA = np.where(inH, bz * (dbH * TH + LA), LA)
        LB = np.where(inH, bx[None, :] * (dbH * TH + LB), LB)
        LC, LD = LCn, LDn
    # chain rule to the model planes
    e11, e13, e33, s11, s13, s33 = mat
    dcaX = 0.5 * gCAx; dcaX[:-1, :] += 0.5 * gCAx[1:, :]
    dcbX = 0.5 * gCBx; dcbX[:-1, :] += 0.5 * gCBx[1:, :]
    dcaZ = 0.5 * gCAz; dcaZ[:, :-1] += 0.5 * gCAz[:, 1:]
    dcbZ = 0.5 * gCBz; dcbZ[:, :-1] += 0.5 * gCBz[:, 1:]

    def chain(er, sg, dca, dcb):
        ep = er * EPS0
        u = sg * dt / (2 * ep)
        w = 1 / (1 + u) ** 2
        de = (dca * 2 * u / ep * w + dcb * (-dt / ep ** 2) * w) * EPS0
        ds = dca * (-dt / ep) * w + dcb * (-dt * dt / (2 * ep * ep)) * w
        return de, ds

    deX, dsX = chain(e11 + e13, s11 + s13, dcaX, dcbX)
    deZ, dsZ = chain(e13 + e33, s13 + s33, dcaZ, dcbZ)
    g = np.stack([deX, deX + deZ, deZ, dsX, dsX + dsZ, dsZ])
    g[0][sk, si] += -acc[0] / e11[sk, si]
    g[2][sk, si] += -acc[1] / e33[sk, si]
    return g


# ---------------------------------------------------------------------------
# seismic2 (legacy/fortran/seismicfdtd.f95:243-384), the default corrected
# physics: the sigmaxz loop's own velocity-gradient memory, b_x_half(i), vx over
# the averaged density.  Arrays (NZ, NX); memory variables on the full grid
# (zero wherever a = 0).  Written the way the CUDA adjoint
# (seidart_gb300/csrc/adjoint_s2.cu) is, from the update coefficients:
#   A11 A13 A15 A33 A35 (loop 1: k >= 1, i <= NX-2), B15 B35 B55 (loop 2:
#   k <= NZ-2, i >= 1), all x dt; dtrx = dt / rho_x, dtrz = dt / rho_z;
#   gxp = 1 - gamma_x, gzp = 1 - gamma_z.

def _rho_avg_parts(method, r, a, b):
    """rho_avg (weights 2, 1, 1) and its partial derivatives in r, a, b."""
    if method == "none":
        return r, np.ones_like(r), np.zeros_like(r), np.zeros_like(r)
    if method == "geometric":
        m = np.sqrt(np.sqrt(r * r * a * b))
        return m, m / (2 * r), m / (4 * a), m / (4 * b)
    if method == "harmonic":
        m = 4.0 / (2.0 / r + 1.0 / a + 1.0 / b)
        return m, m * m / 4 * 2 / (r * r), m * m / 4 / (a * a), m * m / 4 / (b * b)
    return (2 * r + a + b) / 4, np.full_like(r, 0.5), np.full_like(r, 0.25), np.full_like(r, 0.25)


def seismic2_coefficients(mat, dt, density="arithmetic"):
    """The seismic2 update coefficient planes (as sfd_set_model forms them, FP64)."""
    c11, c13, c15, c33, c35, c55, rho, gx, gz = np.asarray(mat, dtype=np.float64)
    NZ, NX = rho.shape
    L1, L2 = np.s_[1:, :-1], np.s_[:-1, 1:]

    def avgA(c):
        out = np.zeros((NZ, NX))
        out[L1] = (c[1:, 1:] + 2 * c[1:, :-1] + c[:-1, :-1]) / 4 * dt
        return out

    def avgB(c):
        out = np.zeros((NZ, NX))
        out[L2] = (c[1:, 1:] + 2 * c[:-1, 1:] + c[:-1, :-1]) / 4 * dt
        return out

    co = {"A11": avgA(c11), "A13": avgA(c13), "A15": avgA(c15), "A33": avgA(c33), "A35": avgA(c35),
          "B15": avgB(c15), "B35": avgB(c35), "B55": avgB(c55), "gxp": 1 - gx, "gzp": 1 - gz}
    dtrx = dt / rho.copy()
    rx, _, _, _ = _rho_avg_parts(density, rho[1:, 1:], rho[1:, :-1], rho[:-1, 1:])
    dtrx[1:, 1:] = dt / rx
    dtrz = np.zeros((NZ, NX))
    rz, _, _, _ = _rho_avg_parts(density, rho[:-1, :-1], rho[:-1, 1:], rho[1:, :-1])
    dtrz[:-1, :-1] = dt / rz
    co["dtrx"], co["dtrz"] = dtrx, dtrz
    return co


def _s2_axes(prof, NX, NZ, dx, dz):
    X, Z = _axes(prof, NX, NZ)
    x = dict(ik=1 / (dx * X[0]), ad=X[1] / dx, b=X[2], ikh=1 / (dx * X[3]), adh=X[4] / dx, bh=X[5])
    z = dict(ik=(1 / (dz * Z[0]))[:, None], ad=(Z[1] / dz)[:, None], b=Z[2][:, None],
             ikh=(1 / (dz * Z[3]))[:, None], adh=(Z[4] / dz)[:, None], bh=Z[5][:, None])
    return ({k: np.broadcast_to(v[None, :], (NZ, NX)) for k, v in x.items()},
            {k: np.broadcast_to(v, (NZ, NX)) for k, v in z.items()})


def _s2_ranges(NX, NZ):
    r = {}
    for name, sl in (("L1", np.s_[1:, :-1]), ("L2", np.s_[:-1, 1:]), ("VX", np.s_[1:, 1:]),
                     ("VZ", np.s_[:-1, :-1]), ("INT", np.s_[1:-1, 1:-1])):
        m = np.zeros((NZ, NX), bool)
        m[sl] = True
        r[name] = m
    return r


def _shift(a, dk, di):
    """b[k, i] = a[k + dk, i + di], zero outside the grid."""
    NZ, NX = a.shape
    b = np.zeros_like(a)
    k0, k1 = max(0, -dk), min(NZ, NZ - dk)
    i0, i1 = max(0, -di), min(NX, NX - di)
    b[k0:k1, i0:i1] = a[k0 + dk:k1 + dk, i0 + di:i1 + di]
    return b


def seismic2_forward(NX, NZ, dx, dz, dt, prof, mat, src_ik, srcfn, nsteps, rec, density="arithmetic",
                     stress_src=None):
    """Returns (traces [nsteps, 2, nrec], states, coefficients) with states[t]
    = (vx, vz, sxx, szz, sxz, P1..P4, Q1..Q4, R1..R4) before step t and
    states[nsteps] the final state."""
    co = seismic2_coefficients(mat, dt, density)
    X, Z = _s2_axes(prof, NX, NZ, dx, dz)
    rg = _s2_ranges(NX, NZ)
    rho = np.asarray(mat, dtype=np.float64)[6]
    si, sk = src_ik
    S = [np.zeros((NZ, NX)) for _ in range(17)]
    states, traces = [], []
    for t in range(nsteps):
        states.append([a.copy() for a in S])
        S = _s2_step(S, co, X, Z, rg, t, si, sk, srcfn, stress_src, dt, rho)
        traces.append(np.stack([S[0][rec[:, 2], rec[:, 0]], S[1][rec[:, 2], rec[:, 0]]]))
    states.append([a.copy() for a in S])
    return np.stack(traces), states, co


def _s2_step(S, co, X, Z, rg, t, si, sk, srcfn, stress_src, dt, rho, parts=False):
    vx, vz, sxx, szz, sxz = S[:5]
    P, Q, R = list(S[5:9]), list(S[9:13]), list(S[13:17])
    L1, L2, VX, VZ, INT = rg["L1"], rg["L2"], rg["VX"], rg["VZ"], rg["INT"]
    a = [_shift(vx, 0, 1) - vx, vz - _shift(vz, -1, 0), _shift(vz, 0, 1) - vz, vx - _shift(vx, -1, 0)]
    pk = [("bh", "adh", "ikh", X), ("b", "ad", "ik", Z), ("b", "ad", "ik", X), ("bh", "adh", "ikh", Z)]
    Pn, e = [], []
    for q in range(4):
        bn, an, kn, ax = pk[q]
        p = np.where(L1, ax[bn] * P[q] + ax[an] * a[q], P[q])
        Pn.append(p)
        e.append(np.where(L1, a[q] * ax[kn] + p, 0.0))
    b = [vx - _shift(vx, 0, -1), _shift(vz, 1, 0) - vz, vz - _shift(vz, 0, -1), _shift(vx, 1, 0) - vx]
    Qn, f = [], []
    for q in range(4):
        bn, an, kn, ax = pk[q]
        p = np.where(L2, ax[bn] * Q[q] + ax[an] * b[q], Q[q])
        Qn.append(p)
        f.append(np.where(L2, b[q] * ax[kn] + p, 0.0))
    sxx1 = sxx + co["A11"] * e[0] + co["A13"] * e[1] + co["A15"] * (e[2] + e[3])
    szz1 = szz + co["A13"] * e[0] + co["A33"] * e[1] + co["A35"] * (e[2] + e[3])
    sxz1 = sxz + co["B15"] * f[0] + co["B35"] * f[1] + co["B55"] * (f[2] + f[3])
    if stress_src is not None:
        sxx1[sk, si] += stress_src[0][t] * dt
        szz1[sk, si] += stress_src[1][t] * dt
        sxz1[sk, si] += stress_src[2][t] * dt
    c = [sxx1 - _shift(sxx1, 0, -1), sxz1 - _shift(sxz1, -1, 0)]
    d = [_shift(sxz1, 0, 1) - sxz1, _shift(szz1, 1, 0) - szz1]
    R1 = np.where(VX, X["b"] * R[0] + X["ad"] * c[0], R[0])
    R2 = np.where(VX, Z["b"] * R[1] + Z["ad"] * c[1], R[1])
    R3 = np.where(VZ, X["bh"] * R[2] + X["adh"] * d[0], R[2])
    R4 = np.where(VZ, Z["bh"] * R[3] + Z["adh"] * d[1], R[3])
    g = np.where(VX, c[0] * X["ik"] + R1 + c[1] * Z["ik"] + R2, 0.0)
    h = np.where(VZ, d[0] * X["ikh"] + R3 + d[1] * Z["ikh"] + R4, 0.0)
    vx1 = np.where(INT, co["gxp"] * vx + co["dtrx"] * g, 0.0)
    vz1 = np.where(INT, co["gzp"] * vz + co["dtrz"] * h, 0.0)
    vx1[sk, si] += srcfn[0][t] * dt / rho[sk, si]
    vz1[sk, si] += srcfn[1][t] * dt / rho[sk, si]
    out = [vx1, vz1, sxx1, szz1, sxz1] + Pn + Qn + [R1, R2, R3, R4]
    if parts:
        return out, dict(a=a, b=b, e=e, f=f, c=c, d=d, g=g, h=h)
    return out


def seismic2_gradient(NX, NZ, dx, dz, dt, prof, mat, src_ik, srcfn, rec, states, resid, density="arithmetic",
                      stress_src=None):
    """dJ/d(c11 c13 c15 c33 c35 c55 rho gamma_x gamma_z) for dJ/d(traces) = resid, FP64."""
    mat = np.asarray(mat, dtype=np.float64)
    co = seismic2_coefficients(mat, dt, density)
    X, Z = _s2_axes(prof, NX, NZ, dx, dz)
    rg = _s2_ranges(NX, NZ)
    L1, L2, VX, VZ, INT = rg["L1"], rg["L2"], rg["VX"], rg["VZ"], rg["INT"]
    rho = mat[6]
    si, sk = src_ik
    Lam = [np.zeros((NZ, NX)) for _ in range(17)]
    G = {k: np.zeros((NZ, NX)) for k in ("A11", "A13", "A15", "A33", "A35", "B15", "B35", "B55", "dtrx", "dtrz",
                                         "gxp", "gzp")}
    g_src = 0.0
    pk = [("bh", "adh", "ikh", X), ("b", "ad", "ik", Z), ("b", "ad", "ik", X), ("bh", "adh", "ikh", Z)]
    for t in range(len(states) - 2, -1, -1):
        S = states[t]
        _, F = _s2_step(S, co, X, Z, rg, t, si, sk, srcfn, stress_src, dt, rho, parts=True)
        Lvx, Lvz, Lsxx, Lszz, Lsxz = [a.copy() for a in Lam[:5]]
        LP, LQ, LR = [a.copy() for a in Lam[5:9]], [a.copy() for a in Lam[9:13]], [a.copy() for a in Lam[13:17]]
        np.add.at(Lvx, (rec[:, 2], rec[:, 0]), resid[t, 0])
        np.add.at(Lvz, (rec[:, 2], rec[:, 0]), resid[t, 1])
        lvx, lvz = np.where(INT, Lvx, 0.0), np.where(INT, Lvz, 0.0)
        g_src += -(lvx[sk, si] * srcfn[0][t] + lvz[sk, si] * srcfn[1][t]) * dt / rho[sk, si] ** 2
        G["dtrx"] += lvx * F["g"]
        G["dtrz"] += lvz * F["h"]
        G["gxp"] += lvx * S[0]
        G["gzp"] += lvz * S[1]
        nvx = co["gxp"] * lvx
        nvz = co["gzp"] * lvz
        # vz loop transposed (VZ)
        lh = co["dtrz"] * lvz
        t3 = LR[2] + lh
        ld1 = np.where(VZ, X["ikh"] * lh + X["adh"] * t3, 0.0)
        LR[2] = np.where(VZ, X["bh"] * t3, LR[2])
        t4 = LR[3] + lh
        ld2 = np.where(VZ, Z["ikh"] * lh + Z["adh"] * t4, 0.0)
        LR[3] = np.where(VZ, Z["bh"] * t4, LR[3])
        Lsxz += _shift(ld1, 0, -1) - ld1
        Lszz += _shift(ld2, -1, 0) - ld2
        # vx loop transposed (VX)
        lg = co["dtrx"] * lvx
        t1 = LR[0] + lg
        lc1 = np.where(VX, X["ik"] * lg + X["ad"] * t1, 0.0)
        LR[0] = np.where(VX, X["b"] * t1, LR[0])
        t2 = LR[1] + lg
        lc2 = np.where(VX, Z["ik"] * lg + Z["ad"] * t2, 0.0)
        LR[1] = np.where(VX, Z["b"] * t2, LR[1])
        Lsxx += lc1 - _shift(lc1, 0, 1)
        Lsxz += lc2 - _shift(lc2, 1, 0)
        # loop 2 transposed (L2)
        lf = np.where(L2, Lsxz, 0.0)
        G["B15"] += lf * F["f"][0]
        G["B35"] += lf * F["f"][1]
        G["B55"] += lf * (F["f"][2] + F["f"][3])
        lfq = [co["B15"] * lf, co["B35"] * lf, co["B55"] * lf, co["B55"] * lf]
        lb = []
        for q in range(4):
            bn, an, kn, ax = pk[q]
            tq = LQ[q] + lfq[q]
            lb.append(np.where(L2, ax[kn] * lfq[q] + ax[an] * tq, 0.0))
            LQ[q] = np.where(L2, ax[bn] * tq, LQ[q])
        nvx += lb[0] - _shift(lb[0], 0, 1)        # b1 = vx(i) - vx(i-1)
        nvz += _shift(lb[1], -1, 0) - lb[1]       # b2 = vz(k+1) - vz(k)
        nvz += lb[2] - _shift(lb[2], 0, 1)        # b3 = vz(i) - vz(i-1)
        nvx += _shift(lb[3], -1, 0) - lb[3]       # b4 = vx(k+1) - vx(k)
        # loop 1 transposed (L1)
        ls, lz = np.where(L1, Lsxx, 0.0), np.where(L1, Lszz, 0.0)
        e = F["e"]
        G["A11"] += ls * e[0]
        G["A13"] += ls * e[1] + lz * e[0]
        G["A15"] += ls * (e[2] + e[3])
        G["A33"] += lz * e[1]
        G["A35"] += lz * (e[2] + e[3])
        le = [co["A11"] * ls + co["A13"] * lz, co["A13"] * ls + co["A33"] * lz]
        le += [co["A15"] * ls + co["A35"] * lz] * 2
        la = []
        for q in range(4):
            bn, an, kn, ax = pk[q]
            tq = LP[q] + le[q]
            la.append(np.where(L1, ax[kn] * le[q] + ax[an] * tq, 0.0))
            LP[q] = np.where(L1, ax[bn] * tq, LP[q])
        nvx += _shift(la[0], 0, -1) - la[0]       # a1 = vx(i+1) - vx(i)
        nvz += la[1] - _shift(la[1], 1, 0)        # a2 = vz(k) - vz(k-1)
        nvz += _shift(la[2], 0, -1) - la[2]       # a3 = vz(i+1) - vz(i)
        nvx += la[3] - _shift(la[3], 1, 0)        # a4 = vx(k) - vx(k-1)
        Lam = [nvx, nvz, Lsxx, Lszz, Lsxz] + LP + LQ + LR
    return seismic2_chain(G, mat, dt, density, src_ik, g_src)


def seismic2_chain(G, mat, dt, density, src_ik, g_src):
    """dJ/d(model planes) from dJ/d(update coefficients): the stiffness
    averages' stencils, the densities' averages, 1 - gamma, the source."""
    c11, c13, c15, c33, c35, c55, rho, gx, gz = mat
    NZ, NX = rho.shape
    w = dt / 4

    def fromA(gA):  # A(k, i) = (c(k, i+1) + 2 c(k, i) + c(k-1, i)) / 4 dt on L1
        return w * (2 * gA + _shift(gA, 0, -1) + _shift(gA, 1, 0))

    def fromB(gB):  # B(k, i) = (c(k+1, i) + 2 c(k, i) + c(k, i-1)) / 4 dt on L2
        return w * (2 * gB + _shift(gB, -1, 0) + _shift(gB, 0, 1))

    out = np.zeros((9, NZ, NX))
    out[0] = fromA(G["A11"])
    out[1] = fromA(G["A13"])
    out[2] = fromA(G["A15"]) + fromB(G["B15"])
    out[3] = fromA(G["A33"])
    out[4] = fromA(G["A35"]) + fromB(G["B35"])
    out[5] = fromB(G["B55"])
    g = np.zeros((NZ, NX))
    # dtrx = dt / rho_x, rho_x = avg(rho(k,i), rho(k,i-1), rho(k-1,i)) on (k >= 1, i >= 1); dt / rho elsewhere
    gd = G["dtrx"]
    m, dr, da, db = _rho_avg_parts(density, rho[1:, 1:], rho[1:, :-1], rho[:-1, 1:])
    u = gd[1:, 1:] * (-dt / m ** 2)
    g[1:, 1:] += u * dr
    g[1:, :-1] += u * da
    g[:-1, 1:] += u * db
    edge = np.ones((NZ, NX), bool)
    edge[1:, 1:] = False
    g[edge] += gd[edge] * (-dt / rho[edge] ** 2)
    gd = G["dtrz"]
    m, dr, da, db = _rho_avg_parts(density, rho[:-1, :-1], rho[:-1, 1:], rho[1:, :-1])
    u = gd[:-1, :-1] * (-dt / m ** 2)
    g[:-1, :-1] += u * dr
    g[:-1, 1:] += u * da
    g[1:, :-1] += u * db
    si, sk = src_ik
    g[sk, si] += g_src
    out[6] = g
    out[7] = -G["gxp"]
    out[8] = -G["gzp"]
    return out
