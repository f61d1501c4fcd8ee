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
