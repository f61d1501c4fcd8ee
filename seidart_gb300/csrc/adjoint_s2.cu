// Discrete adjoint of the seismic2 time step (legacy/fortran/seismicfdtd.f95:
// 247-379, the default corrected physics), for gradients of a receiver-trace
// misfit with respect to the stiffness, density and attenuation planes.
//
// One forward step maps the state (vx, vz, sxx, szz, sxz and the twelve CPML
// memory variables) to the next by
//   loop 1 (k >= 1, i <= NX-2):  a1..a4 = the four velocity differences,
//       P' = b P + ad a (per difference, on its strip), e = a ik + P',
//       sxx' = sxx + A11 e1 + A13 e2 + A15 (e3 + e4), szz' likewise;
//   loop 2 (k <= NZ-2, i >= 1):  b1..b4, Q' = b Q + ad b, f = b ik + Q',
//       sxz' = sxz + B15 f1 + B35 f2 + B55 (f3 + f4);
//   the stress source;
//   vx loop (k >= 1, i >= 1):    c1, c2 = differences of sxx', sxz',
//       R' = b R + ad c, g = c1 ikx + R1' + c2 ikz + R2',
//       vx' = gxp vx + dtrx g on the interior, 0 on the outer planes;
//   vz loop (k <= NZ-2, i <= NX-2): d1, d2 of sxz', szz', h likewise,
//       vz' = gzp vz + dtrz h;
//   the force source; receivers sample vx', vz'.
// with the update coefficients of sfd_set_model (A, B: stiffness averages x
// dt; dtrx, dtrz: dt over the densities; gxp, gzp: 1 - gamma).  The adjoint
// step is its exact transpose in reverse order, written as gathers (each
// thread writes only its own cells) in three phases:
//   v: the velocity half transposed at each cell (after the step's residual
//            is added at the receiver cells): the adjoint of the
//            stress memory variables, the differences' adjoints lc1, lc2,
//            ld1, ld2 (scratch planes), the velocity parts gxp lvx, gzp lvz
//            and the gradients of dtrx, dtrz, gxp, gzp and the source;
//   s: the stresses' adjoints (gathering lc, ld), the stress half
//            transposed at each cell: the adjoint of the velocity-gradient
//            memory variables, la1..la4 and lb1..lb4 (scratch planes) and the
//            gradients of the A and B coefficients;
//   g: the velocities' adjoints, gathering la, lb.
// The g phase of one step and the v phase of the step before it read and
// write only their own cell's adjoint values (their neighbours' come from
// the s phase's scratch planes and the forward states), so one kernel runs
// both at each cell: a segment of n steps is one v kernel, then n s kernels
// and n - 1 fused g + v kernels in turn, then one g kernel.  The residual
// is added by the v phase at the cell's receivers (a per-cell list).
// The FP64 numpy restatement (oracle/numpy_adjoint.py, seismic2_gradient)
// follows the same steps.  The forward states of a checkpoint segment are
// recomputed by the handle's own runs, one step at a time.
#include "adjoint_s2.h"

namespace sfd {

namespace {

constexpr int BX = 32, BY = 8;

__device__ __forceinline__ int mx_idx(int i, int k, int NX, int W) { return k * (2 * W) + strip_idx(i, NX, W); }
__device__ __forceinline__ int mz_idx(int i, int k, int NZ, int P, int W) { return strip_idx(k, NZ, W) * P + i; }

// Memory variables (sfd_num_memory order): 0 dvx_dx (x-strip) 1 dvz_dz (z) 2 dvx_dz (z) 3 dvz_dx (x)
// 4 dsxx_dx (x) 5 dszz_dz (z) 6 dsxz_dx (x) 7 dsxz_dz (z) 8 dvx_dx (x) 9 dvz_dz (z) 10 dvx_dz (z)
// 11 dvz_dx (x), the last four of the sigmaxz loop.
enum { P1 = 0, P2 = 1, P4 = 2, P3 = 3, R1 = 4, R4 = 5, R3 = 6, R2 = 7, Q1 = 8, Q2 = 9, Q4 = 10, Q3 = 11 };

// The v phase of step t at (i, k): S the forward state before the step, S1
// after it, Ln the adjoint of S1 (without the step's residual), Lc that of S.
__device__ __forceinline__ void v_cell(const S2Adj& a, const S2State& S, const S2State& S1, const S2State& Ln,
                                       const S2State& Lc, int t, int i, int k) {
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  const size_t c = (size_t)k * P + i;
  const bool xs = in_strip(i, NX, W), zs = in_strip(k, NZ, W);
  const int mx = xs ? mx_idx(i, k, NX, W) : 0, mz = zs ? mz_idx(i, k, NZ, P, W) : 0;
  const bool inner = i >= 1 && i <= NX - 2 && k >= 1 && k <= NZ - 2;
  const bool vxr = k >= 1 && i >= 1, vzr = k <= NZ - 2 && i <= NX - 2;
  const bool src = i == a.si && k == a.sk;
  // ---- loads (every one before the first store, as in s2adj_s)
  float lvx = inner ? Ln.vx[c] : 0.f, lvz = inner ? Ln.vz[c] : 0.f;
  if (inner)  // this step's residual at the cell's receivers (the traces sample vx', vz')
    for (int r = a.recmap[c]; r >= 0; r = a.recnext[r]) {
      lvx += a.resid[((size_t)t * 2 + 0) * a.nrec + r];
      lvz += a.resid[((size_t)t * 2 + 1) * a.nrec + r];
    }
  const float ikx = a.X.ik[i], ikz = a.Z.ik[k], ikxh = a.X.ikh[i], ikzh = a.Z.ikh[k];
  const float lnR1 = xs ? Ln.m[R1][mx] : 0.f, lnR2 = zs ? Ln.m[R2][mz] : 0.f;
  const float lnR3 = xs ? Ln.m[R3][mx] : 0.f, lnR4 = zs ? Ln.m[R4][mz] : 0.f;
  float dtrx = 0.f, sxx_c = 0.f, sxx_l = 0.f, sxz_c = 0.f, sxz_u = 0.f, adx = 0.f, bx = 0.f, adz = 0.f, bz = 0.f,
        s1R1 = 0.f, s1R2 = 0.f, gdtrx = 0.f;
  if (vxr) {
    dtrx = a.dtrx[c];
    sxx_c = S1.sxx[c]; sxx_l = S1.sxx[c - 1]; sxz_c = S1.sxz[c]; sxz_u = S1.sxz[c - P];
    if (xs) { adx = a.X.ad[i]; bx = a.X.b[i]; s1R1 = S1.m[R1][mx]; }
    if (zs) { adz = a.Z.ad[k]; bz = a.Z.b[k]; s1R2 = S1.m[R2][mz]; }
    if (inner) gdtrx = a.gdtrx[c];
  }
  float dtrz = 0.f, sxz_c2 = 0.f, sxz_r = 0.f, szz_c = 0.f, szz_d = 0.f, adxh = 0.f, bxh = 0.f, adzh = 0.f,
        bzh = 0.f, s1R3 = 0.f, s1R4 = 0.f, gdtrz = 0.f;
  if (vzr) {
    dtrz = a.dtrz[c];
    sxz_c2 = S1.sxz[c]; sxz_r = S1.sxz[c + 1]; szz_c = S1.szz[c]; szz_d = S1.szz[c + P];
    if (xs) { adxh = a.X.adh[i]; bxh = a.X.bh[i]; s1R3 = S1.m[R3][mx]; }
    if (zs) { adzh = a.Z.adh[k]; bzh = a.Z.bh[k]; s1R4 = S1.m[R4][mz]; }
    if (inner) gdtrz = a.gdtrz[c];
  }
  float ggxp = 0.f, ggzp = 0.f, vx0 = 0.f, vz0 = 0.f;
  if (inner) { ggxp = a.ggxp[c]; ggzp = a.ggzp[c]; vx0 = S.vx[c]; vz0 = S.vz[c]; }
  const float gxp = a.gxp[c], gzp = a.gzp[c];
  float fx = 0.f, fz = 0.f, acc = 0.f;
  if (src) { fx = a.srcfn[t]; fz = a.srcfn[a.nstep + t]; acc = *a.srcacc; }
  // ---- arithmetic
  float lc1 = 0.f, lc2 = 0.f, ld1 = 0.f, ld2 = 0.f;
  float oR1 = lnR1, oR2 = lnR2, oR3 = lnR3, oR4 = lnR4;  // the memory variables' adjoints (strip cells)
  if (vxr) {  // vx loop transposed
    const float lg = dtrx * lvx;
    const float c1 = sxx_c - sxx_l, c2 = sxz_c - sxz_u;
    float g = c1 * ikx + c2 * ikz;
    lc1 = ikx * lg;
    lc2 = ikz * lg;
    if (xs) {
      const float tt = lnR1 + lg;
      lc1 += adx * tt;
      oR1 = bx * tt;
      g += s1R1;
    }
    if (zs) {
      const float tt = lnR2 + lg;
      lc2 += adz * tt;
      oR2 = bz * tt;
      g += s1R2;
    }
    if (inner) gdtrx += lvx * g;
  }
  if (vzr) {  // vz loop transposed
    const float lh = dtrz * lvz;
    const float d1 = sxz_r - sxz_c2, d2 = szz_d - szz_c;
    float h = d1 * ikxh + d2 * ikzh;
    ld1 = ikxh * lh;
    ld2 = ikzh * lh;
    if (xs) {
      const float tt = lnR3 + lh;
      ld1 += adxh * tt;
      oR3 = bxh * tt;
      h += s1R3;
    }
    if (zs) {
      const float tt = lnR4 + lh;
      ld2 += adzh * tt;
      oR4 = bzh * tt;
      h += s1R4;
    }
    if (inner) gdtrz += lvz * h;
  }
  if (inner) {
    ggxp += lvx * vx0;
    ggzp += lvz * vz0;
  }
  // ---- stores
  if (xs) { Lc.m[R1][mx] = oR1; Lc.m[R3][mx] = oR3; }
  if (zs) { Lc.m[R2][mz] = oR2; Lc.m[R4][mz] = oR4; }
  if (vxr && inner) a.gdtrx[c] = gdtrx;
  if (vzr && inner) a.gdtrz[c] = gdtrz;
  if (inner) {
    a.ggxp[c] = ggxp;
    a.ggzp[c] = ggzp;
  }
  if (src) *a.srcacc = acc + (lvx * fx + lvz * fz);
  Lc.vx[c] = gxp * lvx;  // the velocities' own parts; the g phase adds the stencil terms
  Lc.vz[c] = gzp * lvz;
  a.tmp[0][c] = lc1;
  a.tmp[1][c] = lc2;
  a.tmp[2][c] = ld1;
  a.tmp[3][c] = ld2;
}

// Every load of a cell first, then the arithmetic, then the stores: the
// arrays are distinct, but the compiler cannot know that and would keep
// each load behind the stores before it.
__global__ void __launch_bounds__(BX * BY) s2adj_s(S2Adj a, S2State S, S2State S1, S2State Ln, S2State Lc) {
  const int i = blockIdx.x * BX + threadIdx.x, k = blockIdx.y * BY + threadIdx.y;
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  if (i >= NX || k >= NZ) return;
  const size_t c = (size_t)k * P + i;
  const float* lc1 = a.tmp[0];
  const float* lc2 = a.tmp[1];
  const float* ld1 = a.tmp[2];
  const float* ld2 = a.tmp[3];
  const bool l2 = k <= NZ - 2 && i >= 1, l1 = k >= 1 && i <= NX - 2;
  const bool xs = in_strip(i, NX, W), zs = in_strip(k, NZ, W);
  const int mx = xs ? mx_idx(i, k, NX, W) : 0, mz = zs ? mz_idx(i, k, NZ, P, W) : 0;
  // (memory variable, strip is x, ik, ad, b) of the four differences of a loop
  const int pm[4] = {P1, P2, P3, P4}, qm[4] = {Q1, Q2, Q3, Q4};
  const bool isx[4] = {true, false, true, false};
  // ---- loads
  const float lnsxx = Ln.sxx[c], lnszz = Ln.szz[c], lnsxz = Ln.sxz[c];
  const float lc1c = lc1[c], lc1r = i + 1 < NX ? lc1[c + 1] : 0.f;
  const float ld2c = ld2[c], ld2u = k >= 1 ? ld2[c - P] : 0.f;
  const float ld1c = ld1[c], ld1l = i >= 1 ? ld1[c - 1] : 0.f;
  const float lc2c = lc2[c], lc2d = k + 1 < NZ ? lc2[c + P] : 0.f;
  const float ik[4] = {a.X.ikh[i], a.Z.ik[k], a.X.ik[i], a.Z.ikh[k]};
  const float ad[4] = {a.X.adh[i], a.Z.ad[k], a.X.ad[i], a.Z.adh[k]};
  const float bb[4] = {a.X.bh[i], a.Z.b[k], a.X.b[i], a.Z.bh[k]};
  const float vxc = S.vx[c], vzc = S.vz[c];
  float vxl = 0.f, vzd = 0.f, vzl = 0.f, vxd = 0.f, B15 = 0.f, B35 = 0.f, B55 = 0.f, gB15 = 0.f, gB35 = 0.f,
        gB55 = 0.f;
  if (l2) {
    vxl = S.vx[c - 1]; vzd = S.vz[c + P]; vzl = S.vz[c - 1]; vxd = S.vx[c + P];
    B15 = a.B15[c]; B35 = a.B35[c]; B55 = a.B55[c];
    gB15 = a.gB15[c]; gB35 = a.gB35[c]; gB55 = a.gB55[c];
  }
  float vxr = 0.f, vzu = 0.f, vzr = 0.f, vxu = 0.f, A11 = 0.f, A13 = 0.f, A15 = 0.f, A33 = 0.f, A35 = 0.f;
  float gA11 = 0.f, gA13 = 0.f, gA15 = 0.f, gA33 = 0.f, gA35 = 0.f;
  if (l1) {
    vxr = S.vx[c + 1]; vzu = S.vz[c - P]; vzr = S.vz[c + 1]; vxu = S.vx[c - P];
    A11 = a.A11[c]; A13 = a.A13[c]; A15 = a.A15[c]; A33 = a.A33[c]; A35 = a.A35[c];
    gA11 = a.gA11[c]; gA13 = a.gA13[c]; gA15 = a.gA15[c]; gA33 = a.gA33[c]; gA35 = a.gA35[c];
  }
  float s1q[4], lnq[4], s1p[4], lnp[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const bool on = isx[q] ? xs : zs;
    const int m = isx[q] ? mx : mz;
    s1q[q] = on && l2 ? S1.m[qm[q]][m] : 0.f;
    lnq[q] = on ? Ln.m[qm[q]][m] : 0.f;
    s1p[q] = on && l1 ? S1.m[pm[q]][m] : 0.f;
    lnp[q] = on ? Ln.m[pm[q]][m] : 0.f;
  }
  // ---- the stresses' adjoints: the next state's plus the velocity half's differences
  const float lsxx = lnsxx + lc1c - lc1r;
  const float lszz = lnszz - ld2c + ld2u;
  const float lsxz = lnsxz - ld1c + ld1l + lc2c - lc2d;
  float la[4] = {0.f, 0.f, 0.f, 0.f}, lb[4] = {0.f, 0.f, 0.f, 0.f};
  float outq[4], outp[4];  // the memory variables' adjoints to store (strip cells)
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    outq[q] = lnq[q];
    outp[q] = lnp[q];
  }
  if (l2) {  // loop 2 transposed
    const float lf = lsxz;
    const float d[4] = {vxc - vxl, vzd - vzc, vzc - vzl, vxd - vxc};
    float f[4];
    const float lfq[4] = {B15 * lf, B35 * lf, B55 * lf, B55 * lf};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const bool on = isx[q] ? xs : zs;
      f[q] = d[q] * ik[q] + (on ? s1q[q] : 0.f);
      lb[q] = ik[q] * lfq[q];
      if (on) {
        const float tt = lnq[q] + lfq[q];
        lb[q] += ad[q] * tt;
        outq[q] = bb[q] * tt;
      }
    }
    gB15 += lf * f[0];
    gB35 += lf * f[1];
    gB55 += lf * (f[2] + f[3]);
  }
  if (l1) {  // loop 1 transposed
    const float ls = lsxx, lz = lszz;
    const float d[4] = {vxr - vxc, vzc - vzu, vzr - vzc, vxc - vxu};
    float e[4];
    const float A15e = A15 * ls + A35 * lz;
    const float le[4] = {A11 * ls + A13 * lz, A13 * ls + A33 * lz, A15e, A15e};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const bool on = isx[q] ? xs : zs;
      e[q] = d[q] * ik[q] + (on ? s1p[q] : 0.f);
      la[q] = ik[q] * le[q];
      if (on) {
        const float tt = lnp[q] + le[q];
        la[q] += ad[q] * tt;
        outp[q] = bb[q] * tt;
      }
    }
    gA11 += ls * e[0];
    gA13 += ls * e[1] + lz * e[0];
    gA15 += ls * (e[2] + e[3]);
    gA33 += lz * e[1];
    gA35 += lz * (e[2] + e[3]);
  }
  // ---- stores
  Lc.sxx[c] = lsxx;
  Lc.szz[c] = lszz;
  Lc.sxz[c] = lsxz;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const bool on = isx[q] ? xs : zs;
    const int m = isx[q] ? mx : mz;
    if (on) {
      Lc.m[qm[q]][m] = outq[q];
      Lc.m[pm[q]][m] = outp[q];
    }
  }
  if (l2) {
    a.gB15[c] = gB15;
    a.gB35[c] = gB35;
    a.gB55[c] = gB55;
  }
  if (l1) {
    a.gA11[c] = gA11;
    a.gA13[c] = gA13;
    a.gA15[c] = gA15;
    a.gA33[c] = gA33;
    a.gA35[c] = gA35;
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    a.tmp[4 + q][c] = la[q];
    a.tmp[8 + q][c] = lb[q];
  }
}

// The g phase at (i, k): Lc's velocities gain the gathered la, lb terms.
__device__ __forceinline__ void g_cell(const S2Adj& a, const S2State& Lc, int i, int k) {
  const int NX = a.NX, NZ = a.NZ, P = a.P;
  const size_t c = (size_t)k * P + i;
  auto T = [&](int q, int di, int dk) -> float {
    const int ii = i + di, kk = k + dk;
    if (ii < 0 || ii >= NX || kk < 0 || kk >= NZ) return 0.f;
    return a.tmp[q][(size_t)kk * P + ii];
  };
  // la: a1 = vx(i+1)-vx(i), a2 = vz(k)-vz(k-1), a3 = vz(i+1)-vz(i), a4 = vx(k)-vx(k-1)
  // lb: b1 = vx(i)-vx(i-1), b2 = vz(k+1)-vz(k), b3 = vz(i)-vz(i-1), b4 = vx(k+1)-vx(k)
  const float gvx = (T(4, -1, 0) - T(4, 0, 0)) + (T(7, 0, 0) - T(7, 0, 1)) + (T(8, 0, 0) - T(8, 1, 0)) +
                    (T(11, 0, -1) - T(11, 0, 0));
  const float gvz = (T(5, 0, 0) - T(5, 0, 1)) + (T(6, -1, 0) - T(6, 0, 0)) + (T(9, 0, -1) - T(9, 0, 0)) +
                    (T(10, 0, 0) - T(10, 1, 0));
  Lc.vx[c] += gvx;
  Lc.vz[c] += gvz;
}

__global__ void __launch_bounds__(BX * BY) s2adj_v(S2Adj a, S2State S, S2State S1, S2State Ln, S2State Lc, int rel) {
  const int i = blockIdx.x * BX + threadIdx.x, k = blockIdx.y * BY + threadIdx.y;
  if (i < a.NX && k < a.NZ) v_cell(a, S, S1, Ln, Lc, a.ctl->base + rel, i, k);
}

__global__ void __launch_bounds__(BX * BY) s2adj_g(S2Adj a, S2State Lc) {
  const int i = blockIdx.x * BX + threadIdx.x, k = blockIdx.y * BY + threadIdx.y;
  if (i < a.NX && k < a.NZ) g_cell(a, Lc, i, k);
}

// g of step base + rel + 1 on G, then v of step base + rel (S, S1, Ln = G, Lc).
__global__ void __launch_bounds__(BX * BY) s2adj_gv(S2Adj a, S2State G, S2State S, S2State S1, S2State Lc, int rel) {
  const int i = blockIdx.x * BX + threadIdx.x, k = blockIdx.y * BY + threadIdx.y;
  if (i >= a.NX || k >= a.NZ) return;
  g_cell(a, G, i, k);
  v_cell(a, S, S1, G, Lc, a.ctl->base + rel, i, k);
}

// The receiver lists of the cells: receivers visited from the last to the
// first, so each cell's list starts at its smallest index (one thread: a
// fixed order, whatever the receivers share).
__global__ void s2adj_recmap(const int* rec, int nrec, int P, int* recmap, int* recnext) {
  if (threadIdx.x || blockIdx.x) return;
  for (int r = nrec - 1; r >= 0; --r) {
    const size_t c = (size_t)rec[3 * r + 2] * P + rec[3 * r];
    recnext[r] = recmap[c];
    recmap[c] = r;
  }
}

}  // namespace

cudaError_t s2_adj_recmap(const int* rec, int nrec, int P, int NZ, int* recmap, int* recnext, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(recmap, 0xff, sizeof(int) * (size_t)P * NZ, s);  // -1 everywhere
  if (e == cudaSuccess && nrec > 0) {
    s2adj_recmap<<<1, 1, 0, s>>>(rec, nrec, P, recmap, recnext);
    e = cudaGetLastError();
  }
  return e;
}

void s2_adj_sweep(const S2Adj& a, char* slots, size_t stride, const S2Offsets& off, char* lam0, char* lam1, int cur,
                  int nsteps, cudaStream_t s) {
  auto state = [&](char* base) {
    S2State S;
    float** f[5] = {&S.vx, &S.vz, &S.sxx, &S.szz, &S.sxz};
    for (int q = 0; q < 5; ++q) *f[q] = (float*)(base + off.o[q]);
    for (int m = 0; m < 12; ++m) S.m[m] = (float*)(base + off.o[5 + m]);
    return S;
  };
  char* lam[2] = {lam0, lam1};
  const dim3 b(BX, BY), g((a.NX + BX - 1) / BX, (a.NZ + BY - 1) / BY);
  const int last = nsteps - 1;
  s2adj_v<<<g, b, 0, s>>>(a, state(slots + stride * (size_t)last), state(slots + stride * (size_t)nsteps),
                          state(lam[cur]), state(lam[cur ^ 1]), last);
  for (int st = last; st >= 0; --st) {  // step base + st: Ln = lam[cur], Lc = lam[cur ^ 1]
    const S2State S = state(slots + stride * (size_t)st), S1 = state(slots + stride * (size_t)(st + 1));
    const S2State Ln = state(lam[cur]), Lc = state(lam[cur ^ 1]);
    s2adj_s<<<g, b, 0, s>>>(a, S, S1, Ln, Lc);
    if (st > 0)  // the next step back: its Ln is this step's Lc, its Lc this step's Ln
      s2adj_gv<<<g, b, 0, s>>>(a, Lc, state(slots + stride * (size_t)(st - 1)), S, Ln, st - 1);
    else
      s2adj_g<<<g, b, 0, s>>>(a, Lc);
    cur ^= 1;
  }
}

}  // namespace sfd
