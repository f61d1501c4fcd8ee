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
  float lvx = inner ? Ln.vx[c] : 0.f, lvz = inner ? Ln.vz[c] : 0.f;
  if (inner)  // this step's residual at the cell's receivers (the traces sample vx', vz')
    for (int r = a.recmap[c]; r >= 0; r = a.recnext[r]) {
      lvx += a.resid[((size_t)t * 2 + 0) * a.nrec + r];
      lvz += a.resid[((size_t)t * 2 + 1) * a.nrec + r];
    }
  float lc1 = 0.f, lc2 = 0.f, ld1 = 0.f, ld2 = 0.f;
  if (vxr) {  // vx loop transposed
    const float lg = a.dtrx[c] * lvx;
    const float c1 = S1.sxx[c] - S1.sxx[c - 1], c2 = S1.sxz[c] - S1.sxz[c - P];
    float g = c1 * a.X.ik[i] + c2 * a.Z.ik[k];
    lc1 = a.X.ik[i] * lg;
    lc2 = a.Z.ik[k] * lg;
    if (xs) {
      const float tt = Ln.m[R1][mx] + lg;
      lc1 += a.X.ad[i] * tt;
      Lc.m[R1][mx] = a.X.b[i] * tt;
      g += S1.m[R1][mx];
    }
    if (zs) {
      const float tt = Ln.m[R2][mz] + lg;
      lc2 += a.Z.ad[k] * tt;
      Lc.m[R2][mz] = a.Z.b[k] * tt;
      g += S1.m[R2][mz];
    }
    if (inner) a.gdtrx[c] += lvx * g;
  } else {
    if (xs) Lc.m[R1][mx] = Ln.m[R1][mx];
    if (zs) Lc.m[R2][mz] = Ln.m[R2][mz];
  }
  if (vzr) {  // vz loop transposed
    const float lh = a.dtrz[c] * lvz;
    const float d1 = S1.sxz[c + 1] - S1.sxz[c], d2 = S1.szz[c + P] - S1.szz[c];
    float h = d1 * a.X.ikh[i] + d2 * a.Z.ikh[k];
    ld1 = a.X.ikh[i] * lh;
    ld2 = a.Z.ikh[k] * lh;
    if (xs) {
      const float tt = Ln.m[R3][mx] + lh;
      ld1 += a.X.adh[i] * tt;
      Lc.m[R3][mx] = a.X.bh[i] * tt;
      h += S1.m[R3][mx];
    }
    if (zs) {
      const float tt = Ln.m[R4][mz] + lh;
      ld2 += a.Z.adh[k] * tt;
      Lc.m[R4][mz] = a.Z.bh[k] * tt;
      h += S1.m[R4][mz];
    }
    if (inner) a.gdtrz[c] += lvz * h;
  } else {
    if (xs) Lc.m[R3][mx] = Ln.m[R3][mx];
    if (zs) Lc.m[R4][mz] = Ln.m[R4][mz];
  }
  if (inner) {
    a.ggxp[c] += lvx * S.vx[c];
    a.ggzp[c] += lvz * S.vz[c];
  }
  if (i == a.si && k == a.sk) *a.srcacc += lvx * a.srcfn[t] + lvz * a.srcfn[a.nstep + t];
  Lc.vx[c] = a.gxp[c] * lvx;  // the velocities' own parts; s2adj_g adds the stencil terms
  Lc.vz[c] = a.gzp[c] * lvz;
  a.tmp[0][c] = lc1;
  a.tmp[1][c] = lc2;
  a.tmp[2][c] = ld1;
  a.tmp[3][c] = ld2;
}

__global__ void __launch_bounds__(BX * BY) s2adj_s(S2Adj a, S2State S, S2State S1, S2State Ln, S2State Lc) {
  const int i = blockIdx.x * BX + threadIdx.x, k = blockIdx.y * BY + threadIdx.y;
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  if (i >= NX || k >= NZ) return;
  const size_t c = (size_t)k * P + i;
  const float* lc1 = a.tmp[0];
  const float* lc2 = a.tmp[1];
  const float* ld1 = a.tmp[2];
  const float* ld2 = a.tmp[3];
  // the stresses' adjoints: the next state's plus the velocity half's differences
  const float lsxx = Ln.sxx[c] + lc1[c] - (i + 1 < NX ? lc1[c + 1] : 0.f);
  const float lszz = Ln.szz[c] - ld2[c] + (k >= 1 ? ld2[c - P] : 0.f);
  const float lsxz = Ln.sxz[c] - ld1[c] + (i >= 1 ? ld1[c - 1] : 0.f) + lc2[c] - (k + 1 < NZ ? lc2[c + P] : 0.f);
  Lc.sxx[c] = lsxx;
  Lc.szz[c] = lszz;
  Lc.sxz[c] = lsxz;
  const bool xs = in_strip(i, NX, W), zs = in_strip(k, NZ, W);
  const int mx = xs ? mx_idx(i, k, NX, W) : 0, mz = zs ? mz_idx(i, k, NZ, P, W) : 0;
  // (memory variable, strip is x, ik, ad, b) of the four differences of a loop
  const int pm[4] = {P1, P2, P3, P4}, qm[4] = {Q1, Q2, Q3, Q4};
  const bool isx[4] = {true, false, true, false};
  const float ik[4] = {a.X.ikh[i], a.Z.ik[k], a.X.ik[i], a.Z.ikh[k]};
  const float ad[4] = {a.X.adh[i], a.Z.ad[k], a.X.ad[i], a.Z.adh[k]};
  const float bb[4] = {a.X.bh[i], a.Z.b[k], a.X.b[i], a.Z.bh[k]};
  float la[4] = {0.f, 0.f, 0.f, 0.f}, lb[4] = {0.f, 0.f, 0.f, 0.f};
  if (k <= NZ - 2 && i >= 1) {  // loop 2 transposed
    const float lf = lsxz;
    const float d[4] = {S.vx[c] - S.vx[c - 1], S.vz[c + P] - S.vz[c], S.vz[c] - S.vz[c - 1], S.vx[c + P] - S.vx[c]};
    float f[4];
    const float lfq[4] = {a.B15[c] * lf, a.B35[c] * lf, a.B55[c] * lf, a.B55[c] * lf};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const bool on = isx[q] ? xs : zs;
      const int m = isx[q] ? mx : mz;
      f[q] = d[q] * ik[q] + (on ? S1.m[qm[q]][m] : 0.f);
      lb[q] = ik[q] * lfq[q];
      if (on) {
        const float tt = Ln.m[qm[q]][m] + lfq[q];
        lb[q] += ad[q] * tt;
        Lc.m[qm[q]][m] = bb[q] * tt;
      }
    }
    a.gB15[c] += lf * f[0];
    a.gB35[c] += lf * f[1];
    a.gB55[c] += lf * (f[2] + f[3]);
  } else {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const bool on = isx[q] ? xs : zs;
      const int m = isx[q] ? mx : mz;
      if (on) Lc.m[qm[q]][m] = Ln.m[qm[q]][m];
    }
  }
  if (k >= 1 && i <= NX - 2) {  // loop 1 transposed
    const float ls = lsxx, lz = lszz;
    const float d[4] = {S.vx[c + 1] - S.vx[c], S.vz[c] - S.vz[c - P], S.vz[c + 1] - S.vz[c], S.vx[c] - S.vx[c - P]};
    float e[4];
    const float A15e = a.A15[c] * ls + a.A35[c] * lz;
    const float le[4] = {a.A11[c] * ls + a.A13[c] * lz, a.A13[c] * ls + a.A33[c] * lz, A15e, A15e};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const bool on = isx[q] ? xs : zs;
      const int m = isx[q] ? mx : mz;
      e[q] = d[q] * ik[q] + (on ? S1.m[pm[q]][m] : 0.f);
      la[q] = ik[q] * le[q];
      if (on) {
        const float tt = Ln.m[pm[q]][m] + le[q];
        la[q] += ad[q] * tt;
        Lc.m[pm[q]][m] = bb[q] * tt;
      }
    }
    a.gA11[c] += ls * e[0];
    a.gA13[c] += ls * e[1] + lz * e[0];
    a.gA15[c] += ls * (e[2] + e[3]);
    a.gA33[c] += lz * e[1];
    a.gA35[c] += lz * (e[2] + e[3]);
  } else {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const bool on = isx[q] ? xs : zs;
      const int m = isx[q] ? mx : mz;
      if (on) Lc.m[pm[q]][m] = Ln.m[pm[q]][m];
    }
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
