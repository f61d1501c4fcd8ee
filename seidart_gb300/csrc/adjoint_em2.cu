// Discrete adjoint of the electromag2 time step (legacy/fortran/electromagfdtd.f95:249-321).
//
// One forward step maps the state s = (Ex, Ez, Hy, A = psi dEx_dz, B = psi dEz_dx,
// C = psi dHy_dz, D = psi dHy_dx) to s' by
//   H half:  A' = bz A + adz dEx,  B' = bx B + adx dEz,
//            Hy' = Hy + dbH (dEz ikx + B' + dEx ikz + A')             (H range)
//   E half:  C' = bzh C + adzh dHz, Ex' = CAx Ex + CBx (dHz ikzh + C')  (Ex range)
//            D' = bxh D + adxh dHx, Ez' = CAz Ez + CBz (dHx ikxh + D')  (Ez range)
//   source, then Dirichlet masks on Ex', Ez', Hy'; receivers sample Ex', Ez'.
// with dEx = Ex(i,k+1) - Ex(i,k), dEz = Ez(i+1,k) - Ez(i,k), dHz = Hy'(i,k) -
// Hy'(i,k-1), dHx = Hy'(i,k) - Hy'(i-1,k), CAx = (caEx(i,k) + caEx(i,k-1))/2 etc.
// (the averaged coefficients are stored per cell).
// The adjoint step is the exact transpose, in reverse order, written as a
// gather (each thread writes only its own cells): first the E half
// transposed, with the coefficient gradients dJ/dCA = lam_E' E,
// dJ/dCB = lam_E' (dH ik + psi') and the source term, then the H half.
// The forward state of each step is recomputed from a checkpoint into
// per-step slots (fused2d em2 step with out-of-place memory variables).
#include "adjoint.h"

namespace sfd {

namespace {

constexpr int BX = 32, BY = 8;

__device__ __forceinline__ bool ex_edge(int i, int k, int NX, int NZ) { return i == 0 || i == NX - 2 || k == 0 || k == NZ - 1; }
__device__ __forceinline__ bool ez_edge(int i, int k, int NX, int NZ) { return i == 0 || i == NX - 1 || k == 0 || k == NZ - 2; }
__device__ __forceinline__ bool hy_edge(int i, int k, int NX, int NZ) { return i == 0 || i == NX - 2 || k == 0 || k == NZ - 2; }
__device__ __forceinline__ bool ex_range(int i, int k, int NX, int NZ) { return i <= NX - 2 && k >= 1 && k <= NZ - 2; }
__device__ __forceinline__ bool ez_range(int i, int k, int NX, int NZ) { return k <= NZ - 2 && i >= 1 && i <= NX - 2; }
__device__ __forceinline__ bool h_range(int i, int k, int NX, int NZ) { return i <= NX - 2 && k <= NZ - 2; }

// Hy' (after the H half of the step from state S) at (i, k) in the H range.
// Away from the Hy Dirichlet edges it equals the stored Hy of the next state
// S1; on the edges (zeroed after the E half read them) it is recomputed.
__device__ __forceinline__ float hprime(const Em2Adj& a, const AdjState& S, const AdjState& S1, int i, int k) {
  const int P = a.P, W = a.W, NX = a.NX, NZ = a.NZ;
  const size_t c = (size_t)k * P + i;
  if (!hy_edge(i, k, NX, NZ)) return S1.Hy[c];
  const float dEx = S.Ex[c + P] - S.Ex[c];
  float vz = dEx * a.Z.ik[k];
  if (in_strip(k, NZ, W)) vz += a.Z.b[k] * S.A[(size_t)strip_idx(k, NZ, W) * P + i] + a.Z.ad[k] * dEx;
  const float dEz = S.Ez[c + 1] - S.Ez[c];
  float vx = dEz * a.X.ik[i];
  if (in_strip(i, NX, W)) vx += a.X.b[i] * S.B[(size_t)k * (2 * W) + strip_idx(i, NX, W)] + a.X.ad[i] * dEz;
  return a.dbH * (vx + vz);  // the previous Hy on an edge is zero
}

__global__ void __launch_bounds__(BX * BY) adj_inject_kernel(Em2Adj a, AdjState L, int t) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= a.nrec) return;
  const int i = a.rec[3 * r], k = a.rec[3 * r + 2];
  const size_t c = (size_t)k * a.P + i;
  atomicAdd(&L.Ex[c], a.resid[((size_t)t * 2 + 0) * a.nrec + r]);
  atomicAdd(&L.Ez[c], a.resid[((size_t)t * 2 + 1) * a.nrec + r]);
}

// ---------------------------------------------------------------------------
// Two passes per step, four cells per thread along x (16-byte loads and
// stores) and kAdjRows rows per thread marched along z: the gx of the next
// row, the Hy' of the previous row and the hA of the previous row stay in
// registers from one row to the next, so no neighbour value is recomputed or
// re-read.
//   adj_e4: masks, the E half transposed, the coefficient gradients, the
//           source term; writes TH (adjoint of Hy') and the E-half parts of
//           lam_Ex, lam_Ez (MEx, MEz) and the new C, D.
//   adj_h4: the H half transposed from TH; writes the adjoint of the state.

constexpr int kAdjRows = 1;

__device__ __forceinline__ float4 ldv(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void stv(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float& ev(float4& v, int e) { return (&v.x)[e]; }
__device__ __forceinline__ float ev(const float4& v, int e) { return (&v.x)[e]; }

// gx of the four cells i0..i0+3 in row k (zero outside the grid / Ex range).
__device__ __forceinline__ float4 gx_row(const Em2Adj& a, const AdjState& L, int i0, int k) {
  float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
  if (k < 0 || k >= a.NZ) return g;
  const size_t c = (size_t)k * a.P + i0;
  const float4 lx = ldv(L.Ex + c), cb = ldv(a.CBx + c);
  const float kz = a.Z.ikh[k] + a.Z.adh[k];
  const bool zs = in_strip(k, a.NZ, a.W);
  float4 lc = g;
  if (zs) lc = ldv(L.C + (size_t)strip_idx(k, a.NZ, a.W) * a.P + i0);
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int i = i0 + e;
    if (i >= a.NX || !ex_range(i, k, a.NX, a.NZ)) continue;
    const float lex = ex_edge(i, k, a.NX, a.NZ) ? 0.0f : ev(lx, e);
    float v = ev(cb, e) * lex * kz;
    if (zs) v += ev(lc, e) * a.Z.adh[k];
    ev(g, e) = v;
  }
  return g;
}

__global__ void __launch_bounds__(BX * BY, 2) adj_e4_kernel(Em2Adj a, AdjState S, AdjState S1, AdjState L,
                                                            AdjState Ln, float* TH, float* MEx, float* MEz, int t) {
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  const int i0 = 4 * (blockIdx.x * BX + threadIdx.x);
  const int kb = (blockIdx.y * BY + threadIdx.y) * kAdjRows;
  if (i0 >= NX || kb >= NZ) return;
  const float4 ikhx = ldv(a.X.ikh + i0), adhx = ldv(a.X.adh + i0), bhx = ldv(a.X.bh + i0);
  bool xs[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) xs[e] = i0 + e < NX && in_strip(i0 + e, NX, W);
  float4 gxk = gx_row(a, L, i0, kb);  // gx of the current row, carried down
  float4 hpm;                          // Hy' of the row above the current one, carried down
#pragma unroll
  for (int e = 0; e < 4; ++e)
    ev(hpm, e) = (kb >= 1 && i0 + e < NX && h_range(i0 + e, kb - 1, NX, NZ)) ? hprime(a, S, S1, i0 + e, kb - 1) : 0.0f;
  for (int r = 0; r < kAdjRows; ++r) {
    const int k = kb + r;
    if (k >= NZ) break;
    const size_t c = (size_t)k * P + i0;
    const bool zs = in_strip(k, NZ, W);
    const size_t mz = (size_t)(zs ? strip_idx(k, NZ, W) : 0) * P + i0;
    const float4 lx = ldv(L.Ex + c), lz = ldv(L.Ez + c), lh = ldv(L.Hy + c);
    const float4 cax = ldv(a.CAx + c), cbx = ldv(a.CBx + c), caz = ldv(a.CAz + c), cbz = ldv(a.CBz + c);
    const float4 sx = ldv(S.Ex + c), sz = ldv(S.Ez + c), s1h = ldv(S1.Hy + c);
    const float4 gxn = gx_row(a, L, i0, k + 1);
    // gz of the four cells and of the cell to the right
    float gzv[5];
#pragma unroll
    for (int e = 0; e < 5; ++e) {
      const int i = i0 + e;
      float v = 0.0f;
      if (i < NX && ez_range(i, k, NX, NZ)) {
        const float lez = ez_edge(i, k, NX, NZ) ? 0.0f : (e < 4 ? ev(lz, e) : L.Ez[c + 4]);
        const float cb = e < 4 ? ev(cbz, e) : a.CBz[c + 4];
        const float kx = e < 4 ? ev(ikhx, e) + ev(adhx, e) : a.X.ikh[i] + a.X.adh[i];
        v = cb * lez * kx;
        if (in_strip(i, NX, W)) v += L.D[(size_t)k * (2 * W) + strip_idx(i, NX, W)] * a.X.adh[i];
      }
      gzv[e] = v;
    }
    // Hy' of this row and of the cell to the left
    float4 hp;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int i = i0 + e;
      ev(hp, e) = (i < NX && h_range(i, k, NX, NZ)) ? (hy_edge(i, k, NX, NZ) ? hprime(a, S, S1, i, k) : ev(s1h, e))
                                                   : 0.0f;
    }
    const float hpl = (i0 >= 1 && h_range(i0 - 1, k, NX, NZ)) ? hprime(a, S, S1, i0 - 1, k) : 0.0f;
    float4 th, mex, mez, gcax = ldv(a.gCAx + c), gcbx = ldv(a.gCBx + c), gcaz = ldv(a.gCAz + c), gcbz = ldv(a.gCBz + c);
    float4 lc = make_float4(0.f, 0.f, 0.f, 0.f), s1c = lc, lnc = lc;
    if (zs) {
      lc = ldv(L.C + mz);
      s1c = ldv(S1.C + mz);
      lnc = lc;
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int i = i0 + e;
      ev(th, e) = 0.0f;
      ev(mex, e) = 0.0f;
      ev(mez, e) = 0.0f;
      if (i >= NX) continue;
      const float lex = ex_edge(i, k, NX, NZ) ? 0.0f : ev(lx, e);
      const float lez = ez_edge(i, k, NX, NZ) ? 0.0f : ev(lz, e);
      const float lhy = hy_edge(i, k, NX, NZ) ? 0.0f : ev(lh, e);
      ev(th, e) = lhy + ev(gxk, e) - ev(gxn, e) + gzv[e] - gzv[e + 1];
      float mx = lex, mzv = lez;
      if (ex_range(i, k, NX, NZ)) {
        mx = ev(cax, e) * lex;
        const float dHz = ev(hp, e) - ev(hpm, e);
        float d = dHz * a.Z.ikh[k];
        if (zs) {
          d += ev(s1c, e);
          ev(lnc, e) = a.Z.bh[k] * (ev(cbx, e) * lex + ev(lc, e));
        }
        ev(gcax, e) += lex * ev(sx, e);
        ev(gcbx, e) += lex * d;
      }
      if (ez_range(i, k, NX, NZ)) {
        mzv = ev(caz, e) * lez;
        const float dHx = ev(hp, e) - (e == 0 ? hpl : ev(hp, e - 1));
        float d = dHx * ev(ikhx, e);
        if (xs[e]) {
          const size_t m = (size_t)k * (2 * W) + strip_idx(i, NX, W);
          d += S1.D[m];
          Ln.D[m] = ev(bhx, e) * (ev(cbz, e) * lez + L.D[m]);
        }
        ev(gcaz, e) += lez * ev(sz, e);
        ev(gcbz, e) += lez * d;
      } else if (xs[e]) {
        const size_t m = (size_t)k * (2 * W) + strip_idx(i, NX, W);
        Ln.D[m] = L.D[m];
      }
      ev(mex, e) = mx;
      ev(mez, e) = mzv;
      if (i == a.si && k == a.sk) {
        a.srcacc[0] += lex * a.srcfn[t];
        a.srcacc[1] += lez * a.srcfn[a.nstep + t];
      }
    }
    if (zs) stv(Ln.C + mz, lnc);
    stv(TH + c, th);
    stv(MEx + c, mex);
    stv(MEz + c, mez);
    stv(a.gCAx + c, gcax);
    stv(a.gCBx + c, gcbx);
    stv(a.gCAz + c, gcaz);
    stv(a.gCBz + c, gcbz);
    gxk = gxn;
    hpm = hp;
  }
}

// hA of the four cells in row k (zero outside the H range).
__device__ __forceinline__ float4 hA_row(const Em2Adj& a, const AdjState& L, const float* TH, int i0, int k) {
  float4 h = make_float4(0.f, 0.f, 0.f, 0.f);
  if (k < 0) return h;
  const size_t c = (size_t)k * a.P + i0;
  const float4 th = ldv(TH + c);
  const float kz = a.Z.ik[k] + a.Z.ad[k];
  const bool zs = in_strip(k, a.NZ, a.W);
  float4 la = h;
  if (zs) la = ldv(L.A + (size_t)strip_idx(k, a.NZ, a.W) * a.P + i0);
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int i = i0 + e;
    if (i >= a.NX || !h_range(i, k, a.NX, a.NZ)) continue;
    float v = a.dbH * ev(th, e) * kz;
    if (zs) v += ev(la, e) * a.Z.ad[k];
    ev(h, e) = v;
  }
  return h;
}

__global__ void __launch_bounds__(BX * BY, 3) adj_h4_kernel(Em2Adj a, AdjState L, AdjState Ln, const float* TH,
                                                         const float* MEx, const float* MEz) {
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  const int i0 = 4 * (blockIdx.x * BX + threadIdx.x);
  const int kb = (blockIdx.y * BY + threadIdx.y) * kAdjRows;
  if (i0 >= NX || kb >= NZ) return;
  const float4 ikx = ldv(a.X.ik + i0), adx = ldv(a.X.ad + i0), bx = ldv(a.X.b + i0);
  float4 hAm = hA_row(a, L, TH, i0, kb - 1);  // hA of the row above, carried down
  for (int r = 0; r < kAdjRows; ++r) {
    const int k = kb + r;
    if (k >= NZ) break;
    const size_t c = (size_t)k * P + i0;
    const float4 th = ldv(TH + c), mex = ldv(MEx + c), mez = ldv(MEz + c);
    const float4 hA = hA_row(a, L, TH, i0, k);
    // hB of the cell to the left and of the four cells
    float hB[5];
#pragma unroll
    for (int e = 0; e < 5; ++e) {
      const int i = i0 - 1 + e;
      float v = 0.0f;
      if (i >= 0 && i < NX && h_range(i, k, NX, NZ)) {
        const float tv = e > 0 ? ev(th, e - 1) : TH[c - 1];
        const float kx = e > 0 ? ev(ikx, e - 1) + ev(adx, e - 1) : a.X.ik[i] + a.X.ad[i];
        v = a.dbH * tv * kx;
        if (in_strip(i, NX, W)) v += L.B[(size_t)k * (2 * W) + strip_idx(i, NX, W)] * a.X.ad[i];
      }
      hB[e] = v;
    }
    const bool zs = in_strip(k, NZ, W);
    float4 lex, lez, lhy;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int i = i0 + e;
      if (i >= NX) {
        ev(lex, e) = ev(lez, e) = ev(lhy, e) = 0.0f;
        continue;
      }
      const bool hr = h_range(i, k, NX, NZ);
      ev(lex, e) = ev(mex, e) + ev(hAm, e) - ev(hA, e);
      ev(lez, e) = ev(mez, e) + hB[e] - hB[e + 1];
      ev(lhy, e) = (hr && hy_edge(i, k, NX, NZ)) ? 0.0f : ev(th, e);
      if (in_strip(i, NX, W)) {
        const size_t m = (size_t)k * (2 * W) + strip_idx(i, NX, W);
        Ln.B[m] = hr ? ev(bx, e) * (a.dbH * ev(th, e) + L.B[m]) : L.B[m];
      }
    }
    stv(Ln.Ex + c, lex);
    stv(Ln.Ez + c, lez);
    stv(Ln.Hy + c, lhy);
    if (zs) {
      const size_t m = (size_t)strip_idx(k, NZ, W) * P + i0;
      const float4 la = ldv(L.A + m);
      float4 na;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = i0 + e;
        ev(na, e) = (i < NX && h_range(i, k, NX, NZ)) ? a.Z.b[k] * (a.dbH * ev(th, e) + ev(la, e)) : ev(la, e);
      }
      stv(Ln.A + m, na);
    }
    hAm = hA;
  }
}

}  // namespace

void adj_step(const Em2Adj& a, const AdjState& S, const AdjState& S1, const AdjState& L, const AdjState& Ln, int t,
              cudaStream_t s) {
  if (a.nrec > 0) adj_inject_kernel<<<(a.nrec + 255) / 256, 256, 0, s>>>(a, L, t);
  const dim3 b(BX, BY), g((a.NX + 4 * BX - 1) / (4 * BX), (a.NZ + BY * kAdjRows - 1) / (BY * kAdjRows));
  adj_e4_kernel<<<g, b, 0, s>>>(a, S, S1, L, Ln, a.TH, a.MEx, a.MEz, t);
  adj_h4_kernel<<<g, b, 0, s>>>(a, L, Ln, a.TH, a.MEx, a.MEz);
}

}  // namespace sfd
