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
// gather (each thread writes only its own cell):
//   adj_e: masks, the E half transposed, the coefficient gradients
//          dJ/dCA = lam_E' E, dJ/dCB = lam_E' (dH ik + psi'), the source term;
//          writes TH = adjoint of Hy' and the E-half parts of lam_Ex, lam_Ez.
//   adj_h: the H half transposed; writes the adjoint of the state s.
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

__device__ __forceinline__ float lam_masked_ex(const Em2Adj& a, const AdjState& L, int i, int k) {
  return ex_edge(i, k, a.NX, a.NZ) ? 0.0f : L.Ex[(size_t)k * a.P + i];
}
__device__ __forceinline__ float lam_masked_ez(const Em2Adj& a, const AdjState& L, int i, int k) {
  return ez_edge(i, k, a.NX, a.NZ) ? 0.0f : L.Ez[(size_t)k * a.P + i];
}

// Adjoint of the dHz difference at Ex-range cell (i, k).
__device__ __forceinline__ float gx_at(const Em2Adj& a, const AdjState& L, int i, int k) {
  if (!ex_range(i, k, a.NX, a.NZ)) return 0.0f;
  const size_t c = (size_t)k * a.P + i;
  const float cb = a.CBx[c];
  float g = cb * lam_masked_ex(a, L, i, k) * (a.Z.ikh[k] + a.Z.adh[k]);
  if (in_strip(k, a.NZ, a.W)) g += L.C[(size_t)strip_idx(k, a.NZ, a.W) * a.P + i] * a.Z.adh[k];
  return g;
}

// Adjoint of the dHx difference at Ez-range cell (i, k).
__device__ __forceinline__ float gz_at(const Em2Adj& a, const AdjState& L, int i, int k) {
  if (!ez_range(i, k, a.NX, a.NZ)) return 0.0f;
  const size_t c = (size_t)k * a.P + i;
  const float cb = a.CBz[c];
  float g = cb * lam_masked_ez(a, L, i, k) * (a.X.ikh[i] + a.X.adh[i]);
  if (in_strip(i, a.NX, a.W)) g += L.D[(size_t)k * (2 * a.W) + strip_idx(i, a.NX, a.W)] * a.X.adh[i];
  return g;
}

__global__ void __launch_bounds__(BX * BY) adj_inject_kernel(Em2Adj a, AdjState L, int t) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= a.nrec) return;
  const int i = a.rec[3 * r], k = a.rec[3 * r + 2];
  const size_t c = (size_t)k * a.P + i;
  atomicAdd(&L.Ex[c], a.resid[((size_t)t * 2 + 0) * a.nrec + r]);
  atomicAdd(&L.Ez[c], a.resid[((size_t)t * 2 + 1) * a.nrec + r]);
}

__global__ void __launch_bounds__(BX * BY) adj_e_kernel(Em2Adj a, AdjState S, AdjState S1, AdjState L, AdjState Ln,
                                                        int t) {
  const int i = blockIdx.x * BX + threadIdx.x;
  const int k = blockIdx.y * BY + threadIdx.y;
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  if (i >= NX || k >= NZ) return;
  const size_t c = (size_t)k * P + i;
  const bool zs = in_strip(k, NZ, W), xs = in_strip(i, NX, W);
  const size_t mz = (size_t)(zs ? strip_idx(k, NZ, W) : 0) * P + i;
  const size_t mx = (size_t)k * (2 * W) + (xs ? strip_idx(i, NX, W) : 0);
  const float lex = lam_masked_ex(a, L, i, k);
  const float lez = lam_masked_ez(a, L, i, k);
  const float lhy = hy_edge(i, k, NX, NZ) ? 0.0f : L.Hy[c];
  // adjoint of Hy' (gather of the dHz / dHx transposes)
  float th = lhy;
  if (i < NX && k < NZ) {
    th += gx_at(a, L, i, k) - (k + 1 < NZ ? gx_at(a, L, i, k + 1) : 0.0f);
    th += gz_at(a, L, i, k) - (i + 1 < NX ? gz_at(a, L, i + 1, k) : 0.0f);
  }
  a.TH[c] = th;
  // Ex half transposed
  float mex = lex, mez = lez;
  if (ex_range(i, k, NX, NZ)) {
    const float ca = a.CAx[c], cb = a.CBx[c];
    mex = ca * lex;
    const float dHz = hprime(a, S, S1, i, k) - hprime(a, S, S1, i, k - 1);
    float d = dHz * a.Z.ikh[k];
    if (zs) {
      const float lc = L.C[mz];
      d += S1.C[mz];  // C' of this step, stored in the next state
      Ln.C[mz] = a.Z.bh[k] * (cb * lex + lc);
    }
    a.gCAx[c] += lex * S.Ex[c];
    a.gCBx[c] += lex * d;
  } else if (zs) {
    Ln.C[mz] = L.C[mz];
  }
  if (ez_range(i, k, NX, NZ)) {
    const float ca = a.CAz[c], cb = a.CBz[c];
    mez = ca * lez;
    const float dHx = hprime(a, S, S1, i, k) - hprime(a, S, S1, i - 1, k);
    float d = dHx * a.X.ikh[i];
    if (xs) {
      const float ld = L.D[mx];
      d += S1.D[mx];  // D' of this step
      Ln.D[mx] = a.X.bh[i] * (cb * lez + ld);
    }
    a.gCAz[c] += lez * S.Ez[c];
    a.gCBz[c] += lez * d;
  } else if (xs) {
    Ln.D[mx] = L.D[mx];
  }
  a.MEx[c] = mex;
  a.MEz[c] = mez;
  if (i == a.si && k == a.sk) {  // source: Ex'(s) += srcx dt / eps11(s)
    a.srcacc[0] += lex * a.srcfn[t];
    a.srcacc[1] += lez * a.srcfn[a.nstep + t];
  }
}

__device__ __forceinline__ float hA_at(const Em2Adj& a, const AdjState& L, int i, int k) {
  if (i < 0 || k < 0 || !h_range(i, k, a.NX, a.NZ)) return 0.0f;
  const size_t c = (size_t)k * a.P + i;
  float h = a.dbH * a.TH[c] * (a.Z.ik[k] + a.Z.ad[k]);
  if (in_strip(k, a.NZ, a.W)) h += L.A[(size_t)strip_idx(k, a.NZ, a.W) * a.P + i] * a.Z.ad[k];
  return h;
}

__device__ __forceinline__ float hB_at(const Em2Adj& a, const AdjState& L, int i, int k) {
  if (i < 0 || k < 0 || !h_range(i, k, a.NX, a.NZ)) return 0.0f;
  const size_t c = (size_t)k * a.P + i;
  float h = a.dbH * a.TH[c] * (a.X.ik[i] + a.X.ad[i]);
  if (in_strip(i, a.NX, a.W)) h += L.B[(size_t)k * (2 * a.W) + strip_idx(i, a.NX, a.W)] * a.X.ad[i];
  return h;
}

__global__ void __launch_bounds__(BX * BY) adj_h_kernel(Em2Adj a, AdjState L, AdjState Ln) {
  const int i = blockIdx.x * BX + threadIdx.x;
  const int k = blockIdx.y * BY + threadIdx.y;
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  if (i >= NX || k >= NZ) return;
  const size_t c = (size_t)k * P + i;
  const bool zs = in_strip(k, NZ, W), xs = in_strip(i, NX, W);
  const float th = a.TH[c];
  const bool hr = h_range(i, k, NX, NZ);
  Ln.Ex[c] = a.MEx[c] + hA_at(a, L, i, k - 1) - hA_at(a, L, i, k);
  Ln.Ez[c] = a.MEz[c] + hB_at(a, L, i - 1, k) - hB_at(a, L, i, k);
  Ln.Hy[c] = (hr && hy_edge(i, k, NX, NZ)) ? 0.0f : th;
  if (zs) {
    const size_t m = (size_t)strip_idx(k, NZ, W) * P + i;
    Ln.A[m] = hr ? a.Z.b[k] * (a.dbH * th + L.A[m]) : L.A[m];
  }
  if (xs) {
    const size_t m = (size_t)k * (2 * W) + strip_idx(i, NX, W);
    Ln.B[m] = hr ? a.X.b[i] * (a.dbH * th + L.B[m]) : L.B[m];
  }
}

}  // namespace

void adj_step(const Em2Adj& a, const AdjState& S, const AdjState& S1, const AdjState& L, const AdjState& Ln, int t,
              cudaStream_t s) {
  dim3 b(BX, BY), g((a.NX + BX - 1) / BX, (a.NZ + BY - 1) / BY);
  if (a.nrec > 0) adj_inject_kernel<<<(a.nrec + 255) / 256, 256, 0, s>>>(a, L, t);
  adj_e_kernel<<<g, b, 0, s>>>(a, S, S1, L, Ln, t);
  adj_h_kernel<<<g, b, 0, s>>>(a, L, Ln);
}

}  // namespace sfd
