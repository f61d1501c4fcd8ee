// electromag2 (legacy/fortran/electromagfdtd.f95:10-326): 2-D TE Yee scheme,
// fields Ex, Ez, Hy, four CPML memory variables.  Two fused kernels per step:
//   half1: Hy update (:249-266) with dEx/dz and dEz/dx memory variables; block
//          (0,0) first records the receivers of the previous step.
//   half2: Ex (:273-283) and Ez (:285-295) updates with the dHy memory
//          variables, the source (:300-301), the Dirichlet edges (:304-317)
//          and the per-block field norm (:320-321).
// Hy edges are zeroed at the end of a Fortran step (:314-317), after Ex/Ez
// have read them; here half1 treats the previous Hy on those edges as zero
// and the finalize kernel zeroes them in memory at the end of each run.
#include "sfd_solvers.h"

namespace sfd {

namespace {

constexpr int BX = 32, BY = 8;

__global__ void __launch_bounds__(BX * BY) em2_h_kernel(Em2Args a, int rel) {
  const Ctl* ctl = a.io.ctl;
  const int t = ctl->base + rel;
  if (blockIdx.x == 0 && blockIdx.y == 0 && t > ctl->run_start) {
    const float* ch[2] = {a.Ex, a.Ez};
    gather_receivers<2>(a.io.rec, a.io.nrec, a.io.traces, t - 1, ch, a.P, 1, false);
  }
  const int i = blockIdx.x * BX + threadIdx.x;
  const int k = blockIdx.y * BY + threadIdx.y;
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  if (i > NX - 2 || k > NZ - 2) return;
  const size_t c = (size_t)k * P + i;
  // dEx/dz, :252-254
  const float dEx = a.Ex[c + P] - a.Ex[c];
  float vz = dEx * a.Z.ik[k];
  if (in_strip(k, NZ, W)) {
    const size_t m = (size_t)strip_idx(k, NZ, W) * P + i;
    const float psi = a.Z.b[k] * a.mExz[m] + a.Z.ad[k] * dEx;
    a.mExz[m] = psi;
    vz += psi;
  }
  // dEz/dx, :257-259
  const float dEz = a.Ez[c + 1] - a.Ez[c];
  float vx = dEz * a.X.ik[i];
  if (in_strip(i, NX, W)) {
    const size_t m = (size_t)k * (2 * W) + strip_idx(i, NX, W);
    const float psi = a.X.b[i] * a.mEzx[m] + a.X.ad[i] * dEz;
    a.mEzx[m] = psi;
    vx += psi;
  }
  const bool edge = (i == 0) | (i == NX - 2) | (k == 0) | (k == NZ - 2);
  const float hy = edge ? 0.0f : a.Hy[c];
  a.Hy[c] = hy + a.dbH * (vx + vz);  // :262
}

__global__ void __launch_bounds__(BX * BY) em2_e_kernel(Em2Args a, int rel) {
  const int t = a.io.ctl->base + rel;
  const int i = blockIdx.x * BX + threadIdx.x;
  const int k = blockIdx.y * BY + threadIdx.y;
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  float norm = 0.0f;
  if (i < NX && k < NZ) {
    const size_t c = (size_t)k * P + i;
    float ex = 0.0f, ez = 0.0f;
    // Ex, :273-283 (k in [1, NZ-2], i in [0, NX-2])
    if (i <= NX - 2) {
      ex = a.Ex[c];
      if (k >= 1 && k <= NZ - 2) {
        const float dH = a.Hy[c] - a.Hy[c - P];
        float d = dH * a.Z.ikh[k];
        if (in_strip(k, NZ, W)) {
          const size_t m = (size_t)strip_idx(k, NZ, W) * P + i;
          const float psi = a.Z.bh[k] * a.mHyz[m] + a.Z.adh[k] * dH;
          a.mHyz[m] = psi;
          d += psi;
        }
        ex = a.CAx[c] * ex + a.CBx[c] * d;
      }
    }
    // Ez, :285-295 (k in [0, NZ-2], i in [1, NX-2])
    if (k <= NZ - 2) {
      ez = a.Ez[c];
      if (i >= 1 && i <= NX - 2) {
        const float dH = a.Hy[c] - a.Hy[c - 1];
        float d = dH * a.X.ikh[i];
        if (in_strip(i, NX, W)) {
          const size_t m = (size_t)k * (2 * W) + strip_idx(i, NX, W);
          const float psi = a.X.bh[i] * a.mHyx[m] + a.X.adh[i] * dH;
          a.mHyx[m] = psi;
          d += psi;
        }
        ez = a.CAz[c] * ez + a.CBz[c] * d;
      }
    }
    // Source, :300-301
    if (i == a.io.si && k == a.io.sk) {
      ex += a.io.src[t];
      ez += a.io.src[a.io.nstep + t];
    }
    // Dirichlet edges, :304-312
    if (i == 0 || i == NX - 2 || k == 0 || k == NZ - 1) ex = 0.0f;
    if (i == 0 || i == NX - 1 || k == 0 || k == NZ - 2) ez = 0.0f;
    if (i <= NX - 2) a.Ex[c] = ex;
    if (k <= NZ - 2) a.Ez[c] = ez;
    norm = norm_monitor(ex, ez);
  }
  block_norm_to_slot(norm, a.io.slots, blockIdx.y * gridDim.x + blockIdx.x);
}

// Last receivers of the run, Hy edges to zero, run norm.
__global__ void em2_finalize_kernel(Em2Args a, int t_last) {
  const float* ch[2] = {a.Ex, a.Ez};
  gather_receivers<2>(a.io.rec, a.io.nrec, a.io.traces, t_last, ch, a.P, 1, false);
  const int NX = a.NX, NZ = a.NZ, P = a.P;
  for (int k = threadIdx.x; k < NZ; k += blockDim.x) {
    a.Hy[(size_t)k * P + 0] = 0.0f;
    a.Hy[(size_t)k * P + NX - 2] = 0.0f;
  }
  for (int i = threadIdx.x; i < NX; i += blockDim.x) {
    a.Hy[i] = 0.0f;
    a.Hy[(size_t)(NZ - 2) * P + i] = 0.0f;
  }
}

}  // namespace

Launch em2_launch(const Em2Args& a) {
  Launch L;
  L.block = dim3(BX, BY, 1);
  L.grid = dim3((a.NX + BX - 1) / BX, (a.NZ + BY - 1) / BY, 1);
  L.nslots = L.grid.x * L.grid.y;
  return L;
}

void em2_half1(const Em2Args& a, const Launch& L, int rel, cudaStream_t s) {
  em2_h_kernel<<<L.grid, L.block, 0, s>>>(a, rel);
}

void em2_half2(const Em2Args& a, const Launch& L, int rel, cudaStream_t s) {
  em2_e_kernel<<<L.grid, L.block, 0, s>>>(a, rel);
}

void em2_finalize(const Em2Args& a, int t_last, cudaStream_t s) { em2_finalize_kernel<<<1, 256, 0, s>>>(a, t_last); }

}  // namespace sfd
