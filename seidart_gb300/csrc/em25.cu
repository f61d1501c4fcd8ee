// electromag25 (legacy/fortran/electromagfdtd.f95:619-1092): 2.5-D Yee scheme
// with Ex Ey Ez Hx Hy Hz, twelve CPML memory variables and y-invariant
// permittivity / conductivity.  One thread per (x, z) column marching along y.
//   half1: Hx (:901-919), Hy (:922-940), Hz (:943-962); block (0,0,0) first
//          records the receivers of the previous step.
//   half2: Ex and Ey (:968-1009), Ez (:1012-1029), source (:1033-1035),
//          Dirichlet faces of E (:1038-1055) and the norm (:1081-1082).
// The H faces (:1057-1078) are zeroed at the end of a Fortran step, after the
// E update has read them; half1 treats the previous H on those faces as zero
// and the finalize kernels zero them in memory at the end of each run.
#include "sfd_solvers.h"

namespace sfd {

namespace {

constexpr int BX = 32, BZ = 4;

__global__ void __launch_bounds__(BX * BZ) em25_h_kernel(Em25Args a, int rel) {
  const Ctl* ctl = a.io.ctl;
  const int t = ctl->base + rel;
  if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && t > ctl->run_start) {
    const float* ch[3] = {a.Ex, a.Ey, a.Ez};
    gather_receivers<3>(a.io.rec, a.io.nrec, a.io.traces, t - 1, ch, a.P, a.NY, true);
  }
  const int i = blockIdx.x * BX + threadIdx.x;
  const int k = blockIdx.y * BZ + threadIdx.y;
  const int NX = a.NX, NY = a.NY, NZ = a.NZ, P = a.P, W = a.W;
  // every H loop runs over i <= NX-2, j <= NY-2, k <= NZ-2
  if (i > NX - 2 || k > NZ - 2) return;
  const int seg = (NY + a.ysplit - 1) / a.ysplit;
  const int j0 = blockIdx.z * seg, j1 = min(NY - 1, j0 + seg);
  const bool xs = in_strip(i, NX, W), zs = in_strip(k, NZ, W);
  const int xsi = xs ? strip_idx(i, NX, W) : 0;
  const int zsi = zs ? strip_idx(k, NZ, W) : 0;
  const float ikx = a.X.ik[i], adx = a.X.ad[i], bx = a.X.b[i];
  const float ikz = a.Z.ik[k], adz = a.Z.ad[k], bz = a.Z.b[k];
  const float ikzh = a.Z.ikh[k], adzh = a.Z.adh[k], bzh = a.Z.bh[k];
  const size_t plane = (size_t)NY * P;
  const float dbH = a.dbH;
  const bool hz_rows = (k >= 1);
  // x/z parts of the H Dirichlet faces (0-based last planes per field)
  const bool fx_x = (i == 0) || (k == 0) || (k == NZ - 2);               // Hx: i=NX-1 is outside the loop
  const bool fy_x = (i == 0) || (i == NX - 2) || (k == 0) || (k == NZ - 2);
  const bool fz_x = (i == 0) || (i == NX - 2) || (k == 0);               // Hz: k=NZ-1 is outside the loop
  // Distinct arrays: the loads of a y step need not wait behind its stores.
  const float* __restrict__ Ex_ = a.Ex;
  const float* __restrict__ Ey_ = a.Ey;
  const float* __restrict__ Ez_ = a.Ez;
  float* __restrict__ Hx_ = a.Hx;
  float* __restrict__ Hy_ = a.Hy;
  float* __restrict__ Hz_ = a.Hz;
  float* __restrict__ mEz_y_ = a.mEz_y;
  float* __restrict__ mEy_z_ = a.mEy_z;
  float* __restrict__ mEx_z_ = a.mEx_z;
  float* __restrict__ mEz_x_ = a.mEz_x;
  float* __restrict__ mEx_y_ = a.mEx_y;
  float* __restrict__ mEy_x_ = a.mEy_x;
  for (int j = j0; j < j1; ++j) {
    const size_t c = ((size_t)k * NY + j) * P + i;
    const bool ys = in_strip(j, NY, W);
    const size_t mx = ((size_t)k * NY + j) * (2 * W) + xsi;
    const size_t my = ((size_t)k * (2 * W) + (ys ? strip_idx(j, NY, W) : 0)) * P + i;
    const size_t mz = ((size_t)zsi * NY + j) * P + i;
    const float iky = a.Y.ik[j], ady = a.Y.ad[j], by = a.Y.b[j];
    const float ikyh = a.Y.ikh[j], adyh = a.Y.adh[j], byh = a.Y.bh[j];
    const float ex = Ex_[c], ey = Ey_[c], ez = Ez_[c];
    // Hx, :904-917
    {
      const float d1 = ez - Ez_[c + P];  // dEz/dy
      float v1 = d1 * ikyh;
      if (ys) { const float m = byh * mEz_y_[my] + adyh * d1; mEz_y_[my] = m; v1 += m; }
      const float d2 = Ey_[c + plane] - ey;  // dEy/dz
      float v2 = d2 * ikzh;
      if (zs) { const float m = bzh * mEy_z_[mz] + adzh * d2; mEy_z_[mz] = m; v2 += m; }
      const float h = (fx_x || j == 0 || j == NY - 2) ? 0.f : Hx_[c];
      Hx_[c] = h + dbH * (v2 + v1);
    }
    // Hy, :925-938
    {
      const float d1 = ex - Ex_[c + plane];  // dEx/dz
      float v1 = d1 * ikz;
      if (zs) { const float m = bz * mEx_z_[mz] + adz * d1; mEx_z_[mz] = m; v1 += m; }
      const float d2 = Ez_[c + 1] - ez;  // dEz/dx
      float v2 = d2 * ikx;
      if (xs) { const float m = bx * mEz_x_[mx] + adx * d2; mEz_x_[mx] = m; v2 += m; }
      const float h = (fy_x || j == 0) ? 0.f : Hy_[c];  // Hy face j=NY-1 is outside the loop
      Hy_[c] = h + dbH * (v2 + v1);
    }
    // Hz, :946-960 (k >= 1)
    if (hz_rows) {
      const float d1 = Ex_[c + P] - ex;  // dEx/dy
      float v1 = d1 * iky;
      if (ys) { const float m = by * mEx_y_[my] + ady * d1; mEx_y_[my] = m; v1 += m; }
      const float d2 = ey - Ey_[c + 1];  // dEy/dx
      float v2 = d2 * ikx;
      if (xs) { const float m = bx * mEy_x_[mx] + adx * d2; mEy_x_[mx] = m; v2 += m; }
      const float h = (fz_x || j == 0 || j == NY - 2) ? 0.f : Hz_[c];
      Hz_[c] = h + dbH * (v2 + v1);
    }
  }
}

__global__ void __launch_bounds__(BX * BZ) em25_e_kernel(Em25Args a, int rel) {
  const int t = a.io.ctl->base + rel;
  const int i = blockIdx.x * BX + threadIdx.x;
  const int k = blockIdx.y * BZ + threadIdx.y;
  const int NX = a.NX, NY = a.NY, NZ = a.NZ, P = a.P, W = a.W;
  const int seg = (NY + a.ysplit - 1) / a.ysplit;
  const int j0 = blockIdx.z * seg, j1 = min(NY, j0 + seg);
  float norm = 0.0f;
  if (i < NX && k < NZ && j0 < j1) {
    const bool XEx = (k >= 1) && (k <= NZ - 2) && (i <= NX - 2);
    const bool XEy = (k >= 1) && (k <= NZ - 2) && (i >= 1) && (i <= NX - 2);
    const bool XEz = (k <= NZ - 2) && (i >= 1) && (i <= NX - 2);
    const size_t pc = (size_t)k * P + i;
    float caX = 0, cbX = 0, caY = 0, cbY = 0, caZ = 0, cbZ = 0;
    if (XEx) { caX = a.caEx[pc]; cbX = a.cbEx[pc]; }
    if (XEy) {  // (4 c(i,k) + c(i-1,k) + c(i,k-1)) / 6, :1004-1006
      caY = (4.f * a.caEy[pc] + a.caEy[pc - 1] + a.caEy[pc - P]) / 6.f;
      cbY = (4.f * a.cbEy[pc] + a.cbEy[pc - 1] + a.cbEy[pc - P]) / 6.f;
    }
    if (XEz) {  // (4 c(i,k) + c(i-1,k) + c(i,k+1)) / 6, :1026-1028
      caZ = (4.f * a.caEz[pc] + a.caEz[pc - 1] + a.caEz[pc + P]) / 6.f;
      cbZ = (4.f * a.cbEz[pc] + a.cbEz[pc - 1] + a.cbEz[pc + P]) / 6.f;
    }
    const bool xs = in_strip(i, NX, W), zs = in_strip(k, NZ, W);
    const int xsi = xs ? strip_idx(i, NX, W) : 0;
    const int zsi = zs ? strip_idx(k, NZ, W) : 0;
    const float ikxh = a.X.ikh[i], adxh = a.X.adh[i], bxh = a.X.bh[i];
    const float ikz = a.Z.ik[k], adz = a.Z.ad[k], bz = a.Z.b[k];
    const float ikzh = a.Z.ikh[k], adzh = a.Z.adh[k], bzh = a.Z.bh[k];
    const size_t plane = (size_t)NY * P;
    const bool fEx = (i == 0) || (i == NX - 2) || (k == 0) || (k == NZ - 1);
    const bool fEy = (i == 0) || (i == NX - 1) || (k == 0) || (k == NZ - 1);
    const bool fEz = (i == 0) || (i == NX - 1) || (k == 0) || (k == NZ - 2);
  // Distinct arrays: the loads of a y step need not wait behind its stores.
  const float* __restrict__ Hx_ = a.Hx;
  const float* __restrict__ Hy_ = a.Hy;
  const float* __restrict__ Hz_ = a.Hz;
  float* __restrict__ Ex_ = a.Ex;
  float* __restrict__ Ey_ = a.Ey;
  float* __restrict__ Ez_ = a.Ez;
  float* __restrict__ mHz_y_ = a.mHz_y;
  float* __restrict__ mHy_z_ = a.mHy_z;
  float* __restrict__ mHz_x_ = a.mHz_x;
  float* __restrict__ mHx_z_ = a.mHx_z;
  float* __restrict__ mHx_y_ = a.mHx_y;
  float* __restrict__ mHy_x_ = a.mHy_x;
    for (int j = j0; j < j1; ++j) {
      const size_t c = ((size_t)k * NY + j) * P + i;
      const bool ys = in_strip(j, NY, W);
      const size_t mx = ((size_t)k * NY + j) * (2 * W) + xsi;
      const size_t my = ((size_t)k * (2 * W) + (ys ? strip_idx(j, NY, W) : 0)) * P + i;
      const size_t mz = ((size_t)zsi * NY + j) * P + i;
      const float ikyh = a.Y.ikh[j], adyh = a.Y.adh[j], byh = a.Y.bh[j];
      float ex = Ex_[c], ey = Ey_[c], ez = Ez_[c];
      if (XEx && j >= 1 && j <= NY - 2) {  // :971-984
        const float d1 = Hz_[c] - Hz_[c - P];  // dHz/dy
        float v1 = d1 * ikyh;
        if (ys) { const float m = byh * mHz_y_[my] + adyh * d1; mHz_y_[my] = m; v1 += m; }
        const float d2 = Hy_[c - plane] - Hy_[c];  // dHy/dz
        float v2 = d2 * ikz;
        if (zs) { const float m = bz * mHy_z_[mz] + adz * d2; mHy_z_[mz] = m; v2 += m; }
        ex = caX * ex + cbX * (v1 + v2);
      }
      if (XEy && j <= NY - 2) {  // :988-1007
        const float d1 = Hz_[c - 1] - Hz_[c];  // dHz/dx
        float v1 = d1 * ikxh;
        if (xs) { const float m = bxh * mHz_x_[mx] + adxh * d1; mHz_x_[mx] = m; v1 += m; }
        const float d2 = Hx_[c] - Hx_[c - plane];  // dHx/dz
        float v2 = d2 * ikzh;
        if (zs) { const float m = bzh * mHx_z_[mz] + adzh * d2; mHx_z_[mz] = m; v2 += m; }
        ey = caY * ey + cbY * (v1 + v2);
      }
      if (XEz && j >= 1 && j <= NY - 2) {  // :1015-1029
        const float d1 = Hx_[c - P] - Hx_[c];  // dHx/dy
        float v1 = d1 * ikyh;
        if (ys) { const float m = byh * mHx_y_[my] + adyh * d1; mHx_y_[my] = m; v1 += m; }
        const float d2 = Hy_[c] - Hy_[c - 1];  // dHy/dx
        float v2 = d2 * ikxh;
        if (xs) { const float m = bxh * mHy_x_[mx] + adxh * d2; mHy_x_[mx] = m; v2 += m; }
        ez = caZ * ez + cbZ * (v1 + v2);
      }
      if (i == a.io.si && j == a.io.sj && k == a.io.sk) {  // :1033-1035
        ex += a.io.src[t];
        ey += a.io.src[a.io.nstep + t];
        ez += a.io.src[2 * a.io.nstep + t];
      }
      if (fEx || j == 0 || j == NY - 1) ex = 0.f;  // :1038-1043
      if (fEy || j == 0 || j == NY - 2) ey = 0.f;  // :1045-1050
      if (fEz || j == 0 || j == NY - 1) ez = 0.f;  // :1052-1057
      Ex_[c] = ex;
      Ey_[c] = ey;
      Ez_[c] = ez;
      norm = fmaxf(norm, norm_monitor(ex, ey, ez));
    }
  }
  block_norm_to_slot(norm, a.io.slots, (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x);
}

// Zero the H Dirichlet faces (:1059-1078) in memory.
__global__ void em25_hfaces_kernel(Em25Args a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y * blockDim.y + threadIdx.y;
  const int NX = a.NX, NY = a.NY, NZ = a.NZ, P = a.P;
  if (i >= NX || k >= NZ) return;
  const bool fx = (i == 0) || (i == NX - 1) || (k == 0) || (k == NZ - 2);
  const bool fy = (i == 0) || (i == NX - 2) || (k == 0) || (k == NZ - 2);
  const bool fz = (i == 0) || (i == NX - 2) || (k == 0) || (k == NZ - 1);
  for (int j = 0; j < NY; ++j) {
    const size_t c = ((size_t)k * NY + j) * P + i;
    if (fx || j == 0 || j == NY - 2) a.Hx[c] = 0.f;
    if (fy || j == 0 || j == NY - 1) a.Hy[c] = 0.f;
    if (fz || j == 0 || j == NY - 2) a.Hz[c] = 0.f;
  }
}

__global__ void em25_finalize_kernel(Em25Args a, int t_last) {
  const float* ch[3] = {a.Ex, a.Ey, a.Ez};
  gather_receivers<3>(a.io.rec, a.io.nrec, a.io.traces, t_last, ch, a.P, a.NY, true);
}

}  // namespace

Launch em25_launch(const Em25Args& a) {
  Launch L;
  L.block = dim3(BX, BZ, 1);
  L.grid = dim3((a.NX + BX - 1) / BX, (a.NZ + BZ - 1) / BZ, a.ysplit);
  L.nslots = L.grid.x * L.grid.y * L.grid.z;
  return L;
}

void em25_half1(const Em25Args& a, const Launch& L, int rel, cudaStream_t s) {
  em25_h_kernel<<<L.grid, L.block, 0, s>>>(a, rel);
}

void em25_half2(const Em25Args& a, const Launch& L, int rel, cudaStream_t s) {
  em25_e_kernel<<<L.grid, L.block, 0, s>>>(a, rel);
}

void em25_finalize(const Em25Args& a, int t_last, cudaStream_t s) {
  dim3 b(32, 8), g((a.NX + 31) / 32, (a.NZ + 7) / 8);
  em25_hfaces_kernel<<<g, b, 0, s>>>(a);
  em25_finalize_kernel<<<1, 256, 0, s>>>(a, t_last);
}

}  // namespace sfd
