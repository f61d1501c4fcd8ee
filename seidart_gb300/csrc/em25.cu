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
#include <type_traits>
#include "sfd_solvers.h"
#include "tma.cuh"

namespace sfd {

namespace {

constexpr int BX = 32, BZ = 4;



// ---------------------------------------------------------------------------
// TMA-staged y-march.  As the seismic25 kernels: each block
// (32 x BZ columns, one y segment) streams its y planes through a ring of
// RING shared-memory stages filled by cp.async.bulk.tensor boxes that one
// thread issues RING - 2 planes ahead, completion on the stage's mbarrier:
//   H kernel: the three E fields with a one-cell halo (x from i0 - 4, rows
//             k0 - 1 .. k0 + BZ) and the three H fields of the own cells; the
//             plane after the segment is staged too (its E only) for the y+
//             differences;
//   E kernel: the three H fields with the halo and the three E fields of the
//             own cells; the y- values are carried in registers.
// The memory variables (strips only) and the results go through plain loads
// and stores.  Every wait is bounded (Em25Args::wait_ns): one that runs out
// sets the control block's error word and the block leaves the kernel.
// Staging replaced a plain y-march whose every step waited a memory round
// trip (0.78 against 0.40 ms per step on a 630 x 70 x 330 grid).
constexpr int HX = 4;                // x halo of the staged tiles (16 bytes)
constexpr int VW = BX + 2 * HX;      // 40 floats per staged row
constexpr int VH = BZ + 2;           // rows k0 - 1 .. k0 + BZ
constexpr int RING = 4;              // staged planes per block
constexpr int HALO3 = 3 * VH * VW;   // three fields with the halo
constexpr int OWN3 = 3 * BZ * BX;    // three fields of the own cells
constexpr int OWN = 736;             // own cells after the halo, 128-byte aligned
constexpr int PSI = OWN + OWN3;      // the two y-strip memory variables of the kernel
constexpr int YTB = PSI + 2 * BZ * BX;  // the y table around the plane: 6 rows x 4 entries from j & ~3
constexpr int STAGE = YTB + 32;      // 5632 bytes
constexpr int FH = VH * VW;          // one field of a halo tile
static_assert(OWN >= HALO3 && (OWN * 4) % 128 == 0 && (PSI * 4) % 128 == 0 && (YTB * 4) % 128 == 0 &&
                  (STAGE * 4) % 128 == 0, "stage alignment");

// Whether every column of the block at (i0, k0) lies off the x and z CPML
// strips and two cells or more inside the grid (off every Dirichlet face of
// E and H: 1 <= i <= NX - 3, 1 <= k <= NZ - 3).
__device__ __forceinline__ bool block_interior(int i0, int k0, int NX, int NZ, int W) {
  return i0 >= max(W, 1) && i0 + BX - 1 <= min(NX - W - 1, NX - 3) && k0 >= max(W, 1) &&
         k0 + BZ - 1 <= min(NZ - W - 1, NZ - 3);
}

__device__ void em25_wait_failed(const Em25Args& a, uint64_t* full, int n, int np) {
  atomicExch(const_cast<int*>(&a.io.ctl->err), 1);
  const int issued = min(np, n + RING);
  for (int m = n; m < issued; ++m) tma::bar_wait(full + m % RING, (m / RING) & 1, a.wait_ns);
}

__global__ void __launch_bounds__(BX * BZ) em25_h_tma_kernel(const __grid_constant__ Em25Args a, int rel) {
  extern __shared__ __align__(128) unsigned char stage_raw[];
  float* const stage = tma::aligned_stage(stage_raw);
  __shared__ __align__(8) uint64_t full[RING];
  const Ctl* ctl = a.io.ctl;
  const int t = ctl->base + rel;
  if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && t > ctl->run_start) {
    const float* ch[3] = {a.Ex, a.Ey, a.Ez};
    gather_receivers<3>(a.io.rec, a.io.nrec, a.io.traces, t - 1, ch, a.P, a.NY, true);
  }
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * BX + tx;
  const int i0 = blockIdx.x * BX, k0 = blockIdx.y * BZ;
  const int NX = a.NX, NY = a.NY, NZ = a.NZ, P = a.P, W = a.W;
  const int seg = (NY + a.ysplit - 1) / a.ysplit;
  const int j0 = blockIdx.z * seg, j1 = min(NY - 1, j0 + seg);  // every H loop runs over j <= NY-2
  if (j0 >= j1) return;  // the whole block
  const int np = j1 - j0 + 1;  // the segment's planes and the next one (its E only)
  if (tid == 0) {
    for (int q = 0; q < RING; ++q) tma::bar_init(full + q, 1);
    tma::fence_bar_init();
  }
  __syncthreads();
  auto issue = [&](int n) {
    float* st = stage + (n % RING) * STAGE;
    uint64_t* bar = full + n % RING;
    const int j = j0 + n;
    const bool own = j < j1, ys = own && in_strip(j, NY, W);
    tma::bar_arrive_expect(bar, (HALO3 + (own ? OWN3 + 24 : 0) + (ys ? 2 * BZ * BX : 0)) * 4u + a.stall_tx);
    tma::load_4d(st, &a.tm_halo, bar, i0 - HX, j, k0 - 1, 0);  // Ex Ey Ez
    if (own) {
      tma::load_4d(st + OWN, &a.tm_own, bar, i0, j, k0, 3);  // Hx Hy Hz
      tma::load_2d(st + YTB, &a.tm_ytab, bar, j & ~3, 0);
    }
    if (ys) tma::load_4d(st + PSI, &a.tm_ypsi_e, bar, i0, strip_idx(j, NY, W), k0, 0);  // dEz_dy dEx_dy
  };
  if (tid == 0)
    for (int n = 0; n < min(RING, np); ++n) issue(n);

  const int i = i0 + tx, k = k0 + ty;
  const bool activec = i <= NX - 2 && k <= NZ - 2;
  const int ic = activec ? i : 0, kc = activec ? k : 0;
  const bool xsc = activec && in_strip(i, NX, W), zsc = activec && in_strip(k, NZ, W);
  const int xsi = xsc ? strip_idx(i, NX, W) : 0;
  const int zsi = zsc ? strip_idx(k, NZ, W) : 0;
  const float ikx = a.X.ik[ic], adx = a.X.ad[ic], bx = a.X.b[ic];
  const float ikz = a.Z.ik[kc], adz = a.Z.ad[kc], bz = a.Z.b[kc];
  const float ikzh = a.Z.ikh[kc], adzh = a.Z.adh[kc], bzh = a.Z.bh[kc];
  const float dbH = a.dbH;
  const bool hz_rowsc = (k >= 1);
  const bool fx_xc = (i == 0) || (k == 0) || (k == NZ - 2);
  const bool fy_xc = (i == 0) || (i == NX - 2) || (k == 0) || (k == NZ - 2);
  const bool fz_xc = (i == 0) || (i == NX - 2) || (k == 0);
  const bool interior = block_interior(i0, k0, NX, NZ, W);
  float* __restrict__ Hx_ = a.Hx;
  float* __restrict__ Hy_ = a.Hy;
  float* __restrict__ Hz_ = a.Hz;
  float* __restrict__ mEz_y_ = a.mEz_y;
  float* __restrict__ mEy_z_ = a.mEy_z;
  float* __restrict__ mEx_z_ = a.mEx_z;
  float* __restrict__ mEz_x_ = a.mEz_x;
  float* __restrict__ mEx_y_ = a.mEx_y;
  float* __restrict__ mEy_x_ = a.mEy_x;
  const int hc = (ty + 1) * VW + tx + HX;  // own cell in a halo tile
  const int oc = ty * BX + tx;             // own cell in an own-cells tile
  size_t c = ((size_t)kc * NY + j0) * P + ic;
  // The march, compiled twice: for blocks of interior columns only (I: no x
  // or z memory variables, no faces) and for the others.
  auto march = [&](auto interior_tag) {
  constexpr bool I = decltype(interior_tag)::value;
  const bool active = I || activec, xs = !I && xsc, zs = !I && zsc, hz_rows = I || hz_rowsc;
  const bool fx_x = !I && fx_xc, fy_x = !I && fy_xc, fz_x = !I && fz_xc;
  for (int n = 0; n < j1 - j0; ++n, c += P) {
    const int j = j0 + n;
    bool ok = tma::bar_wait(full + n % RING, (n / RING) & 1, a.wait_ns);
    if (ok) ok = tma::bar_wait(full + (n + 1) % RING, ((n + 1) / RING) & 1, a.wait_ns);
    if (ok && active) {
      const float* E = stage + (n % RING) * STAGE;         // Ex Ey Ez of plane j, with the halo
      const float* En = stage + ((n + 1) % RING) * STAGE;  // plane j + 1
      const float* H = E + OWN;                            // Hx Hy Hz of the own cells
      const bool ys = in_strip(j, NY, W);
      const size_t mx = ((size_t)k * NY + j) * (2 * W) + xsi;
      const size_t my = ((size_t)k * (2 * W) + (ys ? strip_idx(j, NY, W) : 0)) * P + i;
      const size_t mz = ((size_t)zsi * NY + j) * P + i;
      const float* yt = E + YTB + (j & 3);  // rows ik ad b ikh adh bh of the y table
      const float iky = yt[0], ady = yt[4], by = yt[8], ikyh = yt[12], adyh = yt[16], byh = yt[20];
      const float* Y = E + PSI;             // dEz_dy, dEx_dy of this plane (y strips)
      const float ex = E[hc], ey = E[FH + hc], ez = E[2 * FH + hc];
      {  // Hx, :904-917
        const float d1 = ez - En[2 * FH + hc];  // dEz/dy
        float v1 = d1 * ikyh;
        if (ys) { const float m = byh * Y[oc] + adyh * d1; mEz_y_[my] = m; v1 += m; }
        const float d2 = E[FH + hc + VW] - ey;  // dEy/dz
        float v2 = d2 * ikzh;
        if (zs) { const float m = bzh * mEy_z_[mz] + adzh * d2; mEy_z_[mz] = m; v2 += m; }
        const float h = (fx_x || j == 0 || j == NY - 2) ? 0.f : H[oc];
        Hx_[c] = h + dbH * (v2 + v1);
      }
      {  // Hy, :925-938
        const float d1 = ex - E[hc + VW];  // dEx/dz
        float v1 = d1 * ikz;
        if (zs) { const float m = bz * mEx_z_[mz] + adz * d1; mEx_z_[mz] = m; v1 += m; }
        const float d2 = E[2 * FH + hc + 1] - ez;  // dEz/dx
        float v2 = d2 * ikx;
        if (xs) { const float m = bx * mEz_x_[mx] + adx * d2; mEz_x_[mx] = m; v2 += m; }
        const float h = (fy_x || j == 0) ? 0.f : H[OWN3 / 3 + oc];  // Hy face j=NY-1 is outside the loop
        Hy_[c] = h + dbH * (v2 + v1);
      }
      if (hz_rows) {  // Hz, :946-960 (k >= 1)
        const float d1 = En[hc] - ex;  // dEx/dy
        float v1 = d1 * iky;
        if (ys) { const float m = by * Y[BZ * BX + oc] + ady * d1; mEx_y_[my] = m; v1 += m; }
        const float d2 = ey - E[FH + hc + 1];  // dEy/dx
        float v2 = d2 * ikx;
        if (xs) { const float m = bx * mEy_x_[mx] + adx * d2; mEy_x_[mx] = m; v2 += m; }
        const float h = (fz_x || j == 0 || j == NY - 2) ? 0.f : H[2 * (OWN3 / 3) + oc];
        Hz_[c] = h + dbH * (v2 + v1);
      }
    }
    if (!__syncthreads_and(ok)) {  // every thread is done with plane n (or a wait ran out)
      if (tid == 0) em25_wait_failed(a, full, n, np);
      break;
    }
    if (tid == 0 && n + RING < np) {
      tma::fence_async_smem();
      issue(n + RING);
    }
  }
  };
  if (interior) march(std::true_type{});
  else march(std::false_type{});
}

// 8 blocks per SM (64 registers, no spills): 0.2985 against 0.305 ms per
// step at the 72 registers and 7 blocks the compiler picks by itself (the
// 630 x 70 x 330 grid).
__global__ void __launch_bounds__(BX * BZ, 8) em25_e_tma_kernel(const __grid_constant__ Em25Args a, int rel) {
  extern __shared__ __align__(128) unsigned char stage_raw[];
  float* const stage = tma::aligned_stage(stage_raw);
  __shared__ __align__(8) uint64_t full[RING];
  const int t = a.io.ctl->base + rel;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * BX + tx;
  const int i0 = blockIdx.x * BX, k0 = blockIdx.y * BZ;
  const int NX = a.NX, NY = a.NY, NZ = a.NZ, P = a.P, W = a.W;
  const int seg = (NY + a.ysplit - 1) / a.ysplit;
  const int j0 = blockIdx.z * seg, j1 = min(NY, j0 + seg);
  const int slot = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
  float norm = 0.0f;
  if (j0 >= j1) {  // the whole block
    block_norm_to_slot(norm, a.io.slots, slot);
    return;
  }
  const int np = j1 - j0;
  if (tid == 0) {
    for (int q = 0; q < RING; ++q) tma::bar_init(full + q, 1);
    tma::fence_bar_init();
  }
  __syncthreads();
  auto issue = [&](int n) {
    float* st = stage + (n % RING) * STAGE;
    uint64_t* bar = full + n % RING;
    const int j = j0 + n;
    const bool ys = in_strip(j, NY, W);
    tma::bar_arrive_expect(bar, (HALO3 + OWN3 + 24 + (ys ? 2 * BZ * BX : 0)) * 4u + a.stall_tx);
    tma::load_4d(st, &a.tm_halo, bar, i0 - HX, j, k0 - 1, 3);  // Hx Hy Hz
    tma::load_4d(st + OWN, &a.tm_own, bar, i0, j, k0, 0);     // Ex Ey Ez
    tma::load_2d(st + YTB, &a.tm_ytab, bar, j & ~3, 0);
    if (ys) tma::load_4d(st + PSI, &a.tm_ypsi_h, bar, i0, strip_idx(j, NY, W), k0, 0);  // dHz_dy dHx_dy
  };
  if (tid == 0)
    for (int n = 0; n < min(RING, np); ++n) issue(n);

  const int i = i0 + tx, k = k0 + ty;
  const bool insidec = i < NX && k < NZ;
  const int ic = insidec ? i : 0, kc = insidec ? k : 0;
  const bool XEx = insidec && (k >= 1) && (k <= NZ - 2) && (i <= NX - 2);
  const bool XEy = insidec && (k >= 1) && (k <= NZ - 2) && (i >= 1) && (i <= NX - 2);
  const bool XEz = insidec && (k <= NZ - 2) && (i >= 1) && (i <= NX - 2);
  const size_t pc = (size_t)kc * P + ic;
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
  const bool xsc = insidec && in_strip(i, NX, W), zsc = insidec && in_strip(k, NZ, W);
  const int xsi = xsc ? strip_idx(i, NX, W) : 0;
  const int zsi = zsc ? strip_idx(k, NZ, W) : 0;
  const float ikxh = a.X.ikh[ic], adxh = a.X.adh[ic], bxh = a.X.bh[ic];
  const float ikz = a.Z.ik[kc], adz = a.Z.ad[kc], bz = a.Z.b[kc];
  const float ikzh = a.Z.ikh[kc], adzh = a.Z.adh[kc], bzh = a.Z.bh[kc];
  const bool fExc = (i == 0) || (i == NX - 2) || (k == 0) || (k == NZ - 1);
  const bool fEyc = (i == 0) || (i == NX - 1) || (k == 0) || (k == NZ - 1);
  const bool fEzc = (i == 0) || (i == NX - 1) || (k == 0) || (k == NZ - 2);
  const bool interior = block_interior(i0, k0, NX, NZ, W);
  float* __restrict__ Ex_ = a.Ex;
  float* __restrict__ Ey_ = a.Ey;
  float* __restrict__ Ez_ = a.Ez;
  float* __restrict__ mHz_y_ = a.mHz_y;
  float* __restrict__ mHy_z_ = a.mHy_z;
  float* __restrict__ mHz_x_ = a.mHz_x;
  float* __restrict__ mHx_z_ = a.mHx_z;
  float* __restrict__ mHx_y_ = a.mHx_y;
  float* __restrict__ mHy_x_ = a.mHy_x;
  const int hc = (ty + 1) * VW + tx + HX;
  const int oc = ty * BX + tx;
  size_t c = ((size_t)kc * NY + j0) * P + ic;
  float phx = 0.f, phz = 0.f;  // Hx, Hz of the plane before
  if (insidec && j0 >= 1) { phx = __ldg(a.Hx + c - P); phz = __ldg(a.Hz + c - P); }
  // compiled twice, as the H kernel's march
  auto march = [&](auto interior_tag) {
  constexpr bool I = decltype(interior_tag)::value;
  const bool inside = I || insidec, xs = !I && xsc, zs = !I && zsc;
  const bool XEx_ = I || XEx, XEy_ = I || XEy, XEz_ = I || XEz;
  const bool fEx = !I && fExc, fEy = !I && fEyc, fEz = !I && fEzc;
  for (int n = 0; n < np; ++n, c += P) {
    const int j = j0 + n;
    const bool ok = tma::bar_wait(full + n % RING, (n / RING) & 1, a.wait_ns);
    if (ok && inside) {
      const float* H = stage + (n % RING) * STAGE;  // Hx Hy Hz of plane j, with the halo
      const float* E = H + OWN;                     // Ex Ey Ez of the own cells
      const bool ys = in_strip(j, NY, W);
      const size_t mx = ((size_t)k * NY + j) * (2 * W) + xsi;
      const size_t my = ((size_t)k * (2 * W) + (ys ? strip_idx(j, NY, W) : 0)) * P + i;
      const size_t mz = ((size_t)zsi * NY + j) * P + i;
      const float* yt = H + YTB + (j & 3);  // rows ik ad b ikh adh bh of the y table
      const float ikyh = yt[12], adyh = yt[16], byh = yt[20];
      const float* Y = H + PSI;             // dHz_dy, dHx_dy of this plane (y strips)
      const float hx = H[hc], hy = H[FH + hc], hz = H[2 * FH + hc];
      float ex = E[oc], ey = E[OWN3 / 3 + oc], ez = E[2 * (OWN3 / 3) + oc];
      if (XEx_ && j >= 1 && j <= NY - 2) {  // :971-984
        const float d1 = hz - phz;  // dHz/dy
        float v1 = d1 * ikyh;
        if (ys) { const float m = byh * Y[oc] + adyh * d1; mHz_y_[my] = m; v1 += m; }
        const float d2 = H[FH + hc - VW] - hy;  // dHy/dz
        float v2 = d2 * ikz;
        if (zs) { const float m = bz * mHy_z_[mz] + adz * d2; mHy_z_[mz] = m; v2 += m; }
        ex = caX * ex + cbX * (v1 + v2);
      }
      if (XEy_ && j <= NY - 2) {  // :988-1007
        const float d1 = H[2 * FH + hc - 1] - hz;  // dHz/dx
        float v1 = d1 * ikxh;
        if (xs) { const float m = bxh * mHz_x_[mx] + adxh * d1; mHz_x_[mx] = m; v1 += m; }
        const float d2 = hx - H[hc - VW];  // dHx/dz
        float v2 = d2 * ikzh;
        if (zs) { const float m = bzh * mHx_z_[mz] + adzh * d2; mHx_z_[mz] = m; v2 += m; }
        ey = caY * ey + cbY * (v1 + v2);
      }
      if (XEz_ && j >= 1 && j <= NY - 2) {  // :1015-1029
        const float d1 = phx - hx;  // dHx/dy
        float v1 = d1 * ikyh;
        if (ys) { const float m = byh * Y[BZ * BX + oc] + adyh * d1; mHx_y_[my] = m; v1 += m; }
        const float d2 = hy - H[FH + hc - 1];  // dHy/dx
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
      phx = hx;
      phz = hz;
    }
    if (!__syncthreads_and(ok)) {
      if (tid == 0) em25_wait_failed(a, full, n, np);
      break;
    }
    if (tid == 0 && n + RING < np) {
      tma::fence_async_smem();
      issue(n + RING);
    }
  }
  };
  if (interior) march(std::true_type{});
  else march(std::false_type{});
  block_norm_to_slot(norm, a.io.slots, slot);
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
  em25_h_tma_kernel<<<L.grid, L.block, RING * STAGE * sizeof(float) + tma::kStageSlack, s>>>(a, rel);
}

void em25_half2(const Em25Args& a, const Launch& L, int rel, cudaStream_t s) {
  em25_e_tma_kernel<<<L.grid, L.block, RING * STAGE * sizeof(float) + tma::kStageSlack, s>>>(a, rel);
}

bool em25_make_maps(Em25Args& a, size_t field_stride, const float* ytab) {
  if (!(encode_field_map(&a.tm_halo, a.Ex, a.NX, a.NY, a.NZ, a.P, field_stride, 6, VW, VH, 3) &&
        encode_field_map(&a.tm_own, a.Ex, a.NX, a.NY, a.NZ, a.P, field_stride, 6, BX, BZ, 3)))
    return false;
  // the y-strip memory variables (layout [k][2W][P]) each kernel reads: two arrays
  auto ypsi = [&](CUtensorMap* m, float* m0, float* m1) {
    const size_t d = (size_t)((char*)m1 - (char*)m0);
    if (d % 16) return false;
    const cuuint64_t dims[4] = {(cuuint64_t)a.NX, (cuuint64_t)(2 * a.W), (cuuint64_t)a.NZ, 2};
    const cuuint64_t strides[3] = {(cuuint64_t)a.P * 4, (cuuint64_t)2 * a.W * a.P * 4, (cuuint64_t)d};
    const cuuint32_t box[4] = {BX, 1, BZ, 2};
    return encode_tiled(m, m0, 4, dims, strides, box);
  };
  if (!ypsi(&a.tm_ypsi_e, a.mEz_y, a.mEx_y) || !ypsi(&a.tm_ypsi_h, a.mHz_y, a.mHx_y)) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)axis_stride(a.NY), 6};
  const cuuint64_t strides[1] = {(cuuint64_t)axis_stride(a.NY) * 4};
  const cuuint32_t box[2] = {4, 6};
  return encode_tiled(&a.tm_ytab, (void*)ytab, 2, dims, strides, box);
}

void em25_finalize(const Em25Args& a, int t_last, cudaStream_t s) {
  dim3 b(32, 8), g((a.NX + 31) / 32, (a.NZ + 7) / 8);
  em25_hfaces_kernel<<<g, b, 0, s>>>(a);
  em25_finalize_kernel<<<1, 256, 0, s>>>(a, t_last);
}

}  // namespace sfd
