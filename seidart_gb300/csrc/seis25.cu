// seismic25 (legacy/fortran/seismicfdtd.f95:388-949): 2.5-D anisotropic
// velocity-stress scheme on (NX, NY, NZ) with y-invariant stiffness C(x, z).
//
// Each thread owns one (x, z) column and marches along y, so the 33 averaged
// stiffness values the four stress loops need at that column (formed on the
// host in FP64, y-invariant) and the three averaged densities of the
// velocity loops are read once per column segment instead of once per cell.
//   half1: the four stress loops (:616-678 sigmaxx/yy/zz, :681-725 sigmaxy,
//          :728-771 sigmaxz, :774-815 sigmayz).  The nine velocity-gradient
//          memory variables are shared by the loops in the Fortran and
//          advance once per loop that visits a cell, in loop order; each
//          thread applies the same sequence in registers.  The two
//          derivatives :701-707 leave unscaled are kept as written.  The
//          coefficient pairs of :657 (c16 (dvx_dy + dvz_dy)) and :766 (c45
//          (dvx_dz + dvz_dx)) are kept with the legacy quirks (a.legacy);
//          corrected physics (the default) uses the Voigt pairs c16 (dvx_dy +
//          dvy_dx) and c45 (dvy_dz + dvz_dy).  A stress source is added at its
//          cell after the four loops.
//   half2: vx, vy (:821-870) and vz (:872-896) with the stress-gradient
//          memory variables, optional attenuation v <- v (1 - gamma), the
//          source (:898-900), the six Dirichlet faces (:903-925) and the norm.
//
// Each block (32 x BZ columns, one y segment) streams its y planes through a
// ring of RING shared-memory stages, each filled by cp.async.bulk.tensor
// copies that one thread issues RING - 2 planes ahead and every thread waits
// for on the stage's mbarrier:
//   stress kernel:   the three velocities of the plane with a one-cell halo
//                    (x from i0 - 4, so the box starts on a 16-byte boundary;
//                    rows k0 - 1 .. k0 + BZ), and the six stresses of the
//                    block's own cells;
//   velocity kernel: the six stresses with the halo, the three velocities of
//                    the own cells.
// The plane after the segment is staged too (its velocities or stresses only)
// for the y+ differences; the y- values are carried in registers.  A step
// needs its plane and the next, so RING - 2 planes stay in flight while it
// computes; the memory variables (strips only) and the results go through
// plain loads and stores.  Boxes reaching past the grid read zeros, the
// values the Fortran's loop bounds leave there.  Staging replaced a plain
// y-march whose every step waited a memory round trip (0.682 against 0.587
// ms per step on the 630 x 70 x 330 grid).
#include <type_traits>
#include "sfd_solvers.h"
#include "tma.cuh"

namespace sfd {

namespace {

constexpr int BX = 32, BZ = 4;

// Resident blocks per SM the two kernels are compiled for (registers per
// thread = 65536 / (128 x blocks)); build-time tunables, the defaults the
// measured best on the 630 x 70 x 330 grid (the stress kernel spills at 5).
#ifndef SEIS25_STRESS_BLOCKS
#define SEIS25_STRESS_BLOCKS 4
#endif
#ifndef SEIS25_VELOCITY_BLOCKS
#define SEIS25_VELOCITY_BLOCKS 6
#endif

constexpr int CSTRIDE = 44;            // floats per thread of the stiffness table: 11 float4 slots (odd: no bank conflicts)
constexpr int HX = 4;                  // x halo of the staged tiles (16 bytes)
constexpr int VW = BX + 2 * HX;        // 40 floats per staged row
constexpr int VH = BZ + 2;             // rows k0 - 1 .. k0 + BZ
constexpr int RING = 4;                // staged planes per block
constexpr int HALO3 = 3 * VH * VW;     // velocities with the halo
constexpr int HALO6 = 6 * VH * VW;     // stresses with the halo
constexpr int OWN3 = 3 * BZ * BX;
constexpr int OWN6 = 6 * BZ * BX;
constexpr int YT = 24;                 // the y table around the plane: 6 rows x 4 entries from j & ~3
// stress stage: velocities with the halo, own stresses, y-strip memory variables, y table
constexpr int S_OWN = 736;             // 128-byte aligned after the halo
constexpr int S_PSI = S_OWN + OWN6;
constexpr int S_YT = S_PSI + OWN3;
constexpr int S_STAGE = S_YT + 32;     // 7680 bytes
// velocity stage: stresses with the halo, own velocities, y-strip memory variables, y table
constexpr int V_OWN = HALO6;
constexpr int V_PSI = V_OWN + OWN3;
constexpr int V_YT = V_PSI + OWN3;
constexpr int V_STAGE = V_YT + 32;     // 8960 bytes
static_assert(S_OWN >= HALO3 && (S_OWN * 4) % 128 == 0 && (S_PSI * 4) % 128 == 0 && (S_YT * 4) % 128 == 0 &&
                  (S_STAGE * 4) % 128 == 0, "stage alignment");
static_assert((V_OWN * 4) % 128 == 0 && (V_PSI * 4) % 128 == 0 && (V_YT * 4) % 128 == 0 && (V_STAGE * 4) % 128 == 0,
              "stage alignment");

// Whether every column of the block at (i0, k0) lies off the x and z CPML
// strips and off the boundary planes (1 <= i <= NX - 2, 1 <= k <= NZ - 2).
__device__ __forceinline__ bool block_interior(int i0, int k0, int NX, int NZ, int W) {
  return i0 >= max(W, 1) && i0 + BX - 1 <= min(NX - W - 1, NX - 2) && k0 >= max(W, 1) &&
         k0 + BZ - 1 <= min(NZ - W - 1, NZ - 2);
}

// Records a wait that ran out and lets the copies this block already issued
// land (each again within the limit) before its shared memory is released.
__device__ void staged_wait_failed(const Seis25Args& a, uint64_t* full, int n, int np) {
  atomicExch(const_cast<int*>(&a.io.ctl->err), 1);
  const int issued = min(np, n + RING);
  for (int m = n; m < issued; ++m) tma::bar_wait(full + m % RING, (m / RING) & 1, a.wait_ns);
}

__global__ void __launch_bounds__(BX * BZ, SEIS25_STRESS_BLOCKS)
    seis25_stress_tma_kernel(const __grid_constant__ Seis25Args a, int rel) {
  extern __shared__ __align__(128) unsigned char stage_raw[];
  float* const stage = tma::aligned_stage(stage_raw);
  __shared__ __align__(8) uint64_t full[RING];
  __shared__ __align__(16) float sC[CSTRIDE * BX * BZ];
  const Ctl* ctl = a.io.ctl;
  const int t = ctl->base + rel;
  if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && t > ctl->run_start) {
    const float* ch[3] = {a.vx, a.vy, a.vz};
    gather_receivers<3>(a.io.rec, a.io.nrec, a.io.traces, t - 1, ch, a.P, a.NY, true);
  }
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * BX + tx;
  const int i0 = blockIdx.x * BX, k0 = blockIdx.y * BZ;
  const int NX = a.NX, NY = a.NY, NZ = a.NZ, P = a.P, W = a.W;
  const int seg = (NY + a.ysplit - 1) / a.ysplit;
  const int j0 = blockIdx.z * seg, j1 = min(NY, j0 + seg);
  if (j0 >= j1) return;  // the whole block
  const int np = min(NY, j1 + 1) - j0;
  if (tid == 0) {
    for (int q = 0; q < RING; ++q) tma::bar_init(full + q, 1);
    tma::fence_bar_init();
  }
  __syncthreads();
  auto issue = [&](int n) {  // plane j0 + n into its stage (one thread)
    float* st = stage + (n % RING) * S_STAGE;
    uint64_t* bar = full + n % RING;
    const int j = j0 + n;
    const bool own = j < j1, ys = own && in_strip(j, NY, W);
    tma::bar_arrive_expect(bar, (HALO3 + (own ? OWN6 + YT : 0) + (ys ? OWN3 : 0)) * 4u + a.stall_tx);
    tma::load_4d(st, &a.tm_vhalo, bar, i0 - HX, j, k0 - 1, 0);
    if (own) {
      tma::load_4d(st + S_OWN, &a.tm_sown, bar, i0, j, k0, 3);
      tma::load_2d(st + S_YT, &a.tm_ytab, bar, j & ~3, 0);
    }
    if (ys) tma::load_4d(st + S_PSI, &a.tm_ypsi_v, bar, i0, strip_idx(j, NY, W), k0, 0);
  };
  if (tid == 0)
    for (int n = 0; n < min(RING, np); ++n) issue(n);

  const int i = i0 + tx, k = k0 + ty;
  const bool inside = i < NX && k < NZ;
  const bool L1c = inside && (k >= 1) && (i <= NX - 2);
  const bool L2c = inside && (k >= 1) && (i >= 1);
  const bool L3c = inside && (k <= NZ - 2) && (i >= 1);
  const bool L4c = inside && (k <= NZ - 2) && (i <= NX - 2);
  const bool activec = L1c || L2c || L3c || L4c;
  const int ic = inside ? i : 0, kc = inside ? k : 0;
  // the column's 33 stiffness averages, each thread's in its own row of
  // CSTRIDE floats: a loop's coefficients start on a 16-byte boundary and
  // are read back four at a time (slots 0-14 loop 1, 16-21 loop 2, 24-29
  // loop 3, 32-37 loop 4)
  float* const cs = sC + tid * CSTRIDE;
  {
    const size_t cpl = (size_t)NZ * P, cpc = (size_t)kc * P + ic;
    auto cf = [&](int q, bool on) { return on ? __ldg(a.C + q * cpl + cpc) : 0.0f; };
#pragma unroll
    for (int q = 0; q < 15; ++q) cs[q] = cf(q, L1c);
#pragma unroll
    for (int q = 15; q < 21; ++q) cs[q + 1] = cf(q, L2c);
#pragma unroll
    for (int q = 21; q < 27; ++q) cs[q + 3] = cf(q, L3c);
#pragma unroll
    for (int q = 27; q < 33; ++q) cs[q + 5] = cf(q, L4c);
  }
  const uint32_t cs_addr = tma::smem_addr(cs);
  // four coefficients from shared memory at each use (held in registers for
  // the whole march they would cap the kernel's occupancy)
  auto C4 = [&](int g) -> float4 {
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"(cs_addr + 16 * g));
    return v;
  };

  const bool xsc = inside && in_strip(i, NX, W), zsc = inside && in_strip(k, NZ, W);
  const int xsi = xsc ? strip_idx(i, NX, W) : 0;
  const int zsi = zsc ? strip_idx(k, NZ, W) : 0;
  const float ikx = a.X.ik[ic], ikxh = a.X.ikh[ic], adx = a.X.ad[ic], adxh = a.X.adh[ic];
  const float bx = a.X.b[ic], bxh = a.X.bh[ic];
  const float ikz = a.Z.ik[kc], ikzh = a.Z.ikh[kc], adz = a.Z.ad[kc], adzh = a.Z.adh[kc];
  const float bz = a.Z.b[kc], bzh = a.Z.bh[kc];
  const bool interior = block_interior(i0, k0, NX, NZ, W);
  float* __restrict__ SXX = a.sxx;
  float* __restrict__ SYY = a.syy;
  float* __restrict__ SZZ = a.szz;
  float* __restrict__ SXY = a.sxy;
  float* __restrict__ SXZ = a.sxz;
  float* __restrict__ SYZ = a.syz;
  float* __restrict__ MVXX = a.m_vx_x;
  float* __restrict__ MVYX = a.m_vy_x;
  float* __restrict__ MVZX = a.m_vz_x;
  float* __restrict__ MVXY = a.m_vx_y;
  float* __restrict__ MVYY = a.m_vy_y;
  float* __restrict__ MVZY = a.m_vz_y;
  float* __restrict__ MVXZ = a.m_vx_z;
  float* __restrict__ MVYZ = a.m_vy_z;
  float* __restrict__ MVZZ = a.m_vz_z;
  size_t c = ((size_t)kc * NY + j0) * P + ic;
  float pvx = 0.f, pvy = 0.f, pvz = 0.f;
  if (activec && j0 >= 1) { pvx = __ldg(a.vx + c - P); pvy = __ldg(a.vy + c - P); pvz = __ldg(a.vz + c - P); }
  const int hc = (ty + 1) * VW + tx + HX;  // own cell in a halo tile
  const int oc = ty * BX + tx;             // own cell in an own-cells tile
  // The march, compiled twice: for blocks whose columns all lie off the x
  // and z strips and the boundary planes (I: every loop updates every
  // column, no x or z memory variables) and for the others.
  auto march = [&](auto interior_tag) {
  constexpr bool I = decltype(interior_tag)::value;
  const bool xs = !I && xsc, zs = !I && zsc;
  const bool L1 = I || L1c, L2 = I || L2c, L3 = I || L3c, L4 = I || L4c, active = I || activec;
  for (int n = 0; n < j1 - j0; ++n, c += P) {
    const int j = j0 + n;
    const bool more = n + 1 < np;
    bool ok = tma::bar_wait(full + n % RING, (n / RING) & 1, a.wait_ns);
    if (more && ok) ok = tma::bar_wait(full + (n + 1) % RING, ((n + 1) / RING) & 1, a.wait_ns);
    if (ok && active) {
      const float* V = stage + (n % RING) * S_STAGE;
      const float* Vn = stage + ((n + 1) % RING) * S_STAGE;
      const float* S = V + S_OWN;
      constexpr int F = VH * VW;
      const float cvx = V[hc], cvy = V[F + hc], cvz = V[2 * F + hc];
      const float nvx = more ? Vn[hc] : 0.f, nvy = more ? Vn[F + hc] : 0.f, nvz = more ? Vn[2 * F + hc] : 0.f;
      const float xmx = V[hc - 1], xmy = V[F + hc - 1], xmz = V[2 * F + hc - 1];
      const float xpx = V[hc + 1], xpy = V[F + hc + 1], xpz = V[2 * F + hc + 1];
      const float zmx = V[hc - VW], zmy = V[F + hc - VW], zmz = V[2 * F + hc - VW];
      const float zpx = V[hc + VW], zpy = V[F + hc + VW], zpz = V[2 * F + hc + VW];
      const bool ys = in_strip(j, NY, W);
      const size_t mx = ((size_t)k * NY + j) * (2 * W) + xsi;
      const size_t my = ((size_t)k * (2 * W) + (ys ? strip_idx(j, NY, W) : 0)) * P + i;
      const size_t mz = ((size_t)zsi * NY + j) * P + i;
      float mvxx = 0, mvyx = 0, mvzx = 0, mvxy = 0, mvyy = 0, mvzy = 0, mvxz = 0, mvyz = 0, mvzz = 0;
      if (xs) { mvxx = MVXX[mx]; mvyx = MVYX[mx]; mvzx = MVZX[mx]; }
      if (ys) { const float* Y = V + S_PSI; mvxy = Y[oc]; mvyy = Y[OWN3 / 3 + oc]; mvzy = Y[2 * (OWN3 / 3) + oc]; }
      if (zs) { mvxz = MVXZ[mz]; mvyz = MVYZ[mz]; mvzz = MVZZ[mz]; }
      const bool l1 = L1 && j >= 1, l2 = L2 && j <= NY - 2, l3 = L3 && j >= 1, l4 = L4 && j <= NY - 2;
      const float* yt = V + S_YT + (j & 3);  // rows ik ad b ikh adh bh of the y table
      const float iky = yt[0], ady = yt[4], by = yt[8], ikyh = yt[12], adyh = yt[16], byh = yt[20];
      if (l1) {  // sigmaxx, sigmayy, sigmazz: x+, y-, z- differences (:616-678)
        const float dxx = xpx - cvx, dyx = xpy - cvy, dzx = xpz - cvz;
        const float dyy = cvy - pvy, dxy = cvx - pvx, dzy = cvz - pvz;
        const float dzz = cvz - zmz, dxz = cvx - zmx, dyz = cvy - zmy;
        if (xs) { mvxx = bxh * mvxx + adxh * dxx; mvyx = bxh * mvyx + adxh * dyx; mvzx = bxh * mvzx + adxh * dzx; }
        if (ys) { mvyy = by * mvyy + ady * dyy; mvxy = by * mvxy + ady * dxy; mvzy = by * mvzy + ady * dzy; }
        if (zs) { mvzz = bz * mvzz + adz * dzz; mvxz = bz * mvxz + adz * dxz; mvyz = bz * mvyz + adz * dyz; }
        const float vxx = dxx * ikxh + mvxx, vyx = dyx * ikxh + mvyx, vzx = dzx * ikxh + mvzx;
        const float vyy = dyy * iky + mvyy, vxy = dxy * iky + mvxy, vzy = dzy * iky + mvzy;
        const float vzz = dzz * ikz + mvzz, vxz = dxz * ikz + mvxz, vyz = dyz * ikz + mvyz;
        const float4 c0 = C4(0), c1 = C4(1), c2 = C4(2), c3 = C4(3);  // C(0) .. C(14)
        SXX[c] = S[oc] + (c0.x * vxx + c0.y * vyy + c0.z * vzz + c0.w * (vyz + vzy) + c1.x * (vxz + vzx) +
                          c1.y * (a.legacy ? vxy + vzy : vxy + vyx));  // Q4, :657
        SYY[c] = S[OWN6 / 6 + oc] + (c0.y * vxx + c1.z * vyy + c1.w * vzz + c2.x * (vyz + vzy) +
                                     c2.y * (vxz + vzx) + c2.z * (vyx + vxy));
        SZZ[c] = S[2 * (OWN6 / 6) + oc] + (c0.z * vxx + c1.w * vyy + c2.w * vzz + c3.x * (vyz + vzy) +
                                           c3.y * (vxz + vzx) + c3.z * (vyx + vxy));
      }
      if (l2) {  // sigmaxy: x-, y+, z- (:681-725)
        const float dxx = cvx - xmx, dyx = cvy - xmy, dzx = cvz - xmz;
        const float dyy = nvy - cvy, dxy = nvx - cvx, dzy = nvz - cvz;
        const float dzz = cvz - zmz, dxz = cvx - zmx, dyz = cvy - zmy;
        if (xs) { mvxx = bx * mvxx + adx * dxx; mvyx = bx * mvyx + adx * dyx; mvzx = bx * mvzx + adx * dzx; }
        if (ys) { mvyy = byh * mvyy + adyh * dyy; mvxy = byh * mvxy + adyh * dxy; mvzy = byh * mvzy + adyh * dzy; }
        if (zs) { mvzz = bzh * mvzz + adzh * dzz; mvxz = bzh * mvxz + adzh * dxz; mvyz = bzh * mvyz + adzh * dyz; }
        const float vxx = dxx * ikx + mvxx, vyx = dyx * ikx + mvyx;
        const float vyy = dyy * ikyh + mvyy, vxy = dxy * ikyh + mvxy, vzy = dzy * ikyh + mvzy;
        const float vzz = dzz * ikzh + mvzz, vyz = dyz * ikzh + mvyz;
        const float vzx = dzx * a.idx, vxz = dxz * a.idz;  // left unscaled, :701-707
        const float4 c4 = C4(4), c5 = C4(5);  // C(15) .. C(20)
        SXY[c] = S[3 * (OWN6 / 6) + oc] + (c4.x * vxx + c4.y * vyy + c4.z * vzz + c4.w * (vzy + vyz) +
                                           c5.x * (vzx + vxz) + c5.y * (vyx + vxy));
      }
      if (l3) {  // sigmaxz: x-, y-, z+ (:728-771)
        const float dxx = cvx - xmx, dyx = cvy - xmy, dzx = cvz - xmz;
        const float dyy = cvy - pvy, dzy = cvz - pvz, dxy = cvx - pvx;
        const float dzz = zpz - cvz, dxz = zpx - cvx, dyz = zpy - cvy;
        if (xs) { mvxx = bx * mvxx + adx * dxx; mvyx = bx * mvyx + adx * dyx; mvzx = bx * mvzx + adx * dzx; }
        if (ys) { mvyy = by * mvyy + ady * dyy; mvxy = by * mvxy + ady * dxy; mvzy = by * mvzy + ady * dzy; }
        if (zs) { mvzz = bzh * mvzz + adzh * dzz; mvxz = bzh * mvxz + adzh * dxz; mvyz = bzh * mvyz + adzh * dyz; }
        const float vxx = dxx * ikx + mvxx, vyx = dyx * ikx + mvyx, vzx = dzx * ikx + mvzx;
        const float vyy = dyy * iky + mvyy, vxy = dxy * iky + mvxy, vzy = dzy * iky + mvzy;
        const float vzz = dzz * ikzh + mvzz, vxz = dxz * ikzh + mvxz, vyz = dyz * ikzh + mvyz;
        const float4 c6 = C4(6), c7 = C4(7);  // C(21) .. C(26)
        SXZ[c] = S[4 * (OWN6 / 6) + oc] + (c6.x * vxx + c6.y * vyy + c6.z * vzz +
                                           c6.w * (a.legacy ? vxz + vzx : vyz + vzy) +  // Q4, :766
                                           c7.x * (vxz + vzx) + c7.y * (vxy + vyx));
      }
      if (l4) {  // sigmayz: x+, y+, z+ (:774-815)
        const float dxx = xpx - cvx, dyx = xpy - cvy, dzx = xpz - cvz;
        const float dyy = nvy - cvy, dxy = nvx - cvx, dzy = nvz - cvz;
        const float dzz = zpz - cvz, dxz = zpx - cvx, dyz = zpy - cvy;
        if (xs) { mvxx = bxh * mvxx + adxh * dxx; mvyx = bxh * mvyx + adxh * dyx; mvzx = bxh * mvzx + adxh * dzx; }
        if (ys) { mvyy = byh * mvyy + adyh * dyy; mvxy = byh * mvxy + adyh * dxy; mvzy = byh * mvzy + adyh * dzy; }
        if (zs) { mvzz = bzh * mvzz + adzh * dzz; mvxz = bzh * mvxz + adzh * dxz; mvyz = bzh * mvyz + adzh * dyz; }
        const float vxx = dxx * ikxh + mvxx, vyx = dyx * ikxh + mvyx, vzx = dzx * ikxh + mvzx;
        const float vyy = dyy * ikyh + mvyy, vxy = dxy * ikyh + mvxy, vzy = dzy * ikyh + mvzy;
        const float vzz = dzz * ikzh + mvzz, vxz = dxz * ikzh + mvxz, vyz = dyz * ikzh + mvyz;
        const float4 c8 = C4(8), c9 = C4(9);  // C(27) .. C(32)
        SYZ[c] = S[5 * (OWN6 / 6) + oc] + (c8.x * vxx + c8.y * vyy + c8.z * vzz + c8.w * (vyz + vzy) +
                                           c9.x * (vxz + vzx) + c9.y * (vyx + vxy));
      }
      if (xs) { MVXX[mx] = mvxx; MVYX[mx] = mvyx; MVZX[mx] = mvzx; }
      if (ys) { MVXY[my] = mvxy; MVYY[my] = mvyy; MVZY[my] = mvzy; }
      if (zs) { MVXZ[mz] = mvxz; MVYZ[mz] = mvyz; MVZZ[mz] = mvzz; }
      if (a.io.ssrc && i == a.io.si && j == a.io.sj && k == a.io.sk) {  // stress source: sigma_ij += f_ij(t) dt
        const float* f = a.io.ssrc + t;
        const int ns = a.io.nstep;
        SXX[c] += f[0];
        SYY[c] += f[ns];
        SZZ[c] += f[2 * ns];
        SXY[c] += f[3 * ns];
        SXZ[c] += f[4 * ns];
        SYZ[c] += f[5 * ns];
      }
      pvx = cvx; pvy = cvy; pvz = cvz;
    }
    if (!__syncthreads_and(ok)) {  // every thread is done with plane n (or a wait ran out)
      if (tid == 0) staged_wait_failed(a, full, n, np);
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

__global__ void __launch_bounds__(BX * BZ, SEIS25_VELOCITY_BLOCKS)
    seis25_velocity_tma_kernel(const __grid_constant__ Seis25Args a, int rel) {
  extern __shared__ __align__(128) unsigned char stage_raw[];
  float* const stage = tma::aligned_stage(stage_raw);
  __shared__ __align__(8) uint64_t full[RING];
  const int t = a.io.ctl->base + rel;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * BX + tx;
  const int i0 = blockIdx.x * BX, k0 = blockIdx.y * BZ;
  const int NX = a.NX, NY = a.NY, NZ = a.NZ, P = a.P, W = a.W;
  const int seg = (NY + a.ysplit - 1) / a.ysplit;
  const int j0 = blockIdx.z * seg, j1 = min(NY, j0 + seg);
  float norm = 0.0f;
  const int slot = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
  if (j0 >= j1) {  // the whole block
    block_norm_to_slot(norm, a.io.slots, slot);
    return;
  }
  const int np = min(NY, j1 + 1) - j0;
  if (tid == 0) {
    for (int q = 0; q < RING; ++q) tma::bar_init(full + q, 1);
    tma::fence_bar_init();
  }
  __syncthreads();
  auto issue = [&](int n) {
    float* st = stage + (n % RING) * V_STAGE;
    uint64_t* bar = full + n % RING;
    const int j = j0 + n;
    const bool own = j < j1, ys = own && in_strip(j, NY, W);
    tma::bar_arrive_expect(bar, (HALO6 + (own ? OWN3 + YT : 0) + (ys ? OWN3 : 0)) * 4u + a.stall_tx);
    tma::load_4d(st, &a.tm_shalo, bar, i0 - HX, j, k0 - 1, 3);
    if (own) {
      tma::load_4d(st + V_OWN, &a.tm_vown, bar, i0, j, k0, 0);
      tma::load_2d(st + V_YT, &a.tm_ytab, bar, j & ~3, 0);
    }
    if (ys) tma::load_4d(st + V_PSI, &a.tm_ypsi_s, bar, i0, strip_idx(j, NY, W), k0, 0);
  };
  if (tid == 0)
    for (int n = 0; n < min(RING, np); ++n) issue(n);

  const int i = i0 + tx, k = k0 + ty;
  const bool insidec = i < NX && k < NZ;
  const int ic = insidec ? i : 0, kc = insidec ? k : 0;
  const bool Vx = insidec && (k >= 1) && (i >= 1);
  const bool Vy = insidec && (k >= 1) && (i <= NX - 2);
  const bool Vz = insidec && (k <= NZ - 2) && (i <= NX - 2);
  const size_t pc = (size_t)kc * P + ic;
  const size_t p2 = (size_t)NZ * P;
  const float dtrx = Vx ? a.dtr[pc] : 0.f, dtry = Vy ? a.dtr[p2 + pc] : 0.f, dtrz = Vz ? a.dtr[2 * p2 + pc] : 0.f;
  float gx = 1.f, gy = 1.f, gz = 1.f;
  if (a.atten && insidec) { gx = a.gp[pc]; gy = a.gp[p2 + pc]; gz = a.gp[2 * p2 + pc]; }
  const bool xsc = insidec && in_strip(i, NX, W), zsc = insidec && in_strip(k, NZ, W);
  const int xsi = xsc ? strip_idx(i, NX, W) : 0;
  const int zsi = zsc ? strip_idx(k, NZ, W) : 0;
  const float ikx = a.X.ik[ic], ikxh = a.X.ikh[ic], adx = a.X.ad[ic], adxh = a.X.adh[ic];
  const float bx = a.X.b[ic], bxh = a.X.bh[ic];
  const float ikz = a.Z.ik[kc], ikzh = a.Z.ikh[kc], adz = a.Z.ad[kc], adzh = a.Z.adh[kc];
  const float bz = a.Z.b[kc], bzh = a.Z.bh[kc];
  const bool xfacec = (i == 0) || (i == NX - 1) || (k == 0) || (k == NZ - 1);
  const bool interior = block_interior(i0, k0, NX, NZ, W);
  float* __restrict__ VX = a.vx;
  float* __restrict__ VY = a.vy;
  float* __restrict__ VZ = a.vz;
  float* __restrict__ MSXXX = a.m_sxx_x;
  float* __restrict__ MSXYY = a.m_sxy_y;
  float* __restrict__ MSXZZ = a.m_sxz_z;
  float* __restrict__ MSXYX = a.m_sxy_x;
  float* __restrict__ MSYYY = a.m_syy_y;
  float* __restrict__ MSYZZ = a.m_syz_z;
  float* __restrict__ MSXZX = a.m_sxz_x;
  float* __restrict__ MSYZY = a.m_syz_y;
  float* __restrict__ MSZZZ = a.m_szz_z;
  size_t c = ((size_t)kc * NY + j0) * P + ic;
  float psxy = 0.f, psyz = 0.f;
  if (insidec && j0 >= 1) { psxy = __ldg(a.sxy + c - P); psyz = __ldg(a.syz + c - P); }
  const int hc = (ty + 1) * VW + tx + HX;
  const int oc = ty * BX + tx;
  constexpr int F = VH * VW;  // one field of a halo tile
  // compiled twice, as the stress kernel's march
  auto march = [&](auto interior_tag) {
  constexpr bool I = decltype(interior_tag)::value;
  const bool inside = I || insidec, xs = !I && xsc, zs = !I && zsc, xface = !I && xfacec;
  const bool Vxm = I || Vx, Vym = I || Vy, Vzm = I || Vz;
  for (int n = 0; n < j1 - j0; ++n, c += P) {
    const int j = j0 + n;
    const bool more = n + 1 < np;
    bool ok = tma::bar_wait(full + n % RING, (n / RING) & 1, a.wait_ns);
    if (more && ok) ok = tma::bar_wait(full + (n + 1) % RING, ((n + 1) / RING) & 1, a.wait_ns);
    if (ok && inside) {
      const float* S = stage + (n % RING) * V_STAGE;  // sxx syy szz sxy sxz syz with the halo
      const float* Sn = stage + ((n + 1) % RING) * V_STAGE;
      const float* V = S + V_OWN;
      const float csxx = S[hc], csyy = S[F + hc], cszz = S[2 * F + hc];
      const float csxy = S[3 * F + hc], csxz = S[4 * F + hc], csyz = S[5 * F + hc];
      const float nsyy = more ? Sn[F + hc] : 0.f;
      const bool ys = in_strip(j, NY, W);
      const size_t mx = ((size_t)k * NY + j) * (2 * W) + xsi;
      const size_t my = ((size_t)k * (2 * W) + (ys ? strip_idx(j, NY, W) : 0)) * P + i;
      const size_t mz = ((size_t)zsi * NY + j) * P + i;
      const float* yt = S + V_YT + (j & 3);  // rows ik ad b ikh adh bh of the y table
      const float iky = yt[0], ady = yt[4], by = yt[8], ikyh = yt[12], adyh = yt[16], byh = yt[20];
      float vx = V[oc], vy = V[OWN3 / 3 + oc], vz = V[2 * (OWN3 / 3) + oc];
      const bool ux = Vxm && j >= 1, uy = Vym && j <= NY - 2, uz = Vzm && j >= 1;
      float m1x = 0.f, m1y = 0.f, m1z = 0.f, m2x = 0.f, m2y = 0.f, m2z = 0.f, m3x = 0.f, m3y = 0.f, m3z = 0.f;
      if (xs) {
        if (ux) m1x = MSXXX[mx];
        if (uy) m2x = MSXYX[mx];
        if (uz) m3x = MSXZX[mx];
      }
      if (ys) {  // staged: syy_y sxy_y syz_y
        const float* Y = S + V_PSI;
        m2y = Y[oc];
        m1y = Y[OWN3 / 3 + oc];
        m3y = Y[2 * (OWN3 / 3) + oc];
      }
      if (zs) {
        if (ux) m1z = MSXZZ[mz];
        if (uy) m2z = MSYZZ[mz];
        if (uz) m3z = MSZZZ[mz];
      }
      if (ux) {  // :821-845
        const float d1 = csxx - S[hc - 1], d2 = csxy - psxy, d3 = csxz - S[4 * F + hc - VW];
        float v1 = d1 * ikx, v2 = d2 * iky, v3 = d3 * ikz;
        if (xs) { const float m = bx * m1x + adx * d1; MSXXX[mx] = m; v1 += m; }
        if (ys) { const float m = by * m1y + ady * d2; MSXYY[my] = m; v2 += m; }
        if (zs) { const float m = bz * m1z + adz * d3; MSXZZ[mz] = m; v3 += m; }
        vx = vx * gx + (v1 + v2 + v3) * dtrx;
      }
      if (uy) {  // :847-869
        const float d1 = S[3 * F + hc + 1] - csxy, d2 = nsyy - csyy, d3 = csyz - S[5 * F + hc - VW];
        float v1 = d1 * ikxh, v2 = d2 * ikyh, v3 = d3 * ikz;
        if (xs) { const float m = bxh * m2x + adxh * d1; MSXYX[mx] = m; v1 += m; }
        if (ys) { const float m = byh * m2y + adyh * d2; MSYYY[my] = m; v2 += m; }
        if (zs) { const float m = bz * m2z + adz * d3; MSYZZ[mz] = m; v3 += m; }
        vy = vy * gy + (v1 + v2 + v3) * dtry;
      }
      if (uz) {  // :872-896
        const float d1 = S[4 * F + hc + 1] - csxz, d2 = csyz - psyz, d3 = S[2 * F + hc + VW] - cszz;
        float v1 = d1 * ikxh, v2 = d2 * iky, v3 = d3 * ikzh;
        if (xs) { const float m = bxh * m3x + adxh * d1; MSXZX[mx] = m; v1 += m; }
        if (ys) { const float m = by * m3y + ady * d2; MSYZY[my] = m; v2 += m; }
        if (zs) { const float m = bzh * m3z + adzh * d3; MSZZZ[mz] = m; v3 += m; }
        vz = vz * gz + (v1 + v2 + v3) * dtrz;
      }
      if (i == a.io.si && j == a.io.sj && k == a.io.sk) {  // :898-900
        vx += a.io.src[t];
        vy += a.io.src[a.io.nstep + t];
        vz += a.io.src[2 * a.io.nstep + t];
      }
      if (xface || j == 0 || j == NY - 1) { vx = 0.f; vy = 0.f; vz = 0.f; }  // :903-925
      VX[c] = vx;
      VY[c] = vy;
      VZ[c] = vz;
      norm = fmaxf(norm, norm_monitor(vx, vy, vz));
      psxy = csxy;
      psyz = csyz;
    }
    if (!__syncthreads_and(ok)) {
      if (tid == 0) staged_wait_failed(a, full, n, np);
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

__global__ void seis25_finalize_kernel(Seis25Args a, int t_last) {
  const float* ch[3] = {a.vx, a.vy, a.vz};
  gather_receivers<3>(a.io.rec, a.io.nrec, a.io.traces, t_last, ch, a.P, a.NY, true);
}

}  // namespace

Launch seis25_launch(const Seis25Args& a) {
  Launch L;
  L.block = dim3(BX, BZ, 1);
  L.grid = dim3((a.NX + BX - 1) / BX, (a.NZ + BZ - 1) / BZ, a.ysplit);
  L.nslots = L.grid.x * L.grid.y * L.grid.z;
  return L;
}

void seis25_half1(const Seis25Args& a, const Launch& L, int rel, cudaStream_t s) {
  seis25_stress_tma_kernel<<<L.grid, L.block, RING * S_STAGE * sizeof(float) + tma::kStageSlack, s>>>(a, rel);
}

void seis25_half2(const Seis25Args& a, const Launch& L, int rel, cudaStream_t s) {
  seis25_velocity_tma_kernel<<<L.grid, L.block, RING * V_STAGE * sizeof(float) + tma::kStageSlack, s>>>(a, rel);
}

bool seis25_make_maps(Seis25Args& a, size_t field_stride, const float* ytab) {
  // the stress kernel's static table and staging ring exceed the default 48 KB
  if (cudaFuncSetAttribute(seis25_stress_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           RING * S_STAGE * (int)sizeof(float) + tma::kStageSlack) != cudaSuccess ||
      cudaFuncSetAttribute(seis25_velocity_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           RING * V_STAGE * (int)sizeof(float) + tma::kStageSlack) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  auto make = [&](CUtensorMap* m, int bx, int bz, int nf) {
    return encode_field_map(m, a.vx, a.NX, a.NY, a.NZ, a.P, field_stride, 9, bx, bz, nf);
  };
  if (!(make(&a.tm_vhalo, VW, VH, 3) && make(&a.tm_sown, BX, BZ, 6) && make(&a.tm_shalo, VW, VH, 6) &&
        make(&a.tm_vown, BX, BZ, 3)))
    return false;
  // y-strip memory variables (layout [k][2W][P]): three equally spaced arrays per kernel
  auto ypsi = [&](CUtensorMap* m, float* m0, float* m1, float* m2) {
    const size_t d = (size_t)((char*)m1 - (char*)m0);
    if ((size_t)((char*)m2 - (char*)m1) != d || d % 16) return false;
    const cuuint64_t dims[4] = {(cuuint64_t)a.NX, (cuuint64_t)(2 * a.W), (cuuint64_t)a.NZ, 3};
    const cuuint64_t strides[3] = {(cuuint64_t)a.P * 4, (cuuint64_t)2 * a.W * a.P * 4, (cuuint64_t)d};
    const cuuint32_t box[4] = {BX, 1, BZ, 3};
    return encode_tiled(m, m0, 4, dims, strides, box);
  };
  if (!ypsi(&a.tm_ypsi_v, a.m_vx_y, a.m_vy_y, a.m_vz_y) || !ypsi(&a.tm_ypsi_s, a.m_syy_y, a.m_sxy_y, a.m_syz_y))
    return false;
  // the y table: 6 rows (ik ad b ikh adh bh) of axis_stride(NY) floats
  const cuuint64_t dims[2] = {(cuuint64_t)axis_stride(a.NY), 6};
  const cuuint64_t strides[1] = {(cuuint64_t)axis_stride(a.NY) * 4};
  const cuuint32_t box[2] = {4, 6};
  return encode_tiled(&a.tm_ytab, (void*)ytab, 2, dims, strides, box);
}

void seis25_finalize(const Seis25Args& a, int t_last, cudaStream_t s) {
  seis25_finalize_kernel<<<1, 256, 0, s>>>(a, t_last);
}

}  // namespace sfd
