// SM-resident seismic2 run: every time step of an sfd_run in one cooperative
// launch, with the whole state on chip.
//
// The grid is cut into a uniform ntx x ntz grid of tiles (Seis2ResPlan), one
// CTA per tile for the whole run.  A tile keeps, in shared memory, its five
// fields with a one-cell halo ring, its twelve coefficient planes and its
// twelve CPML memory variables (eight with the legacy quirks, where the two
// stress loops share four).  The per-cell arithmetic is that of the
// single-pass tile (fused2d.cuh: seis2_stress_cell and the per-cell velocity
// code), i.e. the loops of legacy/fortran/seismicfdtd.f95:247-379, so the
// streaming and on-chip forms give the same fields.
//
// A step is two half-steps, each followed by a halo exchange with the four
// neighbouring tiles through tagged 8-byte edge words in global memory (L2),
// as in the electromag2 on-chip run (resident2d.cu):
//   stresses (:247-312) need vx, vz one cell left, right, above and below;
//   velocities (:317-357) need sxx on the left, sxz above and on the right,
//   szz below.
// The cell warps compute a tile's perimeter cells first and write their edge
// values as soon as they are computed (row edges indexed by tile row and
// global x, column edges by tile column and global z, tag = one more than the
// reading step, two copies by the parity of the reading step).  Meanwhile
// four exchange warps, one per neighbour, poll the neighbours' words of the
// same half-step until they carry the expected tag and copy them into the
// halo ring, so the exchange overlaps the interior cells and a step needs
// two block barriers.  A poll gives up after limit_ns (%globaltimer) or when
// another tile has given up, records the failure in the control block, and
// the CTA leaves the run; the host reports SFD_ERR_TIMEOUT.  The launch is
// cooperative, so all tiles are co-resident and a correct run never reaches
// the limit.
#include <algorithm>

#include "resident_common.cuh"

namespace sfd {

using namespace res;

namespace {

constexpr int kS2ExchangeWarps = 4;
constexpr int kS2CellThreads = 256;
constexpr int kS2Threads = 32 * kS2ExchangeWarps + kS2CellThreads;
constexpr int kS2MaxTile = 128;  // tile width and height: two fields of one side fit one warp's poll

// Fields with their halo ring, coefficients, memory variables and the axis
// tables of the tile's columns and rows (floats), then the cell order
// (16-bit (row << 7) | column per cell).
size_t s2_smem(int TW, int TZ) {
  return sizeof(float) * (5 * (size_t)(TZ + 2) * (TW + 2) + 24 * (size_t)TZ * TW + 6 * (size_t)TW + 7 * (size_t)TZ) +
         2 * (((size_t)TZ * TW + 1) & ~(size_t)1);
}

// One warp: copy n words of src0 into dst0[q * st0] and, when src1 is given,
// n words of src1 into dst1[q * st1], each once its tag reads `tag`.  Each
// lane issues the loads of all its pending words before testing any.  False
// (on every lane) if the wait gave up.
__device__ __noinline__ bool fetch2(const uint2* src0, float* dst0, int st0, const uint2* src1, float* dst1, int st1,
                                    int n, unsigned tag, Ctl* ctl, unsigned long long limit_ns) {
  const int lane = threadIdx.x & 31;
  const int total = (src1 ? 2 : 1) * n;
  unsigned pending = 0;
#pragma unroll
  for (int k = 0; k < kResFetchPerLane; ++k)
    if (lane + 32 * k < total) pending |= 1u << k;
  bool ok = true;
  unsigned long long t0 = 0;
  uint2 v[kResFetchPerLane];
  for (int it = 1; pending; ++it) {
#pragma unroll
    for (int k = 0; k < kResFetchPerLane; ++k) {
      const int q = lane + 32 * k;
      if (pending & (1u << k)) v[k] = ld_vol2(q < n ? src0 + q : src1 + (q - n));
    }
#pragma unroll
    for (int k = 0; k < kResFetchPerLane; ++k) {
      const int q = lane + 32 * k;
      if ((pending & (1u << k)) && v[k].y == tag) {
        if (q < n) dst0[q * st0] = __uint_as_float(v[k].x);
        else dst1[(q - n) * st1] = __uint_as_float(v[k].x);
        pending &= ~(1u << k);
      }
    }
    if (pending && (it & 7) == 0 && !keep_polling(ctl, limit_ns, t0)) {
      ok = false;
      break;
    }
  }
  return __all_sync(0xffffffffu, ok);
}

// Edge fields: rows (indexed by tile row and global x) and columns (by tile
// column and global z).
enum : int {
  kEVxFirst = 0,  // vx, vz first row / column: read by the tile above / left
  kEVzFirst = 1,
  kEVxLast = 2,   // vx, vz last row / column: read by the tile below / right
  kEVzLast = 3,
  kESFirst = 4,   // szz first row (tile above), sxz first column (tile left)
  kESLast = 5     // sxz last row (tile below), sxx last column (tile right)
};

// DUMP: a recompute for the adjoint -- every step's state written to its
// slot, the loaded state not written back.
template <bool DUMP>
__global__ void __launch_bounds__(kS2Threads, 1) seis2_resident_kernel(const __grid_constant__ Seis2Resident a) {
  extern __shared__ __align__(16) float smem[];
  __shared__ int s_abort, s_nrec;
  __shared__ int s_rec[2 * kResMaxLocalRec];  // (receiver, halo-frame cell) pairs
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  const int ntx = a.plan.ntx, ntz = a.plan.ntz;
  const int bx = blockIdx.x % ntx, bz = blockIdx.x / ntx;
  const int x0 = a.plan.xb[bx], x1 = a.plan.xb[bx + 1], z0 = a.plan.zb[bz], z1 = a.plan.zb[bz + 1];
  const int tw = x1 - x0, tz = z1 - z0, SW = tw + 2, FS = (tz + 2) * SW, CS = tw * tz;
  const bool up = bz > 0, down = bz < ntz - 1, left = bx > 0, right = bx < ntx - 1;
  float* F = smem;         // vx vz sxx szz sxz, (tz + 2) x (tw + 2) with the halo ring
  float* C = F + 5 * FS;   // A11 A13 A15 A33 A35 B15 B35 B55 dtrx dtrz gxp gzp, tz x tw
  // m_vxx m_vzz m_vxz m_vzx m_sxx_x m_szz_z m_sxz_x m_sxz_z, then the sigmaxz
  // loop's own m2_vxx m2_vzz m2_vxz m2_vzx (corrected physics), tz x tw each
  float* M = C + 12 * CS;
  float* XT = M + 12 * CS;  // x tables at the tile's columns: ik ad b ikh adh bh, tw each
  float* ZT = XT + 6 * tw;  // z tables at the tile's rows, then q3, tz each
  unsigned short* CELL = reinterpret_cast<unsigned short*>(ZT + 7 * tz);  // cell order, see cell_at
  float* VX = F;
  float* VZ = F + FS;
  float* SXX = F + 2 * FS;
  float* SZZ = F + 3 * FS;
  float* SXZ = F + 4 * FS;
  const int tid = threadIdx.x, warp = tid >> 5;
  auto fi = [&](int lr, int lc) { return (lr + 1) * SW + lc + 1; };
  Ctl* ctl = a.io.ctl;
  const int NZp = a.r.NZp;
  auto erow = [&](int par, int f, int b) { return a.r.erow + (size_t)((par * 6 + f) * kResMaxTiles1D + b) * P; };
  auto ecol = [&](int par, int f, int b) { return a.r.ecol + (size_t)((par * 6 + f) * kResMaxTiles1D + b) * NZp; };

  // ---- load the tile: fields, the velocities of the halo ring (the
  // stresses of the ring are exchanged every step), coefficients, memory
  for (int q = tid; q < 5 * FS + 24 * CS; q += kS2Threads) smem[q] = 0.0f;
  if (tid == 0) {
    s_nrec = 0;
    s_abort = 0;
  }
  __syncthreads();
  for (int q = tid; q < FS; q += kS2Threads) {
    const int lr = q / SW - 1, lc = q % SW - 1, k = z0 + lr, i = x0 + lc;
    const bool rin = lr >= 0 && lr < tz, cin = lc >= 0 && lc < tw;
    if (k < 0 || k >= NZ || i < 0 || i >= NX || (!rin && !cin)) continue;
    const size_t g = (size_t)k * P + i;
    VX[q] = a.vx[g];
    VZ[q] = a.vz[g];
    if (rin && cin) {
      SXX[q] = a.sxx[g];
      SZZ[q] = a.szz[g];
      SXZ[q] = a.sxz[g];
    }
  }
  for (int q = tid; q < CS; q += kS2Threads) {
    const int lr = q / tw, lc = q - lr * tw, k = z0 + lr, i = x0 + lc;
    const size_t g = (size_t)k * P + i;
#pragma unroll
    for (int c = 0; c < 12; ++c) C[c * CS + q] = a.coef[c][g];
    if (in_strip(i, NX, W)) {
      const size_t mx = (size_t)k * (2 * W) + strip_idx(i, NX, W);
      M[0 * CS + q] = a.m_vxx[mx];
      M[3 * CS + q] = a.m_vzx[mx];
      M[4 * CS + q] = a.m_sxx_x[mx];
      M[6 * CS + q] = a.m_sxz_x[mx];
      if (!a.legacy) {
        M[8 * CS + q] = a.m2_vxx[mx];
        M[11 * CS + q] = a.m2_vzx[mx];
      }
    }
    if (in_strip(k, NZ, W)) {
      const size_t mz = (size_t)strip_idx(k, NZ, W) * P + i;
      M[1 * CS + q] = a.m_vzz[mz];
      M[2 * CS + q] = a.m_vxz[mz];
      M[5 * CS + q] = a.m_szz_z[mz];
      M[7 * CS + q] = a.m_sxz_z[mz];
      if (!a.legacy) {
        M[9 * CS + q] = a.m2_vzz[mz];
        M[10 * CS + q] = a.m2_vxz[mz];
      }
    }
  }
  {
    const float* xs[6] = {a.X.ik, a.X.ad, a.X.b, a.X.ikh, a.X.adh, a.X.bh};
    const float* zs[7] = {a.Z.ik, a.Z.ad, a.Z.b, a.Z.ikh, a.Z.adh, a.Z.bh, a.q3};
    for (int q = tid; q < 6 * tw; q += kS2Threads) XT[q] = xs[q / tw][x0 + q % tw];
    for (int q = tid; q < 7 * tz; q += kS2Threads) ZT[q] = zs[q / tz][z0 + q % tz];
  }
  for (int q = tid; q < a.io.nrec; q += kS2Threads) {  // receivers of this tile
    const int i = a.io.rec[3 * q], k = a.io.rec[3 * q + 2];
    if (i >= x0 && i < x1 && k >= z0 && k < z1) {
      const int pos = atomicAdd(&s_nrec, 1);
      if (pos < kResMaxLocalRec) {
        s_rec[2 * pos] = q;
        s_rec[2 * pos + 1] = fi(k - z0, i - x0);
      }
    }
  }
  __syncthreads();
  const int nloc = s_nrec;
  const int si = a.io.si, sk = a.io.sk;

  // Cell n of this tile in perimeter-first order: the first and last rows,
  // then the first and last columns, then the interior row by row.
  // Tabulated once (CELL) so the steps do no division.
  auto cell_order = [&](int n, int& lr, int& lc) {
    if (tz <= 2 || tw <= 2) {
      lr = n / tw;
      lc = n - lr * tw;
    } else if (n < 2 * tw) {
      lr = n < tw ? 0 : tz - 1;
      lc = n < tw ? n : n - tw;
    } else if (n < 2 * tw + 2 * (tz - 2)) {
      const int m = n - 2 * tw;
      lr = 1 + (m < tz - 2 ? m : m - (tz - 2));
      lc = m < tz - 2 ? 0 : tw - 1;
    } else {
      const int m = n - 2 * tw - 2 * (tz - 2);
      lr = 1 + m / (tw - 2);
      lc = 1 + m % (tw - 2);
    }
  };
  for (int n = tid; n < CS; n += kS2Threads) {
    int lr, lc;
    cell_order(n, lr, lc);
    CELL[n] = (unsigned short)((lr << 7) | lc);
  }
  __syncthreads();
  auto cell_at = [&](int n, int& lr, int& lc) {
    const unsigned e = CELL[n];
    lr = (int)(e >> 7);
    lc = (int)(e & 127u);
  };
  auto record = [&](int t) {  // receivers of step t, by the exchange warps
    float* tr = a.io.traces + (size_t)t * 2 * a.io.nrec;
    if (nloc <= kResMaxLocalRec) {
      for (int q = tid; q < nloc; q += 32 * kS2ExchangeWarps) {
        const int r = s_rec[2 * q], c = s_rec[2 * q + 1];
        tr[r] = VX[c];
        tr[a.io.nrec + r] = VZ[c];
      }
    } else {
      for (int r = tid; r < a.io.nrec; r += 32 * kS2ExchangeWarps) {
        const int i = a.io.rec[3 * r], k = a.io.rec[3 * r + 2];
        if (i >= x0 && i < x1 && k >= z0 && k < z1) {
          tr[r] = VX[fi(k - z0, i - x0)];
          tr[a.io.nrec + r] = VZ[fi(k - z0, i - x0)];
        }
      }
    }
  };
  const bool xwarp = warp < kS2ExchangeWarps;

  float nrm = 0.0f;
  bool ok = true;
  for (int s = 0; s < a.nsteps; ++s) {
    const int t = a.t0 + s;
    const int ps = s & 1, pv = (s + 1) & 1;  // parities of the stress and velocity edges
    const unsigned ts = (unsigned)s + 1u, tv = (unsigned)s + 2u;

    // ================= stresses (seismicfdtd.f95:247-312) on the cell warps;
    // the exchange warps record the previous step's receivers, then bring in
    // sxx on the left, sxz on the right and above, szz below
    if (xwarp) {
      if (s > 0) record(t - 1);
      bool good = true;
      if (warp == 0 && left)
        good = fetch2(ecol(ps, kESLast, bx - 1) + z0, SXX + fi(0, -1), SW, nullptr, nullptr, 0, tz, ts + a.tag_bias, ctl, a.limit_ns);
      else if (warp == 1 && right)
        good = fetch2(ecol(ps, kESFirst, bx + 1) + z0, SXZ + fi(0, tw), SW, nullptr, nullptr, 0, tz, ts + a.tag_bias, ctl, a.limit_ns);
      else if (warp == 2 && up)
        good = fetch2(erow(ps, kESLast, bz - 1) + x0, SXZ + fi(-1, 0), 1, nullptr, nullptr, 0, tw, ts + a.tag_bias, ctl, a.limit_ns);
      else if (warp == 3 && down)
        good = fetch2(erow(ps, kESFirst, bz + 1) + x0, SZZ + fi(tz, 0), 1, nullptr, nullptr, 0, tw, ts + a.tag_bias, ctl, a.limit_ns);
      if (!good && (tid & 31) == 0) s_abort = 1;
    } else {
      for (int n = tid - 32 * kS2ExchangeWarps; n < CS; n += kS2CellThreads) {
        int lr, lc;
        cell_at(n, lr, lc);
        const int q = lr * tw + lc, k = z0 + lr, i = x0 + lc, f = fi(lr, lc);
        float sxx = SXX[f], szz = SZZ[f], sxz = SXZ[f];
        const bool xs = in_strip(i, NX, W), zs = in_strip(k, NZ, W);
        float mvxx = M[q], mvzz = M[CS + q], mvxz = M[2 * CS + q], mvzx = M[3 * CS + q];
        // the sigmaxz loop's memory: its own (corrected physics) or loop 1's (legacy)
        const bool own2 = !a.legacy;
        const bool loop1 = (k >= 1) && (i <= NX - 2);
        const bool loop2 = (k <= NZ - 2) && (i >= 1);
        if (loop1 || loop2) {
          const float vx0 = VX[f], vz0 = VZ[f];
          const float ikx = XT[lc], ikxh = XT[3 * tw + lc];
          const float ikz = ZT[lr], ikzh = ZT[3 * tz + lr];
          if (loop1) {
            const float d_vx_x = VX[f + 1] - vx0;
            const float d_vz_z = vz0 - VZ[f - SW];
            const float d_vz_x = VZ[f + 1] - vz0;
            const float d_vx_z = vx0 - VX[f - SW];
            if (xs) {  // legacy: b_x_half(j), :255 (the q3 row table); corrected: b_x_half(i)
              mvxx = (a.legacy ? ZT[6 * tz + lr] : XT[5 * tw + lc]) * mvxx + XT[4 * tw + lc] * d_vx_x;
              mvzx = XT[2 * tw + lc] * mvzx + XT[tw + lc] * d_vz_x;
            }
            if (zs) {
              mvzz = ZT[2 * tz + lr] * mvzz + ZT[tz + lr] * d_vz_z;
              mvxz = ZT[5 * tz + lr] * mvxz + ZT[4 * tz + lr] * d_vx_z;
            }
            const float dvx_dx = d_vx_x * ikxh + mvxx;
            const float dvz_dz = d_vz_z * ikz + mvzz;
            const float dvz_dx = d_vz_x * ikx + mvzx;
            const float dvx_dz = d_vx_z * ikzh + mvxz;
            const float A11 = C[q], A13 = C[CS + q], A15 = C[2 * CS + q], A33 = C[3 * CS + q], A35 = C[4 * CS + q];
            const float shear = dvz_dx + dvx_dz;
            sxx = sxx + (A11 * dvx_dx + A13 * dvz_dz + A15 * shear);
            szz = szz + (A13 * dvx_dx + A33 * dvz_dz + A35 * shear);
          }
          if (loop2) {
            const float d_vx_x = vx0 - VX[f - 1];
            const float d_vz_z = VZ[f + SW] - vz0;
            const float d_vz_x = vz0 - VZ[f - 1];
            const float d_vx_z = VX[f + SW] - vx0;
            float mxx = own2 ? M[8 * CS + q] : mvxx, mzz = own2 ? M[9 * CS + q] : mvzz;
            float mxz = own2 ? M[10 * CS + q] : mvxz, mzx = own2 ? M[11 * CS + q] : mvzx;
            if (xs) {
              mxx = XT[5 * tw + lc] * mxx + XT[4 * tw + lc] * d_vx_x;
              mzx = XT[2 * tw + lc] * mzx + XT[tw + lc] * d_vz_x;
            }
            if (zs) {
              mzz = ZT[2 * tz + lr] * mzz + ZT[tz + lr] * d_vz_z;
              mxz = ZT[5 * tz + lr] * mxz + ZT[4 * tz + lr] * d_vx_z;
            }
            const float dvx_dx = d_vx_x * ikxh + mxx;
            const float dvz_dz = d_vz_z * ikz + mzz;
            const float dvz_dx = d_vz_x * ikx + mzx;
            const float dvx_dz = d_vx_z * ikzh + mxz;
            sxz = sxz + (C[5 * CS + q] * dvx_dx + C[6 * CS + q] * dvz_dz + C[7 * CS + q] * (dvz_dx + dvx_dz));
            if (own2) {
              if (xs) { M[8 * CS + q] = mxx; M[11 * CS + q] = mzx; }
              if (zs) { M[9 * CS + q] = mzz; M[10 * CS + q] = mxz; }
            } else {
              mvxx = mxx; mvzz = mzz; mvxz = mxz; mvzx = mzx;
            }
          }
          if (a.io.ssrc && i == si && k == sk) {  // stress source: sigma_ij += f_ij(t) dt
            sxx += a.io.ssrc[t];
            szz += a.io.ssrc[a.io.nstep + t];
            sxz += a.io.ssrc[2 * a.io.nstep + t];
          }
          SXX[f] = sxx;
          SZZ[f] = szz;
          SXZ[f] = sxz;
          if (xs) {
            M[q] = mvxx;
            M[3 * CS + q] = mvzx;
          }
          if (zs) {
            M[CS + q] = mvzz;
            M[2 * CS + q] = mvxz;
          }
        }
        if (right && lc == tw - 1) ll_put1(ecol(ps, kESLast, bx) + k, sxx, ts);
        if (left && lc == 0) ll_put1(ecol(ps, kESFirst, bx) + k, sxz, ts);
        if (down && lr == tz - 1) ll_put1(erow(ps, kESLast, bz) + i, sxz, ts);
        if (up && lr == 0) ll_put1(erow(ps, kESFirst, bz) + i, szz, ts);
      }
    }
    __syncthreads();
    if (s_abort) {
      ok = false;
      break;
    }

    // ================= velocities, source, Dirichlet planes, norm (:317-379)
    // on the cell warps; the exchange warps bring in the velocity halo of the
    // next step
    if (xwarp) {
      bool good = true;
      if (s + 1 < a.nsteps) {
        if (warp == 0 && left)
          good = fetch2(ecol(pv, kEVxLast, bx - 1) + z0, VX + fi(0, -1), SW, ecol(pv, kEVzLast, bx - 1) + z0,
                        VZ + fi(0, -1), SW, tz, tv + a.tag_bias, ctl, a.limit_ns);
        else if (warp == 1 && right)
          good = fetch2(ecol(pv, kEVxFirst, bx + 1) + z0, VX + fi(0, tw), SW, ecol(pv, kEVzFirst, bx + 1) + z0,
                        VZ + fi(0, tw), SW, tz, tv + a.tag_bias, ctl, a.limit_ns);
        else if (warp == 2 && up)
          good = fetch2(erow(pv, kEVxLast, bz - 1) + x0, VX + fi(-1, 0), 1, erow(pv, kEVzLast, bz - 1) + x0,
                        VZ + fi(-1, 0), 1, tw, tv + a.tag_bias, ctl, a.limit_ns);
        else if (warp == 3 && down)
          good = fetch2(erow(pv, kEVxFirst, bz + 1) + x0, VX + fi(tz, 0), 1, erow(pv, kEVzFirst, bz + 1) + x0,
                        VZ + fi(tz, 0), 1, tw, tv + a.tag_bias, ctl, a.limit_ns);
      }
      if (!good && (tid & 31) == 0) s_abort = 1;
    } else {
      for (int n = tid - 32 * kS2ExchangeWarps; n < CS; n += kS2CellThreads) {
        int lr, lc;
        cell_at(n, lr, lc);
        const int q = lr * tw + lc, k = z0 + lr, i = x0 + lc, f = fi(lr, lc);
        const bool xs = in_strip(i, NX, W), zs = in_strip(k, NZ, W);
        const bool interior = (i >= 1) && (i <= NX - 2) && (k >= 1) && (k <= NZ - 2);
        float vx = 0.f, vz = 0.f;
        if (k >= 1 && i >= 1) {  // vx loop, :317-336
          const float d1 = SXX[f] - SXX[f - 1];
          const float d2 = SXZ[f] - SXZ[f - SW];
          float v1 = d1 * XT[lc], v2 = d2 * ZT[lr];
          if (xs) {
            const float m = XT[2 * tw + lc] * M[4 * CS + q] + XT[tw + lc] * d1;
            M[4 * CS + q] = m;
            v1 += m;
          }
          if (zs) {
            const float m = ZT[2 * tz + lr] * M[7 * CS + q] + ZT[tz + lr] * d2;
            M[7 * CS + q] = m;
            v2 += m;
          }
          if (interior) {
            vx = VX[f];
            if (a.atten) vx *= C[10 * CS + q];
            vx = vx + (v1 + v2) * C[8 * CS + q];
          }
        }
        if (k <= NZ - 2 && i <= NX - 2) {  // vz loop, :338-357
          const float d1 = SXZ[f + 1] - SXZ[f];
          const float d2 = SZZ[f + SW] - SZZ[f];
          float v1 = d1 * XT[3 * tw + lc], v2 = d2 * ZT[3 * tz + lr];
          if (xs) {
            const float m = XT[5 * tw + lc] * M[6 * CS + q] + XT[4 * tw + lc] * d1;
            M[6 * CS + q] = m;
            v1 += m;
          }
          if (zs) {
            const float m = ZT[5 * tz + lr] * M[5 * CS + q] + ZT[4 * tz + lr] * d2;
            M[5 * CS + q] = m;
            v2 += m;
          }
          if (interior) {
            vz = VZ[f];
            if (a.atten) vz *= C[11 * CS + q];
            vz = vz + (v1 + v2) * C[9 * CS + q];
          }
        }
        if (i == si && k == sk) {  // :360-361
          vx += a.io.src[t];
          vz += a.io.src[a.io.nstep + t];
        }
        if (!interior) {  // :365-375
          vx = 0.f;
          vz = 0.f;
        }
        VX[f] = vx;
        VZ[f] = vz;
        nrm = fmaxf(nrm, norm_monitor(vx, vz));
        if (left && lc == 0) {
          ll_put1(ecol(pv, kEVxFirst, bx) + k, vx, tv);
          ll_put1(ecol(pv, kEVzFirst, bx) + k, vz, tv);
        }
        if (right && lc == tw - 1) {
          ll_put1(ecol(pv, kEVxLast, bx) + k, vx, tv);
          ll_put1(ecol(pv, kEVzLast, bx) + k, vz, tv);
        }
        if (up && lr == 0) {
          ll_put1(erow(pv, kEVxFirst, bz) + i, vx, tv);
          ll_put1(erow(pv, kEVzFirst, bz) + i, vz, tv);
        }
        if (down && lr == tz - 1) {
          ll_put1(erow(pv, kEVxLast, bz) + i, vx, tv);
          ll_put1(erow(pv, kEVzLast, bz) + i, vz, tv);
        }
      }
    }
    __syncthreads();
    if (s_abort) {
      ok = false;
      break;
    }
    if (DUMP) {  // the state after step t into slot s + 1 (streaming stores: read once, by the adjoint)
      char* slot = a.dump.base + a.dump.stride * (size_t)(s + 1);
      auto arr = [&](int q) { return reinterpret_cast<float*>(slot + a.dump.off[q]); };
      for (int q = tid; q < CS; q += kS2Threads) {
        const int lr = q / tw, lc = q - lr * tw, k = z0 + lr, i = x0 + lc, f = fi(lr, lc);
        const size_t g = (size_t)k * P + i;
        __stcs(arr(0) + g, VX[f]);
        __stcs(arr(1) + g, VZ[f]);
        __stcs(arr(2) + g, SXX[f]);
        __stcs(arr(3) + g, SZZ[f]);
        __stcs(arr(4) + g, SXZ[f]);
        if (in_strip(i, NX, W)) {
          const size_t mx = (size_t)k * (2 * W) + strip_idx(i, NX, W);
          const int xm[6] = {0, 3, 4, 6, 8, 11};
#pragma unroll
          for (int e = 0; e < 6; ++e) __stcs(arr(5 + xm[e]) + mx, M[xm[e] * CS + q]);
        }
        if (in_strip(k, NZ, W)) {
          const size_t mz = (size_t)strip_idx(k, NZ, W) * P + i;
          const int zm[6] = {1, 2, 5, 7, 9, 10};
#pragma unroll
          for (int e = 0; e < 6; ++e) __stcs(arr(5 + zm[e]) + mz, M[zm[e] * CS + q]);
        }
      }
      __syncthreads();  // the next step's stresses overwrite what the dump reads
    }
  }
  if (ok && xwarp && a.nsteps > 0) record(a.t0 + a.nsteps - 1);
  if (!ok) return;  // the state is left as it was loaded; the host reports the timeout
  if (DUMP) {
    block_norm_to_slot(nrm, a.io.slots, blockIdx.x);
    return;
  }

  // ---- write the tile back
  for (int q = tid; q < CS; q += kS2Threads) {
    const int lr = q / tw, lc = q - lr * tw, k = z0 + lr, i = x0 + lc, f = fi(lr, lc);
    const size_t g = (size_t)k * P + i;
    a.vx[g] = VX[f];
    a.vz[g] = VZ[f];
    a.sxx[g] = SXX[f];
    a.szz[g] = SZZ[f];
    a.sxz[g] = SXZ[f];
    if (in_strip(i, NX, W)) {
      const size_t mx = (size_t)k * (2 * W) + strip_idx(i, NX, W);
      a.m_vxx[mx] = M[q];
      a.m_vzx[mx] = M[3 * CS + q];
      a.m_sxx_x[mx] = M[4 * CS + q];
      a.m_sxz_x[mx] = M[6 * CS + q];
      if (!a.legacy) {
        a.m2_vxx[mx] = M[8 * CS + q];
        a.m2_vzx[mx] = M[11 * CS + q];
      }
    }
    if (in_strip(k, NZ, W)) {
      const size_t mz = (size_t)strip_idx(k, NZ, W) * P + i;
      a.m_vzz[mz] = M[CS + q];
      a.m_vxz[mz] = M[2 * CS + q];
      a.m_szz_z[mz] = M[5 * CS + q];
      a.m_sxz_z[mz] = M[7 * CS + q];
      if (!a.legacy) {
        a.m2_vzz[mz] = M[9 * CS + q];
        a.m2_vxz[mz] = M[10 * CS + q];
      }
    }
  }
  block_norm_to_slot(nrm, a.io.slots, blockIdx.x);
}

}  // namespace

bool seis2_resident_plan(int NX, int NZ, int max_ctas, size_t max_smem, Seis2ResPlan* out) {
  max_ctas = std::min(max_ctas, kResMaxTiles);
  long best = -1;
  int bnx = 0, bnz = 0;
  for (int ntz = 1; ntz <= std::min(kResMaxTiles1D, NZ); ++ntz)
    for (int ntx = 1; ntx <= std::min(kResMaxTiles1D, NX) && ntx * ntz <= max_ctas; ++ntx) {
      const int TW = (NX + ntx - 1) / ntx, TZ = (NZ + ntz - 1) / ntz;
      if (TW > kS2MaxTile || TZ > kS2MaxTile || s2_smem(TW, TZ) > max_smem) continue;
      // the largest tile sets the pace; among equals, the shorter perimeter
      const long cost = 4L * TW * TZ + TW + TZ;
      if (best < 0 || cost < best) {
        best = cost;
        bnx = ntx;
        bnz = ntz;
      }
    }
  if (best < 0) return false;
  out->ntx = bnx;
  out->ntz = bnz;
  for (int c = 0; c <= bnx; ++c) out->xb[c] = (int)((long)c * NX / bnx);
  for (int r = 0; r <= bnz; ++r) out->zb[r] = (int)((long)r * NZ / bnz);
  out->smem = s2_smem((NX + bnx - 1) / bnx, (NZ + bnz - 1) / bnz);
  return true;
}

cudaError_t seis2_resident_prepare(const Seis2ResPlan& plan, int* ctas_per_sm) {
  const void* fns[2] = {(const void*)seis2_resident_kernel<false>, (const void*)seis2_resident_kernel<true>};
  int n = 1 << 30;
  for (const void* fn : fns) {
    cudaError_t e = res_allow_max_smem(fn);
    int q = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q, fn, kS2Threads, plan.smem);
    if (e != cudaSuccess) return e;
    n = std::min(n, q);
  }
  *ctas_per_sm = n;
  return cudaSuccess;
}

cudaError_t seis2_resident_launch(const Seis2Resident& a, cudaStream_t s) {
  void* args[] = {(void*)&a};
  const void* fn = a.dump.base ? (const void*)seis2_resident_kernel<true> : (const void*)seis2_resident_kernel<false>;
  return cudaLaunchCooperativeKernel(fn, dim3(a.plan.ntx * a.plan.ntz), dim3(kS2Threads), args, a.plan.smem, s);
}

}  // namespace sfd
