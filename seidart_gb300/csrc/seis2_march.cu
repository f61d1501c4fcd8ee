// seismic2 single-pass step for grids too large for the on-chip run: a
// z-march with TMA-staged rows (legacy/fortran/seismicfdtd.f95:247-379).
//
// A block of 128 threads owns 124 columns (x0 .. x0+123, x0 = 124 bx) and a
// segment of rows [k0, k1).  Thread tx sits on column x0 - 2 + tx.  It marches
// down the stress rows r = k0-1 .. k1: at row r every thread of columns
// x0-1 .. x0+124 forms the three new stresses from the old velocities of rows
// r-1, r, r+1 (the block's own columns and one halo column on each side, the
// stress half-step's halo; rows k0-1 and k1 are the segment's halo rows); the
// new stresses of the last three rows stay in shared memory, and once row r
// is done the own columns update the velocities of row r-1.  Only own rows
// and columns are stored, read from one copy of the ping-pong pair and
// written to the other, as the tile kernels do (fused2d.cuh): both forms run
// the same per-cell operations.
//
// The rows come through a ring of RING shared-memory stages filled by
// cp.async.bulk.tensor boxes of 132 columns from x0 - 4 (16-byte aligned):
// stage m holds the velocities of row r0 - 1 + m and, from m = 2 on, the old
// stresses and the eight stiffness coefficients of row r0 + m - 2 and the
// four velocity coefficients of row r0 + m - 3 (r0 = k0 - 1).  One thread
// issues the boxes RING - 3 stages ahead; every thread waits on the stage's
// mbarrier, bounded by the handle's wait limit.  The memory variables (CPML
// strips only) go through plain loads and stores.
#include "sfd_solvers.h"
#include "tma.cuh"

namespace sfd {

namespace {

constexpr int MT = 128;               // threads per block
constexpr int MW = 124;               // own columns per block
constexpr int MX = 132;               // staged columns: x0 - 4 .. x0 + 127
constexpr int RING = 5;
// Each box lands on a 128-byte boundary of the stage (the alignment a
// tensor copy's shared-memory destination needs).
constexpr int ST_V = 0;               // vx vz of the stage's velocity row (2 x 132 floats)
constexpr int ST_S = 288;             // sxx szz sxz (old) of its stress row (3 x 132)
constexpr int ST_CS = 704;            // A11 A13 A15 A33 A35 B15 B35 B55 of its stress row (8 x 132)
constexpr int ST_CV = 1760;           // dtrx dtrz gxp gzp of its velocity row (4 x 132)
constexpr int STAGE = 2304;           // 9216 bytes
static_assert(ST_S >= 2 * MX && ST_CS >= ST_S + 3 * MX && ST_CV >= ST_CS + 8 * MX && STAGE >= ST_CV + 4 * MX,
              "stage layout");
static_assert(ST_S % 32 == 0 && ST_CS % 32 == 0 && ST_CV % 32 == 0 && STAGE % 32 == 0 && (MX * 4) % 16 == 0,
              "128-byte aligned boxes");
constexpr uint32_t V_BYTES = 2 * MX * 4, SC_BYTES = 15 * MX * 4;

__device__ void march_wait_failed(const Seis2Step& a, uint64_t* full, int n, int nst, unsigned long long limit) {
  atomicExch(&a.io.ctl->err, 1);
  const int issued = min(nst, n + RING);
  for (int m = n; m < issued; ++m) tma::bar_wait(full + m % RING, (m / RING) & 1, limit);
}

__global__ void __launch_bounds__(MT, 4)
    seis2_march_kernel(const __grid_constant__ Seis2Step a, const __grid_constant__ Seis2March mm, int rel) {
  extern __shared__ __align__(128) unsigned char stage_raw[];
  float* const stage = tma::aligned_stage(stage_raw);
  __shared__ float sN[3][3][MX];  // new sxx szz sxz of rows r-2, r-1, r (by r mod 3)
  __shared__ __align__(8) uint64_t full[RING];
  const Ctl* ctl = a.io.ctl;
  const int t = ctl->base + rel;
  if (blockIdx.x == 0 && blockIdx.y == 0 && t > ctl->run_start) {
    const float* ch[2] = {a.vx0, a.vz0};
    gather_receivers<2>(a.io.rec, a.io.nrec, a.io.traces, t - 1, ch, a.P, 1, false);
  }
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  const int tx = threadIdx.x;
  const int x0 = blockIdx.x * MW;
  const int k0 = blockIdx.y * mm.seg, k1 = min(NZ, k0 + mm.seg);
  const int slot = blockIdx.y * gridDim.x + blockIdx.x;
  float norm = 0.0f;
  if (k0 >= k1) {  // the whole block
    block_norm_to_slot(norm, a.io.slots, slot);
    return;
  }
  if (tma::smem_addr(stage) & 127u) {  // the ring's base must be 128-byte aligned: record, copy nothing, leave
    if (tx == 0) atomicExch(&a.io.ctl->err, 1);
    block_norm_to_slot(norm, a.io.slots, slot);
    return;
  }
  const int r0 = k0 - 1;
  const int nst = (k1 - k0 + 2) + 2;  // stages: velocity rows r0-1 .. k1+1
  if (tx == 0) {
    for (int q = 0; q < RING; ++q) tma::bar_init(full + q, 1);
    tma::fence_bar_init();
  }
  __syncthreads();
  auto issue = [&](int m) {
    float* st = stage + (m % RING) * STAGE;
    uint64_t* bar = full + m % RING;
    const bool sc = m >= 2;
    tma::bar_arrive_expect(bar, V_BYTES + (sc ? SC_BYTES : 0u) + mm.stall_tx);
    tma::load_3d(st + ST_V, &mm.tm_v, bar, x0 - 4, r0 - 1 + m, 0);
    if (sc) {
      tma::load_3d(st + ST_S, &mm.tm_s, bar, x0 - 4, r0 + m - 2, 2);
      tma::load_3d(st + ST_CS, &mm.tm_cs, bar, x0 - 4, r0 + m - 2, 0);
      tma::load_3d(st + ST_CV, &mm.tm_cv, bar, x0 - 4, r0 + m - 3, 8);
    }
  };
  if (tx == 0)
    for (int m = 0; m < min(RING, nst); ++m) issue(m);

  const int i = x0 - 2 + tx;  // this thread's column
  const int j = tx + 2;       // its index in a staged row
  const bool scol = tx >= 1 && tx <= MW + 2 && i >= 0 && i < NX;  // forms stresses (own or halo column)
  const bool own = tx >= 2 && tx < MW + 2 && i < NX;               // stores (own column)
  const int ic = (i >= 0 && i < NX) ? i : 0;
  const bool xs = (i >= 0 && i < NX) && in_strip(i, NX, W);
  const int xsi = xs ? strip_idx(i, NX, W) : 0;
  const float ikx = __ldg(a.X.ik + ic), ikxh = __ldg(a.X.ikh + ic), adx = __ldg(a.X.ad + ic), adxh = __ldg(a.X.adh + ic);
  const float bx = __ldg(a.X.b + ic), bxh = __ldg(a.X.bh + ic);
  const bool own2 = !a.legacy;
  for (int n = 0; n < nst - 2; ++n) {
    const int r = r0 + n;
    bool ok = tma::bar_wait(full + n % RING, (n / RING) & 1, mm.wait_ns);
    if (ok) ok = tma::bar_wait(full + (n + 1) % RING, ((n + 1) / RING) & 1, mm.wait_ns);
    if (ok) ok = tma::bar_wait(full + (n + 2) % RING, ((n + 2) / RING) & 1, mm.wait_ns);
    const float* Vu = stage + (n % RING) * STAGE + ST_V;        // velocities of row r - 1
    const float* Vc = stage + ((n + 1) % RING) * STAGE + ST_V;  // row r
    const float* Vd = stage + ((n + 2) % RING) * STAGE + ST_V;  // row r + 1
    const float* St = stage + ((n + 2) % RING) * STAGE;         // old stresses and coefficients of row r
    float* nrow = &sN[(r + 3) % 3][0][0];
    // ---- the stresses of row r (:247-312), the stress source
    if (ok) {
      float sxx = 0.f, szz = 0.f, sxz = 0.f;
      if (scol && r >= 0 && r < NZ) {
        const int c = r * P + i;
        const bool rown = own && r >= k0 && r < k1;
        const bool zs = in_strip(r, NZ, W);
        const int mx = r * (2 * W) + xsi;
        const int mz = (zs ? strip_idx(r, NZ, W) : 0) * P + i;
        sxx = St[ST_S + j];
        szz = St[ST_S + MX + j];
        sxz = St[ST_S + 2 * MX + j];
        float mvxx = 0.f, mvzx = 0.f, mvzz = 0.f, mvxz = 0.f, nvxx = 0.f, nvzx = 0.f, nvzz = 0.f, nvxz = 0.f;
        if (xs) {
          mvxx = a.m_vxx0[mx];
          mvzx = a.m_vzx0[mx];
          if (own2) { nvxx = a.m2_vxx0[mx]; nvzx = a.m2_vzx0[mx]; }
        }
        if (zs) {
          mvzz = a.m_vzz0[mz];
          mvxz = a.m_vxz0[mz];
          if (own2) { nvzz = a.m2_vzz0[mz]; nvxz = a.m2_vxz0[mz]; }
        }
        const bool loop1 = (r >= 1) && (i <= NX - 2);
        const bool loop2 = (r <= NZ - 2) && (i >= 1);
        const float vx0 = Vc[j], vz0 = Vc[MX + j];
        const float ikz = __ldg(a.Z.ik + r), ikzh = __ldg(a.Z.ikh + r);
        if (loop1) {  // :247-281
          const float d_vx_x = Vc[j + 1] - vx0;
          const float d_vz_z = vz0 - Vu[MX + j];
          const float d_vz_x = Vc[MX + j + 1] - vz0;
          const float d_vx_z = vx0 - Vu[j];
          if (xs) {
            const float bq = a.legacy ? __ldg(a.q3 + r) : bxh;  // b_x_half(j) as :255, or (i)
            mvxx = bq * mvxx + adxh * d_vx_x;
            mvzx = bx * mvzx + adx * d_vz_x;
          }
          if (zs) {
            mvzz = __ldg(a.Z.b + r) * mvzz + __ldg(a.Z.ad + r) * d_vz_z;
            mvxz = __ldg(a.Z.bh + r) * mvxz + __ldg(a.Z.adh + r) * d_vx_z;
          }
          const float dvx_dx = d_vx_x * ikxh + mvxx;
          const float dvz_dz = d_vz_z * ikz + mvzz;
          const float dvz_dx = d_vz_x * ikx + mvzx;
          const float dvx_dz = d_vx_z * ikzh + mvxz;
          const float* cs = St + ST_CS + j;
          const float A11 = cs[0], A13 = cs[MX], A15 = cs[2 * MX], A33 = cs[3 * MX], A35 = cs[4 * MX];
          const float shear = dvz_dx + dvx_dz;
          sxx = sxx + (A11 * dvx_dx + A13 * dvz_dz + A15 * shear);
          szz = szz + (A13 * dvx_dx + A33 * dvz_dz + A35 * shear);
        }
        if (loop2) {  // :283-312
          const float d_vx_x = vx0 - Vc[j - 1];
          const float d_vz_z = Vd[MX + j] - vz0;
          const float d_vz_x = vz0 - Vc[MX + j - 1];
          const float d_vx_z = Vd[j] - vx0;
          float mxx = own2 ? nvxx : mvxx, mzx = own2 ? nvzx : mvzx;
          float mzz = own2 ? nvzz : mvzz, mxz = own2 ? nvxz : mvxz;
          if (xs) {
            mxx = bxh * mxx + adxh * d_vx_x;
            mzx = bx * mzx + adx * d_vz_x;
          }
          if (zs) {
            mzz = __ldg(a.Z.b + r) * mzz + __ldg(a.Z.ad + r) * d_vz_z;
            mxz = __ldg(a.Z.bh + r) * mxz + __ldg(a.Z.adh + r) * d_vx_z;
          }
          const float dvx_dx = d_vx_x * ikxh + mxx;
          const float dvz_dz = d_vz_z * ikz + mzz;
          const float dvz_dx = d_vz_x * ikx + mzx;
          const float dvx_dz = d_vx_z * ikzh + mxz;
          const float* cs = St + ST_CS + j;
          sxz = sxz + (cs[5 * MX] * dvx_dx + cs[6 * MX] * dvz_dz + cs[7 * MX] * (dvz_dx + dvx_dz));
          if (own2) { nvxx = mxx; nvzx = mzx; nvzz = mzz; nvxz = mxz; }
          else { mvxx = mxx; mvzx = mzx; mvzz = mzz; mvxz = mxz; }
        }
        if (a.io.ssrc && i == a.io.si && r == a.io.sk) {  // stress source: sigma_ij += f_ij(t) dt
          sxx += __ldg(a.io.ssrc + t);
          szz += __ldg(a.io.ssrc + a.io.nstep + t);
          sxz += __ldg(a.io.ssrc + 2 * a.io.nstep + t);
        }
        if (rown) {
          a.sxx1[c] = sxx;
          a.szz1[c] = szz;
          a.sxz1[c] = sxz;
          if (xs) {
            a.m_vxx1[mx] = mvxx;
            a.m_vzx1[mx] = mvzx;
            if (own2) { a.m2_vxx1[mx] = nvxx; a.m2_vzx1[mx] = nvzx; }
          }
          if (zs) {
            a.m_vzz1[mz] = mvzz;
            a.m_vxz1[mz] = mvxz;
            if (own2) { a.m2_vzz1[mz] = nvzz; a.m2_vxz1[mz] = nvxz; }
          }
        }
      }
      nrow[j] = sxx;
      nrow[MX + j] = szz;
      nrow[2 * MX + j] = sxz;
    }
    ok = __syncthreads_and(ok);  // row r's stresses visible
    // ---- the velocities of row k = r - 1 (:317-379)
    const int k = r - 1;
    if (ok && own && k >= k0 && k < k1) {
      const int c = k * P + i;
      const float* Sm = &sN[(k + 2) % 3][0][0];  // row k - 1
      const float* Sk = &sN[(k + 3) % 3][0][0];  // row k
      const float* Sp = &sN[(k + 4) % 3][0][0];  // row k + 1
      const float* cv = St + ST_CV + j;         // dtrx dtrz gxp gzp of row k
      const bool zs = in_strip(k, NZ, W);
      const int mx = k * (2 * W) + xsi;
      const int mz = (zs ? strip_idx(k, NZ, W) : 0) * P + i;
      const bool interior = (i >= 1) && (i <= NX - 2) && (k >= 1) && (k <= NZ - 2);
      float vx = 0.f, vz = 0.f;
      if (k >= 1 && i >= 1) {  // vx loop, :317-336
        const float d1 = Sk[j] - Sk[j - 1];
        const float d2 = Sk[2 * MX + j] - Sm[2 * MX + j];
        float v1 = d1 * ikx, v2 = d2 * __ldg(a.Z.ik + k);
        if (xs) {
          const float m = bx * a.m_sxx_x[mx] + adx * d1;
          a.m_sxx_x[mx] = m;
          v1 += m;
        }
        if (zs) {
          const float m = __ldg(a.Z.b + k) * a.m_sxz_z[mz] + __ldg(a.Z.ad + k) * d2;
          a.m_sxz_z[mz] = m;
          v2 += m;
        }
        if (interior) {
          vx = Vu[j];  // old vx of row k = r - 1
          if (a.atten) vx *= cv[2 * MX];
          vx = vx + (v1 + v2) * cv[0];
        }
      }
      if (k <= NZ - 2 && i <= NX - 2) {  // vz loop, :338-357
        const float d1 = Sk[2 * MX + j + 1] - Sk[2 * MX + j];
        const float d2 = Sp[MX + j] - Sk[MX + j];
        float v1 = d1 * ikxh, v2 = d2 * __ldg(a.Z.ikh + k);
        if (xs) {
          const float m = bxh * a.m_sxz_x[mx] + adxh * d1;
          a.m_sxz_x[mx] = m;
          v1 += m;
        }
        if (zs) {
          const float m = __ldg(a.Z.bh + k) * a.m_szz_z[mz] + __ldg(a.Z.adh + k) * d2;
          a.m_szz_z[mz] = m;
          v2 += m;
        }
        if (interior) {
          vz = Vu[MX + j];
          if (a.atten) vz *= cv[3 * MX];
          vz = vz + (v1 + v2) * cv[MX];
        }
      }
      if (i == a.io.si && k == a.io.sk) {  // :360-361
        vx += a.io.src[t];
        vz += a.io.src[a.io.nstep + t];
      }
      if (!interior) { vx = 0.f; vz = 0.f; }  // :365-375
      a.vx1[c] = vx;
      a.vz1[c] = vz;
      norm = fmaxf(norm, norm_monitor(vx, vz));
    }
    if (!__syncthreads_and(ok)) {  // every thread is done with stage n (or a wait ran out)
      if (tx == 0) march_wait_failed(a, full, n, nst, mm.wait_ns);
      break;
    }
    if (tx == 0 && n + RING < nst) {
      tma::fence_async_smem();
      issue(n + RING);
    }
  }
  block_norm_to_slot(norm, a.io.slots, slot);
}

}  // namespace

bool seis2_march_prepare(const Seis2Step& a, size_t field_stride, const float* coef, size_t coef_plane,
                         Seis2March* out) {
  if (cudaFuncSetAttribute(seis2_march_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           RING * STAGE * (int)sizeof(float) + tma::kStageSlack) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  // (x, z, field), x extent NX: boxes past the grid's edges read zeros
  auto map3 = [&](CUtensorMap* m, const void* base, int nf, size_t fstride, int boxf) {
    const cuuint64_t dims[3] = {(cuuint64_t)a.NX, (cuuint64_t)a.NZ, (cuuint64_t)nf};
    const cuuint64_t strides[2] = {(cuuint64_t)a.P * 4, (cuuint64_t)fstride * 4};
    const cuuint32_t box[3] = {MX, 1, (cuuint32_t)boxf};
    return encode_tiled(m, const_cast<void*>(base), 3, dims, strides, box);
  };
  return map3(&out->tm_v, a.vx0, 5, field_stride, 2) && map3(&out->tm_s, a.vx0, 5, field_stride, 3) &&
         map3(&out->tm_cs, coef, 12, coef_plane, 8) && map3(&out->tm_cv, coef, 12, coef_plane, 4);
}

Launch seis2_march_launch(const Seis2Step& a, int seg) {
  Launch L;
  L.block = dim3(MT, 1, 1);
  L.grid = dim3((a.NX + MW - 1) / MW, (a.NZ + seg - 1) / seg, 1);
  L.nslots = L.grid.x * L.grid.y;
  return L;
}

void seis2_march(const Seis2Step& a, const Seis2March& m, const Launch& L, int rel, cudaStream_t s) {
  seis2_march_kernel<<<L.grid, L.block, RING * STAGE * sizeof(float) + tma::kStageSlack, s>>>(a, m, rel);
}

}  // namespace sfd
