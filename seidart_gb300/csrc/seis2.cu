// seismic2 (legacy/fortran/seismicfdtd.f95:12-385): 2-D anisotropic
// velocity-stress scheme.  Two fused kernels per step:
//   half1: both stress loops (:247-281 sigmaxx/sigmazz, :283-312 sigmaxz) for
//          one cell per thread, then the stress source at its cell.  With the
//          legacy quirks the four velocity-gradient memory variables are
//          shared by the two loops, as in the Fortran, so at a cell that both
//          loops visit they advance twice, first with the loop-1 stencil and
//          then with the loop-2 stencil, and loop 1 uses b_x_half at the z
//          index (:255), read from a table q3[k] that the host fills from
//          b_x_half.  With corrected physics (the default) the sigmaxz loop
//          has its own four memory variables and loop 1 uses b_x_half(i).
//          Block (0,0) first records the receivers of the previous step.
//   half2: vx (:317-336) and vz (:338-357) with the stress-gradient memory
//          variables, attenuation, the source (:360-361), the Dirichlet edges
//          (:365-375) and the per-block field norm (:378-379).
#include "sfd_solvers.h"

namespace sfd {

namespace {

constexpr int BX = 32, BY = 8;

__global__ void __launch_bounds__(BX * BY) seis2_stress_kernel(Seis2Args a, int rel) {
  const Ctl* ctl = a.io.ctl;
  const int t = ctl->base + rel;
  if (blockIdx.x == 0 && blockIdx.y == 0 && t > ctl->run_start) {
    const float* ch[2] = {a.vx, a.vz};
    gather_receivers<2>(a.io.rec, a.io.nrec, a.io.traces, t - 1, ch, a.P, 1, false);
  }
  const int i = blockIdx.x * BX + threadIdx.x;
  const int k = blockIdx.y * BY + threadIdx.y;
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  if (i >= NX || k >= NZ) return;
  const bool loop1 = (k >= 1) && (i <= NX - 2);  // :247-248
  const bool loop2 = (k <= NZ - 2) && (i >= 1);  // :283-284
  if (!loop1 && !loop2) return;
  const size_t c = (size_t)k * P + i;
  const bool xs = in_strip(i, NX, W), zs = in_strip(k, NZ, W);
  const size_t mx = (size_t)k * (2 * W) + (xs ? strip_idx(i, NX, W) : 0);
  const size_t mz = (size_t)(zs ? strip_idx(k, NZ, W) : 0) * P + i;
  const bool own2 = !a.legacy;
  float m_vxx = 0.f, m_vzx = 0.f, m_vzz = 0.f, m_vxz = 0.f;
  float n_vxx = 0.f, n_vzx = 0.f, n_vzz = 0.f, n_vxz = 0.f;  // the sigmaxz loop's own
  if (xs) {
    m_vxx = a.m_vxx[mx]; m_vzx = a.m_vzx[mx];
    if (own2) { n_vxx = a.m2_vxx[mx]; n_vzx = a.m2_vzx[mx]; }
  }
  if (zs) {
    m_vzz = a.m_vzz[mz]; m_vxz = a.m_vxz[mz];
    if (own2) { n_vzz = a.m2_vzz[mz]; n_vxz = a.m2_vxz[mz]; }
  }
  const float vx0 = a.vx[c], vz0 = a.vz[c];
  const float ikx = a.X.ik[i], ikxh = a.X.ikh[i], ikz = a.Z.ik[k], ikzh = a.Z.ikh[k];

  if (loop1) {
    const float d_vx_x = a.vx[c + 1] - vx0;
    const float d_vz_z = vz0 - a.vz[c - P];
    const float d_vz_x = a.vz[c + 1] - vz0;
    const float d_vx_z = vx0 - a.vx[c - P];
    if (xs) {
      m_vxx = (a.legacy ? a.q3[k] : a.X.bh[i]) * m_vxx + a.X.adh[i] * d_vx_x;
      m_vzx = a.X.b[i] * m_vzx + a.X.ad[i] * d_vz_x;
    }
    if (zs) {
      m_vzz = a.Z.b[k] * m_vzz + a.Z.ad[k] * d_vz_z;
      m_vxz = a.Z.bh[k] * m_vxz + a.Z.adh[k] * d_vx_z;
    }
    const float dvx_dx = d_vx_x * ikxh + m_vxx;
    const float dvz_dz = d_vz_z * ikz + m_vzz;
    const float dvz_dx = d_vz_x * ikx + m_vzx;
    const float dvx_dz = d_vx_z * ikzh + m_vxz;
    const float A11 = a.A11[c], A13 = a.A13[c], A15 = a.A15[c], A33 = a.A33[c], A35 = a.A35[c];
    const float shear = dvz_dx + dvx_dz;
    a.sxx[c] = a.sxx[c] + (A11 * dvx_dx + A13 * dvz_dz + A15 * shear);
    a.szz[c] = a.szz[c] + (A13 * dvx_dx + A33 * dvz_dz + A35 * shear);
  }
  if (loop2) {
    const float d_vx_x = vx0 - a.vx[c - 1];
    const float d_vz_z = a.vz[c + P] - vz0;
    const float d_vz_x = vz0 - a.vz[c - 1];
    const float d_vx_z = a.vx[c + P] - vx0;
    float mxx = own2 ? n_vxx : m_vxx, mzx = own2 ? n_vzx : m_vzx;
    float mzz = own2 ? n_vzz : m_vzz, mxz = own2 ? n_vxz : m_vxz;
    if (xs) {
      mxx = a.X.bh[i] * mxx + a.X.adh[i] * d_vx_x;
      mzx = a.X.b[i] * mzx + a.X.ad[i] * d_vz_x;
    }
    if (zs) {
      mzz = a.Z.b[k] * mzz + a.Z.ad[k] * d_vz_z;
      mxz = a.Z.bh[k] * mxz + a.Z.adh[k] * d_vx_z;
    }
    const float dvx_dx = d_vx_x * ikxh + mxx;
    const float dvz_dz = d_vz_z * ikz + mzz;
    const float dvz_dx = d_vz_x * ikx + mzx;
    const float dvx_dz = d_vx_z * ikzh + mxz;
    const float B15 = a.B15[c], B35 = a.B35[c], B55 = a.B55[c];
    a.sxz[c] = a.sxz[c] + (B15 * dvx_dx + B35 * dvz_dz + B55 * (dvz_dx + dvx_dz));
    if (own2) { n_vxx = mxx; n_vzx = mzx; n_vzz = mzz; n_vxz = mxz; }
    else { m_vxx = mxx; m_vzx = mzx; m_vzz = mzz; m_vxz = mxz; }
  }
  if (xs) {
    a.m_vxx[mx] = m_vxx; a.m_vzx[mx] = m_vzx;
    if (own2) { a.m2_vxx[mx] = n_vxx; a.m2_vzx[mx] = n_vzx; }
  }
  if (zs) {
    a.m_vzz[mz] = m_vzz; a.m_vxz[mz] = m_vxz;
    if (own2) { a.m2_vzz[mz] = n_vzz; a.m2_vxz[mz] = n_vxz; }
  }
  if (a.io.ssrc && i == a.io.si && k == a.io.sk) {  // stress source: sigma_ij += f_ij(t) dt
    a.sxx[c] += a.io.ssrc[t];
    a.szz[c] += a.io.ssrc[a.io.nstep + t];
    a.sxz[c] += a.io.ssrc[2 * a.io.nstep + t];
  }
}

__global__ void __launch_bounds__(BX * BY) seis2_velocity_kernel(Seis2Args a, int rel) {
  const int t = a.io.ctl->base + rel;
  const int i = blockIdx.x * BX + threadIdx.x;
  const int k = blockIdx.y * BY + threadIdx.y;
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  float norm = 0.0f;
  if (i < NX && k < NZ) {
    const size_t c = (size_t)k * P + i;
    const bool xs = in_strip(i, NX, W), zs = in_strip(k, NZ, W);
    const size_t mx = (size_t)k * (2 * W) + (xs ? strip_idx(i, NX, W) : 0);
    const size_t mz = (size_t)(zs ? strip_idx(k, NZ, W) : 0) * P + i;
    const bool interior = (i >= 1) && (i <= NX - 2) && (k >= 1) && (k <= NZ - 2);
    float vx = 0.f, vz = 0.f;
    if (interior) {
      // vx, :317-336 (k in [1, NZ-1], i in [1, NX-1]); edges are zeroed below
      {
        const float d1 = a.sxx[c] - a.sxx[c - 1];
        const float d2 = a.sxz[c] - a.sxz[c - P];
        float v1 = d1 * a.X.ik[i], v2 = d2 * a.Z.ik[k];
        if (xs) {
          const float m = a.X.b[i] * a.m_sxx_x[mx] + a.X.ad[i] * d1;
          a.m_sxx_x[mx] = m;
          v1 += m;
        }
        if (zs) {
          const float m = a.Z.b[k] * a.m_sxz_z[mz] + a.Z.ad[k] * d2;
          a.m_sxz_z[mz] = m;
          v2 += m;
        }
        vx = a.vx[c];
        if (a.atten) vx *= a.gxp[c];
        vx = vx + (v1 + v2) * a.dtrx[c];
      }
      // vz, :338-357 (k in [0, NZ-2], i in [0, NX-2])
      {
        const float d1 = a.sxz[c + 1] - a.sxz[c];
        const float d2 = a.szz[c + P] - a.szz[c];
        float v1 = d1 * a.X.ikh[i], v2 = d2 * a.Z.ikh[k];
        if (xs) {
          const float m = a.X.bh[i] * a.m_sxz_x[mx] + a.X.adh[i] * d1;
          a.m_sxz_x[mx] = m;
          v1 += m;
        }
        if (zs) {
          const float m = a.Z.bh[k] * a.m_szz_z[mz] + a.Z.adh[k] * d2;
          a.m_szz_z[mz] = m;
          v2 += m;
        }
        vz = a.vz[c];
        if (a.atten) vz *= a.gzp[c];
        vz = vz + (v1 + v2) * a.dtrz[c];
      }
    } else {
      // Cells on the outer edges: the Fortran loops still advance the memory
      // variables there before the Dirichlet step zeroes the velocity.
      if (k >= 1 && i >= 1) {  // vx loop covers i = NX-1 and k = NZ-1
        const float d1 = a.sxx[c] - a.sxx[c - 1];
        const float d2 = a.sxz[c] - a.sxz[c - P];
        if (xs) a.m_sxx_x[mx] = a.X.b[i] * a.m_sxx_x[mx] + a.X.ad[i] * d1;
        if (zs) a.m_sxz_z[mz] = a.Z.b[k] * a.m_sxz_z[mz] + a.Z.ad[k] * d2;
      }
      if (k <= NZ - 2 && i <= NX - 2) {  // vz loop covers i = 0 and k = 0
        const float d1 = a.sxz[c + 1] - a.sxz[c];
        const float d2 = a.szz[c + P] - a.szz[c];
        if (xs) a.m_sxz_x[mx] = a.X.bh[i] * a.m_sxz_x[mx] + a.X.adh[i] * d1;
        if (zs) a.m_szz_z[mz] = a.Z.bh[k] * a.m_szz_z[mz] + a.Z.adh[k] * d2;
      }
    }
    // Source, :360-361 (added before the edges are zeroed, as in the Fortran)
    if (i == a.io.si && k == a.io.sk) {
      vx += a.io.src[t];
      vz += a.io.src[a.io.nstep + t];
    }
    if (!interior) { vx = 0.f; vz = 0.f; }  // :365-375
    a.vx[c] = vx;
    a.vz[c] = vz;
    norm = norm_monitor(vx, vz);
  }
  block_norm_to_slot(norm, a.io.slots, blockIdx.y * gridDim.x + blockIdx.x);
}

__global__ void seis2_finalize_kernel(Seis2Args a, int t_last) {
  const float* ch[2] = {a.vx, a.vz};
  gather_receivers<2>(a.io.rec, a.io.nrec, a.io.traces, t_last, ch, a.P, 1, false);
}

}  // namespace

Launch seis2_launch(const Seis2Args& a) {
  Launch L;
  L.block = dim3(BX, BY, 1);
  L.grid = dim3((a.NX + BX - 1) / BX, (a.NZ + BY - 1) / BY, 1);
  L.nslots = L.grid.x * L.grid.y;
  return L;
}

void seis2_half1(const Seis2Args& a, const Launch& L, int rel, cudaStream_t s) {
  seis2_stress_kernel<<<L.grid, L.block, 0, s>>>(a, rel);
}

void seis2_half2(const Seis2Args& a, const Launch& L, int rel, cudaStream_t s) {
  seis2_velocity_kernel<<<L.grid, L.block, 0, s>>>(a, rel);
}

void seis2_finalize(const Seis2Args& a, int t_last, cudaStream_t s) {
  seis2_finalize_kernel<<<1, 256, 0, s>>>(a, t_last);
}

}  // namespace sfd
