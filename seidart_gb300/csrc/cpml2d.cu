// electromag2 and seismic2 steps with the driver's 2-D CPML fields
// (SFD_FLAG_CPML_2D).
//
// The current SeidarT driver writes its CPML coefficients as 2-D fields
// (src/seidart/routines/definitions.py:560-998): one sigma, kappa, alpha,
// acoef, bcoef value per cell and offset, the two axes' profiles combined in
// the corners.  With this flag every derivative direction takes the field's
// value at the cell -- K, a, b of the full offset where the Fortran loop
// reads a full-offset profile, of the half offset where it reads a half one
// -- in place of the per-axis 1-D profiles.  A memory variable then evolves
// wherever a != 0, in both strips, so every memory variable is stored on the
// full grid (index k * P + i) and updated at every cell the Fortran loop
// visits (it stays zero where a = 0).
//
// Otherwise the loops are those of the two-pass kernels (em2.cu, seis2.cu;
// legacy/fortran/electromagfdtd.f95:249-321, seismicfdtd.f95:247-379) with
// the corrected seismic2 physics (the sigmaxz loop's own memory variables);
// the legacy loops read 1-D profiles, so SFD_FLAG_LEGACY_QUIRKS is refused
// with this flag.  These kernels favour clarity over speed: one cell per
// thread, one launch per half-step.
#include "sfd_solvers.h"

namespace sfd {

namespace {

constexpr int BX = 32, BY = 8;

// Derivative d (already divided by the grid step) through the CPML at plane
// offset o (0 full, 1 half) of cell c: psi <- b psi + a d, returns d / K + psi.
__device__ __forceinline__ float cpml2d(const Cpml2d& f, int o, size_t c, float d, float* psi) {
  const float m = f.b[o][c] * *psi + f.a[o][c] * d;
  *psi = m;
  return d * f.ik[o][c] + m;
}

__global__ void __launch_bounds__(BX * BY) em2_c2d_h_kernel(Em2Args a, int rel) {
  const Ctl* ctl = a.io.ctl;
  const int t = ctl->base + rel;
  if (blockIdx.x == 0 && blockIdx.y == 0 && t > ctl->run_start) {
    const float* ch[2] = {a.Ex, a.Ez};
    gather_receivers<2>(a.io.rec, a.io.nrec, a.io.traces, t - 1, ch, a.P, 1, false);
  }
  const int i = blockIdx.x * BX + threadIdx.x;
  const int k = blockIdx.y * BY + threadIdx.y;
  const int NX = a.NX, NZ = a.NZ, P = a.P;
  if (i > NX - 2 || k > NZ - 2) return;
  const size_t c = (size_t)k * P + i;
  const Cpml2d& f = a.c2d;
  const float vz = cpml2d(f, 0, c, (a.Ex[c + P] - a.Ex[c]) * f.idz, a.mExz + c);  // :252-254
  const float vx = cpml2d(f, 0, c, (a.Ez[c + 1] - a.Ez[c]) * f.idx, a.mEzx + c);  // :257-259
  const bool edge = (i == 0) | (i == NX - 2) | (k == 0) | (k == NZ - 2);
  const float hy = edge ? 0.0f : a.Hy[c];
  a.Hy[c] = hy + a.dbH * (vx + vz);  // :262
}

__global__ void __launch_bounds__(BX * BY) em2_c2d_e_kernel(Em2Args a, int rel) {
  const int t = a.io.ctl->base + rel;
  const int i = blockIdx.x * BX + threadIdx.x;
  const int k = blockIdx.y * BY + threadIdx.y;
  const int NX = a.NX, NZ = a.NZ, P = a.P;
  float norm = 0.0f;
  if (i < NX && k < NZ) {
    const size_t c = (size_t)k * P + i;
    const Cpml2d& f = a.c2d;
    float ex = 0.0f, ez = 0.0f;
    if (i <= NX - 2) {  // Ex, :273-283
      ex = a.Ex[c];
      if (k >= 1 && k <= NZ - 2)
        ex = a.CAx[c] * ex + a.CBx[c] * cpml2d(f, 1, c, (a.Hy[c] - a.Hy[c - P]) * f.idz, a.mHyz + c);
    }
    if (k <= NZ - 2) {  // Ez, :285-295
      ez = a.Ez[c];
      if (i >= 1 && i <= NX - 2)
        ez = a.CAz[c] * ez + a.CBz[c] * cpml2d(f, 1, c, (a.Hy[c] - a.Hy[c - 1]) * f.idx, a.mHyx + c);
    }
    if (i == a.io.si && k == a.io.sk) {  // :300-301
      ex += a.io.src[t];
      ez += a.io.src[a.io.nstep + t];
    }
    if (i == 0 || i == NX - 2 || k == 0 || k == NZ - 1) ex = 0.0f;  // :304-312
    if (i == 0 || i == NX - 1 || k == 0 || k == NZ - 2) ez = 0.0f;
    if (i <= NX - 2) a.Ex[c] = ex;
    if (k <= NZ - 2) a.Ez[c] = ez;
    norm = norm_monitor(ex, ez);
  }
  block_norm_to_slot(norm, a.io.slots, blockIdx.y * gridDim.x + blockIdx.x);
}

__global__ void __launch_bounds__(BX * BY) seis2_c2d_stress_kernel(Seis2Args a, int rel) {
  const Ctl* ctl = a.io.ctl;
  const int t = ctl->base + rel;
  if (blockIdx.x == 0 && blockIdx.y == 0 && t > ctl->run_start) {
    const float* ch[2] = {a.vx, a.vz};
    gather_receivers<2>(a.io.rec, a.io.nrec, a.io.traces, t - 1, ch, a.P, 1, false);
  }
  const int i = blockIdx.x * BX + threadIdx.x;
  const int k = blockIdx.y * BY + threadIdx.y;
  const int NX = a.NX, NZ = a.NZ, P = a.P;
  if (i >= NX || k >= NZ) return;
  const bool loop1 = (k >= 1) && (i <= NX - 2);  // :247-248
  const bool loop2 = (k <= NZ - 2) && (i >= 1);  // :283-284
  const size_t c = (size_t)k * P + i;
  const Cpml2d& f = a.c2d;
  const float vx0 = a.vx[c], vz0 = a.vz[c];
  if (loop1) {  // :247-281, memory variables of this loop
    const float dvx_dx = cpml2d(f, 1, c, (a.vx[c + 1] - vx0) * f.idx, a.m_vxx + c);
    const float dvz_dz = cpml2d(f, 0, c, (vz0 - a.vz[c - P]) * f.idz, a.m_vzz + c);
    const float dvz_dx = cpml2d(f, 0, c, (a.vz[c + 1] - vz0) * f.idx, a.m_vzx + c);
    const float dvx_dz = cpml2d(f, 1, c, (vx0 - a.vx[c - P]) * f.idz, a.m_vxz + c);
    const float shear = dvz_dx + dvx_dz;
    a.sxx[c] = a.sxx[c] + (a.A11[c] * dvx_dx + a.A13[c] * dvz_dz + a.A15[c] * shear);
    a.szz[c] = a.szz[c] + (a.A13[c] * dvx_dx + a.A33[c] * dvz_dz + a.A35[c] * shear);
  }
  if (loop2) {  // :283-312, the sigmaxz loop's own memory variables
    const float dvx_dx = cpml2d(f, 1, c, (vx0 - a.vx[c - 1]) * f.idx, a.m2_vxx + c);
    const float dvz_dz = cpml2d(f, 0, c, (a.vz[c + P] - vz0) * f.idz, a.m2_vzz + c);
    const float dvz_dx = cpml2d(f, 0, c, (vz0 - a.vz[c - 1]) * f.idx, a.m2_vzx + c);
    const float dvx_dz = cpml2d(f, 1, c, (a.vx[c + P] - vx0) * f.idz, a.m2_vxz + c);
    a.sxz[c] = a.sxz[c] + (a.B15[c] * dvx_dx + a.B35[c] * dvz_dz + a.B55[c] * (dvz_dx + dvx_dz));
  }
  if (a.io.ssrc && i == a.io.si && k == a.io.sk) {  // stress source: sigma_ij += f_ij(t) dt
    a.sxx[c] += a.io.ssrc[t];
    a.szz[c] += a.io.ssrc[a.io.nstep + t];
    a.sxz[c] += a.io.ssrc[2 * a.io.nstep + t];
  }
}

__global__ void __launch_bounds__(BX * BY) seis2_c2d_velocity_kernel(Seis2Args a, int rel) {
  const int t = a.io.ctl->base + rel;
  const int i = blockIdx.x * BX + threadIdx.x;
  const int k = blockIdx.y * BY + threadIdx.y;
  const int NX = a.NX, NZ = a.NZ, P = a.P;
  float norm = 0.0f;
  if (i < NX && k < NZ) {
    const size_t c = (size_t)k * P + i;
    const Cpml2d& f = a.c2d;
    const bool interior = (i >= 1) && (i <= NX - 2) && (k >= 1) && (k <= NZ - 2);
    float vx = 0.f, vz = 0.f;
    // The memory variables advance on the whole loop range, edges included
    // (the Dirichlet step zeroes the velocity afterwards).
    if (k >= 1 && i >= 1) {  // vx loop, :317-336
      const float d1 = cpml2d(f, 0, c, (a.sxx[c] - a.sxx[c - 1]) * f.idx, a.m_sxx_x + c);
      const float d2 = cpml2d(f, 0, c, (a.sxz[c] - a.sxz[c - P]) * f.idz, a.m_sxz_z + c);
      if (interior) {
        vx = a.vx[c];
        if (a.atten) vx *= a.gxp[c];
        vx = vx + (d1 + d2) * a.dtrx[c];
      }
    }
    if (k <= NZ - 2 && i <= NX - 2) {  // vz loop, :338-357
      const float d1 = cpml2d(f, 1, c, (a.sxz[c + 1] - a.sxz[c]) * f.idx, a.m_sxz_x + c);
      const float d2 = cpml2d(f, 1, c, (a.szz[c + P] - a.szz[c]) * f.idz, a.m_szz_z + c);
      if (interior) {
        vz = a.vz[c];
        if (a.atten) vz *= a.gzp[c];
        vz = vz + (d1 + d2) * a.dtrz[c];
      }
    }
    if (i == a.io.si && k == a.io.sk) {  // :360-361
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

}  // namespace

void em2_c2d_half1(const Em2Args& a, const Launch& L, int rel, cudaStream_t s) {
  em2_c2d_h_kernel<<<L.grid, L.block, 0, s>>>(a, rel);
}
void em2_c2d_half2(const Em2Args& a, const Launch& L, int rel, cudaStream_t s) {
  em2_c2d_e_kernel<<<L.grid, L.block, 0, s>>>(a, rel);
}
void seis2_c2d_half1(const Seis2Args& a, const Launch& L, int rel, cudaStream_t s) {
  seis2_c2d_stress_kernel<<<L.grid, L.block, 0, s>>>(a, rel);
}
void seis2_c2d_half2(const Seis2Args& a, const Launch& L, int rel, cudaStream_t s) {
  seis2_c2d_velocity_kernel<<<L.grid, L.block, 0, s>>>(a, rel);
}

}  // namespace sfd
