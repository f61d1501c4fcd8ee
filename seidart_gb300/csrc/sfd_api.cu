// C ABI, part 1: handle management, FP64 host-side coefficient folding, the
// state layout in the caller's device buffer, and the time loop (on chip in
// one launch, or CUDA graphs of 32 steps of one or two kernels).  Part 2
// (sfd_batch_api.cu) holds the batched runs, part 3 (sfd_adjoint.cu) the
// checkpoints and the adjoints; handle.h the handle they share.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <complex>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "handle.h"
#include "host_pool.h"

namespace sfd {

__global__ void k_begin(Ctl* ctl, float* slots, int nslots, int step) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  for (int s = tid; s < nslots; s += gridDim.x * blockDim.x) slots[s] = 0.0f;
  if (tid == 0) {
    ctl->base = step;
    ctl->run_start = step;
    ctl->maxnorm = 0.0f;
    ctl->nan_seen = 0;
    ctl->err = 0;
  }
}

__global__ void k_advance(Ctl* ctl, int by) { ctl->base += by; }

__global__ void k_reduce_slots(Ctl* ctl, const float* slots, int nslots) {
  float m = 0.0f;
  for (int s = threadIdx.x; s < nslots; s += blockDim.x) m = fmaxf(m, slots[s]);
  __shared__ float red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) ctl->maxnorm = m;
  }
}

}  // namespace sfd

using namespace sfd;

namespace sfd {

void begin_run(sfd_handle_s* h, int64_t step) {
  const Layout& L = h->L;
  k_begin<<<std::min(1024, (L.nslots + 255) / 256 + 1), 256, 0, h->stream>>>(
      (Ctl*)(h->base + L.off_ctl), (float*)(h->base + L.off_slots), L.nslots, (int)step);
}

void reduce_norms(sfd_handle_s* h) {
  const Layout& L = h->L;
  k_reduce_slots<<<1, 1024, 0, h->stream>>>((Ctl*)(h->base + L.off_ctl), (const float*)(h->base + L.off_slots),
                                            L.nslots);
}

}  // namespace sfd

namespace sfd {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(SFD_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

}  // namespace sfd

namespace sfd {
// Replace the calling thread's error message (used by the static-scratch entry point).
void set_error(const char* msg) { g_err = msg ? msg : ""; }
}  // namespace sfd

namespace sfd {

int nfields(int kind) {
  switch (kind) {
    case SFD_SEISMIC2: return 5;
    case SFD_SEISMIC25: return 9;
    case SFD_ELECTROMAG2: return 3;
    case SFD_ELECTROMAG25: return 6;
    case SFD_ELECTROMAG2C: return 6;  // Ex Ez Hy, real and imaginary planes
  }
  return 0;
}
int nchan(int kind) {
  if (kind == SFD_ELECTROMAG2C) return 4;  // Ex re, Ex im, Ez re, Ez im
  return (kind == SFD_SEISMIC25 || kind == SFD_ELECTROMAG25) ? 3 : 2;
}
// Source components the caller gives (real time functions, x [y] z).
int nsrc(int kind) { return kind == SFD_ELECTROMAG2C ? 2 : nchan(kind); }
// Stress source components (sfd_set_stress_source): xx zz xz in 2-D, xx yy zz xy xz yz in 2.5-D.
int nstress(int kind) { return kind == SFD_SEISMIC2 ? 3 : (kind == SFD_SEISMIC25 ? 6 : 0); }
// Density method of the flags: 0 arithmetic, 1 none, 2 geometric, 3 harmonic.
int density_method(int flags) { return (flags & SFD_FLAG_DENSITY_MASK) / SFD_FLAG_DENSITY_NONE; }
int nplanes(int kind) {
  switch (kind) {
    case SFD_SEISMIC2: return 9;
    case SFD_SEISMIC25: return 25;
    case SFD_ELECTROMAG2: return 6;
    case SFD_ELECTROMAG25: return 12;
    case SFD_ELECTROMAG2C: return 9;
  }
  return 0;
}
bool is3(int kind) { return kind == SFD_SEISMIC25 || kind == SFD_ELECTROMAG25; }

// Strip axis of each memory variable, in the oracle's order.
const char* mem_axes(int kind) {
  switch (kind) {
    case SFD_ELECTROMAG2: return "zxzx";              // dEx_dz dEz_dx dHy_dz dHy_dx
    case SFD_SEISMIC2: return "xzzxxzxzxzzx";  // dvx_dx dvz_dz dvx_dz dvz_dx dsxx_dx dszz_dz dsxz_dx dsxz_dz,
                                                // then the sigmaxz loop's own dvx_dx dvz_dz dvx_dz dvz_dx
    case SFD_SEISMIC25: return "xyzxyzxyzxyzxyxzyz";  // dv{x,y,z}_d{x,y,z}, dsxx_dx dsyy_dy dszz_dz dsxy_dx dsxy_dy dsxz_dx dsxz_dz dsyz_dy dsyz_dz
    case SFD_ELECTROMAG25: return "yzzxyxyzxzyx";     // dEz_dy dEy_dz dEx_dz dEz_dx dEx_dy dEy_dx dHz_dy dHy_dz dHz_dx dHx_dz dHx_dy dHy_dx
    case SFD_ELECTROMAG2C: return "zzxxzzxx";         // dEx_dz dEz_dx dHy_dz dHy_dx, each real then imaginary
  }
  return "";
}
int ncoef(int kind) {
  switch (kind) {
    case SFD_SEISMIC2: return 12;   // A11 A13 A15 A33 A35 B15 B35 B55 (averaged, x dt), dt/rho, dt/rho_avg, 1-gx, 1-gz
    case SFD_SEISMIC25: return 39;  // 33 averaged C x dt (stress loops), 3 dt/rho_avg, 3 (1 - gamma)
    case SFD_ELECTROMAG2: return 4;
    case SFD_ELECTROMAG25: return 6;
    case SFD_ELECTROMAG2C: return 8;  // CAx CBx CAz CBz, each real then imaginary
  }
  return 0;
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

int choose_ysplit(const sfd_config& c) {
  if (!is3(c.kind)) return 1;
#ifdef SFD_YSPLIT
  return std::max(1, std::min(SFD_YSPLIT, c.ny));  // build-time override for tuning sweeps
#endif
  // enough columns x segments to fill 152 SMs a few times over, segments of
  // at least 4 cells: each segment pays its staging ring's fill once, so the
  // TMA-staged march favours longer segments than the plain one did (on the
  // 630 x 70 x 330 seismic25 grid 4 segments of 18 planes ran at 26.2
  // Gcell-updates/s, 8 of 9 planes at 24.8, 2 at 25.3, 1 at 23.7)
  const long cols = (long)c.nx * c.nz;
  int s = 1;
  while (cols * s < 152L * 1024 * 4 && s * 4 <= c.ny) s *= 2;
  return s;
}

// Whether the single-pass 2-D steps keep memory variable q in two copies
// (those of the first half-step, re-derived on tile halos).
bool pingpong_mem(int kind, int q) {
  switch (kind) {
    case SFD_ELECTROMAG2: return q < 2;                // dEx_dz dEz_dx
    case SFD_SEISMIC2: return q < 4 || (q >= 8 && q < 12);  // the velocity-gradient ones of both stress loops
  }
  return false;
}
bool has_single_pass(int kind) { return kind == SFD_ELECTROMAG2 || kind == SFD_SEISMIC2; }
bool cpml2d(const sfd_config& c) { return (c.flags & SFD_FLAG_CPML_2D) != 0; }
// Whether a handle steps in the single-pass form (the others: two kernels per step).
bool single_pass(const sfd_config& c) {
  return has_single_pass(c.kind) && !(c.flags & (SFD_FLAG_TWO_PASS | SFD_FLAG_CPML_2D));
}

// Edge fields of an on-chip run (resident.h): electromag2 2, seismic2 6.
int res_edge_fields(int kind) { return kind == SFD_SEISMIC2 ? 6 : 2; }

int grid_slots(const sfd_config& c, int P, int ysplit) {
  (void)P;
  if (is3(c.kind)) return ((c.nx + 31) / 32) * ((c.nz + 3) / 4) * ysplit;
  return ((c.nx + 31) / 32) * ((c.nz + 7) / 8);
}

int validate_cfg(const sfd_config* c) {
  if (!c) return fail(SFD_ERR_BAD_ARG, "config is NULL");
  if (c->kind < SFD_SEISMIC2 || c->kind > SFD_ELECTROMAG2C) return fail(SFD_ERR_BAD_ARG, "unknown solver kind %d", c->kind);
  const bool three = is3(c->kind);
  if (c->npml < 1) return fail(SFD_ERR_BAD_ARG, "npml must be >= 1 (got %d)", c->npml);
  if (c->nx < 2 * c->npml + 2 || c->nz < 2 * c->npml + 2)
    return fail(SFD_ERR_BAD_ARG, "grid %dx%d too small for npml=%d", c->nx, c->nz, c->npml);
  if (three && c->ny < 2 * c->npml + 2) return fail(SFD_ERR_BAD_ARG, "ny=%d too small for npml=%d", c->ny, c->npml);
  if (!three && c->ny != 1) return fail(SFD_ERR_BAD_ARG, "2-D solvers need ny = 1 (got %d)", c->ny);
  if (c->nstep < 1) return fail(SFD_ERR_BAD_ARG, "nstep must be >= 1");
  if (c->nrec < 0) return fail(SFD_ERR_BAD_ARG, "nrec must be >= 0");
  if ((c->flags & ~(SFD_FLAG_TWO_PASS | SFD_FLAG_STREAMING | SFD_FLAG_LEGACY_QUIRKS | SFD_FLAG_DENSITY_MASK |
                    SFD_FLAG_CPML_2D)) != 0)
    return fail(SFD_ERR_BAD_ARG, "unknown flags 0x%x", c->flags);
  if ((c->flags & SFD_FLAG_CPML_2D) && c->kind != SFD_ELECTROMAG2 && c->kind != SFD_SEISMIC2)
    return fail(SFD_ERR_BAD_ARG, "SFD_FLAG_CPML_2D applies to electromag2 and seismic2");
  if ((c->flags & SFD_FLAG_CPML_2D) && (c->flags & SFD_FLAG_LEGACY_QUIRKS))
    return fail(SFD_ERR_BAD_ARG, "SFD_FLAG_CPML_2D excludes SFD_FLAG_LEGACY_QUIRKS (the legacy loops read 1-D profiles)");
  if ((c->flags & (SFD_FLAG_LEGACY_QUIRKS | SFD_FLAG_DENSITY_MASK)) && c->kind != SFD_SEISMIC2 && c->kind != SFD_SEISMIC25)
    return fail(SFD_ERR_BAD_ARG, "SFD_FLAG_LEGACY_QUIRKS and the density flags apply to the seismic kinds only");
  if (!(c->dt > 0) || !(c->dx > 0) || !(c->dz > 0) || (three && !(c->dy > 0)))
    return fail(SFD_ERR_BAD_ARG, "dt and grid steps must be positive");
  const double cells = (double)c->nx * c->ny * c->nz;
  if (cells > 2.0e9) return fail(SFD_ERR_BAD_ARG, "grid of %.3g cells exceeds the 2^31 index range", cells);
  return SFD_OK;
}

void make_layout(const sfd_config& c, Layout* L) {
  L->NX = c.nx; L->NY = c.ny; L->NZ = c.nz; L->W = c.npml;
  L->P = (c.nx + 31) & ~31;
  L->ysplit = choose_ysplit(c);
  L->nslots = grid_slots(c, L->P, L->ysplit);
  L->fsz = (size_t)L->P * c.ny * c.nz;
  size_t o = 0;
  L->off_ctl = o; o += 256;
  L->off_fields = o; o += align256(sizeof(float) * L->fsz * nfields(c.kind));
  const char* ax = mem_axes(c.kind);
  const int nm = (int)strlen(ax);
  for (int m = 0; m < 18; ++m) { L->off_mem[m] = 0; L->mem_sz[m] = 0; }
  for (int m = 0; m < nm; ++m) {
    size_t n = 0;
    if (cpml2d(c)) n = (size_t)L->P * c.nz;  // 2-D CPML fields: every memory variable on the full grid
    else if (ax[m] == 'x') n = (size_t)c.ny * c.nz * 2 * c.npml;
    else if (ax[m] == 'y') n = (size_t)c.nz * 2 * c.npml * L->P;
    else n = (size_t)2 * c.npml * c.ny * L->P;
    L->off_mem[m] = o; L->mem_sz[m] = n;
    o += align256(sizeof(float) * n);
  }
  L->off_fieldsB = 0;
  for (int m = 0; m < 18; ++m) L->off_memB[m] = 0;
  if (single_pass(c)) {
    L->off_fieldsB = o; o += align256(sizeof(float) * L->fsz * nfields(c.kind));
    for (int m = 0; m < nm; ++m)
      if (pingpong_mem(c.kind, m)) { L->off_memB[m] = o; o += align256(sizeof(float) * L->mem_sz[m]); }
  }
  L->coef_plane = (size_t)L->P * c.nz;
  // the update coefficients, then (2-D CPML fields) 1/K, a, b of the full and half offsets
  L->off_coef = o; o += align256(sizeof(float) * L->coef_plane * (ncoef(c.kind) + (cpml2d(c) ? 6 : 0)));
  const int nax = is3(c.kind) ? 3 : 2;
  const int lens[3] = {c.nx, is3(c.kind) ? c.ny : c.nz, c.nz};
  for (int a = 0; a < 3; ++a) L->off_axis[a] = 0;
  for (int a = 0; a < nax; ++a) { L->off_axis[a] = o; o += align256(sizeof(float) * 6 * axis_stride(lens[a])); }
  L->off_q3 = o; o += align256(sizeof(float) * c.nz);
  L->off_src = o; o += align256(sizeof(float) * (size_t)(nchan(c.kind) + nstress(c.kind)) * c.nstep);
  L->off_rec = o; o += align256(sizeof(int) * 3 * (size_t)std::max(1, c.nrec));
  L->off_traces = o; o += align256(sizeof(float) * (size_t)c.nstep * nchan(c.kind) * std::max(1, c.nrec));
  L->off_slots = o; o += align256(sizeof(float) * L->nslots);  // ZB = 1 tiles: the largest grid
  L->off_res = 0;
  if (single_pass(c) && !(c.flags & SFD_FLAG_STREAMING)) {
    L->off_res = o;  // edge arrays of on-chip runs
    o += align256(res_scratch_bytes(L->P, c.nz, res_edge_fields(c.kind)));
  }
  L->total = o;
}

}  // namespace sfd


namespace sfd {

// Rows per thread of the single-pass tiles: two when two-row tiles fill the
// SMs several times over, else one -- on smaller grids the step waits on
// L2, and more, smaller blocks keep more loads in flight (measured on the
// 440 x 240 seismic2 and 1040 x 540 electromag2 grids).
int single_pass_zb(int kind, int nx, int nz) {
#ifdef SFD_SP_ZB
  return SFD_SP_ZB;  // build-time override for tuning sweeps
#endif
  const long tw = kind == SFD_ELECTROMAG2 ? 128 : 32;  // tile width
  const long tiles2 = ((nx + tw - 1) / tw) * (long)((nz + 15) / 16);
  return tiles2 >= 8L * 152 ? 2 : 1;
}

// The 2-D CPML planes of a SFD_FLAG_CPML_2D handle (after the update
// coefficients), empty otherwise.
Cpml2d cpml2d_args(const sfd_handle* h) {
  Cpml2d f;
  const bool on = cpml2d(h->cfg);
  const int nc = ncoef(h->cfg.kind);
  for (int o = 0; o < 2; ++o) {
    f.ik[o] = on ? h->coef(nc + 3 * o) : nullptr;
    f.a[o] = on ? h->coef(nc + 3 * o + 1) : nullptr;
    f.b[o] = on ? h->coef(nc + 3 * o + 2) : nullptr;
  }
  f.idx = (float)(1.0 / h->cfg.dx);
  f.idz = (float)(1.0 / h->cfg.dz);
  return f;
}

// false when the driver refuses a TMA descriptor (seismic25)
bool bind_args(sfd_handle* h) {
  const Layout& L = h->L;
  const sfd_config& c = h->cfg;
  const int NX = c.nx, NY = c.ny, NZ = c.nz;
  const IoArgs io = h->io();
  switch (c.kind) {
    case SFD_ELECTROMAG2: {
      Em2Args& a = h->em2;
      a.NX = NX; a.NZ = NZ; a.P = L.P; a.W = L.W;
      a.Ex = h->fc(0, 0); a.Ez = h->fc(1, 0); a.Hy = h->fc(2, 0);
      a.mExz = h->mc(0, 0); a.mEzx = h->mc(1, 0); a.mHyz = h->mc(2, 0); a.mHyx = h->mc(3, 0);
      a.CAx = h->coef(0); a.CBx = h->coef(1); a.CAz = h->coef(2); a.CBz = h->coef(3);
      a.X = make_axis(h->axis(0), NX); a.Z = make_axis(h->axis(1), NZ);
      a.dbH = (float)(c.dt / kMu0);
      a.c2d = cpml2d_args(h);
      a.io = io;
      h->launch = em2_launch(a);
      for (int p = 0; p < 2 && h->single; ++p) {
        Em2Step& b = h->em2s[p];
        b.NX = NX; b.NZ = NZ; b.P = L.P; b.W = L.W;
        b.Ex0 = h->fc(0, p); b.Ez0 = h->fc(1, p); b.Hy0 = h->fc(2, p);
        b.mExz0 = h->mc(0, p); b.mEzx0 = h->mc(1, p);
        b.Ex1 = h->fc(0, 1 - p); b.Ez1 = h->fc(1, 1 - p); b.Hy1 = h->fc(2, 1 - p);
        b.mExz1 = h->mc(0, 1 - p); b.mEzx1 = h->mc(1, 1 - p);
        b.mHyz = h->mc(2, 0); b.mHyx = h->mc(3, 0);
        b.mHyz0 = b.mHyz; b.mHyx0 = b.mHyx;
        b.CAx = a.CAx; b.CBx = a.CBx; b.CAz = a.CAz; b.CBz = a.CBz;
        b.X = a.X; b.Z = a.Z; b.dbH = a.dbH; b.io = io;
      }
      h->zb = single_pass_zb(c.kind, NX, NZ);
      if (h->single) h->launch1 = em2_step_launch(h->em2s[0], h->zb);
      break;
    }
    case SFD_ELECTROMAG2C: {
      Em2cArgs& a = h->em2c;
      a.NX = NX; a.NZ = NZ; a.P = L.P; a.W = L.W;
      for (int q = 0; q < 2; ++q) {
        a.Ex[q] = h->fc(q, 0); a.Ez[q] = h->fc(2 + q, 0); a.Hy[q] = h->fc(4 + q, 0);
        a.mExz[q] = h->mc(q, 0); a.mEzx[q] = h->mc(2 + q, 0); a.mHyz[q] = h->mc(4 + q, 0); a.mHyx[q] = h->mc(6 + q, 0);
        a.CAx[q] = h->coef(q); a.CBx[q] = h->coef(2 + q); a.CAz[q] = h->coef(4 + q); a.CBz[q] = h->coef(6 + q);
      }
      a.X = make_axis(h->axis(0), NX); a.Z = make_axis(h->axis(1), NZ);
      a.dbH = (float)(c.dt / kMu0);
      a.io = io;
      h->launch = em2c_launch(a);
      break;
    }
    case SFD_SEISMIC2: {
      Seis2Args& a = h->s2;
      a.NX = NX; a.NZ = NZ; a.P = L.P; a.W = L.W; a.atten = 0;
      a.legacy = (c.flags & SFD_FLAG_LEGACY_QUIRKS) ? 1 : 0;
      a.vx = h->fc(0, 0); a.vz = h->fc(1, 0); a.sxx = h->fc(2, 0); a.szz = h->fc(3, 0); a.sxz = h->fc(4, 0);
      a.m_vxx = h->mc(0, 0); a.m_vzz = h->mc(1, 0); a.m_vxz = h->mc(2, 0); a.m_vzx = h->mc(3, 0);
      a.m2_vxx = h->mc(8, 0); a.m2_vzz = h->mc(9, 0); a.m2_vxz = h->mc(10, 0); a.m2_vzx = h->mc(11, 0);
      a.m_sxx_x = h->mc(4, 0); a.m_szz_z = h->mc(5, 0); a.m_sxz_x = h->mc(6, 0); a.m_sxz_z = h->mc(7, 0);
      a.A11 = h->coef(0); a.A13 = h->coef(1); a.A15 = h->coef(2); a.A33 = h->coef(3); a.A35 = h->coef(4);
      a.B15 = h->coef(5); a.B35 = h->coef(6); a.B55 = h->coef(7);
      a.dtrx = h->coef(8); a.dtrz = h->coef(9); a.gxp = h->coef(10); a.gzp = h->coef(11);
      a.q3 = (const float*)(h->base + L.off_q3);
      a.X = make_axis(h->axis(0), NX); a.Z = make_axis(h->axis(1), NZ);
      a.c2d = cpml2d_args(h);
      a.io = io;
      h->launch = seis2_launch(a);
      for (int p = 0; p < 2 && h->single; ++p) {
        Seis2Step& b = h->s2s[p];
        b.NX = NX; b.NZ = NZ; b.P = L.P; b.W = L.W; b.atten = a.atten; b.legacy = a.legacy;
        b.m2_vxx0 = h->mc(8, p); b.m2_vzz0 = h->mc(9, p); b.m2_vxz0 = h->mc(10, p); b.m2_vzx0 = h->mc(11, p);
        b.m2_vxx1 = h->mc(8, 1 - p); b.m2_vzz1 = h->mc(9, 1 - p); b.m2_vxz1 = h->mc(10, 1 - p);
        b.m2_vzx1 = h->mc(11, 1 - p);
        b.vx0 = h->fc(0, p); b.vz0 = h->fc(1, p); b.sxx0 = h->fc(2, p); b.szz0 = h->fc(3, p); b.sxz0 = h->fc(4, p);
        b.vx1 = h->fc(0, 1 - p); b.vz1 = h->fc(1, 1 - p); b.sxx1 = h->fc(2, 1 - p); b.szz1 = h->fc(3, 1 - p);
        b.sxz1 = h->fc(4, 1 - p);
        b.m_vxx0 = h->mc(0, p); b.m_vzz0 = h->mc(1, p); b.m_vxz0 = h->mc(2, p); b.m_vzx0 = h->mc(3, p);
        b.m_vxx1 = h->mc(0, 1 - p); b.m_vzz1 = h->mc(1, 1 - p); b.m_vxz1 = h->mc(2, 1 - p);
        b.m_vzx1 = h->mc(3, 1 - p);
        b.m_sxx_x = h->mc(4, 0); b.m_szz_z = h->mc(5, 0); b.m_sxz_x = h->mc(6, 0); b.m_sxz_z = h->mc(7, 0);
        b.A11 = a.A11; b.A13 = a.A13; b.A15 = a.A15; b.A33 = a.A33; b.A35 = a.A35;
        b.B15 = a.B15; b.B35 = a.B35; b.B55 = a.B55;
        b.dtrx = a.dtrx; b.dtrz = a.dtrz; b.gxp = a.gxp; b.gzp = a.gzp; b.q3 = a.q3;
        b.X = a.X; b.Z = a.Z; b.io = io;
      }
      h->zb = single_pass_zb(c.kind, NX, NZ);
      if (h->single) h->launch1 = seis2_step_launch(h->s2s[0], h->zb);
      break;
    }
    case SFD_SEISMIC25: {
      Seis25Args& a = h->s25;
      a.NX = NX; a.NY = NY; a.NZ = NZ; a.P = L.P; a.W = L.W; a.atten = 0;
      a.legacy = (c.flags & SFD_FLAG_LEGACY_QUIRKS) ? 1 : 0;
      float** F[9] = {&a.vx, &a.vy, &a.vz, &a.sxx, &a.syy, &a.szz, &a.sxy, &a.sxz, &a.syz};
      for (int q = 0; q < 9; ++q) *F[q] = h->f(q);
      // oracle order: dvx_dx dvx_dy dvx_dz dvy_dx dvy_dy dvy_dz dvz_dx dvz_dy dvz_dz
      a.m_vx_x = h->m(0); a.m_vx_y = h->m(1); a.m_vx_z = h->m(2);
      a.m_vy_x = h->m(3); a.m_vy_y = h->m(4); a.m_vy_z = h->m(5);
      a.m_vz_x = h->m(6); a.m_vz_y = h->m(7); a.m_vz_z = h->m(8);
      // dsxx_dx dsyy_dy dszz_dz dsxy_dx dsxy_dy dsxz_dx dsxz_dz dsyz_dy dsyz_dz
      a.m_sxx_x = h->m(9); a.m_syy_y = h->m(10); a.m_szz_z = h->m(11); a.m_sxy_x = h->m(12);
      a.m_sxy_y = h->m(13); a.m_sxz_x = h->m(14); a.m_sxz_z = h->m(15); a.m_syz_y = h->m(16);
      a.m_syz_z = h->m(17);
      a.C = h->coef(0); a.dtr = h->coef(33); a.gp = h->coef(36);
      a.X = make_axis(h->axis(0), NX); a.Y = make_axis(h->axis(1), NY); a.Z = make_axis(h->axis(2), NZ);
      a.idx = (float)(1.0 / c.dx); a.idz = (float)(1.0 / c.dz);
      a.ysplit = L.ysplit;
      a.io = io;
      a.wait_ns = h->wait_ns;
      a.stall_tx = h->stall_waits ? 16u : 0u;
      if (!seis25_make_maps(a, L.fsz, h->axis(1))) return false;
      h->launch = seis25_launch(a);
      break;
    }
    case SFD_ELECTROMAG25: {
      Em25Args& a = h->em25;
      a.NX = NX; a.NY = NY; a.NZ = NZ; a.P = L.P; a.W = L.W;
      a.Ex = h->f(0); a.Ey = h->f(1); a.Ez = h->f(2); a.Hx = h->f(3); a.Hy = h->f(4); a.Hz = h->f(5);
      a.mEz_y = h->m(0); a.mEy_z = h->m(1); a.mEx_z = h->m(2); a.mEz_x = h->m(3); a.mEx_y = h->m(4);
      a.mEy_x = h->m(5); a.mHz_y = h->m(6); a.mHy_z = h->m(7); a.mHz_x = h->m(8); a.mHx_z = h->m(9);
      a.mHx_y = h->m(10); a.mHy_x = h->m(11);
      a.caEx = h->coef(0); a.cbEx = h->coef(1); a.caEy = h->coef(2); a.cbEy = h->coef(3);
      a.caEz = h->coef(4); a.cbEz = h->coef(5);
      a.X = make_axis(h->axis(0), NX); a.Y = make_axis(h->axis(1), NY); a.Z = make_axis(h->axis(2), NZ);
      a.dbH = (float)(c.dt / kMu0);
      a.ysplit = L.ysplit;
      a.io = io;
      a.wait_ns = h->wait_ns;
      a.stall_tx = h->stall_waits ? 16u : 0u;
      if (!em25_make_maps(a, L.fsz, h->axis(1))) return false;
      h->launch = em25_launch(a);
      break;
    }
  }
  return true;
}

void set_io_source(sfd_handle* h, int i, int j, int k) {
  IoArgs* ios[9] = {&h->em2.io, &h->s2.io, &h->s25.io, &h->em25.io, &h->em2c.io,
                    &h->em2s[0].io, &h->em2s[1].io, &h->s2s[0].io, &h->s2s[1].io};
  for (IoArgs* io : ios) { io->si = i; io->sj = j; io->sk = k; }
}

// Whether (i, j, k) is the source cell already set on the handle.
bool same_source_cell(const sfd_handle* h, int i, int j, int k) {
  const IoArgs& io = h->s2.io;  // every argument block holds the same cell
  return io.si == i && io.sj == j && io.sk == k;
}

// Point every argument block at the stress source amplitudes (or at none).
void set_io_ssrc(sfd_handle* h) {
  const IoArgs ref = h->io();
  IoArgs* ios[9] = {&h->em2.io, &h->s2.io, &h->s25.io, &h->em25.io, &h->em2c.io,
                    &h->em2s[0].io, &h->em2s[1].io, &h->s2s[0].io, &h->s2s[1].io};
  for (IoArgs* io : ios) io->ssrc = ref.ssrc;
}

void set_atten(sfd_handle* h, int atten) {
  h->s2.atten = h->s2s[0].atten = h->s2s[1].atten = atten;
  h->s25.atten = atten;
}

// One single-pass step reading copy p (graph capture passes p explicitly).
void launch_step(sfd_handle* h, int p, int rel, cudaStream_t s) {
  if (h->cfg.kind == SFD_ELECTROMAG2) em2_step(h->em2s[p], h->launch1, h->zb, rel, s);
  else seis2_step(h->s2s[p], h->launch1, h->zb, rel, s);
}

void launch_half(sfd_handle* h, int which, int rel, cudaStream_t s) {
  const Launch& L = h->launch;
  switch (h->cfg.kind) {
    case SFD_ELECTROMAG2:
      if (cpml2d(h->cfg)) which == 0 ? em2_c2d_half1(h->em2, L, rel, s) : em2_c2d_half2(h->em2, L, rel, s);
      else which == 0 ? em2_half1(h->em2, L, rel, s) : em2_half2(h->em2, L, rel, s);
      break;
    case SFD_SEISMIC2:
      if (cpml2d(h->cfg)) which == 0 ? seis2_c2d_half1(h->s2, L, rel, s) : seis2_c2d_half2(h->s2, L, rel, s);
      else which == 0 ? seis2_half1(h->s2, L, rel, s) : seis2_half2(h->s2, L, rel, s);
      break;
    case SFD_SEISMIC25: which == 0 ? seis25_half1(h->s25, L, rel, s) : seis25_half2(h->s25, L, rel, s); break;
    case SFD_ELECTROMAG25: which == 0 ? em25_half1(h->em25, L, rel, s) : em25_half2(h->em25, L, rel, s); break;
    case SFD_ELECTROMAG2C: which == 0 ? em2c_half1(h->em2c, L, rel, s) : em2c_half2(h->em2c, L, rel, s); break;
  }
}

void launch_finalize(sfd_handle* h, int t_last, cudaStream_t s) {
  if (h->single) {
    if (h->cfg.kind == SFD_ELECTROMAG2) em2_step_finalize(h->em2s[h->cur], t_last, s);
    else seis2_step_finalize(h->s2s[h->cur], t_last, s);
    return;
  }
  switch (h->cfg.kind) {
    case SFD_ELECTROMAG2: em2_finalize(h->em2, t_last, s); break;
    case SFD_SEISMIC2: seis2_finalize(h->s2, t_last, s); break;
    case SFD_SEISMIC25: seis25_finalize(h->s25, t_last, s); break;
    case SFD_ELECTROMAG25: em25_finalize(h->em25, t_last, s); break;
    case SFD_ELECTROMAG2C: em2c_finalize(h->em2c, t_last, s); break;
  }
}

// Whether runs of this handle can keep the whole state on chip (decided on
// the first run, on the device that is current then).
bool resident_usable(sfd_handle* h) {
  if (h->res_state) return h->res_state > 0;
  h->res_state = -1;
  if (!h->L.off_res || !h->single) return false;
  int dev = 0, nsm = 0, coop = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (!coop) return false;
  const size_t static_smem = 8192;  // receiver list, thread map and reduction buffers of the kernel
  if (h->cfg.kind == SFD_SEISMIC2) {  // a uniform tiling: searched in microseconds, not cached
    Seis2ResPlan plan;
    if (!seis2_resident_plan(h->cfg.nx, h->cfg.nz, std::min(nsm, h->L.nslots), (size_t)optin - static_smem, &plan))
      return false;
    int per_sm = 0;
    if (seis2_resident_prepare(plan, &per_sm) != cudaSuccess || per_sm < 1) {
      cudaGetLastError();
      return false;
    }
    h->s2_plan = plan;
    h->res_state = 1;
    return true;
  }
  // Plans are searched once per grid shape and device (the search takes
  // tens of milliseconds; a survey creates one handle per shot).
  // The forward kernel's plan (interior tiles with kResRows3 rows per
  // thread) and the adjoint sweep's (kResRows everywhere).
  struct PlanKey {
    int nx, nz, npml, ctas, dev;
    size_t smem;
    bool rows3;
  };
  static std::mutex plan_mu;
  static std::vector<std::pair<PlanKey, std::pair<bool, ResPlan>>> plans;
  auto plan_for = [&](bool rows3, ResPlan* plan) {
    const PlanKey key{h->cfg.nx, h->cfg.nz, h->cfg.npml, std::min(nsm, h->L.nslots), dev, (size_t)optin - static_smem,
                      rows3};
    {
      std::lock_guard<std::mutex> lock(plan_mu);
      for (const auto& e : plans)
        if (e.first.nx == key.nx && e.first.nz == key.nz && e.first.npml == key.npml && e.first.ctas == key.ctas &&
            e.first.dev == key.dev && e.first.smem == key.smem && e.first.rows3 == key.rows3) {
          *plan = e.second.second;
          return e.second.first;
        }
    }
    const bool fits = em2_resident_plan(key.nx, key.nz, key.npml, key.ctas, key.smem, plan, rows3);
    std::lock_guard<std::mutex> lock(plan_mu);
    plans.push_back({key, {fits, *plan}});
    return fits;
  };
  ResPlan plan;
  if (!plan_for(true, &plan) || !plan_for(false, &h->res_plan_adj)) return false;
  int per_sm = 0;
  if (em2_resident_prepare(plan, &per_sm) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    return false;
  }
  h->res_plan = plan;
  h->res_state = 1;
  return true;
}

Em2Resident resident_args(const sfd_handle* h, int64_t nsteps) {
  Em2Resident r;
  const Em2Step& b = h->em2s[h->cur];
  r.NX = b.NX; r.NZ = b.NZ; r.P = b.P; r.W = b.W;
  r.Ex = h->fc(0, h->cur); r.Ez = h->fc(1, h->cur); r.Hy = h->fc(2, h->cur);
  r.mExz = h->mc(0, h->cur); r.mEzx = h->mc(1, h->cur); r.mHyz = h->mc(2, 0); r.mHyx = h->mc(3, 0);
  r.CAx = b.CAx; r.CBx = b.CBx; r.CAz = b.CAz; r.CBz = b.CBz;
  r.X = b.X; r.Z = b.Z; r.dbH = b.dbH;
  r.io = b.io;
  r.plan = h->res_plan;
  char* base = h->base + h->L.off_res;
  r.r.erow = (uint2*)base;
  r.r.NZp = res_nzp(h->cfg.nz);
  r.r.ecol = r.r.erow + 4 * kResMaxTiles1D * (size_t)h->L.P;
  r.t0 = (int)h->step;
  r.nsteps = (int)nsteps;
  r.limit_ns = h->wait_ns;
  r.tag_bias = h->stall_waits ? kStallTagBias : 0u;
  r.dump = ResDump{nullptr, 0, {0, 0, 0, 0, 0, 0, 0}};
  r.ckpt = ResDump{nullptr, 0, {0, 0, 0, 0, 0, 0, 0}};
  r.ckpt_every = 0;
  return r;
}

Seis2Resident seis2_resident_args(const sfd_handle* h, int64_t nsteps) {
  Seis2Resident r;
  const Seis2Step& b = h->s2s[h->cur];
  const int p = h->cur;
  r.NX = b.NX; r.NZ = b.NZ; r.P = b.P; r.W = b.W; r.atten = b.atten; r.legacy = b.legacy;
  r.vx = h->fc(0, p); r.vz = h->fc(1, p); r.sxx = h->fc(2, p); r.szz = h->fc(3, p); r.sxz = h->fc(4, p);
  r.m_vxx = h->mc(0, p); r.m_vzz = h->mc(1, p); r.m_vxz = h->mc(2, p); r.m_vzx = h->mc(3, p);
  r.m2_vxx = h->mc(8, p); r.m2_vzz = h->mc(9, p); r.m2_vxz = h->mc(10, p); r.m2_vzx = h->mc(11, p);
  r.m_sxx_x = h->mc(4, 0); r.m_szz_z = h->mc(5, 0); r.m_sxz_x = h->mc(6, 0); r.m_sxz_z = h->mc(7, 0);
  const float* cf[12] = {b.A11, b.A13, b.A15, b.A33, b.A35, b.B15, b.B35, b.B55, b.dtrx, b.dtrz, b.gxp, b.gzp};
  for (int q = 0; q < 12; ++q) r.coef[q] = cf[q];
  r.q3 = b.q3;
  r.X = b.X; r.Z = b.Z;
  r.io = b.io;
  r.plan = h->s2_plan;
  char* base = h->base + h->L.off_res;
  r.r.erow = (uint2*)base;
  r.r.NZp = res_nzp(h->cfg.nz);
  r.r.ecol = r.r.erow + 2 * 6 * kResMaxTiles1D * (size_t)h->L.P;
  r.t0 = (int)h->step;
  r.nsteps = (int)nsteps;
  r.limit_ns = h->wait_ns;
  r.tag_bias = h->stall_waits ? kStallTagBias : 0u;
  r.dump = S2Dump{nullptr, 0, {}};
  return r;
}

int ensure_graph(sfd_handle* h, int p) {
  if (h->graph[p]) return SFD_OK;
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal));
  for (int s = 0; s < kGraphSteps; ++s) {
    if (h->single) {
      launch_step(h, (p + s) & 1, s, h->cap_stream);
    } else {
      launch_half(h, 0, s, h->cap_stream);
      launch_half(h, 1, s, h->cap_stream);
    }
  }
  k_advance<<<1, 1, 0, h->cap_stream>>>((Ctl*)(h->base + h->L.off_ctl), kGraphSteps);
  cudaError_t e = cudaStreamEndCapture(h->cap_stream, &g);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&h->graph[p], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) { h->graph[p] = nullptr; return cuda_fail(e, "cudaGraphInstantiate"); }
  return SFD_OK;
}

void invalidate_graph(sfd_handle* h) {
  for (int p = 0; p < 2; ++p)
    if (h->graph[p]) { cudaGraphExecDestroy(h->graph[p]); h->graph[p] = nullptr; }
  if (h->adj_graph) { cudaGraphExecDestroy(h->adj_graph); h->adj_graph = nullptr; }
}

// Host rows of NX floats -> device rows of pitch P.
int upload_pitched(sfd_handle* h, float* dst, const float* src, size_t rows) {
  CK(cudaMemcpy2DAsync(dst, sizeof(float) * h->L.P, src, sizeof(float) * h->cfg.nx, sizeof(float) * h->cfg.nx, rows,
                       cudaMemcpyHostToDevice, h->stream));
  return SFD_OK;
}

bool check_strip(const double* v, int n, int W) {
  for (int i = W; i < n - W; ++i)
    if (v[i] != 0.0) return false;
  return true;
}

// f(begin, end) over [0, n) in contiguous chunks on the host pool, each
// with at least `grain` items (the calling thread alone for small n).  The
// model set-up's FP64 loops and copies run this way: a 1040 x 540
// electromag2 model is 27 MB of input planes.
template <class F>
void parallel_for(size_t n, const F& f, size_t grain = 1u << 15) {
  const size_t want = std::max<size_t>(1, n / std::max<size_t>(1, grain));
  if (want <= 1) {
    f((size_t)0, n);
    return;
  }
  HostPool& pool = HostPool::get();
  const size_t nt = std::min<size_t>(pool.size(), want);
  const size_t chunk = (n + nt - 1) / nt;
  pool.run((int)nt, [&](int t) {
    const size_t b = std::min(n, (size_t)t * chunk), e = std::min(n, b + chunk);
    if (b < e) f(b, e);
  });
}

// rows [0, nrows) of `ncols` values each, split between threads by whole rows
template <class F>
void parallel_rows(int nrows, int ncols, const F& row) {
  parallel_for((size_t)nrows, [&](size_t b, size_t e) {
    for (size_t k = b; k < e; ++k) row((int)k);
  }, std::max<size_t>(1, (1u << 15) / (size_t)std::max(1, ncols)));
}

// The lowest index reported by any thread (`none` if none was).
struct FirstBad {
  std::atomic<size_t> v;
  explicit FirstBad(size_t none) : v(none) {}
  void note(size_t q) {
    size_t cur = v.load();
    while (q < cur && !v.compare_exchange_weak(cur, q)) {
    }
  }
};

void par_copy(double* dst, const double* src, size_t n) {
  parallel_for(n, [&](size_t b, size_t e) { std::memcpy(dst + b, src + b, sizeof(double) * (e - b)); });
}

bool all_finite(const double* v, size_t n) {
  std::atomic<bool> ok{true};
  parallel_for(n, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i)
      if (!std::isfinite(v[i])) {
        ok = false;
        return;
      }
  });
  return ok;
}

}  // namespace sfd

extern "C" {

int32_t sfd_version(void) { return 100; }

const char* sfd_last_error(void) { return g_err.c_str(); }

int32_t sfd_model_planes(int32_t kind) { return nplanes(kind); }
int32_t sfd_num_fields(int32_t kind) { return nfields(kind); }
int32_t sfd_num_channels(int32_t kind) { return nfields(kind) ? nchan(kind) : 0; }
int32_t sfd_num_memory(int32_t kind) { return (int32_t)strlen(mem_axes(kind)); }

int32_t sfd_state_bytes(const sfd_config* cfg, size_t* bytes) {
  g_err.clear();
  int r = validate_cfg(cfg);
  if (r) return r;
  if (!bytes) return fail(SFD_ERR_BAD_ARG, "bytes is NULL");
  Layout L;
  make_layout(*cfg, &L);
  *bytes = L.total;
  return SFD_OK;
}

int32_t sfd_create(const sfd_config* cfg, void* dev_state, size_t state_bytes, void* stream, sfd_handle** out) {
  return sfd::create_handle(cfg, dev_state, state_bytes, stream, true, out);
}

}  // extern "C"

namespace sfd {

// Handle creation; `graphs` = false creates no capture stream and runs every
// step with plain launches.
int32_t create_handle(const sfd_config* cfg, void* dev_state, size_t state_bytes, void* stream, bool graphs,
                      sfd_handle** out) {
  g_err.clear();
  int r = validate_cfg(cfg);
  if (r) return r;
  if (!out) return fail(SFD_ERR_BAD_ARG, "out is NULL");
  *out = nullptr;
  Layout L;
  make_layout(*cfg, &L);
  if (!dev_state) return fail(SFD_ERR_BAD_ARG, "device state buffer is NULL");
  if (((uintptr_t)dev_state & 255) != 0) return fail(SFD_ERR_BAD_ARG, "device state buffer must be 256-byte aligned");
  if (state_bytes < L.total)
    return fail(SFD_ERR_BAD_ARG, "device state buffer has %zu bytes, needs %zu", state_bytes, L.total);
  cudaPointerAttributes attr;
  cudaError_t e = cudaPointerGetAttributes(&attr, dev_state);
  if (e != cudaSuccess || attr.type != cudaMemoryTypeDevice) {
    cudaGetLastError();
    return fail(SFD_ERR_BAD_ARG, "state buffer is not device memory");
  }
  sfd_handle* h = new sfd_handle_s();
  h->cfg = *cfg;
  h->L = L;
  h->base = (char*)dev_state;
  h->stream = (cudaStream_t)stream;
  h->single = single_pass(*cfg);
  h->cap_stream = nullptr;
  if (graphs) {
    e = cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete h; return cuda_fail(e, "cudaStreamCreateWithFlags"); }
  }
  if (!bind_args(h)) {
    if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
    delete h;
    return fail(SFD_ERR_CUDA, "could not set up the 2.5-D kernels' staged tiles (tensor maps or shared-memory size)");
  }
  e = cudaMemsetAsync(h->base, 0, L.total, h->stream);
  if (e != cudaSuccess) { cudaStreamDestroy(h->cap_stream); delete h; return cuda_fail(e, "cudaMemsetAsync"); }
  *out = h;
  return SFD_OK;
}

// Model plane (sfd_set_model's order) the source amplitude q is divided by,
// for the kinds sfd_set_model_ids takes: electromag2 eps11, eps33;
// electromag25 eps11, eps22, eps33; seismic2 and seismic25 rho.
int src_full_plane(int kind, int q) {
  switch (kind) {
    case SFD_ELECTROMAG2: return q == 0 ? 0 : 2;
    case SFD_ELECTROMAG25: return q == 0 ? 0 : (q == 1 ? 3 : 5);
    case SFD_SEISMIC25: return 21;
  }
  return 6;
}

// Divisor of source component q at cell n (host FP64 value of the model).
int source_divisor(sfd_handle* h, int q, size_t n, double* out) {
  if (!h->mat_ids) {
    *out = h->src_scale(q)[n];
    return SFD_OK;
  }
  int32_t id = 0;
  CK(cudaMemcpyAsync(&id, h->mat_ids + n, sizeof id, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  const int np = nplanes(h->cfg.kind);
  *out = (*h->mat_table)[(size_t)id * np + src_full_plane(h->cfg.kind, q)];
  return SFD_OK;
}

// The FP64 model planes of an id-map model, expanded on the host when first
// needed (the electromag2 adjoint's chain rule reads all six).
int ensure_model_planes(sfd_handle* h) {
  if (!h->mat_ids || h->model) return SFD_OK;
  const size_t N2 = (size_t)h->cfg.nx * h->cfg.nz;
  const int np = nplanes(h->cfg.kind);
  std::vector<int32_t> ids(N2);
  CK(cudaMemcpyAsync(ids.data(), h->mat_ids, sizeof(int32_t) * N2, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  std::shared_ptr<double[]> model(new double[(size_t)np * N2]);
  const std::vector<double>& t = *h->mat_table;
  parallel_for(N2, [&](size_t b, size_t e) {
    for (size_t n = b; n < e; ++n)
      for (int q = 0; q < np; ++q) model[(size_t)q * N2 + n] = t[(size_t)ids[n] * np + q];
  });
  h->model = std::move(model);
  for (int q = 0; q < 4; ++q) h->src_plane[q] = src_full_plane(h->cfg.kind, q);  // all planes kept
  return SFD_OK;
}

}  // namespace sfd

extern "C" {

int32_t sfd_set_model_ids(sfd_handle* h, const int32_t* dev_ids, int32_t nmat, const double* table, int64_t count) {
  g_err.clear();
  if (!h || !dev_ids || !table) return fail(SFD_ERR_BAD_ARG, "NULL argument");
  h->adj_rec_n = 0;  // the recorded states no longer follow from the handle
  const sfd_config& c = h->cfg;
  if (c.kind == SFD_ELECTROMAG2C)
    return fail(SFD_ERR_BAD_ARG, "material-id models are implemented for the real-valued kinds");
  const int np = nplanes(c.kind);
  if (nmat < 1 || count != (int64_t)nmat * np)
    return fail(SFD_ERR_BAD_ARG, "table needs nmat >= 1 rows of %d values (count = nmat * %d), got nmat %d, count %lld", np,
                np, nmat, (long long)count);
  if (count > kMatTableMax) return fail(SFD_ERR_BAD_ARG, "table holds at most %d values", kMatTableMax);
  if (!all_finite(table, (size_t)count)) return fail(SFD_ERR_BAD_ARG, "table contains NaN or Inf");
  cudaPointerAttributes attr;
  cudaError_t pe = cudaPointerGetAttributes(&attr, dev_ids);
  if (pe != cudaSuccess || attr.type != cudaMemoryTypeDevice) {
    cudaGetLastError();
    return fail(SFD_ERR_BAD_ARG, "ids must be device memory");
  }
  int atten = 0;
  for (int m = 0; m < nmat; ++m) {  // the checks of sfd_set_model, per material
    const double* t = table + (size_t)m * np;
    if (c.kind == SFD_ELECTROMAG2) {
      if (!((t[0] + t[1]) * kEps0 > 0) || !((t[1] + t[2]) * kEps0 > 0))
        return fail(SFD_ERR_BAD_ARG, "permittivity must be positive (material %d)", m);
    } else if (c.kind == SFD_ELECTROMAG25) {
      if (!((t[0] + t[1] + t[2]) * kEps0 > 0) || !((t[1] + t[3] + t[4]) * kEps0 > 0) ||
          !((t[2] + t[4] + t[5]) * kEps0 > 0))
        return fail(SFD_ERR_BAD_ARG, "permittivity must be positive (material %d)", m);
    } else if (c.kind == SFD_SEISMIC2) {
      if (!(t[6] > 0)) return fail(SFD_ERR_BAD_ARG, "density must be positive (material %d)", m);
      if (t[7] != 0.0 || t[8] != 0.0) atten = 1;
    } else {
      if (!(t[21] > 0)) return fail(SFD_ERR_BAD_ARG, "density must be positive (material %d)", m);
      if (t[22] != 0.0 || t[23] != 0.0 || t[24] != 0.0) atten = 1;
    }
  }
  MatTable mt;
  mt.nmat = nmat;
  std::memcpy(mt.v, table, sizeof(double) * (size_t)count);
  Ctl* ctl = (Ctl*)(h->base + h->L.off_ctl);
  int* bad = &ctl->pad2;
  CK(cudaMemsetAsync(bad, 0, sizeof(int), h->stream));
  coef_from_ids(c.kind, dev_ids, mt, c.nx, c.nz, h->L.P, c.dt, h->coef(0), h->L.coef_plane, bad, c.flags, h->stream);
  CK(cudaGetLastError());
  int flag = 0;
  CK(cudaMemcpyAsync(&flag, bad, sizeof flag, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (flag) return fail(SFD_ERR_BAD_ARG, "material id outside [0, %d)", nmat);
  if (c.kind == SFD_SEISMIC2 || c.kind == SFD_SEISMIC25)
    set_atten(h, atten);  // any material with attenuation (gamma = 0 cells multiply by 1)
  h->mat_ids = dev_ids;
  h->mat_table = std::make_shared<std::vector<double>>(table, table + count);
  h->model.reset();
  for (int q = 0; q < 4; ++q) h->src_plane[q] = src_full_plane(c.kind, q);
  invalidate_graph(h);
  h->have_model = true;
  return SFD_OK;
}

int32_t sfd_set_model(sfd_handle* h, const double* planes, int64_t count) {
  g_err.clear();
  if (!h || !planes) return fail(SFD_ERR_BAD_ARG, "NULL argument");
  h->adj_rec_n = 0;  // the recorded states no longer follow from the handle
  const sfd_config& c = h->cfg;
  const int NX = c.nx, NZ = c.nz;
  const size_t N2 = (size_t)NX * NZ;
  const int np = nplanes(c.kind);
  if (count != (int64_t)np * (int64_t)N2)
    return fail(SFD_ERR_BAD_ARG, "model needs %d planes of %dx%d = %lld values, got %lld", np, NX, NZ,
                (long long)np * (long long)N2, (long long)count);
  if (!all_finite(planes, (size_t)count)) return fail(SFD_ERR_BAD_ARG, "model contains NaN or Inf");
  const double dt = c.dt;
  // Host buffers are left uninitialised and first touched by the worker
  // threads: zero-filling them on one thread cost more than the arithmetic.
  auto P = [&](int q) { return planes + (size_t)q * N2; };
  auto at = [&](const double* p, int i, int k) { return p[(size_t)i + (size_t)NX * k]; };
  const int nc = ncoef(c.kind);
  std::unique_ptr<float[]> coefs(new float[(size_t)nc * N2]);
  parallel_for((size_t)nc * N2, [&](size_t b, size_t e) { std::memset(coefs.get() + b, 0, sizeof(float) * (e - b)); });
  std::vector<float*> out(nc);
  for (int q = 0; q < nc; ++q) out[q] = coefs.get() + (size_t)q * N2;
  std::vector<int> keep;             // input planes copied into the handle's model
  int src_plane[4] = {0, 0, 0, 0};  // indices into `keep`
  int atten = 0;
  switch (c.kind) {
    case SFD_ELECTROMAG2: {
      // electromagfdtd.f95:164-181
      const double *e11 = P(0), *e13 = P(1), *e33 = P(2), *s11 = P(3), *s13 = P(4), *s33 = P(5);
      std::unique_ptr<double[]> ca[2], cb[2];
      for (int d = 0; d < 2; ++d) { ca[d].reset(new double[N2]); cb[d].reset(new double[N2]); }
      FirstBad bad(N2);  // first cell with a non-positive permittivity
      parallel_rows(NZ, NX, [&](int k) {
        for (size_t q = (size_t)NX * k; q < (size_t)NX * (k + 1); ++q) {
          const double ep[2] = {(e11[q] + e13[q]) * kEps0, (e13[q] + e33[q]) * kEps0};
          const double sg[2] = {s11[q] + s13[q], s13[q] + s33[q]};
          for (int d = 0; d < 2; ++d) {
            if (!(ep[d] > 0)) return bad.note(q);
            ca[d][q] = (1.0 - sg[d] * dt / (2.0 * ep[d])) / (1.0 + sg[d] * dt / (2.0 * ep[d]));
            cb[d][q] = (dt / ep[d]) / (1.0 + sg[d] * dt / (2.0 * ep[d]));
          }
        }
      });
      if (bad.v < N2) return fail(SFD_ERR_BAD_ARG, "permittivity must be positive (cell %zu)", bad.v.load());
      // staggered averages at the Ex points (k >= 1) and the Ez points (i >= 1), :282, :294
      parallel_rows(NZ, NX, [&](int k) {
        for (int i = 0; i < NX; ++i) {
          const size_t n = (size_t)i + (size_t)NX * k;
          if (k >= 1) {
            out[0][n] = (float)((ca[0][n] + ca[0][n - NX]) / 2);
            out[1][n] = (float)((cb[0][n] + cb[0][n - NX]) / 2);
          }
          if (i >= 1) {
            out[2][n] = (float)((ca[1][n] + ca[1][n - 1]) / 2);
            out[3][n] = (float)((cb[1][n] + cb[1][n - 1]) / 2);
          }
        }
      });
      keep = {0, 1, 2, 3, 4, 5};  // all six: the adjoint's chain rule reads them
      src_plane[0] = 0;
      src_plane[1] = 2;
      break;
    }
    case SFD_ELECTROMAG2C: {
      // electromagfdtd.f95:439-451 with complex eps (material_rwc), then the
      // staggered averages of :563 (Ex points, k >= 1) and :574 (Ez points, i >= 1)
      using cd = std::complex<double>;
      std::unique_ptr<cd[]> ca[2], cb[2];
      for (int d = 0; d < 2; ++d) { ca[d].reset(new cd[N2]); cb[d].reset(new cd[N2]); }
      FirstBad bad_re(N2), bad_zero(N2);
      parallel_rows(NZ, NX, [&](int k) {
        for (size_t q = (size_t)NX * k; q < (size_t)NX * (k + 1); ++q) {
          const cd e11(P(0)[q], P(1)[q]), e13(P(2)[q], P(3)[q]), e33(P(4)[q], P(5)[q]);
          const double s11 = P(6)[q], s13 = P(7)[q], s33 = P(8)[q];
          const cd ep[2] = {(e11 + e13) * kEps0, (e13 + e33) * kEps0};
          const double sg[2] = {s11 + s13, s13 + s33};
          for (int d = 0; d < 2; ++d) {
            if (!(ep[d].real() > 0)) return bad_re.note(q);
            ca[d][q] = (1.0 - sg[d] * dt / (2.0 * ep[d])) / (1.0 + sg[d] * dt / (2.0 * ep[d]));
            cb[d][q] = (dt / ep[d]) / (1.0 + sg[d] * dt / (2.0 * ep[d]));
          }
          if (std::norm(e11) == 0.0 || std::norm(e33) == 0.0) return bad_zero.note(q);
        }
      });
      if (bad_re.v <= bad_zero.v && bad_re.v < N2)
        return fail(SFD_ERR_BAD_ARG, "permittivity must have a positive real part (cell %zu)", bad_re.v.load());
      if (bad_zero.v < N2) return fail(SFD_ERR_BAD_ARG, "eps11 and eps33 must be nonzero (cell %zu)", bad_zero.v.load());
      parallel_rows(NZ, NX, [&](int k) {
        for (int i = 0; i < NX; ++i) {
          const size_t n = (size_t)i + (size_t)NX * k;
          if (k >= 1) {
            const cd a = (ca[0][n] + ca[0][n - NX]) / 2.0, b = (cb[0][n] + cb[0][n - NX]) / 2.0;
            out[0][n] = (float)a.real(); out[1][n] = (float)a.imag();
            out[2][n] = (float)b.real(); out[3][n] = (float)b.imag();
          }
          if (i >= 1) {
            const cd a = (ca[1][n] + ca[1][n - 1]) / 2.0, b = (cb[1][n] + cb[1][n - 1]) / 2.0;
            out[4][n] = (float)a.real(); out[5][n] = (float)a.imag();
            out[6][n] = (float)b.real(); out[7][n] = (float)b.imag();
          }
        }
      });
      keep = {0, 1, 4, 5};  // eps11, eps33 (re, im): :581-582
      for (int q = 0; q < 4; ++q) src_plane[q] = q;
      break;
    }
    case SFD_ELECTROMAG25: {
      // electromagfdtd.f95:756-789
      const double *e11 = P(0), *e12 = P(1), *e13 = P(2), *e22 = P(3), *e23 = P(4), *e33 = P(5);
      const double *s11 = P(6), *s12 = P(7), *s13 = P(8), *s22 = P(9), *s23 = P(10), *s33 = P(11);
      FirstBad bad(N2);
      parallel_rows(NZ, NX, [&](int k) {
        for (size_t q = (size_t)NX * k; q < (size_t)NX * (k + 1); ++q) {
          const double ep[3] = {(e11[q] + e12[q] + e13[q]) * kEps0, (e12[q] + e22[q] + e23[q]) * kEps0,
                                (e13[q] + e23[q] + e33[q]) * kEps0};
          const double sg[3] = {s11[q] + s12[q] + s13[q], s12[q] + s22[q] + s23[q], s13[q] + s23[q] + s33[q]};
          for (int d = 0; d < 3; ++d) {
            if (!(ep[d] > 0)) return bad.note(q);
            out[2 * d][q] = (float)((1.0 - sg[d] * dt / (2.0 * ep[d])) / (1.0 + sg[d] * dt / (2.0 * ep[d])));
            out[2 * d + 1][q] = (float)((dt / ep[d]) / (1.0 + sg[d] * dt / (2.0 * ep[d])));
          }
        }
      });
      if (bad.v < N2) return fail(SFD_ERR_BAD_ARG, "permittivity must be positive (cell %zu)", bad.v.load());
      keep = {0, 3, 5};  // eps11 eps22 eps33
      for (int q = 0; q < 3; ++q) src_plane[q] = q;
      break;
    }
    case SFD_SEISMIC2: {
      const double *rho = P(6), *gx = P(7), *gz = P(8);
      const int dm = density_method(c.flags);
      const bool legacy = (c.flags & SFD_FLAG_LEGACY_QUIRKS) != 0;
      // loop-1 points (i <= NX-2, k >= 1): (c(i+1,k) + 2 c(i,k) + c(i,k-1)) / 4 for c11 c13 c15 c33 c35
      // loop-2 points (k <= NZ-2, i >= 1): (c(i,k+1) + 2 c(i,k) + c(i-1,k)) / 4 for c15 c35 c55
      const int A_src[5] = {0, 1, 2, 3, 4}, B_src[3] = {2, 4, 5};
      FirstBad bad(N2);
      std::atomic<int> any_atten{0};
      parallel_rows(NZ, NX, [&](int k) {
        for (size_t n = (size_t)NX * k; n < (size_t)NX * (k + 1); ++n)
          if (!(rho[n] > 0)) return bad.note(n);
        for (int i = 0; i < NX; ++i) {
          const size_t n = (size_t)i + (size_t)NX * k;
          if (i <= NX - 2 && k >= 1)
            for (int q = 0; q < 5; ++q) {
              const double* cc = P(A_src[q]);
              out[q][n] = (float)((cc[n + 1] + 2 * cc[n] + cc[n - NX]) / 4 * dt);
            }
          if (k <= NZ - 2 && i >= 1)
            for (int q = 0; q < 3; ++q) {
              const double* cc = P(B_src[q]);
              out[5 + q][n] = (float)((cc[n + NX] + 2 * cc[n] + cc[n - 1]) / 4 * dt);
            }
        }
        int a = 0;
        for (int i = 0; i < NX; ++i) {
          const size_t n = (size_t)i + (size_t)NX * k;
          // vx: the cell's own rho with the legacy quirks (seismicfdtd.f95:334),
          // else the average the Fortran forms at :320, by the density method
          if (legacy || i < 1 || k < 1)
            out[8][n] = (float)(dt / rho[n]);
          else
            out[8][n] = (float)(dt / rho_avg(dm, 2, rho[n], at(rho, i - 1, k), at(rho, i, k - 1)));
          if (i <= NX - 2 && k <= NZ - 2)  // vz: the average of :342, by the density method (:355)
            out[9][n] = (float)(dt / rho_avg(dm, 2, rho[n], at(rho, i + 1, k), at(rho, i, k + 1)));
          out[10][n] = (float)(1.0 - gx[n]);
          out[11][n] = (float)(1.0 - gz[n]);
          if (gx[n] != 0.0 || gz[n] != 0.0) a = 1;
        }
        if (a) any_atten = 1;
      });
      if (bad.v < N2) return fail(SFD_ERR_BAD_ARG, "density must be positive (cell %zu)", bad.v.load());
      atten = any_atten.load();
      keep = {6};  // rho
      set_atten(h, atten);
      break;
    }
    case SFD_SEISMIC25: {
      const double* rho = P(21);
      // The y-invariant stiffness averages of the four stress loops, in FP64
      // (seismicfdtd.f95:616-815): plane q holds factor x (C(a) + C(b) + C(c)
      // + C(d)) x dt of Voigt entry `cij` over the four cells of its loop,
      // where that loop updates the cell, else 0.  Factors and stencils as the
      // stress kernel (seis25.cu) reads them.
      struct Avg { int loop, cij; double f; };
      static const Avg avg[33] = {
          {1, 0, 0.25}, {1, 1, 0.25}, {1, 2, 0.25}, {1, 3, 0.125}, {1, 4, 0.125}, {1, 5, 0.125},     // p11..p16
          {1, 6, 0.25}, {1, 7, 0.25}, {1, 8, 0.125}, {1, 9, 0.125}, {1, 10, 0.125},                  // p22..p26
          {1, 11, 0.25}, {1, 12, 0.125}, {1, 13, 0.125}, {1, 14, 0.125},                             // p33..p36
          {2, 5, 0.25}, {2, 10, 0.25}, {2, 14, 0.25}, {2, 17, 0.125}, {2, 19, 0.125}, {2, 20, 0.125}, // q16 q26 q36 q46 q56 q66
          {3, 4, 0.25}, {3, 9, 0.25}, {3, 13, 0.25}, {3, 16, 0.125}, {3, 18, 0.125}, {3, 19, 0.125},  // r15 r25 r35 r45 r55 r56
          {4, 3, 0.25}, {4, 8, 0.25}, {4, 12, 0.25}, {4, 15, 0.125}, {4, 16, 0.125}, {4, 17, 0.125}}; // s14 s24 s34 s44 s45 s46
      FirstBad bad(N2);
      std::atomic<int> any_atten{0};
      parallel_rows(NZ, NX, [&](int k) {
        for (size_t n = (size_t)NX * k; n < (size_t)NX * (k + 1); ++n)
          if (!(rho[n] > 0)) return bad.note(n);
        for (int q = 0; q < 33; ++q) {
          const double* C = P(avg[q].cij);
          for (int i = 0; i < NX; ++i) {
            double v = 0.0;
            switch (avg[q].loop) {
              case 1:  // (i+1,k) (i,k) (i,k-1) (i+1,k-1), k >= 1, i <= NX-2
                if (k >= 1 && i <= NX - 2) v = at(C, i + 1, k) + at(C, i, k) + at(C, i, k - 1) + at(C, i + 1, k - 1);
                break;
              case 2:  // (i,k) (i-1,k) (i,k-1) (i-1,k-1), k >= 1, i >= 1
                if (k >= 1 && i >= 1) v = at(C, i, k) + at(C, i - 1, k) + at(C, i, k - 1) + at(C, i - 1, k - 1);
                break;
              case 3:  // (i,k+1) (i,k) (i-1,k) (i-1,k+1), k <= NZ-2, i >= 1
                if (k <= NZ - 2 && i >= 1) v = at(C, i, k + 1) + at(C, i, k) + at(C, i - 1, k) + at(C, i - 1, k + 1);
                break;
              default:  // (i+1,k) (i,k) (i,k+1) (i+1,k+1), k <= NZ-2, i <= NX-2
                if (k <= NZ - 2 && i <= NX - 2) v = at(C, i + 1, k) + at(C, i, k) + at(C, i, k + 1) + at(C, i + 1, k + 1);
                break;
            }
            out[q][(size_t)i + (size_t)NX * k] = (float)(avg[q].f * v * dt);
          }
        }
        int a = 0;
        for (int i = 0; i < NX; ++i) {
          const size_t n = (size_t)i + (size_t)NX * k;
          const double r = rho[n];
          const int dm = density_method(c.flags);
          if (i >= 1 && k >= 1)  // seismicfdtd.f95:825
            out[33][n] = (float)(dt / rho_avg(dm, 4, r, at(rho, i - 1, k), at(rho, i, k - 1)));
          if (i <= NX - 2 && k >= 1)  // :850
            out[34][n] = (float)(dt / rho_avg(dm, 4, r, at(rho, i + 1, k), at(rho, i, k - 1)));
          if (i <= NX - 2 && k <= NZ - 2)  // :876
            out[35][n] = (float)(dt / rho_avg(dm, 4, r, at(rho, i + 1, k), at(rho, i, k + 1)));
          for (int d = 0; d < 3; ++d) {
            const double g = P(22 + d)[n];
            out[36 + d][n] = (float)(1.0 - g);
            if (g != 0.0) a = 1;
          }
        }
        if (a) any_atten = 1;
      });
      if (bad.v < N2) return fail(SFD_ERR_BAD_ARG, "density must be positive (cell %zu)", bad.v.load());
      atten = any_atten.load();
      keep = {21};  // rho
      set_atten(h, atten);
      break;
    }
  }
  {  // the coefficient planes lie back to back on the device, pitch P
    int r = upload_pitched(h, h->coef(0), coefs.get(), (size_t)nc * NZ);
    if (r) return r;
  }
  std::shared_ptr<double[]> model(new double[keep.size() * N2]);
  for (size_t q = 0; q < keep.size(); ++q) par_copy(model.get() + q * N2, P(keep[q]), N2);
  CK(cudaStreamSynchronize(h->stream));  // host buffers go out of scope
  h->model = std::move(model);
  std::memcpy(h->src_plane, src_plane, sizeof src_plane);
  h->mat_ids = nullptr;
  h->mat_table.reset();
  invalidate_graph(h);                   // kernel arguments (atten) may change
  h->have_model = true;
  return SFD_OK;
}

int32_t sfd_set_cpml2d(sfd_handle* h, const double* fields, int64_t count) {
  g_err.clear();
  if (!h || !fields) return fail(SFD_ERR_BAD_ARG, "NULL argument");
  h->adj_rec_n = 0;  // the recorded states no longer follow from the handle
  const sfd_config& c = h->cfg;
  if (!cpml2d(c)) return fail(SFD_ERR_STATE, "sfd_set_cpml2d needs a handle created with SFD_FLAG_CPML_2D");
  const size_t N2 = (size_t)c.nx * c.nz;
  if (count != (int64_t)(6 * N2))
    return fail(SFD_ERR_BAD_ARG, "2-D CPML fields need 6 planes of %dx%d values, got %lld", c.nx, c.nz, (long long)count);
  if (!all_finite(fields, (size_t)count)) return fail(SFD_ERR_BAD_ARG, "2-D CPML fields contain NaN or Inf");
  std::vector<float> planes(6 * N2);
  for (int o = 0; o < 2; ++o) {
    const double *K = fields + (size_t)(3 * o) * N2, *A = K + N2, *B = A + N2;
    float *ik = planes.data() + (size_t)(3 * o) * N2, *a = ik + N2, *b = a + N2;
    for (size_t n = 0; n < N2; ++n) {
      if (!(K[n] > 0)) return fail(SFD_ERR_BAD_ARG, "2-D CPML kappa must be positive (cell %zu)", n);
      ik[n] = (float)(1.0 / K[n]);
      a[n] = (float)A[n];
      b[n] = (float)B[n];
    }
  }
  int r = upload_pitched(h, h->coef(ncoef(c.kind)), planes.data(), 6 * (size_t)c.nz);
  if (r) return r;
  CK(cudaStreamSynchronize(h->stream));
  h->have_cpml = true;
  return SFD_OK;
}

int32_t sfd_set_cpml(sfd_handle* h, const double* prof, int64_t count) {
  g_err.clear();
  if (!h || !prof) return fail(SFD_ERR_BAD_ARG, "NULL argument");
  h->adj_rec_n = 0;  // the recorded states no longer follow from the handle
  const sfd_config& c = h->cfg;
  if (cpml2d(c)) return fail(SFD_ERR_STATE, "a SFD_FLAG_CPML_2D handle takes its CPML from sfd_set_cpml2d");
  const bool three = is3(c.kind);
  const int lens[3] = {c.nx, three ? c.ny : c.nz, c.nz};
  const double deltas[3] = {c.dx, three ? c.dy : c.dz, c.dz};
  const int nax = three ? 3 : 2;
  int64_t need = 0;
  for (int a = 0; a < nax; ++a) need += 6LL * lens[a];
  if (count != need) return fail(SFD_ERR_BAD_ARG, "CPML profiles need %lld values, got %lld", (long long)need, (long long)count);
  if (!all_finite(prof, (size_t)count)) return fail(SFD_ERR_BAD_ARG, "CPML profiles contain NaN or Inf");
  const double* p = prof;
  std::vector<float> q3(c.nz, 0.0f);
  for (int a = 0; a < nax; ++a) {
    const int n = lens[a];
    const double *K = p, *A = p + n, *B = p + 2 * n, *Kh = p + 3 * n, *Ah = p + 4 * n, *Bh = p + 5 * n;
    p += 6 * n;
    static const char* nm = "xyz";
    const char axn = three ? nm[a] : (a == 0 ? 'x' : 'z');
    if (!check_strip(A, n, c.npml) || !check_strip(Ah, n, c.npml))
      return fail(SFD_ERR_BAD_ARG, "CPML a-coefficients of axis %c are nonzero outside the %d-cell strips", axn, c.npml);
    for (int i = 0; i < n; ++i)
      if (!(K[i] > 0) || !(Kh[i] > 0)) return fail(SFD_ERR_BAD_ARG, "CPML kappa of axis %c must be positive", axn);
    const int st = axis_stride(n);
    std::vector<float> t(6 * (size_t)st, 0.0f);
    const double d = deltas[a];
    for (int i = 0; i < n; ++i) {
      t[i] = (float)(1.0 / (d * K[i]));
      t[st + i] = (float)(A[i] / d);
      t[2 * st + i] = (float)B[i];
      t[3 * st + i] = (float)(1.0 / (d * Kh[i]));
      t[4 * st + i] = (float)(Ah[i] / d);
      t[5 * st + i] = (float)Bh[i];
    }
    CK(cudaMemcpyAsync(h->axis(a), t.data(), sizeof(float) * t.size(), cudaMemcpyHostToDevice, h->stream));
    if (a == 0 && c.kind == SFD_SEISMIC2)  // b_x_half read at the z index, seismicfdtd.f95:255
      for (int k = 0; k < c.nz; ++k) q3[k] = (k < c.nx) ? (float)Bh[k] : 0.0f;
    CK(cudaStreamSynchronize(h->stream));
  }
  CK(cudaMemcpyAsync(h->base + h->L.off_q3, q3.data(), sizeof(float) * q3.size(), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  h->have_cpml = true;
  return SFD_OK;
}

int32_t sfd_set_source(sfd_handle* h, int32_t i, int32_t j, int32_t k, const double* srcfn, int32_t ncomp,
                       int32_t nstep) {
  g_err.clear();
  if (!h || !srcfn) return fail(SFD_ERR_BAD_ARG, "NULL argument");
  h->adj_rec_n = 0;  // the recorded states no longer follow from the handle
  const sfd_config& c = h->cfg;
  if (!h->have_model) return fail(SFD_ERR_STATE, "sfd_set_source needs the model (sfd_set_model) first");
  if (ncomp != nsrc(c.kind)) return fail(SFD_ERR_BAD_ARG, "source needs %d components, got %d", nsrc(c.kind), ncomp);
  if (nstep < 1 || nstep > c.nstep) return fail(SFD_ERR_BAD_ARG, "source length %d outside [1, %d]", nstep, c.nstep);
  const bool three = is3(c.kind);
  if (i < 1 || i > c.nx - 3 || k < 1 || k > c.nz - 3 || (three && (j < 1 || j > c.ny - 3)) || (!three && j != 0))
    return fail(SFD_ERR_BAD_ARG, "source cell (%d,%d,%d) must lie inside the grid, away from its outer two planes", i, j, k);
  if (!all_finite(srcfn, (size_t)ncomp * nstep)) return fail(SFD_ERR_BAD_ARG, "source contains NaN or Inf");
  const size_t n = (size_t)i + (size_t)c.nx * k;
  std::vector<float> amp((size_t)nchan(c.kind) * c.nstep, 0.0f);
  if (c.kind == SFD_ELECTROMAG2C) {  // a dt / eps with complex eps: rows Ex re, Ex im, Ez re, Ez im
    for (int q = 0; q < 2; ++q) {
      const std::complex<double> e(h->src_scale(2 * q)[n], h->src_scale(2 * q + 1)[n]);
      for (int t = 0; t < nstep; ++t) {
        const std::complex<double> v = srcfn[(size_t)q * nstep + t] * c.dt / e;
        amp[(size_t)(2 * q) * c.nstep + t] = (float)v.real();
        amp[(size_t)(2 * q + 1) * c.nstep + t] = (float)v.imag();
      }
    }
  } else {
    for (int q = 0; q < ncomp; ++q) {
      double s = 0.0;
      int r = source_divisor(h, q, n, &s);
      if (r) return r;
      for (int t = 0; t < nstep; ++t) amp[(size_t)q * c.nstep + t] = (float)(srcfn[(size_t)q * nstep + t] * c.dt / s);
    }
  }
  if (h->have_ssrc && !same_source_cell(h, i, j, k))
    return fail(SFD_ERR_BAD_ARG, "the force source must lie at the stress source's cell (%d,%d,%d)", h->s2.io.si,
                h->s2.io.sj, h->s2.io.sk);
  CK(cudaMemcpyAsync(h->base + h->L.off_src, amp.data(), sizeof(float) * amp.size(), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  set_io_source(h, i, j, k);
  h->have_force_src = true;
  invalidate_graph(h);
  return SFD_OK;
}

int32_t sfd_set_stress_source(sfd_handle* h, int32_t i, int32_t j, int32_t k, const double* srcfn, int32_t ncomp,
                              int32_t nstep) {
  g_err.clear();
  if (!h) return fail(SFD_ERR_BAD_ARG, "NULL handle");
  h->adj_rec_n = 0;  // the recorded states no longer follow from the handle
  const sfd_config& c = h->cfg;
  const int ns = nstress(c.kind);
  if (!ns) return fail(SFD_ERR_BAD_ARG, "stress sources apply to the seismic kinds only");
  if (ncomp == 0) {  // remove the stress source
    h->have_ssrc = false;
    set_io_ssrc(h);
    invalidate_graph(h);
    return SFD_OK;
  }
  if (!srcfn) return fail(SFD_ERR_BAD_ARG, "NULL source");
  if (ncomp != ns) return fail(SFD_ERR_BAD_ARG, "stress source needs %d components, got %d", ns, ncomp);
  if (nstep < 1 || nstep > c.nstep) return fail(SFD_ERR_BAD_ARG, "source length %d outside [1, %d]", nstep, c.nstep);
  const bool three = is3(c.kind);
  if (i < 1 || i > c.nx - 3 || k < 1 || k > c.nz - 3 || (three && (j < 1 || j > c.ny - 3)) || (!three && j != 0))
    return fail(SFD_ERR_BAD_ARG, "source cell (%d,%d,%d) must lie inside the grid, away from its outer two planes", i, j, k);
  if (h->have_force_src && !same_source_cell(h, i, j, k))
    return fail(SFD_ERR_BAD_ARG, "the stress source must lie at the force source's cell (%d,%d,%d)", h->s2.io.si,
                h->s2.io.sj, h->s2.io.sk);
  if (!all_finite(srcfn, (size_t)ncomp * nstep)) return fail(SFD_ERR_BAD_ARG, "source contains NaN or Inf");
  std::vector<float> amp((size_t)ns * c.nstep, 0.0f);
  for (int q = 0; q < ns; ++q)
    for (int t = 0; t < nstep; ++t) amp[(size_t)q * c.nstep + t] = (float)(srcfn[(size_t)q * nstep + t] * c.dt);
  CK(cudaMemcpyAsync(h->base + h->L.off_src + sizeof(float) * (size_t)nchan(c.kind) * c.nstep, amp.data(),
                     sizeof(float) * amp.size(), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  h->have_ssrc = true;
  set_io_ssrc(h);
  set_io_source(h, i, j, k);
  invalidate_graph(h);
  return SFD_OK;
}

int32_t sfd_set_source_wavelet(sfd_handle* h, int32_t stress, int32_t i, int32_t j, int32_t k, int32_t stype,
                               double f0, double amp, const double* comp, int32_t ncomp) {
  g_err.clear();
  if (!h || !comp) return fail(SFD_ERR_BAD_ARG, "NULL argument");
  h->adj_rec_n = 0;  // the recorded states no longer follow from the handle
  const sfd_config& c = h->cfg;
  if (c.kind == SFD_ELECTROMAG2C) return fail(SFD_ERR_BAD_ARG, "electromag2c sources come through sfd_set_source");
  if (stype < SFD_WAVELET_GAUS0 || stype > SFD_WAVELET_GAUS2) return fail(SFD_ERR_BAD_ARG, "unknown wavelet type %d", stype);
  if (!(f0 > 0.0) || !std::isfinite(f0) || !std::isfinite(amp))
    return fail(SFD_ERR_BAD_ARG, "the wavelet needs a positive finite f0 and a finite amplitude");
  const int want = stress ? nstress(c.kind) : nsrc(c.kind);
  if (stress && !want) return fail(SFD_ERR_BAD_ARG, "stress sources apply to the seismic kinds only");
  if (ncomp != want) return fail(SFD_ERR_BAD_ARG, "the source needs %d components, got %d", want, ncomp);
  if (!all_finite(comp, (size_t)ncomp)) return fail(SFD_ERR_BAD_ARG, "component factors contain NaN or Inf");
  if (!stress && !h->have_model) return fail(SFD_ERR_STATE, "sfd_set_source_wavelet needs the model (sfd_set_model) first");
  const bool three = is3(c.kind);
  if (i < 1 || i > c.nx - 3 || k < 1 || k > c.nz - 3 || (three && (j < 1 || j > c.ny - 3)) || (!three && j != 0))
    return fail(SFD_ERR_BAD_ARG, "source cell (%d,%d,%d) must lie inside the grid, away from its outer two planes", i, j, k);
  if (stress ? (h->have_force_src && !same_source_cell(h, i, j, k)) : (h->have_ssrc && !same_source_cell(h, i, j, k)))
    return fail(SFD_ERR_BAD_ARG, "the force and stress sources must share one cell");
  WaveletComp wc;
  wc.n = ncomp;
  const size_t n = (size_t)i + (size_t)c.nx * k;
  for (int q = 0; q < ncomp; ++q) {
    wc.comp[q] = comp[q];
    wc.div[q] = 1.0;
    if (!stress) {
      int r = source_divisor(h, q, n, &wc.div[q]);
      if (r) return r;
    }
  }
  const size_t rows = stress ? (size_t)ncomp : (size_t)nchan(c.kind);
  float* out = (float*)(h->base + h->L.off_src) + (stress ? (size_t)nchan(c.kind) * c.nstep : 0);
  CK(cudaMemsetAsync(out, 0, sizeof(float) * rows * c.nstep, h->stream));
  CK(wavelet_launch(stype, f0, c.dt, c.nstep, amp, wc, out, (size_t)c.nstep, h->stream));
  if (stress) {
    h->have_ssrc = true;
    set_io_ssrc(h);
  } else {
    h->have_force_src = true;
  }
  set_io_source(h, i, j, k);
  invalidate_graph(h);
  return SFD_OK;
}

int32_t sfd_set_cpml_params(sfd_handle* h, const sfd_cpml_params* p) {
  g_err.clear();
  if (!h || !p) return fail(SFD_ERR_BAD_ARG, "NULL argument");
  h->adj_rec_n = 0;  // the recorded states no longer follow from the handle
  const sfd_config& c = h->cfg;
  if (cpml2d(c)) return fail(SFD_ERR_STATE, "a SFD_FLAG_CPML_2D handle takes its CPML from sfd_set_cpml2d");
  if (p->mode != 0 && p->mode != 1) return fail(SFD_ERR_BAD_ARG, "CPML mode must be 0 (driver) or 1 (legacy)");
  const bool three = is3(c.kind);
  const double vals[7] = {p->sig_max[0], three ? p->sig_max[1] : 0.0, p->sig_max[2], p->alpha_max, p->kappa_max,
                          p->NP, p->NPA};
  for (double v : vals)
    if (!std::isfinite(v) || v < 0.0) return fail(SFD_ERR_BAD_ARG, "CPML parameters must be finite and >= 0");
  if (c.npml < 1) return fail(SFD_ERR_BAD_ARG, "CPML profiles need npml >= 1");
  const int lens[3] = {c.nx, three ? c.ny : c.nz, c.nz};
  const double deltas[3] = {c.dx, three ? c.dy : c.dz, c.dz};
  const double sig[3] = {p->sig_max[0], three ? p->sig_max[1] : p->sig_max[2], p->sig_max[2]};
  const int nax = three ? 3 : 2;
  const bool seismic = c.kind == SFD_SEISMIC2 || c.kind == SFD_SEISMIC25;
  for (int a = 0; a < nax; ++a) {
    CpmlAxisArgs ax;
    ax.n = lens[a]; ax.npml = c.npml; ax.delta = deltas[a]; ax.dt = c.dt; ax.sig_max = sig[a];
    ax.alpha_max = p->alpha_max; ax.kappa_max = p->kappa_max; ax.NP = p->NP; ax.NPA = p->NPA;
    ax.seismic = seismic; ax.legacy = p->mode;
    const int st = axis_stride(lens[a]);
    CK(cudaMemsetAsync(h->axis(a), 0, sizeof(float) * 6 * (size_t)st, h->stream));
    CK(cpml_axis_launch(ax, h->axis(a), st, h->stream));
  }
  float* q3 = (float*)(h->base + h->L.off_q3);
  CK(cudaMemsetAsync(q3, 0, sizeof(float) * c.nz, h->stream));
  if (c.kind == SFD_SEISMIC2)  // b_x_half read at the z index, seismicfdtd.f95:255
    CK(cpml_q3_launch(h->axis(0) + 5 * (size_t)axis_stride(c.nx), c.nx, c.nz, q3, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  h->have_cpml = true;
  return SFD_OK;
}

int32_t sfd_set_receivers(sfd_handle* h, const int32_t* ijk, int32_t nrec) {
  g_err.clear();
  if (!h) return fail(SFD_ERR_BAD_ARG, "NULL handle");
  const sfd_config& c = h->cfg;
  if (nrec != c.nrec) return fail(SFD_ERR_BAD_ARG, "configured for %d receivers, got %d", c.nrec, nrec);
  if (nrec == 0) return SFD_OK;
  if (!ijk) return fail(SFD_ERR_BAD_ARG, "NULL receiver array");
  for (int r = 0; r < nrec; ++r) {
    const int i = ijk[3 * r], j = ijk[3 * r + 1], k = ijk[3 * r + 2];
    if (i < 0 || i >= c.nx || j < 0 || j >= c.ny || k < 0 || k >= c.nz)
      return fail(SFD_ERR_BAD_ARG, "receiver %d at (%d,%d,%d) is outside the grid", r, i, j, k);
  }
  CK(cudaMemcpyAsync(h->base + h->L.off_rec, ijk, sizeof(int) * 3 * (size_t)nrec, cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return SFD_OK;
}

int32_t sfd_reset(sfd_handle* h) {
  g_err.clear();
  if (!h) return fail(SFD_ERR_BAD_ARG, "NULL handle");
  h->adj_rec_n = 0;  // the recorded states no longer follow from the handle
  const Layout& L = h->L;
  CK(cudaMemsetAsync(h->base + L.off_fields, 0, L.off_coef - L.off_fields, h->stream));
  CK(cudaMemsetAsync(h->base + L.off_traces, 0, L.off_slots - L.off_traces, h->stream));
  h->step = 0;
  h->cur = 0;
  return SFD_OK;
}

int32_t sfd_set_field(sfd_handle* h, int32_t field, const float* host, int64_t count) {
  g_err.clear();
  if (!h || !host) return fail(SFD_ERR_BAD_ARG, "NULL argument");
  h->adj_rec_n = 0;  // the recorded states no longer follow from the handle
  const sfd_config& c = h->cfg;
  if (field < 0 || field >= nfields(c.kind)) return fail(SFD_ERR_BAD_ARG, "field %d out of range", field);
  if (count != (int64_t)c.nx * c.ny * c.nz) return fail(SFD_ERR_BAD_ARG, "field needs %d*%d*%d values", c.nx, c.ny, c.nz);
  CK(cudaMemcpy2DAsync(h->f(field), sizeof(float) * h->L.P, host, sizeof(float) * c.nx, sizeof(float) * c.nx,
                       (size_t)c.ny * c.nz, cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return SFD_OK;
}

int32_t sfd_get_field(sfd_handle* h, int32_t field, float* host, int64_t count) {
  g_err.clear();
  if (!h || !host) return fail(SFD_ERR_BAD_ARG, "NULL argument");
  const sfd_config& c = h->cfg;
  if (field < 0 || field >= nfields(c.kind)) return fail(SFD_ERR_BAD_ARG, "field %d out of range", field);
  if (count != (int64_t)c.nx * c.ny * c.nz) return fail(SFD_ERR_BAD_ARG, "field needs %d*%d*%d values", c.nx, c.ny, c.nz);
  CK(cudaMemcpy2DAsync(host, sizeof(float) * c.nx, h->f(field), sizeof(float) * h->L.P, sizeof(float) * c.nx,
                       (size_t)c.ny * c.nz, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return SFD_OK;
}

int32_t sfd_get_field_async(sfd_handle* h, int32_t field, float* host, int64_t count) {
  g_err.clear();
  if (!h || !host) return fail(SFD_ERR_BAD_ARG, "NULL argument");
  const sfd_config& c = h->cfg;
  if (field < 0 || field >= nfields(c.kind)) return fail(SFD_ERR_BAD_ARG, "field %d out of range", field);
  if (count != (int64_t)c.nx * c.ny * c.nz) return fail(SFD_ERR_BAD_ARG, "field needs %d*%d*%d values", c.nx, c.ny, c.nz);
  CK(cudaMemcpy2DAsync(host, sizeof(float) * c.nx, h->f(field), sizeof(float) * h->L.P, sizeof(float) * c.nx,
                       (size_t)c.ny * c.nz, cudaMemcpyDeviceToHost, h->stream));
  return SFD_OK;
}

int32_t sfd_encode_field_i16(sfd_handle* h, int32_t field, void* dev_out, void* dev_minmax) {
  g_err.clear();
  if (!h || !dev_out || !dev_minmax) return fail(SFD_ERR_BAD_ARG, "NULL argument");
  const sfd_config& c = h->cfg;
  if (field < 0 || field >= nfields(c.kind)) return fail(SFD_ERR_BAD_ARG, "field %d out of range", field);
  if (((uintptr_t)dev_out & 1) || ((uintptr_t)dev_minmax & 3))
    return fail(SFD_ERR_BAD_ARG, "misaligned output: int16 codes need 2-byte, min/max 4-byte alignment");
  encode_field_i16(h->f(field), c.nx, h->L.P, (long)c.ny * c.nz, (short*)dev_out, (float*)dev_minmax, h->stream);
  CK(cudaGetLastError());
  return SFD_OK;
}

int32_t sfd_get_memory(sfd_handle* h, int32_t index, float* host, int64_t count) {
  g_err.clear();
  if (!h || !host) return fail(SFD_ERR_BAD_ARG, "NULL argument");
  const sfd_config& c = h->cfg;
  const char* ax = mem_axes(c.kind);
  if (index < 0 || index >= (int)strlen(ax)) return fail(SFD_ERR_BAD_ARG, "memory variable %d out of range", index);
  const int NX = c.nx, NY = c.ny, NZ = c.nz, W = c.npml, P = h->L.P;
  if (count != (int64_t)NX * NY * NZ) return fail(SFD_ERR_BAD_ARG, "memory variable needs %d*%d*%d values", NX, NY, NZ);
  if (cpml2d(c)) {  // stored on the full grid, rows of pitch P
    CK(cudaMemcpy2DAsync(host, sizeof(float) * NX, h->m(index), sizeof(float) * P, sizeof(float) * NX, NZ,
                         cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return SFD_OK;
  }
  std::vector<float> s(h->L.mem_sz[index]);
  CK(cudaMemcpyAsync(s.data(), h->m(index), sizeof(float) * s.size(), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  auto sidx = [](int i, int n, int W_) { return i < W_ ? i : i - (n - 2 * W_); };
  auto ins = [](int i, int n, int W_) { return i < W_ || i >= n - W_; };
  for (int k = 0; k < NZ; ++k)
    for (int j = 0; j < NY; ++j)
      for (int i = 0; i < NX; ++i) {
        float v = 0.0f;
        if (ax[index] == 'x') {
          if (ins(i, NX, W)) v = s[((size_t)k * NY + j) * 2 * W + sidx(i, NX, W)];
        } else if (ax[index] == 'y') {
          if (ins(j, NY, W)) v = s[((size_t)k * 2 * W + sidx(j, NY, W)) * P + i];
        } else {
          if (ins(k, NZ, W)) v = s[((size_t)sidx(k, NZ, W) * NY + j) * P + i];
        }
        host[(size_t)i + (size_t)NX * ((size_t)j + (size_t)NY * k)] = v;
      }
  return SFD_OK;
}

int32_t sfd_run(sfd_handle* h, int64_t nsteps) {
  g_err.clear();
  if (!h) return fail(SFD_ERR_BAD_ARG, "NULL handle");
  h->adj_rec_n = 0;  // the recorded states no longer follow from the handle
  if (!h->have_model || !h->have_cpml) return fail(SFD_ERR_STATE, "sfd_run needs sfd_set_model and sfd_set_cpml first");
  if (nsteps < 0) return fail(SFD_ERR_BAD_ARG, "nsteps must be >= 0");
  if (h->step + nsteps > h->cfg.nstep)
    return fail(SFD_ERR_BAD_ARG, "run to step %lld exceeds the %d source samples", (long long)(h->step + nsteps), h->cfg.nstep);
  if (nsteps == 0) return SFD_OK;
  const Layout& L = h->L;
  Ctl* ctl = (Ctl*)(h->base + L.off_ctl);
  float* slots = (float*)(h->base + L.off_slots);
  k_begin<<<std::min(1024, (L.nslots + 255) / 256 + 1), 256, 0, h->stream>>>(ctl, slots, L.nslots, (int)h->step);
  if (resident_usable(h)) {  // the whole run in one launch, state on chip
    // tags from an earlier run must not match: clear every edge word
    CK(cudaMemsetAsync(h->base + L.off_res, 0, res_scratch_bytes(L.P, L.NZ, res_edge_fields(h->cfg.kind)), h->stream));
    if (h->cfg.kind == SFD_SEISMIC2) CK(seis2_resident_launch(seis2_resident_args(h, nsteps), h->stream));
    else CK(em2_resident_launch(resident_args(h, nsteps), h->stream));
    k_reduce_slots<<<1, 1024, 0, h->stream>>>(ctl, slots, L.nslots);
    CK(cudaGetLastError());
    h->step += nsteps;
    return SFD_OK;
  }
  const int64_t chunks = h->cap_stream ? nsteps / kGraphSteps : 0;
  const int rem = (int)(nsteps - chunks * kGraphSteps);
  if (chunks > 0) {
    int r = ensure_graph(h, h->single ? h->cur : 0);
    if (r) return r;
    for (int64_t q = 0; q < chunks; ++q) CK(cudaGraphLaunch(h->graph[h->single ? h->cur : 0], h->stream));
  }
  for (int s = 0; s < rem; ++s) {
    if (h->single) {
      launch_step(h, h->cur, s, h->stream);
      h->cur ^= 1;
    } else {
      launch_half(h, 0, s, h->stream);
      launch_half(h, 1, s, h->stream);
    }
  }
  launch_finalize(h, (int)(h->step + nsteps - 1), h->stream);
  k_reduce_slots<<<1, 1024, 0, h->stream>>>(ctl, slots, L.nslots);
  CK(cudaGetLastError());
  h->step += nsteps;
  return SFD_OK;
}

int32_t sfd_on_chip(sfd_handle* h, int32_t* tiles_x, int32_t* tiles_z) {  // tiles, tile rows
  g_err.clear();
  if (!h) return fail(SFD_ERR_BAD_ARG, "NULL handle");
  const bool on = resident_usable(h);
  const bool s2 = h->cfg.kind == SFD_SEISMIC2;
  if (tiles_x) *tiles_x = on ? (s2 ? h->s2_plan.ntx * h->s2_plan.ntz : h->res_plan.ntiles) : 0;
  if (tiles_z) *tiles_z = on ? (s2 ? h->s2_plan.ntz : h->res_plan.ntz) : 0;
  return on ? 1 : 0;
}

int32_t sfd_status(sfd_handle* h, int64_t* step, double* maxnorm) {
  g_err.clear();
  if (!h) return fail(SFD_ERR_BAD_ARG, "NULL handle");
  Ctl ctl;
  CK(cudaMemcpyAsync(&ctl, h->base + h->L.off_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (step) *step = h->step;
  if (maxnorm) *maxnorm = (double)ctl.maxnorm;
  if (ctl.err)
    return fail(SFD_ERR_TIMEOUT,
                (h->cfg.kind == SFD_SEISMIC25 || h->cfg.kind == SFD_ELECTROMAG25)
                    ? "2.5-D step: a staged tile did not arrive within %.3g s"
                                             : "on-chip run: a neighbouring tile did not answer within %.3g s",
                (double)h->wait_ns * 1e-9);
  if (!(ctl.maxnorm <= 1.0e25f))
    return fail(SFD_ERR_UNSTABLE, "field norm %g exceeded 1e25 (code became unstable and blew up)", (double)ctl.maxnorm);
  return SFD_OK;
}

int32_t sfd_set_wait_limit(sfd_handle* h, int64_t ns) {
  g_err.clear();
  if (!h) return fail(SFD_ERR_BAD_ARG, "NULL handle");
  if (ns < 0) return fail(SFD_ERR_BAD_ARG, "wait limit must be >= 0 ns (0 = the default 2 s)");
  h->wait_ns = ns == 0 ? kDefaultWaitNs : (unsigned long long)ns;
  h->s25.wait_ns = h->wait_ns;
  h->em25.wait_ns = h->wait_ns;
  invalidate_graph(h);
  return SFD_OK;
}

int32_t sfd_test_stall_waits(sfd_handle* h, int32_t on) {
  g_err.clear();
  if (!h) return fail(SFD_ERR_BAD_ARG, "NULL handle");
  h->stall_waits = on != 0;
  h->s25.stall_tx = h->stall_waits ? 16u : 0u;
  h->em25.stall_tx = h->stall_waits ? 16u : 0u;
  invalidate_graph(h);
  return SFD_OK;
}

int32_t sfd_get_traces(sfd_handle* h, float* host, int64_t count) {
  g_err.clear();
  if (!h || !host) return fail(SFD_ERR_BAD_ARG, "NULL argument");
  const sfd_config& c = h->cfg;
  const int64_t n = (int64_t)c.nstep * nchan(c.kind) * c.nrec;
  if (count != n) return fail(SFD_ERR_BAD_ARG, "traces hold %lld values, got %lld", (long long)n, (long long)count);
  if (n == 0) return SFD_OK;
  CK(cudaMemcpyAsync(host, h->base + h->L.off_traces, sizeof(float) * n, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return SFD_OK;
}

int32_t sfd_launch_half(sfd_handle* h, int32_t which, int32_t count) {
  g_err.clear();
  if (!h) return fail(SFD_ERR_BAD_ARG, "NULL handle");
  if (which != 0 && which != 1) return fail(SFD_ERR_BAD_ARG, "which must be 0 or 1");
  if (count < 0) return fail(SFD_ERR_BAD_ARG, "count must be >= 0");
  if (!h->have_model || !h->have_cpml) return fail(SFD_ERR_STATE, "sfd_launch_half needs sfd_set_model and sfd_set_cpml");
  const Layout& L = h->L;
  k_begin<<<std::min(1024, (L.nslots + 255) / 256 + 1), 256, 0, h->stream>>>((Ctl*)(h->base + L.off_ctl),
                                                                            (float*)(h->base + L.off_slots), L.nslots, 0);
  for (int q = 0; q < count; ++q) {
    if (h->single) {
      launch_step(h, h->cur, 0, h->stream);  // the single-pass kernel is the whole step
      h->cur ^= 1;
    } else {
      launch_half(h, which, 0, h->stream);
    }
  }
  CK(cudaGetLastError());
  return SFD_OK;
}

const float* sfd_traces_device(const sfd_handle* h) {
  return h ? (const float*)(h->base + h->L.off_traces) : nullptr;
}

int32_t sfd_field_device(const sfd_handle* h, int32_t field, float** ptr, int64_t* pitch) {
  g_err.clear();
  if (!h || !ptr) return fail(SFD_ERR_BAD_ARG, "NULL argument");
  if (field < 0 || field >= nfields(h->cfg.kind)) return fail(SFD_ERR_BAD_ARG, "field %d out of range", field);
  *ptr = h->f(field);
  if (pitch) *pitch = h->L.P;
  return SFD_OK;
}

int32_t sfd_destroy(sfd_handle* h) {
  g_err.clear();
  if (!h) return SFD_OK;
  cudaStreamSynchronize(h->stream);
  invalidate_graph(h);
  if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
  delete h;
  return SFD_OK;
}

}  // extern "C"

extern "C" {

int32_t sfd_share_model(sfd_handle* dst, const sfd_handle* src) {
  g_err.clear();
  if (!dst || !src || dst == src) return fail(SFD_ERR_BAD_ARG, "need two different handles");
  const sfd_config &a = dst->cfg, &b = src->cfg;
  if (a.kind != b.kind || a.nx != b.nx || a.ny != b.ny || a.nz != b.nz || a.dt != b.dt || a.flags != b.flags)
    return fail(SFD_ERR_BAD_ARG, "handles differ in kind, grid, dt or flags");
  if (!src->have_model) return fail(SFD_ERR_STATE, "the source handle has no model");
  switch (a.kind) {
    case SFD_ELECTROMAG2: {
      const Em2Args& e = src->em2;
      dst->em2.CAx = e.CAx; dst->em2.CBx = e.CBx; dst->em2.CAz = e.CAz; dst->em2.CBz = e.CBz;
      for (int p = 0; p < 2; ++p) {
        dst->em2s[p].CAx = e.CAx; dst->em2s[p].CBx = e.CBx; dst->em2s[p].CAz = e.CAz; dst->em2s[p].CBz = e.CBz;
      }
      break;
    }
    case SFD_SEISMIC2: {
      const Seis2Args& e = src->s2;
      Seis2Args& d = dst->s2;
      d.A11 = e.A11; d.A13 = e.A13; d.A15 = e.A15; d.A33 = e.A33; d.A35 = e.A35; d.B15 = e.B15; d.B35 = e.B35;
      d.B55 = e.B55; d.dtrx = e.dtrx; d.dtrz = e.dtrz; d.gxp = e.gxp; d.gzp = e.gzp;
      for (int p = 0; p < 2; ++p) {
        Seis2Step& t = dst->s2s[p];
        t.A11 = e.A11; t.A13 = e.A13; t.A15 = e.A15; t.A33 = e.A33; t.A35 = e.A35; t.B15 = e.B15; t.B35 = e.B35;
        t.B55 = e.B55; t.dtrx = e.dtrx; t.dtrz = e.dtrz; t.gxp = e.gxp; t.gzp = e.gzp;
      }
      set_atten(dst, src->s2.atten);
      break;
    }
    default:
      return fail(SFD_ERR_BAD_ARG, "model sharing is implemented for electromag2 and seismic2");
  }
  std::memcpy(dst->src_plane, src->src_plane, sizeof src->src_plane);
  dst->model = src->model;
  dst->mat_ids = src->mat_ids;
  dst->mat_table = src->mat_table;
  dst->have_model = true;
  invalidate_graph(dst);
  return SFD_OK;
}

}  // extern "C"
