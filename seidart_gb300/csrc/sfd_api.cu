// C ABI of the seidart_gb300 FDTD backend: handle management, FP64 host-side
// coefficient folding, state layout in the caller's device buffer, and the
// time loop (CUDA graphs of 32 steps, two fused kernels per step).
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

#include "../../include/seidart_gb300.h"
#include "host_pool.h"
#include "adjoint.h"
#include "adjoint_s2.h"
#include "batch.h"
#include "resident.h"
#include "sfd_solvers.h"

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

namespace {

constexpr double kPI = 3.141592653589793238462643;
constexpr double kMu0 = 4.0 * kPI * 1.0e-7;
constexpr double kEps0 = 8.85418782e-12;
constexpr int kGraphSteps = 32;
constexpr unsigned long long kDefaultWaitNs = 2000000000ull;  // bounded device waits: 2 s
// Added to the awaited edge tags by the timeout test aid: tags are step
// numbers + 1 or 2, so no tile ever writes a biased one.
constexpr unsigned kStallTagBias = 0x40000000u;

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

}  // namespace

namespace sfd {
// Replace the calling thread's error message (used by the static-scratch entry point).
void set_error(const char* msg) { g_err = msg ? msg : ""; }
}  // namespace sfd

namespace {

#define CK(call)                                   \
  do {                                             \
    cudaError_t e_ = (call);                       \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

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

struct Layout {
  int P, NX, NY, NZ, W, ysplit, nslots;
  size_t fsz;                // floats per field
  size_t off_ctl, off_fields, off_mem[18], mem_sz[18], off_fieldsB, off_memB[18], off_coef, coef_plane, off_axis[3],
      off_q3, off_src, off_rec, off_traces, off_slots, off_res, total;
};

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

}  // namespace

struct sfd_handle_s {
  sfd_config cfg;
  Layout L;
  char* base;
  cudaStream_t stream;       // caller's stream
  cudaStream_t cap_stream;   // private stream used only to capture graphs
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // indexed by the parity the graph starts from
  // a seismic2 adjoint segment's work (s2_adjoint_segment) and what it was captured for
  cudaGraphExec_t adj_graph = nullptr;
  int64_t adj_graph_n = 0;
  int adj_graph_cur = 0, adj_graph_seg = 0;
  const char* adj_graph_work = nullptr;
  const float* adj_graph_resid = nullptr;
  bool have_model = false, have_cpml = false;
  bool have_ssrc = false;       // a stress source was set (seismic kinds)
  bool have_force_src = false;  // a force (or E) source was set
  bool single = false;  // single-pass 2-D steps (ping-pong state)
  int cur = 0;          // copy holding the current state (single-pass only)
  int zb = 2;           // rows per thread of the single-pass tiles
  Em2Step em2s[2];      // [p]: reads copy p, writes copy 1-p
  Seis2Step s2s[2];
  Launch launch1;       // single-pass geometry
  int res_state = 0;    // on-chip runs: 0 not yet checked, 1 usable, -1 not usable
  ResPlan res_plan;     // electromag2
  Seis2ResPlan s2_plan;  // seismic2
  int64_t step = 0;
  unsigned long long wait_ns = kDefaultWaitNs;  // longest wait of an on-chip run for a neighbouring tile
  bool stall_waits = false;                     // timeout test aid: waits expect tags no tile writes
  // The FP64 model planes read after sfd_set_model (the source scaling; for
  // electromag2 also the adjoint's chain rule), copied from its input:
  // electromag2 all six planes; electromag2c eps11 eps33 (re, im);
  // electromag25 eps11 eps22 eps33; seismic rho.  Shared, not copied, by
  // sfd_share_model.
  std::shared_ptr<double[]> model;
  int src_plane[4] = {0, 0, 0, 0};  // planes of `model` the source amplitude is divided by (complex: re, im pairs)
  const double* src_scale(int q) const { return model.get() + (size_t)src_plane[q] * cfg.nx * cfg.nz; }
  // sfd_set_model_ids: the caller's device id map and the material table
  // (rows of the kind's model planes); `model` is then expanded from them
  // only when the adjoint needs it
  const int32_t* mat_ids = nullptr;
  std::shared_ptr<std::vector<double>> mat_table;
  // adjoint workspace (electromag2)
  char* adj = nullptr;
  int adj_seg = 0;
  int adj_cur = 0;
  int64_t adj_rec_s0 = 0;  // sfd_adjoint_record: the recorded run's first step and length (0: none)
  int64_t adj_rec_n = 0;
  const float* adj_resid = nullptr;
  int adj_res_state = 0;  // on-chip adjoint sweeps: 0 not yet checked, 1 usable, -1 not usable
  Em2Args em2;
  Em2cArgs em2c;
  Seis2Args s2;
  Seis25Args s25;
  Em25Args em25;
  Launch launch;
  // field q / memory variable q of copy `copy` (copy 1 exists for single-pass kinds)
  float* fc(int q, int copy) const {
    return (float*)(base + (copy ? L.off_fieldsB : L.off_fields)) + (size_t)q * L.fsz;
  }
  float* mc(int q, int copy) const {
    return (float*)(base + ((copy && L.off_memB[q]) ? L.off_memB[q] : L.off_mem[q]));
  }
  float* f(int q) const { return fc(q, single ? cur : 0); }
  float* m(int q) const { return mc(q, single ? cur : 0); }
  float* coef(int q) const { return (float*)(base + L.off_coef) + (size_t)q * L.coef_plane; }
  float* axis(int a) const { return (float*)(base + L.off_axis[a]); }
  IoArgs io() const {
    IoArgs io;
    io.ctl = (Ctl*)(base + L.off_ctl);
    io.slots = (float*)(base + L.off_slots);
    io.src = (const float*)(base + L.off_src);
    io.nstep = cfg.nstep;
    io.ssrc = have_ssrc ? (const float*)(base + L.off_src) + (size_t)nchan(cfg.kind) * cfg.nstep : nullptr;
    io.si = io.sj = io.sk = -1;
    io.rec = (const int*)(base + L.off_rec);
    io.nrec = cfg.nrec;
    io.traces = (float*)(base + L.off_traces);
    return io;
  }
};

namespace {

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
  struct PlanKey {
    int nx, nz, npml, ctas, dev;
    size_t smem;
  };
  static std::mutex plan_mu;
  static std::vector<std::pair<PlanKey, std::pair<bool, ResPlan>>> plans;
  const PlanKey key{h->cfg.nx, h->cfg.nz, h->cfg.npml, std::min(nsm, h->L.nslots), dev, (size_t)optin - static_smem};
  ResPlan plan;
  bool fits = false, cached = false;
  {
    std::lock_guard<std::mutex> lock(plan_mu);
    for (const auto& e : plans)
      if (e.first.nx == key.nx && e.first.nz == key.nz && e.first.npml == key.npml && e.first.ctas == key.ctas &&
          e.first.dev == key.dev && e.first.smem == key.smem) {
        fits = e.second.first;
        plan = e.second.second;
        cached = true;
        break;
      }
  }
  if (!cached) {
    fits = em2_resident_plan(key.nx, key.nz, key.npml, key.ctas, key.smem, &plan);
    std::lock_guard<std::mutex> lock(plan_mu);
    plans.push_back({key, {fits, plan}});
  }
  if (!fits) return false;
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

}  // namespace

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

// ---------------------------------------------------------------------------
// Batched runs: one persistent cooperative launch for many 2-D models.

struct sfd_batch_s {
  std::vector<sfd_handle*> h;
  char* scratch = nullptr;
  cudaStream_t stream = nullptr;
  int zb = 2, bps = 4, nsm = 0;
  unsigned long long limit_ns = kDefaultWaitNs;  // barrier wait limit
  int stall = 0;  // timeout test aid: the barrier waits for one block more than the launch has
  std::vector<BatchModel> models;
  std::vector<int> steps;
  GridBarrier* bar() const { return (GridBarrier*)scratch; }
  std::vector<BatchGroup> groups;
  int* dsteps() const { return (int*)(scratch + 256); }
  BatchModel* dmodels() const { return (BatchModel*)(scratch + 256 + align256(sizeof(int) * h.size())); }
  BatchGroup* dgroups() const {
    return (BatchGroup*)(scratch + 256 + align256(sizeof(int) * h.size()) + align256(sizeof(BatchModel) * h.size()));
  }
};

namespace {
size_t batch_bytes(int n) {
  return 256 + align256(sizeof(int) * n) + align256(sizeof(BatchModel) * (size_t)n) +
         align256(sizeof(BatchGroup) * (size_t)n);
}

// Models that read the same coefficient planes and have the same geometry.
bool same_group(const sfd_handle* a, const sfd_handle* b) {
  if (a->cfg.kind != b->cfg.kind || a->cfg.nx != b->cfg.nx || a->cfg.nz != b->cfg.nz) return false;
  if (a->cfg.kind == SFD_ELECTROMAG2) return a->em2s[0].CAx == b->em2s[0].CAx;
  return a->s2s[0].A11 == b->s2s[0].A11;
}
}  // namespace

extern "C" {

int32_t sfd_batch_scratch_bytes(int32_t nmodels, size_t* bytes) {
  g_err.clear();
  if (nmodels < 1 || !bytes) return fail(SFD_ERR_BAD_ARG, "need nmodels >= 1 and a bytes pointer");
  *bytes = batch_bytes(nmodels);
  return SFD_OK;
}

int32_t sfd_batch_create(sfd_handle* const* handles, int32_t n, void* dev_scratch, size_t bytes, sfd_batch** out) {
  g_err.clear();
  if (!handles || n < 1 || !out) return fail(SFD_ERR_BAD_ARG, "need handles, n >= 1 and out");
  *out = nullptr;
  if (!dev_scratch || ((uintptr_t)dev_scratch & 255)) return fail(SFD_ERR_BAD_ARG, "scratch must be 256-byte aligned device memory");
  if (bytes < batch_bytes(n)) return fail(SFD_ERR_BAD_ARG, "batch scratch has %zu bytes, needs %zu", bytes, batch_bytes(n));
  for (int m = 0; m < n; ++m) {
    sfd_handle* h = handles[m];
    if (!h) return fail(SFD_ERR_BAD_ARG, "handle %d is NULL", m);
    if (!h->single) return fail(SFD_ERR_BAD_ARG, "handle %d: batches take single-pass 2-D handles (seismic2/electromag2, no SFD_FLAG_TWO_PASS)", m);
    if (!h->have_model || !h->have_cpml) return fail(SFD_ERR_STATE, "handle %d has no model or CPML yet", m);
    if (h->stream != handles[0]->stream) return fail(SFD_ERR_BAD_ARG, "all handles of a batch must share one stream");
    for (int q = 0; q < m; ++q)
      if (handles[q] == h) return fail(SFD_ERR_BAD_ARG, "handle %d appears twice", m);
  }
  int dev = 0;
  CK(cudaGetDevice(&dev));
  sfd_batch* b = new sfd_batch_s();
  b->h.assign(handles, handles + n);
  b->scratch = (char*)dev_scratch;
  b->stream = handles[0]->stream;
  cudaError_t e = cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) { delete b; return cuda_fail(e, "cudaDeviceGetAttribute"); }
  *out = b;
  return SFD_OK;
}

int32_t sfd_batch_set_tiling(sfd_batch* b, int32_t zb, int32_t blocks_per_sm) {
  g_err.clear();
  if (!b) return fail(SFD_ERR_BAD_ARG, "NULL batch");
  if (zb != 1 && zb != 2 && zb != 4) return fail(SFD_ERR_BAD_ARG, "zb must be 1, 2 or 4");
  int maxb = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, batch_kernel_ptr(zb), 256, 0));
  if (blocks_per_sm < 1 || blocks_per_sm > maxb)
    return fail(SFD_ERR_BAD_ARG, "blocks_per_sm must be in [1, %d] for zb=%d", maxb, zb);
  b->zb = zb;
  b->bps = blocks_per_sm;
  return SFD_OK;
}

int32_t sfd_batch_run(sfd_batch* b, int64_t nsteps) {
  g_err.clear();
  if (!b) return fail(SFD_ERR_BAD_ARG, "NULL batch");
  if (nsteps < 0) return fail(SFD_ERR_BAD_ARG, "nsteps must be >= 0");
  if (nsteps == 0) return SFD_OK;
  const int n = (int)b->h.size();
  for (int m = 0; m < n; ++m)
    if (b->h[m]->step + nsteps > b->h[m]->cfg.nstep)
      return fail(SFD_ERR_BAD_ARG, "model %d: run to step %lld exceeds its %d source samples", m,
                  (long long)(b->h[m]->step + nsteps), b->h[m]->cfg.nstep);
  int maxb = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, batch_kernel_ptr(b->zb), 256, 0));
  const int bps = std::min(b->bps, maxb);
  if (bps < 1) return fail(SFD_ERR_CUDA, "batch kernel does not fit on an SM");
  b->models.assign(n, BatchModel());
  b->steps.assign(n, 0);
  for (int m = 0; m < n; ++m) {
    sfd_handle* h = b->h[m];
    BatchModel& md = b->models[m];
    md.kind = h->cfg.kind == SFD_ELECTROMAG2 ? SFD_BATCH_EM2 : SFD_BATCH_SEIS2;
    md.gx = md.kind == SFD_BATCH_EM2 ? (h->cfg.nx + 127) / 128 : (h->cfg.nx + 31) / 32;  // em2 tiles are 128 wide
    const int gy = (h->cfg.nz + 8 * b->zb - 1) / (8 * b->zb);
    md.ntiles = md.gx * gy;
    md.nslots = md.ntiles;
    md.cur = h->cur;
    md.em2[0] = h->em2s[0];
    md.em2[1] = h->em2s[1];
    md.s2[0] = h->s2s[0];
    md.s2[1] = h->s2s[1];
    b->steps[m] = (int)h->step;
  }
  b->groups.clear();
  int tile0 = 0;
  for (int m = 0; m < n;) {
    int e = m + 1;
    while (e < n && same_group(b->h[m], b->h[e])) ++e;
    BatchGroup g;
    g.first = m;
    g.n = e - m;
    g.tile0 = tile0;
    g.ntiles = g.n * b->models[m].ntiles;
    tile0 += g.ntiles;
    b->groups.push_back(g);
    m = e;
  }
  const int total = tile0;
  const int grid = std::max(1, std::min(total, bps * b->nsm));
  CK(cudaMemcpyAsync(b->dsteps(), b->steps.data(), sizeof(int) * n, cudaMemcpyHostToDevice, b->stream));
  CK(cudaMemcpyAsync(b->dmodels(), b->models.data(), sizeof(BatchModel) * n, cudaMemcpyHostToDevice, b->stream));
  CK(cudaMemcpyAsync(b->dgroups(), b->groups.data(), sizeof(BatchGroup) * b->groups.size(), cudaMemcpyHostToDevice,
                     b->stream));
  batch_begin(b->dmodels(), n, b->dsteps(), b->bar(), b->stream);
  CK(batch_launch(b->zb, grid, b->dmodels(), b->dgroups(), (int)b->groups.size(), total, (int)nsteps, b->bar(),
                  b->limit_ns, b->stall, b->stream));
  batch_end(b->dmodels(), n, (int)nsteps, b->stream);
  CK(cudaGetLastError());
  for (sfd_handle* h : b->h) {
    h->step += nsteps;
    h->cur ^= (int)(nsteps & 1);
  }
  return SFD_OK;
}

int32_t sfd_batch_set_wait_limit(sfd_batch* b, int64_t ns) {
  g_err.clear();
  if (!b) return fail(SFD_ERR_BAD_ARG, "NULL batch");
  if (ns < 0) return fail(SFD_ERR_BAD_ARG, "wait limit must be >= 0 ns (0 = the default 2 s)");
  b->limit_ns = ns == 0 ? kDefaultWaitNs : (unsigned long long)ns;
  return SFD_OK;
}

int32_t sfd_batch_test_stall_waits(sfd_batch* b, int32_t on) {
  g_err.clear();
  if (!b) return fail(SFD_ERR_BAD_ARG, "NULL batch");
  b->stall = on ? 1 : 0;
  return SFD_OK;
}

int32_t sfd_batch_status(sfd_batch* b, int32_t* failed_model) {
  g_err.clear();
  if (!b) return fail(SFD_ERR_BAD_ARG, "NULL batch");
  if (failed_model) *failed_model = -1;
  GridBarrier bar;
  CK(cudaMemcpyAsync(&bar, b->bar(), sizeof bar, cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  if (bar.err) return fail(SFD_ERR_TIMEOUT, "grid barrier of the batched kernel timed out");
  for (size_t m = 0; m < b->h.size(); ++m) {
    int r = sfd_status(b->h[m], nullptr, nullptr);
    if (r != SFD_OK) {
      if (failed_model) *failed_model = (int32_t)m;
      return r;
    }
  }
  return SFD_OK;
}

int32_t sfd_batch_destroy(sfd_batch* b) {
  g_err.clear();
  if (!b) return SFD_OK;
  cudaStreamSynchronize(b->stream);
  delete b;
  return SFD_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Checkpoints and the electromag2 adjoint.

namespace {

size_t ckpt_bytes(const sfd_handle* h) {
  size_t n = (size_t)nfields(h->cfg.kind) * h->L.fsz;
  const int nm = (int)strlen(mem_axes(h->cfg.kind));
  for (int m = 0; m < nm; ++m) n += h->L.mem_sz[m];
  return n * sizeof(float);
}

// Adjoint workspace layout: two adjoint states, TH/MEx/MEz, four gradient
// planes, the source accumulator, then seg+1 forward state slots.
struct AdjLayout {
  size_t field, zstrip, xstrip, state, lam[2], th, mex, mez, g[4], acc, slots, total;
};

AdjLayout adj_layout(const sfd_handle* h, int seg) {
  AdjLayout A;
  const Layout& L = h->L;
  A.field = align256(sizeof(float) * L.fsz);
  A.zstrip = align256(sizeof(float) * L.mem_sz[0]);  // dEx_dz: z-strip
  A.xstrip = align256(sizeof(float) * L.mem_sz[1]);  // dEz_dx: x-strip
  A.state = 3 * A.field + 2 * A.zstrip + 2 * A.xstrip;
  size_t o = 0;
  A.lam[0] = o; o += A.state;
  A.lam[1] = o; o += A.state;
  A.th = o; o += A.field;
  A.mex = o; o += A.field;
  A.mez = o; o += A.field;
  for (int q = 0; q < 4; ++q) { A.g[q] = o; o += A.field; }
  A.acc = o; o += 256;
  A.slots = o; o += A.state * (size_t)(seg + 1);
  A.total = o;
  return A;
}

AdjState adj_state_at(const AdjLayout& A, char* base) {
  AdjState S;
  S.Ex = (float*)base;
  S.Ez = (float*)(base + A.field);
  S.Hy = (float*)(base + 2 * A.field);
  S.A = (float*)(base + 3 * A.field);
  S.C = (float*)(base + 3 * A.field + A.zstrip);
  S.B = (float*)(base + 3 * A.field + 2 * A.zstrip);
  S.D = (float*)(base + 3 * A.field + 2 * A.zstrip + A.xstrip);
  return S;
}

// Whether the adjoint sweeps of this handle run on chip: its forward runs
// do, and the sweep's larger per-tile shared memory fits too.
bool adjoint_on_chip(sfd_handle* h) {
  if (h->adj_res_state) return h->adj_res_state > 0;
  h->adj_res_state = -1;
  if (!resident_usable(h)) return false;
  int per_sm = 0;
  if (em2_adj_resident_prepare(h->res_plan, h->cfg.nx, h->cfg.nz, h->L.W, &per_sm) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    return false;
  }
  h->adj_res_state = 1;
  return true;
}

int adj_check(const sfd_handle* h) {
  if (!h) return fail(SFD_ERR_BAD_ARG, "NULL handle");
  if (h->cfg.kind == SFD_SEISMIC2) {
    if (h->cfg.flags & (SFD_FLAG_LEGACY_QUIRKS | SFD_FLAG_CPML_2D))
      return fail(SFD_ERR_BAD_ARG,
                  "the seismic2 adjoint follows the corrected physics with 1-D CPML profiles "
                  "(no SFD_FLAG_LEGACY_QUIRKS, no SFD_FLAG_CPML_2D)");
    return SFD_OK;
  }
  if (h->cfg.kind != SFD_ELECTROMAG2 || !h->single)
    return fail(SFD_ERR_BAD_ARG, "the adjoint is implemented for single-pass electromag2 handles and seismic2 handles");
  return SFD_OK;
}

// seismic2 adjoint workspace: two adjoint states, twelve scratch planes,
// twelve gradient planes, the source accumulator, then seg+1 forward state
// slots.  A state holds vx vz sxx szz sxz (full grid) and the twelve memory
// variables (their strips), each array 256-byte aligned.
struct S2AdjLayout {
  size_t field, mem[12], state, lam[2], tmp, g, acc, slots, total;
};

S2AdjLayout s2_adj_layout(const sfd_handle* h, int seg) {
  S2AdjLayout A;
  const Layout& L = h->L;
  A.field = align256(sizeof(float) * L.fsz);
  size_t o = 5 * A.field;
  for (int m = 0; m < 12; ++m) { A.mem[m] = o; o += align256(sizeof(float) * L.mem_sz[m]); }
  A.state = o;
  o = 0;
  A.lam[0] = o; o += A.state;
  A.lam[1] = o; o += A.state;
  A.tmp = o; o += 12 * A.field;
  A.g = o; o += 12 * A.field;
  A.acc = o; o += 256;
  A.slots = o; o += A.state * (size_t)(seg + 1);
  A.total = o;
  return A;
}

S2State s2_state_at(const S2AdjLayout& A, char* base) {
  S2State S;
  float** f[5] = {&S.vx, &S.vz, &S.sxx, &S.szz, &S.sxz};
  for (int q = 0; q < 5; ++q) *f[q] = (float*)(base + q * A.field);
  for (int m = 0; m < 12; ++m) S.m[m] = (float*)(base + A.mem[m]);
  return S;
}

// The handle's current state -> a state slot.
int s2_save_state(sfd_handle* h, const S2AdjLayout& A, char* dst) {
  const size_t fb = sizeof(float) * h->L.fsz;
  for (int q = 0; q < 5; ++q) CK(cudaMemcpyAsync(dst + q * A.field, h->f(q), fb, cudaMemcpyDeviceToDevice, h->stream));
  for (int m = 0; m < 12; ++m)
    CK(cudaMemcpyAsync(dst + A.mem[m], h->m(m), sizeof(float) * h->L.mem_sz[m], cudaMemcpyDeviceToDevice, h->stream));
  return SFD_OK;
}

size_t adj_total(const sfd_handle* h, int seg) {
  return h->cfg.kind == SFD_SEISMIC2 ? s2_adj_layout(h, seg).total : adj_layout(h, seg).total;
}
size_t adj_slots(const sfd_handle* h, int seg) {
  return h->cfg.kind == SFD_SEISMIC2 ? s2_adj_layout(h, seg).slots : adj_layout(h, seg).slots;
}

// One seismic2 segment: the forward states recomputed by the handle's own
// steps into the slots, then the adjoint steps over them, last step first.
// The work of one seismic2 segment after its slot 0 is filled and the
// control block's base set to the segment's first step: the forward
// recompute, slot s -> slot s + 1 (no receivers), then the adjoint steps,
// last first, starting from adjoint state `cur`.  Every address it names is
// the handle's or its adjoint workspace's and every step index is relative
// to the control block's base, so a capture of it replays for any segment of
// the same length.
cudaError_t s2_segment_work(sfd_handle* h, const S2AdjLayout& A, int64_t nsteps, int cur, cudaStream_t stream) {
  const Layout& L = h->L;
  char* slots = h->adj + A.slots;
  cudaError_t e = cudaSuccess;
  if (h->single) {  // the single-pass step kernel between slots; its in-place memory variables copied ahead
    Seis2Step st = h->s2s[0];
    st.io.nrec = 0;
    for (int64_t s = 0; s < nsteps && e == cudaSuccess; ++s) {
      const S2State a0 = s2_state_at(A, slots + A.state * (size_t)s);
      const S2State a1 = s2_state_at(A, slots + A.state * (size_t)(s + 1));
      st.vx0 = a0.vx; st.vz0 = a0.vz; st.sxx0 = a0.sxx; st.szz0 = a0.szz; st.sxz0 = a0.sxz;
      st.vx1 = a1.vx; st.vz1 = a1.vz; st.sxx1 = a1.sxx; st.szz1 = a1.szz; st.sxz1 = a1.sxz;
      st.m_vxx0 = a0.m[0]; st.m_vzz0 = a0.m[1]; st.m_vxz0 = a0.m[2]; st.m_vzx0 = a0.m[3];
      st.m_vxx1 = a1.m[0]; st.m_vzz1 = a1.m[1]; st.m_vxz1 = a1.m[2]; st.m_vzx1 = a1.m[3];
      st.m2_vxx0 = a0.m[8]; st.m2_vzz0 = a0.m[9]; st.m2_vxz0 = a0.m[10]; st.m2_vzx0 = a0.m[11];
      st.m2_vxx1 = a1.m[8]; st.m2_vzz1 = a1.m[9]; st.m2_vxz1 = a1.m[10]; st.m2_vzx1 = a1.m[11];
      e = cudaMemcpyAsync(a1.m[4], a0.m[4], A.mem[8] - A.mem[4], cudaMemcpyDeviceToDevice, stream);
      st.m_sxx_x = a1.m[4]; st.m_szz_z = a1.m[5]; st.m_sxz_x = a1.m[6]; st.m_sxz_z = a1.m[7];
      seis2_step(st, h->launch1, h->zb, (int)s, stream);
    }
  } else {  // the two half-step kernels in place on a copy of the previous slot
    Seis2Args ar = h->s2;
    ar.io.nrec = 0;
    for (int64_t s = 0; s < nsteps && e == cudaSuccess; ++s) {
      char* dst = slots + A.state * (size_t)(s + 1);
      e = cudaMemcpyAsync(dst, slots + A.state * (size_t)s, A.state, cudaMemcpyDeviceToDevice, stream);
      const S2State a1 = s2_state_at(A, dst);
      ar.vx = a1.vx; ar.vz = a1.vz; ar.sxx = a1.sxx; ar.szz = a1.szz; ar.sxz = a1.sxz;
      ar.m_vxx = a1.m[0]; ar.m_vzz = a1.m[1]; ar.m_vxz = a1.m[2]; ar.m_vzx = a1.m[3];
      ar.m_sxx_x = a1.m[4]; ar.m_szz_z = a1.m[5]; ar.m_sxz_x = a1.m[6]; ar.m_sxz_z = a1.m[7];
      ar.m2_vxx = a1.m[8]; ar.m2_vzz = a1.m[9]; ar.m2_vxz = a1.m[10]; ar.m2_vzx = a1.m[11];
      seis2_half1(ar, h->launch, (int)s, stream);
      seis2_half2(ar, h->launch, (int)s, stream);
    }
  }
  if (e != cudaSuccess) return e;
  const Seis2Args& c = h->s2;
  S2Adj a;
  a.NX = h->cfg.nx; a.NZ = h->cfg.nz; a.P = L.P; a.W = L.W;
  const float** co[12] = {&a.A11, &a.A13, &a.A15, &a.A33, &a.A35, &a.B15, &a.B35, &a.B55, &a.dtrx, &a.dtrz, &a.gxp, &a.gzp};
  const float* src_co[12] = {c.A11, c.A13, c.A15, c.A33, c.A35, c.B15, c.B35, c.B55, c.dtrx, c.dtrz, c.gxp, c.gzp};
  for (int q = 0; q < 12; ++q) *co[q] = src_co[q];
  a.X = c.X; a.Z = c.Z;
  for (int q = 0; q < 12; ++q) a.tmp[q] = (float*)(h->adj + A.tmp + q * A.field);
  float** g[12] = {&a.gA11, &a.gA13, &a.gA15, &a.gA33, &a.gA35, &a.gB15, &a.gB35, &a.gB55, &a.gdtrx, &a.gdtrz, &a.ggxp, &a.ggzp};
  for (int q = 0; q < 12; ++q) *g[q] = (float*)(h->adj + A.g + q * A.field);
  a.srcacc = (float*)(h->adj + A.acc);
  a.srcfn = (const float*)(h->base + L.off_src);
  a.nstep = h->cfg.nstep; a.si = h->have_force_src ? c.io.si : -1; a.sk = c.io.sk;
  a.rec = (const int*)(h->base + L.off_rec); a.nrec = h->cfg.nrec; a.resid = h->adj_resid;
  a.ctl = (const Ctl*)(h->base + L.off_ctl);
  for (int64_t s = nsteps - 1; s >= 0; --s) {
    const S2State S = s2_state_at(A, slots + A.state * (size_t)s);
    const S2State S1 = s2_state_at(A, slots + A.state * (size_t)(s + 1));
    const S2State Ln = s2_state_at(A, h->adj + A.lam[cur]);
    const S2State Lc = s2_state_at(A, h->adj + A.lam[1 - cur]);
    s2_adj_step(a, S, S1, Ln, Lc, (int)s, stream);
    cur ^= 1;
  }
  return cudaGetLastError();
}

// One seismic2 segment: slot 0 <- the handle's state, the step base, then
// the segment's work, replayed from a CUDA graph captured on the handle's
// private stream when it has one (one capture per segment length and
// starting adjoint state; the graph is dropped with the handle's others).
int s2_adjoint_segment(sfd_handle* h, int64_t nsteps) {
  const int64_t s0 = h->step;
  const S2AdjLayout A = s2_adj_layout(h, h->adj_seg);
  const Layout& L = h->L;
  int r = s2_save_state(h, A, h->adj + A.slots);
  if (r) return r;
  k_begin<<<std::min(1024, (L.nslots + 255) / 256 + 1), 256, 0, h->stream>>>((Ctl*)(h->base + L.off_ctl),
                                                                            (float*)(h->base + L.off_slots), L.nslots, (int)s0);
  if (!h->cap_stream) {
    CK(s2_segment_work(h, A, nsteps, h->adj_cur, h->stream));
  } else {
    const bool reuse = h->adj_graph && h->adj_graph_n == nsteps && h->adj_graph_cur == h->adj_cur &&
                       h->adj_graph_work == h->adj && h->adj_graph_resid == h->adj_resid &&
                       h->adj_graph_seg == h->adj_seg;
    if (!reuse) {
      if (h->adj_graph) { cudaGraphExecDestroy(h->adj_graph); h->adj_graph = nullptr; }
      cudaGraph_t g = nullptr;
      CK(cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal));
      const cudaError_t ew = s2_segment_work(h, A, nsteps, h->adj_cur, h->cap_stream);
      const cudaError_t ec = cudaStreamEndCapture(h->cap_stream, &g);
      if (ew != cudaSuccess) { if (g) cudaGraphDestroy(g); return cuda_fail(ew, "seismic2 adjoint segment"); }
      if (ec != cudaSuccess) return cuda_fail(ec, "cudaStreamEndCapture");
      const cudaError_t ei = cudaGraphInstantiate(&h->adj_graph, g, 0);
      cudaGraphDestroy(g);
      if (ei != cudaSuccess) { h->adj_graph = nullptr; return cuda_fail(ei, "cudaGraphInstantiate"); }
      h->adj_graph_n = nsteps; h->adj_graph_cur = h->adj_cur; h->adj_graph_work = h->adj;
      h->adj_graph_resid = h->adj_resid; h->adj_graph_seg = h->adj_seg;
    }
    CK(cudaGraphLaunch(h->adj_graph, h->stream));
  }
  h->adj_cur ^= (int)(nsteps & 1);
  return SFD_OK;
}

// dJ/d(c11 c13 c15 c33 c35 c55 rho gamma_x gamma_z) from the gradient planes
// of the update coefficients, in FP64 (the coefficients of sfd_set_model:
// stiffness averages (c(i+1,k) + 2 c(i,k) + c(i,k-1)) dt / 4 on loop-1
// points and (c(i,k+1) + 2 c(i,k) + c(i-1,k)) dt / 4 on loop-2 points,
// dt over the density average of the velocity loops, 1 - gamma, and the
// source amplitude f dt / rho).
int s2_adjoint_gradient(sfd_handle* h, double* out, int64_t count) {
  const int NX = h->cfg.nx, NZ = h->cfg.nz, P = h->L.P;
  const size_t N2 = (size_t)NX * NZ;
  if (!out || count != (int64_t)(9 * N2)) return fail(SFD_ERR_BAD_ARG, "gradient needs 9 planes of %dx%d", NX, NZ);
  const S2AdjLayout A = s2_adj_layout(h, h->adj_seg);
  std::vector<float> g((size_t)12 * P * NZ);
  for (int q = 0; q < 12; ++q)
    CK(cudaMemcpyAsync(g.data() + (size_t)q * P * NZ, h->adj + A.g + q * A.field, sizeof(float) * P * NZ,
                       cudaMemcpyDeviceToHost, h->stream));
  float acc = 0.f;
  CK(cudaMemcpyAsync(&acc, h->adj + A.acc, sizeof acc, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  int r = ensure_model_planes(h);
  if (r) return r;
  const double* rho = h->src_scale(0);
  const double dt = h->cfg.dt, w = dt / 4;
  const int dm = density_method(h->cfg.flags);
  std::fill(out, out + 9 * N2, 0.0);
  auto G = [&](int q, int i, int k) -> double {
    if (i < 0 || i >= NX || k < 0 || k >= NZ) return 0.0;
    return g[(size_t)q * P * NZ + (size_t)k * P + i];
  };
  auto fromA = [&](int q, int i, int k) { return w * (2 * G(q, i, k) + G(q, i - 1, k) + G(q, i, k + 1)); };
  auto fromB = [&](int q, int i, int k) { return w * (2 * G(q, i, k) + G(q, i, k - 1) + G(q, i + 1, k)); };
  // rho_avg(method, 2, r, a, b) and its partial derivatives
  auto parts = [&](double r0, double a0, double b0, double* d) {
    const double m = rho_avg(dm, 2, r0, a0, b0);
    switch (dm) {
      case 1: d[0] = 1; d[1] = 0; d[2] = 0; break;
      case 2: d[0] = m / (2 * r0); d[1] = m / (4 * a0); d[2] = m / (4 * b0); break;
      case 3: d[0] = m * m / (2 * r0 * r0); d[1] = m * m / (4 * a0 * a0); d[2] = m * m / (4 * b0 * b0); break;
      default: d[0] = 0.5; d[1] = 0.25; d[2] = 0.25;
    }
    return m;
  };
  double* grho = out + 6 * N2;
  for (int k = 0; k < NZ; ++k)
    for (int i = 0; i < NX; ++i) {
      const size_t n = (size_t)i + (size_t)NX * k;
      out[n] = fromA(0, i, k);
      out[N2 + n] = fromA(1, i, k);
      out[2 * N2 + n] = fromA(2, i, k) + fromB(5, i, k);
      out[3 * N2 + n] = fromA(3, i, k);
      out[4 * N2 + n] = fromA(4, i, k) + fromB(6, i, k);
      out[5 * N2 + n] = fromB(7, i, k);
      out[7 * N2 + n] = -G(10, i, k);
      out[8 * N2 + n] = -G(11, i, k);
      double d[3];
      const double gx = G(8, i, k), gz = G(9, i, k);
      if (gx != 0.0) {
        if (i >= 1 && k >= 1) {  // dtrx = dt / rho_avg(rho(i,k), rho(i-1,k), rho(i,k-1))
          const double m = parts(rho[n], rho[n - 1], rho[n - NX], d), u = gx * (-dt / (m * m));
          grho[n] += u * d[0];
          grho[n - 1] += u * d[1];
          grho[n - NX] += u * d[2];
        } else {
          grho[n] += gx * (-dt / (rho[n] * rho[n]));
        }
      }
      if (gz != 0.0 && i <= NX - 2 && k <= NZ - 2) {  // dtrz = dt / rho_avg(rho(i,k), rho(i+1,k), rho(i,k+1))
        const double m = parts(rho[n], rho[n + 1], rho[n + NX], d), u = gz * (-dt / (m * m));
        grho[n] += u * d[0];
        grho[n + 1] += u * d[1];
        grho[n + NX] += u * d[2];
      }
    }
  const int si = h->s2.io.si, sk = h->s2.io.sk;
  if (h->have_force_src && si >= 0) {  // vx, vz += f dt / rho at the source cell
    const size_t n = (size_t)si + (size_t)NX * sk;
    grho[n] += -(double)acc / rho[n];
  }
  return SFD_OK;
}

}  // namespace

extern "C" {

int32_t sfd_checkpoint_bytes(const sfd_handle* h, size_t* bytes) {
  g_err.clear();
  if (!h || !bytes) return fail(SFD_ERR_BAD_ARG, "NULL argument");
  *bytes = ckpt_bytes(h);
  return SFD_OK;
}

int32_t sfd_checkpoint_save(sfd_handle* h, void* dev_dst) {
  g_err.clear();
  if (!h || !dev_dst) return fail(SFD_ERR_BAD_ARG, "NULL argument");
  char* d = (char*)dev_dst;
  const size_t fb = sizeof(float) * h->L.fsz;
  for (int q = 0; q < nfields(h->cfg.kind); ++q, d += fb)
    CK(cudaMemcpyAsync(d, h->f(q), fb, cudaMemcpyDeviceToDevice, h->stream));
  const int nm = (int)strlen(mem_axes(h->cfg.kind));
  for (int m = 0; m < nm; ++m) {
    const size_t mb = sizeof(float) * h->L.mem_sz[m];
    CK(cudaMemcpyAsync(d, h->m(m), mb, cudaMemcpyDeviceToDevice, h->stream));
    d += mb;
  }
  return SFD_OK;
}

int32_t sfd_checkpoint_load(sfd_handle* h, const void* dev_src, int64_t step) {
  g_err.clear();
  if (!h || !dev_src) return fail(SFD_ERR_BAD_ARG, "NULL argument");
  h->adj_rec_n = 0;  // the recorded states no longer follow from the handle
  if (step < 0 || step > h->cfg.nstep) return fail(SFD_ERR_BAD_ARG, "step %lld out of range", (long long)step);
  const char* d = (const char*)dev_src;
  const size_t fb = sizeof(float) * h->L.fsz;
  for (int q = 0; q < nfields(h->cfg.kind); ++q, d += fb)
    CK(cudaMemcpyAsync(h->f(q), d, fb, cudaMemcpyDeviceToDevice, h->stream));
  const int nm = (int)strlen(mem_axes(h->cfg.kind));
  for (int m = 0; m < nm; ++m) {
    const size_t mb = sizeof(float) * h->L.mem_sz[m];
    CK(cudaMemcpyAsync(h->m(m), d, mb, cudaMemcpyDeviceToDevice, h->stream));
    d += mb;
  }
  h->step = step;
  return SFD_OK;
}

int32_t sfd_run_checkpointed(sfd_handle* h, int64_t nsteps, void* dev_ckpt, size_t stride, int32_t every) {
  g_err.clear();
  if (!h || !dev_ckpt) return fail(SFD_ERR_BAD_ARG, "NULL argument");
  if (!h->have_model || !h->have_cpml) return fail(SFD_ERR_STATE, "sfd_run needs sfd_set_model and sfd_set_cpml first");
  if (nsteps < 0 || every < 1) return fail(SFD_ERR_BAD_ARG, "need nsteps >= 0 and every >= 1");
  if (h->step + nsteps > h->cfg.nstep)
    return fail(SFD_ERR_BAD_ARG, "run to step %lld exceeds the %d source samples", (long long)(h->step + nsteps), h->cfg.nstep);
  const size_t nb = ckpt_bytes(h);
  if (stride < nb) return fail(SFD_ERR_BAD_ARG, "checkpoint stride %zu is below the %zu bytes of a checkpoint", stride, nb);
  if (((uintptr_t)dev_ckpt | stride) & 3) return fail(SFD_ERR_BAD_ARG, "checkpoints must be 4-byte aligned");
  char* base = (char*)dev_ckpt;
  int r = sfd_checkpoint_save(h, base);
  if (r) return r;
  if (nsteps == 0) return SFD_OK;
  if (h->cfg.kind == SFD_ELECTROMAG2 && resident_usable(h)) {
    // one launch for the whole run, the checkpoints written from chip
    const Layout& L = h->L;
    Ctl* ctl = (Ctl*)(h->base + L.off_ctl);
    float* slots = (float*)(h->base + L.off_slots);
    k_begin<<<std::min(1024, (L.nslots + 255) / 256 + 1), 256, 0, h->stream>>>(ctl, slots, L.nslots, (int)h->step);
    CK(cudaMemsetAsync(h->base + L.off_res, 0, res_scratch_bytes(L.P, L.NZ, res_edge_fields(h->cfg.kind)), h->stream));
    Em2Resident ra = resident_args(h, nsteps);
    ra.ckpt.base = base;
    ra.ckpt.stride = stride;
    const size_t F = sizeof(float) * L.fsz;
    size_t o = 3 * F;
    for (int q = 0; q < 3; ++q) ra.ckpt.off[q] = q * F;
    for (int m = 0; m < 4; ++m) {  // dEx_dz dEz_dx dHy_dz dHy_dx: A B C D
      ra.ckpt.off[3 + m] = o;
      o += sizeof(float) * L.mem_sz[m];
    }
    ra.ckpt_every = every;
    CK(em2_resident_launch(ra, h->stream));
    k_reduce_slots<<<1, 1024, 0, h->stream>>>(ctl, slots, L.nslots);
    CK(cudaGetLastError());
    h->step += nsteps;
    return SFD_OK;
  }
  for (int64_t done = 0; done < nsteps;) {
    const int64_t m = std::min<int64_t>(every, nsteps - done);
    r = sfd_run(h, m);
    if (r) return r;
    done += m;
    if (done < nsteps) {
      r = sfd_checkpoint_save(h, base + (size_t)(done / every) * stride);
      if (r) return r;
    }
  }
  return SFD_OK;
}

int32_t sfd_adjoint_bytes(const sfd_handle* h, int32_t seg_steps, size_t* bytes) {
  g_err.clear();
  int r = adj_check(h);
  if (r) return r;
  if (seg_steps < 1 || !bytes) return fail(SFD_ERR_BAD_ARG, "need seg_steps >= 1 and bytes");
  *bytes = adj_total(h, seg_steps);
  return SFD_OK;
}

int32_t sfd_adjoint_begin(sfd_handle* h, void* dev_work, size_t bytes, int32_t seg_steps, const float* dev_resid) {
  g_err.clear();
  int r = adj_check(h);
  if (r) return r;
  if (!dev_work || ((uintptr_t)dev_work & 255)) return fail(SFD_ERR_BAD_ARG, "workspace must be 256-byte aligned device memory");
  if (seg_steps < 1) return fail(SFD_ERR_BAD_ARG, "seg_steps must be >= 1");
  const size_t total = adj_total(h, seg_steps);
  if (bytes < total) return fail(SFD_ERR_BAD_ARG, "adjoint workspace has %zu bytes, needs %zu", bytes, total);
  if (h->cfg.nrec > 0 && !dev_resid) return fail(SFD_ERR_BAD_ARG, "residual traces are NULL");
  h->adj = (char*)dev_work;
  h->adj_seg = seg_steps;
  h->adj_cur = 0;
  h->adj_resid = dev_resid;
  h->adj_rec_n = 0;
  CK(cudaMemsetAsync(h->adj, 0, adj_slots(h, seg_steps), h->stream));  // adjoint states, gradients, accumulators
  CK(cudaMemsetAsync(&((Ctl*)(h->base + h->L.off_ctl))->err, 0, sizeof(int), h->stream));
  return SFD_OK;
}

// Adjoint slot 0 <- the handle's forward state.
static int em2_save_slot0(sfd_handle* h, const AdjLayout& A) {
  const Layout& L = h->L;
  const AdjState S0 = adj_state_at(A, h->adj + A.slots);
  const size_t fb = sizeof(float) * L.fsz;
  CK(cudaMemcpyAsync(S0.Ex, h->f(0), fb, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(S0.Ez, h->f(1), fb, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(S0.Hy, h->f(2), fb, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(S0.A, h->m(0), sizeof(float) * L.mem_sz[0], cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(S0.B, h->m(1), sizeof(float) * L.mem_sz[1], cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(S0.C, h->m(2), sizeof(float) * L.mem_sz[2], cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(S0.D, h->m(3), sizeof(float) * L.mem_sz[3], cudaMemcpyDeviceToDevice, h->stream));
  return SFD_OK;
}

// Offsets of Ex Ez Hy A B C D inside one adjoint slot.
static void em2_slot_offsets(const AdjLayout& A, size_t off[7]) {
  const size_t F = A.field, ZS = A.zstrip, XS = A.xstrip;
  const size_t o[7] = {0, F, 2 * F, 3 * F, 3 * F + 2 * ZS, 3 * F + ZS, 3 * F + 2 * ZS + XS};
  for (int q = 0; q < 7; ++q) off[q] = o[q];
}

// The on-chip forward run from slot 0 (the state before step s0) that dumps
// the state after step s0 + s into slot s + 1 and leaves the handle's state
// as it was.
static Em2Resident em2_dump_args(sfd_handle* h, const AdjLayout& A, int64_t s0, int64_t nsteps) {
  const AdjState S0 = adj_state_at(A, h->adj + A.slots);
  Em2Resident fr = resident_args(h, nsteps);
  fr.Ex = S0.Ex; fr.Ez = S0.Ez; fr.Hy = S0.Hy;
  fr.mExz = S0.A; fr.mEzx = S0.B; fr.mHyz = S0.C; fr.mHyx = S0.D;
  fr.t0 = (int)s0;
  fr.dump.base = h->adj + A.slots;
  fr.dump.stride = A.state;
  em2_slot_offsets(A, fr.dump.off);
  return fr;
}

// The on-chip adjoint sweep of steps s0 + nsteps - 1 down to s0 over the
// states in slots 0 .. nsteps, in place on the current adjoint state.
static int em2_adjoint_sweep_on_chip(sfd_handle* h, const AdjLayout& A, int64_t s0, int64_t nsteps) {
  const Layout& L = h->L;
  const AdjState Lc = adj_state_at(A, h->adj + A.lam[h->adj_cur]);
  const Em2Args& e = h->em2;
  const Em2Resident fr = resident_args(h, nsteps);
  Em2AdjResident ar;
  ar.NX = h->cfg.nx; ar.NZ = h->cfg.nz; ar.P = L.P; ar.W = L.W;
  ar.Lx = Lc.Ex; ar.Lz = Lc.Ez; ar.Lh = Lc.Hy; ar.LA = Lc.A; ar.LB = Lc.B; ar.LC = Lc.C; ar.LD = Lc.D;
  ar.CAx = e.CAx; ar.CBx = e.CBx; ar.CAz = e.CAz; ar.CBz = e.CBz;
  ar.X = e.X; ar.Z = e.Z; ar.dbH = e.dbH;
  ar.gCAx = (float*)(h->adj + A.g[0]); ar.gCBx = (float*)(h->adj + A.g[1]);
  ar.gCAz = (float*)(h->adj + A.g[2]); ar.gCBz = (float*)(h->adj + A.g[3]);
  ar.srcacc = (float*)(h->adj + A.acc);
  ar.srcfn = (const float*)(h->base + L.off_src);
  ar.nstep = h->cfg.nstep; ar.si = e.io.si; ar.sk = e.io.sk;
  ar.rec = (const int*)(h->base + L.off_rec); ar.nrec = h->cfg.nrec; ar.resid = h->adj_resid;
  ar.slots = h->adj + A.slots;
  ar.stride = A.state;
  em2_slot_offsets(A, ar.off);
  ar.s0 = (int)s0;
  ar.nsteps = (int)nsteps;
  ar.ctl = (Ctl*)(h->base + L.off_ctl);
  ar.plan = h->res_plan;
  ar.r = fr.r;
  ar.limit_ns = fr.limit_ns;
  CK(cudaMemsetAsync(h->base + L.off_res, 0, res_scratch_bytes(L.P, L.NZ), h->stream));
  CK(em2_adj_resident_launch(ar, h->stream));
  CK(cudaGetLastError());
  return SFD_OK;
}

int32_t sfd_adjoint_record(sfd_handle* h, int64_t nsteps) {
  g_err.clear();
  int r = adj_check(h);
  if (r) return r;
  if (!h->adj) return fail(SFD_ERR_STATE, "call sfd_adjoint_begin first");
  if (h->cfg.kind != SFD_ELECTROMAG2 || !adjoint_on_chip(h))
    return fail(SFD_ERR_BAD_ARG, "sfd_adjoint_record needs an electromag2 handle whose runs stay on chip");
  if (nsteps < 1 || nsteps > h->adj_seg)
    return fail(SFD_ERR_BAD_ARG, "recorded run of %lld steps outside [1, %d]", (long long)nsteps, h->adj_seg);
  if (h->step + nsteps > h->cfg.nstep) return fail(SFD_ERR_BAD_ARG, "recorded run goes past the source length");
  const AdjLayout A = adj_layout(h, h->adj_seg);
  const Layout& L = h->L;
  Ctl* ctl = (Ctl*)(h->base + L.off_ctl);
  float* slots = (float*)(h->base + L.off_slots);
  r = em2_save_slot0(h, A);
  if (r) return r;
  k_begin<<<std::min(1024, (L.nslots + 255) / 256 + 1), 256, 0, h->stream>>>(ctl, slots, L.nslots, (int)h->step);
  CK(cudaMemsetAsync(h->base + L.off_res, 0, res_scratch_bytes(L.P, L.NZ), h->stream));
  const Em2Resident own = resident_args(h, nsteps);
  CK(em2_resident_launch(em2_dump_args(h, A, h->step, nsteps), h->stream));  // receivers recorded as in sfd_run
  k_reduce_slots<<<1, 1024, 0, h->stream>>>(ctl, slots, L.nslots);
  // the dumping launch keeps the handle's state: take the last slot's
  const AdjState Sn = adj_state_at(A, h->adj + A.slots + A.state * (size_t)nsteps);
  const size_t fb = sizeof(float) * L.fsz;
  CK(cudaMemcpyAsync(own.Ex, Sn.Ex, fb, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(own.Ez, Sn.Ez, fb, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(own.Hy, Sn.Hy, fb, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(own.mExz, Sn.A, sizeof(float) * L.mem_sz[0], cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(own.mEzx, Sn.B, sizeof(float) * L.mem_sz[1], cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(own.mHyz, Sn.C, sizeof(float) * L.mem_sz[2], cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(own.mHyx, Sn.D, sizeof(float) * L.mem_sz[3], cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaGetLastError());
  h->adj_rec_s0 = h->step;
  h->adj_rec_n = nsteps;
  h->step += nsteps;
  return SFD_OK;
}

int32_t sfd_adjoint_segment(sfd_handle* h, int64_t nsteps) {
  g_err.clear();
  int r = adj_check(h);
  if (r) return r;
  if (!h->adj) return fail(SFD_ERR_STATE, "call sfd_adjoint_begin first");
  if (nsteps < 1 || nsteps > h->adj_seg) return fail(SFD_ERR_BAD_ARG, "segment of %lld steps outside [1, %d]", (long long)nsteps, h->adj_seg);
  if (h->adj_rec_n == nsteps && h->adj_rec_s0 + nsteps == h->step) {
    // sfd_adjoint_record ran these steps and kept every state: sweep only
    h->adj_rec_n = 0;
    return em2_adjoint_sweep_on_chip(h, adj_layout(h, h->adj_seg), h->adj_rec_s0, nsteps);
  }
  h->adj_rec_n = 0;
  const int64_t s0 = h->step;
  if (s0 + nsteps > h->cfg.nstep) return fail(SFD_ERR_BAD_ARG, "segment runs past the source length");
  if (h->cfg.kind == SFD_SEISMIC2) return s2_adjoint_segment(h, nsteps);
  const AdjLayout A = adj_layout(h, h->adj_seg);
  const Layout& L = h->L;
  const int NX = h->cfg.nx, NZ = h->cfg.nz;
  r = em2_save_slot0(h, A);
  if (r) return r;
  if (adjoint_on_chip(h)) {
    // forward recompute on chip: slot s + 1 <- the state after step s0 + s
    Em2Resident fr = em2_dump_args(h, A, s0, nsteps);
    fr.io.nrec = 0;
    CK(cudaMemsetAsync(h->base + L.off_res, 0, res_scratch_bytes(L.P, L.NZ), h->stream));
    CK(em2_resident_launch(fr, h->stream));
    return em2_adjoint_sweep_on_chip(h, A, s0, nsteps);
  }
  // forward recompute: slot s -> slot s+1
  k_begin<<<std::min(1024, (L.nslots + 255) / 256 + 1), 256, 0, h->stream>>>((Ctl*)(h->base + L.off_ctl),
                                                                            (float*)(h->base + L.off_slots), L.nslots, (int)s0);
  Em2Step st = h->em2s[0];
  for (int64_t s = 0; s < nsteps; ++s) {
    const AdjState a0 = adj_state_at(A, h->adj + A.slots + A.state * (size_t)s);
    const AdjState a1 = adj_state_at(A, h->adj + A.slots + A.state * (size_t)(s + 1));
    st.Ex0 = a0.Ex; st.Ez0 = a0.Ez; st.Hy0 = a0.Hy; st.mExz0 = a0.A; st.mEzx0 = a0.B; st.mHyz0 = a0.C; st.mHyx0 = a0.D;
    st.Ex1 = a1.Ex; st.Ez1 = a1.Ez; st.Hy1 = a1.Hy; st.mExz1 = a1.A; st.mEzx1 = a1.B; st.mHyz = a1.C; st.mHyx = a1.D;
    em2_step(st, h->launch1, h->zb, (int)s, h->stream);
  }
  // adjoint sweep over the segment, last step first
  Em2Adj a;
  const Em2Args& e = h->em2;
  a.NX = NX; a.NZ = NZ; a.P = L.P; a.W = L.W;
  a.CAx = e.CAx; a.CBx = e.CBx; a.CAz = e.CAz; a.CBz = e.CBz;
  a.X = e.X; a.Z = e.Z; a.dbH = e.dbH;
  a.TH = (float*)(h->adj + A.th); a.MEx = (float*)(h->adj + A.mex); a.MEz = (float*)(h->adj + A.mez);
  a.gCAx = (float*)(h->adj + A.g[0]); a.gCBx = (float*)(h->adj + A.g[1]);
  a.gCAz = (float*)(h->adj + A.g[2]); a.gCBz = (float*)(h->adj + A.g[3]);
  a.srcacc = (float*)(h->adj + A.acc);
  a.srcfn = (const float*)(h->base + L.off_src);
  a.nstep = h->cfg.nstep; a.si = h->em2.io.si; a.sk = h->em2.io.sk;
  a.rec = (const int*)(h->base + L.off_rec); a.nrec = h->cfg.nrec; a.resid = h->adj_resid;
  for (int64_t s = nsteps - 1; s >= 0; --s) {
    const AdjState S = adj_state_at(A, h->adj + A.slots + A.state * (size_t)s);
    const AdjState S1 = adj_state_at(A, h->adj + A.slots + A.state * (size_t)(s + 1));
    const AdjState Lc = adj_state_at(A, h->adj + A.lam[h->adj_cur]);
    const AdjState Ln = adj_state_at(A, h->adj + A.lam[1 - h->adj_cur]);
    adj_step(a, S, S1, Lc, Ln, (int)(s0 + s), h->stream);
    h->adj_cur ^= 1;
  }
  CK(cudaGetLastError());
  return SFD_OK;
}

int32_t sfd_adjoint_gradient(sfd_handle* h, double* out, int64_t count) {
  g_err.clear();
  int r = adj_check(h);
  if (r) return r;
  if (!h->adj) return fail(SFD_ERR_STATE, "call sfd_adjoint_begin first");
  if (h->cfg.kind == SFD_SEISMIC2) return s2_adjoint_gradient(h, out, count);
  const int NX = h->cfg.nx, NZ = h->cfg.nz, P = h->L.P;
  const size_t N2 = (size_t)NX * NZ;
  if (!out || count != (int64_t)(6 * N2)) return fail(SFD_ERR_BAD_ARG, "gradient needs 6 planes of %dx%d", NX, NZ);
  const AdjLayout A = adj_layout(h, h->adj_seg);
  std::vector<float> g[4];
  for (int q = 0; q < 4; ++q) {
    g[q].resize((size_t)P * NZ);
    CK(cudaMemcpyAsync(g[q].data(), h->adj + A.g[q], sizeof(float) * g[q].size(), cudaMemcpyDeviceToHost, h->stream));
  }
  float acc[2];
  CK(cudaMemcpyAsync(acc, h->adj + A.acc, sizeof acc, cudaMemcpyDeviceToHost, h->stream));
  Ctl ctl;
  CK(cudaMemcpyAsync(&ctl, h->base + h->L.off_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (ctl.err) return fail(SFD_ERR_TIMEOUT, "on-chip adjoint sweep: a neighbouring tile did not answer within 2 s");
  const double dt = h->cfg.dt;
  r = ensure_model_planes(h);
  if (r) return r;
  const double *e11 = h->model.get(), *e13 = e11 + N2, *e33 = e11 + 2 * N2;
  const double *s11 = e11 + 3 * N2, *s13 = e11 + 4 * N2, *s33 = e11 + 5 * N2;
  double *g11 = out, *g13 = out + N2, *g33 = out + 2 * N2, *gs11 = out + 3 * N2, *gs13 = out + 4 * N2,
         *gs33 = out + 5 * N2;
  std::fill(out, out + 6 * N2, 0.0);
  auto G = [&](int q, int i, int k) -> double {
    if (i < 0 || i >= NX || k < 0 || k >= NZ) return 0.0;
    return g[q][(size_t)k * P + i];
  };
  for (int k = 0; k < NZ; ++k)
    for (int i = 0; i < NX; ++i) {
      const size_t n = (size_t)i + (size_t)NX * k;
      // caEx(i,k) enters CAx(i,k) and CAx(i,k+1); caEz(i,k) enters CAz(i,k) and CAz(i+1,k)
      const double dcaX = 0.5 * (G(0, i, k) + G(0, i, k + 1)), dcbX = 0.5 * (G(1, i, k) + G(1, i, k + 1));
      const double dcaZ = 0.5 * (G(2, i, k) + G(2, i + 1, k)), dcbZ = 0.5 * (G(3, i, k) + G(3, i + 1, k));
      // ca = (1-u)/(1+u), cb = (dt/e)/(1+u), u = s dt / (2 e), e = (eps_a + eps_b) eps0 (electromagfdtd.f95:164-176)
      auto chain = [&](double epsr, double sig, double dca, double dcb, double* de, double* ds) {
        const double ep = epsr * kEps0;
        const double u = sig * dt / (2.0 * ep);
        const double w = 1.0 / ((1.0 + u) * (1.0 + u));
        const double dca_de = 2.0 * u / ep * w, dca_ds = -dt / ep * w;
        const double dcb_de = -dt / (ep * ep) * w, dcb_ds = -dt * dt / (2.0 * ep * ep) * w;
        *de = (dca * dca_de + dcb * dcb_de) * kEps0;
        *ds = dca * dca_ds + dcb * dcb_ds;
      };
      double deX, dsX, deZ, dsZ;
      chain(e11[n] + e13[n], s11[n] + s13[n], dcaX, dcbX, &deX, &dsX);
      chain(e13[n] + e33[n], s13[n] + s33[n], dcaZ, dcbZ, &deZ, &dsZ);
      g11[n] = deX;
      g33[n] = deZ;
      g13[n] = deX + deZ;
      gs11[n] = dsX;
      gs33[n] = dsZ;
      gs13[n] = dsX + dsZ;
    }
  // source: Ex(s) += srcx dt / eps11(s), Ez(s) += srcz dt / eps33(s) (electromagfdtd.f95:300-301)
  const int si = h->em2.io.si, sk = h->em2.io.sk;
  if (si >= 0) {
    const size_t n = (size_t)si + (size_t)NX * sk;
    g11[n] += -(double)acc[0] / e11[n];
    g33[n] += -(double)acc[1] / e33[n];
  }
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
