// The handle behind the C ABI, its state layout in the caller's device
// buffer, and the helpers that the ABI's translation units share:
// sfd_api.cu (handles, models, runs), sfd_adjoint.cu (checkpoints and the
// discrete adjoints) and sfd_batch_api.cu (batched runs).  Internal: no
// caller of the library includes it.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "../../include/seidart_gb300.h"
#include "adjoint.h"
#include "adjoint_s2.h"
#include "batch.h"
#include "resident.h"
#include "sfd_solvers.h"

namespace sfd {

constexpr double kPI = 3.141592653589793238462643;
constexpr double kMu0 = 4.0 * kPI * 1.0e-7;
constexpr double kEps0 = 8.85418782e-12;
constexpr int kGraphSteps = 32;
constexpr unsigned long long kDefaultWaitNs = 2000000000ull;  // bounded device waits: 2 s
// Added to the awaited edge tags by the timeout test aid: tags are step
// numbers + 1 or 2, so no tile ever writes a biased one.
constexpr unsigned kStallTagBias = 0x40000000u;

// The calling thread's last error message (sfd_last_error).
extern thread_local std::string g_err;
// Sets the message and returns code.
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);

#define CK(call)                                        \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

int nfields(int kind);
int nchan(int kind);
// Source components the caller gives (real time functions, x [y] z).
int nsrc(int kind);
// Stress source components: xx zz xz in 2-D, xx yy zz xy xz yz in 2.5-D.
int nstress(int kind);
// Density method of the flags: 0 arithmetic, 1 none, 2 geometric, 3 harmonic.
int density_method(int flags);
int nplanes(int kind);
bool is3(int kind);
// Strip axis of each memory variable, in the oracle's order.
const char* mem_axes(int kind);
int ncoef(int kind);
size_t align256(size_t x);
bool cpml2d(const sfd_config& c);
// Whether a handle steps in the single-pass form (the others: two kernels per step).
bool single_pass(const sfd_config& c);
// Edge fields of an on-chip run (resident.h): electromag2 2, seismic2 6.
int res_edge_fields(int kind);

struct Layout {
  int P, NX, NY, NZ, W, ysplit, nslots;
  size_t fsz;  // floats per field
  size_t off_ctl, off_fields, off_mem[18], mem_sz[18], off_fieldsB, off_memB[18], off_coef, coef_plane, off_axis[3],
      off_q3, off_src, off_rec, off_traces, off_slots, off_res, total;
};

}  // namespace sfd

struct sfd_handle_s {
  sfd_config cfg;
  sfd::Layout L;
  char* base;
  cudaStream_t stream;       // caller's stream
  cudaStream_t cap_stream;   // private stream used only to capture graphs
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // indexed by the parity the graph starts from
  // a seismic2 adjoint segment's work (s2_adjoint_segment) and what it was captured for
  cudaGraphExec_t adj_graph = nullptr;
  int64_t adj_graph_n = 0;
  int adj_graph_cur = 0, adj_graph_seg = 0;
  bool adj_graph_sweep_only = false;  // the graph holds the sweep alone (the recompute ran on chip)
  const char* adj_graph_work = nullptr;
  const float* adj_graph_resid = nullptr;
  bool have_model = false, have_cpml = false;
  bool have_ssrc = false;       // a stress source was set (seismic kinds)
  bool have_force_src = false;  // a force (or E) source was set
  bool single = false;  // single-pass 2-D steps (ping-pong state)
  int cur = 0;          // copy holding the current state (single-pass only)
  int zb = 2;           // rows per thread of the single-pass tiles
  sfd::Em2Step em2s[2];      // [p]: reads copy p, writes copy 1-p
  sfd::Seis2Step s2s[2];
  sfd::Launch launch1;       // single-pass geometry
  int res_state = 0;    // on-chip runs: 0 not yet checked, 1 usable, -1 not usable
  sfd::ResPlan res_plan;     // electromag2
  sfd::ResPlan res_plan_adj;  // electromag2, the adjoint sweep's (no three-row tiles)
  sfd::Seis2ResPlan s2_plan;  // seismic2
  int64_t step = 0;
  unsigned long long wait_ns = sfd::kDefaultWaitNs;  // longest wait of an on-chip run for a neighbouring tile
  bool stall_waits = false;                          // timeout test aid: waits expect tags no tile writes
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
  // adjoint workspace
  char* adj = nullptr;
  int adj_seg = 0;
  int adj_cur = 0;
  int64_t adj_rec_s0 = 0;  // sfd_adjoint_record: the recorded run's first step and length (0: none)
  int64_t adj_rec_n = 0;
  const float* adj_resid = nullptr;
  int adj_res_state = 0;  // on-chip adjoint sweeps: 0 not yet checked, 1 usable, -1 not usable
  sfd::Em2Args em2;
  sfd::Em2cArgs em2c;
  sfd::Seis2Args s2;
  sfd::Seis25Args s25;
  sfd::Em25Args em25;
  sfd::Launch launch;
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
  sfd::IoArgs io() const {
    sfd::IoArgs io;
    io.ctl = (sfd::Ctl*)(base + L.off_ctl);
    io.slots = (float*)(base + L.off_slots);
    io.src = (const float*)(base + L.off_src);
    io.nstep = cfg.nstep;
    io.ssrc = have_ssrc ? (const float*)(base + L.off_src) + (size_t)sfd::nchan(cfg.kind) * cfg.nstep : nullptr;
    io.si = io.sj = io.sk = -1;
    io.rec = (const int*)(base + L.off_rec);
    io.nrec = cfg.nrec;
    io.traces = (float*)(base + L.off_traces);
    return io;
  }
};

namespace sfd {

// Starts a run at `step` on the handle's stream: the control block's step
// base and error word, the norm slots cleared.
void begin_run(sfd_handle_s* h, int64_t step);
// The run's largest field norm from the per-block slots into the control block.
void reduce_norms(sfd_handle_s* h);
// Whether this handle's runs go on chip (decided once per handle).
bool resident_usable(sfd_handle_s* h);
// The on-chip electromag2 and seismic2 runs of nsteps steps from the handle's state.
Em2Resident resident_args(const sfd_handle_s* h, int64_t nsteps);
Seis2Resident seis2_resident_args(const sfd_handle_s* h, int64_t nsteps);
// The FP64 model planes, expanded from the material ids if the model came as ids.
int ensure_model_planes(sfd_handle_s* h);

}  // namespace sfd
