// C ABI, part 3: checkpoints and the discrete adjoints -- the electromag2
// adjoint (on chip: a recompute launch and a sweep launch per checkpoint
// segment, or the per-step kernels; without recompute after
// sfd_adjoint_record) and the seismic2 adjoint (recompute by the handle's
// own steps and graph-replayed transposed steps).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "handle.h"

using namespace sfd;

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
  if (em2_adj_resident_prepare(h->res_plan_adj, h->cfg.nx, h->cfg.nz, h->L.W, &per_sm) != cudaSuccess || per_sm < 1) {
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
  size_t field, mem[12], state, lam[2], tmp, g, acc, recmap, recnext, slots, total;
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
  A.recmap = o; o += align256(sizeof(int) * L.P * (size_t)h->cfg.nz);
  A.recnext = o; o += align256(sizeof(int) * (size_t)std::max(1, h->cfg.nrec));
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
cudaError_t s2_segment_work(sfd_handle* h, const S2AdjLayout& A, int64_t nsteps, int cur, bool recompute,
                            cudaStream_t stream) {
  const Layout& L = h->L;
  char* slots = h->adj + A.slots;
  cudaError_t e = cudaSuccess;
  if (!recompute) {
    // the slots already hold the segment's states (the on-chip recompute)
  } else if (h->single) {  // the single-pass step kernel between slots; its in-place memory variables copied ahead
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
  a.recmap = (const int*)(h->adj + A.recmap); a.recnext = (const int*)(h->adj + A.recnext);
  a.nrec = h->cfg.nrec; a.resid = h->adj_resid;
  a.ctl = (const Ctl*)(h->base + L.off_ctl);
  S2Offsets off;
  for (int q = 0; q < 5; ++q) off.o[q] = q * A.field;
  for (int m = 0; m < 12; ++m) off.o[5 + m] = A.mem[m];
  s2_adj_sweep(a, slots, A.state, off, h->adj + A.lam[0], h->adj + A.lam[1], cur, (int)nsteps, stream);
  return cudaGetLastError();
}

// One seismic2 segment: slot 0 <- the handle's state, the step base, then
// the segment's work, replayed from a CUDA graph captured on the handle's
// private stream when it has one (one capture per segment length and
// starting adjoint state; the graph is dropped with the handle's others).
// A handle whose runs go on chip recomputes the segment in one on-chip
// launch (resident_s2.cu, dumping every step's state) ahead of the graph,
// which then holds the adjoint steps alone.
// The on-chip seismic2 run of nsteps steps from slot 0 (the state before
// step s0) that writes the state after step s0 + s into slot s + 1 and
// leaves slot 0 as it was; receivers as the handle's.
Seis2Resident s2_dump_args(const sfd_handle* h, const S2AdjLayout& A, int64_t s0, int64_t nsteps) {
  const S2State S0 = s2_state_at(A, h->adj + A.slots);
  Seis2Resident fr = seis2_resident_args(h, nsteps);
  fr.vx = S0.vx; fr.vz = S0.vz; fr.sxx = S0.sxx; fr.szz = S0.szz; fr.sxz = S0.sxz;
  fr.m_vxx = S0.m[0]; fr.m_vzz = S0.m[1]; fr.m_vxz = S0.m[2]; fr.m_vzx = S0.m[3];
  fr.m_sxx_x = S0.m[4]; fr.m_szz_z = S0.m[5]; fr.m_sxz_x = S0.m[6]; fr.m_sxz_z = S0.m[7];
  fr.m2_vxx = S0.m[8]; fr.m2_vzz = S0.m[9]; fr.m2_vxz = S0.m[10]; fr.m2_vzx = S0.m[11];
  fr.t0 = (int)s0;
  fr.dump.base = h->adj + A.slots;
  fr.dump.stride = A.state;
  for (int q = 0; q < 5; ++q) fr.dump.off[q] = q * A.field;
  for (int m = 0; m < 12; ++m) fr.dump.off[5 + m] = A.mem[m];
  return fr;
}

int s2_adjoint_segment(sfd_handle* h, int64_t nsteps, bool recorded, int64_t s0) {
  const S2AdjLayout A = s2_adj_layout(h, h->adj_seg);
  if (!recorded) {
    int r = s2_save_state(h, A, h->adj + A.slots);
    if (r) return r;
  }
  begin_run(h, s0);
  const bool on_chip = recorded || resident_usable(h);
  if (on_chip && !recorded) {  // the recompute as one on-chip launch that writes every step's state into its slot
    const Layout& L = h->L;
    Seis2Resident fr = s2_dump_args(h, A, s0, nsteps);
    fr.io.nrec = 0;
    CK(cudaMemsetAsync(h->base + L.off_res, 0, res_scratch_bytes(L.P, L.NZ, res_edge_fields(h->cfg.kind)), h->stream));
    CK(seis2_resident_launch(fr, h->stream));
  }
  if (!h->cap_stream) {
    CK(s2_segment_work(h, A, nsteps, h->adj_cur, !on_chip, h->stream));
  } else {
    const bool reuse = h->adj_graph && h->adj_graph_n == nsteps && h->adj_graph_cur == h->adj_cur &&
                       h->adj_graph_work == h->adj && h->adj_graph_resid == h->adj_resid &&
                       h->adj_graph_seg == h->adj_seg && h->adj_graph_sweep_only == on_chip;
    if (!reuse) {
      if (h->adj_graph) { cudaGraphExecDestroy(h->adj_graph); h->adj_graph = nullptr; }
      cudaGraph_t g = nullptr;
      CK(cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal));
      const cudaError_t ew = s2_segment_work(h, A, nsteps, h->adj_cur, !on_chip, h->cap_stream);
      const cudaError_t ec = cudaStreamEndCapture(h->cap_stream, &g);
      if (ew != cudaSuccess) { if (g) cudaGraphDestroy(g); return cuda_fail(ew, "seismic2 adjoint segment"); }
      if (ec != cudaSuccess) return cuda_fail(ec, "cudaStreamEndCapture");
      const cudaError_t ei = cudaGraphInstantiate(&h->adj_graph, g, 0);
      cudaGraphDestroy(g);
      if (ei != cudaSuccess) { h->adj_graph = nullptr; return cuda_fail(ei, "cudaGraphInstantiate"); }
      h->adj_graph_n = nsteps; h->adj_graph_cur = h->adj_cur; h->adj_graph_work = h->adj;
      h->adj_graph_resid = h->adj_resid; h->adj_graph_seg = h->adj_seg; h->adj_graph_sweep_only = on_chip;
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
    begin_run(h, h->step);
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
    reduce_norms(h);
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
  if (h->cfg.kind == SFD_SEISMIC2) {  // each cell's receivers, for the residual of the adjoint's v phase
    const S2AdjLayout A = s2_adj_layout(h, seg_steps);
    CK(s2_adj_recmap((const int*)(h->base + h->L.off_rec), h->cfg.nrec, h->L.P, h->cfg.nz, (int*)(h->adj + A.recmap),
                     (int*)(h->adj + A.recnext), h->stream));
  }
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
  ar.plan = h->res_plan_adj;
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
  if (h->cfg.kind == SFD_ELECTROMAG2 ? !adjoint_on_chip(h) : !resident_usable(h))
    return fail(SFD_ERR_BAD_ARG, "sfd_adjoint_record needs a handle whose runs stay on chip");
  if (nsteps < 1 || nsteps > h->adj_seg)
    return fail(SFD_ERR_BAD_ARG, "recorded run of %lld steps outside [1, %d]", (long long)nsteps, h->adj_seg);
  if (h->step + nsteps > h->cfg.nstep) return fail(SFD_ERR_BAD_ARG, "recorded run goes past the source length");
  if (h->cfg.kind == SFD_SEISMIC2) {
    const S2AdjLayout A = s2_adj_layout(h, h->adj_seg);
    const Layout& L = h->L;
    r = s2_save_state(h, A, h->adj + A.slots);
    if (r) return r;
    begin_run(h, h->step);
    CK(cudaMemsetAsync(h->base + L.off_res, 0, res_scratch_bytes(L.P, L.NZ, res_edge_fields(h->cfg.kind)), h->stream));
    const Seis2Resident own = seis2_resident_args(h, nsteps);
    CK(seis2_resident_launch(s2_dump_args(h, A, h->step, nsteps), h->stream));  // receivers recorded as in sfd_run
    reduce_norms(h);
    // the dumping launch keeps the handle's state: take the last slot's
    const S2State Sn = s2_state_at(A, h->adj + A.slots + A.state * (size_t)nsteps);
    float* dst[17] = {own.vx, own.vz, own.sxx, own.szz, own.sxz, own.m_vxx, own.m_vzz, own.m_vxz, own.m_vzx,
                      own.m_sxx_x, own.m_szz_z, own.m_sxz_x, own.m_sxz_z, own.m2_vxx, own.m2_vzz, own.m2_vxz,
                      own.m2_vzx};
    const float* src[17] = {Sn.vx, Sn.vz, Sn.sxx, Sn.szz, Sn.sxz, Sn.m[0], Sn.m[1], Sn.m[2], Sn.m[3], Sn.m[4], Sn.m[5],
                            Sn.m[6], Sn.m[7], Sn.m[8], Sn.m[9], Sn.m[10], Sn.m[11]};
    for (int q = 0; q < 17; ++q) {
      const size_t n = q < 5 ? L.fsz : L.mem_sz[q - 5];
      CK(cudaMemcpyAsync(dst[q], src[q], sizeof(float) * n, cudaMemcpyDeviceToDevice, h->stream));
    }
    CK(cudaGetLastError());
    h->adj_rec_s0 = h->step;
    h->adj_rec_n = nsteps;
    h->step += nsteps;
    return SFD_OK;
  }
  const AdjLayout A = adj_layout(h, h->adj_seg);
  const Layout& L = h->L;
  r = em2_save_slot0(h, A);
  if (r) return r;
  begin_run(h, h->step);
  CK(cudaMemsetAsync(h->base + L.off_res, 0, res_scratch_bytes(L.P, L.NZ), h->stream));
  const Em2Resident own = resident_args(h, nsteps);
  CK(em2_resident_launch(em2_dump_args(h, A, h->step, nsteps), h->stream));  // receivers recorded as in sfd_run
  reduce_norms(h);
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
    if (h->cfg.kind == SFD_SEISMIC2) return s2_adjoint_segment(h, nsteps, true, h->adj_rec_s0);
    return em2_adjoint_sweep_on_chip(h, adj_layout(h, h->adj_seg), h->adj_rec_s0, nsteps);
  }
  h->adj_rec_n = 0;
  const int64_t s0 = h->step;
  if (s0 + nsteps > h->cfg.nstep) return fail(SFD_ERR_BAD_ARG, "segment runs past the source length");
  if (h->cfg.kind == SFD_SEISMIC2) return s2_adjoint_segment(h, nsteps, false, s0);
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
  begin_run(h, s0);
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
