// Device-side structures of the seismic2 discrete adjoint (adjoint_s2.cu).
#pragma once
#include <cuda_runtime.h>
#include "sfd_solvers.h"

namespace sfd {

// One forward or adjoint state: velocities and stresses on the full grid
// (pitch P), the twelve memory variables in sfd_num_memory order, each on
// its strip (x-strip index k * 2W + strip(i), z-strip strip(k) * P + i).
struct S2State {
  float *vx, *vz, *sxx, *szz, *sxz;
  float* m[12];
};

struct S2Adj {
  int NX, NZ, P, W;
  // update coefficients of the forward step (sfd_set_model)
  const float *A11, *A13, *A15, *A33, *A35, *B15, *B35, *B55, *dtrx, *dtrz, *gxp, *gzp;
  AxisTab X, Z;
  float* tmp[12];  // scratch planes: lc1 lc2 ld1 ld2, la1..la4, lb1..lb4
  // dJ/d(coefficient) per cell, summed over the steps
  float *gA11, *gA13, *gA15, *gA33, *gA35, *gB15, *gB35, *gB55, *gdtrx, *gdtrz, *ggxp, *ggzp;
  float* srcacc;       // sum_t (lam_vx f_x(t) + lam_vz f_z(t)) at the source cell, f the scaled amplitudes
  const float* srcfn;  // scaled source amplitudes [2][nstep]
  int nstep, si, sk;
  const int* recmap;   // per cell (pitch P): its first receiver, or -1
  const int* recnext;  // per receiver: the next one at the same cell, or -1
  int nrec;
  const float* resid;  // dJ/d(trace) [nstep][2][nrec]
  const Ctl* ctl;      // its base + a step's relative index = the step
};

// Byte offsets of vx vz sxx szz sxz and the twelve memory variables inside
// one state (forward slots and adjoint states alike).
struct S2Offsets {
  size_t o[17];
};

// The adjoint steps base + nsteps - 1 down to base (base = a.ctl->base) of
// one segment: slot s (at slots + s * stride) holds the forward state before
// step base + s, slot nsteps the state after the last; lam[cur] is the
// adjoint of that last state, and the adjoint states alternate, so the
// segment ends in lam[cur ^ (nsteps & 1)].  Queued on stream s.
void s2_adj_sweep(const S2Adj& a, char* slots, size_t stride, const S2Offsets& off, char* lam0, char* lam1, int cur,
                  int nsteps, cudaStream_t s);
// recmap (P * NZ cells) and recnext (nrec) of S2Adj from the device receiver
// list rec ((i, j, k) triples).
cudaError_t s2_adj_recmap(const int* rec, int nrec, int P, int NZ, int* recmap, int* recnext, cudaStream_t s);

}  // namespace sfd
