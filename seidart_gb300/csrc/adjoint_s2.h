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
  const int* rec;
  int nrec;
  const float* resid;  // dJ/d(trace) [nstep][2][nrec]
  const Ctl* ctl;      // its base + a step's relative index = the step
};

// One reverse step t = a.ctl->base + rel: S is the forward state before step
// t, S1 the state after it; Ln the adjoint of S1 (receives this step's
// residual), Lc the adjoint of S written in full.
void s2_adj_step(const S2Adj& a, const S2State& S, const S2State& S1, const S2State& Ln, const S2State& Lc, int rel,
                 cudaStream_t s);

}  // namespace sfd
