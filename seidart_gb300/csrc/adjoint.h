// Device-side structures of the electromag2 discrete adjoint (adjoint_em2.cu).
#pragma once
#include <cuda_runtime.h>
#include "sfd_solvers.h"

namespace sfd {

// One state (forward) or adjoint state: fields on the full grid (pitch P),
// memory variables on their strips (A, C: z-strip; B, D: x-strip).
struct AdjState {
  float *Ex, *Ez, *Hy, *A, *B, *C, *D;
};

struct Em2Adj {
  int NX, NZ, P, W;
  const float *CAx, *CBx, *CAz, *CBz;  // staggered-averaged coefficients
  AxisTab X, Z;
  float dbH;
  float *TH, *MEx, *MEz;            // adjoint of Hy', E-half parts of the E adjoints
  float *gCAx, *gCBx, *gCAz, *gCBz; // dJ/d(averaged coefficient) per cell, summed over steps
  float* srcacc;                    // sum_t lam_E(src) * amplitude(t), x and z
  const float* srcfn;               // scaled source amplitudes [2][nstep]
  int nstep, si, sk;
  const int* rec;
  int nrec;
  const float* resid;               // dJ/d(trace) [nstep][2][nrec]
};

// S: forward state before step t, S1: after it (its Hy is Hy' except on the
// Dirichlet edges; its C and D are this step's memory variables).
void adj_step(const Em2Adj& a, const AdjState& S, const AdjState& S1, const AdjState& L, const AdjState& Ln, int t,
              cudaStream_t s);

}  // namespace sfd
