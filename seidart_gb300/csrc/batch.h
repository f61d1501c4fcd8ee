// Device-side description of a batch of 2-D models for the persistent kernel.
#pragma once
#include <algorithm>
#include <cuda_runtime.h>
#include "sfd_solvers.h"

namespace sfd {

#define SFD_BATCH_EM2 0
#define SFD_BATCH_SEIS2 1

struct GridBarrier {
  unsigned count;
  unsigned gen;
  int err;
  int pad;
};

struct BatchModel {
  int kind;    // SFD_BATCH_EM2 / SFD_BATCH_SEIS2
  int gx;      // tiles along x
  int ntiles;  // gx * gy
  int nslots;  // norm slots of the model (= its tile count)
  int cur;     // copy holding the model's state when the run starts
  Em2Step em2[2];
  Seis2Step s2[2];
};

// Consecutive models of one geometry that read the same coefficient planes
// (shots of one model) form a group whose tiles are interleaved: tile q of the
// group is tile q / n of member q % n, so the members' copies of a tile run
// back to back and the shared coefficients come from L2 after the first.
struct BatchGroup {
  int first;   // first model of the group
  int n;       // members
  int tile0;   // first tile number of the group
  int ntiles;  // n * tiles per member
};

const void* batch_kernel_ptr(int zb);
void batch_begin(const BatchModel* models, int nmodels, const int* steps, GridBarrier* bar, cudaStream_t s);
void batch_end(const BatchModel* models, int nmodels, int nsteps, cudaStream_t s);
cudaError_t batch_launch(int zb, int grid, const BatchModel* models, const BatchGroup* groups, int ngroups,
                         int total_tiles, int nsteps, GridBarrier* bar, unsigned long long limit_ns, int extra,
                         cudaStream_t s);

}  // namespace sfd
