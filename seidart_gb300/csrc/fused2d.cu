// Single-pass time steps of the 2-D solvers (electromag2, seismic2).
//
// One launch per time step.  A block owns a tile of 8*ZB rows (128 cells wide
// for electromag2, 32 for seismic2); it
// first computes the first half-step (Hy, or the three stresses) on its tile
// plus the one-cell halo the second half-step needs, keeping those values in
// shared memory, then performs the second half-step (Ex/Ez, or vx/vz) on its
// own cells.  Every field is read from the "old" copy and written to the
// "new" copy of a ping-pong pair, so tiles never see a neighbour's partial
// update; the memory variables of the first half are ping-ponged too (halo
// cells re-derive them), those of the second half are updated in place.
// Each field and coefficient therefore crosses HBM once per step instead of
// the two reads of the two-kernel form.  The arithmetic per cell is the same
// as em2.cu / seis2.cu (legacy/fortran/electromagfdtd.f95:249-321,
// legacy/fortran/seismicfdtd.f95:247-379), so both forms give the same fields.
#include "sfd_solvers.h"
#include "fused2d.cuh"

namespace sfd {

namespace {

constexpr int TX = 32, TY = 8;

template <int ZB>
__global__ void __launch_bounds__(TX * TY) em2_step_kernel(Em2Step a, int rel) {
  __shared__ __align__(16) float sH[TY * ZB + 1][kEm2Row];
  em2_tile<ZB, true>(a, a.io.ctl->base + rel, blockIdx.x, blockIdx.y, gridDim.x, sH);
}

template <int ZB>
__global__ void __launch_bounds__(TX * TY) seis2_step_kernel(Seis2Step a, int rel) {
  __shared__ float sS[3][TY * ZB + 2][TX + 2];
  seis2_tile<ZB, true>(a, a.io.ctl->base + rel, blockIdx.x, blockIdx.y, gridDim.x, sS);
}

__global__ void em2_step_finalize_kernel(Em2Step a, int t_last) {
  const float* ch[2] = {a.Ex0, a.Ez0};  // caller passes the args whose "old" copy is current
  gather_receivers<2>(a.io.rec, a.io.nrec, a.io.traces, t_last, ch, a.P, 1, false);
}

__global__ void seis2_step_finalize_kernel(Seis2Step a, int t_last) {
  const float* ch[2] = {a.vx0, a.vz0};
  gather_receivers<2>(a.io.rec, a.io.nrec, a.io.traces, t_last, ch, a.P, 1, false);
}

}  // namespace

Launch em2_step_launch(const Em2Step& a, int zb) {
  Launch L;
  L.block = dim3(TX, TY, 1);
  L.grid = dim3((a.NX + 4 * TX - 1) / (4 * TX), (a.NZ + TY * zb - 1) / (TY * zb), 1);  // 128-cell-wide tiles
  L.nslots = L.grid.x * L.grid.y;
  return L;
}

void em2_step(const Em2Step& a, const Launch& L, int zb, int rel, cudaStream_t s) {
  switch (zb) {
    case 1: em2_step_kernel<1><<<L.grid, L.block, 0, s>>>(a, rel); break;
    case 2: em2_step_kernel<2><<<L.grid, L.block, 0, s>>>(a, rel); break;
    default: em2_step_kernel<4><<<L.grid, L.block, 0, s>>>(a, rel); break;
  }
}

void em2_step_finalize(const Em2Step& a, int t_last, cudaStream_t s) {
  em2_step_finalize_kernel<<<1, 256, 0, s>>>(a, t_last);
}

Launch seis2_step_launch(const Seis2Step& a, int zb) {
  Launch L;
  L.block = dim3(TX, TY, 1);
  L.grid = dim3((a.NX + TX - 1) / TX, (a.NZ + TY * zb - 1) / (TY * zb), 1);
  L.nslots = L.grid.x * L.grid.y;
  return L;
}

void seis2_step(const Seis2Step& a, const Launch& L, int zb, int rel, cudaStream_t s) {
  switch (zb) {
    case 1: seis2_step_kernel<1><<<L.grid, L.block, 0, s>>>(a, rel); break;
    case 2: seis2_step_kernel<2><<<L.grid, L.block, 0, s>>>(a, rel); break;
    default: seis2_step_kernel<4><<<L.grid, L.block, 0, s>>>(a, rel); break;
  }
}

void seis2_step_finalize(const Seis2Step& a, int t_last, cudaStream_t s) {
  seis2_step_finalize_kernel<<<1, 256, 0, s>>>(a, t_last);
}

}  // namespace sfd
