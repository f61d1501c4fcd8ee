// SM-resident 2-D time stepping: a whole run in one cooperative launch, with
// every tile's fields, coefficients and memory variables held in shared
// memory for all of its steps.
//
// The grid is cut into ntx x ntz tiles of TW x TZ cells, one CTA per tile and
// at most one CTA per SM.  Per step a CTA exchanges only its one-cell edges
// with its neighbours, through small edge arrays in global memory (L2); the
// edge words carry their step, which is the only synchronisation between
// tiles.  Global memory holds the state only before and after the run.
#pragma once
#include <cuda_runtime.h>
#include "sfd_solvers.h"

namespace sfd {

// Largest number of tile rows, and of tiles in one tile row; the edge arrays
// of a handle are sized for it.
constexpr int kResMaxTiles1D = 32;
// Largest number of tiles (CTAs, at most one per SM) of one on-chip run.
constexpr int kResMaxTiles = 256;
// Threads of a CTA: up to 15 warps own the cells (four cells of kResRows
// rows per thread, kResRows3 in interior electromag2 tiles), the last warp
// moves the tile's edges to and from the neighbouring tiles.
constexpr int kResThreads = 512;
constexpr int kResCellThreads = kResThreads - 32;
constexpr int kResRows = 2;
// Rows per thread in an electromag2 tile of interior cells only (no CPML
// strip, no Dirichlet plane), whose cells all take the short update: the
// planner gives such tiles more cells than the others, so that the tiles
// with the longer strip and boundary updates can be made smaller.
constexpr int kResRows3 = 3;
// Receivers a CTA lists in shared memory; a tile holding more scans the
// whole receiver list every step instead.
constexpr int kResMaxLocalRec = 256;

// Tiling of one on-chip run: ntz tile rows, each cut into its own tiles.
// tile[b] packs x0 | x1 << 16, z0 | z1 << 16, row | (index in row) << 16 and
// the tile count of its row | (interior tile: kResRows3 rows per thread) << 16;
// column bounds are multiples of 4 (except NX).
// Tiles that hold CPML strip or boundary cells take the longer update and are
// made smaller.
struct ResPlan {
  int ntiles, ntz;
  int4 tile[kResMaxTiles];
  size_t smem;  // dynamic shared memory of the largest tile
};

// Edge arrays inside a handle's state buffer.  Every edge value travels as
// one 8-byte word {value, tag}, the tag being one more than the step that
// reads the value, so a reader polls the words it needs until their tags
// match and needs no separate flag, fence or second load.  Two copies,
// selected by the parity of the reading step.
struct ResScratch {
  uint2* erow;  // [2 parity][2 fields][kResMaxTiles1D][P]: edge rows
  uint2* ecol;  // [2 parity][2 fields][kResMaxTiles1D][NZp]: edge columns
  int NZp;
};

__host__ __device__ inline int res_nzp(int NZ) { return (NZ + 31) & ~31; }

// Let `fn` take as much dynamic shared memory as the current device allows
// (its opt-in limit less the kernel's static shared memory).  The limit is a
// property of the function, shared by every handle: set to one plan's size,
// a smaller plan prepared later would lower it below a larger plan's launch.
inline cudaError_t res_allow_max_smem(const void* fn) {
  int dev = 0, optin = 0;
  cudaFuncAttributes fa;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, fn);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
  return e;
}
// nf edge fields per direction type (two copies each): 2 for electromag2
// (Ex/Hy rows, Ez/Hy columns), 6 for seismic2.
inline size_t res_scratch_bytes(int P, int NZ, int nf = 2) {
  return sizeof(uint2) * 2 * nf * kResMaxTiles1D * ((size_t)P + (size_t)res_nzp(NZ));
}

// Per-step copies of the state written by a recompute run for the adjoint:
// the state after step t0 + s goes to base + (s + 1) * stride, its Ex, Ez,
// Hy', A (psi dEx_dz, z-strip), B (psi dEz_dx, x-strip), C (psi dHy_dz,
// z-strip) and D (psi dHy_dx, x-strip) at byte offsets off[0..6], in the
// layout of the handle's own arrays.  Hy' is Hy after the step's H half,
// i.e. the stored Hy before its Dirichlet planes are zeroed.  base ==
// nullptr: no copies, and the final state is written back as usual.  With
// copies the run leaves its input state untouched.
struct ResDump {
  char* base;
  size_t stride;
  size_t off[7];
};

struct Em2Resident {
  int NX, NZ, P, W;
  float *Ex, *Ez, *Hy;               // current copy: read before, written after the run
  float *mExz, *mEzx, *mHyz, *mHyx;  // z-, x-, z-, x-strip memory variables of the current copy
  const float *CAx, *CBx, *CAz, *CBz;
  AxisTab X, Z;
  float dbH;
  IoArgs io;
  ResPlan plan;
  ResScratch r;
  int t0, nsteps;
  unsigned long long limit_ns;  // longest wait for a neighbour before the run is abandoned
  unsigned tag_bias;            // added to every awaited edge tag; 0 except in the timeout test aid
  ResDump dump;
  // checkpoints: after every ckpt_every-th step of the run (not its last),
  // the state in the sfd_checkpoint_save layout at ckpt.base + (s / every) * stride
  ResDump ckpt;
  int ckpt_every;
};

// On-chip adjoint sweep over one checkpoint segment: the transposed steps
// t = s0 + nsteps - 1 down to s0, with the adjoint state in registers and
// shared memory for the whole sweep and the same tiling and edge exchange
// as the forward run.  The forward state before step s0 + s is read from
// slots + s * stride (the ResDump layout, slot 0 = the checkpoint).
struct Em2AdjResident {
  int NX, NZ, P, W;
  float *Lx, *Lz, *Lh, *LA, *LB, *LC, *LD;  // adjoint state: read before, written after the sweep
  const float *CAx, *CBx, *CAz, *CBz;       // staggered-averaged update coefficients
  AxisTab X, Z;
  float dbH;
  float *gCAx, *gCBx, *gCAz, *gCBz;  // dJ/d(coefficient) per cell: the sweep adds its sums
  float* srcacc;                     // [2]: sum_t lam_E(source) * amplitude(t)
  const float* srcfn;                // scaled source amplitudes [2][nstep]
  int nstep, si, sk;
  const int* rec;                    // [nrec][3]
  int nrec;
  const float* resid;                // dJ/d(trace) [nstep][2][nrec]
  const char* slots;
  size_t stride;
  size_t off[7];
  int s0, nsteps;
  Ctl* ctl;
  ResPlan plan;
  ResScratch r;
  unsigned long long limit_ns;
};

// On-chip seismic2 run: a uniform ntx x ntz grid of tiles, tile (c, r)
// covering columns [xb[c], xb[c+1]) and rows [zb[r], zb[r+1]).
struct Seis2ResPlan {
  int ntx, ntz;
  int xb[kResMaxTiles1D + 1], zb[kResMaxTiles1D + 1];
  size_t smem;  // dynamic shared memory of the largest tile
};

// A seismic2 run that writes the state after each step s into slot s + 1
// (base + (s + 1) * stride): vx vz sxx szz sxz at off[0..4], the twelve
// memory variables (sfd_num_memory order, on their strips) at off[5..16].
struct S2Dump {
  char* base;
  size_t stride;
  size_t off[17];
};

struct Seis2Resident {
  int NX, NZ, P, W, atten, legacy;
  float *vx, *vz, *sxx, *szz, *sxz;        // current copy: read before, written after the run
  float *m_vxx, *m_vzz, *m_vxz, *m_vzx;    // velocity-gradient memory (x, z, z, x strips), current copy
  float *m2_vxx, *m2_vzz, *m2_vxz, *m2_vzx;  // the sigmaxz loop's own (corrected physics), current copy
  float *m_sxx_x, *m_szz_z, *m_sxz_x, *m_sxz_z;  // stress-gradient memory (x, z, x, z strips)
  const float* coef[12];                   // A11 A13 A15 A33 A35 B15 B35 B55 dtrx dtrz gxp gzp
  const float* q3;
  AxisTab X, Z;
  IoArgs io;
  Seis2ResPlan plan;
  ResScratch r;  // six edge fields
  int t0, nsteps;
  unsigned long long limit_ns;
  unsigned tag_bias;  // added to every awaited edge tag; 0 except in the timeout test aid
  S2Dump dump;        // base != nullptr: dump every step's state, leave the loaded state as it was
};

// Tiling of an NX x NZ seismic2 grid for `max_ctas` CTAs of at most
// `max_smem` bytes; false when the grid does not fit on chip.
bool seis2_resident_plan(int NX, int NZ, int max_ctas, size_t max_smem, Seis2ResPlan* out);
cudaError_t seis2_resident_prepare(const Seis2ResPlan& plan, int* ctas_per_sm);
cudaError_t seis2_resident_launch(const Seis2Resident& a, cudaStream_t s);

// Pick the tiling of an NX x NZ electromag2 grid with npml-cell strips for
// `max_ctas` CTAs of at most `max_smem` bytes of shared memory.  Returns
// false when the grid does not fit on chip.  rows3: tiles of interior cells
// may take kResRows3 rows per thread (the forward kernel's plans; the adjoint
// sweep's tiles all take kResRows).
bool em2_resident_plan(int NX, int NZ, int npml, int max_ctas, size_t max_smem, ResPlan* out, bool rows3);
// Dynamic shared memory of a TW x TZ tile with RB rows per thread.
size_t em2_resident_smem(int TW, int TZ, int RB);
// Set the kernel's shared-memory limit (once per device) and return how many
// CTAs of `smem` bytes fit on one SM.
cudaError_t em2_resident_prepare(const ResPlan& plan, int* ctas_per_sm);
cudaError_t em2_resident_launch(const Em2Resident& a, cudaStream_t s);

// The adjoint sweep's dynamic shared memory for the largest tile of `plan`
// on an NX x NZ grid with W-cell strips; its set-up for `plan` (the kernel's
// shared-memory limit, once per device; how many CTAs fit on one SM, 0 when
// the largest tile does not fit); its launch.
size_t em2_adj_resident_smem(const ResPlan& plan, int NX, int NZ, int W);
cudaError_t em2_adj_resident_prepare(const ResPlan& plan, int NX, int NZ, int W, int* ctas_per_sm);
cudaError_t em2_adj_resident_launch(const Em2AdjResident& a, cudaStream_t s);

}  // namespace sfd
