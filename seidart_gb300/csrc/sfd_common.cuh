// Shared device-side definitions of the seidart_gb300 FDTD kernels.
//
// Layout in HBM (one handle):
//   fields      FP32, x fastest, row pitch P (NX rounded up to 32 floats):
//               2-D  f[k*P + i], 2.5-D f[(k*NY + j)*P + i]
//   memory (psi) CPML memory variables stored on their strip only:
//               x-strip  [rows][2W]   (rows = NZ or NZ*NY), index xs(i)
//               y-strip  [NZ][2W][P]  index ys(j)                  (2.5-D)
//               z-strip  [2W][rows'][P] (rows' = 1 or NY), index zs(k)
//               where W = npml and the strip of an axis of n cells is
//               [0, W) U [n-W, n).  A memory variable psi <- b psi + a d stays
//               zero wherever a = 0, so storing it off the strip is not needed.
//   coefficients per cell (2-D) or per (x, z) column (2.5-D), pitch P.
//   axis tables  per axis 6 x n floats: 1/(delta K), a/delta, b, and the same
//               for the half-node offset.
#pragma once
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

namespace sfd {

// Device control block of a handle.
struct Ctl {
  int base;       // global index of the step the next launch with rel = 0 computes
  int run_start;  // first step of the current sfd_run
  int err;       // a bounded device wait of the last run gave up
  int pad1;
  float maxnorm;  // largest field norm of the last run (after finalize)
  int nan_seen;
  int pad2, pad3;
};

// Per-axis coefficient table (device pointers into one 6*n array).
struct AxisTab {
  const float* ik;   // 1 / (delta * K)
  const float* ad;   // a / delta
  const float* b;    // b
  const float* ikh;  // half-node versions
  const float* adh;
  const float* bh;
};

// Each table row is padded to a multiple of 32 floats so 16-byte vector
// loads of four consecutive entries stay aligned.
__host__ __device__ inline int axis_stride(int n) { return (n + 31) & ~31; }

__host__ __device__ inline AxisTab make_axis(const float* base, int n) {
  const int s = axis_stride(n);
  AxisTab t;
  t.ik = base;
  t.ad = base + s;
  t.b = base + 2 * s;
  t.ikh = base + 3 * s;
  t.adh = base + 4 * s;
  t.bh = base + 5 * s;
  return t;
}

__device__ __forceinline__ bool in_strip(int i, int n, int W) { return i < W || i >= n - W; }
__device__ __forceinline__ int strip_idx(int i, int n, int W) { return i < W ? i : i - (n - 2 * W); }

__device__ __forceinline__ float nan_to_inf(float v) { return (v != v) ? __int_as_float(0x7f800000) : v; }

// Stability monitor value of one cell: |a| + |b| (+ |c|), which bounds the
// 2-norm the Fortran tests (seismicfdtd.f95:378) from above within a factor
// sqrt(2) (sqrt(3)); above 1e24 the exact 2-norm is returned, so the 1e25
// threshold is tested exactly.  NaN propagates through the sum and comes back
// as +inf.
// Density at a staggered velocity point, from the cell's own value r and the
// two neighbours a, b of the Fortran's averaging stencil, weights (w, 1, 1):
// w = 2 in seismic2 (legacy/fortran/seismicfdtd.f95:320, 342), w = 4 in
// seismic25 (:825, 850, 876).  method (sfd_config flags / SFD_FLAG_DENSITY_NONE):
// 0 arithmetic (the Fortran's average), 1 none (r itself), 2 geometric,
// 3 harmonic -- the density_method values the driver passes
// (src/seidart/routines/classes.py:311, 910-924).  The host (sfd_set_model)
// and the device (sfd_set_model_ids) evaluate the same FP64 expression.
__host__ __device__ inline double rho_avg(int method, int w, double r, double a, double b) {
  switch (method) {
    case 1: return r;
    case 2: return w == 2 ? sqrt(sqrt(r * r * a * b)) : cbrt(sqrt(r * r * r * r * a * b));
    case 3: return (w + 2.0) / (w / r + 1.0 / a + 1.0 / b);
  }
  return (w * r + a + b) / (w + 2.0);
}

__device__ __forceinline__ float norm_monitor(float a, float b) {
  const float m = fabsf(a) + fabsf(b);
  return (m <= 1e24f) ? m : nan_to_inf(hypotf(a, b));
}
__device__ __forceinline__ float norm_monitor(float a, float b, float c) {
  const float m = fabsf(a) + fabsf(b) + fabsf(c);
  return (m <= 1e24f) ? m : nan_to_inf(norm3df(a, b, c));
}

// Block-wide max of v (every thread of the block must call it); thread 0 then
// folds it into this block's slot.  No atomics: each block owns its slot.
__device__ __forceinline__ void block_norm_to_slot(float v, float* slots, int slot) {
  __shared__ float wmax[32];
  v = nan_to_inf(v);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nthreads = blockDim.x * blockDim.y * blockDim.z;
  const int warp = tid >> 5, lane = tid & 31;
  if (lane == 0) wmax[warp] = v;
  __syncthreads();
  if (warp == 0) {
    const int nw = (nthreads + 31) >> 5;
    float w = lane < nw ? wmax[lane] : 0.0f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) w = fmaxf(w, __shfl_xor_sync(0xffffffffu, w, o));
    if (lane == 0) slots[slot] = fmaxf(slots[slot], w);
  }
}

// Copy the receiver samples of step t into traces[t][ch][r] (one block).
template <int NCH>
__device__ __forceinline__ void gather_receivers(const int* __restrict__ rec, int nrec, float* __restrict__ traces,
                                                 int t, const float* const* ch, int P, int NY, bool three) {
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nthreads = blockDim.x * blockDim.y * blockDim.z;
  for (int r = tid; r < nrec; r += nthreads) {
    const int i = rec[3 * r], j = rec[3 * r + 1], k = rec[3 * r + 2];
    const size_t c = three ? ((size_t)k * NY + j) * P + i : (size_t)k * P + i;
#pragma unroll
    for (int q = 0; q < NCH; ++q) traces[((size_t)t * NCH + q) * nrec + r] = ch[q][c];
  }
}

__global__ void k_begin(Ctl* ctl, float* slots, int nslots, int step);
__global__ void k_advance(Ctl* ctl, int by);
__global__ void k_reduce_slots(Ctl* ctl, const float* slots, int nslots);

}  // namespace sfd
