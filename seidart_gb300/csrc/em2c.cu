// electromag2c (legacy/fortran/electromagfdtd.f95:329-616): the 2-D TE Yee
// scheme of electromag2 with complex permittivities, hence complex update
// coefficients, fields and CPML memory variables.  Complex arrays are held
// as separate real and imaginary planes (x fastest, pitch P), so each plane
// streams like a real field.  Two kernels per step, as the two-pass
// electromag2 (em2.cu):
//   half1: Hy (:530-549) with the dEx/dz, dEz/dx memory variables; block
//          (0,0) first records the receivers of the previous step;
//   half2: Ex (:556-565), Ez (:567-576) with the dHy memory variables, the
//          source (:581-582), the Dirichlet edges (:585-598) and the norm
//          |sqrt(Ex^2 + Ez^2)| of :601 (complex squares).
// The real axis tables multiply complex values component by component; the
// averaged coefficients multiply as complex numbers.
#include "sfd_solvers.h"

namespace sfd {

namespace {

constexpr int BX = 32, BY = 8;

struct cf {
  float r, i;
};
__device__ __forceinline__ cf cmul(cf a, cf b) { return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r}; }
__device__ __forceinline__ cf cadd(cf a, cf b) { return {a.r + b.r, a.i + b.i}; }
__device__ __forceinline__ cf cscale(float s, cf a) { return {s * a.r, s * a.i}; }

// Stability monitor of one cell: |Exr| + |Exi| + |Ezr| + |Ezi| bounds
// sqrt|Ex^2 + Ez^2| from above; above 1e24 the exact value is returned
// (components scaled by their largest magnitude so the squares cannot
// overflow), so the 1e25 threshold is tested exactly.  NaN -> +inf.
__device__ __forceinline__ float norm_monitor_c(cf ex, cf ez) {
  const float m = fabsf(ex.r) + fabsf(ex.i) + fabsf(ez.r) + fabsf(ez.i);
  if (m <= 1e24f) return m;
  const float s = fmaxf(fmaxf(fabsf(ex.r), fabsf(ex.i)), fmaxf(fabsf(ez.r), fabsf(ez.i)));
  if (!(s < __int_as_float(0x7f800000))) return __int_as_float(0x7f800000);  // inf or NaN
  const cf a = {ex.r / s, ex.i / s}, b = {ez.r / s, ez.i / s};
  const cf w = cadd(cmul(a, a), cmul(b, b));
  return nan_to_inf(s * sqrtf(hypotf(w.r, w.i)));
}

__global__ void __launch_bounds__(BX * BY) em2c_h_kernel(Em2cArgs a, int rel) {
  const Ctl* ctl = a.io.ctl;
  const int t = ctl->base + rel;
  if (blockIdx.x == 0 && blockIdx.y == 0 && t > ctl->run_start) {
    const float* ch[4] = {a.Ex[0], a.Ex[1], a.Ez[0], a.Ez[1]};
    gather_receivers<4>(a.io.rec, a.io.nrec, a.io.traces, t - 1, ch, a.P, 1, false);
  }
  const int i = blockIdx.x * BX + threadIdx.x;
  const int k = blockIdx.y * BY + threadIdx.y;
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  if (i > NX - 2 || k > NZ - 2) return;
  const size_t c = (size_t)k * P + i;
  // dEx/dz, :533-535
  const cf dEx = {a.Ex[0][c + P] - a.Ex[0][c], a.Ex[1][c + P] - a.Ex[1][c]};
  cf vz = cscale(a.Z.ik[k], dEx);
  if (in_strip(k, NZ, W)) {
    const size_t m = (size_t)strip_idx(k, NZ, W) * P + i;
    const cf psi = cadd(cscale(a.Z.b[k], {a.mExz[0][m], a.mExz[1][m]}), cscale(a.Z.ad[k], dEx));
    a.mExz[0][m] = psi.r;
    a.mExz[1][m] = psi.i;
    vz = cadd(vz, psi);
  }
  // dEz/dx, :538-540
  const cf dEz = {a.Ez[0][c + 1] - a.Ez[0][c], a.Ez[1][c + 1] - a.Ez[1][c]};
  cf vx = cscale(a.X.ik[i], dEz);
  if (in_strip(i, NX, W)) {
    const size_t m = (size_t)k * (2 * W) + strip_idx(i, NX, W);
    const cf psi = cadd(cscale(a.X.b[i], {a.mEzx[0][m], a.mEzx[1][m]}), cscale(a.X.ad[i], dEz));
    a.mEzx[0][m] = psi.r;
    a.mEzx[1][m] = psi.i;
    vx = cadd(vx, psi);
  }
  // the previous Hy on its Dirichlet edges is zero (they are zeroed after the E half, :595-598)
  const bool edge = (i == 0) | (i == NX - 2) | (k == 0) | (k == NZ - 2);
  const cf hy = edge ? cf{0.0f, 0.0f} : cf{a.Hy[0][c], a.Hy[1][c]};
  const cf h = cadd(hy, cscale(a.dbH, cadd(vx, vz)));  // :543
  a.Hy[0][c] = h.r;
  a.Hy[1][c] = h.i;
}

__global__ void __launch_bounds__(BX * BY) em2c_e_kernel(Em2cArgs a, int rel) {
  const int t = a.io.ctl->base + rel;
  const int i = blockIdx.x * BX + threadIdx.x;
  const int k = blockIdx.y * BY + threadIdx.y;
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  float norm = 0.0f;
  if (i < NX && k < NZ) {
    const size_t c = (size_t)k * P + i;
    cf ex = {0.0f, 0.0f}, ez = {0.0f, 0.0f};
    // Ex, :556-565 (k in [1, NZ-2], i in [0, NX-2])
    if (i <= NX - 2) {
      ex = {a.Ex[0][c], a.Ex[1][c]};
      if (k >= 1 && k <= NZ - 2) {
        const cf dH = {a.Hy[0][c] - a.Hy[0][c - P], a.Hy[1][c] - a.Hy[1][c - P]};
        cf d = cscale(a.Z.ikh[k], dH);
        if (in_strip(k, NZ, W)) {
          const size_t m = (size_t)strip_idx(k, NZ, W) * P + i;
          const cf psi = cadd(cscale(a.Z.bh[k], {a.mHyz[0][m], a.mHyz[1][m]}), cscale(a.Z.adh[k], dH));
          a.mHyz[0][m] = psi.r;
          a.mHyz[1][m] = psi.i;
          d = cadd(d, psi);
        }
        ex = cadd(cmul({a.CAx[0][c], a.CAx[1][c]}, ex), cmul({a.CBx[0][c], a.CBx[1][c]}, d));
      }
    }
    // Ez, :567-576 (k in [0, NZ-2], i in [1, NX-2])
    if (k <= NZ - 2) {
      ez = {a.Ez[0][c], a.Ez[1][c]};
      if (i >= 1 && i <= NX - 2) {
        const cf dH = {a.Hy[0][c] - a.Hy[0][c - 1], a.Hy[1][c] - a.Hy[1][c - 1]};
        cf d = cscale(a.X.ikh[i], dH);
        if (in_strip(i, NX, W)) {
          const size_t m = (size_t)k * (2 * W) + strip_idx(i, NX, W);
          const cf psi = cadd(cscale(a.X.bh[i], {a.mHyx[0][m], a.mHyx[1][m]}), cscale(a.X.adh[i], dH));
          a.mHyx[0][m] = psi.r;
          a.mHyx[1][m] = psi.i;
          d = cadd(d, psi);
        }
        ez = cadd(cmul({a.CAz[0][c], a.CAz[1][c]}, ez), cmul({a.CBz[0][c], a.CBz[1][c]}, d));
      }
    }
    // Source, :581-582 (amplitudes already divided by the complex permittivity)
    if (i == a.io.si && k == a.io.sk) {
      const int n = a.io.nstep;
      ex = cadd(ex, {a.io.src[t], a.io.src[n + t]});
      ez = cadd(ez, {a.io.src[2 * n + t], a.io.src[3 * n + t]});
    }
    // Dirichlet edges, :585-594
    if (i == 0 || i == NX - 2 || k == 0 || k == NZ - 1) ex = {0.0f, 0.0f};
    if (i == 0 || i == NX - 1 || k == 0 || k == NZ - 2) ez = {0.0f, 0.0f};
    if (i <= NX - 2) {
      a.Ex[0][c] = ex.r;
      a.Ex[1][c] = ex.i;
    }
    if (k <= NZ - 2) {
      a.Ez[0][c] = ez.r;
      a.Ez[1][c] = ez.i;
    }
    norm = norm_monitor_c(ex, ez);
  }
  block_norm_to_slot(norm, a.io.slots, blockIdx.y * gridDim.x + blockIdx.x);
}

// Last receivers of the run, Hy edges to zero.
__global__ void em2c_finalize_kernel(Em2cArgs a, int t_last) {
  const float* ch[4] = {a.Ex[0], a.Ex[1], a.Ez[0], a.Ez[1]};
  gather_receivers<4>(a.io.rec, a.io.nrec, a.io.traces, t_last, ch, a.P, 1, false);
  const int NX = a.NX, NZ = a.NZ, P = a.P;
  for (int q = 0; q < 2; ++q) {
    for (int k = threadIdx.x; k < NZ; k += blockDim.x) {
      a.Hy[q][(size_t)k * P + 0] = 0.0f;
      a.Hy[q][(size_t)k * P + NX - 2] = 0.0f;
    }
    for (int i = threadIdx.x; i < NX; i += blockDim.x) {
      a.Hy[q][i] = 0.0f;
      a.Hy[q][(size_t)(NZ - 2) * P + i] = 0.0f;
    }
  }
}

}  // namespace

Launch em2c_launch(const Em2cArgs& a) {
  Launch L;
  L.block = dim3(BX, BY, 1);
  L.grid = dim3((a.NX + BX - 1) / BX, (a.NZ + BY - 1) / BY, 1);
  L.nslots = L.grid.x * L.grid.y;
  return L;
}

void em2c_half1(const Em2cArgs& a, const Launch& L, int rel, cudaStream_t s) {
  em2c_h_kernel<<<L.grid, L.block, 0, s>>>(a, rel);
}

void em2c_half2(const Em2cArgs& a, const Launch& L, int rel, cudaStream_t s) {
  em2c_e_kernel<<<L.grid, L.block, 0, s>>>(a, rel);
}

void em2c_finalize(const Em2cArgs& a, int t_last, cudaStream_t s) { em2c_finalize_kernel<<<1, 256, 0, s>>>(a, t_last); }

}  // namespace sfd
