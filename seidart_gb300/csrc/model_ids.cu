// Update coefficients from a material-id map, on the device (electromag2,
// seismic2, electromag25, seismic25; the 2.5-D models are y-invariant, so
// their id map is the (x, z) image).
//
// A SeidarT model is an image of material ids (one per cell, the PNG colour
// index) and a table of material properties; the driver expands it into one
// FP64 file per property (classes.py:608-750) that the Fortran reads back
// (readwrite_routines.f95:9-37).  Here the id map (caller-owned device
// int32, x fastest) and the table (passed by value) go to one kernel per
// solver kind, which forms each cell's FP32 coefficients in FP64 with the
// formulas of sfd_set_model, operation for operation, so both paths store
// the same coefficients.  Ids outside [0, nmat) raise a flag in the handle's
// control block and leave their cells' coefficients zero; the host rejects
// the call.
#include "../../include/seidart_gb300.h"
#include "sfd_solvers.h"

namespace sfd {

namespace {

constexpr double kEps0d = 8.85418782e-12;

__device__ __forceinline__ bool id_ok(int id, int nmat) { return id >= 0 && id < nmat; }

// electromag2 (electromagfdtd.f95:164-181): per cell ca, cb on the x and z
// staggered points, averaged over the cell and its neighbour below (Ex
// points, k >= 1) or to the left (Ez points, i >= 1), :282, :294.
__device__ __forceinline__ void em2_cacb(const MatTable& m, int id, int d, double dt, double& ca, double& cb) {
  const double* t = m.v + id * 6;  // eps11 eps13 eps33 sig11 sig13 sig33
  const double ep = (d == 0 ? t[0] + t[1] : t[1] + t[2]) * kEps0d;
  const double sg = d == 0 ? t[3] + t[4] : t[4] + t[5];
  ca = (1.0 - sg * dt / (2.0 * ep)) / (1.0 + sg * dt / (2.0 * ep));
  cb = (dt / ep) / (1.0 + sg * dt / (2.0 * ep));
}

__global__ void em2_coef_from_ids(const int* __restrict__ ids, MatTable m, int NX, int NZ, int P, double dt,
                                  float* CAx, float* CBx, float* CAz, float* CBz, int* bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= NX || k >= NZ) return;
  const size_t n = (size_t)k * NX + i, c = (size_t)k * P + i;
  const int id = ids[n];
  float ax = 0.f, bx = 0.f, az = 0.f, bz = 0.f;
  if (!id_ok(id, m.nmat)) {
    atomicExch(bad, 1);
  } else {
    double ca, cb;
    if (k >= 1) {
      const int up = ids[n - NX];
      if (id_ok(up, m.nmat)) {
        double ca2, cb2;
        em2_cacb(m, id, 0, dt, ca, cb);
        em2_cacb(m, up, 0, dt, ca2, cb2);
        ax = (float)((ca + ca2) / 2);
        bx = (float)((cb + cb2) / 2);
      }
    }
    if (i >= 1) {
      const int lf = ids[n - 1];
      if (id_ok(lf, m.nmat)) {
        double ca2, cb2;
        em2_cacb(m, id, 1, dt, ca, cb);
        em2_cacb(m, lf, 1, dt, ca2, cb2);
        az = (float)((ca + ca2) / 2);
        bz = (float)((cb + cb2) / 2);
      }
    }
  }
  CAx[c] = ax;
  CBx[c] = bx;
  CAz[c] = az;
  CBz[c] = bz;
}

// seismic2 (seismicfdtd.f95:247-357): planes c11 c13 c15 c33 c35 c55 rho
// gamma_x gamma_z.  Stress-loop averages (c(i+1,k) + 2 c(i,k) + c(i,k-1))/4
// and (c(i,k+1) + 2 c(i,k) + c(i-1,k))/4 times dt, dt/rho, the averaged
// dt/rho of the vz points (:341, :355) and 1 - gamma.
__global__ void seis2_coef_from_ids(const int* __restrict__ ids, MatTable m, int NX, int NZ, int P, double dt,
                                    float* coef, size_t plane, int* bad, int dens, int legacy) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= NX || k >= NZ) return;
  const size_t n = (size_t)k * NX + i, c = (size_t)k * P + i;
  const int id = ids[n];
  float out[12];
#pragma unroll
  for (int q = 0; q < 12; ++q) out[q] = 0.f;
  auto val = [&](int cell_id, int q) { return m.v[cell_id * 9 + q]; };
  auto okat = [&](int ii, int kk) { return id_ok(ids[(size_t)kk * NX + ii], m.nmat); };
  if (!id_ok(id, m.nmat)) {
    atomicExch(bad, 1);
  } else {
    const int A_src[5] = {0, 1, 2, 3, 4}, B_src[3] = {2, 4, 5};
    if (i <= NX - 2 && k >= 1 && okat(i + 1, k) && okat(i, k - 1)) {
      const int r = ids[n + 1], u = ids[n - NX];
#pragma unroll
      for (int q = 0; q < 5; ++q)
        out[q] = (float)((val(r, A_src[q]) + 2 * val(id, A_src[q]) + val(u, A_src[q])) / 4 * dt);
    }
    if (k <= NZ - 2 && i >= 1 && okat(i, k + 1) && okat(i - 1, k)) {
      const int d = ids[n + NX], l = ids[n - 1];
#pragma unroll
      for (int q = 0; q < 3; ++q)
        out[5 + q] = (float)((val(d, B_src[q]) + 2 * val(id, B_src[q]) + val(l, B_src[q])) / 4 * dt);
    }
    const double rho = val(id, 6);
    // vx: the cell's own rho with the legacy quirks (:334), else the average of :320
    if (legacy || i < 1 || k < 1 || !okat(i - 1, k) || !okat(i, k - 1))
      out[8] = (float)(dt / rho);
    else
      out[8] = (float)(dt / rho_avg(dens, 2, rho, val(ids[n - 1], 6), val(ids[n - NX], 6)));
    if (i <= NX - 2 && k <= NZ - 2 && okat(i + 1, k) && okat(i, k + 1))  // :342, :355
      out[9] = (float)(dt / rho_avg(dens, 2, rho, val(ids[n + 1], 6), val(ids[n + NX], 6)));
    out[10] = (float)(1.0 - val(id, 7));
    out[11] = (float)(1.0 - val(id, 8));
  }
#pragma unroll
  for (int q = 0; q < 12; ++q) coef[q * plane + c] = out[q];
}

// electromag25 (electromagfdtd.f95:756-789): ca, cb of Ex, Ey, Ez per (x, z)
// column from the row sums of the permittivity and conductivity tensors.
__global__ void em25_coef_from_ids(const int* __restrict__ ids, MatTable m, int NX, int NZ, int P, double dt,
                                   float* coef, size_t plane, int* bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= NX || k >= NZ) return;
  const size_t n = (size_t)k * NX + i, c = (size_t)k * P + i;
  const int id = ids[n];
  float out[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (!id_ok(id, m.nmat)) {
    atomicExch(bad, 1);
  } else {
    const double* t = m.v + id * 12;  // eps11 eps12 eps13 eps22 eps23 eps33, sig11 .. sig33
    const double ep[3] = {(t[0] + t[1] + t[2]) * kEps0d, (t[1] + t[3] + t[4]) * kEps0d, (t[2] + t[4] + t[5]) * kEps0d};
    const double sg[3] = {t[6] + t[7] + t[8], t[7] + t[9] + t[10], t[8] + t[10] + t[11]};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      out[2 * d] = (float)((1.0 - sg[d] * dt / (2.0 * ep[d])) / (1.0 + sg[d] * dt / (2.0 * ep[d])));
      out[2 * d + 1] = (float)((dt / ep[d]) / (1.0 + sg[d] * dt / (2.0 * ep[d])));
    }
  }
#pragma unroll
  for (int q = 0; q < 6; ++q) coef[q * plane + c] = out[q];
}

// seismic25 (seismicfdtd.f95:616-877): the 33 y-invariant stiffness averages
// of the four stress loops (loop, Voigt entry, factor; the table of
// sfd_set_model), the three averaged dt/rho of the velocity loops and
// 1 - gamma per axis.
struct S25Avg {
  int loop, cij;
  double f;
};
__constant__ S25Avg kS25Avg[33] = {
    {1, 0, 0.25}, {1, 1, 0.25}, {1, 2, 0.25}, {1, 3, 0.125}, {1, 4, 0.125}, {1, 5, 0.125},
    {1, 6, 0.25}, {1, 7, 0.25}, {1, 8, 0.125}, {1, 9, 0.125}, {1, 10, 0.125},
    {1, 11, 0.25}, {1, 12, 0.125}, {1, 13, 0.125}, {1, 14, 0.125},
    {2, 5, 0.25}, {2, 10, 0.25}, {2, 14, 0.25}, {2, 17, 0.125}, {2, 19, 0.125}, {2, 20, 0.125},
    {3, 4, 0.25}, {3, 9, 0.25}, {3, 13, 0.25}, {3, 16, 0.125}, {3, 18, 0.125}, {3, 19, 0.125},
    {4, 3, 0.25}, {4, 8, 0.25}, {4, 12, 0.25}, {4, 15, 0.125}, {4, 16, 0.125}, {4, 17, 0.125}};

__global__ void seis25_coef_from_ids(const int* __restrict__ ids, MatTable m, int NX, int NZ, int P, double dt,
                                     float* coef, size_t plane, int* bad, int dens) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= NX || k >= NZ) return;
  const size_t n = (size_t)k * NX + i, c = (size_t)k * P + i;
  const int id = ids[n];
  // the material of cell (ii, kk), or -1 (out of the grid or a bad id)
  auto mat = [&](int ii, int kk) {
    if (ii < 0 || ii >= NX || kk < 0 || kk >= NZ) return -1;
    const int v = ids[(size_t)kk * NX + ii];
    return id_ok(v, m.nmat) ? v : -1;
  };
  auto val = [&](int cell_id, int q) { return m.v[cell_id * 25 + q]; };
  if (!id_ok(id, m.nmat)) {
    atomicExch(bad, 1);
    for (int q = 0; q < 39; ++q) coef[q * plane + c] = 0.f;
    return;
  }
  const int mr = mat(i + 1, k), ml = mat(i - 1, k), mu = mat(i, k - 1), md = mat(i, k + 1);
  const int mru = mat(i + 1, k - 1), mlu = mat(i - 1, k - 1), mld = mat(i - 1, k + 1), mrd = mat(i + 1, k + 1);
  for (int q = 0; q < 33; ++q) {
    const S25Avg av = kS25Avg[q];
    double v = 0.0;
    switch (av.loop) {
      case 1:  // (i+1,k) (i,k) (i,k-1) (i+1,k-1), k >= 1, i <= NX-2
        if (k >= 1 && i <= NX - 2 && mr >= 0 && mu >= 0 && mru >= 0)
          v = val(mr, av.cij) + val(id, av.cij) + val(mu, av.cij) + val(mru, av.cij);
        break;
      case 2:  // (i,k) (i-1,k) (i,k-1) (i-1,k-1), k >= 1, i >= 1
        if (k >= 1 && i >= 1 && ml >= 0 && mu >= 0 && mlu >= 0)
          v = val(id, av.cij) + val(ml, av.cij) + val(mu, av.cij) + val(mlu, av.cij);
        break;
      case 3:  // (i,k+1) (i,k) (i-1,k) (i-1,k+1), k <= NZ-2, i >= 1
        if (k <= NZ - 2 && i >= 1 && md >= 0 && ml >= 0 && mld >= 0)
          v = val(md, av.cij) + val(id, av.cij) + val(ml, av.cij) + val(mld, av.cij);
        break;
      default:  // (i+1,k) (i,k) (i,k+1) (i+1,k+1), k <= NZ-2, i <= NX-2
        if (k <= NZ - 2 && i <= NX - 2 && mr >= 0 && md >= 0 && mrd >= 0)
          v = val(mr, av.cij) + val(id, av.cij) + val(md, av.cij) + val(mrd, av.cij);
        break;
    }
    coef[q * plane + c] = (float)(av.f * v * dt);
  }
  const double r = val(id, 21);
  float o33 = 0.f, o34 = 0.f, o35 = 0.f;
  if (i >= 1 && k >= 1 && ml >= 0 && mu >= 0)  // seismicfdtd.f95:825
    o33 = (float)(dt / rho_avg(dens, 4, r, val(ml, 21), val(mu, 21)));
  if (i <= NX - 2 && k >= 1 && mr >= 0 && mu >= 0)  // :850
    o34 = (float)(dt / rho_avg(dens, 4, r, val(mr, 21), val(mu, 21)));
  if (i <= NX - 2 && k <= NZ - 2 && mr >= 0 && md >= 0)  // :876
    o35 = (float)(dt / rho_avg(dens, 4, r, val(mr, 21), val(md, 21)));
  coef[33 * plane + c] = o33;
  coef[34 * plane + c] = o34;
  coef[35 * plane + c] = o35;
  for (int d = 0; d < 3; ++d) coef[(36 + d) * plane + c] = (float)(1.0 - val(id, 22 + d));
}

}  // namespace

void coef_from_ids(int kind, const int* ids, const MatTable& m, int NX, int NZ, int P, double dt, float* coef,
                   size_t plane, int* bad, int flags, cudaStream_t s) {
  const int dens = (flags & SFD_FLAG_DENSITY_MASK) / SFD_FLAG_DENSITY_NONE;
  const int legacy = (flags & SFD_FLAG_LEGACY_QUIRKS) ? 1 : 0;
  const dim3 b(32, 8), g((NX + 31) / 32, (NZ + 7) / 8);
  switch (kind) {
    case SFD_ELECTROMAG2:
      em2_coef_from_ids<<<g, b, 0, s>>>(ids, m, NX, NZ, P, dt, coef, coef + plane, coef + 2 * plane, coef + 3 * plane,
                                        bad);
      break;
    case SFD_SEISMIC2:
      seis2_coef_from_ids<<<g, b, 0, s>>>(ids, m, NX, NZ, P, dt, coef, plane, bad, dens, legacy);
      break;
    case SFD_ELECTROMAG25: em25_coef_from_ids<<<g, b, 0, s>>>(ids, m, NX, NZ, P, dt, coef, plane, bad); break;
    default: seis25_coef_from_ids<<<g, b, 0, s>>>(ids, m, NX, NZ, P, dt, coef, plane, bad, dens); break;
  }
}

}  // namespace sfd
