// FP64 CPU oracle for the SeidarT FDTD time-stepping path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, loop for loop, the legacy
// Fortran solvers of the reference (legacy/fortran/seismicfdtd.f95 and
// legacy/fortran/electromagfdtd.f95) in double precision so that the CUDA
// kernels of seidart_gb300 can be checked against it and so that bench.py can
// time a CPU baseline.  Nothing in the product path links or calls it.
//
// Parity status: UNPINNED.  The reference ships no tests, golden vectors or
// fixtures for these solvers, its production backend is a prebuilt binary
// whose source is not in the tree, and its Fortran sources cannot be compiled
// (no Fortran compiler on either machine).  The restatement is cross-checked
// against an independent numpy restatement (oracle/numpy_ref.py) and against
// physical known-answer tests in tests/.
//
// Conventions (shared with the CUDA library):
//   * every field and memory variable is stored full-grid, x fastest:
//       2-D  idx = i + NX*k            (k is the z index)
//       2.5-D idx = i + NX*(j + NY*k)  (j is the y index)
//     Fortran index (i,k) of the reference is (i-1, k-1) here.
//   * material arrays are (NX, NZ), x fastest (y-invariant in 2.5-D).
//   * CPML profiles are per axis: K, a, b, K_half, a_half, b_half, each of
//     the axis length, packed x then y then z (y absent in 2-D).
//   * source time functions are packed component-major (x, [y,] z), each of
//     length nstep_src; the value used at global step t is src[t].
//   * receivers are (i, j, k) triples, 0-based full-grid (j = 0 in 2-D);
//     traces are [step][channel][receiver].
//
// Every loop below cites the Fortran lines it restates.

#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>

namespace {

constexpr double kPI = 3.141592653589793238462643;
constexpr double kMu0 = 4.0 * kPI * 1.0e-7;       // electromagfdtd.f95:86
constexpr double kEps0 = 8.85418782e-12;          // electromagfdtd.f95:86
constexpr double kStability = 1.0e25;             // seismicfdtd.f95:88

struct Axis {
  const double *K, *a, *b, *Kh, *ah, *bh;
  int n;
};

static void unpack_axes(const double* prof, int nx, int ny, int nz, bool three, Axis* x, Axis* y, Axis* z) {
  const double* p = prof;
  auto take = [&](Axis* ax, int n) {
    ax->n = n;
    ax->K = p; p += n;
    ax->a = p; p += n;
    ax->b = p; p += n;
    ax->Kh = p; p += n;
    ax->ah = p; p += n;
    ax->bh = p; p += n;
  };
  take(x, nx);
  if (three) take(y, ny);
  take(z, nz);
}

// Density at a staggered velocity point, from the cell's own value r and the
// two neighbours a, b of the Fortran's deltarho stencil, weights (w, 1, 1):
// w = 2 in seismic2 (seismicfdtd.f95:342), w = 4 in seismic25 (:825, :850,
// :876).  method: 0 arithmetic (the Fortran's average), 1 none (r itself),
// 2 geometric, 3 harmonic (the density_method values the driver passes,
// src/seidart/routines/classes.py:311, 910-924).
static double rho_avg(int method, double w, double r, double a, double b) {
  switch (method) {
    case 1: return r;
    case 2: return w == 2.0 ? std::sqrt(std::sqrt(r * r * a * b)) : std::cbrt(std::sqrt(r * r * r * r * a * b));
    case 3: return (w + 2.0) / (w / r + 1.0 / a + 1.0 / b);
  }
  return (w * r + a + b) / (w + 2.0);
}

}  // namespace

template <bool TWO_D>
static int electromag2_impl(int NX, int NZ, double dx, double dz, double dt,
                    const double* prof, const double* mat,
                    int isrc, int ksrc, const double* src, int nstep_src,
                    int it0, int nsteps,
                    double* fld, double* mem,
                    int nrec, const int* rec, double* traces,
                    double* maxnorm, int* blew_up, const double* cpml2d) {
  const size_t N = (size_t)NX * NZ;

  // CPML coefficient q (K a b K_half a_half b_half) of the x (z) axis at cell
  // (i, k): the axis profile at i (k), or, with the driver's 2-D fields
  // (TWO_D), the field's value at the cell -- the same field for every
  // derivative direction
  auto XP = [&](const double* ax, int q, int i, int k) -> double {
    if constexpr (TWO_D) return cpml2d[(size_t)q * N + (size_t)i + (size_t)NX * k];
    else return ax[i];
  };
  auto ZP = [&](const double* ax, int q, int i, int k) -> double {
    if constexpr (TWO_D) return cpml2d[(size_t)q * N + (size_t)i + (size_t)NX * k];
    else return ax[k];
  };
  Axis X, Y, Z;
  unpack_axes(prof, NX, 1, NZ, false, &X, &Y, &Z);
  const double *eps11 = mat, *eps13 = mat + N, *eps33 = mat + 2 * N;
  const double *sig11 = mat + 3 * N, *sig13 = mat + 4 * N, *sig33 = mat + 5 * N;
  double *Ex = fld, *Ez = fld + N, *Hy = fld + 2 * N;
  double *mExz = mem, *mEzx = mem + N, *mHyz = mem + 2 * N, *mHyx = mem + 3 * N;
  auto I = [NX](int i, int k) { return (size_t)i + (size_t)NX * k; };

  // Coefficients, electromagfdtd.f95:164-181.
  std::vector<double> caEx(N), cbEx(N), caEz(N), cbEz(N);
  for (size_t c = 0; c < N; ++c) {
    const double ex = (eps11[c] + eps13[c]) * kEps0, ez = (eps13[c] + eps33[c]) * kEps0;
    const double sx = sig11[c] + sig13[c], sz = sig13[c] + sig33[c];
    caEx[c] = (1.0 - sx * dt / (2.0 * ex)) / (1.0 + sx * dt / (2.0 * ex));
    cbEx[c] = (dt / ex) / (1.0 + sx * dt / (2.0 * ex));
    caEz[c] = (1.0 - sz * dt / (2.0 * ez)) / (1.0 + sz * dt / (2.0 * ez));
    cbEz[c] = (dt / ez) / (1.0 + sz * dt / (2.0 * ez));
  }
  const double daHy = 1.0, dbHy = dt / kMu0;  // :177-179
  const double* srcx = src;
  const double* srcz = src + nstep_src;
  *blew_up = 0;
  double runmax = 0.0;

  for (int s = 0; s < nsteps; ++s) {
    const int t = it0 + s;
    // Hy and its memory variables, :249-266.
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= NZ - 2; ++k)
      for (int i = 0; i <= NX - 2; ++i) {
        const size_t c = I(i, k);
        double dEx_dz = (Ex[I(i, k + 1)] - Ex[c]) / dz;
        mExz[c] = ZP(Z.b, 2, i, k) * mExz[c] + ZP(Z.a, 1, i, k) * dEx_dz;
        dEx_dz = dEx_dz / ZP(Z.K, 0, i, k) + mExz[c];
        double dEz_dx = (Ez[I(i + 1, k)] - Ez[c]) / dx;
        mEzx[c] = XP(X.b, 2, i, k) * mEzx[c] + XP(X.a, 1, i, k) * dEz_dx;
        dEz_dx = dEz_dx / XP(X.K, 0, i, k) + mEzx[c];
        Hy[c] = daHy * Hy[c] + dbHy * (dEz_dx + dEx_dz);
      }
    // Ex, :273-283.
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= NZ - 2; ++k)
      for (int i = 0; i <= NX - 2; ++i) {
        const size_t c = I(i, k), cm = I(i, k - 1);
        double d = (Hy[c] - Hy[cm]) / dz;
        mHyz[c] = ZP(Z.bh, 5, i, k) * mHyz[c] + ZP(Z.ah, 4, i, k) * d;
        d = d / ZP(Z.Kh, 3, i, k) + mHyz[c];
        Ex[c] = ((caEx[c] + caEx[cm]) / 2) * Ex[c] + ((cbEx[c] + cbEx[cm]) / 2) * d;
      }
    // Ez, :285-295.
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= NZ - 2; ++k)
      for (int i = 1; i <= NX - 2; ++i) {
        const size_t c = I(i, k), cm = I(i - 1, k);
        double d = (Hy[c] - Hy[cm]) / dx;
        mHyx[c] = XP(X.bh, 5, i, k) * mHyx[c] + XP(X.ah, 4, i, k) * d;
        d = d / XP(X.Kh, 3, i, k) + mHyx[c];
        Ez[c] = ((caEz[c] + caEz[cm]) / 2) * Ez[c] + ((cbEz[c] + cbEz[cm]) / 2) * d;
      }
    // Source, :300-301 (divided by the relative permittivity, as written).
    {
      const size_t c = I(isrc, ksrc);
      Ex[c] = Ex[c] + srcx[t] * dt / eps11[c];
      Ez[c] = Ez[c] + srcz[t] * dt / eps33[c];
    }
    // Dirichlet edges, :304-317.
    for (int k = 0; k < NZ; ++k) {
      Ex[I(0, k)] = 0; Ex[I(NX - 2, k)] = 0;
      Ez[I(0, k)] = 0; Ez[I(NX - 1, k)] = 0;
      Hy[I(0, k)] = 0; Hy[I(NX - 2, k)] = 0;
    }
    for (int i = 0; i < NX; ++i) {
      Ex[I(i, 0)] = 0; Ex[I(i, NZ - 1)] = 0;
      Ez[I(i, 0)] = 0; Ez[I(i, NZ - 2)] = 0;
      Hy[I(i, 0)] = 0; Hy[I(i, NZ - 2)] = 0;
    }
    // Stability check, :320-321.
    double mx = 0.0;
#pragma omp parallel for reduction(max : mx) schedule(static)
    for (size_t c = 0; c < N; ++c) mx = std::max(mx, std::sqrt(Ex[c] * Ex[c] + Ez[c] * Ez[c]));
    runmax = std::max(runmax, mx);
    for (int r = 0; r < nrec; ++r) {
      const size_t c = I(rec[3 * r], rec[3 * r + 2]);
      traces[((size_t)s * 2 + 0) * nrec + r] = Ex[c];
      traces[((size_t)s * 2 + 1) * nrec + r] = Ez[c];
    }
    if (!(mx <= kStability)) { *blew_up = 1; *maxnorm = runmax; return s + 1; }
  }
  *maxnorm = runmax;
  return nsteps;
}

template <bool TWO_D>
static int seismic2_impl(int NX, int NZ, double dx, double dz, double dt,
                 const double* prof, const double* mat,
                 int isrc, int ksrc, const double* src, int nstep_src,
                 int it0, int nsteps,
                 double* fld, double* mem,
                 int nrec, const int* rec, double* traces,
                 double* maxnorm, int* blew_up, int opts, const double* ssrc, const double* cpml2d) {
  const size_t N = (size_t)NX * NZ;

  // CPML coefficient q (K a b K_half a_half b_half) of the x (z) axis at cell
  // (i, k): the axis profile at i (k), or, with the driver's 2-D fields
  // (TWO_D), the field's value at the cell -- the same field for every
  // derivative direction
  auto XP = [&](const double* ax, int q, int i, int k) -> double {
    if constexpr (TWO_D) return cpml2d[(size_t)q * N + (size_t)i + (size_t)NX * k];
    else return ax[i];
  };
  auto ZP = [&](const double* ax, int q, int i, int k) -> double {
    if constexpr (TWO_D) return cpml2d[(size_t)q * N + (size_t)i + (size_t)NX * k];
    else return ax[k];
  };
  Axis X, Y, Z;
  unpack_axes(prof, NX, 1, NZ, false, &X, &Y, &Z);
  const double *c11 = mat, *c13 = mat + N, *c15 = mat + 2 * N, *c33 = mat + 3 * N;
  const double *c35 = mat + 4 * N, *c55 = mat + 5 * N, *rho = mat + 6 * N;
  const double *gx = mat + 7 * N, *gz = mat + 8 * N;
  double *vx = fld, *vz = fld + N, *sxx = fld + 2 * N, *szz = fld + 3 * N, *sxz = fld + 4 * N;
  double *m_vxx = mem, *m_vzz = mem + N, *m_vxz = mem + 2 * N, *m_vzx = mem + 3 * N;
  double *m_sxx_x = mem + 4 * N, *m_szz_z = mem + 5 * N, *m_sxz_x = mem + 6 * N, *m_sxz_z = mem + 7 * N;
  const bool legacy = opts & 1;
  const int dens = (opts >> 1) & 3;
  // the sigmaxz loop's own velocity-gradient memory (corrected physics); the
  // legacy loops share the first four arrays
  double *m2_vxx = legacy ? m_vxx : mem + 8 * N, *m2_vzz = legacy ? m_vzz : mem + 9 * N;
  double *m2_vxz = legacy ? m_vxz : mem + 10 * N, *m2_vzx = legacy ? m_vzx : mem + 11 * N;
  auto I = [NX](int i, int k) { return (size_t)i + (size_t)NX * k; };
  const double* srcx = src;
  const double* srcz = src + nstep_src;
  *blew_up = 0;
  double runmax = 0.0;

  for (int s = 0; s < nsteps; ++s) {
    const int t = it0 + s;
    // sigmaxx, sigmazz, :247-281.
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= NZ - 1; ++k)
      for (int i = 0; i <= NX - 2; ++i) {
        const size_t c = I(i, k), cxp = I(i + 1, k), czm = I(i, k - 1);
        double dvx_dx = (vx[cxp] - vx[c]) / dx;
        double dvz_dz = (vz[c] - vz[czm]) / dz;
        double dvz_dx = (vz[cxp] - vz[c]) / dx;
        double dvx_dz = (vx[c] - vx[czm]) / dz;
        // legacy: b_x_half(j), :255 (0 past the x axis); corrected: b_x_half(i)
        const double bxh = legacy ? ((k < NX) ? X.bh[k] : 0.0) : XP(X.bh, 5, i, k);
        m_vxx[c] = bxh * m_vxx[c] + XP(X.ah, 4, i, k) * dvx_dx;
        m_vzz[c] = ZP(Z.b, 2, i, k) * m_vzz[c] + ZP(Z.a, 1, i, k) * dvz_dz;
        m_vxz[c] = ZP(Z.bh, 5, i, k) * m_vxz[c] + ZP(Z.ah, 4, i, k) * dvx_dz;
        m_vzx[c] = XP(X.b, 2, i, k) * m_vzx[c] + XP(X.a, 1, i, k) * dvz_dx;
        dvx_dx = dvx_dx / XP(X.Kh, 3, i, k) + m_vxx[c];
        dvz_dz = dvz_dz / ZP(Z.K, 0, i, k) + m_vzz[c];
        dvz_dx = dvz_dx / XP(X.K, 0, i, k) + m_vzx[c];
        dvx_dz = dvx_dz / ZP(Z.Kh, 3, i, k) + m_vxz[c];
        sxx[c] = sxx[c] + (((c11[cxp] + 2 * c11[c] + c11[czm]) / 4) * dvx_dx +
                           ((c13[cxp] + 2 * c13[c] + c13[czm]) / 4) * dvz_dz +
                           ((c15[cxp] + 2 * c15[c] + c15[czm]) / 4) * (dvz_dx + dvx_dz)) * dt;
        szz[c] = szz[c] + (((c13[cxp] + 2 * c13[c] + c13[czm]) / 4) * dvx_dx +
                           ((c33[cxp] + 2 * c33[c] + c33[czm]) / 4) * dvz_dz +
                           ((c35[cxp] + 2 * c35[c] + c35[czm]) / 4) * (dvz_dx + dvx_dz)) * dt;
      }
    // sigmaxz, :283-312: legacy, the same memory arrays again (each advances
    // twice where both loops visit a cell); corrected, its own arrays.
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= NZ - 2; ++k)
      for (int i = 1; i <= NX - 1; ++i) {
        const size_t c = I(i, k), cxm = I(i - 1, k), czp = I(i, k + 1);
        double dvx_dx = (vx[c] - vx[cxm]) / dx;
        double dvz_dz = (vz[czp] - vz[c]) / dz;
        double dvz_dx = (vz[c] - vz[cxm]) / dx;
        double dvx_dz = (vx[czp] - vx[c]) / dz;
        m2_vxx[c] = XP(X.bh, 5, i, k) * m2_vxx[c] + XP(X.ah, 4, i, k) * dvx_dx;
        m2_vzz[c] = ZP(Z.b, 2, i, k) * m2_vzz[c] + ZP(Z.a, 1, i, k) * dvz_dz;
        m2_vxz[c] = ZP(Z.bh, 5, i, k) * m2_vxz[c] + ZP(Z.ah, 4, i, k) * dvx_dz;
        m2_vzx[c] = XP(X.b, 2, i, k) * m2_vzx[c] + XP(X.a, 1, i, k) * dvz_dx;
        dvx_dx = dvx_dx / XP(X.Kh, 3, i, k) + m2_vxx[c];
        dvz_dz = dvz_dz / ZP(Z.K, 0, i, k) + m2_vzz[c];
        dvz_dx = dvz_dx / XP(X.K, 0, i, k) + m2_vzx[c];
        dvx_dz = dvx_dz / ZP(Z.Kh, 3, i, k) + m2_vxz[c];
        sxz[c] = sxz[c] + (((c15[czp] + 2 * c15[c] + c15[cxm]) / 4) * dvx_dx +
                           ((c35[czp] + 2 * c35[c] + c35[cxm]) / 4) * dvz_dz +
                           ((c55[czp] + 2 * c55[c] + c55[cxm]) / 4) * (dvz_dx + dvx_dz)) * dt;
      }
    // Stress source (moment tensor; explosive = equal normal components):
    // sigma_ij += f_ij(t) dt at the source cell, after both stress loops.
    if (ssrc) {
      const size_t c = I(isrc, ksrc);
      sxx[c] += ssrc[t] * dt;
      szz[c] += ssrc[nstep_src + t] * dt;
      sxz[c] += ssrc[2 * (size_t)nstep_src + t] * dt;
    }
    // vx, :317-336.
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= NZ - 1; ++k)
      for (int i = 1; i <= NX - 1; ++i) {
        const size_t c = I(i, k);
        double dsxx_dx = (sxx[c] - sxx[I(i - 1, k)]) / dx;
        double dsxz_dz = (sxz[c] - sxz[I(i, k - 1)]) / dz;
        m_sxx_x[c] = XP(X.b, 2, i, k) * m_sxx_x[c] + XP(X.a, 1, i, k) * dsxx_dx;
        m_sxz_z[c] = ZP(Z.b, 2, i, k) * m_sxz_z[c] + ZP(Z.a, 1, i, k) * dsxz_dz;
        dsxx_dx = dsxx_dx / XP(X.K, 0, i, k) + m_sxx_x[c];
        dsxz_dz = dsxz_dz / ZP(Z.K, 0, i, k) + m_sxz_z[c];
        // legacy: the cell's own rho (:334; the average of :320 is unused);
        // corrected: the average of :320 by the density method
        const double rx = legacy ? rho[c] : rho_avg(dens, 2.0, rho[c], rho[I(i - 1, k)], rho[I(i, k - 1)]);
        vx[c] = vx[c] * (1 - gx[c]) + (dsxx_dx + dsxz_dz) * dt / rx;
      }
    // vz, :338-357.
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= NZ - 2; ++k)
      for (int i = 0; i <= NX - 2; ++i) {
        const size_t c = I(i, k);
        const double deltarho = rho_avg(dens, 2.0, rho[c], rho[I(i + 1, k)], rho[I(i, k + 1)]);  // :342
        double dsxz_dx = (sxz[I(i + 1, k)] - sxz[c]) / dx;
        double dszz_dz = (szz[I(i, k + 1)] - szz[c]) / dz;
        m_sxz_x[c] = XP(X.bh, 5, i, k) * m_sxz_x[c] + XP(X.ah, 4, i, k) * dsxz_dx;
        m_szz_z[c] = ZP(Z.bh, 5, i, k) * m_szz_z[c] + ZP(Z.ah, 4, i, k) * dszz_dz;
        dsxz_dx = dsxz_dx / XP(X.Kh, 3, i, k) + m_sxz_x[c];
        dszz_dz = dszz_dz / ZP(Z.Kh, 3, i, k) + m_szz_z[c];
        vz[c] = vz[c] * (1 - gz[c]) + (dsxz_dx + dszz_dz) * dt / deltarho;
      }
    // Source, :360-361.
    {
      const size_t c = I(isrc, ksrc);
      vx[c] = vx[c] + srcx[t] * dt / rho[c];
      vz[c] = vz[c] + srcz[t] * dt / rho[c];
    }
    // Dirichlet edges, :365-375.
    for (int k = 0; k < NZ; ++k) { vx[I(0, k)] = vx[I(NX - 1, k)] = 0; vz[I(0, k)] = vz[I(NX - 1, k)] = 0; }
    for (int i = 0; i < NX; ++i) { vx[I(i, 0)] = vx[I(i, NZ - 1)] = 0; vz[I(i, 0)] = vz[I(i, NZ - 1)] = 0; }
    // Stability check, :378-379.
    double mx = 0.0;
#pragma omp parallel for reduction(max : mx) schedule(static)
    for (size_t c = 0; c < N; ++c) mx = std::max(mx, std::sqrt(vx[c] * vx[c] + vz[c] * vz[c]));
    runmax = std::max(runmax, mx);
    for (int r = 0; r < nrec; ++r) {
      const size_t c = I(rec[3 * r], rec[3 * r + 2]);
      traces[((size_t)s * 2 + 0) * nrec + r] = vx[c];
      traces[((size_t)s * 2 + 1) * nrec + r] = vz[c];
    }
    if (!(mx <= kStability)) { *blew_up = 1; *maxnorm = runmax; return s + 1; }
  }
  *maxnorm = runmax;
  return nsteps;
}

extern "C" {

// ---------------------------------------------------------------------------
// electromag2: legacy/fortran/electromagfdtd.f95:10-326.
//   mat   = eps11, eps13, eps33, sig11, sig13, sig33   (6 x NX*NZ)
//   fld   = Ex, Ez, Hy                                  (3 x NX*NZ)
//   mem   = dEx_dz, dEz_dx, dHy_dz, dHy_dx              (4 x NX*NZ)
//   src   = srcx, srcz                                  (2 x nstep_src)
//   chans = Ex, Ez
// Returns the number of steps completed; *blew_up = 1 if the norm check of
// electromagfdtd.f95:320-321 fired (the run stops there, as the Fortran does).
int orc_electromag2(int NX, int NZ, double dx, double dz, double dt,
                    const double* prof, const double* mat,
                    int isrc, int ksrc, const double* src, int nstep_src,
                    int it0, int nsteps,
                    double* fld, double* mem,
                    int nrec, const int* rec, double* traces,
                    double* maxnorm, int* blew_up, const double* cpml2d) {
  return cpml2d ? electromag2_impl<true>(NX, NZ, dx, dz, dt, prof, mat, isrc, ksrc, src, nstep_src, it0, nsteps, fld, mem, nrec, rec, traces, maxnorm, blew_up, cpml2d) : electromag2_impl<false>(NX, NZ, dx, dz, dt, prof, mat, isrc, ksrc, src, nstep_src, it0, nsteps, fld, mem, nrec, rec, traces, maxnorm, blew_up, cpml2d);
}

// ---------------------------------------------------------------------------
// electromag2c: legacy/fortran/electromagfdtd.f95:329-616, electromag2 with
// complex permittivities (material_rwc, readwrite_routines.f95:969-988), so
// complex update coefficients, fields and memory variables.  Complex arrays
// travel as (real, imaginary) plane pairs:
//   mat   = eps11 re, im, eps13 re, im, eps33 re, im, sig11, sig13, sig33  (9 x N)
//   fld   = Ex re, im, Ez re, im, Hy re, im                                (6 x N)
//   mem   = dEx_dz re, im, dEz_dx re, im, dHy_dz re, im, dHy_dx re, im     (8 x N)
//   src   = srcx, srcz (real); chans = Ex re, Ex im, Ez re, Ez im
// The norm of :598 is |sqrt(Ex^2 + Ez^2)| with complex squares.
int orc_electromag2c(int NX, int NZ, double dx, double dz, double dt,
                     const double* prof, const double* mat,
                     int isrc, int ksrc, const double* src, int nstep_src,
                     int it0, int nsteps,
                     double* fld, double* mem,
                     int nrec, const int* rec, double* traces,
                     double* maxnorm, int* blew_up) {
  using cd = std::complex<double>;
  const size_t N = (size_t)NX * NZ;
  Axis X, Y, Z;
  unpack_axes(prof, NX, 1, NZ, false, &X, &Y, &Z);
  auto cplx = [&](const double* re, const double* im) {
    std::vector<cd> v(N);
    for (size_t c = 0; c < N; ++c) v[c] = cd(re[c], im[c]);
    return v;
  };
  const std::vector<cd> eps11 = cplx(mat, mat + N), eps13 = cplx(mat + 2 * N, mat + 3 * N),
                        eps33 = cplx(mat + 4 * N, mat + 5 * N);
  const double *sig11 = mat + 6 * N, *sig13 = mat + 7 * N, *sig33 = mat + 8 * N;
  std::vector<cd> Ex = cplx(fld, fld + N), Ez = cplx(fld + 2 * N, fld + 3 * N), Hy = cplx(fld + 4 * N, fld + 5 * N);
  std::vector<cd> mExz = cplx(mem, mem + N), mEzx = cplx(mem + 2 * N, mem + 3 * N),
                  mHyz = cplx(mem + 4 * N, mem + 5 * N), mHyx = cplx(mem + 6 * N, mem + 7 * N);
  auto I = [NX](int i, int k) { return (size_t)i + (size_t)NX * k; };

  // Coefficients, :439-451.
  std::vector<cd> caEx(N), cbEx(N), caEz(N), cbEz(N);
  for (size_t c = 0; c < N; ++c) {
    const cd ex = (eps11[c] + eps13[c]) * kEps0, ez = (eps13[c] + eps33[c]) * kEps0;
    const double sx = sig11[c] + sig13[c], sz = sig13[c] + sig33[c];
    caEx[c] = (1.0 - sx * dt / (2.0 * ex)) / (1.0 + sx * dt / (2.0 * ex));
    cbEx[c] = (dt / ex) / (1.0 + sx * dt / (2.0 * ex));
    caEz[c] = (1.0 - sz * dt / (2.0 * ez)) / (1.0 + sz * dt / (2.0 * ez));
    cbEz[c] = (dt / ez) / (1.0 + sz * dt / (2.0 * ez));
  }
  const double daHy = 1.0, dbHy = dt / kMu0;  // :453-455
  const double* srcx = src;
  const double* srcz = src + nstep_src;
  *blew_up = 0;
  double runmax = 0.0;
  int done = nsteps;

  for (int s = 0; s < nsteps; ++s) {
    const int t = it0 + s;
    // Hy and its memory variables, :530-549.
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= NZ - 2; ++k)
      for (int i = 0; i <= NX - 2; ++i) {
        const size_t c = I(i, k);
        cd dEx_dz = (Ex[I(i, k + 1)] - Ex[c]) / dz;
        mExz[c] = Z.b[k] * mExz[c] + Z.a[k] * dEx_dz;
        dEx_dz = dEx_dz / Z.K[k] + mExz[c];
        cd dEz_dx = (Ez[I(i + 1, k)] - Ez[c]) / dx;
        mEzx[c] = X.b[i] * mEzx[c] + X.a[i] * dEz_dx;
        dEz_dx = dEz_dx / X.K[i] + mEzx[c];
        Hy[c] = daHy * Hy[c] + dbHy * (dEz_dx + dEx_dz);
      }
    // Ex, :556-565.
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= NZ - 2; ++k)
      for (int i = 0; i <= NX - 2; ++i) {
        const size_t c = I(i, k), cm = I(i, k - 1);
        cd d = (Hy[c] - Hy[cm]) / dz;
        mHyz[c] = Z.bh[k] * mHyz[c] + Z.ah[k] * d;
        d = d / Z.Kh[k] + mHyz[c];
        Ex[c] = ((caEx[c] + caEx[cm]) / 2.0) * Ex[c] + ((cbEx[c] + cbEx[cm]) / 2.0) * d;
      }
    // Ez, :567-576.
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= NZ - 2; ++k)
      for (int i = 1; i <= NX - 2; ++i) {
        const size_t c = I(i, k), cm = I(i - 1, k);
        cd d = (Hy[c] - Hy[cm]) / dx;
        mHyx[c] = X.bh[i] * mHyx[c] + X.ah[i] * d;
        d = d / X.Kh[i] + mHyx[c];
        Ez[c] = ((caEz[c] + caEz[cm]) / 2.0) * Ez[c] + ((cbEz[c] + cbEz[cm]) / 2.0) * d;
      }
    // Source, :581-582: divided by the complex relative permittivity.
    {
      const size_t c = I(isrc, ksrc);
      Ex[c] = Ex[c] + srcx[t] * dt / eps11[c];
      Ez[c] = Ez[c] + srcz[t] * dt / eps33[c];
    }
    // Dirichlet edges, :585-598.
    for (int k = 0; k < NZ; ++k) {
      Ex[I(0, k)] = 0.0; Ex[I(NX - 2, k)] = 0.0;
      Ez[I(0, k)] = 0.0; Ez[I(NX - 1, k)] = 0.0;
      Hy[I(0, k)] = 0.0; Hy[I(NX - 2, k)] = 0.0;
    }
    for (int i = 0; i < NX; ++i) {
      Ex[I(i, 0)] = 0.0; Ex[I(i, NZ - 1)] = 0.0;
      Ez[I(i, 0)] = 0.0; Ez[I(i, NZ - 2)] = 0.0;
      Hy[I(i, 0)] = 0.0; Hy[I(i, NZ - 2)] = 0.0;
    }
    // Stability check, :601-602.
    double mx = 0.0;
#pragma omp parallel for reduction(max : mx) schedule(static)
    for (size_t c = 0; c < N; ++c) mx = std::max(mx, std::abs(std::sqrt(Ex[c] * Ex[c] + Ez[c] * Ez[c])));
    runmax = std::max(runmax, mx);
    for (int r = 0; r < nrec; ++r) {
      const size_t c = I(rec[3 * r], rec[3 * r + 2]);
      traces[((size_t)s * 4 + 0) * nrec + r] = Ex[c].real();
      traces[((size_t)s * 4 + 1) * nrec + r] = Ex[c].imag();
      traces[((size_t)s * 4 + 2) * nrec + r] = Ez[c].real();
      traces[((size_t)s * 4 + 3) * nrec + r] = Ez[c].imag();
    }
    if (!(mx <= kStability)) { *blew_up = 1; done = s + 1; break; }
  }
  *maxnorm = runmax;
  auto out = [&](const std::vector<cd>& v, double* re, double* im) {
    for (size_t c = 0; c < N; ++c) { re[c] = v[c].real(); im[c] = v[c].imag(); }
  };
  out(Ex, fld, fld + N); out(Ez, fld + 2 * N, fld + 3 * N); out(Hy, fld + 4 * N, fld + 5 * N);
  out(mExz, mem, mem + N); out(mEzx, mem + 2 * N, mem + 3 * N);
  out(mHyz, mem + 4 * N, mem + 5 * N); out(mHyx, mem + 6 * N, mem + 7 * N);
  return done;
}

// ---------------------------------------------------------------------------
// seismic2: legacy/fortran/seismicfdtd.f95:12-385.
//   mat   = c11, c13, c15, c33, c35, c55, rho, gamma_x, gamma_z  (9 x NX*NZ)
//   fld   = vx, vz, sigmaxx, sigmazz, sigmaxz                     (5 x NX*NZ)
//   mem   = dvx_dx, dvz_dz, dvx_dz, dvz_dx,
//           dsigmaxx_dx, dsigmazz_dz, dsigmaxz_dx, dsigmaxz_dz,
//           dvx_dx, dvz_dz, dvx_dz, dvz_dx of the sigmaxz loop     (12 x NX*NZ)
//   src   = srcx, srcz; chans = vx, vz
//   ssrc  = stress source sxx, szz, sxz (3 x nstep_src) or NULL
//   opts  = bit 0: legacy quirks; bits 1-2: density method (rho_avg)
// With the legacy quirks (opts bit 0) the loops are the Fortran's as written:
//   Q2  the four velocity-gradient memory variables are shared by both stress
//       loops, so they advance twice per step where the loops overlap
//       (:255-262, :291-298); the last four memory arrays stay unused;
//   Q3  the first stress loop indexes b_x_half by the z index (:255); where
//       that index runs past the x axis (NZ > NX) the interior value 0 of the
//       profile writer is used;
//   vx divides by the cell's own rho (:334) although :320 forms the average.
// Without (the default, corrected physics): the sigmaxz loop keeps its own
// four memory variables (each advances once per step), b_x_half(i), and vx
// divides by the average of :320.  The density method applies to the vz
// average (:342) in both modes and to the vx average when it is used.
// gamma_x and gamma_z are taken as given (the legacy file-loading slip of
// :158-159 belongs to the file reader, not the stencil).
int orc_seismic2(int NX, int NZ, double dx, double dz, double dt,
                 const double* prof, const double* mat,
                 int isrc, int ksrc, const double* src, int nstep_src,
                 int it0, int nsteps,
                 double* fld, double* mem,
                 int nrec, const int* rec, double* traces,
                 double* maxnorm, int* blew_up, int opts, const double* ssrc, const double* cpml2d) {
  return cpml2d ? seismic2_impl<true>(NX, NZ, dx, dz, dt, prof, mat, isrc, ksrc, src, nstep_src, it0, nsteps, fld, mem, nrec, rec, traces, maxnorm, blew_up, opts, ssrc, cpml2d) : seismic2_impl<false>(NX, NZ, dx, dz, dt, prof, mat, isrc, ksrc, src, nstep_src, it0, nsteps, fld, mem, nrec, rec, traces, maxnorm, blew_up, opts, ssrc, cpml2d);
}

// ---------------------------------------------------------------------------
// seismic25: legacy/fortran/seismicfdtd.f95:388-949.
//   mat = c11 c12 c13 c14 c15 c16 c22 c23 c24 c25 c26 c33 c34 c35 c36
//         c44 c45 c46 c55 c56 c66 rho gamma_x gamma_y gamma_z  (25 x NX*NZ)
//   fld = vx vy vz sxx syy szz sxy sxz syz                      (9 x NX*NY*NZ)
//   mem = dvx_dx dvx_dy dvx_dz dvy_dx dvy_dy dvy_dz dvz_dx dvz_dy dvz_dz
//         dsxx_dx dsyy_dy dszz_dz dsxy_dx dsxy_dy dsxz_dx dsxz_dz
//         dsyz_dy dsyz_dz                                        (18 x NX*NY*NZ)
//   src = srcx srcy srcz; chans = vx vy vz
//   ssrc = stress source sxx syy szz sxy sxz syz (6 x nstep_src) or NULL
//   opts = bit 0: legacy quirks; bits 1-2: density method (rho_avg)
// The nine velocity-gradient memory variables are shared by the four stress
// loops and advance once per loop (:630-638, :691-699, :750-758, :795-803),
// and the two derivatives that :701-707 leave unscaled stay so, in both
// modes.  Q4: with the legacy quirks the coefficient pairs of :657
// (c16 (dvx_dy + dvz_dy)) and :766 (c45 (dvx_dz + dvz_dx)) are kept as
// written; without (the default) they are the Voigt pairs c16 (dvx_dy +
// dvy_dx) and c45 (dvy_dz + dvz_dy).  Attenuation: the legacy
// routine has none; v <- v (1 - gamma) + ... with y-invariant gamma, as in
// seismic2 (:334, :355), is applied here and reduces to the legacy update
// when gamma = 0.
int orc_seismic25(int NX, int NY, int NZ, double dx, double dy, double dz, double dt,
                  const double* prof, const double* mat,
                  int isrc, int jsrc, int ksrc, const double* src, int nstep_src,
                  int it0, int nsteps,
                  double* fld, double* mem,
                  int nrec, const int* rec, double* traces,
                  double* maxnorm, int* blew_up, int opts, const double* ssrc) {
  const size_t N2 = (size_t)NX * NZ;
  const size_t N = (size_t)NX * NY * NZ;
  const bool legacy = opts & 1;
  const int dens = (opts >> 1) & 3;
  Axis X, Y, Z;
  unpack_axes(prof, NX, NY, NZ, true, &X, &Y, &Z);
  const double* C[21];
  for (int q = 0; q < 21; ++q) C[q] = mat + q * N2;
  const double *c11 = C[0], *c12 = C[1], *c13 = C[2], *c14 = C[3], *c15 = C[4], *c16 = C[5];
  const double *c22 = C[6], *c23 = C[7], *c24 = C[8], *c25 = C[9], *c26 = C[10];
  const double *c33 = C[11], *c34 = C[12], *c35 = C[13], *c36 = C[14];
  const double *c44 = C[15], *c45 = C[16], *c46 = C[17], *c55 = C[18], *c56 = C[19], *c66 = C[20];
  const double *rho = mat + 21 * N2, *gx = mat + 22 * N2, *gy = mat + 23 * N2, *gz = mat + 24 * N2;
  double *vx = fld, *vy = fld + N, *vz = fld + 2 * N;
  double *sxx = fld + 3 * N, *syy = fld + 4 * N, *szz = fld + 5 * N;
  double *sxy = fld + 6 * N, *sxz = fld + 7 * N, *syz = fld + 8 * N;
  double* M[18];
  for (int q = 0; q < 18; ++q) M[q] = mem + q * N;
  double *m_vx_x = M[0], *m_vx_y = M[1], *m_vx_z = M[2], *m_vy_x = M[3], *m_vy_y = M[4], *m_vy_z = M[5];
  double *m_vz_x = M[6], *m_vz_y = M[7], *m_vz_z = M[8];
  double *m_sxx_x = M[9], *m_syy_y = M[10], *m_szz_z = M[11], *m_sxy_x = M[12], *m_sxy_y = M[13];
  double *m_sxz_x = M[14], *m_sxz_z = M[15], *m_syz_y = M[16], *m_syz_z = M[17];
  auto I = [NX, NY](int i, int j, int k) { return (size_t)i + (size_t)NX * ((size_t)j + (size_t)NY * k); };
  auto P = [NX](int i, int k) { return (size_t)i + (size_t)NX * k; };
  // 4-point average of a y-invariant coefficient.
  auto av4 = [&](const double* c, int i0, int k0, int i1, int k1, int i2, int k2, int i3, int k3) {
    return c[P(i0, k0)] + c[P(i1, k1)] + c[P(i2, k2)] + c[P(i3, k3)];
  };
  const double *srcx = src, *srcy = src + nstep_src, *srcz = src + 2 * nstep_src;
  *blew_up = 0;
  double runmax = 0.0;

  for (int s = 0; s < nsteps; ++s) {
    const int t = it0 + s;
    // Loop 1: sigmaxx, sigmayy, sigmazz, :616-678.
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= NZ - 1; ++k)
      for (int j = 1; j <= NY - 1; ++j)
        for (int i = 0; i <= NX - 2; ++i) {
          const size_t c = I(i, j, k);
          double dvx_dx = (vx[I(i + 1, j, k)] - vx[c]) / dx;
          double dvy_dx = (vy[I(i + 1, j, k)] - vy[c]) / dx;
          double dvz_dx = (vz[I(i + 1, j, k)] - vz[c]) / dx;
          double dvy_dy = (vy[c] - vy[I(i, j - 1, k)]) / dy;
          double dvx_dy = (vx[c] - vx[I(i, j - 1, k)]) / dy;
          double dvz_dy = (vz[c] - vz[I(i, j - 1, k)]) / dy;
          double dvz_dz = (vz[c] - vz[I(i, j, k - 1)]) / dz;
          double dvx_dz = (vx[c] - vx[I(i, j, k - 1)]) / dz;
          double dvy_dz = (vy[c] - vy[I(i, j, k - 1)]) / dz;
          m_vx_x[c] = X.bh[i] * m_vx_x[c] + X.ah[i] * dvx_dx;
          m_vy_x[c] = X.bh[i] * m_vy_x[c] + X.ah[i] * dvy_dx;
          m_vz_x[c] = X.bh[i] * m_vz_x[c] + X.ah[i] * dvz_dx;
          m_vy_y[c] = Y.b[j] * m_vy_y[c] + Y.a[j] * dvy_dy;
          m_vx_y[c] = Y.b[j] * m_vx_y[c] + Y.a[j] * dvx_dy;
          m_vz_y[c] = Y.b[j] * m_vz_y[c] + Y.a[j] * dvz_dy;
          m_vz_z[c] = Z.b[k] * m_vz_z[c] + Z.a[k] * dvz_dz;
          m_vx_z[c] = Z.b[k] * m_vx_z[c] + Z.a[k] * dvx_dz;
          m_vy_z[c] = Z.b[k] * m_vy_z[c] + Z.a[k] * dvy_dz;
          dvx_dx = dvx_dx / X.Kh[i] + m_vx_x[c];
          dvy_dx = dvy_dx / X.Kh[i] + m_vy_x[c];
          dvz_dx = dvz_dx / X.Kh[i] + m_vz_x[c];
          dvy_dy = dvy_dy / Y.K[j] + m_vy_y[c];
          dvx_dy = dvx_dy / Y.K[j] + m_vx_y[c];
          dvz_dy = dvz_dy / Y.K[j] + m_vz_y[c];
          dvz_dz = dvz_dz / Z.K[k] + m_vz_z[c];
          dvx_dz = dvx_dz / Z.K[k] + m_vx_z[c];
          dvy_dz = dvy_dz / Z.K[k] + m_vy_z[c];
          auto A = [&](const double* cc) { return av4(cc, i + 1, k, i, k, i, k - 1, i + 1, k - 1); };
          sxx[c] = sxx[c] + ((A(c11) / 4) * dvx_dx + (A(c12) / 4) * dvy_dy + (A(c13) / 4) * dvz_dz +
                             (A(c14) / 8) * (dvy_dz + dvz_dy) + (A(c15) / 8) * (dvx_dz + dvz_dx) +
                             (A(c16) / 8) * (legacy ? dvx_dy + dvz_dy : dvx_dy + dvy_dx)) * dt;  // Q4, :657
          syy[c] = syy[c] + ((A(c12) / 4) * dvx_dx + (A(c22) / 4) * dvy_dy + (A(c23) / 4) * dvz_dz +
                             (A(c24) / 8) * (dvy_dz + dvz_dy) + (A(c25) / 8) * (dvx_dz + dvz_dx) +
                             (A(c26) / 8) * (dvy_dx + dvx_dy)) * dt;
          szz[c] = szz[c] + ((A(c13) / 4) * dvx_dx + (A(c23) / 4) * dvy_dy + (A(c33) / 4) * dvz_dz +
                             (A(c34) / 8) * (dvy_dz + dvz_dy) + (A(c35) / 8) * (dvx_dz + dvz_dx) +
                             (A(c36) / 8) * (dvy_dx + dvx_dy)) * dt;
        }
    // Loop 2: sigmaxy, :681-725 (dvz_dx and dvx_dz are not rescaled, :701-707).
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= NZ - 1; ++k)
      for (int j = 0; j <= NY - 2; ++j)
        for (int i = 1; i <= NX - 1; ++i) {
          const size_t c = I(i, j, k);
          double dvx_dx = (vx[c] - vx[I(i - 1, j, k)]) / dx;
          double dvy_dx = (vy[c] - vy[I(i - 1, j, k)]) / dx;
          double dvz_dx = (vz[c] - vz[I(i - 1, j, k)]) / dx;
          double dvy_dy = (vy[I(i, j + 1, k)] - vy[c]) / dy;
          double dvx_dy = (vx[I(i, j + 1, k)] - vx[c]) / dy;
          double dvz_dy = (vz[I(i, j + 1, k)] - vz[c]) / dy;
          double dvz_dz = (vz[c] - vz[I(i, j, k - 1)]) / dz;
          double dvx_dz = (vx[c] - vx[I(i, j, k - 1)]) / dz;
          double dvy_dz = (vy[c] - vy[I(i, j, k - 1)]) / dz;
          m_vx_x[c] = X.b[i] * m_vx_x[c] + X.a[i] * dvx_dx;
          m_vy_x[c] = X.b[i] * m_vy_x[c] + X.a[i] * dvy_dx;
          m_vz_x[c] = X.b[i] * m_vz_x[c] + X.a[i] * dvz_dx;
          m_vy_y[c] = Y.bh[j] * m_vy_y[c] + Y.ah[j] * dvy_dy;
          m_vx_y[c] = Y.bh[j] * m_vx_y[c] + Y.ah[j] * dvx_dy;
          m_vz_y[c] = Y.bh[j] * m_vz_y[c] + Y.ah[j] * dvz_dy;
          m_vz_z[c] = Z.bh[k] * m_vz_z[c] + Z.ah[k] * dvz_dz;
          m_vx_z[c] = Z.bh[k] * m_vx_z[c] + Z.ah[k] * dvx_dz;
          m_vy_z[c] = Z.bh[k] * m_vy_z[c] + Z.ah[k] * dvy_dz;
          dvx_dx = dvx_dx / X.K[i] + m_vx_x[c];
          dvy_dx = dvy_dx / X.K[i] + m_vy_x[c];
          dvy_dy = dvy_dy / Y.Kh[j] + m_vy_y[c];
          dvx_dy = dvx_dy / Y.Kh[j] + m_vx_y[c];
          dvz_dy = dvz_dy / Y.Kh[j] + m_vz_y[c];
          dvz_dz = dvz_dz / Z.Kh[k] + m_vz_z[c];
          dvy_dz = dvy_dz / Z.Kh[k] + m_vy_z[c];
          auto A = [&](const double* cc) { return av4(cc, i, k, i - 1, k, i, k - 1, i - 1, k - 1); };
          sxy[c] = sxy[c] + ((A(c16) / 4) * dvx_dx + (A(c26) / 4) * dvy_dy + (A(c36) / 4) * dvz_dz +
                             (A(c46) / 8) * (dvz_dy + dvy_dz) + (A(c56) / 8) * (dvz_dx + dvx_dz) +
                             (A(c66) / 8) * (dvy_dx + dvx_dy)) * dt;
        }
    // Loops 3 and 4: sigmaxz (:728-771) then sigmayz (:774-815), inside one k loop.
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= NZ - 2; ++k) {
      for (int j = 1; j <= NY - 1; ++j)
        for (int i = 1; i <= NX - 1; ++i) {
          const size_t c = I(i, j, k);
          double dvx_dx = (vx[c] - vx[I(i - 1, j, k)]) / dx;
          double dvy_dx = (vy[c] - vy[I(i - 1, j, k)]) / dx;
          double dvz_dx = (vz[c] - vz[I(i - 1, j, k)]) / dx;
          double dvy_dy = (vy[c] - vy[I(i, j - 1, k)]) / dy;
          double dvz_dy = (vz[c] - vz[I(i, j - 1, k)]) / dy;
          double dvx_dy = (vx[c] - vx[I(i, j - 1, k)]) / dy;
          double dvz_dz = (vz[I(i, j, k + 1)] - vz[c]) / dz;
          double dvx_dz = (vx[I(i, j, k + 1)] - vx[c]) / dz;
          double dvy_dz = (vy[I(i, j, k + 1)] - vy[c]) / dz;
          m_vx_x[c] = X.b[i] * m_vx_x[c] + X.a[i] * dvx_dx;
          m_vy_x[c] = X.b[i] * m_vy_x[c] + X.a[i] * dvy_dx;
          m_vz_x[c] = X.b[i] * m_vz_x[c] + X.a[i] * dvz_dx;
          m_vy_y[c] = Y.b[j] * m_vy_y[c] + Y.a[j] * dvy_dy;
          m_vx_y[c] = Y.b[j] * m_vx_y[c] + Y.a[j] * dvx_dy;
          m_vz_y[c] = Y.b[j] * m_vz_y[c] + Y.a[j] * dvz_dy;
          m_vz_z[c] = Z.bh[k] * m_vz_z[c] + Z.ah[k] * dvz_dz;
          m_vx_z[c] = Z.bh[k] * m_vx_z[c] + Z.ah[k] * dvx_dz;
          m_vy_z[c] = Z.bh[k] * m_vy_z[c] + Z.ah[k] * dvy_dz;
          dvx_dx = dvx_dx / X.K[i] + m_vx_x[c];
          dvy_dx = dvy_dx / X.K[i] + m_vy_x[c];
          dvz_dx = dvz_dx / X.K[i] + m_vz_x[c];
          dvy_dy = dvy_dy / Y.K[j] + m_vy_y[c];
          dvx_dy = dvx_dy / Y.K[j] + m_vx_y[c];
          dvz_dy = dvz_dy / Y.K[j] + m_vz_y[c];
          dvz_dz = dvz_dz / Z.Kh[k] + m_vz_z[c];
          dvx_dz = dvx_dz / Z.Kh[k] + m_vx_z[c];
          dvy_dz = dvy_dz / Z.Kh[k] + m_vy_z[c];
          auto A = [&](const double* cc) { return av4(cc, i, k + 1, i, k, i - 1, k, i - 1, k + 1); };
          sxz[c] = sxz[c] + ((A(c15) / 4) * dvx_dx + (A(c25) / 4) * dvy_dy + (A(c35) / 4) * dvz_dz +
                             (A(c45) / 8) * (legacy ? dvx_dz + dvz_dx : dvy_dz + dvz_dy) +  // Q4, :766
                             (A(c55) / 8) * (dvx_dz + dvz_dx) + (A(c56) / 8) * (dvx_dy + dvy_dx)) * dt;
        }
      for (int j = 0; j <= NY - 2; ++j)
        for (int i = 0; i <= NX - 2; ++i) {
          const size_t c = I(i, j, k);
          double dvx_dx = (vx[I(i + 1, j, k)] - vx[c]) / dx;
          double dvy_dx = (vy[I(i + 1, j, k)] - vy[c]) / dx;
          double dvz_dx = (vz[I(i + 1, j, k)] - vz[c]) / dx;
          double dvy_dy = (vy[I(i, j + 1, k)] - vy[c]) / dy;
          double dvx_dy = (vx[I(i, j + 1, k)] - vx[c]) / dy;
          double dvz_dy = (vz[I(i, j + 1, k)] - vz[c]) / dy;
          double dvz_dz = (vz[I(i, j, k + 1)] - vz[c]) / dz;
          double dvx_dz = (vx[I(i, j, k + 1)] - vx[c]) / dz;
          double dvy_dz = (vy[I(i, j, k + 1)] - vy[c]) / dz;
          m_vx_x[c] = X.bh[i] * m_vx_x[c] + X.ah[i] * dvx_dx;
          m_vy_x[c] = X.bh[i] * m_vy_x[c] + X.ah[i] * dvy_dx;
          m_vz_x[c] = X.bh[i] * m_vz_x[c] + X.ah[i] * dvz_dx;
          m_vy_y[c] = Y.bh[j] * m_vy_y[c] + Y.ah[j] * dvy_dy;
          m_vx_y[c] = Y.bh[j] * m_vx_y[c] + Y.ah[j] * dvx_dy;
          m_vz_y[c] = Y.bh[j] * m_vz_y[c] + Y.ah[j] * dvz_dy;
          m_vz_z[c] = Z.bh[k] * m_vz_z[c] + Z.ah[k] * dvz_dz;
          m_vx_z[c] = Z.bh[k] * m_vx_z[c] + Z.ah[k] * dvx_dz;
          m_vy_z[c] = Z.bh[k] * m_vy_z[c] + Z.ah[k] * dvy_dz;
          dvx_dx = dvx_dx / X.Kh[i] + m_vx_x[c];
          dvy_dx = dvy_dx / X.Kh[i] + m_vy_x[c];
          dvz_dx = dvz_dx / X.Kh[i] + m_vz_x[c];
          dvy_dy = dvy_dy / Y.Kh[j] + m_vy_y[c];
          dvx_dy = dvx_dy / Y.Kh[j] + m_vx_y[c];
          dvz_dy = dvz_dy / Y.Kh[j] + m_vz_y[c];
          dvz_dz = dvz_dz / Z.Kh[k] + m_vz_z[c];
          dvx_dz = dvx_dz / Z.Kh[k] + m_vx_z[c];
          dvy_dz = dvy_dz / Z.Kh[k] + m_vy_z[c];
          auto A = [&](const double* cc) { return av4(cc, i + 1, k, i, k, i, k + 1, i + 1, k + 1); };
          syz[c] = syz[c] + ((A(c14) / 4) * dvx_dx + (A(c24) / 4) * dvy_dy + (A(c34) / 4) * dvz_dz +
                             (A(c44) / 8) * (dvy_dz + dvz_dy) + (A(c45) / 8) * (dvx_dz + dvz_dx) +
                             (A(c46) / 8) * (dvy_dx + dvx_dy)) * dt;
        }
    }
    // Stress source (moment tensor; explosive = equal normal components):
    // sigma_ij += f_ij(t) dt at the source cell, after the four stress loops.
    if (ssrc) {
      const size_t c = I(isrc, jsrc, ksrc);
      double* S[6] = {sxx, syy, szz, sxy, sxz, syz};
      for (int q = 0; q < 6; ++q) S[q][c] += ssrc[(size_t)q * nstep_src + t] * dt;
    }
    // vx and vy, :821-870.
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= NZ - 1; ++k) {
      for (int j = 1; j <= NY - 1; ++j)
        for (int i = 1; i <= NX - 1; ++i) {
          const size_t c = I(i, j, k);
          const double deltarho = rho_avg(dens, 4.0, rho[P(i, k)], rho[P(i - 1, k)], rho[P(i, k - 1)]);  // :825
          double d1 = (sxx[c] - sxx[I(i - 1, j, k)]) / dx;
          double d2 = (sxy[c] - sxy[I(i, j - 1, k)]) / dy;
          double d3 = (sxz[c] - sxz[I(i, j, k - 1)]) / dz;
          m_sxx_x[c] = X.b[i] * m_sxx_x[c] + X.a[i] * d1;
          m_sxy_y[c] = Y.b[j] * m_sxy_y[c] + Y.a[j] * d2;
          m_sxz_z[c] = Z.b[k] * m_sxz_z[c] + Z.a[k] * d3;
          d1 = d1 / X.K[i] + m_sxx_x[c];
          d2 = d2 / Y.K[j] + m_sxy_y[c];
          d3 = d3 / Z.K[k] + m_sxz_z[c];
          vx[c] = vx[c] * (1 - gx[P(i, k)]) + (d1 + d2 + d3) * dt / deltarho;
        }
      for (int j = 0; j <= NY - 2; ++j)
        for (int i = 0; i <= NX - 2; ++i) {
          const size_t c = I(i, j, k);
          const double deltarho = rho_avg(dens, 4.0, rho[P(i, k)], rho[P(i + 1, k)], rho[P(i, k - 1)]);  // :850
          double d1 = (sxy[I(i + 1, j, k)] - sxy[c]) / dx;
          double d2 = (syy[I(i, j + 1, k)] - syy[c]) / dy;
          double d3 = (syz[c] - syz[I(i, j, k - 1)]) / dz;
          m_sxy_x[c] = X.bh[i] * m_sxy_x[c] + X.ah[i] * d1;
          m_syy_y[c] = Y.bh[j] * m_syy_y[c] + Y.ah[j] * d2;
          m_syz_z[c] = Z.b[k] * m_syz_z[c] + Z.a[k] * d3;
          d1 = d1 / X.Kh[i] + m_sxy_x[c];
          d2 = d2 / Y.Kh[j] + m_syy_y[c];
          d3 = d3 / Z.K[k] + m_syz_z[c];
          vy[c] = vy[c] * (1 - gy[P(i, k)]) + (d1 + d2 + d3) * dt / deltarho;
        }
    }
    // vz, :872-896.
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= NZ - 2; ++k)
      for (int j = 1; j <= NY - 1; ++j)
        for (int i = 0; i <= NX - 2; ++i) {
          const size_t c = I(i, j, k);
          const double deltarho = rho_avg(dens, 4.0, rho[P(i, k)], rho[P(i + 1, k)], rho[P(i, k + 1)]);  // :876
          double d1 = (sxz[I(i + 1, j, k)] - sxz[c]) / dx;
          double d2 = (syz[c] - syz[I(i, j - 1, k)]) / dy;
          double d3 = (szz[I(i, j, k + 1)] - szz[c]) / dz;
          m_sxz_x[c] = X.bh[i] * m_sxz_x[c] + X.ah[i] * d1;
          m_syz_y[c] = Y.b[j] * m_syz_y[c] + Y.a[j] * d2;
          m_szz_z[c] = Z.bh[k] * m_szz_z[c] + Z.ah[k] * d3;
          d1 = d1 / X.Kh[i] + m_sxz_x[c];
          d2 = d2 / Y.K[j] + m_syz_y[c];
          d3 = d3 / Z.Kh[k] + m_szz_z[c];
          vz[c] = vz[c] * (1 - gz[P(i, k)]) + (d1 + d2 + d3) * dt / deltarho;
        }
    // Source, :898-900.
    {
      const size_t c = I(isrc, jsrc, ksrc);
      const double r = rho[P(isrc, ksrc)];
      vx[c] = vx[c] + srcx[t] * dt / r;
      vy[c] = vy[c] + srcy[t] * dt / r;
      vz[c] = vz[c] + srcz[t] * dt / r;
    }
    // Dirichlet faces, :903-925.
    double* V[3] = {vx, vy, vz};
    for (int q = 0; q < 3; ++q) {
      double* v = V[q];
      for (int k = 0; k < NZ; ++k)
        for (int j = 0; j < NY; ++j) { v[I(0, j, k)] = 0; v[I(NX - 1, j, k)] = 0; }
      for (int k = 0; k < NZ; ++k)
        for (int i = 0; i < NX; ++i) { v[I(i, 0, k)] = 0; v[I(i, NY - 1, k)] = 0; }
      for (int j = 0; j < NY; ++j)
        for (int i = 0; i < NX; ++i) { v[I(i, j, 0)] = 0; v[I(i, j, NZ - 1)] = 0; }
    }
    // Stability check, :928-933.
    double mx = 0.0;
#pragma omp parallel for reduction(max : mx) schedule(static)
    for (size_t c = 0; c < N; ++c) mx = std::max(mx, std::sqrt(vx[c] * vx[c] + vy[c] * vy[c] + vz[c] * vz[c]));
    runmax = std::max(runmax, mx);
    for (int r = 0; r < nrec; ++r) {
      const size_t c = I(rec[3 * r], rec[3 * r + 1], rec[3 * r + 2]);
      traces[((size_t)s * 3 + 0) * nrec + r] = vx[c];
      traces[((size_t)s * 3 + 1) * nrec + r] = vy[c];
      traces[((size_t)s * 3 + 2) * nrec + r] = vz[c];
    }
    if (!(mx <= kStability)) { *blew_up = 1; *maxnorm = runmax; return s + 1; }
  }
  *maxnorm = runmax;
  return nsteps;
}

// ---------------------------------------------------------------------------
// electromag25: legacy/fortran/electromagfdtd.f95:619-1092.
//   mat = eps11 eps12 eps13 eps22 eps23 eps33 sig11 sig12 sig13 sig22 sig23 sig33
//   fld = Ex Ey Ez Hx Hy Hz
//   mem = dEz_dy dEy_dz dEx_dz dEz_dx dEx_dy dEy_dx
//         dHz_dy dHy_dz dHz_dx dHx_dz dHx_dy dHy_dx
//   src = srcx srcy srcz; chans = Ex Ey Ez
int orc_electromag25(int NX, int NY, int NZ, double dx, double dy, double dz, double dt,
                     const double* prof, const double* mat,
                     int isrc, int jsrc, int ksrc, const double* src, int nstep_src,
                     int it0, int nsteps,
                     double* fld, double* mem,
                     int nrec, const int* rec, double* traces,
                     double* maxnorm, int* blew_up) {
  const size_t N2 = (size_t)NX * NZ;
  const size_t N = (size_t)NX * NY * NZ;
  Axis X, Y, Z;
  unpack_axes(prof, NX, NY, NZ, true, &X, &Y, &Z);
  const double *e11 = mat, *e12 = mat + N2, *e13 = mat + 2 * N2, *e22 = mat + 3 * N2, *e23 = mat + 4 * N2,
               *e33 = mat + 5 * N2;
  const double *s11 = mat + 6 * N2, *s12 = mat + 7 * N2, *s13 = mat + 8 * N2, *s22 = mat + 9 * N2,
               *s23 = mat + 10 * N2, *s33 = mat + 11 * N2;
  double *Ex = fld, *Ey = fld + N, *Ez = fld + 2 * N, *Hx = fld + 3 * N, *Hy = fld + 4 * N, *Hz = fld + 5 * N;
  double* M[12];
  for (int q = 0; q < 12; ++q) M[q] = mem + q * N;
  double *mEz_y = M[0], *mEy_z = M[1], *mEx_z = M[2], *mEz_x = M[3], *mEx_y = M[4], *mEy_x = M[5];
  double *mHz_y = M[6], *mHy_z = M[7], *mHz_x = M[8], *mHx_z = M[9], *mHx_y = M[10], *mHy_x = M[11];
  auto I = [NX, NY](int i, int j, int k) { return (size_t)i + (size_t)NX * ((size_t)j + (size_t)NY * k); };
  auto P = [NX](int i, int k) { return (size_t)i + (size_t)NX * k; };

  // Coefficients, :756-789.
  std::vector<double> caEx(N2), cbEx(N2), caEy(N2), cbEy(N2), caEz(N2), cbEz(N2);
  for (size_t c = 0; c < N2; ++c) {
    const double ex = (e11[c] + e12[c] + e13[c]) * kEps0;
    const double ey = (e12[c] + e22[c] + e23[c]) * kEps0;
    const double ez = (e13[c] + e23[c] + e33[c]) * kEps0;
    const double sx = s11[c] + s12[c] + s13[c];
    const double sy = s12[c] + s22[c] + s23[c];
    const double sz = s13[c] + s23[c] + s33[c];
    caEx[c] = (1.0 - sx * dt / (2.0 * ex)) / (1.0 + sx * dt / (2.0 * ex));
    cbEx[c] = (dt / ex) / (1.0 + sx * dt / (2.0 * ex));
    caEy[c] = (1.0 - sy * dt / (2.0 * ey)) / (1.0 + sy * dt / (2.0 * ey));
    cbEy[c] = (dt / ey) / (1.0 + sy * dt / (2.0 * ey));
    caEz[c] = (1.0 - sz * dt / (2.0 * ez)) / (1.0 + sz * dt / (2.0 * ez));
    cbEz[c] = (dt / ez) / (1.0 + sz * dt / (2.0 * ez));
  }
  const double dbH = dt / kMu0;  // daH = 1, :779-789
  const double *srcx = src, *srcy = src + nstep_src, *srcz = src + 2 * nstep_src;
  *blew_up = 0;
  double runmax = 0.0;

  for (int s = 0; s < nsteps; ++s) {
    const int t = it0 + s;
    // Hx, :901-919.
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= NZ - 2; ++k)
      for (int i = 0; i <= NX - 2; ++i)
        for (int j = 0; j <= NY - 2; ++j) {
          const size_t c = I(i, j, k);
          double dEz_dy = (Ez[c] - Ez[I(i, j + 1, k)]) / dy;
          mEz_y[c] = Y.bh[j] * mEz_y[c] + Y.ah[j] * dEz_dy;
          dEz_dy = dEz_dy / Y.Kh[j] + mEz_y[c];
          double dEy_dz = (Ey[I(i, j, k + 1)] - Ey[c]) / dz;
          mEy_z[c] = Z.bh[k] * mEy_z[c] + Z.ah[k] * dEy_dz;
          dEy_dz = dEy_dz / Z.Kh[k] + mEy_z[c];
          Hx[c] = Hx[c] + dbH * (dEy_dz + dEz_dy);
        }
    // Hy, :922-940.
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= NZ - 2; ++k)
      for (int i = 0; i <= NX - 2; ++i)
        for (int j = 0; j <= NY - 2; ++j) {
          const size_t c = I(i, j, k);
          double dEx_dz = (Ex[c] - Ex[I(i, j, k + 1)]) / dz;
          mEx_z[c] = Z.b[k] * mEx_z[c] + Z.a[k] * dEx_dz;
          dEx_dz = dEx_dz / Z.K[k] + mEx_z[c];
          double dEz_dx = (Ez[I(i + 1, j, k)] - Ez[c]) / dx;
          mEz_x[c] = X.b[i] * mEz_x[c] + X.a[i] * dEz_dx;
          dEz_dx = dEz_dx / X.K[i] + mEz_x[c];
          Hy[c] = Hy[c] + dbH * (dEz_dx + dEx_dz);
        }
    // Hz, :943-962.
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= NZ - 2; ++k)
      for (int i = 0; i <= NX - 2; ++i)
        for (int j = 0; j <= NY - 2; ++j) {
          const size_t c = I(i, j, k);
          double dEx_dy = (Ex[I(i, j + 1, k)] - Ex[c]) / dy;
          mEx_y[c] = Y.b[j] * mEx_y[c] + Y.a[j] * dEx_dy;
          dEx_dy = dEx_dy / Y.K[j] + mEx_y[c];
          double dEy_dx = (Ey[c] - Ey[I(i + 1, j, k)]) / dx;
          mEy_x[c] = X.b[i] * mEy_x[c] + X.a[i] * dEy_dx;
          dEy_dx = dEy_dx / X.K[i] + mEy_x[c];
          Hz[c] = Hz[c] + dbH * (dEy_dx + dEx_dy);
        }
    // Ex then Ey inside one k loop, :968-1009.
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= NZ - 2; ++k) {
      for (int i = 0; i <= NX - 2; ++i)
        for (int j = 1; j <= NY - 2; ++j) {
          const size_t c = I(i, j, k);
          double dHz_dy = (Hz[c] - Hz[I(i, j - 1, k)]) / dy;
          mHz_y[c] = Y.bh[j] * mHz_y[c] + Y.ah[j] * dHz_dy;
          dHz_dy = dHz_dy / Y.Kh[j] + mHz_y[c];
          double dHy_dz = (Hy[I(i, j, k - 1)] - Hy[c]) / dz;
          mHy_z[c] = Z.b[k] * mHy_z[c] + Z.a[k] * dHy_dz;
          dHy_dz = dHy_dz / Z.K[k] + mHy_z[c];
          Ex[c] = caEx[P(i, k)] * Ex[c] + cbEx[P(i, k)] * (dHz_dy + dHy_dz);
        }
      for (int i = 1; i <= NX - 2; ++i)
        for (int j = 0; j <= NY - 2; ++j) {
          const size_t c = I(i, j, k);
          double dHz_dx = (Hz[I(i - 1, j, k)] - Hz[c]) / dx;
          mHz_x[c] = X.bh[i] * mHz_x[c] + X.ah[i] * dHz_dx;
          dHz_dx = dHz_dx / X.Kh[i] + mHz_x[c];
          double dHx_dz = (Hx[c] - Hx[I(i, j, k - 1)]) / dz;
          mHx_z[c] = Z.bh[k] * mHx_z[c] + Z.ah[k] * dHx_dz;
          dHx_dz = dHx_dz / Z.Kh[k] + mHx_z[c];
          Ey[c] = ((4 * caEy[P(i, k)] + caEy[P(i - 1, k)] + caEy[P(i, k - 1)]) / 6) * Ey[c] +
                  ((4 * cbEy[P(i, k)] + cbEy[P(i - 1, k)] + cbEy[P(i, k - 1)]) / 6) * (dHz_dx + dHx_dz);
        }
    }
    // Ez, :1012-1029.
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= NZ - 2; ++k)
      for (int i = 1; i <= NX - 2; ++i)
        for (int j = 1; j <= NY - 2; ++j) {
          const size_t c = I(i, j, k);
          double dHx_dy = (Hx[I(i, j - 1, k)] - Hx[c]) / dy;
          mHx_y[c] = Y.bh[j] * mHx_y[c] + Y.ah[j] * dHx_dy;
          dHx_dy = dHx_dy / Y.Kh[j] + mHx_y[c];
          double dHy_dx = (Hy[c] - Hy[I(i - 1, j, k)]) / dx;
          mHy_x[c] = X.bh[i] * mHy_x[c] + X.ah[i] * dHy_dx;
          dHy_dx = dHy_dx / X.Kh[i] + mHy_x[c];
          Ez[c] = ((4 * caEz[P(i, k)] + caEz[P(i - 1, k)] + caEz[P(i, k + 1)]) / 6) * Ez[c] +
                  ((4 * cbEz[P(i, k)] + cbEz[P(i - 1, k)] + cbEz[P(i, k + 1)]) / 6) * (dHx_dy + dHy_dx);
        }
    // Source, :1033-1035.
    {
      const size_t c = I(isrc, jsrc, ksrc);
      Ex[c] = Ex[c] + srcx[t] * dt / e11[P(isrc, ksrc)];
      Ey[c] = Ey[c] + srcy[t] * dt / e22[P(isrc, ksrc)];
      Ez[c] = Ez[c] + srcz[t] * dt / e33[P(isrc, ksrc)];
    }
    // Dirichlet faces, :1038-1078.  Each field zeroes its first plane on
    // every axis and its last valid plane (N-1 or N-2 in 0-based terms).
    auto zero_faces = [&](double* f, int lx, int ly, int lz) {
      for (int k = 0; k < NZ; ++k)
        for (int j = 0; j < NY; ++j) { f[I(0, j, k)] = 0; f[I(lx, j, k)] = 0; }
      for (int k = 0; k < NZ; ++k)
        for (int i = 0; i < NX; ++i) { f[I(i, 0, k)] = 0; f[I(i, ly, k)] = 0; }
      for (int j = 0; j < NY; ++j)
        for (int i = 0; i < NX; ++i) { f[I(i, j, 0)] = 0; f[I(i, j, lz)] = 0; }
    };
    zero_faces(Ex, NX - 2, NY - 1, NZ - 1);
    zero_faces(Ey, NX - 1, NY - 2, NZ - 1);
    zero_faces(Ez, NX - 1, NY - 1, NZ - 2);
    zero_faces(Hx, NX - 1, NY - 2, NZ - 2);
    zero_faces(Hy, NX - 2, NY - 1, NZ - 2);
    zero_faces(Hz, NX - 2, NY - 2, NZ - 1);
    // Stability check, :1081-1082.
    double mx = 0.0;
#pragma omp parallel for reduction(max : mx) schedule(static)
    for (size_t c = 0; c < N; ++c) mx = std::max(mx, std::sqrt(Ex[c] * Ex[c] + Ey[c] * Ey[c] + Ez[c] * Ez[c]));
    runmax = std::max(runmax, mx);
    for (int r = 0; r < nrec; ++r) {
      const size_t c = I(rec[3 * r], rec[3 * r + 1], rec[3 * r + 2]);
      traces[((size_t)s * 3 + 0) * nrec + r] = Ex[c];
      traces[((size_t)s * 3 + 1) * nrec + r] = Ey[c];
      traces[((size_t)s * 3 + 2) * nrec + r] = Ez[c];
    }
    if (!(mx <= kStability)) { *blew_up = 1; *maxnorm = runmax; return s + 1; }
  }
  *maxnorm = runmax;
  return nsteps;
}

int orc_num_threads(void) {
#ifdef _OPENMP
  extern int omp_get_max_threads(void);
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
