// Input assembly on the device: source time functions and CPML profiles,
// formed in FP64 and stored in the FP32 forms the step kernels read.
//
// Source wavelets follow the driver's `wavelet`
// (src/seidart/routines/sourcefunction.py:25-57) on its time vector
// `arange(N) * dt` (:262), peak-normalised, times the amplitude and the
// per-component factor (:276-300: R[., 2] * srcfn for the 'ac' forces, the
// moment-tensor entries for stress sources).  The CPML profiles follow the
// driver's cpml_parameters along an edge (src/seidart/routines/
// definitions.py:862-998) or the legacy writer (legacy/prjrun_101424.py:
// 174-303), as the host builder seidart_gb300/cpml.py does.  Every product
// and sum is written with round-to-nearest intrinsics in the host
// formulas' order, so no multiply-add is contracted and the FP64 values
// differ from the host's only where exp and pow do.
#include "seidart_gb300.h"
#include "sfd_solvers.h"

namespace sfd {

namespace {

constexpr double kPi = 3.141592653589793;  // numpy.pi
constexpr double kEps0 = 8.85418782e-12;   // definitions.py:68

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

// x(t) of sourcefunction.py:31-43 before the peak normalisation.
__device__ double wave(int stype, double f, double t) {
  const double to = 1.0 / f;
  if (stype == SFD_WAVELET_GAUS0) {
    const double bw = 0.2 / mul(kPi, f);
    const double a = sub(t, to) / bw;
    return exp(mul(-a, a));
  }
  if (stype == SFD_WAVELET_GAUS1) {
    const double a = mul(mul(kPi, f), sub(t, to));
    const double e = exp(mul(-a, a));
    return mul(sub(1.0, mul(mul(2.0, a), a)), e);
  }
  const double d = sub(t, to);  // gaus2
  const double k = mul(mul(mul(kPi, kPi), f), f);
  const double e = exp(mul(mul(-k, d), d));
  const double k2d = mul(mul(2.0, k), d);
  return mul(mul(k2d, sub(mul(k2d, d), 3.0)), e);
}

// One block: the peak |x| over the nstep samples, then out[q * stride + t] =
// (float)(((comp[q] * (amp * (x / peak))) * dt) / div[q]).
__global__ void __launch_bounds__(1024) k_wavelet(int stype, double f0, double dt, int nstep, double amp,
                                                  WaveletComp wc, float* out, size_t stride) {
  __shared__ double part[32];
  double m = 0.0;
  for (int t = threadIdx.x; t < nstep; t += blockDim.x) m = fmax(m, fabs(wave(stype, f0, mul((double)t, dt))));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) part[0] = m;
  }
  __syncthreads();
  const double peak = part[0];
  for (int t = threadIdx.x; t < nstep; t += blockDim.x) {
    const double s = mul(amp, wave(stype, f0, mul((double)t, dt)) / peak);
    for (int q = 0; q < wc.n; ++q) out[q * stride + t] = __double2float_rn(mul(mul(wc.comp[q], s), dt) / wc.div[q]);
  }
}

// One axis: the full- and half-offset profiles of cpml.py's _profile_1d and
// their FP32 table (1 / (delta K), a / delta, b, the same at the half
// offset), rows of `st` floats; the interior keeps K = 1, a = 0 and b = 1
// (driver) or 0 (legacy).
__global__ void k_cpml_axis(CpmlAxisArgs p, float* tab, int st) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const int ind = i < p.npml ? i : (i >= p.n - p.npml ? p.n - 1 - i : -1);
  const double scale = p.seismic ? p.dt : p.dt / kEps0;
  const double dn = mul(p.delta, (double)p.npml);
  for (int h = 0; h < 2; ++h) {
    double K = 1.0, a = 0.0, b = p.legacy ? 0.0 : 1.0;
    if (ind >= 0) {
      double dist = mul(p.delta, (double)ind);
      if (h) dist = add(dist, p.delta / 2.0);
      dist = sub(dn, dist) / dn;
      if (!p.legacy) {  // rescaled so that the largest distance (index 0) is 1
        const double d0 = h ? sub(dn, p.delta / 2.0) / dn : sub(dn, 0.0) / dn;
        dist = dist / d0;
      }
      const double pw = pow(dist, p.NP);
      const double sigma = mul(p.sig_max, pw);
      K = add(1.0, mul(sub(p.kappa_max, 1.0), pw));
      double alpha = mul(p.alpha_max, pow(sub(1.0, dist), p.NPA));
      b = exp(mul(-add(sigma / K, alpha), scale));
      if (alpha < 0.0) alpha = 0.0;
      if (fabs(sigma) > 1.0e-6) a = mul(sigma, sub(b, 1.0)) / add(mul(K, sigma), mul(K, alpha));
    }
    tab[(3 * h) * st + i] = __double2float_rn(1.0 / mul(p.delta, K));
    tab[(3 * h + 1) * st + i] = __double2float_rn(a / p.delta);
    tab[(3 * h + 2) * st + i] = __double2float_rn(b);
  }
}

// seismicfdtd.f95:255 reads b_x_half at the z index: q3[k] = b_x_half(k)
// for k < NX, else 0.
__global__ void k_cpml_q3(const float* bxh, int nx, int nz, float* q3) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nz) q3[k] = k < nx ? bxh[k] : 0.0f;
}

}  // namespace

cudaError_t wavelet_launch(int stype, double f0, double dt, int nstep, double amp, const WaveletComp& wc, float* out,
                           size_t stride, cudaStream_t s) {
  k_wavelet<<<1, 1024, 0, s>>>(stype, f0, dt, nstep, amp, wc, out, stride);
  return cudaGetLastError();
}

cudaError_t cpml_axis_launch(const CpmlAxisArgs& p, float* tab, int st, cudaStream_t s) {
  k_cpml_axis<<<(p.n + 255) / 256, 256, 0, s>>>(p, tab, st);
  return cudaGetLastError();
}

cudaError_t cpml_q3_launch(const float* bxh, int nx, int nz, float* q3, cudaStream_t s) {
  k_cpml_q3<<<(nz + 255) / 256, 256, 0, s>>>(bxh, nx, nz, q3);
  return cudaGetLastError();
}

}  // namespace sfd
