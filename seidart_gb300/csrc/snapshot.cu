// Block-floating snapshot encoding of one field on the device.
//
// The reference's 2.5-D EM output stores each field of each saved step as
// signed 16-bit integers with the field's min and max (the SEIDART_EM25B1
// block files read by src/seidart/routines/definitions.py:140-212): a value
// v is stored as raw with (raw + 32767) / 65534 = (v - min) / (max - min).
// Encoding on the device halves the bytes that cross to the host.  Two
// kernels on the handle's stream: a min/max reduction into minmax[0..1],
// then the encoding into a dense x-fastest int16 array (no row padding).
#include <algorithm>

#include "sfd_solvers.h"

namespace sfd {

namespace {

// Ordered float atomics: the bit patterns of non-negative floats order like
// signed ints, those of negative floats order in reverse like unsigned ints.
__device__ __forceinline__ void atomic_min_float(float* a, float v) {
  if (v >= 0.0f) atomicMin(reinterpret_cast<int*>(a), __float_as_int(v));
  else atomicMax(reinterpret_cast<unsigned*>(a), __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_float(float* a, float v) {
  if (v >= 0.0f) atomicMax(reinterpret_cast<int*>(a), __float_as_int(v));
  else atomicMin(reinterpret_cast<unsigned*>(a), __float_as_uint(v));
}

__global__ void minmax_init_kernel(float* mm) {
  mm[0] = __int_as_float(0x7f800000);   // +inf
  mm[1] = __int_as_float(0xff800000);   // -inf
}

// rows = NY * NZ rows of NX values, pitch P.  NaNs are skipped.
__global__ void __launch_bounds__(256) minmax_kernel(const float* __restrict__ f, int NX, int P, long rows,
                                                     float* mm) {
  float lo = __int_as_float(0x7f800000), hi = __int_as_float(0xff800000);
  const long n = rows * NX;
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
    const long r = q / NX;
    const float v = __ldg(f + r * P + (q - r * NX));
    lo = fminf(lo, v);
    hi = fmaxf(hi, v);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  __shared__ float slo[8], shi[8];
  if ((threadIdx.x & 31) == 0) {
    slo[threadIdx.x >> 5] = lo;
    shi[threadIdx.x >> 5] = hi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      lo = fminf(lo, slo[w]);
      hi = fmaxf(hi, shi[w]);
    }
    if (lo <= hi) {  // the block saw at least one number
      atomic_min_float(mm, lo);
      atomic_max_float(mm + 1, hi);
    }
  }
}

__global__ void __launch_bounds__(256) encode_kernel(const float* __restrict__ f, int NX, int P, long rows,
                                                     const float* __restrict__ mm, short* __restrict__ out) {
  const float lo = mm[0], hi = mm[1];
  const float scale = hi > lo ? 65534.0f / (hi - lo) : 0.0f;
  const long n = rows * NX;
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
    const long r = q / NX;
    const float v = __ldg(f + r * P + (q - r * NX));
    int raw = 0;
    if (scale > 0.0f) raw = __float2int_rn(fminf(fmaxf((v - lo) * scale, 0.0f), 65534.0f)) - 32767;
    out[q] = (short)raw;
  }
}

}  // namespace

void encode_field_i16(const float* field, int NX, int P, long rows, short* out, float* minmax, cudaStream_t s) {
  const long n = rows * NX;
  const int blocks = (int)std::min<long>(4 * 152, (n + 255) / 256);
  minmax_init_kernel<<<1, 1, 0, s>>>(minmax);
  minmax_kernel<<<blocks, 256, 0, s>>>(field, NX, P, rows, minmax);
  encode_kernel<<<blocks, 256, 0, s>>>(field, NX, P, rows, minmax, out);
}

}  // namespace sfd
