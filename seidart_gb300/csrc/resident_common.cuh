// Device helpers shared by the on-chip (SM-resident) electromag2 kernels:
// the tagged edge words exchanged between tiles through L2, the bounded wait
// for a neighbour's words, and the per-cell mask layout.  Everything here has
// internal linkage, so each translation unit that includes it gets its own copy.
#pragma once
#include "fused2d.cuh"
#include "resident.h"

namespace sfd {
namespace res {
namespace {

__device__ __forceinline__ unsigned long long res_timer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void ll_put4(uint2* p, float4 v, unsigned tag) {
  asm volatile("st.volatile.global.v4.u32 [%0], {%1, %2, %3, %4};" ::"l"(p), "r"(__float_as_uint(v.x)), "r"(tag),
               "r"(__float_as_uint(v.y)), "r"(tag));
  asm volatile("st.volatile.global.v4.u32 [%0], {%1, %2, %3, %4};" ::"l"(p + 2), "r"(__float_as_uint(v.z)),
               "r"(tag), "r"(__float_as_uint(v.w)), "r"(tag));
}

__device__ __forceinline__ void ll_put1(uint2* p, float v, unsigned tag) {
  asm volatile("st.volatile.global.v2.u32 [%0], {%1, %2};" ::"l"(p), "r"(__float_as_uint(v)), "r"(tag));
}

__device__ __forceinline__ uint4 ld_vol4(const uint2* p) {
  uint4 r;
  asm volatile("ld.volatile.global.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "l"(p));
  return r;
}

__device__ __forceinline__ uint2 ld_vol2(const uint2* p) {
  uint2 r;
  asm volatile("ld.volatile.global.v2.u32 {%0, %1}, [%2];" : "=r"(r.x), "=r"(r.y) : "l"(p));
  return r;
}

// Called every few unsuccessful polls: false once the limit has passed or
// any tile has given up.
__device__ __noinline__ bool keep_polling(Ctl* ctl, unsigned long long limit_ns, unsigned long long& t0) {
  const unsigned long long now = res_timer_ns();
  if (t0 == 0) t0 = now;
  if (*(volatile int*)&ctl->err) return false;
  if (now - t0 > limit_ns) {
    atomicExch(&ctl->err, 1);
    return false;
  }
  return true;
}

// One warp: copy `nrow` row words (rsrc) into rdst[q] and `ncol` column words
// (csrc) into cdst[c * cstride], each once its tag reads `tag`.  Each lane
// issues the loads of all its pending words before testing any, so one round
// trip to L2 serves them all.  At most 32 * kResFetchPerLane words.  False
// (on every lane) if a wait gave up.
constexpr int kResFetchPerLane = 8;
__device__ __noinline__ bool fetch_edges(const uint2* rsrc, float* rdst, int nrow, const uint2* csrc, float* cdst, int cstride,
                            int ncol, unsigned tag, Ctl* ctl, unsigned long long limit_ns) {
  const int lane = threadIdx.x & 31;
  const int n = nrow + ncol;
  unsigned pending = 0;
#pragma unroll
  for (int k = 0; k < kResFetchPerLane; ++k)
    if (lane + 32 * k < n) pending |= 1u << k;
  bool ok = true;
  unsigned long long t0 = 0;
  uint2 v[kResFetchPerLane];
  for (int it = 1; pending; ++it) {
#pragma unroll
    for (int k = 0; k < kResFetchPerLane; ++k) {
      const int q = lane + 32 * k;
      if (pending & (1u << k)) v[k] = ld_vol2(q < nrow ? rsrc + q : csrc + (q - nrow));
    }
#pragma unroll
    for (int k = 0; k < kResFetchPerLane; ++k) {
      const int q = lane + 32 * k;
      if ((pending & (1u << k)) && v[k].y == tag) {
        if (q < nrow) rdst[q] = __uint_as_float(v[k].x);
        else cdst[(q - nrow) * cstride] = __uint_as_float(v[k].x);
        pending &= ~(1u << k);
      }
    }
    if (pending && (it & 7) == 0 && !keep_polling(ctl, limit_ns, t0)) {
      ok = false;
      break;
    }
  }
  return __all_sync(0xffffffffu, ok);
}

__device__ __forceinline__ float4 lds4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void sts4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float2 lds2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ void sts2(float* p, float2 v) { *reinterpret_cast<float2*>(p) = v; }
__device__ __forceinline__ float2 ld2(const float* p) { return __ldg(reinterpret_cast<const float2*>(p)); }
__device__ __forceinline__ float& el2(float2& v, int q) { return (&v.x)[q]; }
__device__ __forceinline__ float el2(const float2& v, int q) { return (&v.x)[q]; }

// Per-cell masks of a thread, four bits each (bit e = cell 4tx+e), fixed for
// the run and packed in one word.
enum : unsigned {
  kMH = 0,     // Hy is updated (:249-262: i <= NX-2, k <= NZ-2)
  kMEX = 4,    // Ex is updated (:273-283: i <= NX-2, 1 <= k <= NZ-2)
  kMEZ = 8,    // Ez is updated (:285-295: 1 <= i <= NX-2, k <= NZ-2)
  kMEXZ = 12,  // Ex is a Dirichlet plane (:304-312)
  kMEZZ = 16,  // Ez is a Dirichlet plane
  kMHYZ = 20,  // the stored Hy is a Dirichlet plane (:314-317)
  kMCELL = 24  // i < NX
};
__device__ __forceinline__ bool mbit(unsigned m, unsigned field, int e) { return (m >> (field + e)) & 1u; }

// Threads take the tile's groups (four columns x kResRows rows) in the order
// of their class, 0 .. NC - 1 (the kernels order the groups by update path,
// so each warp runs one path instead of several in turn).  Every thread of
// the CTA calls this with the class of group tid (NC when tid has no group)
// and gets the group it owns (-1: none).  Contains barriers.
template <int NC>
__device__ __noinline__ int class_ordered_group(int cls) {
  __shared__ int s_cnt[kResThreads / 32][NC];
  __shared__ unsigned short s_map[kResCellThreads];
  const int tid = threadIdx.x;
  const unsigned lane = tid & 31, warp = tid >> 5;
  unsigned mine = 0;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const unsigned b = __ballot_sync(0xffffffffu, cls == c);
    if (lane == 0) s_cnt[warp][c] = __popc(b);
    if (cls == c) mine = __popc(b & ((1u << lane) - 1u));
  }
  __syncthreads();
  if (tid == 0) {
    int run = 0;
    for (int c = 0; c < NC; ++c)
      for (int w = 0; w < kResThreads / 32; ++w) {  // the warps of this CTA
        const int n = s_cnt[w][c];
        s_cnt[w][c] = run;
        run += n;
      }
  }
  __syncthreads();
  if (cls < NC) s_map[s_cnt[warp][cls] + mine] = (unsigned short)tid;
  __syncthreads();
  return (tid < kResCellThreads && cls < NC) ? s_map[tid] : -1;
}

}  // namespace
}  // namespace res
}  // namespace sfd
