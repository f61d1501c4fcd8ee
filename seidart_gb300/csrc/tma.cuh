// Tensor-memory-access (TMA) tile loads and the shared-memory mbarriers that
// signal their completion (PTX ISA: cp.async.bulk.tensor, mbarrier).
//
// A block stages tiles of global arrays in shared memory: one thread posts
// the expected byte count on a slot's mbarrier and issues the copies; every
// thread waits on the barrier's phase parity before reading the slot.  Waits
// are bounded by %globaltimer so a copy that never lands ends the launch
// with an error flag instead of a hang.
#pragma once
#include <cuda.h>
#include <cstdint>

namespace sfd {
namespace tma {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// The dynamic shared memory of a kernel begins after its static shared
// variables, at whatever offset their sizes leave, whatever alignment the
// extern declaration states.  Staging rings start at the first 128-byte
// boundary of it, and every box of a stage lies on a 128-byte boundary too
// (the alignment a tensor copy's shared-memory destination needs); the
// launches ask for kStageSlack bytes more than the ring.
constexpr int kStageSlack = 128;
__device__ __forceinline__ float* aligned_stage(unsigned char* raw) {
  const uint32_t a = smem_addr(raw);
  return reinterpret_cast<float*>(raw + ((128u - (a & 127u)) & 127u));
}

__device__ __forceinline__ void bar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Makes the barriers' initialisation visible to the asynchronous proxy (the TMA unit).
__device__ __forceinline__ void fence_bar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// Orders this thread's earlier generic-proxy shared-memory accesses before
// later asynchronous-proxy ones (a slot read by the block, then refilled).
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// One arrival that also expects `bytes` more transaction bytes in this phase.
__device__ __forceinline__ void bar_arrive_expect(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool bar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Waits until the phase of parity `parity` of `bar` has completed, at most
// `limit_ns`; false when the limit ran out.
__device__ __forceinline__ bool bar_wait(uint64_t* bar, uint32_t parity, unsigned long long limit_ns) {
  if (bar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = now_ns();
  while (!bar_try_wait(bar, parity))
    if (now_ns() - t0 > limit_ns) return false;
  return true;
}

// 4-D tile load: the box of `map` at coordinates (c0, c1, c2, c3), innermost
// first, into shared memory at `dst` (128-byte aligned); completion counted on
// `bar`.  c0 times the element size must be a multiple of 16 bytes; boxes
// reaching outside the tensor read zeros there.
__device__ __forceinline__ void load_4d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2,
                                        int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5, %6}], "
      "[%2];" ::"r"(smem_addr(dst)),
      "l"(map), "r"(smem_addr(bar)), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
      : "memory");
}

// 2-D tile load, as load_4d.
__device__ __forceinline__ void load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          smem_addr(dst)),
      "l"(map), "r"(smem_addr(bar)), "r"(c0), "r"(c1)
      : "memory");
}

}  // namespace tma
}  // namespace sfd
