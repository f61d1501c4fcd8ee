// Batched time stepping: many 2-D models (electromag2 shots, seismic2 models
// of uneven size) advance together in ONE persistent cooperative launch.
//
// Work list: every model is cut into the tiles of its single-pass
// step (fused2d.cuh); the tiles of all models are numbered consecutively,
// group by group (BatchGroup: shots sharing a model interleave their tiles).  Each time step, block b
// processes tiles b, b + G, b + 2G, ... with the tile bodies of the per-model
// kernels, then all blocks meet at a grid barrier before the next step.  A
// model's step reads the ping-pong copy p = (cur + s) & 1 and writes the
// other, so the barrier is the only synchronisation.  The tile bodies read
// the fields with coherent loads here (RO = false): a field read through the
// read-only path must not be written during the launch, and this launch
// writes every field in its earlier steps.
//
// The barrier spins on a generation counter with a time limit
// (%globaltimer); on expiry it records an error that the host reads
// (SFD_ERR_TIMEOUT) and every block leaves the kernel.  The launch is
// cooperative, so all blocks are co-resident and the limit is never reached
// in a correct run.
#include "batch.h"
#include "fused2d.cuh"

namespace sfd {

namespace {

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Returns false if the barrier timed out or another block reported a failure.
__device__ bool grid_barrier(GridBarrier* bar, unsigned nblocks, unsigned long long limit_ns) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    ok = 1;
    volatile unsigned* vgen = &bar->gen;
    volatile int* verr = &bar->err;
    const unsigned g = *vgen;
    __threadfence();
    if (atomicAdd(&bar->count, 1u) == nblocks - 1) {
      atomicExch(&bar->count, 0u);
      __threadfence();
      atomicAdd(&bar->gen, 1u);
    } else {
      const unsigned long long t0 = globaltimer_ns();
      while (*vgen == g) {
        if (*verr) { ok = 0; break; }
        if (globaltimer_ns() - t0 > limit_ns) {
          atomicExch(&bar->err, 1);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  __threadfence();  // orders this block's later (coherent) field loads after the other blocks' writes
  return ok != 0;
}

template <int ZB>
__global__ void __launch_bounds__(256, 3)
    batch_kernel(const BatchModel* __restrict__ models, const BatchGroup* __restrict__ groups, int ngroups,
                 int total_tiles, int nsteps, GridBarrier* bar, unsigned long long limit_ns, int extra) {
  __shared__ __align__(16) union {
    float em2[8 * ZB + 1][kEm2Row];
    float s2[3][8 * ZB + 2][34];
  } sm;
  for (int s = 0; s < nsteps; ++s) {
    int g = 0;
    for (int tile = blockIdx.x; tile < total_tiles; tile += gridDim.x) {
      while (g + 1 < ngroups && tile >= groups[g + 1].tile0) ++g;  // tiles ascend per block
      const BatchGroup& gr = groups[g];
      const int q = tile - gr.tile0;
      const BatchModel& md = models[gr.first + q % gr.n];
      const int lt = q / gr.n;
      const int bx = lt % md.gx, by = lt / md.gx;
      const int p = (md.cur + s) & 1;
      if (md.kind == SFD_BATCH_EM2) {
        const Em2Step& a = md.em2[p];
        em2_tile<ZB, false>(a, a.io.ctl->base + s, bx, by, md.gx, sm.em2);
      } else {
        const Seis2Step& a = md.s2[p];
        seis2_tile<ZB, false>(a, a.io.ctl->base + s, bx, by, md.gx, sm.s2);
      }
      __syncthreads();  // shared tile buffers are reused by the next tile
    }
    if (!grid_barrier(bar, gridDim.x + extra, limit_ns)) return;
  }
}

__global__ void batch_begin_kernel(const BatchModel* models, int nmodels, const int* steps, GridBarrier* bar) {
  for (int m = blockIdx.x; m < nmodels; m += gridDim.x) {
    const BatchModel& md = models[m];
    const IoArgs& io = (md.kind == SFD_BATCH_EM2) ? md.em2[0].io : md.s2[0].io;
    for (int q = threadIdx.x; q < md.nslots; q += blockDim.x) io.slots[q] = 0.0f;
    if (threadIdx.x == 0) {
      io.ctl->base = steps[m];
      io.ctl->run_start = steps[m];
      io.ctl->maxnorm = 0.0f;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    bar->count = 0;
    bar->gen = 0;
    bar->err = 0;
  }
}

// Receivers of the last step (from the copy that is current after the run)
// and the run norm of every model.
__global__ void batch_end_kernel(const BatchModel* models, int nmodels, int nsteps) {
  for (int m = blockIdx.x; m < nmodels; m += gridDim.x) {
    const BatchModel& md = models[m];
    const int p = (md.cur + nsteps) & 1;
    const IoArgs& io = (md.kind == SFD_BATCH_EM2) ? md.em2[p].io : md.s2[p].io;
    const int t_last = io.ctl->base + nsteps - 1;
    if (md.kind == SFD_BATCH_EM2) {
      const float* ch[2] = {md.em2[p].Ex0, md.em2[p].Ez0};
      gather_receivers<2>(io.rec, io.nrec, io.traces, t_last, ch, md.em2[p].P, 1, false);
    } else {
      const float* ch[2] = {md.s2[p].vx0, md.s2[p].vz0};
      gather_receivers<2>(io.rec, io.nrec, io.traces, t_last, ch, md.s2[p].P, 1, false);
    }
    float mx = 0.0f;
    for (int q = threadIdx.x; q < md.nslots; q += blockDim.x) mx = fmaxf(mx, io.slots[q]);
    __shared__ float red[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
      float r = 0.0f;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = fmaxf(r, red[w]);
      io.ctl->maxnorm = r;
    }
    __syncthreads();
  }
}

}  // namespace

const void* batch_kernel_ptr(int zb) {
  switch (zb) {
    case 1: return (const void*)batch_kernel<1>;
    case 2: return (const void*)batch_kernel<2>;
    default: return (const void*)batch_kernel<4>;
  }
}

void batch_begin(const BatchModel* models, int nmodels, const int* steps, GridBarrier* bar, cudaStream_t s) {
  batch_begin_kernel<<<std::min(nmodels, 1024), 256, 0, s>>>(models, nmodels, steps, bar);
}

void batch_end(const BatchModel* models, int nmodels, int nsteps, cudaStream_t s) {
  batch_end_kernel<<<std::min(nmodels, 1024), 256, 0, s>>>(models, nmodels, nsteps);
}

cudaError_t batch_launch(int zb, int grid, const BatchModel* models, const BatchGroup* groups, int ngroups,
                         int total_tiles, int nsteps, GridBarrier* bar, unsigned long long limit_ns, int extra,
                         cudaStream_t s) {
  void* args[] = {(void*)&models, (void*)&groups, (void*)&ngroups, (void*)&total_tiles, (void*)&nsteps,
                  (void*)&bar, (void*)&limit_ns, (void*)&extra};
  return cudaLaunchCooperativeKernel(batch_kernel_ptr(zb), dim3(grid), dim3(32, 8), args, 0, s);
}

}  // namespace sfd
