// C ABI, part 2: batched runs -- one persistent cooperative launch
// (batch.cu) advancing many 2-D models, each with its own handle.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "handle.h"

using namespace sfd;

struct sfd_batch_s {
  std::vector<sfd_handle*> h;
  char* scratch = nullptr;
  cudaStream_t stream = nullptr;
  int zb = 2, bps = 4, nsm = 0;
  unsigned long long limit_ns = kDefaultWaitNs;  // barrier wait limit
  int stall = 0;  // timeout test aid: the barrier waits for one block more than the launch has
  std::vector<BatchModel> models;
  std::vector<int> steps;
  GridBarrier* bar() const { return (GridBarrier*)scratch; }
  std::vector<BatchGroup> groups;
  int* dsteps() const { return (int*)(scratch + 256); }
  BatchModel* dmodels() const { return (BatchModel*)(scratch + 256 + align256(sizeof(int) * h.size())); }
  BatchGroup* dgroups() const {
    return (BatchGroup*)(scratch + 256 + align256(sizeof(int) * h.size()) + align256(sizeof(BatchModel) * h.size()));
  }
};

namespace {
size_t batch_bytes(int n) {
  return 256 + align256(sizeof(int) * n) + align256(sizeof(BatchModel) * (size_t)n) +
         align256(sizeof(BatchGroup) * (size_t)n);
}

// Models that read the same coefficient planes and have the same geometry.
bool same_group(const sfd_handle* a, const sfd_handle* b) {
  if (a->cfg.kind != b->cfg.kind || a->cfg.nx != b->cfg.nx || a->cfg.nz != b->cfg.nz) return false;
  if (a->cfg.kind == SFD_ELECTROMAG2) return a->em2s[0].CAx == b->em2s[0].CAx;
  return a->s2s[0].A11 == b->s2s[0].A11;
}
}  // namespace

extern "C" {

int32_t sfd_batch_scratch_bytes(int32_t nmodels, size_t* bytes) {
  g_err.clear();
  if (nmodels < 1 || !bytes) return fail(SFD_ERR_BAD_ARG, "need nmodels >= 1 and a bytes pointer");
  *bytes = batch_bytes(nmodels);
  return SFD_OK;
}

int32_t sfd_batch_create(sfd_handle* const* handles, int32_t n, void* dev_scratch, size_t bytes, sfd_batch** out) {
  g_err.clear();
  if (!handles || n < 1 || !out) return fail(SFD_ERR_BAD_ARG, "need handles, n >= 1 and out");
  *out = nullptr;
  if (!dev_scratch || ((uintptr_t)dev_scratch & 255)) return fail(SFD_ERR_BAD_ARG, "scratch must be 256-byte aligned device memory");
  if (bytes < batch_bytes(n)) return fail(SFD_ERR_BAD_ARG, "batch scratch has %zu bytes, needs %zu", bytes, batch_bytes(n));
  for (int m = 0; m < n; ++m) {
    sfd_handle* h = handles[m];
    if (!h) return fail(SFD_ERR_BAD_ARG, "handle %d is NULL", m);
    if (!h->single) return fail(SFD_ERR_BAD_ARG, "handle %d: batches take single-pass 2-D handles (seismic2/electromag2, no SFD_FLAG_TWO_PASS)", m);
    if (!h->have_model || !h->have_cpml) return fail(SFD_ERR_STATE, "handle %d has no model or CPML yet", m);
    if (h->stream != handles[0]->stream) return fail(SFD_ERR_BAD_ARG, "all handles of a batch must share one stream");
    for (int q = 0; q < m; ++q)
      if (handles[q] == h) return fail(SFD_ERR_BAD_ARG, "handle %d appears twice", m);
  }
  int dev = 0;
  CK(cudaGetDevice(&dev));
  sfd_batch* b = new sfd_batch_s();
  b->h.assign(handles, handles + n);
  b->scratch = (char*)dev_scratch;
  b->stream = handles[0]->stream;
  cudaError_t e = cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) { delete b; return cuda_fail(e, "cudaDeviceGetAttribute"); }
  *out = b;
  return SFD_OK;
}

int32_t sfd_batch_set_tiling(sfd_batch* b, int32_t zb, int32_t blocks_per_sm) {
  g_err.clear();
  if (!b) return fail(SFD_ERR_BAD_ARG, "NULL batch");
  if (zb != 1 && zb != 2 && zb != 4) return fail(SFD_ERR_BAD_ARG, "zb must be 1, 2 or 4");
  int maxb = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, batch_kernel_ptr(zb), 256, 0));
  if (blocks_per_sm < 1 || blocks_per_sm > maxb)
    return fail(SFD_ERR_BAD_ARG, "blocks_per_sm must be in [1, %d] for zb=%d", maxb, zb);
  b->zb = zb;
  b->bps = blocks_per_sm;
  return SFD_OK;
}

int32_t sfd_batch_run(sfd_batch* b, int64_t nsteps) {
  g_err.clear();
  if (!b) return fail(SFD_ERR_BAD_ARG, "NULL batch");
  if (nsteps < 0) return fail(SFD_ERR_BAD_ARG, "nsteps must be >= 0");
  if (nsteps == 0) return SFD_OK;
  const int n = (int)b->h.size();
  for (int m = 0; m < n; ++m)
    if (b->h[m]->step + nsteps > b->h[m]->cfg.nstep)
      return fail(SFD_ERR_BAD_ARG, "model %d: run to step %lld exceeds its %d source samples", m,
                  (long long)(b->h[m]->step + nsteps), b->h[m]->cfg.nstep);
  int maxb = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, batch_kernel_ptr(b->zb), 256, 0));
  const int bps = std::min(b->bps, maxb);
  if (bps < 1) return fail(SFD_ERR_CUDA, "batch kernel does not fit on an SM");
  b->models.assign(n, BatchModel());
  b->steps.assign(n, 0);
  for (int m = 0; m < n; ++m) {
    sfd_handle* h = b->h[m];
    BatchModel& md = b->models[m];
    md.kind = h->cfg.kind == SFD_ELECTROMAG2 ? SFD_BATCH_EM2 : SFD_BATCH_SEIS2;
    md.gx = md.kind == SFD_BATCH_EM2 ? (h->cfg.nx + 127) / 128 : (h->cfg.nx + 31) / 32;  // em2 tiles are 128 wide
    const int gy = (h->cfg.nz + 8 * b->zb - 1) / (8 * b->zb);
    md.ntiles = md.gx * gy;
    md.nslots = md.ntiles;
    md.cur = h->cur;
    md.em2[0] = h->em2s[0];
    md.em2[1] = h->em2s[1];
    md.s2[0] = h->s2s[0];
    md.s2[1] = h->s2s[1];
    b->steps[m] = (int)h->step;
  }
  b->groups.clear();
  int tile0 = 0;
  for (int m = 0; m < n;) {
    int e = m + 1;
    while (e < n && same_group(b->h[m], b->h[e])) ++e;
    BatchGroup g;
    g.first = m;
    g.n = e - m;
    g.tile0 = tile0;
    g.ntiles = g.n * b->models[m].ntiles;
    tile0 += g.ntiles;
    b->groups.push_back(g);
    m = e;
  }
  const int total = tile0;
  const int grid = std::max(1, std::min(total, bps * b->nsm));
  CK(cudaMemcpyAsync(b->dsteps(), b->steps.data(), sizeof(int) * n, cudaMemcpyHostToDevice, b->stream));
  CK(cudaMemcpyAsync(b->dmodels(), b->models.data(), sizeof(BatchModel) * n, cudaMemcpyHostToDevice, b->stream));
  CK(cudaMemcpyAsync(b->dgroups(), b->groups.data(), sizeof(BatchGroup) * b->groups.size(), cudaMemcpyHostToDevice,
                     b->stream));
  batch_begin(b->dmodels(), n, b->dsteps(), b->bar(), b->stream);
  CK(batch_launch(b->zb, grid, b->dmodels(), b->dgroups(), (int)b->groups.size(), total, (int)nsteps, b->bar(),
                  b->limit_ns, b->stall, b->stream));
  batch_end(b->dmodels(), n, (int)nsteps, b->stream);
  CK(cudaGetLastError());
  for (sfd_handle* h : b->h) {
    h->step += nsteps;
    h->cur ^= (int)(nsteps & 1);
  }
  return SFD_OK;
}

int32_t sfd_batch_set_wait_limit(sfd_batch* b, int64_t ns) {
  g_err.clear();
  if (!b) return fail(SFD_ERR_BAD_ARG, "NULL batch");
  if (ns < 0) return fail(SFD_ERR_BAD_ARG, "wait limit must be >= 0 ns (0 = the default 2 s)");
  b->limit_ns = ns == 0 ? kDefaultWaitNs : (unsigned long long)ns;
  return SFD_OK;
}

int32_t sfd_batch_test_stall_waits(sfd_batch* b, int32_t on) {
  g_err.clear();
  if (!b) return fail(SFD_ERR_BAD_ARG, "NULL batch");
  b->stall = on ? 1 : 0;
  return SFD_OK;
}

int32_t sfd_batch_status(sfd_batch* b, int32_t* failed_model) {
  g_err.clear();
  if (!b) return fail(SFD_ERR_BAD_ARG, "NULL batch");
  if (failed_model) *failed_model = -1;
  GridBarrier bar;
  CK(cudaMemcpyAsync(&bar, b->bar(), sizeof bar, cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  if (bar.err) return fail(SFD_ERR_TIMEOUT, "grid barrier of the batched kernel timed out");
  for (size_t m = 0; m < b->h.size(); ++m) {
    int r = sfd_status(b->h[m], nullptr, nullptr);
    if (r != SFD_OK) {
      if (failed_model) *failed_model = (int32_t)m;
      return r;
    }
  }
  return SFD_OK;
}

int32_t sfd_batch_destroy(sfd_batch* b) {
  g_err.clear();
  if (!b) return SFD_OK;
  cudaStreamSynchronize(b->stream);
  delete b;
  return SFD_OK;
}

}  // extern "C"
