// One electromag2 shot for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: code running inside a
// host application that owns every device allocation and exposes no
// allocator, a plugin loaded into a process whose memory policy forbids new
// device allocations, or an embedding where allocation would break a memory
// budget fixed in advance.  sfd_electromag2_run_static serves them: it keeps
// the whole device state of the shot (fields, CPML memory, coefficients, axis
// tables, source, receivers, traces, norm slots) in one file-scope device
// array of fixed size, so the call allocates nothing.  The caller passes its
// inputs and receives its outputs in host memory.
//
// The shot runs the two-pass electromag2 form (one kernel per half-step,
// fields updated in place), the one that needs a single copy of the state:
// config flags other than 0 or SFD_FLAG_TWO_PASS are rejected.
//
// The array is 32 MiB.  Every GPU that loads this library holds it until the
// process exits.  The library is built without relocatable device code, so
// this file is its own CUDA module; under the runtime's default lazy module
// loading the module, and with it the 32 MiB, is loaded on a device at the
// first call there (at library load only with CUDA_MODULE_LOADING=EAGER).
// That first call can therefore fail with SFD_ERR_CUDA when the device has no
// 32 MiB left: a caller with a fixed device-memory budget should make one
// early call (a tiny shot) before it commits the rest of its memory.  A
// configuration whose state does not fit is rejected with
// SFD_ERR_BAD_ARG.  Every call shares the one array and keeps whatever the
// previous call left in it, so each call clears the whole state first;
// calls whose GPU work overlaps (several host threads, or streams that are
// not serialised) race on the array and must not be issued.  The first call
// on a device looks up the array's device address (cudaGetSymbolAddress) with
// that device current; make that first call before any stream capture.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/seidart_gb300.h"
#include "sfd_solvers.h"

namespace {

constexpr size_t kStaticScratchBytes = size_t(32) << 20;  // 32 MiB
constexpr int kMaxDevices = 64;

// In host code this name is a host-side stand-in, not a device address: the
// device address comes from cudaGetSymbolAddress below.
__device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_static_mu;
void* g_static_addr[kMaxDevices] = {};

int32_t fail_static(int32_t code, const char* msg) {
  sfd::set_error(msg);
  return code;
}

// Device address of the scratch array on the current device (looked up once per device).
cudaError_t static_scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_static_mu);
  if (!g_static_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return e;
    g_static_addr[dev] = p;
  }
  *out = g_static_addr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" int32_t sfd_electromag2_run_static(const sfd_config* cfg, const double* model, const double* profiles,
                                              int32_t isrc, int32_t ksrc, const double* srcfn,
                                              const int32_t* rec_ijk, float* traces, void* stream) {
  if (!cfg || !model || !profiles || !srcfn || (cfg->nrec > 0 && (!rec_ijk || !traces)))
    return fail_static(SFD_ERR_BAD_ARG, "NULL argument");
  if (cfg->kind != SFD_ELECTROMAG2)
    return fail_static(SFD_ERR_BAD_ARG, "sfd_electromag2_run_static runs electromag2 only");
  if (cfg->flags != 0 && cfg->flags != SFD_FLAG_TWO_PASS)
    return fail_static(SFD_ERR_BAD_ARG,
                       "sfd_electromag2_run_static runs the two-pass form: flags must be 0 or SFD_FLAG_TWO_PASS");
  sfd_config c = *cfg;
  c.flags = SFD_FLAG_TWO_PASS;  // two kernels per step: one copy of the state
  size_t need = 0;
  int32_t r = sfd_state_bytes(&c, &need);
  if (r != SFD_OK) return r;
  if (need > kStaticScratchBytes) {
    char buf[256];
    std::snprintf(buf, sizeof buf,
                  "electromag2 %dx%d with %d steps and %d receivers needs %zu bytes of device state; "
                  "the static scratch of sfd_electromag2_run_static holds %zu",
                  c.nx, c.nz, c.nstep, c.nrec, need, kStaticScratchBytes);
    return fail_static(SFD_ERR_BAD_ARG, buf);
  }
  void* base = nullptr;
  cudaError_t e = static_scratch_address(&base);
  if (e != cudaSuccess) {
    char buf[256];
    std::snprintf(buf, sizeof buf, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    return fail_static(SFD_ERR_CUDA, buf);
  }
  sfd_handle* h = nullptr;
  r = sfd::create_handle(&c, base, kStaticScratchBytes, stream, false, &h);  // clears the whole state
  if (r != SFD_OK) return r;
  const int64_t n2 = (int64_t)c.nx * c.nz;
  if ((r = sfd_set_model(h, model, 6 * n2)) == SFD_OK &&
      (r = sfd_set_cpml(h, profiles, 6 * (int64_t)(c.nx + c.nz))) == SFD_OK &&
      (r = sfd_set_source(h, isrc, 0, ksrc, srcfn, 2, c.nstep)) == SFD_OK &&
      (r = sfd_set_receivers(h, rec_ijk, c.nrec)) == SFD_OK && (r = sfd_run(h, c.nstep)) == SFD_OK) {
    r = c.nrec > 0 ? sfd_get_traces(h, traces, (int64_t)c.nstep * 2 * c.nrec) : SFD_OK;
    if (r == SFD_OK) r = sfd_status(h, nullptr, nullptr);
  }
  // keep the message of the failing call, then release the host-side handle
  const std::string msg = sfd_last_error();
  sfd_destroy(h);
  if (r != SFD_OK) sfd::set_error(msg.c_str());
  return r;
}
