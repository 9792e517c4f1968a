// gb_aba_derivatives_noalloc: the batched ABA derivatives for callers that must
// not allocate device memory.
//
// Who cannot allocate: real-time control loops, whose cycle must not wait on
// an allocator (the reference's own algorithms promise not to allocate, and
// unittest/crba.cpp checks it with Eigen's malloc guard), and plugins hosted by
// an application that owns every device allocation and its budget.
// gb_aba_derivatives takes its per-configuration workspace from
// cudaMallocAsync; this entry point instead uses the fixed device array below.
//
// The array is kNoAllocScratchBytes (64 MiB) and is held by every GPU that
// loads this library until the process exits.  A call needs a fixed number of
// workspace bytes per configuration (about 66 KB for the 32-dof humanoid in
// FP64, 47 KB mixed, i.e. up to ~1000 / ~1400 configurations per call; the
// error message of a rejected call states both figures); larger
// batches are rejected with GB_ERR_SIZE.  Every call shares the
// array: calls whose kernels overlap on the GPU (different streams, or other
// host threads) race on it and must be serialised by the caller.  The kernels
// write every workspace entry before reading it, so the contents a previous
// call left behind need no clearing.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "gb_internal.h"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;

// The workspace.  In host code its name is only a host-side stand-in: the
// device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_scratch_ptr[kMaxDevices] = {nullptr};

// Resolves the device address of the array on the current device, once per
// device.  This happens inside the first call made on a device, so that first
// call must come before any stream capture.  The address is kept for the life
// of the process: after a cudaDeviceReset the module is loaded again and the
// array may move, so this entry point must not be used after a device reset.
int scratch_on_current_device(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return gbi::cuda_error(e, "gb_aba_derivatives_noalloc");
  if (dev < 0 || dev >= kMaxDevices) return gbi::set_error(GB_ERR_UNSUPPORTED, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mutex);
  if (g_scratch_ptr[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return gbi::cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return GB_OK;
}

}  // namespace

extern "C" {

int gb_aba_derivatives_noalloc(const gb_model* M, int precision, int layout, long B, const double* q,
                               const double* v, const double* tau, double* ddq_dq, double* ddq_dv, double* Minv,
                               double* ddq, void* stream) {
  int rc = gbi::check_common(M, precision, layout, B);
  if (rc != GB_OK) return rc;
  if (B == 0) return GB_OK;
  const size_t need = gbi::aba_derivs_workspace_bytes(M, precision, B);
  if (need > kNoAllocScratchBytes)
    return gbi::set_error(GB_ERR_SIZE, "gb_aba_derivatives_noalloc: batch " + std::to_string(B) + " needs " +
                                           std::to_string(need) + " bytes of workspace, the fixed scratch holds " +
                                           std::to_string(kNoAllocScratchBytes) + "; split the batch");
  const void* ptrs[] = {q, v, tau, ddq_dq, ddq_dv, Minv};
  const char* names[] = {"q", "v", "tau", "ddq_dq", "ddq_dv", "Minv"};
  for (int k = 0; k < 6; ++k) {
    rc = gbi::check_ptr(ptrs[k], names[k]);
    if (rc != GB_OK) return rc;
  }
  if (ddq) {
    rc = gbi::check_ptr(ddq, "ddq");
    if (rc != GB_OK) return rc;
  }
  void* ws = nullptr;
  rc = scratch_on_current_device(&ws);
  if (rc != GB_OK) return rc;
  const long nn = (long)M->nv * M->nv;
  using gbi::arr;
  return gbi::launch_aba_derivs_on_workspace(
      M, precision, B, arr(q, layout, B, M->nq), arr(v, layout, B, M->nv), arr(tau, layout, B, M->nv),
      arr(ddq_dq, layout, B, nn), arr(ddq_dv, layout, B, nn), arr(Minv, layout, B, nn), arr(ddq, layout, B, M->nv), ws,
      (cudaStream_t)stream);
}

}  // extern "C"
