// A 3D solve that allocates nothing: the scratch space the solver needs (its
// dependency counters, work-ticket counter, status word, per-source set-up
// and branch records) lives in one fixed array compiled into this library
// instead of a workspace the caller allocates.
//
// Who needs it: callers that cannot call cudaMalloc or hand over a second
// device buffer. Examples are a host framework that reserves all device
// memory for its own allocator and forbids hidden allocations, a latency-
// critical loop where cudaMalloc/cudaFree would implicitly synchronise the
// device, or a foreign-language binding that can pass the input and output
// buffers it already owns but cannot manage another device allocation's
// lifetime. The caller still passes the model, the sources and the output
// arrays; only the scratch comes from here.
//
// Limits and sharing:
//  * The array holds FTEIK_NOALLOC_SCRATCH_BYTES (64 MiB). Every GPU that loads
//    the library keeps it until the process exits. A problem whose scratch
//    would not fit (fteik3d_workspace_bytes(...) above that size) is rejected
//    with FTEIK_WORKSPACE_TOO_SMALL before any GPU work.
//  * Every call on a device uses the same array, and the array keeps what the
//    last call left in it. The solve clears what must start at zero (counters,
//    status, ticket) and refills the branch records itself, with memsets on
//    the caller's stream. Two calls that overlap on the GPU (different streams
//    or host threads at once) race on the array and corrupt each other's
//    results: serialise them.
//  * The first call on each device performs a one-time set-up on that device
//    (it looks up the array's device address with cudaGetSymbolAddress while
//    that device is current). Make that first call before any stream capture.
//  * cudaDeviceReset (or anything else that replaces the device's primary
//    context) reloads the library's device code, so the array may move. Every
//    later call that is not made during a stream capture looks the address up
//    again and keeps the new one; after a reset, make one call outside any
//    capture before capturing calls again.
#include <cstdio>
#include <mutex>

#include "common.cuh"
#include "fteik_gb300.h"
#include "runtime.h"

namespace fteik {

// The scratch array itself. Host code must not pass `g_noalloc_scratch` to a
// kernel directly: in host code the name is a host-side stand-in, not a device
// address. The set-up below obtains the device address.
static __device__ __align__(256) unsigned char g_noalloc_scratch[FTEIK_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device: looked up on the
// device's first call, with that device current, and again on every call made
// outside a stream capture (a device reset may have moved it). During a
// capture the cached address is used.
static int noalloc_scratch(void** out, cudaStream_t stream) {
  int dev = 0;
  FTEIK_CHECK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return kInvalidArgument;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  bool capturing = true;
  if (cudaStreamIsCapturing(stream, &cs) == cudaSuccess)
    capturing = cs != cudaStreamCaptureStatusNone;
  else
    (void)cudaGetLastError();  // an illegal query during another capture: treat as capturing
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev] || !capturing) {
    void* ptr = nullptr;
    FTEIK_CHECK(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
    if (!ptr) return kCudaError;
    g_noalloc_ptr[dev] = ptr;
  }
  *out = g_noalloc_ptr[dev];
  return kOk;
}

}  // namespace fteik

using namespace fteik;

extern "C" int fteik3d_solve_noalloc(const double* slow, int nz, int nx, int ny, double dz,
                                     double dx, double dy, const double* sources, int nsrc,
                                     int nsweep, int grad, double* tt, double* ttgrad,
                                     double* vzero, long long spin_limit, void* stream) {
  const size_t need = fteik3d_workspace_bytes(nz, nx, ny, nsrc, grad);
  if (need == 0) return kInvalidArgument;
  if (need > (size_t)FTEIK_NOALLOC_SCRATCH_BYTES) {
    set_last_error("fteik3d_solve_noalloc: this problem needs %zu bytes of scratch, above the "
                   "fixed maximum of %zu bytes",
                   need, (size_t)FTEIK_NOALLOC_SCRATCH_BYTES);
    return kWorkspaceTooSmall;
  }
  void* scratch = nullptr;
  const int rc0 = noalloc_scratch(&scratch, (cudaStream_t)stream);
  if (rc0 != kOk) return rc0;
  const int rc = fteik3d_solve_async(slow, nz, nx, ny, dz, dx, dy, sources, nsrc, nsweep, grad,
                                     tt, ttgrad, vzero, scratch, FTEIK_NOALLOC_SCRATCH_BYTES,
                                     spin_limit, stream);
  if (rc != kOk) return rc;
  return fteik_workspace_status(scratch, stream);
}
