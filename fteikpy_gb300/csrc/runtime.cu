// Host-side runtime of the C ABI: error reporting, occupancy-derived launch
// shapes, and the status word of a solve workspace.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <unordered_map>

#include "common.cuh"
#include "fteik_gb300.h"
#include "runtime.h"

namespace fteik {

static thread_local char g_last_error[256] = "";

int record_cuda_error(cudaError_t err, const char* what) {
  std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s", what, cudaGetErrorString(err));
  return kCudaError;
}

void set_last_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

int sm_count() {
  static int count = 0;
  if (count == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev);
    if (count <= 0) count = 1;
  }
  return count;
}

int resident_blocks(const void* kernel, int threads, size_t smem) {
  static std::mutex mu;
  static std::unordered_map<const void*, int> cache;
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find(kernel);
  if (it != cache.end()) return it->second;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) !=
          cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  const int blocks = per_sm * sm_count();
  cache[kernel] = blocks;
  return blocks;
}

int grid_for(long long n, int threads) {
  long long blocks = (n + threads - 1) / threads;
  const long long cap = 8LL * sm_count();
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return (int)blocks;
}

static long long g_options[kOptCount] = {-1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1};

long long option_value(int opt) { return (opt >= 0 && opt < kOptCount) ? g_options[opt] : -1; }

static thread_local bool g_timing = false;
static thread_local cudaEvent_t g_ev[2] = {nullptr, nullptr};

bool kernel_timing_on() { return g_timing; }

void timing_events(cudaEvent_t* start, cudaEvent_t* stop) {
  *start = g_timing ? g_ev[0] : nullptr;
  *stop = g_timing ? g_ev[1] : nullptr;
}

// FP64 issue-rate probe: independent DFMA chains, 4 per thread.
__global__ void fp64_probe_kernel(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3 + 1.0, x1 = x0 + 0.1, x2 = x0 + 0.2, x3 = x0 + 0.3;
  for (int i = 0; i < iters; ++i) {
    x0 = __fma_rn(x0, a, b);
    x1 = __fma_rn(x1, a, b);
    x2 = __fma_rn(x2, a, b);
    x3 = __fma_rn(x3, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3;
}

}  // namespace fteik

using namespace fteik;

extern "C" int fteik_set_option(const char* name, long long value) {
  if (!name) return kInvalidArgument;
  if (std::strcmp(name, "sweep_coef") == 0) {
    g_options[kOptSweepCoef] = value < 0 ? -1 : (value ? 1 : 0);
    return kOk;
  }
  if (std::strcmp(name, "sweep_pencil") == 0) {
    if (value >= 0 && value != 2 && value != 4 && value != 8) return kInvalidArgument;
    g_options[kOptSweepPencil] = value < 0 ? -1 : value;
    return kOk;
  }
  if (std::strcmp(name, "sweep_chunk") == 0) {
    if (value >= 0 && (value < 1 || value > 64 || (value & (value - 1)) != 0))
      return kInvalidArgument;
    g_options[kOptSweepChunk] = value < 0 ? -1 : value;
    return kOk;
  }
  if (std::strcmp(name, "sweep_keep_test") == 0) {
    g_options[kOptKeepTest] = value < 0 ? -1 : (value ? 1 : 0);
    return kOk;
  }
  if (std::strcmp(name, "sweep_team") == 0) {
    g_options[kOptSweepTeam] = value < 0 ? -1 : (value ? 1 : 0);
    return kOk;
  }
  if (std::strcmp(name, "sweep2d_warp") == 0) {
    if (value > 2) return kInvalidArgument;
    g_options[kOptSweep2dWarp] = value < 0 ? -1 : value;
    return kOk;
  }
  if (std::strcmp(name, "sweep2d_keys") == 0) {
    g_options[kOptSweep2dKeys] = value < 0 ? -1 : (value ? 1 : 0);
    return kOk;
  }
  if (std::strcmp(name, "sweep2d_speculate") == 0) {
    g_options[kOptSweep2dSpec] = value < 0 ? -1 : (value ? 1 : 0);
    return kOk;
  }
  if (std::strcmp(name, "ray_lanes") == 0) {
    if (value >= 0 && value != 1 && value != 4 && value != 32) return kInvalidArgument;
    g_options[kOptRayLanes] = value < 0 ? -1 : value;
    return kOk;
  }
  if (std::strcmp(name, "sweep2d_wait_ns") == 0) {
    g_options[kOptSweep2dWaitNs] = value < 0 ? -1 : value;
    return kOk;
  }
  if (std::strcmp(name, "adjoint_chunk") == 0) {
    if (value >= 0 && (value < 1 || value > 64 || (value & (value - 1)) != 0))
      return kInvalidArgument;
    g_options[kOptAdjointChunk] = value < 0 ? -1 : value;
    return kOk;
  }
  return kInvalidArgument;
}

extern "C" int fteik_get_option(const char* name, long long* value) {
  if (!name || !value) return kInvalidArgument;
  if (std::strcmp(name, "sweep_coef") == 0) *value = g_options[kOptSweepCoef];
  else if (std::strcmp(name, "sweep_pencil") == 0) *value = g_options[kOptSweepPencil];
  else if (std::strcmp(name, "sweep_chunk") == 0) *value = g_options[kOptSweepChunk];
  else if (std::strcmp(name, "sweep_keep_test") == 0) *value = g_options[kOptKeepTest];
  else if (std::strcmp(name, "sweep_team") == 0) *value = g_options[kOptSweepTeam];
  else if (std::strcmp(name, "adjoint_chunk") == 0) *value = g_options[kOptAdjointChunk];
  else if (std::strcmp(name, "sweep2d_keys") == 0) *value = g_options[kOptSweep2dKeys];
  else if (std::strcmp(name, "sweep2d_warp") == 0) *value = g_options[kOptSweep2dWarp];
  else if (std::strcmp(name, "sweep2d_speculate") == 0) *value = g_options[kOptSweep2dSpec];
  else if (std::strcmp(name, "sweep2d_wait_ns") == 0) *value = g_options[kOptSweep2dWaitNs];
  else if (std::strcmp(name, "ray_lanes") == 0) *value = g_options[kOptRayLanes];
  else return kInvalidArgument;
  return kOk;
}

extern "C" int fteik_kernel_timing(int on) {
  g_timing = on != 0;
  if (g_timing && !g_ev[0]) {
    FTEIK_CHECK(cudaEventCreate(&g_ev[0]));
    FTEIK_CHECK(cudaEventCreate(&g_ev[1]));
  }
  return kOk;
}

extern "C" int fteik_last_sweep_ms(float* ms) {
  if (!g_timing || !g_ev[1] || !ms) return kInvalidArgument;
  FTEIK_CHECK(cudaEventSynchronize(g_ev[1]));
  FTEIK_CHECK(cudaEventElapsedTime(ms, g_ev[0], g_ev[1]));
  return kOk;
}

extern "C" int fteik_fp64_peak(double* scratch, int nblocks, int iters, double* flops_per_s,
                               void* stream) {
  if (!scratch || nblocks < 1 || iters < 1 || !flops_per_s) return kInvalidArgument;
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t e0, e1;
  FTEIK_CHECK(cudaEventCreate(&e0));
  FTEIK_CHECK(cudaEventCreate(&e1));
  fp64_probe_kernel<<<nblocks, 256, 0, st>>>(scratch, 16, 0.999999, 1e-7);
  FTEIK_CHECK(cudaEventRecord(e0, st));
  fp64_probe_kernel<<<nblocks, 256, 0, st>>>(scratch, iters, 0.999999, 1e-7);
  FTEIK_CHECK(cudaEventRecord(e1, st));
  FTEIK_CHECK(cudaEventSynchronize(e1));
  float ms = 0.f;
  FTEIK_CHECK(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *flops_per_s = 2.0 * 4.0 * iters * (double)nblocks * 256.0 / (ms * 1e-3);
  return kOk;
}

__global__ void sqrt_rn_kernel(const double* x, long long n, double* out) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    out[q] = sqrt_rn(x[q]);
}

extern "C" int fteik_sqrt_rn(const double* x, long long n, double* out, void* stream) {
  if (n < 0 || (n > 0 && (!x || !out))) return kInvalidArgument;
  if (n == 0) return kOk;
  const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 16);
  sqrt_rn_kernel<<<(int)blocks, 256, 0, (cudaStream_t)stream>>>(x, n, out);
  FTEIK_CHECK(cudaGetLastError());
  return kOk;
}

__global__ void div_rn_kernel(const double* x, long long n, double c, double nc, double y,
                              double* out) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    out[q] = div_tk(x[q], c, nc, y);
}

extern "C" int fteik_div_rn(const double* x, long long n, double c, double* out, void* stream) {
  if (n < 0 || (n > 0 && (!x || !out)) || !(c > 0.0) || !std::isfinite(c)) return kInvalidArgument;
  if (n == 0) return kOk;
  const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 16);
  div_rn_kernel<<<(int)blocks, 256, 0, (cudaStream_t)stream>>>(x, n, c, -c, 1.0 / c, out);
  FTEIK_CHECK(cudaGetLastError());
  return kOk;
}

__global__ void recip_rn_kernel(const double* x, long long n, double* out) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    out[q] = recip_rn(x[q]);
}

extern "C" int fteik_recip_rn(const double* x, long long n, double* out, void* stream) {
  if (n < 0 || (n > 0 && (!x || !out))) return kInvalidArgument;
  if (n == 0) return kOk;
  const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 16);
  recip_rn_kernel<<<(int)blocks, 256, 0, (cudaStream_t)stream>>>(x, n, out);
  FTEIK_CHECK(cudaGetLastError());
  return kOk;
}

extern "C" const char* fteik_version(void) { return "fteik_gb300 0.1.0 (sm_103a)"; }

extern "C" const char* fteik_last_error(void) { return g_last_error; }

extern "C" int fteik_workspace_status(const void* workspace, void* stream) {
  FTEIK_CHECK(cudaStreamSynchronize((cudaStream_t)stream));
  int status = 0;
  FTEIK_CHECK(cudaMemcpy(&status, workspace, sizeof(int), cudaMemcpyDeviceToHost));
  return status;
}
