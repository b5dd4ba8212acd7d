// Model preparation on the device: slowness = 1.0 / velocity, the first step
// of Eikonal2D/3D.solve (fteikpy/_solver.py:49-50,120-121), fused with the
// range check that the solver kernels rely on (exact power-of-two scalings
// need slowness squared to stay a normal double).
#include "common.cuh"
#include "fteik_gb300.h"
#include "runtime.h"

namespace fteik {

__global__ void slowness_kernel(const double* v, long long n, double* s, int* bad) {
  int local_bad = 0;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const double x = 1.0 / v[q];
    s[q] = x;
    if (!(x > 1e-150 && x < 1e150)) local_bad = 1;
  }
  if (__any_sync(0xffffffffu, local_bad) && (threadIdx.x & 31) == 0) atomicOr(bad, 1);
}

}  // namespace fteik

using namespace fteik;

extern "C" int fteik_slowness(const double* velocity, long long n, double* slow, int* flag,
                              void* stream) {
  if (n < 1 || !velocity || !slow || !flag) return kInvalidArgument;
  cudaStream_t st = (cudaStream_t)stream;
  FTEIK_CHECK(cudaMemsetAsync(flag, 0, sizeof(int), st));
  slowness_kernel<<<grid_for(n, 256), 256, 0, st>>>(velocity, n, slow, flag);
  FTEIK_CHECK(cudaGetLastError());
  FTEIK_CHECK(cudaStreamSynchronize(st));
  int bad = 0;
  FTEIK_CHECK(cudaMemcpy(&bad, flag, sizeof(int), cudaMemcpyDeviceToHost));
  return bad ? kInvalidArgument : kOk;
}
