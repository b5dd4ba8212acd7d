// Host-side helpers shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>

namespace fteik {

// Records the CUDA error text for fteik_last_error() and returns kCudaError.
int record_cuda_error(cudaError_t err, const char* what);

// Records a formatted message for fteik_last_error().
void set_last_error(const char* fmt, ...);

#define FTEIK_CHECK(call)                                          \
  do {                                                             \
    cudaError_t err_ = (call);                                     \
    if (err_ != cudaSuccess) return record_cuda_error(err_, #call); \
  } while (0)

// Streaming multiprocessors of the current device (cached).
int sm_count();

// Blocks of `threads` threads that stay resident at once on the current
// device for `kernel` (cached per kernel).
int resident_blocks(const void* kernel, int threads, size_t smem = 0);

// Grid size for a grid-stride loop over n items: a multiple of the SM count.
int grid_for(long long n, int threads);

// When kernel timing is on (fteik_kernel_timing), the pair of events that the
// 3D solve records around its sweep kernel on the launching stream; else null.
void timing_events(cudaEvent_t* start, cudaEvent_t* stop);
bool kernel_timing_on();

// Tuning options (fteik_set_option); -1 = automatic.
enum Option : int {
  kOptSweepCoef = 0,    // 3D sweep coefficients: 1 precomputed arrays, 0 slowness cells
  kOptSweepPencil = 1,  // 3D pencil width along x: 2, 4 or 8 (the pencil is w x 32/w)
  kOptSweepChunk = 2,   // 3D steps between progress publications: 1, 2, 4, ... 64
  kOptKeepTest = 3,     // 3D unchanged-node test before the 2D/3D operators: 0 off
  kOptSweepTeam = 4,    // 3D team kernel (compacted operators): 1 on, 0 off
  kOptAdjointChunk = 5, // adjoint reverse sweeps: steps between progress publications
  kOptSweep2dKeys = 6,  // 2D sweeps: 0 forces IEEE comparisons (else integer keys when exact)
  kOptSweep2dWarp = 7,  // 2D sweeps: 2 a block per source, 1 a warp, 0 one thread
  kOptSweep2dSpec = 8,  // 2D warp sweeps: 0 turns off the speculated updates (same results)
  kOptSweep2dWaitNs = 9,  // 2D block sweeps: bound of one wait between warps, in ns
  kOptRayLanes = 10,      // rays: lanes per ray, 32, 4 or 1
  kOptCount = 11,
};
long long option_value(int opt);

}  // namespace fteik
