// Host-side launchers of the collision kernels.  Each kernel family lives in
// its own translation unit (ptg_wave_lcfa.cu, ptg_wave_lma.cu,
// ptg_queue_v*.cu) so that the library builds in parallel; the engine calls
// them through these functions.
#pragma once
#include <cuda_runtime.h>

namespace ptg {
struct WaveArgs;
struct QueueArgs;

// One wave of collide_wave<model> (block size 128).
cudaError_t launch_wave_lcfa(int model, int grid, cudaStream_t s, const WaveArgs& a);
cudaError_t launch_wave_lma(int model, int grid, cudaStream_t s, const WaveArgs& a);
const void* wave_kernel_lcfa(int model);
const void* wave_kernel_lma(int model);

// The persistent multi-collision queue kernel (128 threads per block):
// variant 0 with the registers it needs, variant 1 capped for 3 blocks/SM.
cudaError_t launch_queue_v0(int grid, cudaStream_t s, const QueueArgs& q);
cudaError_t launch_queue_v1(int grid, cudaStream_t s, const QueueArgs& q);
const void* queue_kernel_v0();
const void* queue_kernel_v1();
}  // namespace ptg
