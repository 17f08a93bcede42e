// Queue kernel variant 0: 128 threads per block, __launch_bounds__ minimum
// of 1 block(s) per SM.
#include "ptg_launch.h"
#include "ptg_queue.cuh"

namespace ptg {

cudaError_t launch_queue_v0(int grid, cudaStream_t s, const QueueArgs& q) {
    collide_queue<1><<<grid, 128, 0, s>>>(q);
    return cudaGetLastError();
}

const void* queue_kernel_v0() { return (const void*)collide_queue<1>; }

}  // namespace ptg
