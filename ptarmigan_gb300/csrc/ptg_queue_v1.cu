// Queue kernel variant 1: 128 threads per block, __launch_bounds__ minimum
// of 3 block(s) per SM.
#include "ptg_launch.h"
#include "ptg_queue.cuh"

namespace ptg {

cudaError_t launch_queue_v1(int grid, cudaStream_t s, const QueueArgs& q) {
    collide_queue<3><<<grid, 128, 0, s>>>(q);
    return cudaGetLastError();
}

const void* queue_kernel_v1() { return (const void*)collide_queue<3>; }

}  // namespace ptg
