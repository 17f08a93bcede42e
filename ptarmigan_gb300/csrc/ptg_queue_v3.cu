// Queue kernel variant 3: many collisions stepped in lockstep (one step per
// pass, emissions served by the warp), 128 threads per block.
#include "ptg_launch.h"
#include "ptg_queue.cuh"

namespace ptg {

cudaError_t launch_queue_v3(int grid, cudaStream_t s, const QueueArgs& q) {
    collide_queue_lockstep<1><<<grid, 128, 0, s>>>(q);
    return cudaGetLastError();
}

const void* queue_kernel_v3() { return (const void*)collide_queue_lockstep<1>; }

}  // namespace ptg
