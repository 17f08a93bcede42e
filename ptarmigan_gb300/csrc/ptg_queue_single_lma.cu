// Single-collision queue kernel (collide_queue_single) for a batch of one
// collision in an LMA field model (PlaneWave or FocusedLaser).
#include "ptg_launch.h"
#include "ptg_queue.cuh"

namespace ptg {

cudaError_t launch_queue_single_lma(int model, int grid, cudaStream_t s, const QueueArgs& q) {
    if (model == M_PLANE_WAVE)
        collide_queue_single<M_PLANE_WAVE><<<grid, 128, 0, s>>>(q);
    else if (model == M_FOCUSED_LASER)
        collide_queue_single<M_FOCUSED_LASER><<<grid, 128, 0, s>>>(q);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

const void* queue_kernel_single_lma(int model) {
    if (model == M_PLANE_WAVE) return (const void*)collide_queue_single<M_PLANE_WAVE>;
    if (model == M_FOCUSED_LASER) return (const void*)collide_queue_single<M_FOCUSED_LASER>;
    return nullptr;
}

}  // namespace ptg
