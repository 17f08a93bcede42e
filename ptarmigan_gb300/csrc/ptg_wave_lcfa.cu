// collide_wave instantiations for the LCFA field models (FastPlaneWave,
// FastFocusedLaser).
#include "ptg_collide.cuh"
#include "ptg_launch.h"

namespace ptg {

cudaError_t launch_wave_lcfa(int model, int grid, int threads, cudaStream_t s, const WaveArgs& a) {
    if (model == M_FAST_PLANE_WAVE)
        collide_wave<M_FAST_PLANE_WAVE><<<grid, threads, 0, s>>>(a);
    else if (model == M_FAST_FOCUSED_LASER)
        collide_wave<M_FAST_FOCUSED_LASER><<<grid, threads, 0, s>>>(a);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

const void* wave_kernel_lcfa(int model) {
    if (model == M_FAST_PLANE_WAVE) return (const void*)collide_wave<M_FAST_PLANE_WAVE>;
    if (model == M_FAST_FOCUSED_LASER) return (const void*)collide_wave<M_FAST_FOCUSED_LASER>;
    return nullptr;
}

}  // namespace ptg
