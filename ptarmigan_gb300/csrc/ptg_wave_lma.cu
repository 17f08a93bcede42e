// collide_wave instantiations for the LMA field models (PlaneWave,
// FocusedLaser).
#include "ptg_collide.cuh"
#include "ptg_launch.h"

namespace ptg {

cudaError_t launch_wave_lma(int model, int grid, int threads, cudaStream_t s, const WaveArgs& a) {
    if (model == M_PLANE_WAVE)
        collide_wave<M_PLANE_WAVE><<<grid, threads, 0, s>>>(a);
    else if (model == M_FOCUSED_LASER)
        collide_wave<M_FOCUSED_LASER><<<grid, threads, 0, s>>>(a);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

const void* wave_kernel_lma(int model) {
    if (model == M_PLANE_WAVE) return (const void*)collide_wave<M_PLANE_WAVE>;
    if (model == M_FOCUSED_LASER) return (const void*)collide_wave<M_FOCUSED_LASER>;
    return nullptr;
}

}  // namespace ptg
