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
// threads: 128, or 32 for a wave smaller than the resident grid (at most
// 4 x grid blocks of 32 then, the same lanes)
cudaError_t launch_wave_lcfa(int model, int grid, int threads, cudaStream_t s, const WaveArgs& a);
cudaError_t launch_wave_lma(int model, int grid, int threads, cudaStream_t s, const WaveArgs& a);
const void* wave_kernel_lcfa(int model);
const void* wave_kernel_lma(int model);

// The persistent multi-collision queue kernel (128 threads per block):
// variant 0 with the registers it needs, variant 1 capped for 3 blocks/SM,
// variant 2 the single-collision kernel (one instantiation per field model,
// M_* values).
cudaError_t launch_queue_v0(int grid, cudaStream_t s, const QueueArgs& q);
cudaError_t launch_queue_v1(int grid, cudaStream_t s, const QueueArgs& q);
const void* queue_kernel_v0();
const void* queue_kernel_v1();
// variant 3: many collisions stepped in lockstep (ptg_queue_v3.cu)
cudaError_t launch_queue_v3(int grid, cudaStream_t s, const QueueArgs& q);
const void* queue_kernel_v3();
cudaError_t launch_queue_single_lma(int model, int grid, cudaStream_t s, const QueueArgs& q);
cudaError_t launch_queue_single_lcfa(int model, int grid, cudaStream_t s, const QueueArgs& q);
const void* queue_kernel_single_lma(int model);
const void* queue_kernel_single_lcfa(int model);

// Regeneration of the LP Breit-Wheeler mid-range CDF (ptg_regen.cu).
cudaError_t launch_regen_lpm_partial(unsigned long long first, unsigned long long count, const int* n_of,
                                     const double* a_of, const double* eta_of, double* ws, int cap, double* rates,
                                     int* bad, cudaStream_t s);
cudaError_t launch_regen_lpm_cdf(int npoints, const int* nmin_of, const int* nmax_of, const unsigned long long* off_of,
                                 const double* rates, double* cdf_out, double* total_out, cudaStream_t s);

// The learned CP proposal (ptg_mlp.cu).
struct MlpDev;
struct LmaTables;
// Packs the weights into `packed` (mlp_packed_bytes()) and runs the batch.
cudaError_t launch_mlp_infer(const MlpDev& m, void* packed, const float* x, unsigned long long n, float* out,
                             cudaStream_t s);
size_t mlp_packed_bytes();
cudaError_t launch_mlp_grad(const MlpDev& m, const void* data, unsigned long long first, int rows, float tau,
                            float* partial, float* loss, int blocks, cudaStream_t s);
cudaError_t launch_mlp_adam(float* p, float* mom, float* vel, const float* partial, int nblocks, float lr, int step,
                            const MlpDev& m, cudaStream_t s);
cudaError_t launch_mlp_sync(const float* p, const MlpDev& m, cudaStream_t s);
cudaError_t launch_mlp_data(const LmaTables* t, unsigned long long n, unsigned long long seed, double a_lo,
                            double a_hi, double e_lo, double e_hi, void* out, cudaStream_t s);
size_t sampler_point_bytes();
cudaError_t launch_sampler_features(const LmaTables* t, unsigned long long n, unsigned long long seed, double a_lo,
                                    double a_hi, double e_lo, double e_hi, float* x_out, void* pts, cudaStream_t s);
cudaError_t launch_sampler_run(const LmaTables* t, unsigned long long n, unsigned long long seed, double a_lo,
                               double a_hi, double e_lo, double e_hi, int learned, const float* env, const void* pts,
                               float margin, unsigned long long* counter, double* v_out, unsigned* evals,
                               unsigned* fallbacks, int* status, cudaStream_t s);
// Primary beams on the device (ptg_beam.cu).
struct BeamArgs {
    int species, gamma_dstr, radial_dstr, custom_len;
    double gamma_mean, gamma_sigma, gamma_min, gamma_max, rho;
    const double* custom_cdf;  // device [len][2]
    double sigma_x, sigma_y, x_max, y_max, r_max, sigma_z, rms_div;
    double angle, cos_a, sin_a, cos_p, sin_p;  // collision angle and plane
    double off_x, off_y, off_z, initial_z;
    double pol[4], weight;
};
cudaError_t launch_build_beam(const BeamArgs& b, unsigned long long n, unsigned long long seed,
                              unsigned long long first_id, int* species, double* r, double* u, double* pol,
                              double* weight, unsigned long long* id, unsigned long long* parent_id,
                              unsigned long long* errors, cudaStream_t s);
// Distribution output (ptg_hgram.cu): the particle set, its functions and
// the binning of one histogram.
struct HgramArgs {
    const int* species;
    const double *u, *r, *pol, *weight, *payload, *parent_chi, *icount, *work;
    unsigned long long n;
    int want_species, dim, func[2], wfunc, log_bins, filter_func;
    double scale[2], fmin, fmax;
    // binning (fill pass)
    double gmin[2], bin_sz[2];
    unsigned long long nbins[2];
    int density_log;  // scale log-binned weights by the bin's linear width
};
cudaError_t launch_hgram_stats(const HgramArgs& h, int blocks, double* partials, cudaStream_t s);
cudaError_t launch_hgram_fill(const HgramArgs& h, int blocks, double* counts, cudaStream_t s);
// Summary-statistic sums: h.func[0] is the variable, h.func[1] the weight
// function, h.filter_func / fmin / fmax the exclusive filter; 9 doubles per
// block.
cudaError_t launch_particle_sums(const HgramArgs& h, double shift, int blocks, double* partials, cudaStream_t s);
int mlp_param_count();
size_t mlp_sample_bytes();
}  // namespace ptg
