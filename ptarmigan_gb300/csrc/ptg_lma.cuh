// LMA nonlinear Compton emission and Breit-Wheeler pair creation
// (nonlinear_compton/*, pair_creation/*) on the device.
#pragma once
#include "ptg_fields.cuh"
#include "ptg_math.cuh"

namespace ptg {

// Device pointers to the LMA rate and CDF tables (loaded from data files).
struct LmaTables {
    const double* nlc_lp_rate;   // [68][61]
    const double* nlc_lp_cdf;    // [4148][16][2]
    const double* nlc_cp_rate;   // [70][61]
    const double* nlc_cp_cdf;    // [4270][32][2] or null
    const double* bw_cp_total;   // [121][74][2]
    const double* bw_lp_total;   // [61][25][2]
    const double* bw_lp_cdf;     // [1525][16][3]
    const double* bw_lp_mid_total;  // [157][36][2]
    const double* bw_lp_mid_cdf;    // [5652][16][3] or null
};

// plane_wave.rs:251-282 / focused_laser.rs:260-281
__device__ __noinline__ int lma_radiate(const FieldParams& f, const LmaTables& t, d4 r, d4 u, double dt, Draws& rng,
                                        bool classical, bool* emitted, d4* k, d4* u_prime, d3* pol, double* a_eff,
                                        double* chi, double* absorption, uint32_t* rej) {
    *emitted = false;
    return 9;  // PTG_ERR_UNSUPPORTED until the LMA samplers land
}

// plane_wave.rs:284-316 / focused_laser.rs:283-306
__device__ __noinline__ int lma_pair_create(const FieldParams& f, const LmaTables& t, d4 r, d4 ell, d4 pol, double dt,
                                            Draws& rng, double rate_increase, double* prob, d4* pol_new,
                                            bool* created, d4* ue, d4* up, double* frac, double* a_eff, double* chi,
                                            double* absorption, uint32_t* rej) {
    *prob = 0.0;
    *pol_new = pol;
    *created = false;
    return 9;
}

}  // namespace ptg
