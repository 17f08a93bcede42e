// Oracle (test infrastructure only): LMA emission and pair creation
// (nonlinear_compton/*, pair_creation/*) and the Bessel functions they use,
// FP64 CPU restatement.
#pragma once
#include <string>

#include "fields.h"

namespace orc {

// LMA tables loaded from the package's .ptgt files (orc_load_tables).
struct LmaTables {
    const double* nlc_lp_rate = nullptr;   // [68][61] ln rate
    const double* nlc_lp_cdf = nullptr;    // [4148][16][2]
    const double* nlc_cp_rate = nullptr;   // [70][61] ln rate
    const double* nlc_cp_cdf = nullptr;    // [4270][32][2] (regenerated)
    const double* nlc_lp_cl_rate = nullptr;  // [61]
    const double* nlc_lp_cl_cdf = nullptr;   // [61][16][2]
    const double* nlc_cp_cl_rate = nullptr;  // [61]
    const double* nlc_cp_cl_cdf = nullptr;   // [61][32][2]
    const double* bw_cp_total = nullptr;   // [121][74][2]
    const double* bw_lp_total = nullptr;   // [61][25][2]
    const double* bw_lp_cdf = nullptr;     // [1525][16][3]
    const double* bw_lp_mid_total = nullptr;  // [157][36][2]
    const double* bw_lp_mid_cdf = nullptr;    // [5652][16][3] (regenerated)
};
extern LmaTables g_lma;
bool load_lma_tables(const std::string& dir, std::string* err);

// special_functions/bessel.rs
double bessel_j(double x, int n);
void bessel_j_pm(double x, int n, double* jm1, double* j, double* jp1);
double bessel_triple_j_mid(int n, double x);
double bessel_j_asymptotic(int n, double x);

// nonlinear_compton/cp/mod.rs
double cp_diff_partial_rate(int n, double a, double eta, double v);
double cp_ceiling_diff_partial_rate(int n, double a, double eta);
double cp_partial_rate(int n, double a, double eta);
double cp_spectrum_low_eta(int n, double a, double v);
bool cp_rate(double a, double eta, double* out);
bool cp_classical_rate(double a, double eta, double* out);
int cp_invert(double a, double eta, double frac);
int cp_sample(double a, double eta, DrawStream& rng, int* n, double* s, double* theta, Stokes* sv, uint64_t* rej);

// nonlinear_compton/lp/linear.rs
double lp_linear_rate(double a, double eta);

// special_functions/double_bessel.rs
double double_bessel_at(int n, double x_max, double y_max, double x, double y);
double double_bessel_evaluate(int n, double x, double y);
double double_bessel_spa(int n, double x, double y);
double lp_ceiling_at(int n, double a, double eta);

// nonlinear_compton/lp/mod.rs
int lp_sum_limit(double a, double eta);
void lp_partial_rate(int n, double a, double eta, double* integral, double* mx);
bool lp_rate(double a, double eta, double* out);
bool lp_classical_rate(double a, double eta, double* out);
int lp_harmonic_index(double a, double eta, double frac);
int lp_sample(double a, double eta, DrawStream& rng, int* n, double* s, double* theta, Stokes* sv, uint64_t* rej);

// nonlinear_compton/{cp,lp}/classical.rs
double cp_cl_integrated(int n, double a);
double lp_cl_partial_rate(int n, double a);
int cp_classical_sample(double a, double eta, DrawStream& rng, int* n, double* s, double* theta, Stokes* sv,
                        uint64_t* rej);
int lp_classical_sample(double a, double eta, DrawStream& rng, int* n, double* s, double* theta, Stokes* sv,
                        uint64_t* rej);

// nonlinear_compton/mod.rs
bool nlc_probability(const V4& k, const V4& q, double dt, int pol, bool classical, double* p);
int nlc_generate(const V4& k, const V4& q, int pol, double pol_angle, bool classical, DrawStream& rng, int* n,
                 V4* k_prime, Stokes* sv, uint64_t* rej);

// pair_creation/cp/mod.rs and pair_creation/mod.rs
void cp_pair_integrate(int n, double a, double eta, double* re, double* im);
void cp_pair_by_summation(double a, double eta, double f[2]);
bool cp_pair_by_lookup(double a, double eta, double f[2]);
bool cp_pair_rates(double a, double eta, double f[2]);
bool bw_probability(const V4& ell, const Stokes& sv, const V4& k, double a, double dt, int pol, double pol_angle,
                    double* prob, Stokes* sv_out);
// pair_creation/lp
bool lp_pair_rates(double a, double eta, double f[2]);
int lp_pair_sample(double a, double eta, double sv1, double sv2, DrawStream& rng, int* n, double* s, double* theta,
                   uint64_t* rej);
void lp_pair_dd_rate(int n, double a, double eta, double s, double theta, double out[2]);
void lp_pair_partial_rate(int n, double a, double eta, double out[2]);
void lp_pair_by_summation(double a, double eta, double cdf[48]);
int bw_generate(const V4& ell, const Stokes& sv, const V4& k, double a, int pol, double pol_angle, DrawStream& rng,
                int* n, V4* q, uint64_t* rej);

// plane_wave.rs:251-282 / focused_laser.rs:260-281
int lma_radiate(const Laser& laser, const V4& r, const V4& u, double dt, DrawStream& rng, bool classical,
                bool* emitted, RadiationEvent* ev, uint64_t* rejections);
// plane_wave.rs:284-316 / focused_laser.rs:283-306
int lma_pair_create(const Laser& laser, const V4& r, const V4& ell, const Stokes& pol, double dt, DrawStream& rng,
                    double rate_increase, double* prob, Stokes* pol_new, bool* created, PairEvent* ev,
                    uint64_t* rejections);

// Standard normal from two uniforms (Box-Muller), used for the finite
// bandwidth of the LMA lasers.
double std_normal(DrawStream& rng);

}  // namespace orc
