// Oracle (test infrastructure only): FP64 CPU restatement of ptarmigan's
// L0/L1 numerics on the collision path — constants, pwmci, Airy functions,
// LCFA photon emission and LCFA pair creation.  Each function cites the
// reference file:line it follows.  Not part of the product library.
#pragma once
#include "geom.h"
#include "rng.h"

namespace orc {

// src/constants.rs:4-30
constexpr double SPEED_OF_LIGHT = 2.997925e8;
constexpr double SPEED_OF_LIGHT_SQD = 89875517873681764.0;
constexpr double VACUUM_PERMITTIVITY = 8.854188e-12;
constexpr double ELECTRON_CHARGE = -1.602177e-19;
constexpr double ELEMENTARY_CHARGE = 1.602177e-19;
constexpr double ELECTRON_MASS = 9.109383e-31;
constexpr double ELECTRON_MASS_MEV = 0.510999;
constexpr double CRITICAL_FIELD = 1.323285e18;
constexpr double ALPHA_FINE = 7.29735257e-3;
constexpr double COMPTON_TIME = 1.28808867e-21;
constexpr double PI = 3.14159265358979323846;

// pwmci.rs:4-306 — piecewise monotonic cubic interpolation over rows of
// [x, f] (stride 2 doubles).  `ok` is false where the reference returns None.
struct Pwmci {
    const double* tbl;
    int len;
    bool ext;
    Pwmci(const double* t, int n, bool extrapolate = false) : tbl(t), len(n), ext(extrapolate) {}
    double evaluate(double x, bool* ok) const;
    double invert(double f, bool* ok) const;
};

// special_functions/airy.rs:41-136
double airy_ai(double x, bool* ok);
double airy_ai_prime(double x, bool* ok);
double bessel_k_1_3(double x, bool* ok);
double bessel_k_2_3(double x, bool* ok);

// lcfa/photon_emission/mod.rs
double lcfa_photon_rate(double chi, double gamma);
double lcfa_classical_rate(double chi, double gamma);
void lcfa_photon_sample(double chi, double gamma, double r1, double r2, double r3, double* omega_mc2,
                        bool* has_theta, double* theta, double* cphi);
void lcfa_classical_sample(double chi, double gamma, double r1, double r2, double r3, double* omega_mc2,
                           bool* has_theta, double* theta, double* cphi);
Stokes lcfa_stokes_parameters(const V4& k, double chi, double gamma, V3 v, V3 w);
Stokes lcfa_classical_stokes_parameters(const V4& k, double chi, double gamma, V3 v, V3 w);
double gaunt_factor(double chi);

// lcfa/pair_creation/mod.rs
void lcfa_auxiliary_t(double chi, double* t_par, double* t_perp);
double lcfa_pair_probability(const V4& ell, const Stokes& sv, double chi, const V3& a_perp, double dt,
                             Stokes* sv_new);
double lcfa_pair_spectrum(double s, double chi, double sv1);
double lcfa_pair_spectrum_ceiling(double chi, double sv1);
double lcfa_pair_angular_spectrum(double y, double s, double chi, double sv1);
double lcfa_pair_angular_spectrum_ceiling(double s, double chi, double sv1);
// Returns false if a rejection loop hit its iteration cap.
bool lcfa_pair_sample(const V4& ell, const Stokes& sv, double chi, const V3& a_perp, DrawStream& rng,
                      double* gamma_p, double* cos_theta, double* phi, double* s_out, double* z_out);

// Iteration cap for every rejection loop (the reference's loops are
// unbounded; a particle that hits the cap is retired with an error code).
constexpr int REJECTION_CAP = 1 << 20;

}  // namespace orc
