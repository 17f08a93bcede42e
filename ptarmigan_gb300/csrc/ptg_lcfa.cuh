// LCFA quantum synchrotron emission and Breit-Wheeler pair creation on the
// device: rates per step, samplers per event.
//
// Follows lcfa/photon_emission/mod.rs and lcfa/pair_creation/mod.rs (cited
// per function).  The tables are the reference's, compiled into global
// memory from ptg_tables_small.h.
#pragma once
#include "ptg_math.cuh"

#define PTG_TABLE_DECL static __device__ const
#define PTG_TABLE_INF (__longlong_as_double(0x7ff0000000000000LL))
#include "../tables/ptg_tables_small.h"

namespace ptg {

// ------------------------------------------------------------- Airy ----
__device__ __forceinline__ double series_up_to(const double (*s)[20], double x) {
    double sum = 0.0;
    for (int k = 0; k < 20; ++k) {
        int p = (int)s[1][k];
        if (p >= 20) break;
        sum += s[0][k] * powi(x, p);
    }
    return sum;
}

// y^p for y > 0 as exp(p ln y): within a few ulp of pow(y, p) for the
// |p ln y| of a few units met here, at a fraction of pow's cost (pow
// carries its logarithm to extra precision).  The fractional powers of the
// Airy and Bessel functions below are taken this way, or as x sqrt(x) and
// cbrt(x)^2; the reference's powf and these agree to a few ulp.
__device__ __forceinline__ double pow_by_log(double y, double p) { return exp(p * log(y)); }
__device__ __forceinline__ double pow_two_thirds(double x) {
    double c = cbrt(x);
    return c * c;
}

// special_functions/airy.rs:41-78 (x >= 0)
static __device__ __noinline__ double airy_ai(double x) {
    if (x < 1.0) return series_up_to(PTG_AIRY_SMALL_X, x);
    double s = 2.0 * (x * sqrt(x)) / 3.0;
    double a = 0.262183997088323 * pow_by_log(s, -1.0 / 6.0) * exp(-s);
    const double *nodes, *weights;
    int n;
    if (x < 2.0) {
        nodes = PTG_GL_M16_NODES_40, weights = PTG_GL_M16_WEIGHTS_40, n = 40;
    } else if (x < 10.0) {
        nodes = PTG_GL_M16_NODES_16, weights = PTG_GL_M16_WEIGHTS_16, n = 16;
    } else {
        nodes = PTG_GL_M16_NODES_4, weights = PTG_GL_M16_WEIGHTS_4, n = 4;
    }
    double integral = 0.0;
    for (int k = 0; k < n; ++k) integral += weights[k] * pow_by_log(2.0 + nodes[k] / s, -1.0 / 6.0);
    return a * integral;
}

// special_functions/airy.rs:80-118 (x >= 0)
static __device__ __noinline__ double airy_ai_prime(double x) {
    if (x < 1.0) return series_up_to(PTG_AIRY_PRIME_SMALL_X, x);
    double s = 2.0 * (x * sqrt(x)) / 3.0;
    double b = -0.2898380090915846 * pow_by_log(s, 1.0 / 6.0) * exp(-s);
    const double *nodes, *weights;
    int n;
    if (x < 2.0) {
        nodes = PTG_GL_P16_NODES_32, weights = PTG_GL_P16_WEIGHTS_32, n = 32;
    } else if (x < 4.0) {
        nodes = PTG_GL_P16_NODES_16, weights = PTG_GL_P16_WEIGHTS_16, n = 16;
    } else if (x < 11.0) {
        nodes = PTG_GL_P16_NODES_8, weights = PTG_GL_P16_WEIGHTS_8, n = 8;
    } else {
        nodes = PTG_GL_P16_NODES_4, weights = PTG_GL_P16_WEIGHTS_4, n = 4;
    }
    double integral = 0.0;
    for (int k = 0; k < n; ++k) integral += weights[k] * pow_by_log(2.0 + nodes[k] / s, 1.0 / 6.0);
    return b * integral;
}

// airy.rs:120-136; negative arguments give 0 (the reference's None is
// unwrapped to 0 by every caller on this path).
__device__ __forceinline__ double bessel_k13(double x) {
    if (!(x >= 0.0)) return 0.0;  // powf(1.5 x, 2/3) is NaN there
    double y = pow_two_thirds(1.5 * x);
    return PI * cbrt(2.0 * SQRT_3 / x) * airy_ai(y);
}
__device__ __forceinline__ double bessel_k23(double x) {
    if (!(x >= 0.0)) return 0.0;
    double y = pow_two_thirds(1.5 * x);
    const double THREE_TO_MINUS_SIXTH = 0.83268317765560429;  // 3^(-1/6)
    return -PI * THREE_TO_MINUS_SIXTH * pow_two_thirds(2.0 / x) * airy_ai_prime(y);
}

// ------------------------------------------- quantum synchrotron rate ----
// lcfa/photon_emission/mod.rs:13-33, per second
__device__ __forceinline__ double lcfa_photon_rate(double chi, double gamma) {
    double h;
    if (chi < 0.01) {
        h = 5.0 * FRAC_PI_3 * (1.0 - 8.0 * chi / (5.0 * SQRT_3));
    } else if (chi >= 100.0) {
        double c = cbrt(chi);
        h = -1019.4661473121777 + 1786.716527650374 * c * c;
        h = 1750.6263395722715 + c * c * h;
        h = -2260.1819695887225 + c * h;
        h = 0.00296527643253334 * h / (chi * chi);
    } else {
        double index = (log(chi) - PTG_LCFA_LN_H_CHI_TABLE[0][0]) / PTG_LCFA_PH_DELTA_LN_CHI;
        double w = index - trunc(index);
        int i = (int)floor(index);
        double ln_h = (1.0 - w) * PTG_LCFA_LN_H_CHI_TABLE[i][1] + w * PTG_LCFA_LN_H_CHI_TABLE[i + 1][1];
        h = exp(ln_h);
    }
    return SQRT_3 * ALPHA_FINE * chi * h / (2.0 * PI * gamma * COMPTON_TIME);
}

__device__ __forceinline__ double lcfa_classical_rate(double chi, double gamma) {
    return SQRT_3 * ALPHA_FINE * chi * (5.0 * FRAC_PI_3) / (2.0 * PI * gamma * COMPTON_TIME);
}

// lcfa/photon_emission/mod.rs:35-69.  A CDF record is [coeff, power, 31x(x,f)].
__device__ __forceinline__ double from_linear_cdf_table(double global_zero, double local_zero, double rand,
                                                        const double* cdf) {
    double coeff = cdf[0], power = cdf[1];
    const double* tb = cdf + 2;
    double r_zero;
    if (local_zero < tb[0]) {
        r_zero = coeff * pow(local_zero - global_zero, power);
    } else {
        if (!pw_evaluate(tb, 31, false, local_zero, &r_zero)) return local_zero;
    }
    double r = r_zero + (1.0 - r_zero) * rand;
    double y;
    if (r <= tb[1]) {
        y = exp((log(r) - log(coeff)) / power) + global_zero;
    } else if (!pw_invert(tb, 31, false, r, &y)) {
        y = local_zero;
    }
    return y;
}

// lcfa/photon_emission/classical.rs:24-61
static __device__ __noinline__ void lcfa_classical_sample(double chi, double gamma, double rand1, double rand2,
                                                   double rand3, double* omega_mc2, double* theta) {
    double delta = acos((-9.0 + 50.0 * rand2 - 25.0 * (rand2 * rand2)) / 16.0);
    double z = powi((2.0 + 4.0 * cos(delta / 3.0)) / (5.0 * (1.0 - rand2)), 3);
    double ln_rand = log(rand1);
    const double* ct = &PTG_LCFA_CLASSICAL_SPECTRUM_TABLE[0][0];
    double x;
    if (ln_rand < ct[1]) {
        x = 1.020377255 * pow(rand1, 0.6);
    } else {
        double ln_x;
        if (!pw_invert(ct, 41, false, ln_rand, &ln_x)) ln_x = ct[2 * 40];
        x = exp(ln_x);
    }
    double u = 3.0 * chi * x / (2.0 * z);
    *omega_mc2 = u * gamma;
    double cos_theta = (gamma - pow(z, 2.0 / 3.0) / (2.0 * gamma)) / sqrt(gamma * gamma - 1.0);
    *theta = cos_theta >= 1.0 ? 0.0 : (cos_theta >= -1.0 ? acos(cos_theta) : -1.0);
}

// lcfa/photon_emission/mod.rs:80-231.  *theta < 0 encodes the reference's
// `None` (polar angle would exceed pi).
static __device__ __noinline__ void lcfa_photon_sample(double chi, double gamma, double rand1, double rand2, double rand3,
                                                double* omega_mc2, double* theta) {
    double lnchi = log(chi);
    if (lnchi <= PTG_LCFA_PH_LN_CHI_MIN) {
        double om;
        lcfa_classical_sample(chi, gamma, rand1, rand2, rand3, &om, theta);
        *omega_mc2 = om * gamma / (gamma + om);
        return;
    }
    double index = (lnchi - PTG_LCFA_PH_LN_CHI_MIN) / PTG_LCFA_PH_LN_CHI_STEP;
    double weight = index - trunc(index);
    int idx = (int)floor(index);
    double u;
    if (idx >= 40) {
        const double* hc = &PTG_LCFA_HIGH_CHI_CDF[0][0];
        const double* hp = &PTG_LCFA_HIGH_CHI_PEAK_CDF[0][0];
        double u_bdy = (chi - 8.0) / 8.0;
        double p_lower, p_higher, tmp;
        double lub = log(u_bdy);
        if (lub < hc[0]) {
            p_lower = 1.06327715546 * cbrt(u_bdy);
        } else if (lub < hc[62]) {
            pw_evaluate(hc, 32, false, lub, &tmp);
            p_lower = 1.0 - exp(-1.0 * exp(tmp));
        } else {
            p_lower = 1.0 - 0.265819288864 * pow(u_bdy, -2.0 / 3.0);
        }
        double y_bdy = u_bdy / chi - 1.0 / 9.0;
        double scale = 0.84626000931 * pow(chi, -2.0 / 3.0);
        double lyb = log(y_bdy);
        if (lyb < hp[0]) {
            p_higher = scale * (1.0 - 7.7567692587 * y_bdy);
        } else if (lyb < hp[62]) {
            pw_evaluate(hp, 32, true, lyb, &tmp);
            p_higher = scale * exp(-1.0 * exp(tmp));
        } else {
            p_higher = scale * 0.46534912384 * exp(-0.45 * u_bdy / chi) * pow(y_bdy, -5.0 / 3.0);
        }
        double r = rand1 * (p_lower + p_higher);
        if (r <= p_lower) {
            double target = log(-log(1.0 - r));
            if (target < hc[1]) {
                double uu = powi(r / 1.06327715546, 3);
                u = uu + 1.5 * uu * uu;
            } else if (target < hc[63]) {
                pw_invert(hc, 32, false, target, &tmp);
                u = exp(tmp);
            } else {
                u = pow(0.265819288864 / (1.0 - r), 1.5);
            }
        } else {
            double target = (p_lower + p_higher - r) / scale;
            double y;
            if (target < hp[1]) {
                y = (1.0 - target) / 7.7567692587;
            } else {
                pw_invert(hp, 32, true, log(-1.0 * log(target)), &tmp);
                y = exp(tmp);
            }
            u = (y + 1.0 / 9.0) * chi;
        }
    } else {
        const double* lo = PTG_LCFA_QUANTUM_CDF[idx];
        const double* up = PTG_LCFA_QUANTUM_CDF[idx + 1];
        double lr = log(rand1);
        double ln_lo, ln_up;
        if (lr <= lo[3]) {
            ln_lo = (lr - log(lo[0])) / lo[1];
        } else if (!pw_invert(lo + 2, 31, false, lr, &ln_lo)) {
            ln_lo = lo[2 + 60];
        }
        if (lr <= up[3]) {
            ln_up = (lr - log(up[0])) / up[1];
        } else if (!pw_invert(up + 2, 31, false, lr, &ln_up)) {
            ln_up = up[2 + 60];
        }
        u = exp((1.0 - weight) * ln_lo + weight * ln_up);
    }

    double beta = 2.0 * u / (3.0 * chi);
    double delta = (1.0 + (1.0 + u) * (1.0 + u)) * pow(beta, -2.0 / 3.0) / (1.0 + u);
    double dindex = (log(delta) - PTG_LCFA_PH_LN_DELTA_MIN) / PTG_LCFA_PH_LN_DELTA_STEP;
    double dweight = dindex - trunc(dindex);
    double dfl = floor(dindex);
    int di = dfl < 0.0 ? 0 : (int)dfl;
    double y;
    if (di >= 30) {
        y = from_linear_cdf_table(0.0, beta, rand2, PTG_LCFA_Y_INFINITE_DELTA_CDF);
    } else {
        double gz = pow(delta, -1.5);
        double y_lo = from_linear_cdf_table(gz, beta, rand2, PTG_LCFA_Y_CDF[di]);
        double y_up = from_linear_cdf_table(gz, beta, rand2, PTG_LCFA_Y_CDF[di + 1]);
        y = (1.0 - dweight) * y_lo + dweight * y_up;
    }
    double z = fmax(y / beta, 1.0);
    double cos_theta = (gamma - pow(z, 2.0 / 3.0) / (2.0 * gamma)) / sqrt(gamma * gamma - 1.0);
    *theta = cos_theta >= 1.0 ? 0.0 : (cos_theta >= -1.0 ? acos(cos_theta) : -1.0);
    *omega_mc2 = gamma * u / (1.0 + u);
}

// lcfa/photon_emission/mod.rs:239-298 (quantum) and classical.rs:70-118.
// Returns [Q, U, V] with I = 1.
static __device__ __noinline__ d3 lcfa_stokes(d4 k, double chi, double gamma, d3 v, d3 w, bool classical) {
    v = normalize(v);
    w = normalize(w);
    d3 n = normalize(mk3(k.x, k.y, k.z));
    double u = classical ? k.t / gamma : k.t / (gamma - k.t);
    double beta = asin(dot(n, normalize(cross(v, w))));
    double mu = sqrt(beta * beta + 1.0 / (gamma * gamma));
    double gm = gamma * mu;
    double eta = u * (gm * gm * gm) / (3.0 * chi);
    double k13 = bessel_k13(eta);
    double k23 = bessel_k23(eta);
    double a = mu * k23, b = beta * k13;
    double g, xi0, xi2;
    if (classical) {
        g = b * b + a * a;
        xi0 = (a * a - b * b) / g;
        xi2 = 2.0 * beta * mu * k13 * k23 / g;
    } else {
        double um = u * mu;
        g = 0.5 * (um * um) * (k13 * k13 + k23 * k23) / (1.0 + u) + a * a + b * b;
        xi0 = (a * a - b * b) / g;
        xi2 = 2.0 * (1.0 + 0.5 * u * u / (1.0 + u)) * beta * mu * k13 * k23 / g;
    }
    double phi;
    if (classical) {
        phi = asin((w - dot(n, w) * n).y);
    } else {
        d3 e1 = mk3(k.z, 0.0, -k.x);
        e1 = (norm_sqr(e1) == 0.0) ? mk3(1.0, 0.0, 0.0) : normalize(e1);
        phi = acos(fmin(fmax(dot(e1, w), -1.0), 1.0));
        phi = dsign(dot(cross(w, e1), n)) * phi;
    }
    double s2, c2;
    sincos(2.0 * phi, &s2, &c2);
    return mk3(c2 * xi0, -s2 * xi0, xi2);
}

// lcfa/photon_emission/mod.rs:330-346 (modified Landau-Lifshitz)
static __device__ __noinline__ double gaunt_factor(double chi) {
    if (chi <= 1.0e-3) return 1.0 - 55.0 * SQRT_3 * chi / 16.0 + 48.0 * chi * chi;
    if (chi > 500.0) {
        double c = cbrt(chi);
        double g = -1.0000341464898563 + 0.5563810015417746 * c * c;
        g = 2.6235881916750565 + c * c * g;
        g = -3.8106418922532588 + c * g;
        return g / (chi * chi * chi);
    }
    double v = 0.0;
    pw_evaluate(&PTG_LCFA_GAUNT_FACTOR_TABLE[0][0], 25, false, log(chi), &v);
    return exp(v);
}

// ------------------------------------------------- pair creation ---------
// lcfa/pair_creation/mod.rs:13-40
__device__ __forceinline__ void lcfa_auxiliary_t(double chi, double* t_par, double* t_perp) {
    const double(*T)[3] = PTG_LCFA_LN_T_CHI_TABLE;
    const double D = PTG_LCFA_PAIR_DELTA_LN_CHI;
    if (chi <= 0.01) {
        *t_par = 0.0, *t_perp = 0.0;
    } else if (chi < 1.0) {
        int i = (int)((log(chi) - T[0][0]) / D);
        double e0 = exp(T[i][0]), e1 = exp(T[i + 1][0]);
        double dx = (chi - e0) / (e1 - e0);
        double par = (1.0 - dx) / T[i][1] + dx / T[i + 1][1];
        double perp = (1.0 - dx) / T[i][2] + dx / T[i + 1][2];
        *t_par = exp(1.0 / par), *t_perp = exp(1.0 / perp);
    } else if (chi < 100.0) {
        double lc = log(chi);
        int i = (int)((lc - T[0][0]) / D);
        double dx = (lc - T[i][0]) / D;
        *t_par = exp((1.0 - dx) * T[i][1] + dx * T[i + 1][1]);
        *t_perp = exp((1.0 - dx) * T[i][2] + dx * T[i + 1][2]);
    } else {
        double c = cbrt(chi);
        *t_par = 0.3036898468348568 / c - 2.0 / (3.0 * chi);
        *t_perp = 0.4555347702522852 / c - 2.0 / (3.0 * chi);
    }
}

// polarization.rs:58-97: Stokes parameters in the basis with principal
// axis a (perpendicular to k); also returns cos 2θ, sin 2θ.
__device__ __forceinline__ d4 stokes_in_basis(d4 sv, d3 a, d3 k, double* c2, double* s2) {
    double k_mag = hypot(k.x, k.z);
    double a_mag = sqrt(norm_sqr(a));
    double ct = (k_mag == 0.0) ? a.x / a_mag : (k.z * a.x - k.x * a.z) / (k_mag * a_mag);
    double det = (k_mag == 0.0) ? (-k.y * a.z + k.z * a.y) : (a.y * (k.x * k.x + k.z * k.z) - k.y * (a.x * k.x + a.z * k.z));
    double sign = -dsign(det);
    ct = fmin(fmax(ct, -1.0), 1.0);
    double st = sign * sqrt(1.0 - ct * ct);
    *c2 = ct * ct - st * st;
    *s2 = 2.0 * ct * st;
    return d4{sv.t, *c2 * sv.x - *s2 * sv.y, *s2 * sv.x + *c2 * sv.y, sv.z};
}

// lcfa/pair_creation/mod.rs:48-73.  Returns the probability; *sv_new is the
// photon's Stokes vector if no pair is created.
__device__ __forceinline__ double lcfa_pair_probability(d4 ell, d4 sv_in, double chi, d3 a_perp, double dt,
                                                        d4* sv_new) {
    double c2, s2;
    d4 sv = stokes_in_basis(sv_in, a_perp, mk3(ell.x, ell.y, ell.z), &c2, &s2);
    double tpar, tperp;
    lcfa_auxiliary_t(chi, &tpar, &tperp);
    double pre = ALPHA_FINE * chi * dt / (COMPTON_TIME * ell.t);
    double prob = ALPHA_FINE * chi * (0.5 * (1.0 + sv.x) * tpar + 0.5 * (1.0 - sv.x) * tperp) * dt / (COMPTON_TIME * ell.t);
    double prob_avg = ALPHA_FINE * chi * 0.5 * (tpar + tperp) * dt / (COMPTON_TIME * ell.t);
    double delta = ALPHA_FINE * chi * 0.5 * (tpar - tperp) * dt / (COMPTON_TIME * ell.t);
    (void)pre;
    double sv1 = (sv.x * (1.0 - prob_avg) - delta) / (1.0 - prob);
    double sv2 = sv.y * (1.0 - prob_avg) / (1.0 - prob);
    *sv_new = d4{sv.t, c2 * sv1 + s2 * sv2, -s2 * sv1 + c2 * sv2, sv.z * (1.0 - prob_avg) / (1.0 - prob)};
    return prob;
}

// Per-node constants of the Gauss-Laguerre pair spectrum
// (lcfa/pair_creation/mod.rs:80-89): w, t, cosh(2t/3), cosh(t/3)/cosh(t),
// cosh(t).  Filled once by the host.
struct PairGL {
    double w[32], t[32], c23[32], c13_over_c1[32], c1[32];
    // FP32 copies of the per-step rate tables (ln h(chi) and ln T(chi))
    float ln_h32[41][2];
    float ln_t32[81][3];
};

// lcfa/pair_creation/mod.rs:80-89
__device__ __forceinline__ double lcfa_pair_spectrum(double s, double chi, double sv1, const PairGL& gl) {
    double ss = s * (1.0 - s);
    double xi = 2.0 / (3.0 * chi * ss);
    double a = 1.0 / ss - sv1 - 2.0;
    double sum = 0.0;
#pragma unroll 4
    for (int k = 0; k < 32; ++k) {
        double pre = exp(-xi * gl.c1[k] + gl.t[k]);
        sum += gl.w[k] * pre * (a * gl.c23[k] + gl.c13_over_c1[k]);
    }
    return sum;
}

// lcfa/pair_creation/mod.rs:93-110
__device__ __forceinline__ double lcfa_pair_spectrum_ceiling(double chi, double sv1, const PairGL& gl) {
    double chi_switch = exp((1.5 - sv1) / SQRT_3);
    double mx;
    if (chi < chi_switch) {
        mx = lcfa_pair_spectrum(0.5, chi, sv1, gl);
    } else if (chi > 100.0) {
        mx = lcfa_pair_spectrum(4.0 / (3.0 * chi), chi, sv1, gl);
    } else {
        double m = -0.94866 + 0.170159 * sv1;
        mx = lcfa_pair_spectrum(0.5 * pow(chi_switch, -m) * pow(chi, m), chi, sv1, gl);
    }
    return 1.05 * mx;
}

// lcfa/pair_creation/mod.rs:115-126
__device__ __forceinline__ double lcfa_pair_angular_spectrum(double y, double s, double chi, double sv1) {
    double xi = 2.0 / (3.0 * chi * s * (1.0 - s));
    double pre = s / (1.0 - s) + (1.0 - s) / s - sv1;
    double z = 1.0 + 4.0 * chi * y * y;
    return y * (1.0 + pre * pow(z, 2.0 / 3.0)) * bessel_k13(xi * z);
}

// lcfa/pair_creation/mod.rs:130-141
__device__ __forceinline__ double lcfa_pair_angular_ceiling(double s, double chi, double sv1) {
    double y_peak = 0.216 + (0.259 - 0.216) * (1.0 - tanh(pow(8.3 / chi, 2.0 / 3.0)));
    double q = 1.0 - 2.0 * s;
    double y = y_peak * sqrt(1.0 - q * q);
    return 1.05 * lcfa_pair_angular_spectrum(y, s, chi, sv1);
}

// lcfa/pair_creation/mod.rs:180-217 with :141-173.  Returns false if a
// rejection loop reached its cap.
static __device__ __noinline__ bool lcfa_pair_sample(d4 ell, d4 sv_in, double chi, d3 a_perp, Draws& rng, const PairGL& gl,
                                              double* gamma_p, double* cos_theta, double* phi, uint32_t* rejections) {
    double c2, s2;
    d4 sv = stokes_in_basis(sv_in, a_perp, mk3(ell.x, ell.y, ell.z), &c2, &s2);
    double mx = lcfa_pair_spectrum_ceiling(chi, sv.x, gl);
    double s = 0.0;
    int it;
    for (it = 0; it < rng.cap; ++it) {
        double ss = rng.next(), u = rng.next();
        if (u <= lcfa_pair_spectrum(ss, chi, sv.x, gl) / mx) {
            s = ss;
            break;
        }
    }
    *rejections += it;
    if (it == rng.cap) return false;
    double amx = lcfa_pair_angular_ceiling(s, chi, sv.x);
    double z = 1.0;
    for (it = 0; it < rng.cap; ++it) {
        double y = rng.next(), u = rng.next();
        if (u <= lcfa_pair_angular_spectrum(y, s, chi, sv.x) / amx) {
            z = 1.0 + 4.0 * chi * y * y;
            break;
        }
    }
    *rejections += it;
    if (it == rng.cap) return false;
    // azimuth (lcfa/pair_creation/mod.rs:141-173)
    double arg = 2.0 * z / (3.0 * chi * s * (1.0 - s));
    double k_ratio = (arg < 1.0e-4) ? 0.6368498843179743 / cbrt(arg)
                                    : 1.0 + 1.0 / (1.4624087952220928 * cbrt(arg) + 1.023821552056939 * sqrt(arg) + 6.0 * arg);
    double z23 = pow(z, 2.0 / 3.0);
    double s1 = s * s + (1.0 - s) * (1.0 - s);
    double A = 1.0 + z23 * s1 / (s * (1.0 - s));
    double Cc = z23, Dd = z23 - 1.0;
    double Ee = pow(z, 1.0 / 3.0) * (z23 - 1.0) * s1 * k_ratio / (s * (1.0 - s));
    double amax = -HUGE_VAL;
    for (int i = 0; i < 32; ++i) {
        double p = 2.0 * PI * i / 32.0;
        double f = A + (cos(2.0 * p) * (1.0 - Cc) - Cc) * sv.x - Dd * sin(2.0 * p) * sv.y + Ee * sin(p) * sv.z;
        amax = fmax(amax, f);
    }
    amax *= 1.1;
    double ph = 0.0;
    for (it = 0; it < rng.cap; ++it) {
        double p = 2.0 * PI * rng.next();
        double u = rng.next();
        double f = A + (cos(2.0 * p) * (1.0 - Cc) - Cc) * sv.x - Dd * sin(2.0 * p) * sv.y + Ee * sin(p) * sv.z;
        if (u <= f / amax) {
            ph = p;
            break;
        }
    }
    *rejections += it;
    if (it == rng.cap) return false;
    double gp = s * ell.t;
    double ct = (2.0 * gp * gp - z23) / (2.0 * gp * gp - 1.0);
    *gamma_p = gp;
    *cos_theta = fmax(ct, -1.0);
    *phi = ph;
    return true;
}

}  // namespace ptg
