// LMA nonlinear Breit-Wheeler pair creation on the device (circular
// polarisation): the double-differential partial rate, its integral, the
// total rate by table lookup or by explicit harmonic summation, the Stokes
// update of a photon that survives a step, and the positron sampler with its
// zero-momentum-frame kinematics.
//
// Follows pair_creation/cp/mod.rs and pair_creation/mod.rs (cited per
// function).  FP64: the probability is accumulated in FP64 and the rates
// span hundreds of orders of magnitude.
#pragma once
#include "ptg_nlc.cuh"

namespace ptg {

constexpr double PAIR_LASER_S3 = -1.0;

// pair_creation/cp/mod.rs:38-43
__device__ __forceinline__ void bw_s_bounds(int n, double a, double eta, double* s_min, double* s_max) {
    double sn = 2.0 * n * eta / (1.0 + a * a);
    *s_min = fmin(0.5 * (1.0 - sqrt(1.0 - 4.0 / sn)), 0.5);
    *s_max = 0.5;
}

// pair_creation/cp/mod.rs:47-64
__device__ __forceinline__ void bw_elements(int n, double a, double eta, double s, double* unpol, double* d12,
                                            double* d3) {
    double ell = n;
    double a2 = a * a;
    double sn = 2.0 * ell * eta / (1.0 + a2);
    double tmp = 1.0 / (sn * s * (1.0 - s));
    double z = sqrt((4.0 * ell * ell) * (a2 / (1.0 + a2)) * tmp * (1.0 - tmp));
    double jm, j, jp;
    j_pm(z, n, &jm, &j, &jp);
    double q = (1.0 - s) / s + s / (1.0 - s);
    double la = ell * a / z;
    *unpol = j * j + 0.25 * a2 * q * (jm * jm + jp * jp - 2.0 * j * j);
    *d12 = (2.0 * la * la - (1.0 + a2)) * j * j - 0.5 * a2 * (jm * jm + jp * jp);
    *d3 = 0.25 * a2 * q * (1.0 - 2.0 / (sn * s * (1.0 - s))) * (jm * jm - jp * jp);
}

// pair_creation/cp/mod.rs:66-72.  (2 theta).sin_cos() returns (sin, cos)
// and the reference names them (cos_2theta, sin_2theta) in that order.
__device__ __forceinline__ double bw_fully_resolved(int n, double a, double eta, double s, double theta, double sv1,
                                                    double sv2, double sv3) {
    double unpol, d12, d3;
    bw_elements(n, a, eta, s, &unpol, &d12, &d3);
    double sn2, cs2;
    sincos(2.0 * theta, &sn2, &cs2);
    return (unpol - (sv1 * sn2 + sv2 * cs2) * d12 - PAIR_LASER_S3 * sv3 * d3) / (2.0 * PI);
}

// pair_creation/cp/mod.rs:74-87: [S3 = +1, S3 = -1] components
__device__ __forceinline__ void bw_over_theta(int n, double a, double eta, double s, double* re, double* im) {
    double unpol, d12, d3;
    bw_elements(n, a, eta, s, &unpol, &d12, &d3);
    *re = unpol - PAIR_LASER_S3 * d3;
    *im = unpol + PAIR_LASER_S3 * d3;
}

// pair_creation/cp/mod.rs:92-186: integral over s and theta, both S3 parts
static __device__ __noinline__ void bw_integrate(int n, double a, double eta, double* out_re, double* out_im) {
    double ell = n;
    double sn = 2.0 * ell * eta / (1.0 + a * a);
    *out_re = 0.0, *out_im = 0.0;
    if (sn <= 4.0) return;
    double a2 = a * a;
    double w1 = 1.0 / ell + 1.0;
    double beta = a2 * a2 * w1 * w1 + 16.0 * (a2 - 2.0) * (a2 - 2.0) / (sn * sn) - 8.0 * a2 * (a2 - 2.0) / sn;
    beta = sqrt(beta) / (a2 - 2.0);
    double alpha = (a2 + 2.0 * ell) / (ell * (2.0 - a2)) - 4.0 / sn;
    double s_peak = 0.5 * (1.0 - sqrt(alpha + beta));
    double s_min, s_max;
    bw_s_bounds(n, a, eta, &s_min, &s_max);
    double lo[3], hi[3];
    int nseg;
    if (isfinite(s_peak)) {
        double s_mid = 2.0 * s_peak - s_min;
        if (s_mid > s_max) {
            nseg = 2;
            lo[0] = s_min, hi[0] = s_peak, lo[1] = s_peak, hi[1] = s_max;
        } else {
            nseg = 3;
            lo[0] = s_min, hi[0] = s_peak, lo[1] = s_peak, hi[1] = s_mid, lo[2] = s_mid, hi[2] = s_max;
        }
    } else {
        nseg = 1;
        lo[0] = s_min, hi[0] = s_max;
    }
    double tr = 0.0, ti = 0.0;
    for (int g = 0; g < nseg; ++g) {
        double r = 0.0, i = 0.0;
        double h = 0.5 * (hi[g] - lo[g]), m = 0.5 * (lo[g] + hi[g]);
        for (int k = 0; k < 32; ++k) {
            double sr, si;
            bw_over_theta(n, a, eta, h * PTG_GAUSS_32_NODES[k] + m, &sr, &si);
            r += h * PTG_GAUSS_32_WEIGHTS[k] * sr;
            i += h * PTG_GAUSS_32_WEIGHTS[k] * si;
        }
        tr += r, ti += i;
    }
    *out_re = 2.0 * tr, *out_im = 2.0 * ti;
}

// pair_creation/cp/mod.rs:349-365
__device__ __forceinline__ void bw_sum_limits(double a, double eta, int* n_min, int* n_max) {
    double nm = ceil(2.0 * (1.0 + a * a) / eta);
    double range = 2.0 * (0.25 + a * a) / eta + 13.0 * a * (2.0 + a);
    double test = 0.25 - (1.0 + a * a) / (2.0 * nm * eta);
    if (test <= 2.220446049250313e-16) {
        *n_min = (int)nm + 1;
        *n_max = (int)(nm + 1.0 + range);
    } else {
        *n_min = (int)nm;
        *n_max = (int)(nm + range);
    }
}

// pair_creation/cp/mod.rs:363-365: rate below exp(-200)
__device__ __forceinline__ bool bw_is_too_small(double a, double eta) {
    double q = log10(a) + 2.0;
    return log10(eta) < -1.0 - q * q / 4.5;
}

// The same decision, taken in FP32 wherever the two sides differ by more
// than 1e-3 (their FP32 rounding is below 1e-6), else in FP64: the same
// answer as bw_is_too_small at every (a, eta).
__device__ __forceinline__ bool bw_is_too_small_fast(double a, double eta) {
    float q = log10f((float)a) + 2.0f;
    float d = log10f((float)eta) - (-1.0f - q * q / 4.5f);
    if (d < -1e-3f) return true;
    if (d > 1e-3f) return false;
    return bw_is_too_small(a, eta);
}

// pair_creation/cp/mod.rs:385-393
static __device__ __noinline__ void bw_by_summation(double a, double eta, double* f0, double* f1) {
    int n0, n1;
    bw_sum_limits(a, eta, &n0, &n1);
    double re = 0.0, im = 0.0;
    for (int n = n0; n <= n1; ++n) {
        double r, i;
        bw_integrate(n, a, eta, &r, &i);
        re += r, im += i;
    }
    *f0 = re, *f1 = im;
}

// pair_creation/cp/mod.rs:395-448; false where the reference panics
// `nodes`, when not NULL, holds the table's node positions exp(LN_MIN_A + i
// LN_A_STEP), i < 74, then exp(LN_MIN_ETA + j LN_ETA_STEP), j < 121,
// evaluated once when the tables are loaded.
static __device__ __noinline__ bool bw_by_lookup(const double* T, double a, double eta, double* f0, double* f1,
                                                 const double* nodes = nullptr) {
    const double LMA = PTG_BW_CP_LN_MIN_A, LME = PTG_BW_CP_LN_MIN_ETA, SA = PTG_BW_CP_LN_A_STEP, SE = PTG_BW_CP_LN_ETA_STEP;
    const int NC = 74, NR = 121;
    double x = log(a), y = log(eta);
    if (x < LMA) return false;
    if (y < LME) {
        *f0 = *f1 = 0.0;
        return true;
    }
    int ix = (int)((x - LMA) / SA), iy = (int)((y - LME) / SE);
    if (!(ix < NC - 1 && iy < NR - 1)) return false;
    const double* p00 = T + ((size_t)iy * NC + ix) * 2;
    const double* p01 = p00 + 2;
    const double* p10 = p00 + 2 * NC;
    const double* p11 = p10 + 2;
    double f[2];
    if (a * eta > 2.0) {
        double dx = (x - LMA) / SA - ix, dy = (y - LME) / SE - iy;
        double w0 = (1.0 - dx) * (1.0 - dy), w1 = dx * (1.0 - dy), w2 = (1.0 - dx) * dy, w3 = dx * dy;
        for (int k = 0; k < 2; ++k) f[k] = exp(w0 * p00[k] + w1 * p01[k] + w2 * p10[k] + w3 * p11[k]);
    } else {
        double a_min, a_max, e_min, e_max;
        if (nodes != nullptr) {
            a_min = nodes[ix], a_max = nodes[ix + 1];
            e_min = nodes[NC + iy], e_max = nodes[NC + iy + 1];
        } else {
            a_min = exp(LMA + ix * SA), a_max = exp(LMA + (ix + 1) * SA);
            e_min = exp(LME + iy * SE), e_max = exp(LME + (iy + 1) * SE);
        }
        double dx = (a - a_min) / (a_max - a_min), dy = (eta - e_min) / (e_max - e_min);
        double w0 = (1.0 - dx) * (1.0 - dy), w1 = dx * (1.0 - dy), w2 = (1.0 - dx) * dy, w3 = dx * dy;
        for (int k = 0; k < 2; ++k) f[k] = exp(1.0 / (w0 / p00[k] + w1 / p01[k] + w2 / p10[k] + w3 / p11[k]));
    }
    *f0 = f[0], *f1 = f[1];
    return true;
}

// A bound on each component of bw_by_summation's result, in closed form.
// For x >= 0 and m >= 0, |J_m(x)| <= (x/2)^m / m!.  The integrand of
// bw_integrate is at most J_n^2 (1 + k) + k (J_{n-1}^2 + J_{n+1}^2) with
// k = a^2 q / 2, the Bessel argument is at most n c with c = a / sqrt(1 +
// a^2), and the quadrature weights of a harmonic sum to s_max - s_min <=
// 1/2 while bw_integrate doubles the sum.  With u_n = (n c / 2)^n / n!,
// J_{n-1} <= u_n 2 / c, J_n <= u_n and J_{n+1} <= u_n c / 2, so harmonic n
// contributes at most u_n^2 (1 + k_n K) with K = 1 + 4 / c^2 + c^2 / 4.
// q falls as s_min rises and s_min >= 1 / s_n, so q <= 1 + beta n with
// beta = 2 eta / (1 + a^2).  u_{n+1} / u_n = (c / 2)(1 + 1/n)^n < r = e c
// / 2, and n! >= sqrt(2 pi n) (n / e)^n gives u_{n0} <= r^n0 / sqrt(2 pi
// n0).  Summing over every n >= n0 (bw_sum_limits' first harmonic) with
// rho = r^2 < 1 (a < 0.3 here: rho < 0.16):
//   sum <= r^(2 n0) / (2 pi n0) [(A + B n0) / (1 - rho) + B rho / (1 - rho)^2]
// with A = 1 + a^2 K / 2 and B = a^2 K beta / 2.  One exponential and one
// logarithm, where a harmonic-by-harmonic bound would take one of each and
// a log-gamma per harmonic.
__device__ __forceinline__ double bw_summation_bound(double a, double eta) {
    int n0, n1;
    bw_sum_limits(a, eta, &n0, &n1);
    double a2 = a * a;
    double c = a / sqrt(1.0 + a2);
    double r = 0.5 * 2.718281828459045 * c;
    double rho = r * r;
    if (!(rho < 1.0)) return HUGE_VAL;
    double K = 1.0 + 4.0 / (c * c) + 0.25 * c * c;
    double beta = 2.0 * eta / (1.0 + a2);
    double A = 1.0 + 0.5 * a2 * K, B = 0.5 * a2 * K * beta;
    double n = (double)n0;
    double lead = exp(2.0 * n * log(r)) / (2.0 * PI * n);
    double om = 1.0 - rho;
    return lead * ((A + B * n) / om + B * rho / (om * om));
}

// Per-step pair probabilities below this, after the event biasing
// (p max(1, rate_increase)), are taken as zero where the rate would
// otherwise be summed harmonic by harmonic.  Then no uniform draw passes
// p ri but an exact zero (draws are multiples of 2^-53), the Stokes
// factors (1 - p_avg) / (1 - p) of bw_probability round to exactly 1 (p is
// below half an ulp of 1), the Stokes vector's third component moves by
// less than 2^-54, and the interaction count by less than 2^-54 per step.
constexpr double PAIR_PROB_NEGLIGIBLE = 0x1p-54;

// exp(LN_MIN_A) of the CP total-rate table, the smallest amplitude it covers,
// as the host's libm rounds it (0.3); evaluating it on every step cost an
// FP64 exponential.
constexpr double BW_CP_MIN_A = 0.3;

// TotalRate::value / probability dispatch (pair_creation/cp/mod.rs:265-287)
__device__ __forceinline__ bool bw_rates(const double* T, double a, double eta, double* f0, double* f1) {
    if (a < 0.02 || bw_is_too_small(a, eta)) {
        *f0 = *f1 = 0.0;
        return true;
    }
    if (a < BW_CP_MIN_A) {
        bw_by_summation(a, eta, f0, f1);
        return true;
    }
    return bw_by_lookup(T, a, eta, f0, f1);
}

// Work of a photon step left by its lane for the whole warp (the wave
// kernel and the single-collision queue kernel), in two kinds:
//   BW_DEFER_RATE: the CP Breit-Wheeler rate needs the harmonic sum; the
//     lane records a and eta; the warp sums the harmonics with one
//     Gauss-Legendre node per lane (bw_by_summation_warp);
//   BW_DEFER_HARMONIC: a pair is created and its harmonic is sampled; the
//     lane records a, eta, S3 and its uniform draw; the warp walks the
//     harmonics' cumulative sum (bw_sample_harmonic_warp) and evaluates the
//     ceiling of the s spectrum for the harmonic it finds.
// The lane abandons the step and repeats it once served; the repeat draws
// the same numbers, reaches the same request and takes the warp's result.
constexpr int BW_DEFER_RATE = 1;
constexpr int BW_DEFER_HARMONIC = 2;
struct BwDefer {
    double a, eta, sv3, u;  // the request
    double f0, f1, s_ceil;  // the results: the rates and the s ceiling
    int n;                  // the sampled harmonic, -1 out of table
    int kind;
    int pend;  // 0: none; 1: waiting for the warp; 2: served
};

// Status of bw_probability and bw_sample for a step left to the warp
constexpr int BW_DEFERRED = -1;

// pair_creation/cp/mod.rs:199-207: the largest of the theta-integrated
// spectrum's values at the 32 Gauss-Legendre nodes over [s_min, 1/2] (NaN
// values are passed over, as f64::max does)
__device__ __forceinline__ double bw_s_node_value(int n, double a, double eta, double sv3, int k) {
    double s_min, s_max;
    bw_s_bounds(n, a, eta, &s_min, &s_max);
    double s = 0.5 * (s_max - s_min) * PTG_GAUSS_32_NODES[k] + 0.5 * (s_min + s_max);
    double re, im;
    bw_over_theta(n, a, eta, s, &re, &im);
    return 0.5 * (re * (1.0 + sv3) + im * (1.0 - sv3));
}

static __device__ __noinline__ double bw_s_ceiling(int n, double a, double eta, double sv3) {
    double mx = __longlong_as_double(0x7ff8000000000000LL);
    for (int k = 0; k < 32; ++k) mx = fmax(mx, bw_s_node_value(n, a, eta, sv3, k));
    return mx;
}

// pair_creation/cp/mod.rs:191-243: s by rejection on the theta-integrated
// spectrum under 1.5 x `ceil` (bw_s_ceiling), the side of s = 1/2, then
// theta by rejection.
static __device__ __noinline__ int bw_sample_s_theta(int n, double a, double eta, double sv1, double sv2, double sv3,
                                                     double ceil, Draws& rng, double* s_out, double* theta_out,
                                                     uint32_t* rej) {
    double s_min, s_max;
    bw_s_bounds(n, a, eta, &s_min, &s_max);
    double mx = 1.5 * ceil;
    double s = 0.0;
    int it;
    for (it = 0; it < rng.cap; ++it) {
        double ss = s_min + (s_max - s_min) * rng.next();
        double z = mx * rng.next();
        double re, im;
        bw_over_theta(n, a, eta, ss, &re, &im);
        if (z < 0.5 * (re * (1.0 + sv3) + im * (1.0 - sv3))) {
            s = ss;
            break;
        }
    }
    *rej += it;
    if (it == rng.cap) return 4;
    if (rng.next() < 0.5) s = 1.0 - s;
    double theta_opt = 0.5 * atan2(sv2, sv1);
    double tm = -HUGE_VAL;
    for (int i = 0; i < 4; ++i) tm = fmax(tm, bw_fully_resolved(n, a, eta, s, theta_opt + i * FRAC_PI_2, sv1, sv2, sv3));
    tm *= 1.01;
    double theta = 0.0;
    for (it = 0; it < rng.cap; ++it) {
        double th = 2.0 * PI * rng.next();
        double z = tm * rng.next();
        if (z < bw_fully_resolved(n, a, eta, s, th, sv1, sv2, sv3)) {
            theta = th;
            break;
        }
    }
    *rej += it;
    if (it == rng.cap) return 4;
    *s_out = s;
    *theta_out = theta;
    return 0;
}

// pair_creation/cp/mod.rs:314-346: harmonic by explicit summation.  With
// `bdf`, the harmonic and the s ceiling are left to the warp
// (BW_DEFER_HARMONIC): returns BW_DEFERRED until the warp has served them.
static __device__ __noinline__ int bw_sample(const double* T, double a, double eta, double sv1, double sv2, double sv3,
                                             Draws& rng, int* n_out, double* s, double* theta, uint32_t* rej,
                                             BwDefer* bdf = nullptr) {
    double u = rng.next();
    int index;
    double ceil;
    if (bdf != nullptr) {
        if (!(bdf->pend == 2 && bdf->kind == BW_DEFER_HARMONIC && bdf->a == a && bdf->eta == eta && bdf->sv3 == sv3 &&
              bdf->u == u)) {
            bdf->a = a, bdf->eta = eta, bdf->sv3 = sv3, bdf->u = u;
            bdf->kind = BW_DEFER_HARMONIC;
            bdf->pend = 1;
            return BW_DEFERRED;
        }
        bdf->pend = 0;
        if (bdf->n < 0) return 2;
        index = bdf->n;
        ceil = bdf->s_ceil;
    } else {
        int n0, n1;
        bw_sum_limits(a, eta, &n0, &n1);
        double f0, f1;
        if (!bw_rates(T, a, eta, &f0, &f1)) return 2;
        double target = 0.5 * (f0 * (1.0 + sv3) + f1 * (1.0 - sv3)) * u;
        double cum = 0.0;
        index = -1;
        for (int k = n0; k <= n1; ++k) {
            double re, im;
            bw_integrate(k, a, eta, &re, &im);
            cum += 0.5 * ((1.0 + sv3) * re + (1.0 - sv3) * im);
            if (cum > target) {
                index = k;
                break;
            }
        }
        if (index == -1) index = n1 - 1;
        ceil = bw_s_ceiling(index, a, eta, sv3);
    }
    *n_out = index;
    return bw_sample_s_theta(index, a, eta, sv1, sv2, sv3, ceil, rng, s, theta, rej);
}

// polarization.rs:101-130: Stokes parameters in the LMA basis
__device__ __forceinline__ d4 stokes_in_lma_basis(d4 sv, d4 k) {
    StokesBasis b = lma_stokes_basis(k);
    d3 g = stokes_rotate_cs(mk3(sv.x, sv.y, sv.z), b.c2, b.s2);
    return d4{sv.t, g.x, g.y, g.z};
}

// polarization.rs:132-141.  At theta = +-0 (the default polarisation angle)
// sincos(2 theta) is (+-0, 1) exactly, so the call is skipped.
__device__ __forceinline__ d4 stokes_rotate_by(d4 sv, double theta) {
    double s2, c2;
    if (theta == 0.0) {
        s2 = 2.0 * theta;
        c2 = 1.0;
    } else {
        sincos(2.0 * theta, &s2, &c2);
    }
    return d4{sv.t, c2 * sv.x + s2 * sv.y, -s2 * sv.x + c2 * sv.y, sv.z};
}

// Lane k's share of bw_integrate (pair_creation/cp/mod.rs:92-186) for
// harmonic n: node k of each of the harmonic's segments, weighted (the
// factor 2 of bw_integrate is left to the caller).
__device__ __forceinline__ void bw_integrate_lane(int n, double a, double eta, double xk, double wk, double* re,
                                                  double* im) {
    *re = 0.0, *im = 0.0;
    double ell = n;
    double sn = 2.0 * ell * eta / (1.0 + a * a);
    if (sn <= 4.0) return;
    double a2 = a * a;
    double w1 = 1.0 / ell + 1.0;
    double beta = a2 * a2 * w1 * w1 + 16.0 * (a2 - 2.0) * (a2 - 2.0) / (sn * sn) - 8.0 * a2 * (a2 - 2.0) / sn;
    beta = sqrt(beta) / (a2 - 2.0);
    double alpha = (a2 + 2.0 * ell) / (ell * (2.0 - a2)) - 4.0 / sn;
    double s_peak = 0.5 * (1.0 - sqrt(alpha + beta));
    double s_min, s_max;
    bw_s_bounds(n, a, eta, &s_min, &s_max);
    double lo[3], hi[3];
    int nseg;
    if (isfinite(s_peak)) {
        double s_mid = 2.0 * s_peak - s_min;
        if (s_mid > s_max) {
            nseg = 2;
            lo[0] = s_min, hi[0] = s_peak, lo[1] = s_peak, hi[1] = s_max;
        } else {
            nseg = 3;
            lo[0] = s_min, hi[0] = s_peak, lo[1] = s_peak, hi[1] = s_mid, lo[2] = s_mid, hi[2] = s_max;
        }
    } else {
        nseg = 1;
        lo[0] = s_min, hi[0] = s_max;
    }
    for (int g = 0; g < nseg; ++g) {
        double h = 0.5 * (hi[g] - lo[g]), m = 0.5 * (lo[g] + hi[g]);
        double sr, si;
        bw_over_theta(n, a, eta, h * xk + m, &sr, &si);
        *re += h * wk * sr;
        *im += h * wk * si;
    }
}

// bw_by_summation (pair_creation/cp/mod.rs:385-393) evaluated by the 32
// lanes of a converged warp: lane k evaluates node k of every segment of
// every harmonic (bw_integrate's 32-point rule), and the sums are reduced
// over the lanes in a fixed order.  Equal to the serial sum up to the
// order of its additions.
static __device__ __noinline__ void bw_by_summation_warp(double a, double eta, double* f0, double* f1) {
    const unsigned all = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    int n0, n1;
    bw_sum_limits(a, eta, &n0, &n1);
    const double xk = PTG_GAUSS_32_NODES[lane], wk = PTG_GAUSS_32_WEIGHTS[lane];
    double re = 0.0, im = 0.0;
    for (int n = n0; n <= n1; ++n) {
        double r, i;
        bw_integrate_lane(n, a, eta, xk, wk, &r, &i);
        re += r, im += i;
    }
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_down_sync(all, re, o);
        im += __shfl_down_sync(all, im, o);
    }
    *f0 = 2.0 * __shfl_sync(all, re, 0);
    *f1 = 2.0 * __shfl_sync(all, im, 0);
}

// The harmonic of bw_sample (pair_creation/cp/mod.rs:314-346) and the s
// ceiling of bw_sample_s_theta (cp/mod.rs:199-207), evaluated by the 32
// lanes of a converged warp for one lane's request: the rates (the warp's
// harmonic sum below a = 0.3, else the table), then the cumulative sum over
// harmonics with lane k evaluating node k of every segment, reduced by a
// butterfly (every lane holds the same sum, so the walk stops on the same
// harmonic in every lane), then the ceiling's 32 nodes one per lane.  The
// harmonic is the serial walk's up to the order of the additions; the
// ceiling is the serial maximum exactly.  n_out is -1 where the rate
// lookup is out of table.
static __device__ __noinline__ void bw_sample_harmonic_warp(const double* T, const double* nodes, double a, double eta,
                                                            double sv3, double u, int* n_out, double* ceil_out,
                                                            double* f0_out, double* f1_out) {
    const unsigned all = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    double f0, f1;
    bool ok = true;
    if (a < 0.02 || bw_is_too_small(a, eta)) {
        f0 = f1 = 0.0;
    } else if (a < BW_CP_MIN_A) {
        bw_by_summation_warp(a, eta, &f0, &f1);
    } else {
        ok = bw_by_lookup(T, a, eta, &f0, &f1, nodes);
    }
    *f0_out = f0, *f1_out = f1;
    if (!ok) {
        *n_out = -1;
        *ceil_out = 0.0;
        return;
    }
    int n0, n1;
    bw_sum_limits(a, eta, &n0, &n1);
    const double xk = PTG_GAUSS_32_NODES[lane], wk = PTG_GAUSS_32_WEIGHTS[lane];
    double target = 0.5 * (f0 * (1.0 + sv3) + f1 * (1.0 - sv3)) * u;
    double cum = 0.0;
    int index = -1;
    for (int n = n0; n <= n1; ++n) {
        double re, im;
        bw_integrate_lane(n, a, eta, xk, wk, &re, &im);
        for (int o = 16; o > 0; o >>= 1) {
            re += __shfl_xor_sync(all, re, o);
            im += __shfl_xor_sync(all, im, o);
        }
        cum += 0.5 * ((1.0 + sv3) * (2.0 * re) + (1.0 - sv3) * (2.0 * im));
        if (cum > target) {
            index = n;
            break;
        }
    }
    if (index == -1) index = n1 - 1;
    double mx = bw_s_node_value(index, a, eta, sv3, lane);
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(all, mx, o));
    *n_out = index;
    *ceil_out = mx;
}

// pair_creation/mod.rs:21-42 + cp/mod.rs:280-309 (CP).  Returns 1, 0 out of
// table, or BW_DEFERRED when the harmonic sum is left to the warp (bdf not
// NULL).
static __device__ __noinline__ int bw_probability(const double* T, d4 ell, d4 sv_in, d4 k, double a, double dt,
                                                  double pol_angle, double* prob, d4* sv_out,
                                                  double rate_increase = 1.0, BwDefer* bdf = nullptr,
                                                  const double* nodes = nullptr) {
    double eta = dot4(k, ell);
    double dphi = eta * dt / (COMPTON_TIME * ell.t);
    double f0, f1;
    double c = ALPHA_FINE * dphi / eta;
    // TotalRate::value's dispatch (bw_rates), its too-small test taken once
    if (a < 0.02 || bw_is_too_small_fast(a, eta)) {
        f0 = f1 = 0.0;
    } else if (a < BW_CP_MIN_A) {
        if (c * fmax(1.0, rate_increase) * bw_summation_bound(a, eta) < PAIR_PROB_NEGLIGIBLE) {
            // the summed rate cannot give a probability that matters: skip it
            f0 = f1 = 0.0;
        } else if (bdf != nullptr) {
            // the warp's sum: served for this step's rate, or with the
            // harmonic of this step's pair (which bw_sample then takes)
            if (!(bdf->pend == 2 && bdf->a == a && bdf->eta == eta)) {
                bdf->a = a, bdf->eta = eta;
                bdf->kind = BW_DEFER_RATE;
                bdf->pend = 1;
                return BW_DEFERRED;
            }
            f0 = bdf->f0, f1 = bdf->f1;
            if (bdf->kind == BW_DEFER_RATE) bdf->pend = 0;
        } else {
            bw_by_summation(a, eta, &f0, &f1);
        }
    } else if (!bw_by_lookup(T, a, eta, &f0, &f1, nodes)) {
        return 0;
    }
    StokesBasis bs = lma_stokes_basis(ell);
    d3 g0 = stokes_rotate_cs(mk3(sv_in.x, sv_in.y, sv_in.z), bs.c2, bs.s2);
    d4 sv = stokes_rotate_by(d4{sv_in.t, g0.x, g0.y, g0.z}, pol_angle);
    double p = c * (0.5 * ((f0 + f1) + sv.z * (f0 - f1)));
    double p_avg = c * (0.5 * (f0 + f1));
    double delta = c * (0.5 * (f0 - f1));
    d4 o = d4{sv.t, sv.x * (1.0 - p_avg) / (1.0 - p), sv.y * (1.0 - p_avg) / (1.0 - p), (sv.z * (1.0 - p_avg) - delta) / (1.0 - p)};
    o = stokes_rotate_by(o, -pol_angle);
    d3 g = stokes_rotate_cs(mk3(o.x, o.y, o.z), bs.c2, -bs.s2);
    *sv_out = d4{o.t, g.x, g.y, g.z};
    *prob = p;
    return 1;
}

// pair_creation/mod.rs:62-110: the positron momentum for a sampled
// harmonic n, s and azimuth (rms amplitude a).  Returns a ptg status.
static __device__ __noinline__ int bw_kinematics(d4 ell, d4 k, double a, double pol_angle, int n, double s, double cphi,
                                                 d4* q_out) {
    double eta = dot4(k, ell);
    double j = n;
    double e_zmf = sqrt(0.5 * j * eta);
    double p_zmf = sqrt(0.5 * j * eta - 1.0 - a * a);
    double ct = (1.0 - 2.0 * s) * e_zmf / p_zmf;
    if (!(ct <= 1.0 && ct >= -1.0)) return 3;
    d4 t = d4{ell.t + j * k.t, ell.x + j * k.x, ell.y + j * k.y, ell.z + j * k.z};
    double m = sqrt(dot4(t, t));
    d4 uz = d4{t.t / m, t.x / m, t.y / m, t.z / m};
    d4 jk = boost_by(d4{j * k.t, j * k.x, j * k.y, j * k.z}, uz);
    d3 along = -normalize(mk3(jk.x, jk.y, jk.z));
    double sp, cp;
    sincos(pol_angle, &sp, &cp);
    d4 e4 = boost_by(d4{0.0, cp, sp, 0.0}, uz);
    d3 eps = normalize(mk3(e4.x, e4.y, e4.z));
    eps = normalize(cross(along, cross(eps, along)));
    double sc, cc;
    sincos(cphi, &sc, &cc);
    d3 perp = rotate_around(eps, along, sc, cc);
    d3 q3 = p_zmf * (ct * along + sqrt(1.0 - ct * ct) * perp);
    d4 q = d4{sqrt(1.0 + a * a + dot(q3, q3)), q3.x, q3.y, q3.z};
    q = boost_by(q, d4{uz.t, -uz.x, -uz.y, -uz.z});
    double s_new = 1.0 - dot4(k, q) / dot4(k, ell);
    if (!(fabs(s - s_new) / s < 1.0e-3)) return 3;
    *q_out = q;
    return 0;
}

// pair_creation/mod.rs:49-110 (CP): the positron momentum
static __device__ __noinline__ int bw_generate(const double* T, d4 ell, d4 sv_in, d4 k, double a, double pol_angle, Draws& rng,
                                        int* n_out, d4* q_out, uint32_t* rej, BwDefer* bdf = nullptr) {
    double eta = dot4(k, ell);
    d4 sv = stokes_rotate_by(stokes_in_lma_basis(sv_in, ell), pol_angle);
    int n;
    double s, cphi;
    int st = bw_sample(T, a, eta, sv.x, sv.y, sv.z, rng, &n, &s, &cphi, rej, bdf);
    if (st != 0) return st;
    *n_out = n;
    return bw_kinematics(ell, k, a, pol_angle, n, s, cphi, q_out);
}

}  // namespace ptg
