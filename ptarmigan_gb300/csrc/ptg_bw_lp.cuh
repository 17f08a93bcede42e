// Nonlinear Breit-Wheeler pair creation in a linearly polarised background
// (pair_creation/lp/**): the total rates from the shipped tables (main
// table for 0.1 < a < 25, mid-range table for a < 2 at eta' = eta / (1 +
// a^2/2) in [0.05, 2)), the harmonic order by CDF inversion, and (s, theta)
// by rejection under the double-differential rate, which needs J(n, x, y)
// (ptg_lp.cuh) in the lane's workspace.  `a` is the peak amplitude
// (rms a times sqrt 2).
#pragma once
#include "ptg_lp.cuh"
#include "ptg_math.cuh"

namespace ptg {

// pair_creation/lp/tables/pol_dep.rs: values at S_1 = +1 (par), -1 (perp)
struct PolDep {
    double par, perp;
    __host__ __device__ double interp(double sv1) const { return 0.5 * ((par + perp) + sv1 * (par - perp)); }
};
__host__ __device__ __forceinline__ PolDep pd_at(const double* v) { return PolDep{v[0], v[1]}; }
__host__ __device__ __forceinline__ PolDep operator+(PolDep a, PolDep b) { return PolDep{a.par + b.par, a.perp + b.perp}; }
__host__ __device__ __forceinline__ PolDep operator-(PolDep a, PolDep b) { return PolDep{a.par - b.par, a.perp - b.perp}; }
__host__ __device__ __forceinline__ PolDep operator*(double s, PolDep a) { return PolDep{s * a.par, s * a.perp}; }
__host__ __device__ __forceinline__ PolDep operator*(PolDep a, double s) { return PolDep{a.par * s, a.perp * s}; }
__host__ __device__ __forceinline__ PolDep operator*(PolDep a, PolDep b) { return PolDep{a.par * b.par, a.perp * b.perp}; }
__host__ __device__ __forceinline__ PolDep operator/(PolDep a, PolDep b) { return PolDep{a.par / b.par, a.perp / b.perp}; }
// Div<f64> of the reference multiplies by the reciprocal
__host__ __device__ __forceinline__ PolDep pd_div(PolDep a, double s) { return a * (1.0 / s); }
__host__ __device__ __forceinline__ PolDep pd_exp(PolDep a) { return PolDep{exp(a.par), exp(a.perp)}; }
__host__ __device__ __forceinline__ PolDep pd_ln(PolDep a) { return PolDep{log(a.par), log(a.perp)}; }
__host__ __device__ __forceinline__ PolDep pd_pow(PolDep a, PolDep m) { return PolDep{pow(a.par, m.par), pow(a.perp, m.perp)}; }

// Rust's `as i32` on an f64: saturating, NaN -> 0.
__host__ __device__ __forceinline__ int as_i32(double x) {
    if (x != x) return 0;
    if (x >= 2147483647.0) return 2147483647;
    if (x <= -2147483648.0) return -2147483647 - 1;
    return (int)x;
}

// pair_creation/lp/mod.rs:345-374
__host__ __device__ __forceinline__ void lpp_sum_limits(double a, double eta, int* n_min_out, int* n_max_out) {
    double n_min = ceil(2.0 * (1.0 + 0.5 * a * a) / eta);
    double range = a < 1.0 ? 2.0 + (2.0 + 20.0 * a * a) * exp(-sqrt(0.5 * eta))
                           : 3.0 + 2.8 * pow(a, 8.0 / 3.0) / cbrt(eta) + 0.25 * a * a * a * sqrt(eta);
    double test = 0.25 - (1.0 + 0.5 * a * a) / (2.0 * n_min * eta);
    if (test <= 2.220446049250313e-16) {
        *n_min_out = as_i32(n_min) + 1;
        *n_max_out = as_i32(n_min + 1.0 + range);
    } else {
        *n_min_out = as_i32(n_min);
        *n_max_out = as_i32(n_min + range);
    }
}

__device__ __forceinline__ bool lpp_is_negligible(double a, double eta) {
    double l = log10(a) + 2.0;
    return log10(eta) < -1.0 - l * l / 4.5;
}

// pair_creation/lp/tables/mod.rs:19-58
__device__ __forceinline__ bool lpp_main_contains(double a, double eta) {
    return log(a) >= PTG_BW_LP_LN_MIN_A && a < 25.0 && log(eta) >= PTG_BW_LP_LN_MIN_ETA && eta < 2.0;
}

static __device__ __noinline__ bool lpp_main_interpolate(const double* T /* [61][25][2] */, double a, double eta,
                                                         double f[2]) {
    const double LMA = PTG_BW_LP_LN_MIN_A, LME = PTG_BW_LP_LN_MIN_ETA, SA = PTG_BW_LP_LN_A_STEP,
                 SE = PTG_BW_LP_LN_ETA_STEP;
    int ia = (int)((log(a) - LMA) / SA);
    int ie = (int)((log(eta) - LME) / SE);
    if (ia < 0 || ie < 0 || ia >= 24 || ie >= 60) return false;
#define LPP_AT(e, c) pd_at(T + ((size_t)(e) * 25 + (c)) * 2)
    PolDep r;
    if (a * eta > 2.0) {
        double da = (log(a) - LMA) / SA - ia;
        double de = (log(eta) - LME) / SE - ie;
        r = (1.0 - da) * (1.0 - de) * LPP_AT(ie, ia) + da * (1.0 - de) * LPP_AT(ie, ia + 1) +
            (1.0 - da) * de * LPP_AT(ie + 1, ia) + da * de * LPP_AT(ie + 1, ia + 1);
    } else {
        double a_min = exp(LMA + ia * SA), a_max = exp(LMA + (ia + 1) * SA);
        double e_min = exp(LME + ie * SE), e_max = exp(LME + (ie + 1) * SE);
        double da = ((a_min * a_max / a) - a_min) / (a_max - a_min);
        double de = ((e_min * e_max / eta) - e_min) / (e_max - e_min);
        r = LPP_AT(ie, ia) * da * de + LPP_AT(ie, ia + 1) * (1.0 - da) * de + LPP_AT(ie + 1, ia) * da * (1.0 - de) +
            LPP_AT(ie + 1, ia + 1) * (1.0 - da) * (1.0 - de);
    }
#undef LPP_AT
    PolDep e = pd_exp(r);
    f[0] = e.par, f[1] = e.perp;
    return true;
}

// pair_creation/lp/tables/mid_range/mod.rs:9-98
__device__ __forceinline__ bool lpp_mid_contains(double a, double eta) {
    double lep = log(eta / (1.0 + 0.5 * a * a));
    return log(a) > PTG_BW_LPM_LN_MIN_A && a < 2.0 && lep > PTG_BW_LPM_LN_MIN_ETA_PRIME && lep < PTG_BW_LPM_LN_MAX_ETA_PRIME;
}

static __device__ __noinline__ PolDep lpp_mid_interp_eta_prime(const double* T /* [157][36][2] */, double ep, int ia) {
    const double D = PTG_BW_LPM_ETA_PRIME_DENSITY;
    int ie = as_i32(D * (exp(PTG_BW_LPM_LN_MAX_ETA_PRIME) / ep - 1.0));
    if (ie % (int)D == (int)D - 1) ie -= 1;
    if (ie < 0) ie = 0;
    if (ie > 154) ie = 154;
    double l0 = 2.0 / (1.0 + (double)(ie + 2) / D), m0 = 2.0 / (1.0 + (double)(ie + 1) / D), u0 = 2.0 / (1.0 + (double)ie / D);
    PolDep l1 = pd_at(T + ((size_t)(ie + 2) * 36 + ia) * 2), m1 = pd_at(T + ((size_t)(ie + 1) * 36 + ia) * 2),
           u1 = pd_at(T + ((size_t)ie * 36 + ia) * 2);
    PolDep m = pd_div(pd_ln((u1 - l1) / (m1 - l1)), log((u0 - l0) / (m0 - l0)));
    PolDep alpha = (m1 - l1) / pd_pow(PolDep{m0 - l0, m0 - l0}, m);
    PolDep r = alpha * pd_pow(PolDep{ep - l0, ep - l0}, m) + l1;
    double w_lo = (log(ep) - log(l0)) / (log(m0) - log(l0));
    double w_hi = (log(ep) - log(m0)) / (log(u0) - log(m0));
    if (!isfinite(r.par)) r.par = ep < m0 ? (1.0 - w_lo) * l1.par + w_lo * m1.par : (1.0 - w_hi) * m1.par + w_hi * u1.par;
    if (!isfinite(r.perp))
        r.perp = ep < m0 ? (1.0 - w_lo) * l1.perp + w_lo * m1.perp : (1.0 - w_hi) * m1.perp + w_hi * u1.perp;
    return r;
}

static __device__ __noinline__ void lpp_mid_interpolate(const double* T, double a, double eta, double f[2]) {
    const double LMA = PTG_BW_LPM_LN_MIN_A, SA = PTG_BW_LPM_LN_A_STEP;
    int ia = as_i32((log(a) - LMA) / SA);
    if (ia < 0) ia = 0;
    if (ia > 34) ia = 34;
    double ep = eta / (1.0 + 0.5 * a * a);
    PolDep r;
    if (a < 0.5) {
        double da = (log(a) - LMA) / SA - ia;
        r = (1.0 - da) * lpp_mid_interp_eta_prime(T, ep, ia) + da * lpp_mid_interp_eta_prime(T, ep, ia + 1);
    } else {
        double a_min = exp(LMA + ia * SA), a_max = exp(LMA + (ia + 1) * SA);
        double da = (a - a_min) / (a_max - a_min);
        r = pd_div((1.0 - da) * a_min * lpp_mid_interp_eta_prime(T, ep, ia) +
                       da * a_max * lpp_mid_interp_eta_prime(T, ep, ia + 1),
                   a);
    }
    PolDep e = pd_exp(r);
    f[0] = e.par, f[1] = e.perp;
}

// pair_creation/lp/mod.rs:380-420: [f_par, f_perp]; zero where negligible
// or outside both tables, as in the reference
__device__ __forceinline__ bool lpp_rates(const double* main_total, const double* mid_total, double a, double eta,
                                          double f[2]) {
    f[0] = f[1] = 0.0;
    if (lpp_is_negligible(a, eta)) return true;
    if (lpp_mid_contains(a, eta)) {
        lpp_mid_interpolate(mid_total, a, eta, f);
        return true;
    }
    if (lpp_main_contains(a, eta)) return lpp_main_interpolate(main_total, a, eta, f);
    return true;
}

// pair_creation/lp/tables/mod.rs:60-113 (main-table harmonic inversion)
static __device__ __noinline__ int lpp_main_invert(const double* T /* [1525][16][3] */, double a, double eta,
                                                   double sv1, double frac) {
    double fa = (log(a) - PTG_BW_LP_CDF_MIN_0) / PTG_BW_LP_CDF_STEP_0;
    double fe = (log(eta) - PTG_BW_LP_CDF_MIN_1) / PTG_BW_LP_CDF_STEP_1;
    int ia = (int)fa, ie = (int)fe;
    double da = fa - trunc(fa), de = fe - trunc(fe);
    int idx[4] = {25 * ie + ia, 25 * ie + ia + 1, 25 * (ie + 1) + ia, 25 * (ie + 1) + ia + 1};
    double w[4] = {(1.0 - da) * (1.0 - de), da * (1.0 - de), (1.0 - da) * de, da * de};
    double u = 0.0;
    double ff = log(-1.0 * log(1.0 - frac));
    for (int k = 0; k < 4; ++k) {
        if (idx[k] < 0 || idx[k] >= 1525) return -1;
        const double* src = T + (size_t)idx[k] * 48;
        double n_min = src[0];
        double f_max = PolDep{src[46], src[47]}.interp(sv1);
        double tb[30];
        for (int i = 0; i < 15; ++i) {
            tb[2 * i] = log(src[3 * i] - n_min + 1.0);
            tb[2 * i + 1] = log(-1.0 * log(1.0 - PolDep{src[3 * i + 1], src[3 * i + 2]}.interp(sv1) / f_max));
        }
        double uk = 0.0;
        pw_invert(tb, 15, true, ff, &uk);
        u += uk * w[k];
    }
    int n_min, n_max;
    lpp_sum_limits(a, eta, &n_min, &n_max);
    return as_i32((double)n_min + expm1(u)) + 1;
}

// pair_creation/lp/tables/mid_range/mod.rs:100-270 (mid-range inversion,
// regenerated CDF table [5652][16][3]).  -2: table missing.
static __device__ __noinline__ int lpp_mid_invert(const double* T, const double* mid_total, double a, double eta,
                                                  double sv1, double frac) {
    if (!T) return -2;
    const double LMA = PTG_BW_LPM_LN_MIN_A, SA = PTG_BW_LPM_LN_A_STEP, D = PTG_BW_LPM_ETA_PRIME_DENSITY;
    const double EMAX = exp(PTG_BW_LPM_LN_MAX_ETA_PRIME);
    int ia = as_i32((log(a) - LMA) / SA);
    double da = (log(a) - LMA) / SA - ia;
    double ep = eta / (1.0 + 0.5 * a * a);
    int ie0 = as_i32(D * (EMAX / ep - 1.0));
    bool bdy = ie0 % (int)D == (int)D - 1;
    int ie = bdy ? ie0 - 1 : ie0;
    int n_min, n_max;
    lpp_sum_limits(a, eta, &n_min, &n_max);
    double fr[2];
    lpp_mid_interpolate(mid_total, a, eta, fr);
    double total_rate = 0.5 * ((fr[0] + fr[1]) + sv1 * (fr[0] - fr[1]));
    double p_lowest = 0.0;
    if (bdy) {
        // interpolate_lowest_harmonic: weights of the unshifted bracket
        double lower = EMAX / (1.0 + (double)(ie0 + 1) / D), upper = EMAX / (1.0 + (double)ie0 / D);
        double de = (log(ep) - log(lower)) / (log(upper) - log(lower));
        int jx[4] = {36 * ie0 + ia, 36 * ie0 + ia + 1, 36 * (ie0 + 1) + ia, 36 * (ie0 + 1) + ia + 1};
        double wx[4] = {(1.0 - da) * de, da * de, (1.0 - da) * (1.0 - de), da * (1.0 - de)};
        double acc = 0.0;
        for (int k = 0; k < 4; ++k) {
            if (jx[k] < 0 || jx[k] >= 5652) return -1;
            const double* tb = T + (size_t)jx[k] * 48;
            double fr0 = 0.0;
            if (!(tb[0] > (double)n_min)) fr0 = PolDep{tb[1], tb[2]}.interp(sv1) / PolDep{tb[46], tb[47]}.interp(sv1);
            double v = fr0 * total_rate;
            acc += wx[k] * (v * v * v);
        }
        p_lowest = cbrt(acc) / total_rate;
        if (frac <= p_lowest) return n_min;
    }
    double lower = EMAX / (1.0 + (double)(ie + 1) / D), upper = EMAX / (1.0 + (double)ie / D);
    double de = (log(ep) - log(lower)) / (log(upper) - log(lower));
    int idx[4] = {36 * ie + ia, 36 * ie + ia + 1, 36 * (ie + 1) + ia, 36 * (ie + 1) + ia + 1};
    double w[4] = {(1.0 - da) * de, da * de, (1.0 - da) * (1.0 - de), da * (1.0 - de)};
    double n = 0.0;
    for (int k = 0; k < 4; ++k) {
        if (idx[k] < 0 || idx[k] >= 5652) return -1;
        const double* src = T + (size_t)idx[k] * 48;
        double f_max = PolDep{src[46], src[47]}.interp(sv1);
        double tb[32];
        for (int i = 0; i < 16; ++i) {
            tb[2 * i] = src[3 * i];
            tb[2 * i + 1] = PolDep{src[3 * i + 1], src[3 * i + 2]}.interp(sv1) / f_max;
        }
        double nk = 0.0;
        bool ok = true;
        if (bdy) {
            if (tb[0] == (double)n_min) {
                double t01 = tb[1];
                for (int i = 0; i < 16; ++i) tb[2 * i + 1] = (t01 - tb[2 * i + 1] + p_lowest * (tb[2 * i + 1] - 1.0)) / (t01 - 1.0);
            }
            ok = pw_invert(tb, 16, false, frac, &nk);
        } else if (frac <= tb[1]) {
            nk = tb[0] - 0.1;
        } else {
            ok = pw_invert(tb, 16, false, frac, &nk);
        }
        if (!ok) return -1;
        n += nk * w[k];
    }
    return isfinite(n) ? as_i32(ceil(n)) : -1;
}

// pair_creation/lp/theta_bound.rs:11-101
struct LppTheta {
    double s[16], f[16];
    __device__ __forceinline__ double at(double arg) const {
        double val = f[15];
        for (int i = 1; i < 16; ++i) {
            if (arg > s[i]) {
                double wt = (arg - s[i - 1]) / (s[i] - s[i - 1]);
                val = wt * f[i] + (1.0 - wt) * f[i - 1];
                break;
            }
        }
        return fmin(val, PI / 2.0);
    }
};

static __device__ __noinline__ void lpp_theta_bound(int n, double a, double eta, LppTheta* tb) {
    double s_min = 0.5, s_max = 0.5 + sqrt(0.25 - (1.0 + 0.5 * a * a) / (2.0 * n * eta));
    for (int i = 0; i < 16; ++i) {
        double z = cos(PI * i / 15.0);
        double si = s_min + 0.5 * (z + 1.0) * (s_max - s_min);
        tb->s[i] = si;
        double r_n = sqrt(2.0 * n * eta * si * (1.0 - si) - (1.0 + 0.5 * a * a));
        double x = a * r_n / (eta * si * (1.0 - si));
        double y = a * a / (8.0 * eta * si * (1.0 - si));
        double x_crit = y > n / 6.0 ? 4.0 * sqrt(y) * sqrt(n - 2.0 * y) : n + 2.0 * y;
        double ln_j_crit = log(0.443) - log((double)n) / 3.0;
        double ln_j_bdy = fmin(ln_double_bessel_x_zero(n % 2 == 0 ? n : n + 1, y), ln_j_crit);
        double ct = fmax(1.0 - x_crit * log(0.01) / (x * (ln_j_bdy - ln_j_crit)), -1.0);
        double fi = acos(ct);
        tb->f[i] = isnan(fi) ? PI : fi;
    }
    double f_min = tb->f[0];
    for (int i = 1; i < 16; ++i) {
        if (tb->f[i] < f_min)
            f_min = tb->f[i];
        else
            tb->f[i] = f_min;
    }
}

// pair_creation/lp/mod.rs:57-90: the three contributions to the rate
static __device__ __noinline__ void lpp_elements(const DbGeom& g, const DbWork& w, double a, double eta, double s,
                                                 double theta, double* unpol, double* d1, double* d2) {
    int n = g.n;
    double r2 = 2.0 * n * eta * s * (1.0 - s) - (1.0 + 0.5 * a * a);
    if (!(r2 > 0.0)) {
        *unpol = *d1 = *d2 = 0.0;
        return;
    }
    double rn = sqrt(r2);
    double ct = cos(theta), st = sin(theta);
    double x = a * rn * ct / (eta * s * (1.0 - s));
    double y = a * a / (8.0 * eta * s * (1.0 - s));
    double j[5];
    if (!db_evaluate(g, w, x, y, j)) {
        *unpol = *d1 = *d2 = NAN;
        return;
    }
    double g0 = j[2], g1 = 0.5 * (j[1] + j[3]), g2 = 0.25 * (j[0] + 2.0 * j[2] + j[4]);
    double h_s = 0.5 / (s * (1.0 - s)) - 1.0;
    *unpol = g0 * g0 + a * a * h_s * (g1 * g1 - g0 * g2);
    double c1 = g0 * rn * ct - g1 * a;
    double q = g0 * st;
    *d1 = c1 * c1 - q * q * r2;
    *d2 = 2.0 * g0 * rn * st * c1;
}

__device__ __forceinline__ double lpp_fully_resolved(const DbGeom& g, const DbWork& w, double a, double eta, double s,
                                                     double theta, double sv1, double sv2) {
    double u, d1, d2;
    lpp_elements(g, w, a, eta, s, theta, &u, &d1, &d2);
    return (u - sv1 * d1 - sv2 * d2) / (2.0 * PI);
}

// pair_creation/lp/mod.rs:229-295: ceiling and rejection sampling of
// (s, theta) at harmonic n.  Returns a ptg status.
static __device__ __noinline__ int lpp_sample_s_theta(const DbGeom& g, const DbWork& w, double a, double eta, double sv1,
                                                      double sv2, Draws& rng, double* s_out, double* theta_out,
                                                      uint32_t* rej) {
    int n = g.n;
    double s_min = 0.5, s_max = fmax(0.5 + sqrt(0.25 - (1.0 + 0.5 * a * a) / (2.0 * n * eta)), 0.5);
    LppTheta tb;
    lpp_theta_bound(n, a, eta, &tb);
    double centre = 0.5 + sqrt(0.25 - (1.0 + a * a) / (2.0 * n * eta));
    double lower = s_min, upper = s_max;
    if (isfinite(centre)) {
        lower = fmax(centre - 0.2, s_min);
        upper = 0.5 * (centre + s_max);
    }
    double mx = NAN;
    for (int i = 0; i < 50; ++i) mx = rmax(mx, lpp_fully_resolved(g, w, a, eta, lower + (upper - lower) * (double)i / 50.0, 0.0, sv1, sv2));
    mx *= 1.2;
    double s = 0.0, theta = 0.0;
    int it;
    for (it = 0; it < rng.cap; ++it) {
        double ss = s_min + (s_max - s_min) * rng.next();
        double th = (PI / 2.0) * rng.next();
        if (th > tb.at(ss)) continue;
        double z = mx * rng.next();
        if (z < lpp_fully_resolved(g, w, a, eta, ss, th, sv1, sv2)) {
            s = ss, theta = th;
            break;
        }
    }
    *rej += it;
    if (it == rng.cap) return 4;
    if ((int)(2.0 * rng.next()) == 0) s = 1.0 - s;
    int quadrant = (int)(4.0 * rng.next());
    if (quadrant == 1)
        theta = PI - theta;
    else if (quadrant == 2)
        theta = PI + theta;
    else if (quadrant == 3)
        theta = 2.0 * PI - theta;
    *s_out = s;
    *theta_out = theta;
    return 0;
}

// pair_creation/lp/mod.rs:424-441: harmonic, s and theta of a pair event
static __device__ __noinline__ int lpp_sample(const double* main_cdf, const double* mid_cdf, const double* mid_total,
                                              const DbWork& w, double a, double eta, double sv1, double sv2,
                                              Draws& rng, int* n_out, double* s, double* theta, uint32_t* rej) {
    if (w.base == nullptr) return 8;
    double frac = rng.next();
    int n;
    if (lpp_mid_contains(a, eta))
        n = lpp_mid_invert(mid_cdf, mid_total, a, eta, sv1, frac);
    else if (lpp_main_contains(a, eta))
        n = lpp_main_invert(main_cdf, a, eta, sv1, frac);
    else
        return 2;
    if (n == -2) return 8;  // PTG_ERR_TABLES
    if (n < 1) return 2;
    DbWork wk;
    DbGeom g;
    int slot = -1;
    int st = db_take(w, n, &wk, &g, &slot);
    if (st != 0) return st;
    *n_out = n;
    st = lpp_sample_s_theta(g, wk, a, eta, sv1, sv2, rng, s, theta, rej);
    if (slot >= 0) db_pool_release(w.pool, slot);
    return st;
}

}  // namespace ptg
