// LMA nonlinear Compton scattering on the device: Bessel functions J_n,
// the circularly polarised (CP) partial rates, total rate and sampler, and
// the zero-momentum-frame kinematics that turn a sample into a photon.
//
// Follows special_functions/bessel.rs, nonlinear_compton/cp/mod.rs,
// nonlinear_compton/cp/tables/mod.rs and nonlinear_compton/mod.rs (cited per
// function).  All FP64: these run once per emission, not per step.
#pragma once
#include "ptg_lcfa.cuh"
#include "ptg_math.cuh"

namespace ptg {

constexpr double FRAC_PI_2 = 1.57079632679489661923;
constexpr double FRAC_PI_4 = 0.78539816339744830962;

// ------------------------------------------------------------ Bessel ---
// special_functions/bessel.rs:117-176: (J_{n-1}, J_n, J_{n+1})(x) by Miller's
// backward recurrence normalised with J_0 + 2 sum J_2k = 1; O(n) work.
static __device__ __noinline__ void triple_j(int n, double x, double* a, double* b, double* c) {
    if (x == 0.0) {
        *a = (n == 1) ? 1.0 : 0.0;
        *b = (n == 0) ? 1.0 : 0.0;
        *c = (n == -1) ? 1.0 : 0.0;
        return;
    }
    double v = x / (double)n;
    int nmax = 1 + n + (int)(5.0 / (1.0 - 0.9 * v));
    if ((nmax & 1) != 0) nmax += 1;
    int n_even = (n & 1) == 0 ? 1 : 0;
    int k_stop = n - 1 - n_even;
    double q0 = 1.0, q1 = 0.0, q2 = 0.0, q3 = 0.0;
    double total = 0.0;
    double inv_x = 1.0 / x;
    for (int k = nmax; k >= k_stop; k -= 2) {
        q3 = q1;
        q2 = q0;
        q1 = (double)(2 * (k + 2)) * q2 * inv_x - q3;
        q0 = (double)(2 * (k + 1)) * q1 * inv_x - q2;
        total += q0;
    }
    double t0, t1, t2;
    if (n_even) {
        t0 = q1, t1 = q2, t2 = q3;
    } else {
        t0 = q0, t1 = q1, t2 = q2;
    }
    for (int k = k_stop - 2; k >= 0; k -= 2) {
        q3 = q1;
        q2 = q0;
        q1 = (double)(2 * (k + 2)) * q2 * inv_x - q3;
        q0 = (double)(2 * (k + 1)) * q1 * inv_x - q2;
        total += q0;
    }
    double norm = 2.0 * total - q0;
    if (isnan(norm)) {
        *a = *b = *c = 0.0;
    } else {
        double in = 1.0 / norm;
        *a = t0 * in;
        *b = t1 * in;
        *c = t2 * in;
    }
}

// special_functions/bessel.rs:178-199: uniform asymptotic expansion (n >= 1000).
// The fractional powers as cbrt(x)^2, sqrt(sqrt(x)) and w sqrt(w) (the
// reference's powf to a few ulp; NaN where powf is NaN).
static __device__ __noinline__ double j_asymptotic(int n, double x) {
    double m = (double)n;
    double z = x / m;
    double zeta;
    if (z < 1.0) {
        double r = sqrt(1.0 - z * z);
        double tmp = log((1.0 + r) / z) - r;
        zeta = tmp >= 0.0 ? pow_two_thirds(1.5 * tmp) : __longlong_as_double(0x7ff8000000000000LL);
    } else {
        double tmp = sqrt(z * z - 1.0) - acos(1.0 / z);
        zeta = tmp >= 0.0 ? -pow_two_thirds(1.5 * tmp) : __longlong_as_double(0x7ff8000000000000LL);
    }
    double m13 = cbrt(m);
    double arg = (m13 * m13) * zeta;
    double ai = arg >= 0.0 ? airy_ai(arg) : 0.0;
    double aip = arg >= 0.0 ? airy_ai_prime(arg) : 0.0;
    double w = 1.0 - z * z;
    double pre = 4.0 * zeta / w;
    double bk = 5.0 / (48.0 * zeta * zeta) - (2.0 + 3.0 * z * z) / (24.0 * sqrt(zeta) * (w * sqrt(w)));
    return sqrt(sqrt(pre)) * (ai / m13 - aip * bk / (m * (m13 * m13)));
}

// bessel.rs:26-34
__device__ __forceinline__ void j_pm(double x, int n, double* jm1, double* j, double* jp1) {
    if (n < 1000) {
        triple_j(n, x, jm1, j, jp1);
    } else {
        double jn = j_asymptotic(n, x);
        double jp = j_asymptotic(n + 1, x);
        *jm1 = (double)(2 * n) * jn / x - jp;
        *j = jn;
        *jp1 = jp;
    }
}

// ------------------------------------------------- CP partial rates ----
// J_{n-1}, J_n, J_{n+1} at one argument
struct Jtrip {
    double m, j, p;
};

// nonlinear_compton/cp/mod.rs:17-38: dW_n/dv, v = s / s_max, with the
// Bessel triple it evaluates (at the same argument as cp_finish forms from
// the same v, so that an accepted sample's triple serves cp_finish_j).  One
// out-of-line copy: every sampler, on a lane or a warp, gets the same
// rounding (inlined, the compiler may contract 1 + a a differently).
static __device__ __noinline__ double cp_diff_partial_rate_j(int n, double a, double eta, double v, Jtrip* jt) {
    if (v < 0.0 || v >= 1.0) {
        *jt = Jtrip{0.0, 0.0, 0.0};
        return 0.0;
    }
    double sn = 2.0 * n * eta / (1.0 + a * a);
    double smax = sn / (1.0 + sn);
    double vs = v * smax;
    double w = vs / (sn * (1.0 - vs));
    double z = sqrt(4.0 * ((double)n * (double)n) * (a * a / (1.0 + a * a)) * w * (1.0 - w));
    double jm, j, jp;
    j_pm(z, n, &jm, &j, &jp);
    *jt = Jtrip{jm, j, jp};
    return -smax * (j * j + 0.5 * a * a * (1.0 + 0.5 * vs * vs / (1.0 - vs)) * (2.0 * j * j - jp * jp - jm * jm));
}

// The same without the triple, inline (the ceilings' 32 points)
__device__ __forceinline__ double cp_diff_partial_rate(int n, double a, double eta, double v) {
    if (v < 0.0 || v >= 1.0) return 0.0;
    double sn = 2.0 * n * eta / (1.0 + a * a);
    double smax = sn / (1.0 + sn);
    double vs = v * smax;
    double w = vs / (sn * (1.0 - vs));
    double z = sqrt(4.0 * ((double)n * (double)n) * (a * a / (1.0 + a * a)) * w * (1.0 - w));
    double jm, j, jp;
    j_pm(z, n, &jm, &j, &jp);
    return -smax * (j * j + 0.5 * a * a * (1.0 + 0.5 * vs * vs / (1.0 - vs)) * (2.0 * j * j - jp * jp - jm * jm));
}

// nonlinear_compton/cp/mod.rs:42-75: the k-th of the 32 points (k in
// [0, 32)) at which the ceiling takes the spectrum's maximum.
__device__ __forceinline__ double cp_ceiling_point(int n, double a, double eta, int k) {
    double sn = 2.0 * n * eta / (1.0 + a * a);
    int n_switch = (int)(32.3 * (1.0 + 0.476 * pow(a, 1.56)));
    if (sn < 2.0 || n < n_switch) {
        double v_opt = (1.0 + sn) / (2.0 + sn);
        return k < 16 ? k * v_opt / 16.0 : v_opt + (k - 16) * (1.0 - v_opt) / 16.0;
    }
    double u = k < 16 ? 0.5 * (1.0 + sn) * (PTG_GAUSS_16_NODES[k] + 1.0)
                      : (1.0 + sn) + 0.5 * 2.0 * (1.0 + sn) * (PTG_GAUSS_16_NODES[k - 16] + 1.0);
    return u / (1.0 + u);
}

// nonlinear_compton/cp/mod.rs:42-75: 1.2 x the largest of those values
static __device__ __noinline__ double cp_ceiling(int n, double a, double eta) {
    double mx = -HUGE_VAL;
    for (int k = 0; k < 32; ++k) mx = fmax(mx, cp_diff_partial_rate(n, a, eta, cp_ceiling_point(n, a, eta, k)));
    return 1.2 * mx;
}

// nonlinear_compton/cp/mod.rs:92-136: integral of dW_n/dv over v (GL-32 x 2)
static __device__ __noinline__ double cp_partial_rate(int n, double a, double eta) {
    double sn = 2.0 * n * eta / (1.0 + a * a);
    int n_switch = (int)(32.3 * (1.0 + 0.476 * pow(a, 1.56)));
    double lower = 0.0, upper = 0.0;
    if (sn < 2.0 || n < n_switch) {
        double vmid = (1.0 + sn) / (2.0 + sn);
        for (int k = 0; k < 32; ++k) {
            double v = 0.5 * vmid * (PTG_GAUSS_32_NODES[k] + 1.0);
            lower += 0.5 * vmid * PTG_GAUSS_32_WEIGHTS[k] * cp_diff_partial_rate(n, a, eta, v);
        }
        for (int k = 0; k < 32; ++k) {
            double v = vmid + 0.5 * (1.0 - vmid) * (PTG_GAUSS_32_NODES[k] + 1.0);
            upper += 0.5 * (1.0 - vmid) * PTG_GAUSS_32_WEIGHTS[k] * cp_diff_partial_rate(n, a, eta, v);
        }
    } else {
        for (int k = 0; k < 32; ++k) {
            double u = 0.5 * (1.0 + sn) * (PTG_GAUSS_32_NODES[k] + 1.0);
            lower += 0.5 * (1.0 + sn) * PTG_GAUSS_32_WEIGHTS[k] * cp_diff_partial_rate(n, a, eta, u / (1.0 + u)) /
                     ((1.0 + u) * (1.0 + u));
        }
        for (int k = 0; k < 32; ++k) {
            double u = (1.0 + sn) + (1.0 + sn) * (PTG_GAUSS_32_NODES[k] + 1.0);
            upper += (1.0 + sn) * PTG_GAUSS_32_WEIGHTS[k] * cp_diff_partial_rate(n, a, eta, u / (1.0 + u)) /
                     ((1.0 + u) * (1.0 + u));
        }
    }
    return lower + upper;
}

// ------------------------------------------------------- CP rates ------
struct NlcTables {
    const double* lp_rate;   // [68][61] ln rate
    const double* lp_cdf;    // [4148][16][2]
    const double* cp_rate;   // [70][61] ln rate
    const double* cp_cdf;    // [4270][32][2]
    const double* cp_cl_rate;  // [61]
    const double* lp_cl_rate;  // [61]
    const double* cp_cl_cdf;   // [61][32][2]
    const double* lp_cl_cdf;   // [61][16][2]
    const double* cp_cdf_log;  // [4270][32][2]: cp_cdf's nodes as [ln n, ln(-ln(1 - cdf))], or NULL
};

// nonlinear_compton/cp/classical.rs:22-43
__device__ __forceinline__ bool cp_classical_rate(const NlcTables& t, double a, double eta, double* out) {
    double x = log(a);
    if (x < PTG_NLC_CL_MIN) {
        *out = 2.0 * a * a * eta / 3.0;
        return true;
    }
    int ix = (int)((x - PTG_NLC_CL_MIN) / PTG_NLC_CL_STEP);
    if (ix >= 60) return false;
    double dx = (x - PTG_NLC_CL_MIN) / PTG_NLC_CL_STEP - ix;
    *out = eta * exp((1.0 - dx) * t.cp_cl_rate[ix] + dx * t.cp_cl_rate[ix + 1]);
    return true;
}

// nonlinear_compton/cp/mod.rs:160-176 and tables/mod.rs:11-35
__device__ __forceinline__ bool cp_rate(const NlcTables& t, double a, double eta, double* out) {
    const double MIN0 = PTG_NLC_CP_MIN_0, MIN1 = PTG_NLC_CP_MIN_1, S0 = PTG_NLC_CP_STEP_0, S1 = PTG_NLC_CP_STEP_1;
    double la = log(a), le = log(eta);
    if (le < MIN1) return cp_classical_rate(t, a, eta, out);
    if (la < MIN0) {
        double q = 1.0 + 2.0 * eta;
        *out = a * a * (2.0 + 8.0 * eta + 9.0 * eta * eta + eta * eta * eta) / (2.0 * eta * q * q) -
               a * a * (2.0 + 2.0 * eta - eta * eta) * log(q) / (4.0 * eta * eta);
        return true;
    }
    if (!(a < 20.0 && eta < 2.0)) return false;
    int ia = (int)((la - MIN0) / S0);
    int ie = (int)((le - MIN1) / S1);
    if (ia >= 60 || ie >= 69) return false;
    double da = (la - MIN0) / S0 - ia;
    double de = (le - MIN1) / S1 - ie;
    const double* T = t.cp_rate;
    double f = (1.0 - da) * (1.0 - de) * T[ie * 61 + ia] + da * (1.0 - de) * T[ie * 61 + ia + 1] +
               (1.0 - da) * de * T[(ie + 1) * 61 + ia] + da * de * T[(ie + 1) * 61 + ia + 1];
    *out = exp(f);
    return true;
}

// cp_rate's table branch in FP32, where it certainly applies: a and eta
// strictly inside the table (away from its edges by more than the FP32
// rounding of their logarithms).  Returns false elsewhere (the caller then
// evaluates cp_rate).  T32: the CP ln-rate table in FP32; ln_a: ln a in
// FP32 (NaN or -inf where a is not positive).
__device__ __forceinline__ bool rate32_cp(const float* T32, float ln_a, double eta, float* out) {
    const float LN_A_MAX = 2.99523f;  // ln 19.99
    if (T32 == nullptr || !(ln_a < LN_A_MAX && eta < 1.999 && eta > 0.0)) return false;
    const float MIN0 = (float)PTG_NLC_CP_MIN_0, MIN1 = (float)PTG_NLC_CP_MIN_1;
    const float I0 = (float)(1.0 / PTG_NLC_CP_STEP_0), I1 = (float)(1.0 / PTG_NLC_CP_STEP_1);
    float ta = (ln_a - MIN0) * I0, te = (logf((float)eta) - MIN1) * I1;
    if (!(ta > 1e-3f && te > 1e-3f && ta < 59.99f && te < 68.99f)) return false;
    int ia = (int)ta, ie = (int)te;
    float da = ta - (float)ia, de = te - (float)ie;
    const float* p = T32 + ie * 61 + ia;
    float f = (1.0f - da) * (1.0f - de) * p[0] + da * (1.0f - de) * p[1] + (1.0f - da) * de * p[61] + da * de * p[62];
    *out = expf(f);
    return true;
}

// nonlinear_compton/cp/tables/mod.rs:37-121: harmonic index from the CDF
// table (four grid corners, each inverted in [ln n, ln(-ln(1 - cdf))]).
// The CDF coordinate of a harmonic-CDF node, ln(-ln(1 - cdf)).
__device__ __forceinline__ double cp_cdf_log_node(double cdf) { return log(-1.0 * log(1.0 - cdf)); }

// `logt`, when not NULL, holds the corner's nodes already transformed (the
// same expressions evaluated once when the tables are loaded).
static __device__ __noinline__ double cp_cdf_corner(const double* table, const double* logt, double frac) {
    if (frac <= table[1]) return 0.9;
    double rs[62];
    if (logt == nullptr) {
        for (int i = 0; i < 31; ++i) {
            rs[2 * i] = log(table[2 * i]);
            rs[2 * i + 1] = cp_cdf_log_node(table[2 * i + 1]);
        }
        logt = rs;
    }
    double f2 = log(-1.0 * log(1.0 - frac));
    double v = 0.0;
    pw_invert(logt, 31, true, f2, &v);
    return exp(v);
}

static __device__ __noinline__ int cp_invert(const NlcTables& t, double a, double eta, double frac) {
    const double MIN0 = PTG_NLC_CP_MIN_0, MIN1 = PTG_NLC_CP_MIN_1, S0 = PTG_NLC_CP_STEP_0, S1 = PTG_NLC_CP_STEP_1;
    double la = log(a), le = log(eta);
    if (la <= MIN0) return 1;
    int ix = (int)((la - MIN0) / S0);
    double dx = (la - MIN0) / S0 - ix;
    auto corner = [&](size_t row) {
        return cp_cdf_corner(t.cp_cdf + row * 64, t.cp_cdf_log ? t.cp_cdf_log + row * 64 : nullptr, frac);
    };
    if (le <= MIN1) {
        double n = corner((size_t)ix) * (1.0 - dx) + corner((size_t)(ix + 1)) * dx;
        return (int)ceil(n);
    }
    int iy = (int)((le - MIN1) / S1);
    double dy = (le - MIN1) / S1 - iy;
    double n = corner((size_t)(61 * iy + ix)) * ((1.0 - dx) * (1.0 - dy)) +
               corner((size_t)(61 * iy + ix + 1)) * (dx * (1.0 - dy)) +
               corner((size_t)(61 * (iy + 1) + ix)) * ((1.0 - dx) * dy) +
               corner((size_t)(61 * (iy + 1) + ix + 1)) * (dx * dy);
    return (int)ceil(n);
}

// nonlinear_compton/cp/mod.rs:181-234.  Returns a ptg status.
// nonlinear_compton/cp/mod.rs:181-200: v = s / s_max by rejection under
// the flat ceiling mx.  Returns a ptg status.
// `jt`, when not NULL, receives the accepted trial's Bessel triple.
static __device__ __noinline__ int cp_sample_v_under(int n, double a, double eta, double mx, Draws& rng,
                                                     double* v_out, uint32_t* rej, Jtrip* jt = nullptr) {
    int it;
    for (it = 0; it < rng.cap; ++it) {
        double vv = rng.next(), u = rng.next();
        Jtrip tj;
        if (u <= cp_diff_partial_rate_j(n, a, eta, vv, &tj) / mx) {
            *v_out = vv;
            if (jt) *jt = tj;
            break;
        }
    }
    *rej += it;
    return it == rng.cap ? 4 : 0;  // PTG_ERR_REJECTION_CAP
}

// The same under the reference's ceiling.
static __device__ __noinline__ int cp_sample_v(int n, double a, double eta, Draws& rng, double* v_out, uint32_t* rej,
                                               Jtrip* jt = nullptr) {
    return cp_sample_v_under(n, a, eta, cp_ceiling(n, a, eta), rng, v_out, rej, jt);
}

// nonlinear_compton/cp/mod.rs:200-234: s, the azimuth and the Stokes
// parameters once v is sampled, given the Bessel triple at the emission's
// argument (the accepted trial's, from cp_diff_partial_rate_j).
static __device__ __noinline__ void cp_finish_j(int n, double a, double eta, double v, Jtrip jt, Draws& rng,
                                                double* s_out, double* theta_out, d3* sv_out) {
    double sn = 2.0 * n * eta / (1.0 + a * a);
    double s = v * (sn / (1.0 + sn));
    double theta = 2.0 * PI * rng.next();
    double w = s / (sn * (1.0 - s));
    double z = sqrt((double)(4 * n) * (double)n * (a * a / (1.0 + a * a)) * w * (1.0 - w));
    double jm = jt.m, j = jt.j, jp = jt.p;
    const double LASER_S3 = -1.0;
    double nz = (double)n / z;
    double xi0 = (1.0 - s + 1.0 / (1.0 - s)) * (jm * jm + jp * jp - 2.0 * j * j) - (2.0 * j / a) * (2.0 * j / a);
    double xi1 = 2.0 * (jm * jm + jp * jp - 2.0 * j * j) + 8.0 * j * j * (1.0 - nz * nz - 0.5 / (a * a));
    double xi3 = LASER_S3 * (1.0 - s + 1.0 / (1.0 - s)) * (1.0 - 2.0 * s / (sn * (1.0 - s))) * (jm * jm - jp * jp);
    double q = xi1 / xi0, u = 0.0, vv = xi3 / xi0;
    // rotate_by(pi/2 + theta): Stokes rotate by 2 angle
    double s2, c2;
    sincos(2.0 * (FRAC_PI_2 + theta), &s2, &c2);
    *sv_out = mk3(c2 * q + s2 * u, -s2 * q + c2 * u, vv);
    *s_out = s;
    *theta_out = theta;
}

// The same, evaluating the Bessel triple at the emission's argument.
static __device__ __noinline__ void cp_finish(int n, double a, double eta, double v, Draws& rng, double* s_out,
                                              double* theta_out, d3* sv_out) {
    Jtrip jt;
    cp_diff_partial_rate_j(n, a, eta, v, &jt);
    cp_finish_j(n, a, eta, v, jt, rng, s_out, theta_out, sv_out);
}

// nonlinear_compton/cp/mod.rs:181-234.  Returns a ptg status.
static __device__ __noinline__ int cp_sample(const NlcTables& t, double a, double eta, Draws& rng, int* n_out, double* s_out,
                                      double* theta_out, d3* sv_out, uint32_t* rej) {
    if (t.cp_cdf == nullptr) return 8;  // PTG_ERR_TABLES
    int n = cp_invert(t, a, eta, rng.next());
    if (n < 1) n = 1;
    double v = 0.0;
    Jtrip jt;
    int st = cp_sample_v(n, a, eta, rng, &v, rej, &jt);
    if (st != 0) return st;
    cp_finish_j(n, a, eta, v, jt, rng, s_out, theta_out, sv_out);
    *n_out = n;
    return 0;
}

// ------------------------------------------------------- ZMF kinematics -
__device__ __forceinline__ double dot4(d4 a, d4 b) { return a.t * b.t - a.x * b.x - a.y * b.y - a.z * b.z; }

// four_vector.rs:68-81
__device__ __forceinline__ d4 boost_by(d4 v, d4 u) {
    double gamma = u.t;
    double beta = sqrt(1.0 - 1.0 / (gamma * gamma));
    d3 n = normalize(mk3(u.x, u.y, u.z));
    d3 z = mk3(v.x, v.y, v.z);
    double nz = dot(n, z);
    return d4{gamma * (v.t - beta * nz), z.x + (gamma - 1.0) * nz * n.x - gamma * beta * v.t * n.x,
              z.y + (gamma - 1.0) * nz * n.y - gamma * beta * v.t * n.y,
              z.z + (gamma - 1.0) * nz * n.z - gamma * beta * v.t * n.z};
}

// polarization.rs:101-155: the rotation between the global Stokes basis and
// the LMA basis of a photon of momentum k, as (cos, sin) of twice the
// angle.  Into the LMA basis it is (c2, s2); out of it the reference's sine
// changes sign and its cosine does not, so it is (c2, -s2) exactly.
struct StokesBasis {
    double c2, s2;
};
__device__ __forceinline__ StokesBasis lma_stokes_basis(d4 k) {
    double k_minus = k.t - k.z;
    double c = (k.z * k_minus - k.x * k.x) / (k_minus * hypot(k.x, k.z));
    double sign = dsign(k.x * k.y);
    c = fmin(fmax(c, -1.0), 1.0);
    double s = sign * sqrt(1.0 - c * c);
    return StokesBasis{c * c - s * s, 2.0 * c * s};
}

__device__ __forceinline__ d3 stokes_rotate_cs(d3 sv, double c2, double s2) {
    return mk3(c2 * sv.x - s2 * sv.y, s2 * sv.x + c2 * sv.y, sv.z);
}

// Stokes parameters from the LMA basis
__device__ __forceinline__ d3 stokes_from_lma_basis(d3 sv, d4 k) {
    StokesBasis b = lma_stokes_basis(k);
    return stokes_rotate_cs(sv, b.c2, -b.s2);
}

// nonlinear_compton/mod.rs:58-138 for a sampled (n, s, cphi, Stokes):
// builds k' in the zero-momentum frame and boosts it to the lab.
static __device__ __noinline__ int nlc_kinematics(d4 k, d4 q, double a, double eta, int n, double s, double cphi, d3 sv,
                                           double pol_angle, bool classical, d4* k_out, d3* sv_out) {
    double ell = n;
    double p_zmf = classical ? ell * eta / sqrt(1.0 + a * a) : ell * eta / sqrt(1.0 + a * a + 2.0 * ell * eta);
    double ct = classical ? 1.0 - s * (1.0 + a * a) / (ell * eta) : 1.0 - s * (1.0 + a * a + 2.0 * ell * eta) / (ell * eta);
    if (!(ct <= 1.0 && ct >= -1.0)) return 3;  // PTG_ERR_SANITY
    d4 uz;
    if (classical) {
        double m = sqrt(dot4(q, q));
        uz = d4{q.t / m, q.x / m, q.y / m, q.z / m};
    } else {
        d4 t = d4{q.t + ell * k.t, q.x + ell * k.x, q.y + ell * k.y, q.z + ell * k.z};
        double m = sqrt(dot4(t, t));
        uz = d4{t.t / m, t.x / m, t.y / m, t.z / m};
    }
    d3 along;
    if (classical) {
        d4 b = boost_by(d4{ell * k.t, ell * k.x, ell * k.y, ell * k.z}, uz);
        along = normalize(mk3(b.x, b.y, b.z));
    } else {
        d4 b = boost_by(q, uz);
        along = -normalize(mk3(b.x, b.y, b.z));
    }
    double sp, cp;
    sincos(pol_angle, &sp, &cp);
    d4 e4 = boost_by(d4{0.0, cp, sp, 0.0}, uz);
    d3 eps = normalize(mk3(e4.x, e4.y, e4.z));
    eps = normalize(cross(along, cross(eps, along)));
    double sc, cc;
    sincos(cphi, &sc, &cc);
    d3 perp = rotate_around(eps, along, sc, cc);
    d3 kp = p_zmf * (ct * along + sqrt(1.0 - ct * ct) * perp);
    d4 kprime = d4{sqrt(dot(kp, kp)), kp.x, kp.y, kp.z};
    kprime = boost_by(kprime, d4{uz.t, -uz.x, -uz.y, -uz.z});
    // sv.rotate_by(-pol_angle), then into the global basis
    double s2, c2;
    sincos(-2.0 * pol_angle, &s2, &c2);
    d3 r = mk3(c2 * sv.x + s2 * sv.y, -s2 * sv.x + c2 * sv.y, sv.z);
    *sv_out = stokes_from_lma_basis(r, kprime);
    double s_new = dot4(k, kprime) / dot4(k, q);
    if (!(fabs(s - s_new) / s < 1.0e-2)) return 3;
    *k_out = kprime;
    return 0;
}


// ---------------------------------------------- classical CP emission ----
// nonlinear_compton/cp/mod.rs:78-86
__device__ __forceinline__ double cp_spectrum_low_eta(int n, double a, double v) {
    if (v < 0.0 || v >= 1.0) return 0.0;
    double z = sqrt(4.0 * a * a * ((double)n * n) * v * (1.0 - v) / (1.0 + a * a));
    double jm, j, jp;
    j_pm(z, n, &jm, &j, &jp);
    return n * (a * a * jm * jm - 2.0 * (1.0 + a * a) * j * j + a * a * jp * jp) / (1.0 + a * a);
}

// nonlinear_compton/cp/classical.rs:45-75
static __device__ __noinline__ double cp_cl_ceiling(int n, double a) {
    double n_switch = round(3.0 * (1.0 + 0.54 * pow(a, 2.75)));
    double mx = NAN;
    if (n == 1) {
        mx = cp_spectrum_low_eta(n, a, 0.99);
    } else if (a < 0.15 || n > (int)n_switch) {
        mx = cp_spectrum_low_eta(n, a, 0.5);
    } else {
        double b = a < 0.5 ? 2.3 * a : 0.8 * exp(-(a - 0.5) / 3.5) + 0.35;
        double v = 1.0 - 0.5 * pow(log((double)n), b) / pow(log(n_switch), b);
        for (int i = -4; i < 4; ++i) {
            double f = cp_spectrum_low_eta(n, a, fmin(v + 0.1 * (double)i / 4.0, 1.0));
            mx = isnan(mx) ? f : (isnan(f) ? mx : fmax(mx, f));
        }
    }
    return 1.1 * mx;
}

// nonlinear_compton/cp/classical.rs:87-130 (cdf_table [61][32][2])
static __device__ __noinline__ int cp_cl_harmonic_index(const NlcTables& t, double a, double frac) {
    if (log(a) <= PTG_NLC_CL_MIN) return 1;
    int ix = (int)((log(a) - PTG_NLC_CL_MIN) / PTG_NLC_CL_STEP);
    double dx = (log(a) - PTG_NLC_CL_MIN) / PTG_NLC_CL_STEP - ix;
    if (ix >= 60) return -1;
    double n = cp_cdf_corner(t.cp_cl_cdf + (size_t)ix * 64, nullptr, frac) * (1.0 - dx) +
               cp_cdf_corner(t.cp_cl_cdf + (size_t)(ix + 1) * 64, nullptr, frac) * dx;
    if (!isfinite(n)) return -1;
    double c = ceil(n);
    return c >= 2147483647.0 ? 2147483647 : (int)c;
}

// nonlinear_compton/cp/classical.rs:132-175.  Returns a ptg status.
static __device__ __noinline__ int cp_classical_sample(const NlcTables& t, double a, double eta, Draws& rng, int* n_out,
                                                       double* s_out, double* theta_out, d3* sv_out, uint32_t* rej) {
    if (t.cp_cl_cdf == nullptr) return 8;
    int n = cp_cl_harmonic_index(t, a, rng.next());
    if (n < 1) return 2;
    double mx = cp_cl_ceiling(n, a);
    double v = 0.0;
    int it;
    for (it = 0; it < rng.cap; ++it) {
        double vv = rng.next(), u = rng.next();
        if (u <= cp_spectrum_low_eta(n, a, vv) / mx) {
            v = vv;
            break;
        }
    }
    *rej += it;
    if (it == rng.cap) return 4;
    double s = v * (2.0 * n * eta / (1.0 + a * a));
    double theta = 2.0 * PI * rng.next();
    double z = sqrt((double)(4 * n * n) * (a * a / (1.0 + a * a)) * v * (1.0 - v));
    double jm, j, jp;
    j_pm(z, n, &jm, &j, &jp);
    double xi0 = 2.0 * (jm * jm + jp * jp - 2.0 * j * j) - (2.0 * j / a) * (2.0 * j / a);
    double xi1 = 2.0 * (jm * jm + jp * jp - 2.0 * j * j) + 8.0 * j * j * (1.0 - ((double)n / z) * ((double)n / z) - 0.5 / (a * a));
    double xi3 = 2.0 * (1.0 - 2.0 * v) * (jm * jm - jp * jp);
    double q = xi1 / xi0, u2 = 0.0 / xi0, v3 = xi3 / xi0;
    // rotate_by(pi/2 + theta)
    double s2, c2;
    sincos(2.0 * (PI / 2.0 + theta), &s2, &c2);
    *sv_out = mk3(c2 * q + s2 * u2, -s2 * q + c2 * u2, v3);
    *n_out = n;
    *s_out = s;
    *theta_out = theta;
    return 0;
}

}  // namespace ptg
