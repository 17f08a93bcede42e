// Oracle (test infrastructure only): see physics.h.
#include "physics.h"

#include <algorithm>
#include <cmath>

#include "../ptarmigan_gb300/tables/ptg_tables_small.h"

namespace orc {

// Rust's f64::powi lowers to binary exponentiation (compiler-rt __powidf2).
static inline double powi(double a, int b) {
    bool recip = b < 0;
    unsigned n = recip ? (unsigned)(-b) : (unsigned)b;
    double r = 1.0;
    while (true) {
        if (n & 1u) r *= a;
        n >>= 1;
        if (n == 0) break;
        a *= a;
    }
    return recip ? 1.0 / r : r;
}
static inline double fract(double x) { return x - std::trunc(x); }
static inline double clampd(double x, double lo, double hi) { return std::min(std::max(x, lo), hi); }

// ---------------------------------------------------------------- pwmci ---
// pwmci.rs:238-306 FitParameters::construct / evaluate
struct Fit {
    double x0, x1, f0, f1, m0, m1;
    double eval(double x) const {
        double t = (x - x0) / (x1 - x0);
        double h00 = (1.0 + 2.0 * t) * powi(1.0 - t, 2);
        double h10 = t * powi(1.0 - t, 2);
        double h01 = powi(t, 2) * (3.0 - 2.0 * t);
        double h11 = powi(t, 2) * (t - 1.0);
        return f0 * h00 + f1 * h01 + (x1 - x0) * (m0 * h10 + m1 * h11);
    }
};

static Fit construct_fit(int i, const double* tb, int len) {
    auto X = [&](int k) { return tb[2 * k]; };
    auto F = [&](int k) { return tb[2 * k + 1]; };
    double sec[3];
    if (i == 1) {
        sec[0] = (F(i) - F(i - 1)) / (X(i) - X(i - 1));
        sec[1] = sec[0];
        sec[2] = (F(i + 1) - F(i)) / (X(i + 1) - X(i));
    } else if (i == len - 1) {
        sec[0] = (F(i - 1) - F(i - 2)) / (X(i - 1) - X(i - 2));
        sec[1] = (F(i) - F(i - 1)) / (X(i) - X(i - 1));
        sec[2] = sec[1];
    } else {
        sec[0] = (F(i - 1) - F(i - 2)) / (X(i - 1) - X(i - 2));
        sec[1] = (F(i) - F(i - 1)) / (X(i) - X(i - 1));
        sec[2] = (F(i + 1) - F(i)) / (X(i + 1) - X(i));
    }
    double m0 = (sec[0] * sec[1] > 0.0) ? 0.5 * (sec[0] + sec[1]) : 0.0;
    double m1 = (sec[1] * sec[2] > 0.0) ? 0.5 * (sec[1] + sec[2]) : 0.0;
    if (sec[1] != 0.0) {
        if (m0 / sec[1] > 3.0) m0 = 3.0 * sec[1];
    }
    if (sec[2] != 0.0) {
        if (m1 / sec[2] > 3.0) m1 = 3.0 * sec[2];
    }
    return Fit{X(i - 1), X(i), F(i - 1), F(i), m0, m1};
}

enum Loc { BELOW, WITHIN, ABOVE };

// pwmci.rs:50-66: reverse linear scan for the last row with key < v
static void locate(const double* tb, int len, int col, double v, int* i, Loc* loc) {
    int found = -1;
    for (int k = len - 1; k >= 0; --k) {
        if (v > tb[2 * k + col]) {
            found = k;
            break;
        }
    }
    if (found < 0) {
        *i = 1;
        *loc = BELOW;
    } else if (found == len - 1) {
        *i = len - 1;
        *loc = ABOVE;
    } else {
        *i = found + 1;
        *loc = WITHIN;
    }
}

double Pwmci::evaluate(double x, bool* ok) const {
    int i;
    Loc loc;
    locate(tbl, len, 0, x, &i, &loc);
    if (loc == WITHIN) {
        *ok = true;
        return construct_fit(i, tbl, len).eval(x);
    }
    if (ext) {
        double x1 = tbl[2 * (i - 1)], f1 = tbl[2 * (i - 1) + 1];
        double x2 = tbl[2 * i], f2 = tbl[2 * i + 1];
        *ok = true;
        return f1 + (f2 - f1) * (x - x1) / (x2 - x1);
    }
    *ok = false;
    return 0.0;
}

static bool is_between(double x, double mn, double mx) {
    if (mn < mx) return x > mn && x < mx;
    if (mx < mn) return x > mx && x < mn;
    return true;
}

// pwmci.rs:102-229: Brent-style inverse quadratic / secant / bisection
double Pwmci::invert(double f, bool* ok) const {
    int i;
    Loc loc;
    locate(tbl, len, 1, f, &i, &loc);
    if (loc != WITHIN) {
        if (ext) {
            double x1 = tbl[2 * (i - 1)], f1 = tbl[2 * (i - 1) + 1];
            double x2 = tbl[2 * i], f2 = tbl[2 * i + 1];
            *ok = true;
            return x1 + (f - f1) * (x2 - x1) / (f2 - f1);
        }
        *ok = false;
        return 0.0;
    }
    Fit fit = construct_fit(i, tbl, len);
    struct Root {
        double x, f;
    } root[4] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
    root[0].x = tbl[2 * (i - 1)];
    root[0].f = tbl[2 * (i - 1) + 1] - f;
    root[1].x = tbl[2 * i];
    root[1].f = tbl[2 * i + 1] - f;
    if (std::fabs(root[1].f) < std::fabs(root[0].f)) std::swap(root[0], root[1]);
    root[2] = root[1];
    bool prev_bisect = false;
    for (int it = 0; it < 32; ++it) {
        double s;
        if (root[0].f != root[2].f && root[1].f != root[2].f) {
            double r = root[0].f / root[2].f;
            double ss = root[0].f / root[1].f;
            double t = root[1].f / root[2].f;
            double p = ss * (t * (r - t) * (root[2].x - root[0].x) - (1.0 - r) * (root[0].x - root[1].x));
            double q = (t - 1.0) * (r - 1.0) * (ss - 1.0);
            s = root[0].x + p / q;
        } else {
            s = root[0].x - (root[0].f * (root[0].x - root[1].x) / (root[0].f - root[1].f));
        }
        if (!is_between(s, 0.25 * (3.0 * root[1].x + root[0].x), root[0].x) ||
            (prev_bisect && std::fabs(s - root[0].x) >= 0.5 * std::fabs(root[0].x - root[2].x)) ||
            (!prev_bisect && std::fabs(s - root[0].x) >= 0.5 * std::fabs(root[2].x - root[3].x))) {
            prev_bisect = true;
            s = 0.5 * (root[0].x + root[1].x);
        } else {
            prev_bisect = false;
        }
        root[3] = root[2];
        root[2] = root[0];
        root[0].x = s;
        root[0].f = fit.eval(s) - f;
        if (root[1].f * root[0].f >= 0.0) {
            root[1] = root[0];
            root[0] = root[2];
        }
        if (std::fabs(root[1].f) < std::fabs(root[0].f)) std::swap(root[0], root[1]);
        double err = std::fabs(root[1].x - root[0].x) / std::fabs(root[0].x);
        if (err < 1.0e-6 || root[0].f == 0.0) break;
    }
    *ok = true;
    return root[0].x;
}

// ----------------------------------------------------------------- airy ---
static double series_up_to(const double (*s)[20], double x, int max_pow) {
    double sum = 0.0;
    for (int k = 0; k < 20; ++k) {
        int p = (int)s[1][k];
        if (p >= max_pow) break;
        sum += s[0][k] * powi(x, p);
    }
    return sum;
}

// airy.rs:41-78
double airy_ai(double x, bool* ok) {
    if (x < 0.0) {
        *ok = false;
        return 0.0;
    }
    *ok = true;
    if (x < 1.0) return series_up_to(PTG_AIRY_SMALL_X, x, 20);
    double s = 2.0 * std::pow(x, 1.5) / 3.0;
    double a = 0.262183997088323 * std::pow(s, -1.0 / 6.0) * std::exp(-s);
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
    for (int k = 0; k < n; ++k) integral += weights[k] * std::pow(2.0 + nodes[k] / s, -1.0 / 6.0);
    return a * integral;
}

// airy.rs:80-118
double airy_ai_prime(double x, bool* ok) {
    if (x < 0.0) {
        *ok = false;
        return 0.0;
    }
    *ok = true;
    if (x < 1.0) return series_up_to(PTG_AIRY_PRIME_SMALL_X, x, 20);
    double s = 2.0 * std::pow(x, 1.5) / 3.0;
    double b = -0.2898380090915846 * std::pow(s, 1.0 / 6.0) * std::exp(-s);
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
    for (int k = 0; k < n; ++k) integral += weights[k] * std::pow(2.0 + nodes[k] / s, 1.0 / 6.0);
    return b * integral;
}

// airy.rs:120-127
double bessel_k_1_3(double x, bool* ok) {
    double y = airy_ai(std::pow(1.5 * x, 2.0 / 3.0), ok);
    if (!*ok) return 0.0;
    return PI * std::cbrt(2.0 * std::sqrt(3.0) / x) * y;
}

// airy.rs:129-136
double bessel_k_2_3(double x, bool* ok) {
    double y = airy_ai_prime(std::pow(1.5 * x, 2.0 / 3.0), ok);
    if (!*ok) return 0.0;
    return -PI * std::pow(3.0, -1.0 / 6.0) * std::pow(2.0 / x, 2.0 / 3.0) * y;
}

// ------------------------------------------------ LCFA photon emission ---
// lcfa/photon_emission/mod.rs:13-33
double lcfa_photon_rate(double chi, double gamma) {
    double h;
    if (chi < 0.01) {
        h = 5.0 * (PI / 3.0) * (1.0 - 8.0 * chi / (5.0 * std::sqrt(3.0)));
    } else if (chi >= 100.0) {
        double c = std::cbrt(chi);
        h = -1019.4661473121777 + 1786.716527650374 * c * c;
        h = 1750.6263395722715 + c * c * h;
        h = -2260.1819695887225 + c * h;
        h = 0.00296527643253334 * h / (chi * chi);
    } else {
        double index = (std::log(chi) - PTG_LCFA_LN_H_CHI_TABLE[0][0]) / PTG_LCFA_PH_DELTA_LN_CHI;
        double w = fract(index);
        int i = (int)std::floor(index);
        double ln_h = (1.0 - w) * PTG_LCFA_LN_H_CHI_TABLE[i][1] + w * PTG_LCFA_LN_H_CHI_TABLE[i + 1][1];
        h = std::exp(ln_h);
    }
    return std::sqrt(3.0) * ALPHA_FINE * chi * h / (2.0 * PI * gamma * COMPTON_TIME);
}

// lcfa/photon_emission/classical.rs:11-14
double lcfa_classical_rate(double chi, double gamma) {
    double h = 5.0 * (PI / 3.0);
    return std::sqrt(3.0) * ALPHA_FINE * chi * h / (2.0 * PI * gamma * COMPTON_TIME);
}

// CDF record layout: [coeff, power, 31 x (x, f)]
static inline const double* cdf_table(const double* rec) { return rec + 2; }

// lcfa/photon_emission/mod.rs:35-69
static double from_linear_cdf_table(double global_zero, double local_zero, double rand, const double* cdf) {
    double coeff = cdf[0], power = cdf[1];
    const double* tb = cdf_table(cdf);
    double r_zero;
    if (local_zero < tb[0]) {
        r_zero = coeff * std::pow(local_zero - global_zero, power);
    } else {
        bool ok;
        double tmp = Pwmci(tb, 31).evaluate(local_zero, &ok);
        if (!ok) return local_zero;
        r_zero = tmp;
    }
    double r = r_zero + (1.0 - r_zero) * rand;
    double y;
    if (r <= tb[1]) {
        double tmp = (std::log(r) - std::log(coeff)) / power;
        y = std::exp(tmp) + global_zero;
    } else {
        bool ok;
        double res = Pwmci(tb, 31).invert(r, &ok);
        y = ok ? res : local_zero;
    }
    return y;
}

// lcfa/photon_emission/mod.rs:80-231
void lcfa_photon_sample(double chi, double gamma, double rand1, double rand2, double rand3, double* omega_mc2,
                        bool* has_theta, double* theta_out, double* cphi) {
    double index = (std::log(chi) - PTG_LCFA_PH_LN_CHI_MIN) / PTG_LCFA_PH_LN_CHI_STEP;
    double weight = fract(index);
    double fl = std::floor(index);
    int idx = fl < 0.0 ? 0 : (int)fl;  // Rust `as usize` saturates at 0

    if (std::log(chi) <= PTG_LCFA_PH_LN_CHI_MIN) {
        double om;
        lcfa_classical_sample(chi, gamma, rand1, rand2, rand3, &om, has_theta, theta_out, cphi);
        *omega_mc2 = om * gamma / (gamma + om);
        return;
    }

    double u;
    if (idx >= 41 - 1) {
        double u_bdy = (chi - 8.0) / 8.0;
        const double* hc = &PTG_LCFA_HIGH_CHI_CDF[0][0];
        const double* hp = &PTG_LCFA_HIGH_CHI_PEAK_CDF[0][0];
        Pwmci lower(hc, 32);
        double p_lower;
        bool ok;
        if (std::log(u_bdy) < hc[0]) {
            p_lower = 1.06327715546 * std::cbrt(u_bdy);
        } else if (std::log(u_bdy) < hc[2 * 31]) {
            double y = lower.evaluate(std::log(u_bdy), &ok);
            p_lower = 1.0 - std::exp(-1.0 * std::exp(y));
        } else {
            p_lower = 1.0 - 0.265819288864 * std::pow(u_bdy, -2.0 / 3.0);
        }
        double y_bdy = u_bdy / chi - 1.0 / 9.0;
        double scale = 0.84626000931 * std::pow(chi, -2.0 / 3.0);
        Pwmci higher(hp, 32, true);
        double p_higher;
        if (std::log(y_bdy) < hp[0]) {
            p_higher = scale * (1.0 - 7.7567692587 * y_bdy);
        } else if (std::log(y_bdy) < hp[2 * 31]) {
            double t = higher.evaluate(std::log(y_bdy), &ok);
            p_higher = scale * std::exp(-1.0 * std::exp(t));
        } else {
            p_higher = scale * 0.46534912384 * std::exp(-0.45 * u_bdy / chi) * std::pow(y_bdy, -5.0 / 3.0);
        }
        double r = rand1 * (p_lower + p_higher);
        if (r <= p_lower) {
            double target = std::log(-std::log(1.0 - r));
            if (target < hc[1]) {
                double uu = powi(r / 1.06327715546, 3);
                u = uu + 1.5 * uu * uu;
            } else if (target < hc[2 * 31 + 1]) {
                u = std::exp(lower.invert(target, &ok));
            } else {
                u = std::pow(0.265819288864 / (1.0 - r), 1.5);
            }
        } else {
            double target = (p_lower + p_higher - r) / scale;
            double y;
            if (target < hp[1]) {
                y = (1.0 - target) / 7.7567692587;
            } else {
                double tg = std::log(-1.0 * std::log(target));
                y = std::exp(higher.invert(tg, &ok));
            }
            u = (y + 1.0 / 9.0) * chi;
        }
    } else {
        const double* lo = PTG_LCFA_QUANTUM_CDF[idx];
        const double* up = PTG_LCFA_QUANTUM_CDF[idx + 1];
        double lr = std::log(rand1);
        bool ok;
        double ln_u_lower, ln_u_upper;
        if (lr <= cdf_table(lo)[1]) {
            ln_u_lower = (lr - std::log(lo[0])) / lo[1];
        } else {
            double res = Pwmci(cdf_table(lo), 31).invert(lr, &ok);
            ln_u_lower = ok ? res : cdf_table(lo)[2 * 30];
        }
        if (lr <= cdf_table(up)[1]) {
            ln_u_upper = (lr - std::log(up[0])) / up[1];
        } else {
            double res = Pwmci(cdf_table(up), 31).invert(lr, &ok);
            ln_u_upper = ok ? res : cdf_table(up)[2 * 30];
        }
        u = std::exp((1.0 - weight) * ln_u_lower + weight * ln_u_upper);
    }

    // polar angle
    double beta = 2.0 * u / (3.0 * chi);
    double delta = (1.0 + powi(1.0 + u, 2)) * std::pow(beta, -2.0 / 3.0) / (1.0 + u);
    double dindex = (std::log(delta) - PTG_LCFA_PH_LN_DELTA_MIN) / PTG_LCFA_PH_LN_DELTA_STEP;
    double dweight = fract(dindex);
    double dfl = std::floor(dindex);
    int di = dfl < 0.0 ? 0 : (int)dfl;
    double y;
    if (di >= 31 - 1) {
        y = from_linear_cdf_table(0.0, beta, rand2, PTG_LCFA_Y_INFINITE_DELTA_CDF);
    } else {
        double gz = std::pow(delta, -1.5);
        double y_lower = from_linear_cdf_table(gz, beta, rand2, PTG_LCFA_Y_CDF[di]);
        double y_upper = from_linear_cdf_table(gz, beta, rand2, PTG_LCFA_Y_CDF[di + 1]);
        y = (1.0 - dweight) * y_lower + dweight * y_upper;
    }
    double z = std::max(y / beta, 1.0);
    double cos_theta = (gamma - std::pow(z, 2.0 / 3.0) / (2.0 * gamma)) / std::sqrt(powi(gamma, 2) - 1.0);
    if (cos_theta >= 1.0) {
        *has_theta = true;
        *theta_out = 0.0;
    } else if (cos_theta >= -1.0) {
        *has_theta = true;
        *theta_out = std::acos(cos_theta);
    } else {
        *has_theta = false;
        *theta_out = 0.0;
    }
    *omega_mc2 = gamma * u / (1.0 + u);
    *cphi = 2.0 * PI * rand3;
}

// lcfa/photon_emission/classical.rs:24-61
void lcfa_classical_sample(double chi, double gamma, double rand1, double rand2, double rand3, double* omega_mc2,
                           bool* has_theta, double* theta_out, double* cphi) {
    double delta = std::acos((-9.0 + 50.0 * rand2 - 25.0 * powi(rand2, 2)) / 16.0);
    double z = powi((2.0 + 4.0 * std::cos(delta / 3.0)) / (5.0 * (1.0 - rand2)), 3);
    double ln_rand = std::log(rand1);
    const double* ct = &PTG_LCFA_CLASSICAL_SPECTRUM_TABLE[0][0];
    double x;
    if (ln_rand < ct[1]) {
        x = 1.020377255 * std::pow(rand1, 0.6);
    } else {
        bool ok;
        double ln_x = Pwmci(ct, 41).invert(ln_rand, &ok);
        if (!ok) ln_x = ct[2 * 40];
        x = std::exp(ln_x);
    }
    double u = 3.0 * chi * x / (2.0 * z);
    *omega_mc2 = u * gamma;
    double cos_theta = (gamma - std::pow(z, 2.0 / 3.0) / (2.0 * gamma)) / std::sqrt(powi(gamma, 2) - 1.0);
    if (cos_theta >= 1.0) {
        *has_theta = true;
        *theta_out = 0.0;
    } else if (cos_theta >= -1.0) {
        *has_theta = true;
        *theta_out = std::acos(cos_theta);
    } else {
        *has_theta = false;
        *theta_out = 0.0;
    }
    *cphi = 2.0 * PI * rand3;
}

// lcfa/photon_emission/mod.rs:239-298
Stokes lcfa_stokes_parameters(const V4& k, double chi, double gamma, V3 v, V3 w) {
    v = v.normalize();
    w = w.normalize();
    V3 n = k.spatial().normalize();
    double u = k.t / (gamma - k.t);
    double beta = std::asin(n * v.cross(w).normalize());
    double mu = std::sqrt(beta * beta + 1.0 / (gamma * gamma));
    double eta = u * powi(gamma * mu, 3) / (3.0 * chi);
    bool ok;
    double k13 = bessel_k_1_3(eta, &ok);
    if (!ok) k13 = 0.0;
    double k23 = bessel_k_2_3(eta, &ok);
    if (!ok) k23 = 0.0;
    double g = 0.5 * powi(u * mu, 2) * (k13 * k13 + k23 * k23) / (1.0 + u) + powi(mu * k23, 2) + powi(beta * k13, 2);
    double xi0 = (powi(mu * k23, 2) - powi(beta * k13, 2)) / g;
    double xi1 = 0.0;
    double xi2 = 2.0 * (1.0 + 0.5 * u * u / (1.0 + u)) * beta * mu * k13 * k23 / g;
    V3 e1(k.z, 0.0, -k.x);
    if (e1.norm_sqr() == 0.0)
        e1 = V3(1, 0, 0);
    else
        e1 = e1.normalize();
    double phi = std::acos(clampd(e1 * w, -1.0, 1.0));
    double sign = signum(w.cross(e1) * n);
    phi = sign * phi;
    double c2 = std::cos(2.0 * phi), s2 = std::sin(2.0 * phi);
    return Stokes(1.0, c2 * xi0 + s2 * xi1, -s2 * xi0 + c2 * xi1, xi2);
}

// lcfa/photon_emission/classical.rs:70-118
Stokes lcfa_classical_stokes_parameters(const V4& k, double chi, double gamma, V3 v, V3 w) {
    v = v.normalize();
    w = w.normalize();
    V3 n = k.spatial().normalize();
    double u = k.t / gamma;
    double beta = std::asin(n * v.cross(w).normalize());
    double mu = std::sqrt(beta * beta + 1.0 / (gamma * gamma));
    double eta = u * powi(gamma * mu, 3) / (3.0 * chi);
    bool ok;
    double k13 = bessel_k_1_3(eta, &ok);
    if (!ok) k13 = 0.0;
    double k23 = bessel_k_2_3(eta, &ok);
    if (!ok) k23 = 0.0;
    double g = powi(beta * k13, 2) + powi(mu * k23, 2);
    double xi0 = (powi(mu * k23, 2) - powi(beta * k13, 2)) / g;
    double xi1 = 0.0;
    double xi2 = 2.0 * beta * mu * k13 * k23 / g;
    double phi = std::asin((w - (n * w) * n) * V3(0.0, 1.0, 0.0));
    double c2 = std::cos(2.0 * phi), s2 = std::sin(2.0 * phi);
    return Stokes(1.0, c2 * xi0 + s2 * xi1, -s2 * xi0 + c2 * xi1, xi2);
}

// lcfa/photon_emission/mod.rs:330-346
double gaunt_factor(double chi) {
    if (chi <= 1.0e-3) {
        return 1.0 - 55.0 * std::sqrt(3.0) * chi / 16.0 + 48.0 * chi * chi;
    } else if (chi > 500.0) {
        double coeff = 0.5563810015417746;
        double c = std::cbrt(chi);
        double g = -1.0000341464898563 + coeff * c * c;
        g = 2.6235881916750565 + c * c * g;
        g = -3.8106418922532588 + c * g;
        return g / powi(chi, 3);
    }
    bool ok;
    return std::exp(Pwmci(&PTG_LCFA_GAUNT_FACTOR_TABLE[0][0], 25).evaluate(std::log(chi), &ok));
}

// ------------------------------------------------- LCFA pair creation ---
// lcfa/pair_creation/mod.rs:13-40
void lcfa_auxiliary_t(double chi, double* t_par, double* t_perp) {
    const double(*T)[3] = PTG_LCFA_LN_T_CHI_TABLE;
    const double D = PTG_LCFA_PAIR_DELTA_LN_CHI;
    if (chi <= 0.01) {
        *t_par = 0.0;
        *t_perp = 0.0;
    } else if (chi < 1.0) {
        int i = (int)((std::log(chi) - T[0][0]) / D);
        double dx = (chi - std::exp(T[i][0])) / (std::exp(T[i + 1][0]) - std::exp(T[i][0]));
        double par = (1.0 - dx) / T[i][1] + dx / T[i + 1][1];
        double perp = (1.0 - dx) / T[i][2] + dx / T[i + 1][2];
        *t_par = std::exp(1.0 / par);
        *t_perp = std::exp(1.0 / perp);
    } else if (chi < 100.0) {
        int i = (int)((std::log(chi) - T[0][0]) / D);
        double dx = (std::log(chi) - T[i][0]) / D;
        double par = (1.0 - dx) * T[i][1] + dx * T[i + 1][1];
        double perp = (1.0 - dx) * T[i][2] + dx * T[i + 1][2];
        *t_par = std::exp(par);
        *t_perp = std::exp(perp);
    } else {
        *t_par = 0.3036898468348568 / std::cbrt(chi) - 2.0 / (3.0 * chi);
        *t_perp = 0.4555347702522852 / std::cbrt(chi) - 2.0 / (3.0 * chi);
    }
}

// lcfa/pair_creation/mod.rs:48-73
double lcfa_pair_probability(const V4& ell, const Stokes& sv_in, double chi, const V3& a_perp, double dt,
                             Stokes* sv_new) {
    double c2, s2;
    Stokes sv = sv_in.in_basis(a_perp, ell.spatial(), &c2, &s2);
    double par_proj = 0.5 * (1.0 + sv.q);
    double perp_proj = 0.5 * (1.0 - sv.q);
    double t_par, t_perp;
    lcfa_auxiliary_t(chi, &t_par, &t_perp);
    double prob = ALPHA_FINE * chi * (par_proj * t_par + perp_proj * t_perp) * dt / (COMPTON_TIME * ell.t);
    double prob_avg = ALPHA_FINE * chi * 0.5 * (t_par + t_perp) * dt / (COMPTON_TIME * ell.t);
    double delta = ALPHA_FINE * chi * 0.5 * (t_par - t_perp) * dt / (COMPTON_TIME * ell.t);
    double sv1 = (sv.q * (1.0 - prob_avg) - delta) / (1.0 - prob);
    double sv2 = sv.u * (1.0 - prob_avg) / (1.0 - prob);
    *sv_new = Stokes(sv.i, c2 * sv1 + s2 * sv2, -s2 * sv1 + c2 * sv2, sv.v * (1.0 - prob_avg) / (1.0 - prob));
    return prob;
}

// lcfa/pair_creation/mod.rs:80-89
double lcfa_pair_spectrum(double s, double chi, double sv1) {
    double sum = 0.0;
    for (int k = 0; k < 32; ++k) {
        double t = PTG_GL_NODES[k], w = PTG_GL_WEIGHTS[k];
        double xi = 2.0 / (3.0 * chi * s * (1.0 - s));
        double pre = std::exp(-xi * std::cosh(t) + t);
        sum += w * pre * ((1.0 / (s * (1.0 - s)) - sv1 - 2.0) * std::cosh(2.0 * t / 3.0) + std::cosh(t / 3.0) / std::cosh(t));
    }
    return sum;
}

// lcfa/pair_creation/mod.rs:93-110
double lcfa_pair_spectrum_ceiling(double chi, double sv1) {
    double chi_switch = std::exp((1.5 - sv1) / std::sqrt(3.0));
    double mx;
    if (chi < chi_switch) {
        mx = lcfa_pair_spectrum(0.5, chi, sv1);
    } else if (chi > 100.0) {
        mx = lcfa_pair_spectrum(4.0 / (3.0 * chi), chi, sv1);
    } else {
        double m = -0.94866 + 0.170159 * sv1;
        double s = 0.5 * std::pow(chi_switch, -m) * std::pow(chi, m);
        mx = lcfa_pair_spectrum(s, chi, sv1);
    }
    return 1.05 * mx;
}

// lcfa/pair_creation/mod.rs:115-126
double lcfa_pair_angular_spectrum(double y, double s, double chi, double sv1) {
    double xi = 2.0 / (3.0 * chi * s * (1.0 - s));
    double pre = s / (1.0 - s) + (1.0 - s) / s - sv1;
    double z = 1.0 + 4.0 * chi * y * y;
    bool ok;
    double k = bessel_k_1_3(xi * z, &ok);
    if (!ok) k = 0.0;
    return y * (1.0 + pre * std::pow(z, 2.0 / 3.0)) * k;
}

// lcfa/pair_creation/mod.rs:130-141
double lcfa_pair_angular_spectrum_ceiling(double s, double chi, double sv1) {
    double y_min = 0.216, y_max = 0.259;
    double y_peak = y_min + (y_max - y_min) * (1.0 - std::tanh(std::pow(8.3 / chi, 2.0 / 3.0)));
    double y = y_peak * std::sqrt(1.0 - powi(1.0 - 2.0 * s, 2));
    return 1.05 * lcfa_pair_angular_spectrum(y, s, chi, sv1);
}

static double azimuthal_spectrum(double phi, double a, double b, double c, double d, double e, const Stokes& sv) {
    return a + b * (std::cos(2.0 * phi) * (1.0 - c) - c) * sv.q - d * std::sin(2.0 * phi) * sv.u + e * std::sin(phi) * sv.v;
}

// lcfa/pair_creation/mod.rs:141-173
static bool sample_azimuthal_angle(double s, double z, double chi, const Stokes& sv, DrawStream& rng, double* out) {
    double arg = 2.0 * z / (3.0 * chi * s * (1.0 - s));
    double k_ratio = (arg < 1.0e-4) ? 0.6368498843179743 / std::cbrt(arg)
                                    : 1.0 + 1.0 / (1.4624087952220928 * std::cbrt(arg) + 1.023821552056939 * std::sqrt(arg) + 6.0 * arg);
    double z23 = std::pow(z, 2.0 / 3.0);
    double a = 1.0 + z23 * (powi(s, 2) + powi(1.0 - s, 2)) / (s * (1.0 - s));
    double b = 1.0;
    double c = z23;
    double d = z23 - 1.0;
    double e = std::pow(z, 1.0 / 3.0) * (z23 - 1.0) * (powi(s, 2) + powi(1.0 - s, 2)) * k_ratio / (s * (1.0 - s));
    double mx = -HUGE_VAL;
    for (int i = 0; i < 32; ++i) mx = std::max(mx, azimuthal_spectrum(2.0 * PI * i / 32.0, a, b, c, d, e, sv));
    mx *= 1.1;
    for (int it = 0; it < REJECTION_CAP; ++it) {
        double phi = 2.0 * PI * rng.next();
        double u = rng.next();
        double f = azimuthal_spectrum(phi, a, b, c, d, e, sv);
        if (u <= f / mx) {
            *out = phi;
            return true;
        }
    }
    *out = 0.0;
    return false;
}

// lcfa/pair_creation/mod.rs:180-217
bool lcfa_pair_sample(const V4& ell, const Stokes& sv_in, double chi, const V3& a_perp, DrawStream& rng,
                      double* gamma_p, double* cos_theta, double* phi, double* s_out, double* z_out) {
    double gamma = ell.t;
    double c2, s2;
    Stokes sv = sv_in.in_basis(a_perp, ell.spatial(), &c2, &s2);
    double mx = lcfa_pair_spectrum_ceiling(chi, sv.q);
    double s = 0.0;
    bool found = false;
    for (int it = 0; it < REJECTION_CAP; ++it) {
        double ss = rng.next();
        double u = rng.next();
        double f = lcfa_pair_spectrum(ss, chi, sv.q);
        if (u <= f / mx) {
            s = ss;
            found = true;
            break;
        }
    }
    if (!found) return false;
    double amx = lcfa_pair_angular_spectrum_ceiling(s, chi, sv.q);
    double z = 1.0;
    found = false;
    for (int it = 0; it < REJECTION_CAP; ++it) {
        double y = rng.next();
        double u = rng.next();
        double f = lcfa_pair_angular_spectrum(y, s, chi, sv.q);
        if (u <= f / amx) {
            z = 1.0 + 4.0 * chi * y * y;
            found = true;
            break;
        }
    }
    if (!found) return false;
    double ph;
    if (!sample_azimuthal_angle(s, z, chi, sv, rng, &ph)) return false;
    double gp = s * gamma;
    double ct = (2.0 * gp * gp - std::pow(z, 2.0 / 3.0)) / (2.0 * gp * gp - 1.0);
    ct = std::max(ct, -1.0);
    *gamma_p = gp;
    *cos_theta = ct;
    *phi = ph;
    *s_out = s;
    *z_out = z;
    return true;
}

}  // namespace orc
