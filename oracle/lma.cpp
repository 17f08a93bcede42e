// Oracle (test infrastructure only): see lma.h.
#include "lma.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../ptarmigan_gb300/tables/ptg_tables_small.h"

namespace orc {

LmaTables g_lma;

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

// Rust's `as i32` on f64: saturating, NaN -> 0.
static int rust_as_i32(double x) {
    if (std::isnan(x)) return 0;
    if (x >= 2147483647.0) return 2147483647;
    if (x <= -2147483648.0) return (-2147483647 - 1);
    return (int)x;
}
static inline double sq(double x) { return x * x; }
constexpr double FRAC_PI_2 = 1.57079632679489661923132169163975144;
constexpr double FRAC_PI_4 = 0.785398163397448309615660845819875721;
constexpr double SQRT_2 = 1.41421356237309504880168872420969808;

// ----------------------------------------------------------- tables ----
static std::vector<std::vector<double>> g_store;

static bool read_ptgt(const std::string& path, std::vector<double>* data) {
    FILE* fp = std::fopen(path.c_str(), "rb");
    if (!fp) return false;
    char magic[4];
    uint32_t nd = 0;
    bool ok = std::fread(magic, 1, 4, fp) == 4 && std::memcmp(magic, "PTGT", 4) == 0 && std::fread(&nd, 4, 1, fp) == 1 &&
              nd > 0 && nd < 8;
    size_t n = 1;
    if (ok) {
        std::vector<uint32_t> shape(nd);
        ok = std::fread(shape.data(), 4, nd, fp) == nd;
        for (uint32_t d : shape) n *= d;
    }
    if (ok) {
        data->resize(n);
        ok = std::fread(data->data(), 8, n, fp) == n;
    }
    std::fclose(fp);
    return ok;
}

bool load_lma_tables(const std::string& dir, std::string* err) {
    struct Want {
        const char* name;
        const double** slot;
        size_t count;
        bool required;
    } wants[] = {
        {"nlc_lp_rate", &g_lma.nlc_lp_rate, 68 * 61, true},
        {"nlc_lp_cdf", &g_lma.nlc_lp_cdf, 4148 * 16 * 2, true},
        {"nlc_cp_rate", &g_lma.nlc_cp_rate, 70 * 61, true},
        {"nlc_cp_cdf", &g_lma.nlc_cp_cdf, 4270 * 32 * 2, false},
        {"nlc_lp_classical_rate", &g_lma.nlc_lp_cl_rate, 61, true},
        {"nlc_lp_classical_cdf", &g_lma.nlc_lp_cl_cdf, 61 * 16 * 2, true},
        {"nlc_cp_classical_rate", &g_lma.nlc_cp_cl_rate, 61, true},
        {"nlc_cp_classical_cdf", &g_lma.nlc_cp_cl_cdf, 61 * 32 * 2, true},
        {"bw_cp_total", &g_lma.bw_cp_total, 121 * 74 * 2, true},
        {"bw_lp_total", &g_lma.bw_lp_total, 61 * 25 * 2, true},
        {"bw_lp_cdf", &g_lma.bw_lp_cdf, 1525 * 16 * 3, true},
        {"bw_lp_mid_total", &g_lma.bw_lp_mid_total, 157 * 36 * 2, true},
        {"bw_lp_mid_cdf", &g_lma.bw_lp_mid_cdf, 5652 * 16 * 3, false},
    };
    for (auto& w : wants) {
        std::vector<double> data;
        std::string path = dir + "/" + w.name + ".ptgt";
        if (!read_ptgt(path, &data)) {
            if (w.required) {
                *err = "cannot read " + path;
                return false;
            }
            continue;
        }
        if (data.size() != w.count) {
            *err = path + " has the wrong size";
            return false;
        }
        g_store.push_back(std::move(data));
        *w.slot = g_store.back().data();
    }
    return true;
}

// ----------------------------------------------------------- Bessel ----
// special_functions/bessel.rs:38-70
static double j0(double x) {
    if (x < 0.1) return 1.0 - x * x / 4.0 + x * x * x * x / 64.0;
    if (x < 5.0) {
        double s = 0.0;
        for (int k = 0; k < 16; ++k)
            s += PTG_GAUSS_16_WEIGHTS[k] * 0.5 * std::cos(-x * std::sin(FRAC_PI_2 * (PTG_GAUSS_16_NODES[k] + 1.0)));
        return s;
    }
    if (x < 20.0) {
        double s = 0.0;
        for (int k = 0; k < 32; ++k)
            s += PTG_GAUSS_32_WEIGHTS[k] * 0.5 * std::cos(-x * std::sin(FRAC_PI_2 * (PTG_GAUSS_32_NODES[k] + 1.0)));
        return s;
    }
    double pre = std::sqrt(2.0 / (PI * x));
    double phase = FRAC_PI_4 - x;
    if (x < 60.0)
        return pre * ((1.0 - 9.0 / (128.0 * x * x) + 3675.0 / (32768.0 * x * x * x * x) - 0.5725014209747314 * powi(x, -6)) *
                          std::cos(phase) -
                      (1.0 / (8.0 * x) - 75.0 / (1024.0 * x * x * x) + 0.2271080017089844 * powi(x, -5)) * std::sin(phase));
    return pre * ((1.0 - 9.0 / (128.0 * x * x) + 3675.0 / (32768.0 * x * x * x * x)) * std::cos(phase) -
                  (1.0 / (8.0 * x) - 75.0 / (1024.0 * x * x * x)) * std::sin(phase));
}

// special_functions/bessel.rs:72-112
static double j1(double x) {
    if (x < 0.1) return (x / 2.0) * (1.0 - x * x / 8.0 + x * x * x * x / 192.0);
    if (x < 5.0) {
        double s = 0.0;
        for (int k = 0; k < 16; ++k) {
            double t = FRAC_PI_2 * (PTG_GAUSS_16_NODES[k] + 1.0);
            s += PTG_GAUSS_16_WEIGHTS[k] * 0.5 * std::cos(t - x * std::sin(t));
        }
        return s;
    }
    if (x < 20.0) {
        double s = 0.0;
        for (int k = 0; k < 32; ++k) {
            double t = FRAC_PI_2 * (PTG_GAUSS_32_NODES[k] + 1.0);
            s += PTG_GAUSS_32_WEIGHTS[k] * 0.5 * std::cos(t - x * std::sin(t));
        }
        return s;
    }
    double pre = std::sqrt(2.0 / (PI * x));
    double phase = FRAC_PI_4 + x;
    if (x < 60.0)
        return pre * (-(1.0 + 15.0 / (128.0 * x * x) - 4725.0 / (32768.0 * x * x * x * x) + 0.6765925884246826 * powi(x, -6)) *
                          std::cos(phase) +
                      (3.0 / (8.0 * x) - 105.0 / (1024.0 * x * x * x) + 0.2775764465332031 * powi(x, -5)) * std::sin(phase));
    return pre * (-(1.0 + 15.0 / (128.0 * x * x) - 4725.0 / (32768.0 * x * x * x * x)) * std::cos(phase) +
                  (3.0 / (8.0 * x) - 105.0 / (1024.0 * x * x * x)) * std::sin(phase));
}

static inline int rem_euclid2(int n) { return ((n % 2) + 2) % 2; }

// special_functions/bessel.rs:117-176: Miller's backward recurrence,
// normalised by J0 + 2 sum J_2k = 1.
static void triple_j(int n, double x, double* a, double* b, double* c) {
    if (x == 0.0) {
        *a = (n == 1) ? 1.0 : 0.0;
        *b = (n == 0) ? 1.0 : 0.0;
        *c = (n == -1) ? 1.0 : 0.0;
        return;
    }
    double v = x / (double)n;
    int nmax = 1 + n + (int)(5.0 / (1.0 - 0.9 * v));
    if (rem_euclid2(nmax) != 0) nmax += 1;
    int n_even = rem_euclid2(n) == 0 ? 1 : 0;
    int k_stop = n - 1 - n_even;
    double quad[4] = {1.0, 0.0, 0.0, 0.0};
    double total = 0.0;
    // (k_stop..=nmax).rev().step_by(2): nmax, nmax-2, ... >= k_stop
    for (int k = nmax; k >= k_stop; k -= 2) {
        quad[3] = quad[1];
        quad[2] = quad[0];
        quad[1] = (double)(2 * (k + 2)) * quad[2] / x - quad[3];
        quad[0] = (double)(2 * (k + 1)) * quad[1] / x - quad[2];
        total += quad[0];
    }
    int idx = n_even;
    double t0 = quad[idx], t1 = quad[idx + 1], t2 = quad[idx + 2];
    // (0..=k_stop).rev().step_by(2).skip(1): k_stop-2, k_stop-4, ... >= 0
    if (k_stop >= 0) {
        for (int k = k_stop - 2; k >= 0; k -= 2) {
            quad[3] = quad[1];
            quad[2] = quad[0];
            quad[1] = (double)(2 * (k + 2)) * quad[2] / x - quad[3];
            quad[0] = (double)(2 * (k + 1)) * quad[1] / x - quad[2];
            total += quad[0];
        }
    }
    double norm = 2.0 * total - quad[0];
    if (std::isnan(norm)) {
        *a = *b = *c = 0.0;
    } else {
        *a = t0 / norm;
        *b = t1 / norm;
        *c = t2 / norm;
    }
}

// special_functions/bessel.rs:178-199: uniform asymptotic (Airy) expansion
static double zeta_at(double z) {
    if (z < 1.0) {
        double tmp = std::log((1.0 + std::sqrt(1.0 - z * z)) / z) - std::sqrt(1.0 - z * z);
        return std::pow(3.0 * tmp / 2.0, 2.0 / 3.0);
    }
    double tmp = std::sqrt(z * z - 1.0) - std::acos(1.0 / z);
    return -std::pow(3.0 * tmp / 2.0, 2.0 / 3.0);
}

double bessel_j_asymptotic(int n, double x) {
    double m = (double)n;
    double z = x / m;
    double zeta = zeta_at(z);
    bool ok;
    double arg = std::pow(m, 2.0 / 3.0) * zeta;
    double ai = airy_ai(arg, &ok);
    if (!ok) ai = 0.0;
    double aip = airy_ai_prime(arg, &ok);
    if (!ok) aip = 0.0;
    double pre = 4.0 * zeta / (1.0 - z * z);
    double bk = 5.0 / (48.0 * zeta * zeta) - (2.0 + 3.0 * z * z) / (24.0 * std::sqrt(zeta) * std::pow(1.0 - z * z, 1.5));
    return std::pow(pre, 0.25) * (ai / std::pow(m, 1.0 / 3.0) - aip * bk / std::pow(m, 5.0 / 3.0));
}

double bessel_triple_j_mid(int n, double x) {
    double a, b, c;
    triple_j(n, x, &a, &b, &c);
    return b;
}

// bessel.rs:26-34
void bessel_j_pm(double x, int n, double* jm1, double* j, double* jp1) {
    if (n < 1000) {
        triple_j(n, x, jm1, j, jp1);
    } else {
        double jn = bessel_j_asymptotic(n, x);
        double jp = bessel_j_asymptotic(n + 1, x);
        *jm1 = (double)(2 * n) * jn / x - jp;
        *j = jn;
        *jp1 = jp;
    }
}

// bessel.rs:18-24
double bessel_j(double x, int n) {
    if (n == 0) return j0(x);
    if (n == 1) return j1(x);
    return bessel_triple_j_mid(n, x);
}

// --------------------------------------------------- CP LMA emission ---
// nonlinear_compton/cp/mod.rs:17-38
double cp_diff_partial_rate(int n, double a, double eta, double v) {
    if (v < 0.0 || v >= 1.0) return 0.0;
    double sn = 2.0 * n * eta / (1.0 + a * a);
    double smax = sn / (1.0 + sn);
    double vs = v * smax;
    double z = std::sqrt(4.0 * powi((double)n, 2) * (a * a / (1.0 + a * a)) * (vs / (sn * (1.0 - vs))) *
                         (1.0 - vs / (sn * (1.0 - vs))));
    double jm, j, jp;
    bessel_j_pm(z, n, &jm, &j, &jp);
    return -smax * (powi(j, 2) + 0.5 * a * a * (1.0 + 0.5 * powi(vs, 2) / (1.0 - vs)) * (2.0 * powi(j, 2) - powi(jp, 2) - powi(jm, 2)));
}

// nonlinear_compton/cp/mod.rs:42-75
double cp_ceiling_diff_partial_rate(int n, double a, double eta) {
    double sn = 2.0 * n * eta / (1.0 + a * a);
    int n_switch = (int)(32.3 * (1.0 + 0.476 * std::pow(a, 1.56)));
    double mx;
    if (sn < 2.0 || n < n_switch) {
        double v_opt = (1.0 + sn) / (2.0 + sn);
        double lower = -HUGE_VAL, upper = -HUGE_VAL;
        for (int i = 0; i < 16; ++i) lower = std::max(lower, cp_diff_partial_rate(n, a, eta, i * v_opt / 16.0));
        for (int i = 0; i < 16; ++i)
            upper = std::max(upper, cp_diff_partial_rate(n, a, eta, v_opt + i * (1.0 - v_opt) / 16.0));
        mx = std::max(lower, upper);
    } else {
        double lower = -HUGE_VAL, upper = -HUGE_VAL;
        for (int k = 0; k < 16; ++k) {
            double u = 0.5 * (1.0 + sn) * (PTG_GAUSS_16_NODES[k] + 1.0);
            lower = std::max(lower, cp_diff_partial_rate(n, a, eta, u / (1.0 + u)));
        }
        for (int k = 0; k < 16; ++k) {
            double u = (1.0 + sn) + 0.5 * 2.0 * (1.0 + sn) * (PTG_GAUSS_16_NODES[k] + 1.0);
            upper = std::max(upper, cp_diff_partial_rate(n, a, eta, u / (1.0 + u)));
        }
        mx = std::max(lower, upper);
    }
    return 1.2 * mx;
}

// nonlinear_compton/cp/mod.rs:78-87
double cp_spectrum_low_eta(int n, double a, double v) {
    if (v < 0.0 || v >= 1.0) return 0.0;
    double z = std::sqrt(4.0 * a * a * powi((double)n, 2) * v * (1.0 - v) / (1.0 + a * a));
    double jm, j, jp;
    bessel_j_pm(z, n, &jm, &j, &jp);
    return n * (a * a * powi(jm, 2) - 2.0 * (1.0 + a * a) * powi(j, 2) + a * a * powi(jp, 2)) / (1.0 + a * a);
}

// nonlinear_compton/cp/mod.rs:92-136
double cp_partial_rate(int n, double a, double eta) {
    double sn = 2.0 * n * eta / (1.0 + a * a);
    int n_switch = (int)(32.3 * (1.0 + 0.476 * std::pow(a, 1.56)));
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
            lower += 0.5 * (1.0 + sn) * PTG_GAUSS_32_WEIGHTS[k] * cp_diff_partial_rate(n, a, eta, u / (1.0 + u)) / powi(1.0 + u, 2);
        }
        for (int k = 0; k < 32; ++k) {
            double u = (1.0 + sn) + 0.5 * 2.0 * (1.0 + sn) * (PTG_GAUSS_32_NODES[k] + 1.0);
            upper += 0.5 * 2.0 * (1.0 + sn) * PTG_GAUSS_32_WEIGHTS[k] * cp_diff_partial_rate(n, a, eta, u / (1.0 + u)) /
                     powi(1.0 + u, 2);
        }
    }
    return lower + upper;
}

// nonlinear_compton/cp/classical.rs:22-43
bool cp_classical_rate(double a, double eta, double* out) {
    double x = std::log(a);
    if (x < PTG_NLC_CL_MIN) {
        *out = 2.0 * a * a * eta / 3.0;
        return true;
    }
    int ix = (int)((x - PTG_NLC_CL_MIN) / PTG_NLC_CL_STEP);
    if (ix < 61 - 1) {
        double dx = (x - PTG_NLC_CL_MIN) / PTG_NLC_CL_STEP - ix;
        double f = (1.0 - dx) * g_lma.nlc_cp_cl_rate[ix] + dx * g_lma.nlc_cp_cl_rate[ix + 1];
        *out = eta * std::exp(f);
        return true;
    }
    return false;
}

// nonlinear_compton/cp/mod.rs:160-176, tables/mod.rs:11-35
bool cp_rate(double a, double eta, double* out) {
    const double MIN0 = PTG_NLC_CP_MIN_0, MIN1 = PTG_NLC_CP_MIN_1, S0 = PTG_NLC_CP_STEP_0, S1 = PTG_NLC_CP_STEP_1;
    if (std::log(eta) < MIN1) return cp_classical_rate(a, eta, out);
    if (std::log(a) < MIN0) {
        *out = a * a * (2.0 + 8.0 * eta + 9.0 * eta * eta + eta * eta * eta) / (2.0 * eta * powi(1.0 + 2.0 * eta, 2)) -
               a * a * (2.0 + 2.0 * eta - eta * eta) * std::log(1.0 + 2.0 * eta) / (4.0 * eta * eta);
        return true;
    }
    bool contains = std::log(a) >= MIN0 && a < 20.0 && std::log(eta) >= MIN1 && eta < 2.0;
    if (!contains) return false;
    int ia = (int)((std::log(a) - MIN0) / S0);
    int ie = (int)((std::log(eta) - MIN1) / S1);
    if (ia >= 61 - 1 || ie >= 70 - 1) return false;
    double da = (std::log(a) - MIN0) / S0 - ia;
    double de = (std::log(eta) - MIN1) / S1 - ie;
    const double* T = g_lma.nlc_cp_rate;
    double f = (1.0 - da) * (1.0 - de) * T[ie * 61 + ia] + da * (1.0 - de) * T[ie * 61 + ia + 1] +
               (1.0 - da) * de * T[(ie + 1) * 61 + ia] + da * de * T[(ie + 1) * 61 + ia + 1];
    *out = std::exp(f);
    return true;
}

// nonlinear_compton/cp/tables/mod.rs:37-45: [ln n, ln(-ln(1 - cdf))] of the first 31 rows
static void cp_rescale(double frac, const double* table, double* frac2, double* out /*[31][2]*/) {
    for (int i = 0; i < 31; ++i) {
        out[2 * i] = std::log(table[2 * i]);
        out[2 * i + 1] = std::log(-1.0 * std::log(1.0 - table[2 * i + 1]));
    }
    *frac2 = std::log(-1.0 * std::log(1.0 - frac));
}

// nonlinear_compton/cp/tables/mod.rs:47-121 (needs the regenerated CDF table)
int cp_invert(double a, double eta, double frac) {
    const double MIN0 = PTG_NLC_CP_MIN_0, MIN1 = PTG_NLC_CP_MIN_1, S0 = PTG_NLC_CP_STEP_0, S1 = PTG_NLC_CP_STEP_1;
    const double* T = g_lma.nlc_cp_cdf;
    if (std::log(a) <= MIN0) return 1;
    auto corner = [&](int idx) {
        const double* table = T + (size_t)idx * 64;
        if (frac <= table[1]) return 0.9;
        double f2, rs[62];
        cp_rescale(frac, table, &f2, rs);
        bool ok;
        return std::exp(Pwmci(rs, 31, true).invert(f2, &ok));
    };
    if (std::log(eta) <= MIN1) {
        int ix = (int)((std::log(a) - MIN0) / S0);
        double dx = (std::log(a) - MIN0) / S0 - ix;
        double n = corner(ix) * (1.0 - dx) + corner(ix + 1) * dx;
        return (int)std::ceil(n);
    }
    int ix = (int)((std::log(a) - MIN0) / S0);
    int iy = (int)((std::log(eta) - MIN1) / S1);
    double dx = (std::log(a) - MIN0) / S0 - ix;
    double dy = (std::log(eta) - MIN1) / S1 - iy;
    int idx[4] = {61 * iy + ix, 61 * iy + ix + 1, 61 * (iy + 1) + ix, 61 * (iy + 1) + ix + 1};
    double w[4] = {(1.0 - dx) * (1.0 - dy), dx * (1.0 - dy), (1.0 - dx) * dy, dx * dy};
    double n = 0.0;
    for (int k = 0; k < 4; ++k) n += corner(idx[k]) * w[k];
    return (int)std::ceil(n);
}

// nonlinear_compton/cp/mod.rs:181-234
int cp_sample(double a, double eta, DrawStream& rng, int* n_out, double* s_out, double* theta_out, Stokes* sv_out,
              uint64_t* rej) {
    if (!g_lma.nlc_cp_cdf) return PTG_ERR_TABLES;
    int n = cp_invert(a, eta, rng.next());
    double mx = cp_ceiling_diff_partial_rate(n, a, eta);
    double v = 0.0;
    int it;
    for (it = 0; it < REJECTION_CAP; ++it) {
        double vv = rng.next(), u = rng.next();
        if (u <= cp_diff_partial_rate(n, a, eta, vv) / mx) {
            v = vv;
            break;
        }
    }
    *rej += it;
    if (it == REJECTION_CAP) return PTG_ERR_REJECTION_CAP;
    double sn = 2.0 * n * eta / (1.0 + a * a);
    double s = v * (sn / (1.0 + sn));
    double theta = 2.0 * PI * rng.next();
    double z = std::sqrt((double)(4 * n * n) * (a * a / (1.0 + a * a)) * (s / (sn * (1.0 - s))) * (1.0 - s / (sn * (1.0 - s))));
    double jm, j, jp;
    bessel_j_pm(z, n, &jm, &j, &jp);
    const double LASER_S3 = -1.0;
    double xi0 = (1.0 - s + 1.0 / (1.0 - s)) * (jm * jm + jp * jp - 2.0 * j * j) - powi(2.0 * j / a, 2);
    double xi1 = 2.0 * (jm * jm + jp * jp - 2.0 * j * j) + 8.0 * j * j * (1.0 - powi((double)n / z, 2) - 0.5 / (a * a));
    double xi2 = 0.0;
    double xi3 = LASER_S3 * (1.0 - s + 1.0 / (1.0 - s)) * (1.0 - 2.0 * s / (sn * (1.0 - s))) * (jm * jm - jp * jp);
    Stokes sv(1.0, xi1 / xi0, xi2 / xi0, xi3 / xi0);
    *sv_out = sv.rotate_by(FRAC_PI_2 + theta);
    *n_out = n;
    *s_out = s;
    *theta_out = theta;
    return PTG_OK;
}

// nonlinear_compton/lp/linear.rs:6-48
double lp_linear_rate(double a, double eta) {
    double eta2 = eta * eta, eta3 = eta2 * eta;
    if (eta > 1.0e-3)
        return (a * a / 8.0) *
               (0.5 + 4.0 / eta - 0.5 / ((1.0 + 2.0 * eta) * (1.0 + 2.0 * eta)) + (1.0 - 2.0 / eta - 2.0 / eta2) * std::log(1.0 + 2.0 * eta));
    return (a * a / 8.0) * (8.0 * eta / 3.0 - 16.0 * eta2 / 3.0 + 208.0 * eta3 / 15.0);
}



// Complex arithmetic with the semantics of num-complex 0.4.0 (the crate the
// reference uses for the saddle-point double Bessel function): products by
// the full formula, sqrt exact on the real axis, ln/exp through polar form,
// acos(z) = -i ln(i sqrt(1 - z^2) + z).  Signed zeros follow IEEE, which
// decides the branch of sqrt and therefore of acos for real z > 1.
struct Cx {
    double re, im;
};
static inline Cx cx_mul(Cx a, Cx b) { return Cx{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
static inline Cx cx_add(Cx a, Cx b) { return Cx{a.re + b.re, a.im + b.im}; }
static inline Cx cx_sub(Cx a, Cx b) { return Cx{a.re - b.re, a.im - b.im}; }
static inline Cx cx_scale(double s, Cx a) { return Cx{s * a.re, s * a.im}; }
static inline double cx_norm(Cx a) { return std::hypot(a.re, a.im); }
static inline double cx_arg(Cx a) { return std::atan2(a.im, a.re); }
static inline Cx cx_from_polar(double r, double t) { return Cx{r * std::cos(t), r * std::sin(t)}; }
static inline Cx cx_ln(Cx a) { return Cx{std::log(cx_norm(a)), cx_arg(a)}; }
static inline Cx cx_exp(Cx a) { return cx_from_polar(std::exp(a.re), a.im); }
static inline Cx cx_sin(Cx a) { return Cx{std::sin(a.re) * std::cosh(a.im), std::cos(a.re) * std::sinh(a.im)}; }
static inline Cx cx_sqrt(Cx a) {
    if (a.im == 0.0) {
        if (!std::signbit(a.re)) return Cx{std::sqrt(a.re), a.im};
        double im = std::sqrt(-a.re);
        return std::signbit(a.im) ? Cx{0.0, -im} : Cx{0.0, im};
    }
    if (a.re == 0.0) {
        double x = std::sqrt(std::fabs(a.im) / 2.0);
        return std::signbit(a.im) ? Cx{x, -x} : Cx{x, x};
    }
    return cx_from_polar(std::sqrt(cx_norm(a)), cx_arg(a) / 2.0);
}
static inline Cx cx_acos(Cx z) {
    const Cx I{0.0, 1.0}, ONE{1.0, 0.0}, NEG_I{-0.0, -1.0};
    return cx_mul(NEG_I, cx_ln(cx_add(cx_mul(cx_sqrt(cx_sub(ONE, cx_mul(z, z))), I), z)));
}

// ------------------------------------------------------- DoubleBessel --
struct DoubleBessel;
static double lp_ceiling(double a, double eta, DoubleBessel& dj);
// special_functions/double_bessel.rs:7-410: J(n, x, y) = (1/pi) int_0^pi
// cos(-n t + x cos t - y sin t) dt, for indices n-2..n+2
struct DbElem {
    double xi[3], lambda[2], f, g, h;
};

struct DoubleBessel {
    int n, k_min;
    double x_max, y_max;
    std::vector<DbElem> tbl;
    static constexpr int DELTA = 100;

    DoubleBessel(int n_, double xm, double ym) : n(n_) {
        int n_minus_bound = (int)std::floor(-2.0 * ym - xm);
        int n_plus_bound = xm > 4.0 * (2.0 - SQRT_2) * ym ? (int)std::ceil(xm) : (int)std::ceil(2.0 * ym + xm * xm / (16.0 * ym));
        int size = n_plus_bound - n_minus_bound + 2 * DELTA;
        tbl.assign(size, DbElem{{1.0, 1.0, 1.0}, {1.0, 1.0}, 0.0, 0.0, 0.0});
        k_min = n_minus_bound - DELTA;
        x_max = std::fabs(xm);
        y_max = std::fabs(ym);
    }

    // double_bessel.rs:142-246
    void around(double x, double y, double j[5]) {
        int n_minus = (int)std::floor(-2.0 * y - x);
        int n_plus = (8.0 * y > x) ? (int)std::ceil(2.0 * y + x * x / (16.0 * y)) : (int)std::ceil(-2.0 * y + x);
        size_t len = tbl.size();
        for (size_t i = 1; i < len; ++i) {
            int k = (int)i + k_min;
            DbElem& t = tbl[i];
            const DbElem& p = tbl[i - 1];
            t.xi[0] = -x - 4.0 * y * y / p.xi[2];
            t.xi[1] = 2.0 * (double)(k - 1) - 2.0 * y * p.xi[0] / p.xi[2];
            t.xi[2] = -x - 2.0 * y * p.xi[1] / p.xi[2];
            t.lambda[0] = t.xi[0] - 2.0 * y * t.xi[2] / p.lambda[1];
            t.lambda[1] = t.xi[1] - p.lambda[0] * t.xi[2] / p.lambda[1];
        }
        double initial = n < 2000 ? 1.0e-100 : 1.0e-300;
        tbl[len - 1].f = 0.0;
        tbl[len - 2].f = 1.0 * initial;
        tbl[len - 3].f = 2.0 * initial;
        tbl[len - 1].g = 0.0;
        tbl[len - 2].g = 1.0 / initial;
        tbl[len - 3].g = -(2.0 * y * tbl[len - 1].g + tbl[len - 2].lambda[0] * tbl[len - 2].g) / tbl[len - 2].lambda[1];
        int k_match = (n_plus + n_minus) / 2;
        size_t i_match = (size_t)(k_match - k_min);
        tbl[i_match].f = 0.0;
        tbl[i_match].g = 0.0;
        for (long i = (long)len - 4; i >= 0; --i) {
            tbl[i].f = -(2.0 * y * tbl[i + 3].f + tbl[i + 2].xi[0] * tbl[i + 2].f + tbl[i + 2].xi[1] * tbl[i + 1].f) / tbl[i + 2].xi[2];
            tbl[i].g = -(2.0 * y * tbl[i + 2].g + tbl[i + 1].lambda[0] * tbl[i + 1].g) / tbl[i + 1].lambda[1];
            if (tbl[i].f > 1.0 && std::fabs(tbl[i_match].g) < 1.0e200) {
                for (size_t jj = (size_t)i; jj < len; ++jj) {
                    tbl[jj].f *= 1.0e-100;
                    tbl[jj].g *= 1.0e100;
                }
            }
        }
        double f_match = tbl[i_match].f, g_match = tbl[i_match].g;
        double sum_linear = 0.0, rss = 0.0;
        for (size_t i = 0; i < i_match; ++i) {
            tbl[i].h = tbl[i].g;
            sum_linear += tbl[i].h;
            rss = std::hypot(rss, tbl[i].h);
        }
        for (size_t i = i_match; i < len; ++i) {
            tbl[i].h = g_match * tbl[i].f / f_match;
            sum_linear += tbl[i].h;
            rss = std::hypot(rss, tbl[i].h);
        }
        size_t it = (size_t)(n - k_min);
        for (int q = 0; q < 5; ++q) {
            const DbElem& t = tbl[it - 2 + q];
            double val = signum(t.h / sum_linear) * std::fabs(t.h) / rss;
            j[q] = std::isfinite(val) ? val : 0.0;
        }
    }

    // double_bessel.rs:272-355 (saddle-point approximation)
    static double j_spa(int ni, double x, double y) {
        double n = ni;
        if (n <= -2.0 * y + x) {
            double ct = y > 0.0 ? x / (8.0 * y) - std::sqrt(x * x / (64.0 * y * y) + 0.5 - n / (4.0 * y)) : n / x;
            double th = std::acos(ct);
            double f = x * std::sin(th) - y * std::sin(2.0 * th);
            double d2f = -x * std::sin(th) + 4.0 * y * std::sin(2.0 * th);
            double phi = FRAC_PI_4 * signum(d2f);
            return std::cos(f - n * th + phi) * std::sqrt(2.0 / (PI * std::fabs(d2f)));
        } else if (8.0 * y < x || n > 2.0 * y + x * x / (16.0 * y)) {
            double disc = x * x / (64.0 * y * y) + 0.5 - n / (4.0 * y);
            Cx ct;
            if (std::isnan(disc))
                ct = Cx{n / x, 0.0};
            else if (disc < 0.0)
                ct = Cx{x / (8.0 * y), std::sqrt(-disc)};
            else
                ct = Cx{x / (8.0 * y) - std::sqrt(disc), 0.0};
            const Cx I{0.0, 1.0};
            Cx th = cx_acos(ct);
            Cx th2 = cx_scale(2.0, th);
            Cx f = cx_mul(I, cx_sub(cx_add(cx_scale(-n, th), cx_scale(x, cx_sin(th))), cx_scale(y, cx_sin(th2))));
            Cx d2f = cx_mul(I, cx_add(cx_scale(-x, cx_sin(th)), cx_scale(4.0 * y, cx_sin(th2))));
            Cx phase = cx_add(f, Cx{0.0, (PI - cx_arg(d2f)) / 2.0});
            double term;
            if (f.im == 0.0 && d2f.im == 0.0) {
                term = 0.5 * std::exp(-f.re) * std::sqrt(2.0 / (PI * cx_norm(d2f)));
            } else {
                term = cx_exp(phase).re * std::sqrt(2.0 / (PI * cx_norm(d2f)));
            }
            return disc != 0.0 ? term : 0.0;
        } else {
            double r = std::sqrt(x * x / (64.0 * y * y) + 0.5 - n / (4.0 * y));
            double ct0 = x / (8.0 * y) - r, ct1 = x / (8.0 * y) + r;
            double th0 = std::acos(ct0), th1 = std::acos(ct1);
            double f0 = x * std::sin(th0) - y * std::sin(2.0 * th0), f1 = x * std::sin(th1) - y * std::sin(2.0 * th1);
            double d0 = -x * std::sin(th0) + 4.0 * y * std::sin(2.0 * th0);
            double d1 = -x * std::sin(th1) + 4.0 * y * std::sin(2.0 * th1);
            double p0 = FRAC_PI_4 * signum(d0), p1 = FRAC_PI_4 * signum(d1);
            return std::cos(f0 - n * th0 + p0) * std::sqrt(2.0 / (PI * std::fabs(d0))) +
                   std::cos(f1 - n * th1 + p1) * std::sqrt(2.0 / (PI * std::fabs(d1)));
        }
    }

    // double_bessel.rs:396-410
    bool use_saddle_point(double x, double y) const {
        if (n <= 10) return false;
        double ne = n * (1.0 - std::sqrt(10.0 / n));
        double xc = y > ne / 6.0 ? 4.0 * std::sqrt(y * (ne - 2.0 * y)) : ne + 2.0 * y;
        return x < xc;
    }

    // double_bessel.rs:386-392
    void evaluate(double x, double y, double j[5]) {
        if (use_saddle_point(x, y)) {
            for (int q = 0; q < 5; ++q) j[q] = j_spa(n - 2 + q, x, y);
        } else {
            around(x, y, j);
        }
    }
};

double double_bessel_at(int n, double x_max, double y_max, double x, double y) {
    DoubleBessel dj(n, x_max, y_max);
    double j[5];
    dj.around(x, y, j);
    return j[2];
}

double double_bessel_spa(int n, double x, double y) { return DoubleBessel::j_spa(n, x, y); }

double lp_ceiling_at(int n, double a, double eta) {
    DoubleBessel dj(n, n * SQRT_2, n * 0.5);
    return lp_ceiling(a, eta, dj);
}

double double_bessel_evaluate(int n, double x, double y) {
    DoubleBessel dj(n, n * SQRT_2, n * 0.5);
    double j[5];
    dj.evaluate(x, y, j);
    return j[2];
}

// ------------------------------------------------- LP LMA emission ------
// nonlinear_compton/lp/mod.rs:21-50
static double lp_ddpr(double a, double eta, double s, double theta, DoubleBessel& dj) {
    int n = dj.n;
    double sn = 2.0 * n * eta / (1.0 + 0.5 * a * a);
    double wn = std::min(s / (sn * (1.0 - s)), 1.0);
    double alpha = 2.0 * n * a * std::cos(theta) * std::sqrt(wn * (1.0 - wn)) / std::sqrt(1.0 + 0.5 * a * a);
    double beta = a * a * s / (8.0 * eta * (1.0 - s));
    double j[5];
    dj.evaluate(alpha, beta, j);
    double g0, g1, g2;
    if (n % 2 == 0) {
        g0 = j[2], g1 = -0.5 * (j[1] + j[3]), g2 = 0.25 * (j[0] + 2.0 * j[2] + j[4]);
    } else {
        g0 = -j[2], g1 = 0.5 * (j[1] + j[3]), g2 = -0.25 * (j[0] + 2.0 * j[2] + j[4]);
    }
    return (-g0 * g0 - a * a * (1.0 + 0.5 * s * s / (1.0 - s)) * (g0 * g2 - g1 * g1)) / (2.0 * PI);
}

// nonlinear_compton/lp/mod.rs:338-344
int lp_sum_limit(double a, double eta) {
    double m = 3.0 - 0.4 * std::pow(eta, 0.25);
    double n_max = 6.0 * (1.0 + a * a) + 2.0 * std::pow(a, m);
    return (int)std::ceil(n_max);
}

// nonlinear_compton/lp/mod.rs:53-140
static double lp_ceiling(double a, double eta, DoubleBessel& dj) {
    int n = dj.n;
    double sn = 2.0 * n * eta / (1.0 + 0.5 * a * a);
    double smax = sn / (1.0 + sn);
    double mx = -HUGE_VAL;
    if (n == 1) {
        mx = std::max(lp_ddpr(a, eta, 0.01 * smax, FRAC_PI_2, dj), lp_ddpr(a, eta, 0.99 * smax, FRAC_PI_2, dj));
    } else if (a <= 2.0) {
        for (int i = 1; i <= 32; ++i) mx = std::max(mx, lp_ddpr(a, eta, smax * (0.4 + 0.6 * i / 32.0), 0.0, dj));
    } else if (a <= 5.0) {
        int n_switch = (int)std::ceil(1.3 * std::pow(a, 1.2));
        if (n < n_switch) {
            double theta = FRAC_PI_2 * (1.0 - std::log((double)n) / std::log((double)n_switch));
            for (int i = 0; i <= 32; ++i) mx = std::max(mx, lp_ddpr(a, eta, smax * i / 32.0, theta, dj));
        } else {
            double x_min = std::max(4.0 * n * eta / (3.0 * a * a + 4.0 * n * eta), 0.4);
            int n_max = lp_sum_limit(a, eta);
            int cnt = n < n_max / 2 ? 32 : 64;
            for (int i = 1; i <= cnt; ++i) mx = std::max(mx, lp_ddpr(a, eta, smax * (x_min + (1.0 - x_min) * i / cnt), 0.0, dj));
        }
    } else {
        int n_switch = (int)std::ceil(a * a);
        if (n < n_switch) {
            double nn = n, ns = n_switch;
            double theta = FRAC_PI_2 * (std::pow(nn, -0.7) - std::pow(ns, -0.7)) / (1.0 - std::pow(ns, -0.7));
            for (int i = 1; i <= 64; ++i) mx = std::max(mx, lp_ddpr(a, eta, smax * (0.3 + 0.7 * i / 64.0), theta, dj));
        } else {
            double x_min = std::max(4.0 * n * eta / (3.0 * a * a + 4.0 * n * eta), 0.3);
            double x_peak = (1.0 + sn) / (2.0 + sn);
            int len = n > 10 * n_switch ? 64 : (n > 3 * n_switch ? 42 : 32);
            for (int i = 1; i <= len; ++i)
                mx = std::max(mx, lp_ddpr(a, eta, smax * (x_min + (x_peak - x_min) * i / len), 0.0, dj));
        }
    }
    return 1.15 * mx;
}

// nonlinear_compton/lp/mod.rs:142-302
struct ThetaBound {
    double s[16], f[16];

    static double ln_double_bessel_x_zero(int ni, double y) {
        double n = ni;
        double z = std::sqrt(n / (4.0 * y) - 0.5);
        const Cx I{0.0, 1.0};
        Cx theta{FRAC_PI_2, std::log(std::sqrt(1.0 + z * z) - z)};
        Cx s2 = cx_sin(cx_scale(2.0, theta));
        Cx f = cx_mul(I, cx_sub(cx_scale(-n, theta), cx_scale(y, s2)));
        Cx f2 = cx_mul(I, cx_scale(4.0 * y, s2));
        double e = 0.5 * (PI - cx_arg(f2));
        Cx phase = cx_add(f, cx_mul(I, Cx{e, 0.0}));
        return std::log(std::sqrt(2.0 / (PI * cx_norm(f2)))) + phase.re + std::log(std::fabs(std::cos(phase.im)));
    }

    static ThetaBound for_harmonic(int n, double a, double eta) {
        ThetaBound tb;
        double sn = 2.0 * n * eta / (1.0 + 0.5 * a * a);
        for (int i = 0; i < 16; ++i) {
            double z = std::cos(PI * i / 15.0);
            tb.s[i] = 0.5 * (z + 1.0) * sn / (1.0 + sn);
            double wn = std::min(tb.s[i] / (sn * (1.0 - tb.s[i])), 1.0);
            double x = 2.0 * n * a * std::sqrt(wn * (1.0 - wn)) / std::sqrt(1.0 + 0.5 * a * a);
            double y = a * a * tb.s[i] / (8.0 * eta * (1.0 - tb.s[i]));
            double x_crit = y > n / 6.0 ? 4.0 * std::sqrt(y) * std::sqrt(n - 2.0 * y) : n + 2.0 * y;
            double ln_j_crit = std::log(0.443) - std::log((double)n) / 3.0;
            double ln_j_bdy = (n % 2 == 0) ? ln_double_bessel_x_zero(n, y) : ln_double_bessel_x_zero(n + 1, y);
            ln_j_bdy = std::fmin(ln_j_bdy, ln_j_crit);
            double ct = 1.0 - x_crit * std::log(0.01) / (x * (ln_j_bdy - ln_j_crit));
            ct = std::fmax(ct, -1.0);
            tb.f[i] = std::acos(ct);
            if (std::isnan(tb.f[i])) tb.f[i] = PI;
        }
        double f_min = tb.f[0];
        for (int i = 1; i < 16; ++i) {
            if (tb.f[i] < f_min)
                f_min = tb.f[i];
            else
                tb.f[i] = f_min;
        }
        return tb;
    }

    // nonlinear_compton/lp/mod.rs:209-268: the bound at fixed v = s / s_max
    static ThetaBound for_harmonic_low_eta(int n, double a) {
        ThetaBound tb;
        for (int i = 0; i < 16; ++i) {
            double z = std::cos(PI * i / 15.0);
            double v = 0.5 * (z + 1.0);
            tb.s[i] = v;
            double x = 2.0 * n * a * std::sqrt(v * (1.0 - v) / (1.0 + 0.5 * a * a));
            double y = 0.25 * n * a * a * v / (1.0 + 0.5 * a * a);
            double x_crit = y > n / 6.0 ? 4.0 * std::sqrt(y) * std::sqrt(n - 2.0 * y) : n + 2.0 * y;
            double ln_j_crit = std::log(0.443) - std::log((double)n) / 3.0;
            double ln_j_bdy = std::fmin(ln_double_bessel_x_zero(n % 2 == 0 ? n : n + 1, y), ln_j_crit);
            double ct = std::fmax(1.0 - x_crit * std::log(0.01) / (x * (ln_j_bdy - ln_j_crit)), -1.0);
            tb.f[i] = std::acos(ct);
            if (std::isnan(tb.f[i])) tb.f[i] = PI;
        }
        double f_min = tb.f[0];
        for (int i = 1; i < 16; ++i) {
            if (tb.f[i] < f_min)
                f_min = tb.f[i];
            else
                tb.f[i] = f_min;
        }
        return tb;
    }

    double at(double arg) const {
        double val = f[15];
        for (int i = 1; i < 16; ++i) {
            if (arg > s[i]) {
                double w = (arg - s[i - 1]) / (s[i] - s[i - 1]);
                val = w * f[i] + (1.0 - w) * f[i - 1];
                break;
            }
        }
        return std::fmin(val, FRAC_PI_2);
    }
};

// nonlinear_compton/lp/mod.rs:306-400
static void lp_single_diff(double a, double eta, double s, double theta_max, DoubleBessel& dj, double* integral, double* mx) {
    double sum = 0.0, m = 0.0;
    for (int k = 0; k < 32; ++k) {
        double theta = 0.5 * (PTG_GAUSS_32_NODES[k] + 1.0) * theta_max;
        double rate = lp_ddpr(a, eta, s, theta, dj);
        sum += 4.0 * (0.5 * theta_max) * PTG_GAUSS_32_WEIGHTS[k] * rate;
        m = std::max(m, rate);
    }
    *integral = sum;
    *mx = m;
}

void lp_partial_rate(int n, double a, double eta, double* integral, double* mx) {
    double sn = 2.0 * n * eta / (1.0 + 0.5 * a * a);
    double smax = sn / (1.0 + sn);
    double s_peak = sn / (2.0 + sn);
    DoubleBessel dj(n, n * SQRT_2, n * 0.5);
    ThetaBound tb = ThetaBound::for_harmonic(n, a, eta);
    auto seg = [&](const double* nodes, const double* weights, int nn, double s0, double s1, double* I, double* M) {
        double acc = 0.0, m = 0.0;
        for (int k = 0; k < nn; ++k) {
            double s = s0 + 0.5 * (s1 - s0) * (nodes[k] + 1.0);
            double r, mm;
            lp_single_diff(a, eta, s, tb.at(s), dj, &r, &mm);
            acc += weights[k] * 0.5 * (s1 - s0) * r;
            m = std::max(m, mm);
        }
        *I = acc;
        *M = m;
    };
    if (sn < 1.0) {
        double l, lm, u, um;
        seg(PTG_GAUSS_32_NODES, PTG_GAUSS_32_WEIGHTS, 32, 0.0, s_peak, &l, &lm);
        seg(PTG_GAUSS_32_NODES, PTG_GAUSS_32_WEIGHTS, 32, s_peak, smax, &u, &um);
        *integral = u + l;
        *mx = std::max(um, lm);
    } else {
        double l, lm, md, mm, u, um;
        seg(PTG_GAUSS_16_NODES, PTG_GAUSS_16_WEIGHTS, 16, 0.0, smax - 2.0 * (smax - s_peak), &l, &lm);
        seg(PTG_GAUSS_32_NODES, PTG_GAUSS_32_WEIGHTS, 32, smax - 2.0 * (smax - s_peak), s_peak, &md, &mm);
        seg(PTG_GAUSS_32_NODES, PTG_GAUSS_32_WEIGHTS, 32, s_peak, smax, &u, &um);
        *integral = l + md + u;
        *mx = std::max(lm, std::max(mm, um));
    }
}

// nonlinear_compton/lp/classical.rs:189-210
bool lp_classical_rate(double a, double eta, double* out) {
    double x = std::log(a);
    if (x < PTG_NLC_CL_MIN) {
        *out = a * a * eta / 3.0;
        return true;
    }
    int ix = (int)((x - PTG_NLC_CL_MIN) / PTG_NLC_CL_STEP);
    if (ix >= 60) return false;
    double dx = (x - PTG_NLC_CL_MIN) / PTG_NLC_CL_STEP - ix;
    double f = (1.0 - dx) * g_lma.nlc_lp_cl_rate[ix] + dx * g_lma.nlc_lp_cl_rate[ix + 1];
    double prefactor = 2.0 * eta / (1.0 + 0.5 * a * a);
    *out = prefactor * std::exp(f);
    return true;
}

// nonlinear_compton/lp/mod.rs:399-463
bool lp_rate(double a, double eta, double* out) {
    const double MIN0 = PTG_NLC_LP_MIN_0, MIN1 = PTG_NLC_LP_MIN_1, S0 = PTG_NLC_LP_STEP_0, S1 = PTG_NLC_LP_STEP_1;
    const double* T = g_lma.nlc_lp_rate;
    double x = std::log(a), y = std::log(eta);
    if (x < MIN0) {
        *out = lp_linear_rate(a, eta);
        return true;
    }
    int ix = (int)((x - MIN0) / S0);
    double dx = (x - MIN0) / S0 - ix;
    if (ix >= 60) return false;
    if (y < MIN1) {
        double f = (1.0 - dx) * T[ix] + dx * T[ix + 1];
        *out = std::exp(f - MIN1) * eta;
        return true;
    }
    int iy = (int)((y - MIN1) / S1);
    if (ix < 61 - 1 && iy < 68 - 1) {
        double dy = (y - MIN1) / S1 - iy;
        double f = (1.0 - dx) * (1.0 - dy) * T[iy * 61 + ix] + dx * (1.0 - dy) * T[iy * 61 + ix + 1] +
                   (1.0 - dx) * dy * T[(iy + 1) * 61 + ix] + dx * dy * T[(iy + 1) * 61 + ix + 1];
        *out = std::exp(f);
        return true;
    }
    return false;
}

// nonlinear_compton/lp/mod.rs:465-553
static double lp_cdf_corner(const double* table, double frac, double a) {
    if (frac <= table[1]) return 0.9;
    bool ok;
    if (a < 5.0) {
        // the reference unwraps this inversion (a panic beyond the last node)
        double n = Pwmci(table, 16).invert(frac, &ok);
        return ok ? n : NAN;
    }
    double rs[30];
    for (int i = 0; i < 15; ++i) {
        rs[2 * i] = std::log(table[2 * i]);
        rs[2 * i + 1] = std::log(-1.0 * std::log(1.0 - table[2 * i + 1]));
    }
    double f2 = std::log(-1.0 * std::log(1.0 - frac));
    return std::exp(Pwmci(rs, 15, true).invert(f2, &ok));
}

int lp_harmonic_index(double a, double eta, double frac) {
    const double MIN0 = PTG_NLC_LP_CDF_MIN_0, MIN1 = PTG_NLC_LP_CDF_MIN_1, S0 = PTG_NLC_LP_CDF_STEP_0, S1 = PTG_NLC_LP_CDF_STEP_1;
    const double* T = g_lma.nlc_lp_cdf;
    if (std::log(a) <= MIN0) return 1;
    int ix = (int)((std::log(a) - MIN0) / S0);
    double dx = (std::log(a) - MIN0) / S0 - ix;
    if (ix >= 60) return -1;
    if (std::log(eta) <= MIN1) {
        double n = lp_cdf_corner(T + (size_t)ix * 32, frac, a) * (1.0 - dx) + lp_cdf_corner(T + (size_t)(ix + 1) * 32, frac, a) * dx;
        return std::isfinite(n) ? (int)std::ceil(n) : -1;
    }
    int iy = (int)((std::log(eta) - MIN1) / S1);
    if (61 * (iy + 1) + ix + 1 >= 4148) return -1;
    double dy = (std::log(eta) - MIN1) / S1 - iy;
    int idx[4] = {61 * iy + ix, 61 * iy + ix + 1, 61 * (iy + 1) + ix, 61 * (iy + 1) + ix + 1};
    double w[4] = {(1.0 - dx) * (1.0 - dy), dx * (1.0 - dy), (1.0 - dx) * dy, dx * dy};
    double n = 0.0;
    for (int k = 0; k < 4; ++k) n += lp_cdf_corner(T + (size_t)idx[k] * 32, frac, a) * w[k];
    return std::isfinite(n) ? (int)std::ceil(n) : -1;
}

// nonlinear_compton/lp/mod.rs:586-676
int lp_sample(double a, double eta, DrawStream& rng, int* n_out, double* s_out, double* theta_out, Stokes* sv_out,
              uint64_t* rej) {
    int n = lp_harmonic_index(a, eta, rng.next());
    if (n < 1) return PTG_ERR_OUT_OF_TABLE;
    DoubleBessel dj(n, n * SQRT_2, n * 0.5);
    ThetaBound tb = ThetaBound::for_harmonic(n, a, eta);
    double sn = 2.0 * n * eta / (1.0 + 0.5 * a * a);
    double smax = sn / (1.0 + sn);
    double mx = lp_ceiling(a, eta, dj);
    double s = 0.0, theta = 0.0;
    int it;
    for (it = 0; it < REJECTION_CAP; ++it) {
        double ss = smax * rng.next();
        double th = FRAC_PI_2 * rng.next();
        if (th > tb.at(ss)) continue;
        double z = mx * rng.next();
        if (z < lp_ddpr(a, eta, ss, th, dj)) {
            s = ss, theta = th;
            break;
        }
    }
    *rej += it;
    if (it == REJECTION_CAP) return PTG_ERR_REJECTION_CAP;
    int quadrant = (int)(4.0 * rng.next());  // gen_range(0, 4)
    if (quadrant == 1)
        theta = PI - theta;
    else if (quadrant == 2)
        theta = PI + theta;
    else if (quadrant == 3)
        theta = 2.0 * PI - theta;
    double wn = std::min(s / (sn * (1.0 - s)), 1.0);
    double x = -2.0 * n * a * std::cos(theta) * std::sqrt(wn * (1.0 - wn)) / std::sqrt(1.0 + 0.5 * a * a);
    double y = a * a * s / (8.0 * eta * (1.0 - s));
    double j[5];
    dj.evaluate(std::fabs(x), y, j);
    double A0, A1, A2;
    if (x > 0.0) {
        A0 = j[2], A1 = 0.5 * (j[1] + j[3]), A2 = 0.25 * (j[0] + 2.0 * j[2] + j[4]);
    } else if (n % 2 == 0) {
        A0 = j[2], A1 = -0.5 * (j[1] + j[3]), A2 = 0.25 * (j[0] + 2.0 * j[2] + j[4]);
    } else {
        A0 = -j[2], A1 = 0.5 * (j[1] + j[3]), A2 = -0.25 * (j[0] + 2.0 * j[2] + j[4]);
    }
    double u = std::sqrt(2.0 * n * eta * (1.0 - s) / s - (1.0 + 0.5 * a * a));
    double xi0 = (1.0 - s + 1.0 / (1.0 - s)) * (powi(A1, 2) - A0 * A2) - 2.0 * powi(A0 / a, 2);
    double xi1 = 2.0 * (powi(A1, 2) - A0 * A2) - 2.0 * (1.0 + 2.0 * u * u * powi(std::sin(theta), 2)) * powi(A0 / a, 2);
    double xi2 = -1.0 * (2.0 * powi(u * A0 / a, 2) * std::sin(2.0 * theta) + 4.0 * u * A0 * A1 * std::sin(theta) / a);
    *sv_out = Stokes(1.0, xi1 / xi0, xi2 / xi0, 0.0);
    *n_out = n;
    *s_out = s;
    *theta_out = theta;
    return PTG_OK;
}

// ------------------------------------------------- LMA NLC dispatch ----

// ------------------------------------------------ classical LMA emission --
// nonlinear_compton/cp/classical.rs:45-175
static double cp_cl_ceiling(int n, double a) {
    double n_switch = std::round(3.0 * (1.0 + 0.54 * std::pow(a, 2.75)));
    double mx;
    if (n == 1) {
        mx = cp_spectrum_low_eta(n, a, 0.99);
    } else if (a < 0.15 || n > (int)n_switch) {
        mx = cp_spectrum_low_eta(n, a, 0.5);
    } else {
        double b = a < 0.5 ? 2.3 * a : 0.8 * std::exp(-(a - 0.5) / 3.5) + 0.35;
        double v = 1.0 - 0.5 * std::pow(std::log((double)n), b) / std::pow(std::log(n_switch), b);
        mx = NAN;
        for (int i = -4; i < 4; ++i) {
            double f = cp_spectrum_low_eta(n, a, std::fmin(v + 0.1 * (double)i / 4.0, 1.0));
            mx = std::isnan(mx) ? f : (std::isnan(f) ? mx : std::max(mx, f));
        }
    }
    return 1.1 * mx;
}

// cdf_table: [61][32][2] over ln a, two-point interpolation, inversion in
// [ln n, ln(-ln(1 - cdf))]; -1 if the lookup fails
static int cp_cl_harmonic_index(double a, double frac) {
    const double* T = g_lma.nlc_cp_cl_cdf;
    if (std::log(a) <= PTG_NLC_CL_MIN) return 1;
    int ix = (int)((std::log(a) - PTG_NLC_CL_MIN) / PTG_NLC_CL_STEP);
    double dx = (std::log(a) - PTG_NLC_CL_MIN) / PTG_NLC_CL_STEP - ix;
    if (ix >= 60) return -1;
    double n = 0.0;
    for (int k = 0; k < 2; ++k) {
        const double* tb = T + (size_t)(ix + k) * 64;
        double w = k == 0 ? 1.0 - dx : dx;
        double nk;
        if (frac <= tb[1]) {
            nk = 0.9;
        } else {
            double rs[62];
            for (int i = 0; i < 31; ++i) {
                rs[2 * i] = std::log(tb[2 * i]);
                rs[2 * i + 1] = std::log(-1.0 * std::log(1.0 - tb[2 * i + 1]));
            }
            bool ok;
            nk = std::exp(Pwmci(rs, 31, true).invert(std::log(-1.0 * std::log(1.0 - frac)), &ok));
        }
        n += nk * w;
    }
    return std::isfinite(n) ? rust_as_i32(std::ceil(n)) : -1;
}

int cp_classical_sample(double a, double eta, DrawStream& rng, int* n_out, double* s_out, double* theta_out,
                        Stokes* sv_out, uint64_t* rej) {
    int n = cp_cl_harmonic_index(a, rng.next());
    if (n < 1) return PTG_ERR_OUT_OF_TABLE;
    double mx = cp_cl_ceiling(n, a);
    double v = 0.0;
    int it;
    for (it = 0; it < REJECTION_CAP; ++it) {
        double vv = rng.next(), u = rng.next();
        if (u <= cp_spectrum_low_eta(n, a, vv) / mx) {
            v = vv;
            break;
        }
    }
    *rej += it;
    if (it == REJECTION_CAP) return PTG_ERR_REJECTION_CAP;
    double sn = 2.0 * n * eta / (1.0 + a * a);
    double s = v * sn;
    double theta = 2.0 * PI * rng.next();
    double z = std::sqrt((double)(4 * n * n) * (a * a / (1.0 + a * a)) * v * (1.0 - v));
    double jm, j, jp;
    bessel_j_pm(z, n, &jm, &j, &jp);
    double xi0 = 2.0 * (jm * jm + jp * jp - 2.0 * j * j) - powi(2.0 * j / a, 2);
    double xi1 = 2.0 * (jm * jm + jp * jp - 2.0 * j * j) + 8.0 * j * j * (1.0 - powi((double)n / z, 2) - 0.5 / (a * a));
    double xi3 = 2.0 * (1.0 - 2.0 * v) * (jm * jm - jp * jp);
    Stokes sv(1.0, xi1 / xi0, 0.0 / xi0, xi3 / xi0);
    *sv_out = sv.rotate_by(FRAC_PI_2 + theta);
    *n_out = n;
    *s_out = s;
    *theta_out = theta;
    return PTG_OK;
}

// nonlinear_compton/lp/classical.rs:19-120
static double lp_cl_ddpr(double a, double v, double theta, DoubleBessel& dj) {
    int n = dj.n;
    double x = 2.0 * n * a * std::cos(theta) * std::sqrt(v * (1.0 - v) / (1.0 + 0.5 * a * a));
    double y = 0.25 * n * a * a * v / (1.0 + 0.5 * a * a);
    double j[5];
    dj.evaluate(x, y, j);
    double g0, g1, g2;
    if (n % 2 == 0) {
        g0 = j[2], g1 = -0.5 * (j[1] + j[3]), g2 = 0.25 * (j[0] + 2.0 * j[2] + j[4]);
    } else {
        g0 = -j[2], g1 = 0.5 * (j[1] + j[3]), g2 = -0.25 * (j[0] + 2.0 * j[2] + j[4]);
    }
    return (-g0 * g0 - a * a * (g0 * g2 - g1 * g1)) / (2.0 * PI);
}

static double lp_cl_ceiling(double a, DoubleBessel& dj) {
    int n = dj.n;
    double mx = NAN;
    auto upd = [&](double f) { mx = std::isnan(mx) ? f : (std::isnan(f) ? mx : std::max(mx, f)); };
    if (n == 1) {
        upd(lp_cl_ddpr(a, 0.01, FRAC_PI_2, dj));
    } else if (a <= 1.5) {
        double v_min = 0.1 + (9.0 / std::sqrt((double)n) - 1.0) / 10.0;
        double v_max = std::fmin(v_min + 0.4, 1.0);
        for (int i = 1; i <= 16; ++i) upd(lp_cl_ddpr(a, v_min + (v_max - v_min) * (double)i / 16.0, 0.0, dj));
    } else if (a < 5.0) {
        int n_switch = rust_as_i32(3.0 * std::pow(a / 2.0, 4.0 / 3.0));
        double theta = n > n_switch ? 0.0 : FRAC_PI_2 * (1.0 - std::log((double)n) / std::log((double)n_switch));
        double v_min = std::fmin(0.35 + (7.0 / std::sqrt((double)n) - 1.0) / 9.0, 0.55);
        double v_max = 0.55 + (7.0 / std::sqrt((double)n) - 1.0) / 9.0;
        int num = a > 4.0 ? 32 : 16;
        for (int i = 0; i < num; ++i) upd(lp_cl_ddpr(a, v_min + (v_max - v_min) * (double)i / num, theta, dj));
    } else {
        double n_switch = 10.0 * powi(a / 5.0, 2);
        double theta = 0.0;
        if (!(n > rust_as_i32(n_switch))) {
            double pw = 0.3 + (0.7 - 0.3) * (std::log(a) - std::log(5.0)) / (std::log(20.0) - std::log(5.0));
            theta = FRAC_PI_2 * (std::pow((double)n, -pw) - std::pow(n_switch, -pw)) / (1.0 - std::pow(n_switch, -pw));
        }
        double v_min = 0.3 + 0.4 * std::log((double)n) * std::pow((double)n, -0.7);
        double v_max = v_min + 0.2;
        int num = a > 8.0 ? 64 : 32;
        for (int i = 0; i < num; ++i) upd(lp_cl_ddpr(a, v_min + (v_max - v_min) * (double)i / num, theta, dj));
    }
    return 1.1 * mx;
}

static int lp_cl_harmonic_index(double a, double frac) {
    const double* T = g_lma.nlc_lp_cl_cdf;
    if (std::log(a) <= PTG_NLC_CL_MIN) return 1;
    int ix = (int)((std::log(a) - PTG_NLC_CL_MIN) / PTG_NLC_CL_STEP);
    double dx = (std::log(a) - PTG_NLC_CL_MIN) / PTG_NLC_CL_STEP - ix;
    if (ix >= 60) return -1;
    double n = 0.0;
    for (int k = 0; k < 2; ++k) {
        const double* tb = T + (size_t)(ix + k) * 32;
        double w = k == 0 ? 1.0 - dx : dx;
        double nk = 0.9;
        if (!(frac <= tb[1])) {
            bool ok;
            nk = Pwmci(tb, 16).invert(frac, &ok);
            if (!ok) return -1;  // the reference unwraps this inversion
        }
        n += nk * w;
    }
    return std::isfinite(n) ? rust_as_i32(std::ceil(n)) : -1;
}


// nonlinear_compton/cp/mod.rs:137-153
double cp_cl_integrated(int n, double a) {
    double lower = 0.0, upper = 0.0;
    for (int k = 0; k < 32; ++k) lower += 0.25 * PTG_GAUSS_32_WEIGHTS[k] * cp_spectrum_low_eta(n, a, 0.25 * (PTG_GAUSS_32_NODES[k] + 1.0));
    for (int k = 0; k < 32; ++k) upper += 0.25 * PTG_GAUSS_32_WEIGHTS[k] * cp_spectrum_low_eta(n, a, 0.25 * (PTG_GAUSS_32_NODES[k] + 3.0));
    return lower + upper;
}

// nonlinear_compton/lp/classical.rs:113-180 (integral over v and theta)
double lp_cl_partial_rate(int n, double a) {
    DoubleBessel dj(n, n * SQRT_2, n * 0.5);
    ThetaBound tb = ThetaBound::for_harmonic_low_eta(n, a);
    auto single = [&](double v, double tmax) {
        double acc = 0.0;
        for (int k = 0; k < 32; ++k) {
            double th = 0.5 * (PTG_GAUSS_32_NODES[k] + 1.0) * tmax;
            acc += 4.0 * (0.5 * tmax) * PTG_GAUSS_32_WEIGHTS[k] * lp_cl_ddpr(a, v, th, dj);
        }
        return acc;
    };
    double lower = 0.0, middle = 0.0, upper = 0.0;
    for (int k = 0; k < 32; ++k) {
        double v = 0.5 * (PTG_GAUSS_32_NODES[k] + 1.0) * 0.5;
        lower += PTG_GAUSS_32_WEIGHTS[k] * (0.5 * 0.5) * single(v, tb.at(v));
    }
    for (int k = 0; k < 32; ++k) {
        double v = 0.5 + 0.5 * (PTG_GAUSS_32_NODES[k] + 1.0) * 0.25;
        middle += PTG_GAUSS_32_WEIGHTS[k] * (0.5 * 0.25) * single(v, tb.at(v));
    }
    for (int k = 0; k < 32; ++k) {
        double v = 0.75 + 0.5 * (PTG_GAUSS_32_NODES[k] + 1.0) * 0.25;
        upper += PTG_GAUSS_32_WEIGHTS[k] * (0.5 * 0.25) * single(v, tb.at(v));
    }
    return lower + middle + upper;
}

int lp_classical_sample(double a, double eta, DrawStream& rng, int* n_out, double* s_out, double* theta_out,
                        Stokes* sv_out, uint64_t* rej) {
    int n = lp_cl_harmonic_index(a, rng.next());
    if (n < 1) return PTG_ERR_OUT_OF_TABLE;
    DoubleBessel dj(n, n * SQRT_2, n * 0.5);
    ThetaBound tb = ThetaBound::for_harmonic_low_eta(n, a);
    double smax = 2.0 * n * eta / (1.0 + 0.5 * a * a);
    double mx = lp_cl_ceiling(a, dj);
    double v = 0.0, s = 0.0, theta = 0.0;
    int it;
    for (it = 0; it < REJECTION_CAP; ++it) {
        double vv = rng.next();
        double ss = vv * smax;
        double th = FRAC_PI_2 * rng.next();
        if (th > tb.at(vv)) continue;
        double z = mx * rng.next();
        if (z < lp_cl_ddpr(a, vv, th, dj)) {
            v = vv, s = ss, theta = th;
            break;
        }
    }
    *rej += it;
    if (it == REJECTION_CAP) return PTG_ERR_REJECTION_CAP;
    int quadrant = (int)(4.0 * rng.next());
    if (quadrant == 1)
        theta = PI - theta;
    else if (quadrant == 2)
        theta = PI + theta;
    else if (quadrant == 3)
        theta = 2.0 * PI - theta;
    double x = 2.0 * n * a * std::cos(theta) * std::sqrt(v * (1.0 - v) / (1.0 + 0.5 * a * a));
    double y = 0.25 * n * a * a * v / (1.0 + 0.5 * a * a);
    double j[5];
    dj.evaluate(x, y, j);
    double A0, A1, A2;
    if (n % 2 == 0) {
        A0 = j[2], A1 = -0.5 * (j[1] + j[3]), A2 = 0.25 * (j[0] + 2.0 * j[2] + j[4]);
    } else {
        A0 = -j[2], A1 = 0.5 * (j[1] + j[3]), A2 = -0.25 * (j[0] + 2.0 * j[2] + j[4]);
    }
    double u = std::sqrt((1.0 + 0.5 * a * a) * (1.0 - v) / v);
    double xi0 = 2.0 * (powi(A1, 2) - A0 * A2) - 2.0 * powi(A0 / a, 2);
    double xi1 = 2.0 * (powi(A1, 2) - A0 * A2) - 2.0 * (1.0 + 2.0 * u * u * powi(std::sin(theta), 2)) * powi(A0 / a, 2);
    double xi2 = 2.0 * powi(u * A0 / a, 2) * std::sin(2.0 * theta) + 4.0 * u * A0 * A1 * std::sin(theta) / a;
    *sv_out = Stokes(1.0, xi1 / xi0, xi2 / xi0, 0.0);
    *n_out = n;
    *s_out = s;
    *theta_out = theta;
    return PTG_OK;
}


// nonlinear_compton/mod.rs:19-47
bool nlc_probability(const V4& k, const V4& q, double dt, int pol, bool classical, double* p) {
    double a_sqd = q * q - 1.0;
    double a = a_sqd >= 0.0 ? std::sqrt(a_sqd) : 0.0;
    double eta = k * q;
    double dphi = dt * eta / (COMPTON_TIME * q.t);
    double f;
    bool ok;
    if (pol == PTG_POL_CIRCULAR) {
        ok = classical ? cp_classical_rate(a, eta, &f) : cp_rate(a, eta, &f);
    } else {
        ok = classical ? lp_classical_rate(a * SQRT_2, eta, &f) : lp_rate(a * SQRT_2, eta, &f);
    }
    if (!ok) return false;
    *p = ALPHA_FINE * f * dphi / eta;
    return true;
}

// nonlinear_compton/mod.rs:58-138
int nlc_generate(const V4& k, const V4& q, int pol, double pol_angle, bool classical, DrawStream& rng, int* n_out,
                 V4* k_out, Stokes* sv_out, uint64_t* rej) {
    double a = std::sqrt(q * q - 1.0);
    double eta = k * q;
    int n;
    double s, cphi;
    Stokes sv;
    int st;
    if (pol == PTG_POL_CIRCULAR)
        st = classical ? cp_classical_sample(a, eta, rng, &n, &s, &cphi, &sv, rej)
                       : cp_sample(a, eta, rng, &n, &s, &cphi, &sv, rej);
    else
        st = classical ? lp_classical_sample(a * SQRT_2, eta, rng, &n, &s, &cphi, &sv, rej)
                       : lp_sample(a * SQRT_2, eta, rng, &n, &s, &cphi, &sv, rej);
    if (st != PTG_OK) return st;
    double ell = n;
    double p_zmf = classical ? ell * eta / std::sqrt(1.0 + a * a) : ell * eta / std::sqrt(1.0 + a * a + 2.0 * ell * eta);
    double ct = classical ? 1.0 - s * (1.0 + a * a) / (ell * eta) : 1.0 - s * (1.0 + a * a + 2.0 * ell * eta) / (ell * eta);
    if (!(ct <= 1.0 && ct >= -1.0)) return PTG_ERR_SANITY;
    V4 u_zmf;
    if (classical) {
        u_zmf = q / std::sqrt(q.t * q.t - q.x * q.x - q.y * q.y - q.z * q.z);
    } else {
        V4 t = q + ell * k;
        u_zmf = t / std::sqrt(t * t);
    }
    V3 along = classical ? (ell * k).boost_by(u_zmf).spatial().normalize() : -(q.boost_by(u_zmf).spatial().normalize());
    V4 eps4(0.0, std::cos(pol_angle), std::sin(pol_angle), 0.0);
    V3 eps = eps4.boost_by(u_zmf).spatial().normalize();
    eps = along.cross(eps.cross(along)).normalize();
    V3 perp = eps.rotate_around(along, cphi);
    V3 kp = p_zmf * (ct * along + std::sqrt(1.0 - ct * ct) * perp);
    V4 kprime = V4::lightlike(kp.x, kp.y, kp.z);
    V4 rev(u_zmf.t, -u_zmf.x, -u_zmf.y, -u_zmf.z);
    kprime = kprime.boost_by(rev);
    sv = sv.rotate_by(-pol_angle);
    sv = sv.from_lma_basis(kprime);
    double s_new = (k * kprime) / (k * q);
    double err = std::fabs(s - s_new) / s;
    if (err >= 1.0e-2) return PTG_ERR_SANITY;
    *n_out = n;
    *k_out = kprime;
    *sv_out = sv;
    return PTG_OK;
}

double std_normal(DrawStream& rng) {
    double u1 = rng.next(), u2 = rng.next();
    return std::sqrt(-2.0 * std::log(1.0 - u1)) * std::cos(2.0 * PI * u2);
}

// plane_wave.rs:251-282, focused_laser.rs:260-281
int lma_radiate(const Laser& L, const V4& r, const V4& u, double dt, DrawStream& rng, bool classical, bool* emitted,
                RadiationEvent* ev, uint64_t* rej) {
    *emitted = false;
    double a = std::sqrt(L.a_sqd(r));
    double chirp = 1.0;
    if (L.d.model == PTG_PLANE_WAVE) {
        double phase = L.wavevector * r;
        chirp = 1.0 + 2.0 * L.d.chirp_b * phase;
        if (chirp < 0.0 && a > 0.0) return PTG_ERR_SANITY;
    }
    double width = 1.0;
    if (L.bandwidth != 0.0) {
        width = 1.0 + L.bandwidth * std_normal(rng);
        if (!(width > 0.0)) return PTG_ERR_SANITY;
    }
    V4 kappa = (SPEED_OF_LIGHT * COMPTON_TIME) * L.wavevector * chirp * width;
    double prob;
    if (!nlc_probability(kappa, u, dt, L.d.polarization, classical, &prob)) return PTG_ERR_OUT_OF_TABLE;
    if (rng.next() < prob) {
        int n;
        V4 k;
        Stokes pol;
        int st = nlc_generate(kappa, u, L.d.polarization, L.d.pol_angle, classical, rng, &n, &k, &pol, rej);
        if (st != PTG_OK) return st;
        ev->k = k;
        ev->u_prime = u + (double)n * kappa - k;
        ev->pol = pol;
        ev->a_eff = a;
        ev->chi = a * (u * kappa);
        ev->absorption = (double)n * kappa.t;
        *emitted = true;
    }
    return PTG_OK;
}

// ------------------------------------------------- CP LMA pair creation --
// pair_creation/cp/mod.rs:24-243 (DoubleDiffPartialRate) and :248-449 (TotalRate)
static const double PAIR_LASER_S3 = -1.0;

static void cpp_s_bounds(int n, double a, double eta, double* s_min, double* s_max) {
    double sn = 2.0 * n * eta / (1.0 + powi(a, 2));
    double smin = 0.5 * (1.0 - std::sqrt(1.0 - 4.0 / sn));
    *s_min = std::min(smin, 0.5);
    *s_max = 0.5;
}

static void cpp_elements(int n, double a, double eta, double s, double* unpol, double* d12, double* d3) {
    double ell = n;
    double sn = 2.0 * ell * eta / (1.0 + powi(a, 2));
    double tmp = 1.0 / (sn * s * (1.0 - s));
    double z = std::sqrt((4.0 * ell * ell) * (powi(a, 2) / (1.0 + powi(a, 2))) * tmp * (1.0 - tmp));
    double jm, j, jp;
    bessel_j_pm(z, n, &jm, &j, &jp);
    *unpol = powi(j, 2) + 0.25 * powi(a, 2) * ((1.0 - s) / s + s / (1.0 - s)) * (powi(jm, 2) + powi(jp, 2) - 2.0 * powi(j, 2));
    *d12 = (2.0 * powi(ell * a / z, 2) - (1.0 + powi(a, 2))) * powi(j, 2) - 0.5 * powi(a, 2) * (powi(jm, 2) + powi(jp, 2));
    *d3 = 0.25 * powi(a, 2) * ((1.0 - s) / s + s / (1.0 - s)) * (1.0 - 2.0 / (sn * s * (1.0 - s))) * (powi(jm, 2) - powi(jp, 2));
}

// pair_creation/cp/mod.rs:66-72.  (2 theta).sin_cos() returns (sin, cos):
// the reference binds them to (cos_2theta, sin_2theta) in that order.
static double cpp_fully_resolved(int n, double a, double eta, double s, double theta, double sv1, double sv2, double sv3) {
    double unpol, d12, d3;
    cpp_elements(n, a, eta, s, &unpol, &d12, &d3);
    double cos_2theta = std::sin(2.0 * theta), sin_2theta = std::cos(2.0 * theta);
    return (unpol - (sv1 * cos_2theta + sv2 * sin_2theta) * d12 - PAIR_LASER_S3 * sv3 * d3) / (2.0 * PI);
}

static void cpp_over_theta(int n, double a, double eta, double s, double* re, double* im) {
    double unpol, d12, d3;
    cpp_elements(n, a, eta, s, &unpol, &d12, &d3);
    *re = unpol - PAIR_LASER_S3 * d3;
    *im = unpol + PAIR_LASER_S3 * d3;
}

static double cpp_over_theta_s3(int n, double a, double eta, double s, double sv3) {
    double re, im;
    cpp_over_theta(n, a, eta, s, &re, &im);
    return 0.5 * (re * (1.0 + sv3) + im * (1.0 - sv3));
}

// pair_creation/cp/mod.rs:92-186
void cp_pair_integrate(int n, double a, double eta, double* out_re, double* out_im) {
    double ell = n;
    double sn = 2.0 * ell * eta / (1.0 + a * a);
    *out_re = 0.0, *out_im = 0.0;
    if (sn <= 4.0) return;
    double beta = powi(a, 4) * powi(1.0 / ell + 1.0, 2) + 16.0 * powi(a * a - 2.0, 2) / (sn * sn) - 8.0 * a * a * (a * a - 2.0) / sn;
    beta = std::sqrt(beta) / (a * a - 2.0);
    double alpha = (a * a + 2.0 * ell) / (ell * (2.0 - a * a)) - 4.0 / sn;
    double tmp = alpha + beta;
    double s_peak = 0.5 * (1.0 - std::sqrt(tmp));
    double s_min, s_max;
    cpp_s_bounds(n, a, eta, &s_min, &s_max);
    auto seg = [&](double lo, double hi, double* re, double* im) {
        double r = 0.0, i = 0.0;
        for (int k = 0; k < 32; ++k) {
            double s = 0.5 * (hi - lo) * PTG_GAUSS_32_NODES[k] + 0.5 * (lo + hi);
            double sr, si;
            cpp_over_theta(n, a, eta, s, &sr, &si);
            r += 0.5 * (hi - lo) * PTG_GAUSS_32_WEIGHTS[k] * sr;
            i += 0.5 * (hi - lo) * PTG_GAUSS_32_WEIGHTS[k] * si;
        }
        *re = r, *im = i;
    };
    if (std::isfinite(s_peak)) {
        double s_mid = 2.0 * s_peak - s_min;
        if (s_mid > s_max) {
            double lr, li, ur, ui;
            seg(s_min, s_peak, &lr, &li);
            seg(s_peak, s_max, &ur, &ui);
            *out_re = 2.0 * (ur + lr), *out_im = 2.0 * (ui + li);
        } else {
            double lr, li, mr, mi, ur, ui;
            seg(s_min, s_peak, &lr, &li);
            seg(s_peak, s_mid, &mr, &mi);
            seg(s_mid, s_max, &ur, &ui);
            *out_re = 2.0 * (lr + mr + ur), *out_im = 2.0 * (li + mi + ui);
        }
    } else {
        double tr, ti;
        seg(s_min, s_max, &tr, &ti);
        *out_re = 2.0 * tr, *out_im = 2.0 * ti;
    }
}

// pair_creation/cp/mod.rs:349-365
static void cpp_sum_limits(double a, double eta, int* n_min, int* n_max) {
    double nm = std::ceil(2.0 * (1.0 + a * a) / eta);
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

static bool cpp_is_too_small(double a, double eta) {
    return std::log10(eta) < -1.0 - powi(std::log10(a) + 2.0, 2) / 4.5;
}

void cp_pair_by_summation(double a, double eta, double f[2]) {
    int n0, n1;
    cpp_sum_limits(a, eta, &n0, &n1);
    double re = 0.0, im = 0.0;
    for (int n = n0; n <= n1; ++n) {
        double r, i;
        cp_pair_integrate(n, a, eta, &r, &i);
        re += r, im += i;
    }
    f[0] = re, f[1] = im;
}

// pair_creation/cp/mod.rs:395-448; false where the reference panics
bool cp_pair_by_lookup(double a, double eta, double f[2]) {
    const double LMA = PTG_BW_CP_LN_MIN_A, LME = PTG_BW_CP_LN_MIN_ETA, SA = PTG_BW_CP_LN_A_STEP, SE = PTG_BW_CP_LN_ETA_STEP;
    const int NC = 74, NR = 121;
    const double* T = g_lma.bw_cp_total;
    double x = std::log(a), y = std::log(eta);
    if (x < LMA) return false;
    if (y < LME) {
        f[0] = f[1] = 0.0;
        return true;
    }
    int ix = (int)((x - LMA) / SA), iy = (int)((y - LME) / SE);
    if (!(ix < NC - 1 && iy < NR - 1)) return false;
    auto P = [&](int r, int c, int k) { return T[((size_t)r * NC + c) * 2 + k]; };
    if (a * eta > 2.0) {
        double dx = (x - LMA) / SA - ix, dy = (y - LME) / SE - iy;
        double w[4] = {(1.0 - dx) * (1.0 - dy), dx * (1.0 - dy), (1.0 - dx) * dy, dx * dy};
        for (int k = 0; k < 2; ++k)
            f[k] = std::exp(w[0] * P(iy, ix, k) + w[1] * P(iy, ix + 1, k) + w[2] * P(iy + 1, ix, k) + w[3] * P(iy + 1, ix + 1, k));
    } else {
        double a_min = std::exp(LMA + ix * SA), a_max = std::exp(LMA + (ix + 1) * SA);
        double e_min = std::exp(LME + iy * SE), e_max = std::exp(LME + (iy + 1) * SE);
        double dx = (a - a_min) / (a_max - a_min), dy = (eta - e_min) / (e_max - e_min);
        double w[4] = {(1.0 - dx) * (1.0 - dy), dx * (1.0 - dy), (1.0 - dx) * dy, dx * dy};
        for (int k = 0; k < 2; ++k) {
            double g = w[0] / P(iy, ix, k) + w[1] / P(iy, ix + 1, k) + w[2] / P(iy + 1, ix, k) + w[3] / P(iy + 1, ix + 1, k);
            f[k] = std::exp(1.0 / g);
        }
    }
    return true;
}

// TotalRate::probability / value dispatch (pair_creation/cp/mod.rs:265-309)
bool cp_pair_rates(double a, double eta, double f[2]) {
    if (a < 0.02 || cpp_is_too_small(a, eta)) {
        f[0] = f[1] = 0.0;
        return true;
    }
    if (a < std::exp(PTG_BW_CP_LN_MIN_A)) {
        cp_pair_by_summation(a, eta, f);
        return true;
    }
    return cp_pair_by_lookup(a, eta, f);
}

// pair_creation/cp/mod.rs:280-309
static double cpp_probability(const double f[2], double eta, const Stokes& sv, double dphi, Stokes* out) {
    double f0 = f[0], f1 = f[1];
    double prob = ALPHA_FINE * (0.5 * ((f0 + f1) + sv.v * (f0 - f1))) * dphi / eta;
    double prob_avg = ALPHA_FINE * (0.5 * (f0 + f1)) * dphi / eta;
    double delta = ALPHA_FINE * (0.5 * (f0 - f1)) * dphi / eta;
    *out = Stokes(sv.i, sv.q * (1.0 - prob_avg) / (1.0 - prob), sv.u * (1.0 - prob_avg) / (1.0 - prob),
                  (sv.v * (1.0 - prob_avg) - delta) / (1.0 - prob));
    return prob;
}

// pair_creation/cp/mod.rs:191-243
static int cpp_sample_s_theta(int n, double a, double eta, double sv1, double sv2, double sv3, DrawStream& rng,
                              double* s_out, double* theta_out, uint64_t* rej) {
    double s_min, s_max;
    cpp_s_bounds(n, a, eta, &s_min, &s_max);
    double mx = NAN;
    for (int k = 0; k < 32; ++k) {
        double s = 0.5 * (s_max - s_min) * PTG_GAUSS_32_NODES[k] + 0.5 * (s_min + s_max);
        double v = cpp_over_theta_s3(n, a, eta, s, sv3);
        mx = std::isnan(mx) ? v : (std::isnan(v) ? mx : std::max(mx, v));
    }
    mx *= 1.5;
    double s = 0.0;
    int it;
    for (it = 0; it < REJECTION_CAP; ++it) {
        double ss = s_min + (s_max - s_min) * rng.next();
        double z = mx * rng.next();
        if (z < cpp_over_theta_s3(n, a, eta, ss, sv3)) {
            s = ss;
            break;
        }
    }
    *rej += it;
    if (it == REJECTION_CAP) return PTG_ERR_REJECTION_CAP;
    if (rng.next() < 0.5) s = 1.0 - s;  // gen_range(0, 2) == 0
    double theta_opt = 0.5 * std::atan2(sv2, sv1);
    double tm = -HUGE_VAL;
    for (int i = 0; i < 4; ++i) tm = std::max(tm, cpp_fully_resolved(n, a, eta, s, theta_opt + i * FRAC_PI_2, sv1, sv2, sv3));
    tm *= 1.01;
    double theta = 0.0;
    for (it = 0; it < REJECTION_CAP; ++it) {
        double th = 2.0 * PI * rng.next();
        double z = tm * rng.next();
        if (z < cpp_fully_resolved(n, a, eta, s, th, sv1, sv2, sv3)) {
            theta = th;
            break;
        }
    }
    *rej += it;
    if (it == REJECTION_CAP) return PTG_ERR_REJECTION_CAP;
    *s_out = s;
    *theta_out = theta;
    return PTG_OK;
}

// pair_creation/cp/mod.rs:314-346: harmonic by explicit summation
static int cpp_sample(double a, double eta, double sv1, double sv2, double sv3, DrawStream& rng, int* n_out, double* s,
                      double* theta, uint64_t* rej) {
    int n0, n1;
    cpp_sum_limits(a, eta, &n0, &n1);
    double f[2];
    if (!cp_pair_rates(a, eta, f)) return PTG_ERR_OUT_OF_TABLE;
    double target = 0.5 * (f[0] * (1.0 + sv3) + f[1] * (1.0 - sv3));
    target = target * rng.next();
    double cum = 0.0;
    int index = -1;
    for (int k = n0; k <= n1; ++k) {
        double re, im;
        cp_pair_integrate(k, a, eta, &re, &im);
        cum += 0.5 * ((1.0 + sv3) * re + (1.0 - sv3) * im);
        if (cum > target) {
            index = k;
            break;
        }
    }
    if (index == -1) index = n1 - 1;
    *n_out = index;
    return cpp_sample_s_theta(index, a, eta, sv1, sv2, sv3, rng, s, theta, rej);
}


// ------------------------------------------------ LP Breit-Wheeler ----
// pair_creation/lp/**: rates from the shipped tables (main and mid-range),
// harmonic index by CDF inversion, (s, theta) by rejection.


// pair_creation/lp/tables/pol_dep.rs: a pair (S_1 = +1, S_1 = -1)
struct PolDep {
    double par, perp;
    double interp(double sv1) const { return 0.5 * ((par + perp) + sv1 * (par - perp)); }
};
static inline PolDep pd(const double* v) { return PolDep{v[0], v[1]}; }
static inline PolDep operator+(PolDep a, PolDep b) { return PolDep{a.par + b.par, a.perp + b.perp}; }
static inline PolDep operator-(PolDep a, PolDep b) { return PolDep{a.par - b.par, a.perp - b.perp}; }
static inline PolDep operator*(double s, PolDep a) { return PolDep{s * a.par, s * a.perp}; }
static inline PolDep operator*(PolDep a, double s) { return PolDep{a.par * s, a.perp * s}; }
static inline PolDep operator*(PolDep a, PolDep b) { return PolDep{a.par * b.par, a.perp * b.perp}; }
static inline PolDep operator/(PolDep a, PolDep b) { return PolDep{a.par / b.par, a.perp / b.perp}; }
static inline PolDep pd_div(PolDep a, double s) { return a * (1.0 / s); }  // Div<f64>: times the reciprocal
static inline PolDep pd_exp(PolDep a) { return PolDep{std::exp(a.par), std::exp(a.perp)}; }
static inline PolDep pd_ln(PolDep a) { return PolDep{std::log(a.par), std::log(a.perp)}; }
static inline PolDep pd_powf(PolDep a, PolDep m) { return PolDep{std::pow(a.par, m.par), std::pow(a.perp, m.perp)}; }

// pair_creation/lp/mod.rs:345-370
static void lpp_sum_limits(double a, double eta, int* n_min_out, int* n_max_out) {
    double n_min = std::ceil(2.0 * (1.0 + 0.5 * a * a) / eta);
    double range = a < 1.0 ? 2.0 + (2.0 + 20.0 * a * a) * std::exp(-std::sqrt(0.5 * eta))
                           : 3.0 + 2.8 * std::pow(a, 8.0 / 3.0) / std::cbrt(eta) + 0.25 * a * a * a * std::sqrt(eta);
    double test = 0.25 - (1.0 + 0.5 * a * a) / (2.0 * n_min * eta);
    if (test <= 2.220446049250313e-16) {
        *n_min_out = rust_as_i32(n_min) + 1;
        *n_max_out = rust_as_i32(n_min + 1.0 + range);
    } else {
        *n_min_out = rust_as_i32(n_min);
        *n_max_out = rust_as_i32(n_min + range);
    }
}

// pair_creation/lp/mod.rs:371-374
static bool lpp_is_negligible(double a, double eta) {
    return std::log10(eta) < -1.0 - std::pow(std::log10(a) + 2.0, 2) / 4.5;
}

// pair_creation/lp/tables/mod.rs:19-58
static bool lpp_main_contains(double a, double eta) {
    return std::log(a) >= PTG_BW_LP_LN_MIN_A && a < 25.0 && std::log(eta) >= PTG_BW_LP_LN_MIN_ETA && eta < 2.0;
}

static bool lpp_main_interpolate(double a, double eta, double f[2]) {
    const double* T = g_lma.bw_lp_total;  // [61][25][2]
    const double LMA = PTG_BW_LP_LN_MIN_A, LME = PTG_BW_LP_LN_MIN_ETA, SA = PTG_BW_LP_LN_A_STEP, SE = PTG_BW_LP_LN_ETA_STEP;
    int ia = (int)((std::log(a) - LMA) / SA);
    int ie = (int)((std::log(eta) - LME) / SE);
    if (ia < 0 || ie < 0 || ia >= 25 - 1 || ie >= 61 - 1) return false;
    auto at = [&](int e, int c) { return pd(T + ((size_t)e * 25 + c) * 2); };
    PolDep r;
    if (a * eta > 2.0) {
        double da = (std::log(a) - LMA) / SA - ia;
        double de = (std::log(eta) - LME) / SE - ie;
        r = (1.0 - da) * (1.0 - de) * at(ie, ia) + da * (1.0 - de) * at(ie, ia + 1) + (1.0 - da) * de * at(ie + 1, ia) +
            da * de * at(ie + 1, ia + 1);
    } else {
        double a_min = std::exp(LMA + ia * SA), a_max = std::exp(LMA + (ia + 1) * SA);
        double e_min = std::exp(LME + ie * SE), e_max = std::exp(LME + (ie + 1) * SE);
        double da = ((a_min * a_max / a) - a_min) / (a_max - a_min);
        double de = ((e_min * e_max / eta) - e_min) / (e_max - e_min);
        r = at(ie, ia) * da * de + at(ie, ia + 1) * (1.0 - da) * de + at(ie + 1, ia) * da * (1.0 - de) +
            at(ie + 1, ia + 1) * (1.0 - da) * (1.0 - de);
    }
    PolDep e = pd_exp(r);
    f[0] = e.par, f[1] = e.perp;
    return true;
}

// pair_creation/lp/tables/mid_range/mod.rs:9-98
static bool lpp_mid_contains(double a, double eta) {
    double ln_a = std::log(a);
    double lep = std::log(eta / (1.0 + 0.5 * a * a));
    return ln_a > PTG_BW_LPM_LN_MIN_A && a < 2.0 && lep > PTG_BW_LPM_LN_MIN_ETA_PRIME && lep < PTG_BW_LPM_LN_MAX_ETA_PRIME;
}

static PolDep lpp_mid_interp_eta_prime(double ep, int ia) {
    const double* T = g_lma.bw_lp_mid_total;  // [157][36][2]
    const double D = PTG_BW_LPM_ETA_PRIME_DENSITY;
    int ie = rust_as_i32(D * (std::exp(PTG_BW_LPM_LN_MAX_ETA_PRIME) / ep - 1.0));
    if (ie % (int)D == (int)D - 1) ie -= 1;
    auto at = [&](int e) { return pd(T + ((size_t)e * 36 + ia) * 2); };
    double l0 = 2.0 / (1.0 + (double)(ie + 2) / D), m0 = 2.0 / (1.0 + (double)(ie + 1) / D), u0 = 2.0 / (1.0 + (double)ie / D);
    PolDep l1 = at(ie + 2), m1 = at(ie + 1), u1 = at(ie);
    PolDep m = pd_div(pd_ln((u1 - l1) / (m1 - l1)), std::log((u0 - l0) / (m0 - l0)));
    PolDep alpha = (m1 - l1) / pd_powf(PolDep{m0 - l0, m0 - l0}, m);
    PolDep r = alpha * pd_powf(PolDep{ep - l0, ep - l0}, m) + l1;
    if (!std::isfinite(r.par)) {
        if (ep < m0) {
            double w = (std::log(ep) - std::log(l0)) / (std::log(m0) - std::log(l0));
            r.par = (1.0 - w) * l1.par + w * m1.par;
        } else {
            double w = (std::log(ep) - std::log(m0)) / (std::log(u0) - std::log(m0));
            r.par = (1.0 - w) * m1.par + w * u1.par;
        }
    }
    if (!std::isfinite(r.perp)) {
        if (ep < m0) {
            double w = (std::log(ep) - std::log(l0)) / (std::log(m0) - std::log(l0));
            r.perp = (1.0 - w) * l1.perp + w * m1.perp;
        } else {
            double w = (std::log(ep) - std::log(m0)) / (std::log(u0) - std::log(m0));
            r.perp = (1.0 - w) * m1.perp + w * u1.perp;
        }
    }
    return r;
}

static void lpp_mid_interpolate(double a, double eta, double f[2]) {
    const double LMA = PTG_BW_LPM_LN_MIN_A, SA = PTG_BW_LPM_LN_A_STEP;
    int ia = rust_as_i32((std::log(a) - LMA) / SA);
    double ep = eta / (1.0 + 0.5 * a * a);
    PolDep r;
    if (a < 0.5) {
        double da = (std::log(a) - LMA) / SA - ia;
        r = (1.0 - da) * lpp_mid_interp_eta_prime(ep, ia) + da * lpp_mid_interp_eta_prime(ep, ia + 1);
    } else {
        double a_min = std::exp(LMA + ia * SA), a_max = std::exp(LMA + (ia + 1) * SA);
        double da = (a - a_min) / (a_max - a_min);
        r = pd_div((1.0 - da) * a_min * lpp_mid_interp_eta_prime(ep, ia) + da * a_max * lpp_mid_interp_eta_prime(ep, ia + 1), a);
    }
    PolDep e = pd_exp(r);
    f[0] = e.par, f[1] = e.perp;
}

// pair_creation/lp/mod.rs:380-420: [f_par, f_perp]; false outside every table
bool lp_pair_rates(double a, double eta, double f[2]) {
    f[0] = f[1] = 0.0;
    if (lpp_is_negligible(a, eta)) return true;
    if (lpp_mid_contains(a, eta)) {
        lpp_mid_interpolate(a, eta, f);
        return true;
    }
    if (lpp_main_contains(a, eta)) return lpp_main_interpolate(a, eta, f);
    return true;  // outside both tables the reference takes the rate as zero
}

// pair_creation/lp/mod.rs:385-420 (probability and Stokes update)
static double lpp_probability(const double f[2], double eta, const Stokes& sv, double dphi, Stokes* out) {
    double f0 = f[0], f1 = f[1];
    double prob = ALPHA_FINE * (0.5 * ((f0 + f1) + sv.q * (f0 - f1))) * dphi / eta;
    double prob_avg = ALPHA_FINE * (0.5 * (f0 + f1)) * dphi / eta;
    double delta = ALPHA_FINE * (0.5 * (f0 - f1)) * dphi / eta;
    *out = Stokes(sv.i, (sv.q * (1.0 - prob_avg) - delta) / (1.0 - prob), sv.u * (1.0 - prob_avg) / (1.0 - prob),
                  sv.v * (1.0 - prob_avg) / (1.0 - prob));
    return prob;
}

// pair_creation/lp/tables/mod.rs:60-113
static int lpp_main_invert(double a, double eta, double sv1, double frac) {
    const double* T = g_lma.bw_lp_cdf;  // [1525][16][3]
    double fa = (std::log(a) - PTG_BW_LP_CDF_MIN_0) / PTG_BW_LP_CDF_STEP_0;
    double fe = (std::log(eta) - PTG_BW_LP_CDF_MIN_1) / PTG_BW_LP_CDF_STEP_1;
    int ia = (int)fa, ie = (int)fe;
    double da = fa - std::trunc(fa), de = fe - std::trunc(fe);
    int idx[4] = {25 * ie + ia, 25 * ie + ia + 1, 25 * (ie + 1) + ia, 25 * (ie + 1) + ia + 1};
    double w[4] = {(1.0 - da) * (1.0 - de), da * (1.0 - de), (1.0 - da) * de, da * de};
    double u = 0.0;
    for (int k = 0; k < 4; ++k) {
        if (idx[k] < 0 || idx[k] >= 1525) return -1;
        const double* src = T + (size_t)idx[k] * 48;
        double n_min = src[0];
        double f_max = PolDep{src[45 + 1], src[45 + 2]}.interp(sv1);
        double tb[30];
        for (int i = 0; i < 15; ++i) {
            tb[2 * i] = std::log(src[3 * i] - n_min + 1.0);
            double f = PolDep{src[3 * i + 1], src[3 * i + 2]}.interp(sv1);
            tb[2 * i + 1] = std::log(-1.0 * std::log(1.0 - f / f_max));
        }
        bool ok;
        double uk = Pwmci(tb, 15, true).invert(std::log(-1.0 * std::log(1.0 - frac)), &ok);
        u += uk * w[k];
    }
    int n_min, n_max;
    lpp_sum_limits(a, eta, &n_min, &n_max);
    double n = (double)n_min + std::expm1(u);
    return rust_as_i32(n) + 1;
}

// pair_creation/lp/tables/mid_range/mod.rs:100-270 (needs the regenerated
// mid-range CDF)
static int lpp_mid_corners(double a, double eta, int ie_out[1], int idx[4], double w[4], bool* next_to_bdy) {
    const double LMA = PTG_BW_LPM_LN_MIN_A, SA = PTG_BW_LPM_LN_A_STEP, D = PTG_BW_LPM_ETA_PRIME_DENSITY;
    int ia = rust_as_i32((std::log(a) - LMA) / SA);
    double da = (std::log(a) - LMA) / SA - ia;
    double ep = eta / (1.0 + 0.5 * a * a);
    int ie = rust_as_i32(D * (std::exp(PTG_BW_LPM_LN_MAX_ETA_PRIME) / ep - 1.0));
    *next_to_bdy = ie % (int)D == (int)D - 1;
    if (*next_to_bdy) ie -= 1;
    double lower = std::exp(PTG_BW_LPM_LN_MAX_ETA_PRIME) / (1.0 + (double)(ie + 1) / D);
    double upper = std::exp(PTG_BW_LPM_LN_MAX_ETA_PRIME) / (1.0 + (double)ie / D);
    double de = (std::log(ep) - std::log(lower)) / (std::log(upper) - std::log(lower));
    idx[0] = 36 * ie + ia, idx[1] = 36 * ie + ia + 1, idx[2] = 36 * (ie + 1) + ia, idx[3] = 36 * (ie + 1) + ia + 1;
    w[0] = (1.0 - da) * de, w[1] = da * de, w[2] = (1.0 - da) * (1.0 - de), w[3] = da * (1.0 - de);
    ie_out[0] = ie;
    for (int k = 0; k < 4; ++k)
        if (idx[k] < 0 || idx[k] >= 5652) return -1;
    return 0;
}

static int lpp_mid_invert(double a, double eta, double sv1, double frac) {
    const double* T = g_lma.bw_lp_mid_cdf;  // [5652][16][3]
    if (!T) return -2;
    int ie, idx[4];
    double w[4];
    bool bdy;
    if (lpp_mid_corners(a, eta, &ie, idx, w, &bdy) < 0) return -1;
    int n_min, n_max;
    lpp_sum_limits(a, eta, &n_min, &n_max);
    double fr[2];
    lpp_mid_interpolate(a, eta, fr);
    double total_rate = 0.5 * ((fr[0] + fr[1]) + sv1 * (fr[0] - fr[1]));
    double p_lowest = 0.0;
    if (bdy) {
        // interpolate_lowest_harmonic (mid_range/mod.rs:100-150), with the
        // weights of that function's own (unshifted) eta' bracket
        const double LMA = PTG_BW_LPM_LN_MIN_A, SA = PTG_BW_LPM_LN_A_STEP, D = PTG_BW_LPM_ETA_PRIME_DENSITY;
        int ia = rust_as_i32((std::log(a) - LMA) / SA);
        double da = (std::log(a) - LMA) / SA - ia;
        double ep = eta / (1.0 + 0.5 * a * a);
        int ie0 = rust_as_i32(D * (std::exp(PTG_BW_LPM_LN_MAX_ETA_PRIME) / ep - 1.0));
        double lower = std::exp(PTG_BW_LPM_LN_MAX_ETA_PRIME) / (1.0 + (double)(ie0 + 1) / D);
        double upper = std::exp(PTG_BW_LPM_LN_MAX_ETA_PRIME) / (1.0 + (double)ie0 / D);
        double de = (std::log(ep) - std::log(lower)) / (std::log(upper) - std::log(lower));
        int jx[4] = {36 * ie0 + ia, 36 * ie0 + ia + 1, 36 * (ie0 + 1) + ia, 36 * (ie0 + 1) + ia + 1};
        double wx[4] = {(1.0 - da) * de, da * de, (1.0 - da) * (1.0 - de), da * (1.0 - de)};
        double acc = 0.0;
        for (int k = 0; k < 4; ++k) {
            if (jx[k] < 0 || jx[k] >= 5652) return -1;
            const double* tb = T + (size_t)jx[k] * 48;
            double fr0 = 0.0;
            if (!(tb[0] > (double)n_min)) {
                double f = PolDep{tb[1], tb[2]}.interp(sv1);
                double f_max = PolDep{tb[46], tb[47]}.interp(sv1);
                fr0 = f / f_max;
            }
            acc += wx[k] * std::pow(fr0 * total_rate, 3);
        }
        double rate_lowest = std::cbrt(acc);
        p_lowest = rate_lowest / total_rate;
        if (frac <= p_lowest) return n_min;
    }
    double n = 0.0;
    for (int k = 0; k < 4; ++k) {
        const double* src = T + (size_t)idx[k] * 48;
        double f_max = PolDep{src[46], src[47]}.interp(sv1);
        double tb[32];
        for (int i = 0; i < 16; ++i) {
            tb[2 * i] = src[3 * i];
            tb[2 * i + 1] = PolDep{src[3 * i + 1], src[3 * i + 2]}.interp(sv1) / f_max;
        }
        double nk;
        bool ok = true;
        if (bdy) {
            if (tb[0] == (double)n_min) {
                double t01 = tb[1];
                for (int i = 0; i < 16; ++i) tb[2 * i + 1] = (t01 - tb[2 * i + 1] + p_lowest * (tb[2 * i + 1] - 1.0)) / (t01 - 1.0);
            }
            nk = Pwmci(tb, 16).invert(frac, &ok);
        } else {
            nk = frac <= tb[1] ? tb[0] - 0.1 : Pwmci(tb, 16).invert(frac, &ok);
        }
        if (!ok) return -1;  // the reference unwraps this inversion
        n += nk * w[k];
    }
    return std::isfinite(n) ? rust_as_i32(std::ceil(n)) : -1;
}

// pair_creation/lp/theta_bound.rs:11-101
struct LppThetaBound {
    double s[16], f[16];
    void init(int n, double a, double eta) {
        double s_min = 0.5;
        double s_max = 0.5 + std::sqrt(0.25 - (1.0 + 0.5 * a * a) / (2.0 * n * eta));
        for (int i = 0; i < 16; ++i) {
            double z = std::cos(PI * i / 15.0);
            s[i] = s_min + 0.5 * (z + 1.0) * (s_max - s_min);
            double r_n = std::sqrt(2.0 * n * eta * s[i] * (1.0 - s[i]) - (1.0 + 0.5 * a * a));
            double x = a * r_n / (eta * s[i] * (1.0 - s[i]));
            double y = a * a / (8.0 * eta * s[i] * (1.0 - s[i]));
            double x_crit = y > n / 6.0 ? 4.0 * std::sqrt(y) * std::sqrt(n - 2.0 * y) : n + 2.0 * y;
            double ln_j_crit = std::log(0.443) - std::log((double)n) / 3.0;
            double ln_j_bdy = ThetaBound::ln_double_bessel_x_zero(n % 2 == 0 ? n : n + 1, y);
            ln_j_bdy = std::fmin(ln_j_bdy, ln_j_crit);
            double ct = std::fmax(1.0 - x_crit * std::log(0.01) / (x * (ln_j_bdy - ln_j_crit)), -1.0);
            f[i] = std::acos(ct);
            if (std::isnan(f[i])) f[i] = PI;
        }
        double f_min = f[0];
        for (int i = 1; i < 16; ++i) {
            if (f[i] < f_min)
                f_min = f[i];
            else
                f[i] = f_min;
        }
    }
    double at(double arg) const {
        double val = f[15];
        for (int i = 1; i < 16; ++i) {
            if (arg > s[i]) {
                double wt = (arg - s[i - 1]) / (s[i] - s[i - 1]);
                val = wt * f[i] + (1.0 - wt) * f[i - 1];
                break;
            }
        }
        return std::fmin(val, FRAC_PI_2);
    }
};

// pair_creation/lp/mod.rs:27-114: the double-differential partial rate
struct LppRate {
    int n;
    double a, eta;
    DoubleBessel dj;
    LppThetaBound tb;
    LppRate(int n_, double a_, double eta_) : n(n_), a(a_), eta(eta_), dj(n_, n_ * SQRT_2, n_ * 0.5) { tb.init(n, a, eta); }
    void s_bounds(double* s_min, double* s_max) const {
        *s_min = 0.5;
        *s_max = std::fmax(0.5 + std::sqrt(0.25 - (1.0 + 0.5 * a * a) / (2.0 * n * eta)), 0.5);
    }
    void elements(double s, double theta, double* unpol, double* d1, double* d2) {
        double r2 = 2.0 * n * eta * s * (1.0 - s) - (1.0 + 0.5 * a * a);
        if (!(r2 > 0.0)) {
            *unpol = *d1 = *d2 = 0.0;
            return;
        }
        double rn = std::sqrt(r2);
        double x = a * rn * std::cos(theta) / (eta * s * (1.0 - s));
        double y = a * a / (8.0 * eta * s * (1.0 - s));
        double j[5];
        dj.evaluate(x, y, j);
        double g0 = j[2], g1 = 0.5 * (j[1] + j[3]), g2 = 0.25 * (j[0] + 2.0 * j[2] + j[4]);
        double h_s = 0.5 / (s * (1.0 - s)) - 1.0;
        *unpol = powi(g0, 2) + a * a * h_s * (powi(g1, 2) - g0 * g2);
        *d1 = powi(g0 * rn * std::cos(theta) - g1 * a, 2) - powi(g0 * std::sin(theta), 2) * r2;
        *d2 = 2.0 * g0 * rn * std::sin(theta) * (g0 * rn * std::cos(theta) - g1 * a);
    }
    double fully_resolved(double s, double theta, double sv1, double sv2) {
        double u, d1, d2;
        elements(s, theta, &u, &d1, &d2);
        return (u - sv1 * d1 - sv2 * d2) / (2.0 * PI);
    }
    // (unpol - delta, unpol + delta) / 2 pi: the two linear polarisations
    void at(double s, double theta, double out[2]) {
        double u, d1, d2;
        elements(s, theta, &u, &d1, &d2);
        out[0] = (u - d1) / (2.0 * PI);
        out[1] = (u + d1) / (2.0 * PI);
    }
    double ceiling(double sv1, double sv2) {
        double s_min, s_max;
        s_bounds(&s_min, &s_max);
        double centre = 0.5 + std::sqrt(0.25 - (1.0 + a * a) / (2.0 * n * eta));
        double lower = s_min, upper = s_max;
        if (std::isfinite(centre)) {
            lower = std::fmax(centre - 0.2, s_min);
            upper = 0.5 * (centre + s_max);
        }
        double mx = NAN;
        for (int i = 0; i < 50; ++i) {
            double v = fully_resolved(lower + (upper - lower) * (double)i / 50.0, 0.0, sv1, sv2);
            mx = std::isnan(mx) ? v : (std::isnan(v) ? mx : std::max(mx, v));
        }
        return 1.2 * mx;
    }
    int sample(double sv1, double sv2, DrawStream& rng, double* s_out, double* theta_out, uint64_t* rej) {
        double s_min, s_max;
        s_bounds(&s_min, &s_max);
        double mx = ceiling(sv1, sv2);
        double s = 0.0, theta = 0.0;
        int it;
        for (it = 0; it < REJECTION_CAP; ++it) {
            double ss = s_min + (s_max - s_min) * rng.next();
            double th = FRAC_PI_2 * rng.next();
            if (th > tb.at(ss)) continue;
            double z = mx * rng.next();
            if (z < fully_resolved(ss, th, sv1, sv2)) {
                s = ss, theta = th;
                break;
            }
        }
        *rej += it;
        if (it == REJECTION_CAP) return PTG_ERR_REJECTION_CAP;
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
        return PTG_OK;
    }
};

// pair_creation/lp/mod.rs:424-441
int lp_pair_sample(double a, double eta, double sv1, double sv2, DrawStream& rng, int* n_out, double* s, double* theta,
                   uint64_t* rej) {
    double frac = rng.next();
    int n;
    if (lpp_mid_contains(a, eta))
        n = lpp_mid_invert(a, eta, sv1, frac);
    else if (lpp_main_contains(a, eta))
        n = lpp_main_invert(a, eta, sv1, frac);
    else
        return PTG_ERR_OUT_OF_TABLE;
    if (n == -2) return PTG_ERR_TABLES;
    if (n < 1) return PTG_ERR_OUT_OF_TABLE;
    LppRate r(n, a, eta);
    *n_out = n;
    return r.sample(sv1, sv2, rng, s, theta, rej);
}


// ------------------------------------- LP Breit-Wheeler table generator --
// quadrature/adaptive.rs:1-370: adaptive 2-D Clenshaw-Curtis integration of
// a complex integrand (here the two linear polarisations)
struct C2 {
    double re, im;
};
static inline C2 c2_add(C2 a, C2 b) { return C2{a.re + b.re, a.im + b.im}; }
static inline C2 c2_sub(C2 a, C2 b) { return C2{a.re - b.re, a.im - b.im}; }
static inline C2 c2_scale(double s, C2 a) { return C2{s * a.re, s * a.im}; }

struct AdRegion {
    C2 integral, error;
    double x[2], y[2];
    C2 cache[3][3];
};

static const double CC5[5][3] = {{0.0, 1.0 / 30.0, 1.0 / 6.0},
                                 {0.1464466094067262, 4.0 / 15.0, 0.0},
                                 {0.5, 2.0 / 5.0, 2.0 / 3.0},
                                 {0.8535533905932738, 4.0 / 15.0, 0.0},
                                 {1.0, 1.0 / 30.0, 1.0 / 6.0}};
static const double CC5_EXT[9] = {0.0, 0.1464466094067262, 0.5, 0.8535533905932738, 1.0,
                                  1.1464466094067262, 1.5, 1.8535533905932738, 2.0};
static const double CC9[9][3] = {{0.0000000000000000, 0.0079365079365079, 1.0 / 30.0},
                                 {0.0380602337443566, 0.0731093246080091, 0.0},
                                 {0.1464466094067262, 0.1396825396825397, 4.0 / 15.0},
                                 {0.3086582838174551, 0.1808589293602449, 0.0},
                                 {0.5000000000000000, 0.1968253968253968, 2.0 / 5.0},
                                 {0.6913417161825449, 0.1808589293602449, 0.0},
                                 {0.8535533905932738, 0.1396825396825397, 4.0 / 15.0},
                                 {0.9619397662556434, 0.0731093246080091, 0.0},
                                 {1.0000000000000000, 0.0079365079365079, 1.0 / 30.0}};
static const double CC9_EXT[17] = {0.0000000000000000, 0.0380602337443566, 0.1464466094067262, 0.3086582838174551,
                                   0.5000000000000000, 0.6913417161825449, 0.8535533905932738, 0.9619397662556434,
                                   1.0000000000000000, 1.0380602337443566, 1.1464466094067262, 1.3086582838174551,
                                   1.5000000000000000, 1.6913417161825449, 1.8535533905932738, 1.9619397662556434,
                                   2.0000000000000000};

template <class F, class R>
static AdRegion ad_new(F& f, R& inside, double x0, double x1, double y0, double y1) {
    AdRegion g;
    C2 result{0.0, 0.0}, error{0.0, 0.0};
    for (int i = 0; i < 5; ++i) {
        double y = y0 + CC5[i][0] * (y1 - y0);
        for (int j = 0; j < 5; ++j) {
            double x = x0 + CC5[j][0] * (x1 - x0);
            C2 z = inside(x, y) ? f(x, y) : C2{0.0, 0.0};
            result = c2_add(result, c2_scale(CC5[i][1] * CC5[j][1] * (y1 - y0) * (x1 - x0), z));
            error = c2_add(error, c2_scale(CC5[i][2] * CC5[j][2] * (y1 - y0) * (x1 - x0), z));
            if (i % 2 == 0 && j % 2 == 0) g.cache[i / 2][j / 2] = z;
        }
    }
    g.integral = result;
    g.error = c2_sub(result, error);
    g.x[0] = x0, g.x[1] = x1, g.y[0] = y0, g.y[1] = y1;
    return g;
}

static AdRegion ad_child(C2 res, C2 err, double xa, double xb, double ya, double yb, const C2 c[3][3]) {
    AdRegion g;
    g.integral = res;
    g.error = c2_sub(res, err);
    g.x[0] = xa, g.x[1] = xb, g.y[0] = ya, g.y[1] = yb;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) g.cache[i][j] = c[i][j];
    return g;
}

// Region::custom_partition (adaptive.rs:33-152)
template <class F, class R>
static void ad_custom_partition(const AdRegion& r, F& f, R& inside, bool sx, double xs, bool sy, double ys,
                                AdRegion out[4]) {
    double x0 = r.x[0], x1 = r.x[1], y0 = r.y[0], y1 = r.y[1];
    double x_mid = sx ? xs : 0.5 * (x0 + x1);
    double y_mid = sy ? ys : 0.5 * (y0 + y1);
    C2 z[9][9];
    for (int i = 0; i < 9; ++i) {
        double ty = CC5_EXT[i];
        double y = i < 4 ? y0 + ty * (y_mid - y0) : y_mid + (ty - 1.0) * (y1 - y_mid);
        for (int j = 0; j < 9; ++j) {
            double tx = CC5_EXT[j];
            double x = j < 4 ? x0 + tx * (x_mid - x0) : x_mid + (tx - 1.0) * (x1 - x_mid);
            if (i % 8 == 0 && j % 8 == 0)
                z[i][j] = r.cache[i / 4][j / 4];
            else if (i % 4 == 0 && j % 4 == 0 && !sx && !sy)
                z[i][j] = r.cache[i / 4][j / 4];
            else
                z[i][j] = inside(x, y) ? f(x, y) : C2{0.0, 0.0};
        }
    }
    C2 res[4], err[4];
    for (int q = 0; q < 4; ++q) res[q] = err[q] = C2{0.0, 0.0};
    for (int rr = 0; rr < 2; ++rr)
        for (int cc = 0; cc < 2; ++cc)
            for (int i = 0; i < 5; ++i)
                for (int j = 0; j < 5; ++j) {
                    C2 val = z[i + 4 * rr][j + 4 * cc];
                    double dy = rr < 1 ? y_mid - y0 : y1 - y_mid;
                    double dx = cc < 1 ? x_mid - x0 : x1 - x_mid;
                    res[2 * rr + cc] = c2_add(res[2 * rr + cc], c2_scale(CC5[j][1] * CC5[i][1] * dx * dy, val));
                    err[2 * rr + cc] = c2_add(err[2 * rr + cc], c2_scale(CC5[j][2] * CC5[i][2] * dx * dy, val));
                }
    C2 cb[3][3] = {{z[0][0], z[0][2], z[0][4]}, {z[2][0], z[2][2], z[2][4]}, {z[4][0], z[4][2], z[4][4]}};
    C2 cr[3][3] = {{z[0][4], z[0][6], z[0][8]}, {z[2][4], z[2][6], z[2][8]}, {z[4][4], z[4][6], z[4][8]}};
    C2 ct[3][3] = {{z[4][0], z[4][2], z[4][4]}, {z[6][0], z[6][2], z[6][4]}, {z[8][0], z[8][2], z[8][4]}};
    C2 cu[3][3] = {{z[4][4], z[4][6], z[4][8]}, {z[6][4], z[6][6], z[6][8]}, {z[8][4], z[8][6], z[8][8]}};
    out[0] = ad_child(res[0], err[0], x0, x_mid, y0, y_mid, cb);
    out[1] = ad_child(res[1], err[1], x_mid, x1, y0, y_mid, cr);
    out[2] = ad_child(res[2], err[2], x0, x_mid, y_mid, y1, ct);
    out[3] = ad_child(res[3], err[3], x_mid, x1, y_mid, y1, cu);
}

// Region::partition (adaptive.rs:180-300)
template <class F, class R>
static void ad_partition(const AdRegion& r, F& f, R& inside, AdRegion out[4]) {
    double x0 = r.x[0], x1 = r.x[1], y0 = r.y[0], y1 = r.y[1];
    double x_mid = 0.5 * (x0 + x1), y_mid = 0.5 * (y0 + y1);
    static thread_local C2 z[17][17];
    for (int i = 0; i < 17; ++i) {
        double y = y0 + 0.5 * CC9_EXT[i] * (y1 - y0);
        for (int j = 0; j < 17; ++j) {
            double x = x0 + 0.5 * CC9_EXT[j] * (x1 - x0);
            if (i % 8 == 0 && j % 8 == 0)
                z[i][j] = r.cache[i / 8][j / 8];
            else
                z[i][j] = inside(x, y) ? f(x, y) : C2{0.0, 0.0};
        }
    }
    C2 res[4], err[4];
    for (int q = 0; q < 4; ++q) res[q] = err[q] = C2{0.0, 0.0};
    for (int rr = 0; rr < 2; ++rr)
        for (int cc = 0; cc < 2; ++cc)
            for (int i = 0; i < 9; ++i)
                for (int j = 0; j < 9; ++j) {
                    C2 val = z[i + 8 * rr][j + 8 * cc];
                    double dy = 0.5 * (y1 - y0), dx = 0.5 * (x1 - x0);
                    res[2 * rr + cc] = c2_add(res[2 * rr + cc], c2_scale(CC9[j][1] * CC9[i][1] * dx * dy, val));
                    err[2 * rr + cc] = c2_add(err[2 * rr + cc], c2_scale(CC9[j][2] * CC9[i][2] * dx * dy, val));
                }
    C2 cb[3][3] = {{z[0][0], z[0][4], z[0][8]}, {z[4][0], z[4][4], z[4][8]}, {z[8][0], z[8][4], z[8][8]}};
    C2 cr[3][3] = {{z[0][8], z[0][12], z[0][16]}, {z[4][8], z[4][12], z[4][16]}, {z[8][8], z[8][12], z[8][16]}};
    C2 ct[3][3] = {{z[8][0], z[8][4], z[8][8]}, {z[12][0], z[12][4], z[12][8]}, {z[16][0], z[16][4], z[16][8]}};
    C2 cu[3][3] = {{z[8][8], z[8][12], z[8][16]}, {z[12][8], z[12][12], z[12][16]}, {z[16][8], z[16][12], z[16][16]}};
    out[0] = ad_child(res[0], err[0], x0, x_mid, y0, y_mid, cb);
    out[1] = ad_child(res[1], err[1], x_mid, x1, y0, y_mid, cr);
    out[2] = ad_child(res[2], err[2], x0, x_mid, y_mid, y1, ct);
    out[3] = ad_child(res[3], err[3], x_mid, x1, y_mid, y1, cu);
}

// integrate_2d (adaptive.rs:316-370)
template <class F, class R>
static C2 ad_integrate_2d(F f, double x0, bool has_xd, double xd, double x1, double y0, bool has_yd, double yd, double y1,
                          R inside, double tol, int max_recursion) {
    std::vector<AdRegion> regions;
    regions.reserve(64);
    AdRegion first = ad_new(f, inside, x0, x1, y0, y1);
    if (!has_xd && !has_yd) {
        regions.push_back(first);
    } else {
        AdRegion q[4];
        ad_custom_partition(first, f, inside, has_xd, xd, has_yd, yd, q);
        for (auto& g : q) regions.push_back(g);
    }
    C2 integral{0.0, 0.0};
    for (int it = 0; it < max_recursion; ++it) {
        C2 i_sum{0.0, 0.0}, e_sum{0.0, 0.0};
        for (const auto& g : regions) {
            i_sum = c2_add(i_sum, g.integral);
            e_sum = c2_add(e_sum, g.error);
        }
        integral = i_sum;
        if (std::fabs(e_sum.re) <= tol * std::fabs(i_sum.re) && std::fabs(e_sum.im) <= tol * std::fabs(i_sum.im)) break;
        AdRegion worst = regions.back();
        regions.pop_back();
        AdRegion q[4];
        ad_partition(worst, f, inside, q);
        for (auto& g : q) regions.push_back(g);
        std::stable_sort(regions.begin(), regions.end(), [](const AdRegion& a, const AdRegion& b) {
            return a.error.re * a.error.re + a.error.im * a.error.im < b.error.re * b.error.re + b.error.im * b.error.im;
        });
    }
    return integral;
}

// pair_creation/lp/mod.rs:115-227: DoubleDiffPartialRate::integrate, the
// partial rate for the two linear polarisations (multiply by alpha/eta)
static C2 lpp_integrate(int n, double a, double eta) {
    LppRate r(n, a, eta);
    double s_min, s_max;
    r.s_bounds(&s_min, &s_max);
    auto at = [&](double s, double th) {
        double o[2];
        r.at(s, th, o);
        return C2{o[0], o[1]};
    };
    if (r.tb.at(0.5) < 0.75 * FRAC_PI_2) {
        double s_peak = 0.5 + std::sqrt(0.25 - (1.0 + a * a) / (2.0 * n * eta));
        bool has_peak = s_peak > s_min + 2.0 * (s_max - s_min) / 3.0;
        double theta_split = r.tb.at(has_peak ? s_peak : 0.5);
        LppThetaBound tb = r.tb;
        C2 v = ad_integrate_2d(at, s_min, has_peak, s_peak, s_max, 0.0, true, theta_split, FRAC_PI_2,
                               [&](double s, double th) { return th < tb.at(s); }, 1.0e-3, 16);
        return c2_scale(4.0 * 2.0, v);
    }
    double s_peak = std::fmin(0.5 + std::sqrt(0.25 - (1.0 + a * a) / (2.0 * n * eta)), 0.5);
    C2 integral{0.0, 0.0};
    auto segment = [&](double s0, double s1, const double* nodes, const double* weights, int nn) {
        C2 acc{0.0, 0.0};
        for (int k = 0; k < nn; ++k) {
            double s = s0 + 0.5 * (nodes[k] + 1.0) * (s1 - s0);
            double mt = r.tb.at(s);
            C2 sd{0.0, 0.0};
            for (int q = 0; q < 32; ++q) {
                double th = 0.5 * (PTG_GAUSS_32_NODES[q] + 1.0) * mt;
                sd = c2_add(sd, c2_scale(0.5 * PTG_GAUSS_32_WEIGHTS[q] * mt, at(s, th)));
            }
            acc = c2_add(acc, c2_scale(0.5 * weights[k] * (s1 - s0), sd));
        }
        return acc;
    };
    if (s_peak < s_min + 2.0 * (s_max - s_min) / 3.0) {
        s_peak = std::fmin(s_peak, s_min + (s_max - s_min) / 3.0);
        integral = c2_add(segment(s_min, s_peak, PTG_GAUSS_32_NODES, PTG_GAUSS_32_WEIGHTS, 32),
                          segment(s_peak, s_max, PTG_GAUSS_32_NODES, PTG_GAUSS_32_WEIGHTS, 32));
    } else {
        double delta = s_max - s_peak;
        integral = c2_add(c2_add(segment(s_min, s_max - 2.0 * delta, PTG_GAUSS_16_NODES, PTG_GAUSS_16_WEIGHTS, 16),
                                 segment(s_max - 2.0 * delta, s_peak, PTG_GAUSS_32_NODES, PTG_GAUSS_32_WEIGHTS, 32)),
                          segment(s_peak, s_max, PTG_GAUSS_32_NODES, PTG_GAUSS_32_WEIGHTS, 32));
    }
    return c2_scale(2.0 * 4.0, integral);
}

void lp_pair_partial_rate(int n, double a, double eta, double out[2]) {
    C2 v = lpp_integrate(n, a, eta);
    out[0] = v.re, out[1] = v.im;
}

// pair_creation/lp/mod.rs:443-507: TotalRate::by_summation, the 16 CDF
// nodes [n, cumulative par, cumulative perp]
void lp_pair_by_summation(double a, double eta, double cdf[48]) {
    int n_min, n_max;
    lpp_sum_limits(a, eta, &n_min, &n_max);
    std::vector<C2> cum;
    C2 total{0.0, 0.0};
    for (int n = n_min; n <= n_max; ++n) {
        total = c2_add(total, lpp_integrate(n, a, eta));
        cum.push_back(total);
    }
    double delta = (double)(n_max - n_min);
    double u_max = std::log(1.0 + delta);
    for (int i = 0; i < 48; ++i) cdf[i] = 0.0;
    cdf[0] = (double)n_min;
    double u = 0.0, du = u_max / 15.0;
    for (int i = 1; i <= 15; ++i) {
        u = u + du;
        double nn = (double)n_min + std::expm1(u);
        if (std::round(nn) <= cdf[3 * (i - 1)]) {
            nn = cdf[3 * (i - 1)] + 1.0;
            u = std::log(nn - (double)n_min + 1.0);
            du = (u_max - u) / (15.0 - (double)i);
        } else {
            nn = std::round(nn);
        }
        cdf[3 * i] = nn;
    }
    for (int i = 0; i < 16; ++i) {
        size_t index = (size_t)rust_as_i32(cdf[3 * i]) - (size_t)n_min;
        const C2& c = index < cum.size() ? cum[index] : cum.back();
        cdf[3 * i + 1] = c.re;
        cdf[3 * i + 2] = c.im;
    }
}

// DoubleDiffPartialRate::at, for tests of the regenerated tables
void lp_pair_dd_rate(int n, double a, double eta, double s, double theta, double out[2]) {
    LppRate r(n, a, eta);
    r.at(s, theta, out);
}


// pair_creation/mod.rs:21-42 (CP only: LP added with its sampler)
bool bw_probability(const V4& ell, const Stokes& sv_in, const V4& k, double a, double dt, int pol, double pol_angle,
                    double* prob, Stokes* sv_out) {
    double eta = k * ell;
    Stokes sv = sv_in.in_lma_basis(ell).rotate_by(pol_angle);
    double dphi = eta * dt / (COMPTON_TIME * ell.t);
    double f[2];
    Stokes out;
    if (pol == PTG_POL_CIRCULAR) {
        if (!cp_pair_rates(a, eta, f)) return false;
        *prob = cpp_probability(f, eta, sv, dphi, &out);
    } else {
        if (!lp_pair_rates(a * SQRT_2, eta, f)) return false;
        *prob = lpp_probability(f, eta, sv, dphi, &out);
    }
    *sv_out = out.rotate_by(-pol_angle).from_lma_basis(ell);
    return true;
}

// pair_creation/mod.rs:49-110
int bw_generate(const V4& ell, const Stokes& sv_in, const V4& k, double a, int pol, double pol_angle, DrawStream& rng,
                int* n_out, V4* q_out, uint64_t* rej) {
    double eta = k * ell;
    Stokes sv = sv_in.in_lma_basis(ell).rotate_by(pol_angle);
    int n;
    double s, cphi;
    int st = pol == PTG_POL_CIRCULAR ? cpp_sample(a, eta, sv.q, sv.u, sv.v, rng, &n, &s, &cphi, rej)
                                     : lp_pair_sample(a * SQRT_2, eta, sv.q, sv.u, rng, &n, &s, &cphi, rej);
    if (st != PTG_OK) return st;
    double j = n;
    double e_zmf = std::sqrt(0.5 * j * eta);
    double p_zmf = std::sqrt(0.5 * j * eta - 1.0 - a * a);
    double ct = (1.0 - 2.0 * s) * e_zmf / p_zmf;
    if (!(ct <= 1.0 && ct >= -1.0)) return PTG_ERR_SANITY;
    V4 t = ell + j * k;
    V4 u_zmf = t / std::sqrt(t * t);
    V3 along = -((j * k).boost_by(u_zmf).spatial().normalize());
    V4 e4(0.0, std::cos(pol_angle), std::sin(pol_angle), 0.0);
    V3 eps = e4.boost_by(u_zmf).spatial().normalize();
    eps = along.cross(eps.cross(along)).normalize();
    V3 perp = eps.rotate_around(along, cphi);
    V3 q3 = p_zmf * (ct * along + std::sqrt(1.0 - ct * ct) * perp);
    V4 q(std::sqrt(1.0 + a * a + q3.x * q3.x + q3.y * q3.y + q3.z * q3.z), q3.x, q3.y, q3.z);
    q = q.boost_by(V4(u_zmf.t, -u_zmf.x, -u_zmf.y, -u_zmf.z));
    double s_new = 1.0 - (k * q) / (k * ell);
    if (!(std::fabs(s - s_new) / s < 1.0e-3)) return PTG_ERR_SANITY;
    *n_out = n;
    *q_out = q;
    return PTG_OK;
}

// plane_wave.rs:284-316 / focused_laser.rs:283-306
int lma_pair_create(const Laser& L, const V4& r, const V4& ell, const Stokes& pol, double dt, DrawStream& rng,
                    double rate_increase, double* prob, Stokes* pol_new, bool* created, PairEvent* ev, uint64_t* rej) {
    *created = false;
    *prob = 0.0;
    *pol_new = pol;
    double a = std::sqrt(L.a_sqd(r));
    double chirp = 1.0;
    if (L.d.model == PTG_PLANE_WAVE) {
        chirp = 1.0 + 2.0 * L.d.chirp_b * (L.wavevector * r);
        if (chirp < 0.0 && a > 0.0) return PTG_ERR_SANITY;
    }
    V4 kappa = (SPEED_OF_LIGHT * COMPTON_TIME * chirp) * L.wavevector;
    if (!bw_probability(ell, pol, kappa, a, dt, L.d.polarization, L.d.pol_angle, prob, pol_new))
        return PTG_ERR_OUT_OF_TABLE;
    double ri = (*prob * rate_increase > 0.1) ? 0.1 / *prob : rate_increase;
    if (rng.next() < *prob * ri) {
        int n;
        V4 q;
        int st = bw_generate(ell, pol, kappa, a, L.d.polarization, L.d.pol_angle, rng, &n, &q, rej);
        if (st != PTG_OK) return st;
        ev->u_e = ell + (double)n * kappa - q;
        ev->u_p = q;
        ev->frac = 1.0 / ri;
        ev->a_eff = a;
        ev->chi = a * (ell * kappa);
        ev->absorption = (double)n * kappa.t;
        *created = true;
    }
    return PTG_OK;
}

}  // namespace orc
