// Nonlinear Compton scattering in a linearly polarised background (LMA):
// the generalised Bessel function J(n, x, y), the double-differential rate
// in (s, theta), its rejection ceiling, the harmonic index from the CDF
// table, and the sampler with the emitted photon's Stokes parameters.
//
// J(n, x, y) follows special_functions/double_bessel.rs: a forward
// recurrence (five coefficients per order, kept in a per-lane workspace in
// global memory), a backward recurrence for the two solutions f and g with
// rescaling, and normalisation over all orders.  Here the backward pass
// accumulates the normalisation sums as it goes instead of storing f, g and
// h, so only the five forward coefficients need memory: 40 bytes per order,
// about 3.83 n + 200 orders.  The workspace is lane-interleaved (element e,
// coefficient c of a lane at base[(5 e + c) * 32]) so that a warp's
// accesses coalesce.
#pragma once
#include "ptg_math.cuh"
#include "ptg_nlc.cuh"

namespace ptg {

// ---------------------------------------------------------- complex -----
// Complex arithmetic with the semantics of num-complex 0.4 (products by the
// full formula, sqrt exact on the axes, ln and exp through polar form,
// acos(z) = -i ln(i sqrt(1 - z^2) + z)); signed zeros pick the branch of
// sqrt and hence of acos for real z > 1.
struct cxd {
    double re, im;
};
__host__ __device__ __forceinline__ cxd cx_mul(cxd a, cxd b) { return cxd{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__host__ __device__ __forceinline__ cxd cx_add(cxd a, cxd b) { return cxd{a.re + b.re, a.im + b.im}; }
__host__ __device__ __forceinline__ cxd cx_sub(cxd a, cxd b) { return cxd{a.re - b.re, a.im - b.im}; }
__host__ __device__ __forceinline__ cxd cx_scale(double s, cxd a) { return cxd{s * a.re, s * a.im}; }
__host__ __device__ __forceinline__ double cx_norm(cxd a) { return hypot(a.re, a.im); }
__host__ __device__ __forceinline__ double cx_arg(cxd a) { return atan2(a.im, a.re); }
__host__ __device__ __forceinline__ cxd cx_from_polar(double r, double t) { return cxd{r * cos(t), r * sin(t)}; }
__host__ __device__ __forceinline__ cxd cx_ln(cxd a) { return cxd{log(cx_norm(a)), cx_arg(a)}; }
__host__ __device__ __forceinline__ cxd cx_exp(cxd a) { return cx_from_polar(exp(a.re), a.im); }
__host__ __device__ __forceinline__ cxd cx_sin(cxd a) { return cxd{sin(a.re) * cosh(a.im), cos(a.re) * sinh(a.im)}; }
__host__ __device__ __forceinline__ cxd cx_sqrt(cxd a) {
    if (a.im == 0.0) {
        if (!signbit(a.re)) return cxd{sqrt(a.re), a.im};
        double im = sqrt(-a.re);
        return signbit(a.im) ? cxd{0.0, -im} : cxd{0.0, im};
    }
    if (a.re == 0.0) {
        double x = sqrt(fabs(a.im) / 2.0);
        return signbit(a.im) ? cxd{x, -x} : cxd{x, x};
    }
    return cx_from_polar(sqrt(cx_norm(a)), cx_arg(a) / 2.0);
}
__host__ __device__ __forceinline__ cxd cx_acos(cxd z) {
    const cxd I{0.0, 1.0}, ONE{1.0, 0.0}, NEG_I{-0.0, -1.0};
    return cx_mul(NEG_I, cx_ln(cx_add(cx_mul(cx_sqrt(cx_sub(ONE, cx_mul(z, z))), I), z)));
}

// ----------------------------------------------------- DoubleBessel -----
// A pool of large workspaces shared by all lanes, for harmonic orders
// beyond a lane's own slot (pair creation at small eta).  Slot k holds
// `cap` orders at base + k * cap * 5; state[k] is 0 (free) or 1 (taken).
struct DbPool {
    double* base;
    unsigned* state;
    int cap, slots;
};

struct DbWork {
    double* base;  // coefficient c of order e at base[(5 e + c) * stride]
    int cap;       // orders the slot holds
    int stride;    // 32 for a lane-interleaved warp slot, 1 for a pooled slot
    DbPool pool;   // larger slots for orders beyond `cap` (may be empty)
};

// Takes a free pool slot (bounded wait: slots are held only for the
// duration of one sample).  Returns -1 if none freed up in time.
__device__ __forceinline__ int db_pool_acquire(const DbPool& p, unsigned hint) {
    if (!p.base || p.slots <= 0) return -1;
    for (int it = 0; it < (1 << 16); ++it) {
        for (int q = 0; q < p.slots; ++q) {
            int k = (int)((hint + (unsigned)q) % (unsigned)p.slots);
            if (atomicCAS(p.state + k, 0u, 1u) == 0u) {
                __threadfence();
                return k;
            }
        }
        __nanosleep(2000);
    }
    return -1;
}

__device__ __forceinline__ void db_pool_release(const DbPool& p, int k) {
    __threadfence();
    atomicExch(p.state + k, 0u);
}

struct DbGeom {
    int n, k_min, len;
};

// double_bessel.rs:39-83 (DoubleBessel::at_index with x_max = n sqrt 2,
// y_max = n / 2).  Returns false if the workspace is too small.
__host__ __device__ __forceinline__ bool db_geom(int n, int cap, DbGeom* g) {
    double xm = n * SQRT_2, ym = n * 0.5;
    int nmb = (int)floor(-2.0 * ym - xm);
    int npb = xm > 4.0 * (2.0 - SQRT_2) * ym ? (int)ceil(xm) : (int)ceil(2.0 * ym + xm * xm / (16.0 * ym));
    g->n = n;
    g->len = npb - nmb + 200;
    g->k_min = nmb - 100;
    return g->len <= cap;
}

// Scaled sum of squares: value = scale * sqrt(ssq), overflow-safe.
struct Ssq {
    double scale, ssq;
    __host__ __device__ __forceinline__ void add(double x) {
        double ax = fabs(x);
        if (ax == 0.0 || !(ax == ax)) {
            if (!(ax == ax)) ssq = ax;
            return;
        }
        if (ax > scale) {
            double r = scale / ax;
            ssq = 1.0 + ssq * r * r;
            scale = ax;
        } else {
            double r = ax / scale;
            ssq += r * r;
        }
    }
    __host__ __device__ __forceinline__ double value() const { return scale * sqrt(ssq); }
};

// double_bessel.rs:142-246: J(n-2..n+2, x, y) by recurrence.  Returns false
// on a workspace too small for n.
static __host__ __device__ __noinline__ bool db_around(const DbGeom& g, const DbWork& w, double x, double y, double j[5]) {
    const int len = g.len;
    double* W = w.base;
    const size_t stride = (size_t)w.stride;
#define DBW(e, c) W[((size_t)(e) * 5 + (c)) * stride]
    // forward recurrence from the default element (all coefficients 1)
    {
        double p0 = 1.0, p1 = 1.0, p2 = 1.0, q0 = 1.0, q1 = 1.0;
        for (int i = 1; i < len; ++i) {
            int k = i + g.k_min;
            double x0 = -x - 4.0 * y * y / p2;
            double x1 = 2.0 * (double)(k - 1) - 2.0 * y * p0 / p2;
            double x2 = -x - 2.0 * y * p1 / p2;
            double l0 = x0 - 2.0 * y * x2 / q1;
            double l1 = x1 - q0 * x2 / q1;
            DBW(i, 0) = x0;
            DBW(i, 1) = x1;
            DBW(i, 2) = x2;
            DBW(i, 3) = l0;
            DBW(i, 4) = l1;
            p0 = x0, p1 = x1, p2 = x2, q0 = l0, q1 = l1;
        }
    }
    int n_minus = (int)floor(-2.0 * y - x);
    int n_plus = (8.0 * y > x) ? (int)ceil(2.0 * y + x * x / (16.0 * y)) : (int)ceil(-2.0 * y + x);
    int i_match = (n_plus + n_minus) / 2 - g.k_min;
    int i_target = g.n - g.k_min;
    if (i_match < 1 || i_match > len - 4 || i_target < 2 || i_target + 2 > len - 4) return false;
    const double initial = g.n < 2000 ? 1.0e-100 : 1.0e-300;
    // window: f[i+1], f[i+2], f[i+3]; g[i+1], g[i+2]
    double f1 = 2.0 * initial, f2 = 1.0 * initial, f3 = 0.0;
    double g2 = 1.0 / initial;
    double g1 = -(2.0 * y * 0.0 + DBW(len - 2, 3) * g2) / DBW(len - 2, 4);
    // sums over the f branch (orders >= i_match) and the g branch (< i_match)
    double sum_f = f3 + f2 + f1, sum_g = 0.0;
    Ssq sq_f{0.0, 1.0}, sq_g{0.0, 1.0};
    sq_f.add(f3);
    sq_f.add(f2);
    sq_f.add(f1);
    double g_match = 0.0, f_match = 0.0;
    double tv[5] = {0.0, 0.0, 0.0, 0.0, 0.0};  // f or g at the five target orders
    for (int i = len - 4; i >= 0; --i) {
        double fi = -(2.0 * y * f3 + DBW(i + 2, 0) * f2 + DBW(i + 2, 1) * f1) / DBW(i + 2, 2);
        double gi = -(2.0 * y * g2 + DBW(i + 1, 3) * g1) / DBW(i + 1, 4);
        if (i >= i_match) {
            sum_f += fi;
            sq_f.add(fi);
        } else {
            sum_g += gi;
            sq_g.add(gi);
        }
        if (i == i_match) {
            g_match = gi;
            f_match = fi;
        }
        int t = i - (i_target - 2);
        if (t >= 0 && t < 5) tv[t] = i >= i_match ? fi : gi;
        double gm_now = i > i_match ? 0.0 : g_match;
        if (fi > 1.0 && fabs(gm_now) < 1.0e200) {
            // every order >= i: f *= 1e-100, g *= 1e100
            fi *= 1.0e-100, f1 *= 1.0e-100, f2 *= 1.0e-100;
            gi *= 1.0e100, g1 *= 1.0e100;
            sum_f *= 1.0e-100;
            sq_f.scale *= 1.0e-100;
            sum_g *= 1.0e100;
            sq_g.scale *= 1.0e100;
            if (i <= i_match) {
                g_match *= 1.0e100;
                f_match *= 1.0e-100;
            }
            for (int q = 0; q < 5; ++q) {
                int e = i_target - 2 + q;
                if (e >= i) tv[q] *= (e >= i_match) ? 1.0e-100 : 1.0e100;
            }
        }
        f3 = f2, f2 = f1, f1 = fi;
        g2 = g1, g1 = gi;
    }
#undef DBW
    // g_match / f_match alone can overflow; sum_f / f_match and the f-branch
    // norm over |f_match| stay near 1 (f peaks at the matching order)
    double sum_linear = sum_g + g_match * (sum_f / f_match);
    double rss = hypot(sq_g.value(), fabs(g_match) * (sq_f.value() / fabs(f_match)));
    for (int q = 0; q < 5; ++q) {
        int e = i_target - 2 + q;
        double h = e < i_match ? tv[q] : g_match * tv[q] / f_match;
        double r = h / sum_linear;
        double sgn = r > 0.0 ? 1.0 : (r < 0.0 ? -1.0 : (signbit(r) ? -1.0 : 1.0));
        double val = sgn * fabs(h) / rss;
        j[q] = isfinite(val) ? val : 0.0;
    }
    return true;
}

// double_bessel.rs:272-355: saddle-point approximation for large order.
static __host__ __device__ __noinline__ double db_spa(int ni, double x, double y) {
    double n = ni;
    if (n <= -2.0 * y + x) {
        double ct = y > 0.0 ? x / (8.0 * y) - sqrt(x * x / (64.0 * y * y) + 0.5 - n / (4.0 * y)) : n / x;
        double th = acos(ct);
        double f = x * sin(th) - y * sin(2.0 * th);
        double d2f = -x * sin(th) + 4.0 * y * sin(2.0 * th);
        double phi = (PI / 4.0) * (d2f > 0.0 ? 1.0 : (d2f < 0.0 ? -1.0 : (signbit(d2f) ? -1.0 : 1.0)));
        return cos(f - n * th + phi) * sqrt(2.0 / (PI * fabs(d2f)));
    } else if (8.0 * y < x || n > 2.0 * y + x * x / (16.0 * y)) {
        double disc = x * x / (64.0 * y * y) + 0.5 - n / (4.0 * y);
        cxd ct;
        if (isnan(disc))
            ct = cxd{n / x, 0.0};
        else if (disc < 0.0)
            ct = cxd{x / (8.0 * y), sqrt(-disc)};
        else
            ct = cxd{x / (8.0 * y) - sqrt(disc), 0.0};
        const cxd I{0.0, 1.0};
        cxd th = cx_acos(ct);
        cxd s1 = cx_sin(th), s2 = cx_sin(cx_scale(2.0, th));
        cxd f = cx_mul(I, cx_sub(cx_add(cx_scale(-n, th), cx_scale(x, s1)), cx_scale(y, s2)));
        cxd d2f = cx_mul(I, cx_add(cx_scale(-x, s1), cx_scale(4.0 * y, s2)));
        cxd phase = cx_add(f, cxd{0.0, (PI - cx_arg(d2f)) / 2.0});
        double term;
        if (f.im == 0.0 && d2f.im == 0.0)
            term = 0.5 * exp(-f.re) * sqrt(2.0 / (PI * cx_norm(d2f)));
        else
            term = cx_exp(phase).re * sqrt(2.0 / (PI * cx_norm(d2f)));
        return disc != 0.0 ? term : 0.0;
    } else {
        double r = sqrt(x * x / (64.0 * y * y) + 0.5 - n / (4.0 * y));
        double out = 0.0;
        for (int b = 0; b < 2; ++b) {
            double ct = x / (8.0 * y) + (b == 0 ? -r : r);
            double th = acos(ct);
            double f = x * sin(th) - y * sin(2.0 * th);
            double d2f = -x * sin(th) + 4.0 * y * sin(2.0 * th);
            double phi = (PI / 4.0) * (d2f > 0.0 ? 1.0 : (d2f < 0.0 ? -1.0 : (signbit(d2f) ? -1.0 : 1.0)));
            out += cos(f - n * th + phi) * sqrt(2.0 / (PI * fabs(d2f)));
        }
        return out;
    }
}

// double_bessel.rs:386-410
__host__ __device__ __forceinline__ bool db_evaluate(const DbGeom& g, const DbWork& w, double x, double y, double j[5]) {
    if (g.n > 10) {
        double ne = g.n * (1.0 - sqrt(10.0 / g.n));
        double xc = y > ne / 6.0 ? 4.0 * sqrt(y * (ne - 2.0 * y)) : ne + 2.0 * y;
        if (x < xc) {
            for (int q = 0; q < 5; ++q) j[q] = db_spa(g.n - 2 + q, x, y);
            return true;
        }
    }
    return db_around(g, w, x, y, j);
}

// ------------------------------------------------------ LP emission -----
// nonlinear_compton/lp/mod.rs:21-50.  Returns NaN on a workspace failure.
static __device__ __noinline__ double lp_ddpr(double a, double eta, double s, double theta, const DbGeom& g, const DbWork& w) {
    int n = g.n;
    double sn = 2.0 * n * eta / (1.0 + 0.5 * a * a);
    double wn = fmin(s / (sn * (1.0 - s)), 1.0);
    double alpha = 2.0 * n * a * cos(theta) * sqrt(wn * (1.0 - wn)) / sqrt(1.0 + 0.5 * a * a);
    double beta = a * a * s / (8.0 * eta * (1.0 - s));
    double j[5];
    if (!db_evaluate(g, w, alpha, beta, j)) return NAN;
    double g0, g1, g2;
    if (n % 2 == 0) {
        g0 = j[2], g1 = -0.5 * (j[1] + j[3]), g2 = 0.25 * (j[0] + 2.0 * j[2] + j[4]);
    } else {
        g0 = -j[2], g1 = 0.5 * (j[1] + j[3]), g2 = -0.25 * (j[0] + 2.0 * j[2] + j[4]);
    }
    return (-g0 * g0 - a * a * (1.0 + 0.5 * s * s / (1.0 - s)) * (g0 * g2 - g1 * g1)) / (2.0 * PI);
}

// f64::max, which ignores a NaN operand
__device__ __forceinline__ double rmax(double a, double b) { return isnan(a) ? b : (isnan(b) ? a : fmax(a, b)); }

// nonlinear_compton/lp/mod.rs:338-344
__device__ __forceinline__ int lp_sum_limit(double a, double eta) {
    double m = 3.0 - 0.4 * pow(eta, 0.25);
    return (int)ceil(6.0 * (1.0 + a * a) + 2.0 * pow(a, m));
}

// nonlinear_compton/lp/mod.rs:53-140: the points (s, theta) at which the
// ceiling scans the rate, as a plan the scan walks point by point (a lane
// each in the cooperative sampler).
struct LpCeilPlan {
    double smax, theta, x0, x1;
    int i0, cnt, mode;  // mode 4: n = 1 (two points)
};

__device__ __forceinline__ void lp_ceiling_plan(double a, double eta, int n, LpCeilPlan* p) {
    double sn = 2.0 * n * eta / (1.0 + 0.5 * a * a);
    p->smax = sn / (1.0 + sn);
    p->theta = 0.0, p->x0 = 0.0, p->x1 = 1.0;
    p->i0 = 1, p->cnt = 32;
    if (n == 1) {
        p->mode = 4;
    } else if (a <= 2.0) {
        p->mode = 0;
    } else if (a <= 5.0) {
        int n_switch = (int)ceil(1.3 * pow(a, 1.2));
        if (n < n_switch) {
            p->theta = (PI / 2.0) * (1.0 - log((double)n) / log((double)n_switch));
            p->i0 = 0;
            p->mode = 2;
        } else {
            p->x0 = fmax(4.0 * n * eta / (3.0 * a * a + 4.0 * n * eta), 0.4);
            p->cnt = n < lp_sum_limit(a, eta) / 2 ? 32 : 64;
            p->mode = 3;
        }
    } else {
        int n_switch = (int)ceil(a * a);
        if (n < n_switch) {
            double ns = n_switch;
            p->theta = (PI / 2.0) * (pow((double)n, -0.7) - pow(ns, -0.7)) / (1.0 - pow(ns, -0.7));
            p->cnt = 64;
            p->mode = 1;
        } else {
            p->x0 = fmax(4.0 * n * eta / (3.0 * a * a + 4.0 * n * eta), 0.3);
            p->x1 = (1.0 + sn) / (2.0 + sn);
            p->cnt = n > 10 * n_switch ? 64 : (n > 3 * n_switch ? 42 : 32);
            p->mode = 3;
        }
    }
}

__device__ __forceinline__ int lp_ceiling_points(const LpCeilPlan& p) { return p.mode == 4 ? 2 : p.cnt - p.i0 + 1; }

// Point k of the scan (k < lp_ceiling_points).
__device__ __forceinline__ void lp_ceiling_point(const LpCeilPlan& p, int k, double* s, double* theta) {
    if (p.mode == 4) {
        *s = (k == 0 ? 0.01 : 0.99) * p.smax;
        *theta = PI / 2.0;
        return;
    }
    int i = p.i0 + k;
    *theta = p.theta;
    if (p.mode == 0)
        *s = p.smax * (0.4 + 0.6 * (double)i / 32.0);
    else if (p.mode == 1)
        *s = p.smax * (0.3 + 0.7 * (double)i / 64.0);
    else if (p.mode == 2)
        *s = p.smax * (double)i / 32.0;
    else
        *s = p.smax * (p.x0 + (p.x1 - p.x0) * (double)i / (double)p.cnt);
}

// The ceiling: 1.15 x the largest rate over the plan's points (NaN-ignoring).
static __device__ __noinline__ double lp_ceiling(double a, double eta, const DbGeom& g, const DbWork& w) {
    LpCeilPlan p;
    lp_ceiling_plan(a, eta, g.n, &p);
    double mx = NAN;
    for (int k = 0, np = lp_ceiling_points(p); k < np; ++k) {
        double s, theta;
        lp_ceiling_point(p, k, &s, &theta);
        mx = rmax(mx, lp_ddpr(a, eta, s, theta, g, w));
    }
    return 1.15 * mx;
}

// nonlinear_compton/lp/mod.rs:142-302
struct ThetaBound {
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

static __device__ __noinline__ double ln_double_bessel_x_zero(int ni, double y) {
    double n = ni;
    double z = sqrt(n / (4.0 * y) - 0.5);
    const cxd I{0.0, 1.0};
    cxd theta{PI / 2.0, log(sqrt(1.0 + z * z) - z)};
    cxd s2 = cx_sin(cx_scale(2.0, theta));
    cxd f = cx_mul(I, cx_sub(cx_scale(-n, theta), cx_scale(y, s2)));
    cxd f2 = cx_mul(I, cx_scale(4.0 * y, s2));
    double e = 0.5 * (PI - cx_arg(f2));
    cxd phase = cx_add(f, cx_mul(I, cxd{e, 0.0}));
    return log(sqrt(2.0 / (PI * cx_norm(f2)))) + phase.re + log(fabs(cos(phase.im)));
}

// Point i of the 16-point bound on theta as a function of s.
__device__ __forceinline__ void theta_bound_point(int n, double a, double eta, int i, double* s_i, double* f_i) {
    double sn = 2.0 * n * eta / (1.0 + 0.5 * a * a);
    double z = cos(PI * i / 15.0);
    double si = 0.5 * (z + 1.0) * sn / (1.0 + sn);
    *s_i = si;
    double wn = fmin(si / (sn * (1.0 - si)), 1.0);
    double x = 2.0 * n * a * sqrt(wn * (1.0 - wn)) / sqrt(1.0 + 0.5 * a * a);
    double y = a * a * si / (8.0 * eta * (1.0 - si));
    double x_crit = y > n / 6.0 ? 4.0 * sqrt(y) * sqrt(n - 2.0 * y) : n + 2.0 * y;
    double ln_j_crit = log(0.443) - log((double)n) / 3.0;
    double ln_j_bdy = ln_double_bessel_x_zero(n % 2 == 0 ? n : n + 1, y);
    ln_j_bdy = fmin(ln_j_bdy, ln_j_crit);
    double ct = 1.0 - x_crit * log(0.01) / (x * (ln_j_bdy - ln_j_crit));
    ct = fmax(ct, -1.0);
    double fi = acos(ct);
    *f_i = isnan(fi) ? PI : fi;
}

// The bound made non-increasing in s (the points run from s_max down).
__device__ __forceinline__ void theta_bound_finish(ThetaBound* tb) {
    double f_min = tb->f[0];
    for (int i = 1; i < 16; ++i) {
        if (tb->f[i] < f_min)
            f_min = tb->f[i];
        else
            tb->f[i] = f_min;
    }
}

static __device__ __noinline__ void theta_bound(int n, double a, double eta, ThetaBound* tb) {
    for (int i = 0; i < 16; ++i) theta_bound_point(n, a, eta, i, &tb->s[i], &tb->f[i]);
    theta_bound_finish(tb);
}

// nonlinear_compton/lp/linear.rs
__device__ __forceinline__ double lp_linear_rate(double a, double eta) {
    double eta2 = eta * eta, eta3 = eta2 * eta;
    if (eta > 1.0e-3)
        return (a * a / 8.0) * (0.5 + 4.0 / eta - 0.5 / ((1.0 + 2.0 * eta) * (1.0 + 2.0 * eta)) +
                                (1.0 - 2.0 / eta - 2.0 / eta2) * log(1.0 + 2.0 * eta));
    return (a * a / 8.0) * (8.0 * eta / 3.0 - 16.0 * eta2 / 3.0 + 208.0 * eta3 / 15.0);
}

// nonlinear_compton/lp/classical.rs:189-210
__device__ __forceinline__ bool lp_classical_rate(const NlcTables& t, double a, double eta, double* out) {
    double x = log(a);
    if (x < PTG_NLC_CL_MIN) {
        *out = a * a * eta / 3.0;
        return true;
    }
    int ix = (int)((x - PTG_NLC_CL_MIN) / PTG_NLC_CL_STEP);
    if (ix >= 60) return false;
    double dx = (x - PTG_NLC_CL_MIN) / PTG_NLC_CL_STEP - ix;
    double f = (1.0 - dx) * t.lp_cl_rate[ix] + dx * t.lp_cl_rate[ix + 1];
    double prefactor = 2.0 * eta / (1.0 + 0.5 * a * a);
    *out = prefactor * exp(f);
    return true;
}

// nonlinear_compton/lp/mod.rs:414-457
__device__ __forceinline__ bool lp_rate(const NlcTables& t, double a, double eta, double* out) {
    const double MIN0 = PTG_NLC_LP_MIN_0, MIN1 = PTG_NLC_LP_MIN_1, S0 = PTG_NLC_LP_STEP_0, S1 = PTG_NLC_LP_STEP_1;
    const double* T = t.lp_rate;
    double x = log(a), y = log(eta);
    if (x < MIN0) {
        *out = lp_linear_rate(a, eta);
        return true;
    }
    int ix = (int)((x - MIN0) / S0);
    double dx = (x - MIN0) / S0 - ix;
    if (ix >= 60) return false;
    if (y < MIN1) {
        *out = exp((1.0 - dx) * T[ix] + dx * T[ix + 1] - MIN1) * eta;
        return true;
    }
    int iy = (int)((y - MIN1) / S1);
    if (iy >= 67) return false;
    double dy = (y - MIN1) / S1 - iy;
    double f = (1.0 - dx) * (1.0 - dy) * T[iy * 61 + ix] + dx * (1.0 - dy) * T[iy * 61 + ix + 1] +
               (1.0 - dx) * dy * T[(iy + 1) * 61 + ix] + dx * dy * T[(iy + 1) * 61 + ix + 1];
    *out = exp(f);
    return true;
}

// lp_rate's table branch in FP32, where it certainly applies (peak
// amplitude a, strictly inside the table); false elsewhere.  T32: the LP
// ln-rate table in FP32; ln_a: ln a in FP32 (NaN or -inf where a is not
// positive).
__device__ __forceinline__ bool rate32_lp(const float* T32, float ln_a, double eta, float* out) {
    if (T32 == nullptr || !(eta > 0.0)) return false;
    const float MIN0 = (float)PTG_NLC_LP_MIN_0, MIN1 = (float)PTG_NLC_LP_MIN_1;
    const float I0 = (float)(1.0 / PTG_NLC_LP_STEP_0), I1 = (float)(1.0 / PTG_NLC_LP_STEP_1);
    float ta = (ln_a - MIN0) * I0, te = (logf((float)eta) - MIN1) * I1;
    if (!(ta > 1e-3f && te > 1e-3f && ta < 59.99f && te < 66.99f)) return false;
    int ia = (int)ta, ie = (int)te;
    float da = ta - (float)ia, de = te - (float)ie;
    const float* p = T32 + ie * 61 + ia;
    float f = (1.0f - da) * (1.0f - de) * p[0] + da * (1.0f - de) * p[1] + (1.0f - da) * de * p[61] + da * de * p[62];
    *out = expf(f);
    return true;
}

// nonlinear_compton/lp/mod.rs:459-553: one grid corner of the harmonic CDF
// (16 nodes of [n, cdf]); NaN where the reference's inversion would fail.
static __device__ __noinline__ double lp_cdf_corner(const double* table, double frac, double a) {
    if (frac <= table[1]) return 0.9;
    double v = 0.0;
    if (a < 5.0) return pw_invert(table, 16, false, frac, &v) ? v : NAN;
    double rs[30];
    for (int i = 0; i < 15; ++i) {
        rs[2 * i] = log(table[2 * i]);
        rs[2 * i + 1] = log(-1.0 * log(1.0 - table[2 * i + 1]));
    }
    pw_invert(rs, 15, true, log(-1.0 * log(1.0 - frac)), &v);
    return exp(v);
}

// Returns the harmonic order, or -1 if the lookup failed.
static __device__ __noinline__ int lp_harmonic_index(const NlcTables& t, double a, double eta, double frac) {
    const double MIN0 = PTG_NLC_LP_CDF_MIN_0, MIN1 = PTG_NLC_LP_CDF_MIN_1, S0 = PTG_NLC_LP_CDF_STEP_0,
                 S1 = PTG_NLC_LP_CDF_STEP_1;
    const double* T = t.lp_cdf;
    double la = log(a), le = log(eta);
    if (la <= MIN0) return 1;
    int ix = (int)((la - MIN0) / S0);
    double dx = (la - MIN0) / S0 - ix;
    if (ix >= 60) return -1;
    double n;
    if (le <= MIN1) {
        n = lp_cdf_corner(T + (size_t)ix * 32, frac, a) * (1.0 - dx) +
            lp_cdf_corner(T + (size_t)(ix + 1) * 32, frac, a) * dx;
    } else {
        int iy = (int)((le - MIN1) / S1);
        if ((size_t)(61 * (iy + 1) + ix + 1) >= 4148) return -1;
        double dy = (le - MIN1) / S1 - iy;
        n = lp_cdf_corner(T + (size_t)(61 * iy + ix) * 32, frac, a) * ((1.0 - dx) * (1.0 - dy)) +
            lp_cdf_corner(T + (size_t)(61 * iy + ix + 1) * 32, frac, a) * (dx * (1.0 - dy)) +
            lp_cdf_corner(T + (size_t)(61 * (iy + 1) + ix) * 32, frac, a) * ((1.0 - dx) * dy) +
            lp_cdf_corner(T + (size_t)(61 * (iy + 1) + ix + 1) * 32, frac, a) * (dx * dy);
    }
    return isfinite(n) ? (int)ceil(n) : -1;
}

// lp_harmonic_index by a converged warp: the (up to) four grid corners
// are inverted on lanes 0-3 at once and combined in lp_harmonic_index's
// order and expression, so every lane returns its harmonic (or -1).
static __device__ __noinline__ int lp_harmonic_index_warp(const NlcTables& t, double a, double eta, double frac) {
    const unsigned all = 0xffffffffu;
    const int lane = (int)(threadIdx.x & 31u);
    const double MIN0 = PTG_NLC_LP_CDF_MIN_0, MIN1 = PTG_NLC_LP_CDF_MIN_1, S0 = PTG_NLC_LP_CDF_STEP_0,
                 S1 = PTG_NLC_LP_CDF_STEP_1;
    const double* T = t.lp_cdf;
    double la = log(a), le = log(eta);
    if (la <= MIN0) return 1;
    int ix = (int)((la - MIN0) / S0);
    double dx = (la - MIN0) / S0 - ix;
    if (ix >= 60) return -1;
    bool edge = le <= MIN1;
    int iy = edge ? 0 : (int)((le - MIN1) / S1);
    if (!edge && (size_t)(61 * (iy + 1) + ix + 1) >= 4148) return -1;
    double dy = edge ? 0.0 : (le - MIN1) / S1 - iy;
    double v = 0.0;
    if (lane < (edge ? 2 : 4)) {
        size_t row = edge ? (size_t)(ix + lane) : (size_t)(61 * (iy + (lane >> 1)) + ix + (lane & 1));
        v = lp_cdf_corner(T + row * 32, frac, a);
    }
    double c0 = __shfl_sync(all, v, 0), c1 = __shfl_sync(all, v, 1);
    double n;
    if (edge) {
        n = c0 * (1.0 - dx) + c1 * dx;
    } else {
        double c2 = __shfl_sync(all, v, 2), c3 = __shfl_sync(all, v, 3);
        n = c0 * ((1.0 - dx) * (1.0 - dy)) + c1 * (dx * (1.0 - dy)) + c2 * ((1.0 - dx) * dy) + c3 * (dx * dy);
    }
    return isfinite(n) ? (int)ceil(n) : -1;
}

static __device__ __noinline__ int lp_sample_n(const NlcTables& t, const DbWork& w, const DbGeom& g, double a,
                                               double eta, Draws& rng, int* n_out, double* s_out, double* theta_out,
                                               d3* sv_out, uint32_t* rej);

// The workspace for harmonic n: the lane's own slot, or a pooled one
// (returned in *slot, to release) when n needs more orders.
__device__ __forceinline__ int db_take(const DbWork& w, int n, DbWork* wk, DbGeom* g, int* slot) {
    *slot = -1;
    if (db_geom(n, w.cap, g)) {
        *wk = w;
        return 0;
    }
    int k = db_pool_acquire(w.pool, (unsigned)(blockIdx.x * 131u + threadIdx.x));
    if (k < 0) return w.pool.slots > 0 ? 11 : 9;  // PTG_ERR_TIMEOUT / PTG_ERR_UNSUPPORTED
    *wk = DbWork{w.pool.base + (size_t)k * w.pool.cap * 5, w.pool.cap, 1, w.pool};
    if (!db_geom(n, w.pool.cap, g)) {
        db_pool_release(w.pool, k);
        return 9;
    }
    *slot = k;
    return 0;
}

// nonlinear_compton/lp/mod.rs:586-676: harmonic, s, azimuth theta in
// [0, 2 pi) and the Stokes vector (in the LMA basis) of the emitted photon.
// Returns a ptg status.
static __device__ __noinline__ int lp_sample(const NlcTables& t, const DbWork& w, double a, double eta, Draws& rng,
                                      int* n_out, double* s_out, double* theta_out, d3* sv_out, uint32_t* rej) {
    if (t.lp_cdf == nullptr || w.base == nullptr) return 8;  // PTG_ERR_TABLES
    int n = lp_harmonic_index(t, a, eta, rng.next());
    if (n < 1) return 2;  // PTG_ERR_OUT_OF_TABLE
    DbWork wk;
    int slot = -1;
    DbGeom g;
    int st = db_take(w, n, &wk, &g, &slot);
    if (st != 0) return st;
    st = lp_sample_n(t, wk, g, a, eta, rng, n_out, s_out, theta_out, sv_out, rej);
    if (slot >= 0) db_pool_release(w.pool, slot);
    return st;
}

static __device__ __noinline__ int lp_finish(int n, double a, double eta, double s, double theta, const DbGeom& g,
                                             const DbWork& w, Draws& rng, int* n_out, double* s_out, double* theta_out,
                                             d3* sv_out);

// lp_sample for a harmonic whose J(n, x, y) workspace is ready.
static __device__ __noinline__ int lp_sample_n(const NlcTables& t, const DbWork& w, const DbGeom& g, double a,
                                               double eta, Draws& rng, int* n_out, double* s_out, double* theta_out,
                                               d3* sv_out, uint32_t* rej) {
    int n = g.n;
    ThetaBound tb;
    theta_bound(n, a, eta, &tb);
    double sn = 2.0 * n * eta / (1.0 + 0.5 * a * a);
    double smax = sn / (1.0 + sn);
    double mx = lp_ceiling(a, eta, g, w);
    double s = 0.0, theta = 0.0;
    int it;
    for (it = 0; it < rng.cap; ++it) {
        double ss = smax * rng.next();
        double th = (PI / 2.0) * rng.next();
        if (th > tb.at(ss)) continue;
        double z = mx * rng.next();
        if (z < lp_ddpr(a, eta, ss, th, g, w)) {
            s = ss, theta = th;
            break;
        }
    }
    *rej += it;
    if (it == rng.cap) return 4;  // PTG_ERR_REJECTION_CAP
    return lp_finish(n, a, eta, s, theta, g, w, rng, n_out, s_out, theta_out, sv_out);
}

// The accepted (s, theta in [0, pi/2]): the quadrant of the azimuth and the
// photon's Stokes parameters.
static __device__ __noinline__ int lp_finish(int n, double a, double eta, double s, double theta, const DbGeom& g,
                                             const DbWork& w, Draws& rng, int* n_out, double* s_out, double* theta_out,
                                             d3* sv_out) {
    double sn = 2.0 * n * eta / (1.0 + 0.5 * a * a);
    int quadrant = (int)(4.0 * rng.next());
    if (quadrant == 1)
        theta = PI - theta;
    else if (quadrant == 2)
        theta = PI + theta;
    else if (quadrant == 3)
        theta = 2.0 * PI - theta;
    double wn = fmin(s / (sn * (1.0 - s)), 1.0);
    double x = -2.0 * n * a * cos(theta) * sqrt(wn * (1.0 - wn)) / sqrt(1.0 + 0.5 * a * a);
    double y = a * a * s / (8.0 * eta * (1.0 - s));
    double j[5];
    if (!db_evaluate(g, w, fabs(x), y, j)) return 9;
    double A0, A1, A2;
    if (x > 0.0) {
        A0 = j[2], A1 = 0.5 * (j[1] + j[3]), A2 = 0.25 * (j[0] + 2.0 * j[2] + j[4]);
    } else if (n % 2 == 0) {
        A0 = j[2], A1 = -0.5 * (j[1] + j[3]), A2 = 0.25 * (j[0] + 2.0 * j[2] + j[4]);
    } else {
        A0 = -j[2], A1 = 0.5 * (j[1] + j[3]), A2 = -0.25 * (j[0] + 2.0 * j[2] + j[4]);
    }
    double u = sqrt(2.0 * n * eta * (1.0 - s) / s - (1.0 + 0.5 * a * a));
    double st = sin(theta);
    double xi0 = (1.0 - s + 1.0 / (1.0 - s)) * (A1 * A1 - A0 * A2) - 2.0 * (A0 / a) * (A0 / a);
    double xi1 = 2.0 * (A1 * A1 - A0 * A2) - 2.0 * (1.0 + 2.0 * u * u * st * st) * (A0 / a) * (A0 / a);
    double xi2 = -1.0 * (2.0 * (u * A0 / a) * (u * A0 / a) * sin(2.0 * theta) + 4.0 * u * A0 * A1 * st / a);
    *sv_out = mk3(xi1 / xi0, xi2 / xi0, 0.0);
    *n_out = n;
    *s_out = s;
    *theta_out = theta;
    return 0;
}


// Draws held by lane `src`, for every lane of the warp.
__device__ __forceinline__ Draws shfl_draws(const Draws& d, int src) {
    const unsigned all = 0xffffffffu;
    Draws o;
    o.k0 = __shfl_sync(all, d.k0, src);
    o.k1 = __shfl_sync(all, d.k1, src);
    o.s_lo = __shfl_sync(all, d.s_lo, src);
    o.s_hi = __shfl_sync(all, d.s_hi, src);
    o.step = __shfl_sync(all, d.step, src);
    o.block = __shfl_sync(all, d.block, src);
    for (int q = 0; q < 4; ++q) o.w[q] = __shfl_sync(all, d.w[q], src);
    o.pos = __shfl_sync(all, d.pos, src);
    o.cap = __shfl_sync(all, d.cap, src);
    return o;
}

// lp_sample carried out by all 32 lanes of a converged warp, each with its
// own DoubleBessel workspace `w`, for one emission whose a, eta and draws
// every lane holds.  Every lane returns the same result, and it is
// lp_sample's on the same draws: the ceiling's points are spread over the
// lanes (the NaN-ignoring max does not depend on the order), and the
// rejection trials are dealt out in the order the serial sampler draws them
// (every lane replays the draws, which are cheap next to the rate), so
// that lane k evaluates the k-th trial that passes the theta bound; the
// first accepted trial in draw order is taken, with the draws as they stood
// after it.
static __device__ __noinline__ int lp_sample_warp(const NlcTables& t, const DbWork& w, double a, double eta,
                                                  Draws& rng, int* n_out, double* s_out, double* theta_out,
                                                  d3* sv_out, uint32_t* rej) {
    const unsigned all = 0xffffffffu;
    const int lane = (int)(threadIdx.x & 31u);
    if (t.lp_cdf == nullptr || w.base == nullptr) return 8;  // PTG_ERR_TABLES
    int n = lp_harmonic_index_warp(t, a, eta, rng.next());
    if (n < 1) return 2;  // PTG_ERR_OUT_OF_TABLE
    DbGeom g;
    if (!db_geom(n, w.cap, &g)) {
        // the harmonic needs a pooled workspace: lane 0 samples alone
        int st = 0, nn = 0;
        double s = 0.0, th = 0.0;
        d3 sv = mk3(0.0, 0.0, 0.0);
        uint32_t r0 = 0;
        if (lane == 0) {
            DbWork wk;
            int slot = -1;
            st = db_take(w, n, &wk, &g, &slot);
            if (st == 0) {
                st = lp_sample_n(t, wk, g, a, eta, rng, &nn, &s, &th, &sv, &r0);
                if (slot >= 0) db_pool_release(w.pool, slot);
            }
        }
        __syncwarp();
        st = __shfl_sync(all, st, 0);
        *n_out = __shfl_sync(all, nn, 0);
        *s_out = __shfl_sync(all, s, 0);
        *theta_out = __shfl_sync(all, th, 0);
        *sv_out = mk3(__shfl_sync(all, sv.x, 0), __shfl_sync(all, sv.y, 0), __shfl_sync(all, sv.z, 0));
        *rej += __shfl_sync(all, r0, 0);
        rng = shfl_draws(rng, 0);
        return st;
    }
    // the bound on theta: point i on lane i
    ThetaBound tb;
    {
        double si = 0.0, fi = 0.0;
        if (lane < 16) theta_bound_point(n, a, eta, lane, &si, &fi);
        for (int i = 0; i < 16; ++i) {
            tb.s[i] = __shfl_sync(all, si, i);
            tb.f[i] = __shfl_sync(all, fi, i);
        }
        theta_bound_finish(&tb);
    }
    // the ceiling: its points spread over the lanes
    LpCeilPlan p;
    lp_ceiling_plan(a, eta, n, &p);
    double mx = NAN;
    for (int k = lane, np = lp_ceiling_points(p); k < np; k += 32) {
        double s, theta;
        lp_ceiling_point(p, k, &s, &theta);
        mx = rmax(mx, lp_ddpr(a, eta, s, theta, g, w));
    }
    for (int o = 16; o > 0; o >>= 1) mx = rmax(mx, __shfl_xor_sync(all, mx, o));
    mx = 1.15 * mx;
    // rejection, 32 trials that pass the theta bound at a time
    double sn = 2.0 * n * eta / (1.0 + 0.5 * a * a);
    double smax = sn / (1.0 + sn);
    Draws r = rng;
    int it = 0;
    while (it < r.cap) {
        int my_it = -1;
        double my_s = 0.0, my_th = 0.0, my_z = 0.0;
        Draws my_r = r;
        for (int k = 0; k < 32 && it < r.cap; ++it) {
            double ss = smax * r.next();
            double th = (PI / 2.0) * r.next();
            if (th > tb.at(ss)) continue;
            double z = mx * r.next();
            if (k == lane) my_it = it, my_s = ss, my_th = th, my_z = z, my_r = r;
            ++k;
        }
        bool acc = my_it >= 0 && my_z < lp_ddpr(a, eta, my_s, my_th, g, w);
        unsigned m = __ballot_sync(all, acc);
        if (m != 0u) {
            int win = __ffs(m) - 1;
            int acc_it = __shfl_sync(all, my_it, win);
            double s = __shfl_sync(all, my_s, win);
            double theta = __shfl_sync(all, my_th, win);
            rng = shfl_draws(my_r, win);
            *rej += acc_it;
            return lp_finish(n, a, eta, s, theta, g, w, rng, n_out, s_out, theta_out, sv_out);
        }
    }
    rng = r;
    *rej += r.cap;
    return 4;  // PTG_ERR_REJECTION_CAP
}

// ---------------------------------------------- classical LP emission ----
// nonlinear_compton/lp/classical.rs:19-40 (v = s / s_max)
static __device__ __noinline__ double lp_cl_ddpr(double a, double v, double theta, const DbGeom& g, const DbWork& w) {
    int n = g.n;
    double x = 2.0 * n * a * cos(theta) * sqrt(v * (1.0 - v) / (1.0 + 0.5 * a * a));
    double y = 0.25 * n * a * a * v / (1.0 + 0.5 * a * a);
    double j[5];
    if (!db_evaluate(g, w, x, y, j)) return NAN;
    double g0, g1, g2;
    if (n % 2 == 0) {
        g0 = j[2], g1 = -0.5 * (j[1] + j[3]), g2 = 0.25 * (j[0] + 2.0 * j[2] + j[4]);
    } else {
        g0 = -j[2], g1 = 0.5 * (j[1] + j[3]), g2 = -0.25 * (j[0] + 2.0 * j[2] + j[4]);
    }
    return (-g0 * g0 - a * a * (g0 * g2 - g1 * g1)) / (2.0 * PI);
}

// nonlinear_compton/lp/classical.rs:43-108
static __device__ __noinline__ double lp_cl_ceiling(double a, const DbGeom& g, const DbWork& w) {
    int n = g.n;
    double mx = NAN;
    if (n == 1) {
        mx = lp_cl_ddpr(a, 0.01, PI / 2.0, g, w);
    } else if (a <= 1.5) {
        double v_min = 0.1 + (9.0 / sqrt((double)n) - 1.0) / 10.0;
        double v_max = fmin(v_min + 0.4, 1.0);
        for (int i = 1; i <= 16; ++i) mx = rmax(mx, lp_cl_ddpr(a, v_min + (v_max - v_min) * (double)i / 16.0, 0.0, g, w));
    } else if (a < 5.0) {
        double nsw = 3.0 * pow(a / 2.0, 4.0 / 3.0);
        int n_switch = nsw >= 2147483647.0 ? 2147483647 : (int)nsw;
        double theta = n > n_switch ? 0.0 : (PI / 2.0) * (1.0 - log((double)n) / log((double)n_switch));
        double v_min = fmin(0.35 + (7.0 / sqrt((double)n) - 1.0) / 9.0, 0.55);
        double v_max = 0.55 + (7.0 / sqrt((double)n) - 1.0) / 9.0;
        int num = a > 4.0 ? 32 : 16;
        for (int i = 0; i < num; ++i) mx = rmax(mx, lp_cl_ddpr(a, v_min + (v_max - v_min) * (double)i / num, theta, g, w));
    } else {
        double n_switch = 10.0 * (a / 5.0) * (a / 5.0);
        double theta = 0.0;
        if (!(n > (int)n_switch)) {
            double pw = 0.3 + (0.7 - 0.3) * (log(a) - log(5.0)) / (log(20.0) - log(5.0));
            theta = (PI / 2.0) * (pow((double)n, -pw) - pow(n_switch, -pw)) / (1.0 - pow(n_switch, -pw));
        }
        double v_min = 0.3 + 0.4 * log((double)n) * pow((double)n, -0.7);
        double v_max = v_min + 0.2;
        int num = a > 8.0 ? 64 : 32;
        for (int i = 0; i < num; ++i) mx = rmax(mx, lp_cl_ddpr(a, v_min + (v_max - v_min) * (double)i / num, theta, g, w));
    }
    return 1.1 * mx;
}

// nonlinear_compton/lp/mod.rs:209-268 (ThetaBound at fixed v)
static __device__ __noinline__ void theta_bound_low_eta(int n, double a, ThetaBound* tb) {
    for (int i = 0; i < 16; ++i) {
        double z = cos(PI * i / 15.0);
        double v = 0.5 * (z + 1.0);
        tb->s[i] = v;
        double x = 2.0 * n * a * sqrt(v * (1.0 - v) / (1.0 + 0.5 * a * a));
        double y = 0.25 * n * a * a * v / (1.0 + 0.5 * a * a);
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

// nonlinear_compton/lp/classical.rs:213-252 (cdf_table [61][16][2])
static __device__ __noinline__ int lp_cl_harmonic_index(const NlcTables& t, double a, double frac) {
    if (log(a) <= PTG_NLC_CL_MIN) return 1;
    int ix = (int)((log(a) - PTG_NLC_CL_MIN) / PTG_NLC_CL_STEP);
    double dx = (log(a) - PTG_NLC_CL_MIN) / PTG_NLC_CL_STEP - ix;
    if (ix >= 60) return -1;
    double n = 0.0;
    for (int k = 0; k < 2; ++k) {
        const double* tb = t.lp_cl_cdf + (size_t)(ix + k) * 32;
        double nk = 0.9;
        if (!(frac <= tb[1]) && !pw_invert(tb, 16, false, frac, &nk)) return -1;
        n += nk * (k == 0 ? 1.0 - dx : dx);
    }
    if (!isfinite(n)) return -1;
    double c = ceil(n);
    return c >= 2147483647.0 ? 2147483647 : (int)c;
}

static __device__ __noinline__ int lp_classical_sample_n(const DbGeom& g, const DbWork& w, double a, double eta,
                                                         Draws& rng, double* s_out, double* theta_out, d3* sv_out,
                                                         uint32_t* rej) {
    int n = g.n;
    ThetaBound tb;
    theta_bound_low_eta(n, a, &tb);
    double smax = 2.0 * n * eta / (1.0 + 0.5 * a * a);
    double mx = lp_cl_ceiling(a, g, w);
    double v = 0.0, s = 0.0, theta = 0.0;
    int it;
    for (it = 0; it < rng.cap; ++it) {
        double vv = rng.next();
        double ss = vv * smax;
        double th = (PI / 2.0) * rng.next();
        if (th > tb.at(vv)) continue;
        double z = mx * rng.next();
        if (z < lp_cl_ddpr(a, vv, th, g, w)) {
            v = vv, s = ss, theta = th;
            break;
        }
    }
    *rej += it;
    if (it == rng.cap) return 4;
    int quadrant = (int)(4.0 * rng.next());
    if (quadrant == 1)
        theta = PI - theta;
    else if (quadrant == 2)
        theta = PI + theta;
    else if (quadrant == 3)
        theta = 2.0 * PI - theta;
    double x = 2.0 * n * a * cos(theta) * sqrt(v * (1.0 - v) / (1.0 + 0.5 * a * a));
    double y = 0.25 * n * a * a * v / (1.0 + 0.5 * a * a);
    double j[5];
    if (!db_evaluate(g, w, x, y, j)) return 9;
    double A0, A1, A2;
    if (n % 2 == 0) {
        A0 = j[2], A1 = -0.5 * (j[1] + j[3]), A2 = 0.25 * (j[0] + 2.0 * j[2] + j[4]);
    } else {
        A0 = -j[2], A1 = 0.5 * (j[1] + j[3]), A2 = -0.25 * (j[0] + 2.0 * j[2] + j[4]);
    }
    double u = sqrt((1.0 + 0.5 * a * a) * (1.0 - v) / v);
    double st = sin(theta);
    double xi0 = 2.0 * (A1 * A1 - A0 * A2) - 2.0 * (A0 / a) * (A0 / a);
    double xi1 = 2.0 * (A1 * A1 - A0 * A2) - 2.0 * (1.0 + 2.0 * u * u * st * st) * (A0 / a) * (A0 / a);
    double xi2 = 2.0 * (u * A0 / a) * (u * A0 / a) * sin(2.0 * theta) + 4.0 * u * A0 * A1 * st / a;
    *sv_out = mk3(xi1 / xi0, xi2 / xi0, 0.0);
    *s_out = s;
    *theta_out = theta;
    return 0;
}

// nonlinear_compton/lp/classical.rs:257-330.  Returns a ptg status.
static __device__ __noinline__ int lp_classical_sample(const NlcTables& t, const DbWork& w, double a, double eta,
                                                       Draws& rng, int* n_out, double* s_out, double* theta_out,
                                                       d3* sv_out, uint32_t* rej) {
    if (t.lp_cl_cdf == nullptr || w.base == nullptr) return 8;
    int n = lp_cl_harmonic_index(t, a, rng.next());
    if (n < 1) return 2;
    DbWork wk;
    DbGeom g;
    int slot = -1;
    int st = db_take(w, n, &wk, &g, &slot);
    if (st != 0) return st;
    *n_out = n;
    st = lp_classical_sample_n(g, wk, a, eta, rng, s_out, theta_out, sv_out, rej);
    if (slot >= 0) db_pool_release(w.pool, slot);
    return st;
}

// Orders a DoubleBessel workspace must hold for harmonics up to n.
__host__ __device__ inline int db_len_for(int n) {
    double xm = n * 1.4142135623730951, ym = n * 0.5;
    int nmb = (int)floor(-2.0 * ym - xm);
    int npb = xm > 4.0 * (2.0 - 1.4142135623730951) * ym ? (int)ceil(xm) : (int)ceil(2.0 * ym + xm * xm / (16.0 * ym));
    return npb - nmb + 200;
}

}  // namespace ptg
