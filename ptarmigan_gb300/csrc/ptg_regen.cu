// Table regeneration on the device: the LP Breit-Wheeler mid-range CDF
// (pair_creation/lp/tables/mid_range/cdf.rs, absent from the reference
// tree).  Its generator is pair_creation/lp/mod.rs:1063-1163: at every node
// (eta' = 2 / (1 + i/4), a = 10^(-7/5 + j/20)) TotalRate::by_summation sums
// DoubleDiffPartialRate::integrate over the harmonics and keeps 16 CDF
// nodes.  Pass 1 runs one thread per (node, harmonic) with the direct or
// the adaptive 2-D integration of quadrature/adaptive.rs; pass 2 one thread
// per node for the cumulative sums and the node selection.
#include "ptg_bw_lp.cuh"
#include "ptg_launch.h"

namespace ptg {

struct C2 {
    double re, im;
};
__device__ __forceinline__ C2 c2_add(C2 a, C2 b) { return C2{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ C2 c2_sub(C2 a, C2 b) { return C2{a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ C2 c2_scale(double s, C2 a) { return C2{s * a.re, s * a.im}; }

struct AdRegion {
    C2 integral, error;
    double x0, x1, y0, y1;
    C2 cache[3][3];
};

__constant__ double CC5[5][3] = {{0.0, 1.0 / 30.0, 1.0 / 6.0},
                                 {0.1464466094067262, 4.0 / 15.0, 0.0},
                                 {0.5, 2.0 / 5.0, 2.0 / 3.0},
                                 {0.8535533905932738, 4.0 / 15.0, 0.0},
                                 {1.0, 1.0 / 30.0, 1.0 / 6.0}};
__constant__ double CC5_EXT[9] = {0.0, 0.1464466094067262, 0.5, 0.8535533905932738, 1.0,
                                  1.1464466094067262, 1.5, 1.8535533905932738, 2.0};
__constant__ double CC9[9][3] = {{0.0000000000000000, 0.0079365079365079, 1.0 / 30.0},
                                 {0.0380602337443566, 0.0731093246080091, 0.0},
                                 {0.1464466094067262, 0.1396825396825397, 4.0 / 15.0},
                                 {0.3086582838174551, 0.1808589293602449, 0.0},
                                 {0.5000000000000000, 0.1968253968253968, 2.0 / 5.0},
                                 {0.6913417161825449, 0.1808589293602449, 0.0},
                                 {0.8535533905932738, 0.1396825396825397, 4.0 / 15.0},
                                 {0.9619397662556434, 0.0731093246080091, 0.0},
                                 {1.0000000000000000, 0.0079365079365079, 1.0 / 30.0}};
__constant__ double CC9_EXT[17] = {0.0000000000000000, 0.0380602337443566, 0.1464466094067262, 0.3086582838174551,
                                   0.5000000000000000, 0.6913417161825449, 0.8535533905932738, 0.9619397662556434,
                                   1.0000000000000000, 1.0380602337443566, 1.1464466094067262, 1.3086582838174551,
                                   1.5000000000000000, 1.6913417161825449, 1.8535533905932738, 1.9619397662556434,
                                   2.0000000000000000};

// The integrand of DoubleDiffPartialRate::integrate: the rate for the two
// linear polarisations, (unpol -/+ delta_1) / 2 pi, inside theta < bound(s).
struct LppIntegrand {
    DbGeom g;
    DbWork w;
    double a, eta;
    LppTheta tb;
    __device__ bool inside(double s, double th) const { return th < tb.at(s); }
    __device__ C2 operator()(double s, double th) const {
        double u, d1, d2;
        lpp_elements(g, w, a, eta, s, th, &u, &d1, &d2);
        return C2{(u - d1) / (2.0 * PI), (u + d1) / (2.0 * PI)};
    }
};

__device__ C2 ad_eval(const LppIntegrand& f, double x, double y) { return f.inside(x, y) ? f(x, y) : C2{0.0, 0.0}; }

__device__ void ad_new(const LppIntegrand& f, double x0, double x1, double y0, double y1, AdRegion* g) {
    C2 result{0.0, 0.0}, error{0.0, 0.0};
    for (int i = 0; i < 5; ++i) {
        double y = y0 + CC5[i][0] * (y1 - y0);
        for (int j = 0; j < 5; ++j) {
            double x = x0 + CC5[j][0] * (x1 - x0);
            C2 z = ad_eval(f, x, y);
            result = c2_add(result, c2_scale(CC5[i][1] * CC5[j][1] * (y1 - y0) * (x1 - x0), z));
            error = c2_add(error, c2_scale(CC5[i][2] * CC5[j][2] * (y1 - y0) * (x1 - x0), z));
            if (i % 2 == 0 && j % 2 == 0) g->cache[i / 2][j / 2] = z;
        }
    }
    g->integral = result;
    g->error = c2_sub(result, error);
    g->x0 = x0, g->x1 = x1, g->y0 = y0, g->y1 = y1;
}

// Region::custom_partition (x split and/or y split requested)
__device__ void ad_custom_partition(const AdRegion& r, const LppIntegrand& f, bool sx, double xs, bool sy, double ys,
                                    AdRegion* out) {
    double x0 = r.x0, x1 = r.x1, y0 = r.y0, y1 = r.y1;
    double xm = sx ? xs : 0.5 * (x0 + x1), ym = sy ? ys : 0.5 * (y0 + y1);
    C2 z[9][9];
    for (int i = 0; i < 9; ++i) {
        double ty = CC5_EXT[i];
        double y = i < 4 ? y0 + ty * (ym - y0) : ym + (ty - 1.0) * (y1 - ym);
        for (int j = 0; j < 9; ++j) {
            double tx = CC5_EXT[j];
            double x = j < 4 ? x0 + tx * (xm - x0) : xm + (tx - 1.0) * (x1 - xm);
            if (i % 8 == 0 && j % 8 == 0)
                z[i][j] = r.cache[i / 4][j / 4];
            else if (i % 4 == 0 && j % 4 == 0 && !sx && !sy)
                z[i][j] = r.cache[i / 4][j / 4];
            else
                z[i][j] = ad_eval(f, x, y);
        }
    }
    for (int rr = 0; rr < 2; ++rr)
        for (int cc = 0; cc < 2; ++cc) {
            C2 res{0.0, 0.0}, err{0.0, 0.0};
            double dy = rr < 1 ? ym - y0 : y1 - ym;
            double dx = cc < 1 ? xm - x0 : x1 - xm;
            for (int i = 0; i < 5; ++i)
                for (int j = 0; j < 5; ++j) {
                    C2 val = z[i + 4 * rr][j + 4 * cc];
                    res = c2_add(res, c2_scale(CC5[j][1] * CC5[i][1] * dx * dy, val));
                    err = c2_add(err, c2_scale(CC5[j][2] * CC5[i][2] * dx * dy, val));
                }
            AdRegion& o = out[2 * rr + cc];
            o.integral = res;
            o.error = c2_sub(res, err);
            o.x0 = cc ? xm : x0, o.x1 = cc ? x1 : xm, o.y0 = rr ? ym : y0, o.y1 = rr ? y1 : ym;
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) o.cache[i][j] = z[4 * rr + 2 * i][4 * cc + 2 * j];
        }
}

// Region::partition (even split, 9-point Clenshaw-Curtis per child)
__device__ void ad_partition(const AdRegion& r, const LppIntegrand& f, AdRegion* out) {
    double x0 = r.x0, x1 = r.x1, y0 = r.y0, y1 = r.y1;
    double xm = 0.5 * (x0 + x1), ym = 0.5 * (y0 + y1);
    C2 z[17][17];
    for (int i = 0; i < 17; ++i) {
        double y = y0 + 0.5 * CC9_EXT[i] * (y1 - y0);
        for (int j = 0; j < 17; ++j) {
            double x = x0 + 0.5 * CC9_EXT[j] * (x1 - x0);
            z[i][j] = (i % 8 == 0 && j % 8 == 0) ? r.cache[i / 8][j / 8] : ad_eval(f, x, y);
        }
    }
    for (int rr = 0; rr < 2; ++rr)
        for (int cc = 0; cc < 2; ++cc) {
            C2 res{0.0, 0.0}, err{0.0, 0.0};
            double dy = 0.5 * (y1 - y0), dx = 0.5 * (x1 - x0);
            for (int i = 0; i < 9; ++i)
                for (int j = 0; j < 9; ++j) {
                    C2 val = z[i + 8 * rr][j + 8 * cc];
                    res = c2_add(res, c2_scale(CC9[j][1] * CC9[i][1] * dx * dy, val));
                    err = c2_add(err, c2_scale(CC9[j][2] * CC9[i][2] * dx * dy, val));
                }
            AdRegion& o = out[2 * rr + cc];
            o.integral = res;
            o.error = c2_sub(res, err);
            o.x0 = cc ? xm : x0, o.x1 = cc ? x1 : xm, o.y0 = rr ? ym : y0, o.y1 = rr ? y1 : ym;
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) o.cache[i][j] = z[8 * rr + 4 * i][8 * cc + 4 * j];
        }
}

__device__ __forceinline__ double ad_key(const AdRegion& g) { return g.error.re * g.error.re + g.error.im * g.error.im; }

// integrate_2d: at most 4 + 3 * 16 regions
__device__ C2 ad_integrate_2d(const LppIntegrand& f, double x0, bool has_xd, double xd, double x1, double y0,
                              bool has_yd, double yd, double y1, double tol, int max_recursion) {
    AdRegion regions[4 + 3 * 16];
    int nr = 0;
    AdRegion first;
    ad_new(f, x0, x1, y0, y1, &first);
    if (!has_xd && !has_yd) {
        regions[nr++] = first;
    } else {
        ad_custom_partition(first, f, has_xd, xd, has_yd, yd, regions);
        nr = 4;
    }
    C2 integral{0.0, 0.0};
    for (int it = 0; it < max_recursion; ++it) {
        C2 is{0.0, 0.0}, es{0.0, 0.0};
        for (int k = 0; k < nr; ++k) {
            is = c2_add(is, regions[k].integral);
            es = c2_add(es, regions[k].error);
        }
        integral = is;
        if (fabs(es.re) <= tol * fabs(is.re) && fabs(es.im) <= tol * fabs(is.im)) break;
        AdRegion worst = regions[--nr];
        ad_partition(worst, f, regions + nr);
        nr += 4;
        // stable insertion sort by squared error norm
        for (int k = 1; k < nr; ++k) {
            AdRegion v = regions[k];
            double key = ad_key(v);
            int m = k - 1;
            while (m >= 0 && ad_key(regions[m]) > key) {
                regions[m + 1] = regions[m];
                --m;
            }
            regions[m + 1] = v;
        }
    }
    return integral;
}

// DoubleDiffPartialRate::integrate (pair_creation/lp/mod.rs:115-227)
__device__ C2 lpp_integrate(const LppIntegrand& f) {
    int n = f.g.n;
    double a = f.a, eta = f.eta;
    double s_min = 0.5, s_max = fmax(0.5 + sqrt(0.25 - (1.0 + 0.5 * a * a) / (2.0 * n * eta)), 0.5);
    if (f.tb.at(0.5) < 0.75 * (PI / 2.0)) {
        double s_peak = 0.5 + sqrt(0.25 - (1.0 + a * a) / (2.0 * n * eta));
        bool has_peak = s_peak > s_min + 2.0 * (s_max - s_min) / 3.0;
        double theta_split = f.tb.at(has_peak ? s_peak : 0.5);
        C2 v = ad_integrate_2d(f, s_min, has_peak, s_peak, s_max, 0.0, true, theta_split, PI / 2.0, 1.0e-3, 16);
        return c2_scale(4.0 * 2.0, v);
    }
    double s_peak = fmin(0.5 + sqrt(0.25 - (1.0 + a * a) / (2.0 * n * eta)), 0.5);
    auto segment = [&](double s0, double s1, const double* nodes, const double* weights, int nn) {
        C2 acc{0.0, 0.0};
        for (int k = 0; k < nn; ++k) {
            double s = s0 + 0.5 * (nodes[k] + 1.0) * (s1 - s0);
            double mt = f.tb.at(s);
            C2 sd{0.0, 0.0};
            for (int q = 0; q < 32; ++q) {
                double th = 0.5 * (PTG_GAUSS_32_NODES[q] + 1.0) * mt;
                sd = c2_add(sd, c2_scale(0.5 * PTG_GAUSS_32_WEIGHTS[q] * mt, f(s, th)));
            }
            acc = c2_add(acc, c2_scale(0.5 * weights[k] * (s1 - s0), sd));
        }
        return acc;
    };
    C2 integral;
    if (s_peak < s_min + 2.0 * (s_max - s_min) / 3.0) {
        s_peak = fmin(s_peak, s_min + (s_max - s_min) / 3.0);
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

// Pass 1: one thread per (node, harmonic); job k integrates harmonic
// n_of[k] at (a_of[k], eta_of[k]) into rates[2k], rates[2k+1].  The lane's
// J(n, x, y) workspace: slot (k - first) of `ws` (cap orders each).
__global__ void k_regen_lpm_partial(unsigned long long first, unsigned long long count, const int* n_of,
                                    const double* a_of, const double* eta_of, double* ws, int cap, double* rates,
                                    int* bad) {
    unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (t >= count) return;
    unsigned long long k = first + t;
    LppIntegrand f;
    f.a = a_of[k];
    f.eta = eta_of[k];
    if (!db_geom(n_of[k], cap, &f.g)) {
        atomicAdd(bad, 1);
        rates[2 * k] = rates[2 * k + 1] = NAN;
        return;
    }
    f.w = DbWork{ws + (t >> 5) * (size_t)cap * 5 * 32 + (t & 31), cap, 32};
    lpp_theta_bound(f.g.n, f.a, f.eta, &f.tb);
    C2 v = lpp_integrate(f);
    rates[2 * k] = v.re;
    rates[2 * k + 1] = v.im;
}

// Pass 2: one thread per node: cumulative sums over n_min..n_max and the
// 16 log-spaced CDF nodes of TotalRate::by_summation.
__global__ void k_regen_lpm_cdf(int npoints, const int* nmin_of, const int* nmax_of, const unsigned long long* off_of,
                                const double* rates, double* cdf_out /* [np][16][3] */, double* total_out /* [np][2] */) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npoints) return;
    int n_min = nmin_of[p], n_max = nmax_of[p];
    const double* r = rates + 2 * off_of[p];
    int len = n_max - n_min + 1;
    double* c = cdf_out + (size_t)p * 48;
    for (int i = 0; i < 48; ++i) c[i] = 0.0;
    c[0] = (double)n_min;
    double u_max = log(1.0 + (double)(n_max - n_min));
    double u = 0.0, du = u_max / 15.0;
    for (int i = 1; i <= 15; ++i) {
        u = u + du;
        double nn = (double)n_min + expm1(u);
        if (round(nn) <= c[3 * (i - 1)]) {
            nn = c[3 * (i - 1)] + 1.0;
            u = log(nn - (double)n_min + 1.0);
            du = (u_max - u) / (15.0 - (double)i);
        } else {
            nn = round(nn);
        }
        c[3 * i] = nn;
    }
    for (int i = 0; i < 16; ++i) {
        long long index = (long long)as_i32(c[3 * i]) - (long long)n_min;
        if (index < 0 || index >= len) index = len - 1;
        double re = 0.0, im = 0.0;
        for (long long k = 0; k <= index; ++k) {
            re = re + r[2 * k];
            im = im + r[2 * k + 1];
        }
        c[3 * i + 1] = re;
        c[3 * i + 2] = im;
    }
    total_out[2 * p] = c[46];
    total_out[2 * p + 1] = c[47];
}

cudaError_t launch_regen_lpm_partial(unsigned long long first, unsigned long long count, const int* n_of,
                                     const double* a_of, const double* eta_of, double* ws, int cap, double* rates,
                                     int* bad, cudaStream_t s) {
    k_regen_lpm_partial<<<(unsigned)((count + 63) / 64), 64, 0, s>>>(first, count, n_of, a_of, eta_of, ws, cap, rates,
                                                                     bad);
    return cudaGetLastError();
}

cudaError_t launch_regen_lpm_cdf(int npoints, const int* nmin_of, const int* nmax_of, const unsigned long long* off_of,
                                 const double* rates, double* cdf_out, double* total_out, cudaStream_t s) {
    k_regen_lpm_cdf<<<(npoints + 63) / 64, 64, 0, s>>>(npoints, nmin_of, nmax_of, off_of, rates, cdf_out, total_out);
    return cudaGetLastError();
}

}  // namespace ptg
