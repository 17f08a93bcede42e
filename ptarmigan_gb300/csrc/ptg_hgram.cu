// Distribution output on the device: the particle functions of
// output/functions.rs and the two passes of Histogram::generate_1d/2d
// (output/hgram.rs:209-448): the set's extent, total weight and size, then
// the binning.  The host turns the extent into bins exactly as the
// reference does (ptg_engine.cu, ptg_histogram).
#include <cfloat>

#include "ptg_launch.h"
#include "ptg_math.cuh"

namespace ptg {

// geometry/polarization.rs:159-214 (project_onto), for the projection of a
// particle's polarization on the x or y axis.
__device__ double pol_project(const double* sv, double nx, double ny, double nz, double ax, double ay, double az) {
    double frac = hypot(hypot(sv[1], sv[2]), sv[3]) / sv[0];
    // the transverse axes of the ellipse
    double mag = hypot(nx, nz);
    double x0, x1, x2;
    if (mag == 0.0) {
        x0 = 1.0, x1 = 0.0, x2 = 0.0;
    } else {
        x0 = nz / mag, x1 = 0.0, x2 = -nx / mag;
    }
    double y0 = x1 * nz - x2 * ny, y1 = x2 * nx - x0 * nz, y2 = x0 * ny - x1 * nx;
    double am = sqrt(ax * ax + ay * ay + az * az);
    ax /= am, ay /= am, az /= am;
    double xa = x0 * ax + x1 * ay + x2 * az, ya = y0 * ax + y1 * ay + y2 * az;
    double unpol = 0.5 * (xa * xa + ya * ya);
    if (!(frac > 0.0)) return unpol;
    double q = sv[1] / (frac * sv[0]), uu = sv[2] / (frac * sv[0]), v = sv[3] / (frac * sv[0]);
    double ex;
    if (1.0 + q < 1.0e-12) {
        double x_sqd = uu * uu + v * v;
        double delta = 0.5 * x_sqd + 0.125 * x_sqd * x_sqd;
        ex = sqrt(0.5 * delta);
    } else {
        ex = sqrt(0.5 * (1.0 + q));
    }
    double eyr, eyi;
    if (ex == 0.0) {
        eyr = 1.0, eyi = 0.0;
    } else {
        eyr = 0.5 * uu / ex, eyi = -0.5 * v / ex;
    }
    double pr = ex * xa + eyr * ya, pi = eyi * ya;
    double pol = pr * pr + pi * pi;
    return frac * pol + (1.0 - frac) * unpol;
}

// output/functions.rs:109-242 (momenta in MeV, positions in m)
__device__ double out_value(const HgramArgs& h, unsigned long long i, int f) {
    const double m = ELECTRON_MASS_MEV;
    const double* u = h.u + 4 * i;
    const double* r = h.r + 4 * i;
    switch (f) {
        case 0: return atan2(m * u[1], m * u[3]);
        case 1: return atan2(m * u[2], m * u[3]);
        case 2: return atan2(hypot(m * u[1], m * u[2]), -(m * u[3]));
        case 3: return atan2(hypot(m * u[1], m * u[2]), m * u[3]);
        case 4: return m * u[1];
        case 5: return m * u[2];
        case 6: return m * u[3];
        case 7: return hypot(m * u[1], m * u[2]);
        case 8: return hypot(m * u[1], m * u[2]) / (m * u[0] - m * u[3]);
        case 9: return m * u[1] / (m * u[0] - m * u[3]);
        case 10: return m * u[2] / (m * u[0] - m * u[3]);
        case 11: return m * u[0] - m * u[3];
        case 12: return m * u[0] + m * u[3];
        case 13: return u[0];
        case 14: return u[0] * m;
        case 15: return 1.0;
        case 16: return r[1];
        case 17: return r[2];
        case 18: return r[3];
        case 19: return hypot(r[1], r[2]);
        case 20: return h.payload[i];
        case 21: return h.parent_chi[i];
        case 22: return h.icount[i];
        case 23: return h.work[i] * m;
        case 24: return h.pol[4 * i + 1];
        case 25: return h.pol[4 * i + 2];
        case 26: return h.pol[4 * i + 3];
        case 29: return h.weight[i];
        case 30: return h.pol[4 * i + 3] * h.weight[i];
        default: {
            // pol_x, pol_y: along the normalised three-momentum
            double n = sqrt(u[1] * u[1] + u[2] * u[2] + u[3] * u[3]);
            double ax = f == 27 ? 1.0 : 0.0, ay = f == 27 ? 0.0 : 1.0;
            return pol_project(h.pol + 4 * i, u[1] / n, u[2] / n, u[3] / n, ax, ay, 0.0);
        }
    }
}

// output/functions.rs:244-263
__device__ double out_weight(const HgramArgs& h, unsigned long long i) {
    double w = h.weight[i];
    switch (h.wfunc) {
        case 1: return w * (h.u[4 * i] * ELECTRON_MASS_MEV);
        case 2: return out_value(h, i, 27) * w;
        case 3: return out_value(h, i, 28) * w;
        case 4: return h.pol[4 * i + 3] * w;
        default: return w;
    }
}

__device__ __forceinline__ bool out_accepts(const HgramArgs& h, unsigned long long i) {
    if (h.filter_func < 0) return true;
    double v = out_value(h, i, h.filter_func);
    return v >= h.fmin && v < h.fmax;
}

__device__ __forceinline__ double axis_value(const HgramArgs& h, unsigned long long i, int k) {
    double v = out_value(h, i, h.func[k]) * h.scale[k];
    return h.log_bins ? log(v) : v;
}

// Pass 1: per block, [min0, max0, min1, max1, total weight, particles]
// over the particles of the species (hgram.rs:150-165, 222-238).
__global__ void __launch_bounds__(256) k_hgram_stats(HgramArgs h, double* partials) {
    __shared__ double sh[6][8];
    double mn0 = DBL_MAX, mx0 = -DBL_MAX, mn1 = DBL_MAX, mx1 = -DBL_MAX, tot = 0.0, cnt = 0.0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < h.n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        if (h.species[i] != h.want_species) continue;
        cnt += 1.0;
        tot += out_weight(h, i);
        if (!out_accepts(h, i)) continue;
        double v0 = axis_value(h, i, 0);
        if (isfinite(v0)) mn0 = fmin(mn0, v0), mx0 = fmax(mx0, v0);
        if (h.dim == 2) {
            double v1 = axis_value(h, i, 1);
            if (isfinite(v1)) mn1 = fmin(mn1, v1), mx1 = fmax(mx1, v1);
        }
    }
    double v[6] = {mn0, mx0, mn1, mx1, tot, cnt};
    for (int off = 16; off > 0; off >>= 1) {
        v[0] = fmin(v[0], __shfl_down_sync(0xffffffffu, v[0], off));
        v[1] = fmax(v[1], __shfl_down_sync(0xffffffffu, v[1], off));
        v[2] = fmin(v[2], __shfl_down_sync(0xffffffffu, v[2], off));
        v[3] = fmax(v[3], __shfl_down_sync(0xffffffffu, v[3], off));
        v[4] += __shfl_down_sync(0xffffffffu, v[4], off);
        v[5] += __shfl_down_sync(0xffffffffu, v[5], off);
    }
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
        for (int k = 0; k < 6; ++k) sh[k][warp] = v[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        int nw = blockDim.x >> 5;
        double o[6] = {sh[0][0], sh[1][0], sh[2][0], sh[3][0], sh[4][0], sh[5][0]};
        for (int w = 1; w < nw; ++w) {
            o[0] = fmin(o[0], sh[0][w]), o[1] = fmax(o[1], sh[1][w]);
            o[2] = fmin(o[2], sh[2][w]), o[3] = fmax(o[3], sh[3][w]);
            o[4] += sh[4][w], o[5] += sh[5][w];
        }
        for (int k = 0; k < 6; ++k) partials[6 * blockIdx.x + k] = o[k];
    }
}

// Rust's `f as usize` for the bin index: negative and NaN go to 0.
__device__ __forceinline__ unsigned long long bin_index(double x) {
    double f = floor(x);
    if (!(f > 0.0)) return 0ull;
    return f >= 1.8446744073709552e19 ? ~0ull : (unsigned long long)f;
}

// exp(min + bin * size) * expm1(size) (hgram.rs:167-169)
__device__ __forceinline__ double linear_bin_vol(double mn, double sz, unsigned long long bin) {
    return exp(mn + (double)bin * sz) * expm1(sz);
}

// Pass 2: the binning (hgram.rs:257-292 and 380-412).  Counts are summed
// with atomics, in shared memory when they fit.
__global__ void __launch_bounds__(256) k_hgram_fill(HgramArgs h, double* counts) {
    extern __shared__ double sc[];
    unsigned long long ncts = h.nbins[0] * (h.dim == 2 ? h.nbins[1] : 1ull);
    bool shared = ncts <= 6144ull;
    if (shared) {
        for (unsigned long long k = threadIdx.x; k < ncts; k += blockDim.x) sc[k] = 0.0;
        __syncthreads();
    }
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < h.n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        if (h.species[i] != h.want_species) continue;
        double v0 = axis_value(h, i, 0), v1 = h.dim == 2 ? axis_value(h, i, 1) : 0.0;
        double w = out_weight(h, i);
        if (!isfinite(v0) || !isfinite(v1)) continue;
        if (!out_accepts(h, i)) continue;
        unsigned long long fbin;
        if (h.dim == 1) {
            unsigned long long b = bin_index((v0 - h.gmin[0]) / h.bin_sz[0]);
            if (h.density_log) w = w * h.bin_sz[0] / linear_bin_vol(h.gmin[0], h.bin_sz[0], b);
            fbin = b;
        } else {
            unsigned long long b0 = h.bin_sz[0] == 0.0 ? 0ull : bin_index((v0 - h.gmin[0]) / h.bin_sz[0]);
            unsigned long long b1 = h.bin_sz[1] == 0.0 ? 0ull : bin_index((v1 - h.gmin[1]) / h.bin_sz[1]);
            if (h.density_log) {
                w *= h.bin_sz[0] == 0.0 ? 1.0 : h.bin_sz[0] / linear_bin_vol(h.gmin[0], h.bin_sz[0], b0);
                w *= h.bin_sz[1] == 0.0 ? 1.0 : h.bin_sz[1] / linear_bin_vol(h.gmin[1], h.bin_sz[1], b1);
            }
            // row index times the row's length, as the reference indexes
            // (hgram.rs:407: bin[1] * nbins[1] + bin[0])
            fbin = b1 * h.nbins[1] + b0;
        }
        if (fbin < ncts) {
            if (shared)
                atomicAdd(&sc[fbin], w);
            else
                atomicAdd(&counts[fbin], w);
        }
    }
    if (shared) {
        __syncthreads();
        for (unsigned long long k = threadIdx.x; k < ncts; k += blockDim.x)
            if (sc[k] != 0.0) atomicAdd(&counts[k], sc[k]);
    }
}

// Summary-statistic sums (output/stats.rs:265-410): per block, [total,
// subtotal, count, min, max, sum of w (v - shift), sum of w (v - shift)^2,
// sum of w cos v, sum of w sin v].
__global__ void __launch_bounds__(256) k_particle_sums(HgramArgs h, double shift, double* partials) {
    __shared__ double sh[9][8];
    double a[9] = {0.0, 0.0, 0.0, HUGE_VAL, -HUGE_VAL, 0.0, 0.0, 0.0, 0.0};
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < h.n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        if (h.species[i] != h.want_species) continue;
        double v = out_value(h, i, h.func[0]), w = out_value(h, i, h.func[1]);
        double vw = v * w;
        a[0] += vw;
        bool within = true;
        if (h.filter_func >= 0) {
            double f = out_value(h, i, h.filter_func);
            within = f > h.fmin && f < h.fmax;
        }
        if (!within) continue;
        a[1] += vw;
        a[2] += w;
        if (vw < a[3]) a[3] = vw;
        if (vw > a[4]) a[4] = vw;
        double d = v - shift;
        a[5] += w * d;
        a[6] += w * (d * d);
        a[7] += w * cos(v);
        a[8] += w * sin(v);
    }
    for (int off = 16; off > 0; off >>= 1) {
        for (int k = 0; k < 9; ++k) {
            double o = __shfl_down_sync(0xffffffffu, a[k], off);
            a[k] = k == 3 ? fmin(a[k], o) : (k == 4 ? fmax(a[k], o) : a[k] + o);
        }
    }
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
        for (int k = 0; k < 9; ++k) sh[k][warp] = a[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 0; k < 9; ++k) {
            double o = sh[k][0];
            for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
                o = k == 3 ? fmin(o, sh[k][w]) : (k == 4 ? fmax(o, sh[k][w]) : o + sh[k][w]);
            partials[9 * blockIdx.x + k] = o;
        }
    }
}

cudaError_t launch_particle_sums(const HgramArgs& h, double shift, int blocks, double* partials, cudaStream_t s) {
    k_particle_sums<<<blocks, 256, 0, s>>>(h, shift, partials);
    return cudaGetLastError();
}

cudaError_t launch_hgram_stats(const HgramArgs& h, int blocks, double* partials, cudaStream_t s) {
    k_hgram_stats<<<blocks, 256, 0, s>>>(h, partials);
    return cudaGetLastError();
}

cudaError_t launch_hgram_fill(const HgramArgs& h, int blocks, double* counts, cudaStream_t s) {
    unsigned long long ncts = h.nbins[0] * (h.dim == 2 ? h.nbins[1] : 1ull);
    size_t smem = ncts <= 6144ull ? 8 * (size_t)ncts : 0;
    k_hgram_fill<<<blocks, 256, smem, s>>>(h, counts);
    return cudaGetLastError();
}

}  // namespace ptg
