// Device math for the collision-loop kernels: physical constants, small
// vector types, the counter-based random streams and pwmci.
//
// Constants are ptarmigan's (src/constants.rs:4-30), which differ from
// CODATA in the last digits; using them keeps the physics comparable.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ptg {

constexpr double SPEED_OF_LIGHT = 2.997925e8;
constexpr double SPEED_OF_LIGHT_SQD = 89875517873681764.0;
constexpr double ELECTRON_CHARGE = -1.602177e-19;
constexpr double ELEMENTARY_CHARGE = 1.602177e-19;
constexpr double ELECTRON_MASS = 9.109383e-31;
constexpr double ELECTRON_MASS_MEV = 0.510999;
constexpr double CRITICAL_FIELD = 1.323285e18;
constexpr double ALPHA_FINE = 7.29735257e-3;
constexpr double COMPTON_TIME = 1.28808867e-21;
constexpr double PI = 3.14159265358979323846;
constexpr double FRAC_PI_3 = 1.04719755119659774615;
constexpr double LN_2 = 0.693147180559945309417;
constexpr double SQRT_3 = 1.73205080756887729353;
constexpr double SQRT_2 = 1.41421356237309504880;

// Cap on every rejection loop: the reference's loops are unbounded; here a
// particle that exceeds the cap is retired with PTG_ERR_REJECTION_CAP.
constexpr int REJECTION_CAP = 1 << 16;

struct d3 {
    double x, y, z;
};
struct d4 {
    double t, x, y, z;
};

__host__ __device__ __forceinline__ d3 mk3(double x, double y, double z) { return d3{x, y, z}; }
__host__ __device__ __forceinline__ d3 operator+(d3 a, d3 b) { return d3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ __forceinline__ d3 operator-(d3 a, d3 b) { return d3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ __forceinline__ d3 operator-(d3 a) { return d3{-a.x, -a.y, -a.z}; }
__host__ __device__ __forceinline__ d3 operator*(double s, d3 a) { return d3{s * a.x, s * a.y, s * a.z}; }
__host__ __device__ __forceinline__ d3 operator/(d3 a, double s) { return d3{a.x / s, a.y / s, a.z / s}; }
__host__ __device__ __forceinline__ double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ d3 cross(d3 a, d3 b) {
    return d3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__host__ __device__ __forceinline__ double norm_sqr(d3 a) { return dot(a, a); }
__device__ __forceinline__ d3 normalize(d3 a) { return a / sqrt(norm_sqr(a)); }

// Right-handed rotation about a unit axis (three_vector.rs:77-95)
__device__ __forceinline__ d3 rotate_around(d3 v, d3 a, double s, double c) {
    return d3{(c + a.x * a.x * (1.0 - c)) * v.x + (a.x * a.y * (1.0 - c) - a.z * s) * v.y +
                  (a.x * a.z * (1.0 - c) + a.y * s) * v.z,
              (a.y * a.x * (1.0 - c) + a.z * s) * v.x + (c + a.y * a.y * (1.0 - c)) * v.y +
                  (a.y * a.z * (1.0 - c) - a.x * s) * v.z,
              (a.z * a.x * (1.0 - c) - a.y * s) * v.x + (a.z * a.y * (1.0 - c) + a.x * s) * v.y +
                  (c + a.z * a.z * (1.0 - c)) * v.z};
}

__device__ __forceinline__ double dsign(double v) { return signbit(v) ? -1.0 : 1.0; }

// Binary exponentiation, the lowering of Rust's f64::powi.
__device__ __forceinline__ double powi(double a, int b) {
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

// ------------------------------------------------------------------ RNG --
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).  Key = 64-bit run
// seed; counter = (step, block, stream_lo, stream_hi).  Every particle owns
// a 64-bit stream id fixed at creation, so its draws do not depend on which
// thread or wave runs it.
__device__ __forceinline__ uint4 philox(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ uint64_t primary_stream(uint64_t global_index) {
    return mix64(global_index + 0x9E3779B97F4A7C15ull);
}
__host__ __device__ __forceinline__ uint64_t child_stream(uint64_t parent, uint32_t step, uint32_t slot) {
    uint64_t tag = ((uint64_t)step << 2) | (uint64_t)slot;
    return mix64(parent + 0x9E3779B97F4A7C15ull * (tag + 1));
}

// Draws of one particle step.  Block b of step s yields two 53-bit
// uniforms in [0, 1).
struct Draws {
    uint32_t k0, k1, s_lo, s_hi, step, block;
    uint32_t w[4];
    int pos;
    int cap;  // iterations any rejection loop drawing from this stream may take
    __device__ __forceinline__ void begin(uint64_t seed, uint64_t stream, uint32_t st, int rej_cap = REJECTION_CAP) {
        k0 = (uint32_t)seed;
        k1 = (uint32_t)(seed >> 32);
        s_lo = (uint32_t)stream;
        s_hi = (uint32_t)(stream >> 32);
        step = st;
        block = 0;
        pos = 4;
        cap = rej_cap;
    }
    __device__ __forceinline__ double next() {
        if (pos >= 4) {
            uint4 o = philox(make_uint4(step, block, s_lo, s_hi), k0, k1);
            w[0] = o.x, w[1] = o.y, w[2] = o.z, w[3] = o.w;
            ++block;
            pos = 0;
        }
        uint64_t m = ((uint64_t)w[pos] << 21) | (uint64_t)(w[pos + 1] >> 11);
        pos += 2;
        return (double)m * (1.0 / 9007199254740992.0);
    }
    // The state after d more draws (d >= 0), with at most one block
    // generated.  Word index of the next draw: 4 (block - 1) + pos.
    __device__ __forceinline__ void skip(int d) {
        uint32_t at = 4u * block - 4u + (uint32_t)pos + 2u * (uint32_t)d;
        uint32_t b = at >> 2;
        if ((at & 3u) == 0u) {
            block = b;  // the next draw starts block b
            pos = 4;
        } else if (b + 1u != block) {
            uint4 o = philox(make_uint4(step, b, s_lo, s_hi), k0, k1);
            w[0] = o.x, w[1] = o.y, w[2] = o.z, w[3] = o.w;
            block = b + 1u;
            pos = 2;
        } else {
            pos = 2;  // the second draw of the block already in w
        }
    }
};

// ---------------------------------------------------------------- pwmci --
// Piecewise monotonic cubic interpolation over rows of [x, f]
// (pwmci.rs:47-306).  The segment search is the reference's reverse scan;
// tables are 15-41 rows.
struct PwFit {
    double x0, x1, f0, f1, m0, m1;
    __device__ __forceinline__ double eval(double x) const {
        double t = (x - x0) / (x1 - x0);
        double omt = 1.0 - t;
        double h00 = (1.0 + 2.0 * t) * (omt * omt);
        double h10 = t * (omt * omt);
        double h01 = (t * t) * (3.0 - 2.0 * t);
        double h11 = (t * t) * (t - 1.0);
        return f0 * h00 + f1 * h01 + (x1 - x0) * (m0 * h10 + m1 * h11);
    }
};

__device__ __forceinline__ PwFit pw_fit(int i, const double* tb, int len) {
    double s0, s1, s2;
    s1 = (tb[2 * i + 1] - tb[2 * i - 1]) / (tb[2 * i] - tb[2 * i - 2]);
    s0 = (i == 1) ? s1 : (tb[2 * i - 1] - tb[2 * i - 3]) / (tb[2 * i - 2] - tb[2 * i - 4]);
    s2 = (i == len - 1) ? s1 : (tb[2 * i + 3] - tb[2 * i + 1]) / (tb[2 * i + 2] - tb[2 * i]);
    double m0 = (s0 * s1 > 0.0) ? 0.5 * (s0 + s1) : 0.0;
    double m1 = (s1 * s2 > 0.0) ? 0.5 * (s1 + s2) : 0.0;
    if (s1 != 0.0 && m0 / s1 > 3.0) m0 = 3.0 * s1;
    if (s2 != 0.0 && m1 / s2 > 3.0) m1 = 3.0 * s2;
    return PwFit{tb[2 * i - 2], tb[2 * i], tb[2 * i - 1], tb[2 * i + 1], m0, m1};
}

// Returns -1 below, 0 within, +1 above; *i is the upper row of the segment.
__device__ __forceinline__ int pw_locate(const double* tb, int len, int col, double v, int* i) {
    int found = -1;
    for (int k = len - 1; k >= 0; --k) {
        if (v > tb[2 * k + col]) {
            found = k;
            break;
        }
    }
    if (found < 0) {
        *i = 1;
        return -1;
    }
    if (found == len - 1) {
        *i = len - 1;
        return 1;
    }
    *i = found + 1;
    return 0;
}

__device__ __forceinline__ bool pw_evaluate(const double* tb, int len, bool ext, double x, double* out) {
    int i;
    int loc = pw_locate(tb, len, 0, x, &i);
    if (loc == 0) {
        *out = pw_fit(i, tb, len).eval(x);
        return true;
    }
    if (!ext) return false;
    double x1 = tb[2 * i - 2], f1 = tb[2 * i - 1], x2 = tb[2 * i], f2 = tb[2 * i + 1];
    *out = f1 + (f2 - f1) * (x - x1) / (x2 - x1);
    return true;
}

__device__ __forceinline__ bool pw_between(double x, double mn, double mx) {
    if (mn < mx) return x > mn && x < mx;
    if (mx < mn) return x > mx && x < mn;
    return true;
}

// pwmci.rs:102-229: inverse quadratic interpolation with secant and
// bisection fall-backs, at most 32 iterations, relative tolerance 1e-6.
static __device__ __noinline__ bool pw_invert(const double* tb, int len, bool ext, double f, double* out) {
    int i;
    int loc = pw_locate(tb, len, 1, f, &i);
    if (loc != 0) {
        if (!ext) return false;
        double x1 = tb[2 * i - 2], f1 = tb[2 * i - 1], x2 = tb[2 * i], f2 = tb[2 * i + 1];
        *out = x1 + (f - f1) * (x2 - x1) / (f2 - f1);
        return true;
    }
    PwFit fit = pw_fit(i, tb, len);
    double rx0 = tb[2 * i - 2], rf0 = tb[2 * i - 1] - f;
    double rx1 = tb[2 * i], rf1 = tb[2 * i + 1] - f;
    if (fabs(rf1) < fabs(rf0)) {
        double tx = rx0, tf = rf0;
        rx0 = rx1, rf0 = rf1, rx1 = tx, rf1 = tf;
    }
    double rx2 = rx1, rf2 = rf1, rx3 = 0.0;
    bool prev_bisect = false;
    for (int it = 0; it < 32; ++it) {
        double s;
        if (rf0 != rf2 && rf1 != rf2) {
            double r = rf0 / rf2, ss = rf0 / rf1, t = rf1 / rf2;
            double p = ss * (t * (r - t) * (rx2 - rx0) - (1.0 - r) * (rx0 - rx1));
            double q = (t - 1.0) * (r - 1.0) * (ss - 1.0);
            s = rx0 + p / q;
        } else {
            s = rx0 - (rf0 * (rx0 - rx1) / (rf0 - rf1));
        }
        if (!pw_between(s, 0.25 * (3.0 * rx1 + rx0), rx0) ||
            (prev_bisect && fabs(s - rx0) >= 0.5 * fabs(rx0 - rx2)) ||
            (!prev_bisect && fabs(s - rx0) >= 0.5 * fabs(rx2 - rx3))) {
            prev_bisect = true;
            s = 0.5 * (rx0 + rx1);
        } else {
            prev_bisect = false;
        }
        rx3 = rx2;
        rx2 = rx0;
        rf2 = rf0;
        rx0 = s;
        rf0 = fit.eval(s) - f;
        if (rf1 * rf0 >= 0.0) {
            rx1 = rx0, rf1 = rf0;
            rx0 = rx2, rf0 = rf2;
        }
        if (fabs(rf1) < fabs(rf0)) {
            double tx = rx0, tf = rf0;
            rx0 = rx1, rf0 = rf1, rx1 = tx, rf1 = tf;
        }
        double err = fabs(rx1 - rx0) / fabs(rx0);
        if (err < 1.0e-6 || rf0 == 0.0) break;
    }
    *out = rx0;
    return true;
}

}  // namespace ptg
