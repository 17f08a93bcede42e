// LMA emission and pair creation for the PlaneWave and FocusedLaser models:
// the per-step probability at the local (a, eta) and, on an event, the
// sample and its kinematics.
#pragma once
#include "ptg_fields.cuh"
#include "ptg_math.cuh"
#include "ptg_bw.cuh"
#include "ptg_bw_lp.cuh"
#include "ptg_lp.cuh"
#include "ptg_mlp.cuh"
#include "ptg_nlc.cuh"

namespace ptg {

// Device pointers to the LMA rate and CDF tables (loaded from data files).
struct LmaTables {
    const double* nlc_lp_rate;      // [68][61] ln rate
    const double* nlc_lp_cdf;       // [4148][16][2]
    const double* nlc_cp_rate;      // [70][61] ln rate
    const double* nlc_cp_cdf;       // [4270][32][2] (regenerated)
    const double* nlc_lp_cl_rate;   // [61]
    const double* nlc_cp_cl_rate;   // [61]
    const double* bw_cp_total;      // [121][74][2]
    const double* bw_lp_total;      // [61][25][2]
    const double* bw_lp_cdf;        // [1525][16][3]
    const double* bw_lp_mid_total;  // [157][36][2]
    const double* bw_lp_mid_cdf;    // [5652][16][3] (regenerated)
    const double* nlc_cp_cl_cdf;    // [61][32][2]
    const double* nlc_lp_cl_cdf;    // [61][16][2]
    // FP32 copies of the two emission rate tables, for the per-step bound
    const float* nlc_lp_rate32;     // [68][61]
    const float* nlc_cp_rate32;     // [70][61]
    // nlc_cp_cdf's nodes as [ln n, ln(-ln(1 - cdf))], the coordinates its
    // inversion works in, evaluated once on the device at load
    const double* nlc_cp_cdf_log;   // [4270][32][2]
    // the CP Breit-Wheeler total-rate table's node positions in a (74) and
    // eta (121), computed once at load
    const double* bw_cp_nodes;
    // below the rate tables' smallest amplitude the emission rate is
    // a^2 K(eta) (cp: nonlinear_compton/cp/mod.rs:160-176; lp: the linear
    // rate of lp/mod.rs:459-553); upper bounds of K over SMALL_A_CELLS cells
    // of ln eta, in FP32, built at load (small_a_bounds)
    const float* nlc_cp_small32;    // [SMALL_A_CELLS]
    const float* nlc_lp_small32;    // [SMALL_A_CELLS]
};

// The cells of the small-amplitude bound tables: ln eta from ln 1e-3 (where
// both rates' formulas change) to ln 2.
constexpr int SMALL_A_CELLS = 512;
constexpr double SMALL_A_LN_ETA0 = -6.907755278982137;
constexpr double SMALL_A_LN_ETA1 = 0.6931471805599453;

// An upper bound on the emission rate where the amplitude lies below the
// rate table (ln a below ln_a_min by more than FP32 rounding): (float)a^2
// times the bound on K for eta's cell.  False where it does not certainly
// apply (then the FP64 rate is evaluated).  `a2` is the square of the
// amplitude the rate formula takes.
__device__ __forceinline__ bool rate32_small_a(const float* K32, float ln_a, float ln_a_min, double a2, double eta,
                                               float* out) {
    if (K32 == nullptr || !(ln_a < ln_a_min - 1e-5f) || !(a2 > 0.0) || !(eta > 0.0)) return false;
    const float L0 = (float)SMALL_A_LN_ETA0;
    const float INV = (float)(SMALL_A_CELLS / (SMALL_A_LN_ETA1 - SMALL_A_LN_ETA0));
    float x = (logf((float)eta) - L0) * INV;
    if (!(x > 1e-3f && x < (float)SMALL_A_CELLS - 1e-3f)) return false;
    *out = (float)a2 * K32[(int)x];
    return true;
}

// The per-step emission probability is first evaluated in FP32 from the
// FP32 rate tables (rate32_cp / rate32_lp).  Its relative error is below
// 2e-5: the logarithms of a and eta are within about 1e-6 and so the table
// coordinates within 2.1e-5 of a cell; the tables' ln-rate changes by at
// most 0.23 per cell and has magnitude at most 16, so the interpolated
// ln-rate is within 1.5e-5; expf and the products add under 1e-6.  Below
// the tables' smallest amplitude an upper bound takes its place
// (rate32_small_a: at least the rate, within 2^-8 plus K's variation over
// a cell of it, and within a few ulp of FP32 rounding).  A draw
// above the FP32 probability by more than 2^-10 of it is a step without an
// emission whatever the FP64 probability is; every other draw is decided
// against the FP64 probability, as the reference decides it.  The decisions
// are therefore the reference's, and the FP64 rate is evaluated on only
// about as many steps as emit.
constexpr double PROB32_MARGIN = 1.0 / 1024.0;

__device__ __forceinline__ NlcTables nlc_view(const LmaTables& t) {
    return NlcTables{t.nlc_lp_rate,    t.nlc_lp_cdf,     t.nlc_cp_rate,   t.nlc_cp_cdf,
                     t.nlc_cp_cl_rate, t.nlc_lp_cl_rate, t.nlc_cp_cl_cdf, t.nlc_lp_cl_cdf,
                     t.nlc_cp_cdf_log};
}

// Standard normal from two uniforms (Box-Muller), for the finite bandwidth.
__device__ __forceinline__ double std_normal(Draws& rng) {
    double u1 = rng.next(), u2 = rng.next();
    return sqrt(-2.0 * log(1.0 - u1)) * cos(2.0 * PI * u2);
}

// An LP emission sampled by its whole warp (the wave kernel): the lane
// records the emission's a, eta and draws and abandons the step; the warp
// samples it with lp_sample_warp; the lane then repeats the step, which
// reproduces everything up to the sample (same inputs, same draws), and
// takes the stored sample with the draws as they stood after it.
struct LpDefer {
    Draws rng;      // the draws at the sample; after it, once served
    double a, eta;  // amplitude (LP: the peak a sqrt 2) and eta of the emission
    double s, theta;
    d3 sv;
    int n, status;
    int pend;  // 0: none; 1: waiting for the warp; 2: served
    int circular;  // the emitting lane's laser polarisation
    uint32_t rej;
};

// lma_radiate's status for an emission left to the warp
constexpr int LMA_DEFERRED = 101;

// cp_ceiling (nonlinear_compton/cp/mod.rs:42-75) with its 32 points spread
// over the lanes of a converged warp; the NaN-ignoring maximum does not
// depend on the order, so every lane returns cp_ceiling's value.
__device__ __forceinline__ double cp_ceiling_warp(int n, double a, double eta) {
    const unsigned all = 0xffffffffu;
    const int lane = (int)(threadIdx.x & 31u);
    double mx = fmax(-HUGE_VAL, cp_diff_partial_rate(n, a, eta, cp_ceiling_point(n, a, eta, lane)));
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(all, mx, o));
    return 1.2 * mx;
}

// cp_sample_v_under (v and u per trial, accepted when u <= f(v) / mx) by the
// 32 lanes of a converged warp: the trials are dealt out in the order the
// serial sampler draws them, lane k evaluating the k-th of each round of
// 32; the first accepted trial in draw order is taken, with the draws as
// they stood after it.  Every lane returns the serial sampler's result.
__device__ __forceinline__ Jtrip shfl_jtrip(const Jtrip& t, int src) {
    const unsigned all = 0xffffffffu;
    return Jtrip{__shfl_sync(all, t.m, src), __shfl_sync(all, t.j, src), __shfl_sync(all, t.p, src)};
}

// `jt`, when not NULL, receives the accepted trial's Bessel triple.
static __device__ __noinline__ int cp_trials_warp(int n, double a, double eta, double mx, Draws& rng, double* v_out,
                                                  uint32_t* rej, Jtrip* jt = nullptr) {
    const unsigned all = 0xffffffffu;
    const int lane = (int)(threadIdx.x & 31u);
    Draws r = rng;
    for (int it0 = 0; it0 < r.cap; it0 += 32) {
        // this lane's trial: it0 + lane, after the 2 draws of each trial before it
        Draws my_r = r;
        my_r.skip(2 * lane);
        double vv = my_r.next(), u = my_r.next();
        Jtrip tj{0.0, 0.0, 0.0};
        bool acc = it0 + lane < r.cap && u <= cp_diff_partial_rate_j(n, a, eta, vv, &tj) / mx;
        unsigned m = __ballot_sync(all, acc);
        if (m != 0u) {
            int win = __ffs(m) - 1;
            *v_out = __shfl_sync(all, vv, win);
            Jtrip w = shfl_jtrip(tj, win);
            if (jt) *jt = w;
            rng = shfl_draws(my_r, win);
            *rej += (uint32_t)(it0 + win);
            return 0;
        }
        r = shfl_draws(my_r, 31);
    }
    rng = r;
    *rej += (uint32_t)r.cap;
    return 4;  // PTG_ERR_REJECTION_CAP
}

// cp_invert (nonlinear_compton/cp/tables/mod.rs:37-121) by a converged
// warp: the (up to) four grid corners are inverted on lanes 0-3 at once
// and combined in cp_invert's order and expression, so every lane returns
// cp_invert's harmonic.
static __device__ __noinline__ int cp_invert_warp(const NlcTables& t, double a, double eta, double frac) {
    const unsigned all = 0xffffffffu;
    const int lane = (int)(threadIdx.x & 31u);
    const double MIN0 = PTG_NLC_CP_MIN_0, MIN1 = PTG_NLC_CP_MIN_1, S0 = PTG_NLC_CP_STEP_0, S1 = PTG_NLC_CP_STEP_1;
    double la = log(a), le = log(eta);
    if (la <= MIN0) return 1;
    int ix = (int)((la - MIN0) / S0);
    double dx = (la - MIN0) / S0 - ix;
    bool edge = le <= MIN1;
    int iy = edge ? 0 : (int)((le - MIN1) / S1);
    double dy = edge ? 0.0 : (le - MIN1) / S1 - iy;
    // lane c < 4: corner (ix + (c & 1), iy + (c >> 1)); on the eta edge only
    // the two corners of row ix, ix + 1
    double v = 0.0;
    if (lane < (edge ? 2 : 4)) {
        size_t row = edge ? (size_t)(ix + lane) : (size_t)(61 * (iy + (lane >> 1)) + ix + (lane & 1));
        v = cp_cdf_corner(t.cp_cdf + row * 64, t.cp_cdf_log ? t.cp_cdf_log + row * 64 : nullptr, frac);
    }
    double c0 = __shfl_sync(all, v, 0), c1 = __shfl_sync(all, v, 1);
    double n;
    if (edge) {
        n = c0 * (1.0 - dx) + c1 * dx;
    } else {
        double c2 = __shfl_sync(all, v, 2), c3 = __shfl_sync(all, v, 3);
        n = c0 * ((1.0 - dx) * (1.0 - dy)) + c1 * (dx * (1.0 - dy)) + c2 * ((1.0 - dx) * dy) + c3 * (dx * dy);
    }
    return (int)ceil(n);
}

// cp_sample (nonlinear_compton/cp/mod.rs:181-234) carried out by all 32
// lanes of a converged warp for one emission whose a, eta and draws every
// lane holds.  Every lane returns the same result, and it is cp_sample's on
// the same draws: the harmonic comes from the same table inversion, the 32
// points of the ceiling are spread over the lanes (cp_ceiling_warp) and the
// rejection trials are dealt out over them (cp_trials_warp).
static __device__ __noinline__ int cp_sample_warp(const NlcTables& t, double a, double eta, Draws& rng, int* n_out,
                                                  double* s_out, double* theta_out, d3* sv_out, uint32_t* rej) {
    if (t.cp_cdf == nullptr) return 8;  // PTG_ERR_TABLES
    int n = cp_invert_warp(t, a, eta, rng.next());
    if (n < 1) n = 1;
    double mx = cp_ceiling_warp(n, a, eta);
    double v = 0.0;
    Jtrip jt;
    int st = cp_trials_warp(n, a, eta, mx, rng, &v, rej, &jt);
    if (st != 0) return st;
    cp_finish_j(n, a, eta, v, jt, rng, s_out, theta_out, sv_out);
    *n_out = n;
    return 0;
}

// One hidden layer of the warp forward pass: this lane's units l and l + 32
// from the 64 inputs `h` (the warp's scratch), in mlp_forward_lane's order.
__device__ __forceinline__ void mlp_hidden_warp(const uint32_t (*w)[32], const float* b, const float* h, float* out) {
    const int lane = (int)(threadIdx.x & 31u);
    float z0 = b[lane], z1 = b[lane + 32];
    const float4* h4 = reinterpret_cast<const float4*>(h);
#pragma unroll 4
    for (int q = 0; q < MLP_H / 4; ++q) {
        float4 v = h4[q];
        uint32_t w0 = w[4 * q][lane], w1 = w[4 * q + 1][lane], w2 = w[4 * q + 2][lane], w3 = w[4 * q + 3][lane];
        z0 += bf16_lo(w0) * v.x;
        z1 += bf16_hi(w0) * v.x;
        z0 += bf16_lo(w1) * v.y;
        z1 += bf16_hi(w1) * v.y;
        z0 += bf16_lo(w2) * v.z;
        z1 += bf16_hi(w2) * v.z;
        z0 += bf16_lo(w3) * v.w;
        z1 += bf16_hi(w3) * v.w;
    }
    out[lane] = silu(z0);
    out[lane + 32] = silu(z1);
}

// mlp_forward_lane by the 32 lanes of a converged warp from the network
// staged in shared memory (mlp_stage): lane l computes units l and l + 32
// of each hidden layer (and unit l of the output for l < 16) with the same
// products in the same order, so every lane returns the lane forward
// pass's outputs bit for bit.  `sh` is the warp's scratch of 2 x 64 floats
// in shared memory, 16-byte aligned.
static __device__ __noinline__ void mlp_forward_warp(const MlpShared& net, const float x[MLP_IN], float out[MLP_OUT],
                                                     float* sh) {
    const int lane = (int)(threadIdx.x & 31u);
    float* ha = sh;
    float* hb = sh + MLP_H;
    float z0 = net.b0[lane], z1 = net.b0[lane + 32];
    for (int i = 0; i < MLP_IN; ++i) {
        uint32_t w = net.w0[i][lane];
        z0 += bf16_lo(w) * x[i];
        z1 += bf16_hi(w) * x[i];
    }
    ha[lane] = silu(z0);
    ha[lane + 32] = silu(z1);
    __syncwarp();
    mlp_hidden_warp(net.w1, net.b1, ha, hb);
    __syncwarp();
    mlp_hidden_warp(net.w2, net.b2, hb, ha);
    __syncwarp();
    if (lane < MLP_OUT) {
        float z = net.b3[lane];
        for (int i = 0; i < MLP_H; ++i) z += __bfloat162float(net.w3[i][lane]) * ha[i];
        hb[lane] = z;
    }
    __syncwarp();
    for (int q = 0; q < MLP_OUT; ++q) out[q] = hb[q];
    __syncwarp();
}

// cp_sample_v_learned (ptg_mlp.cuh) by the 32 lanes of a converged warp,
// with the serial sampler's draws and results: in one round lanes 0-15
// evaluate the 16 trials under the learned envelope (trial k after the 3
// draws of each trial before it) while lane 16 evaluates f(v*), which
// scales the envelope; the first trial in draw order that accepts or finds
// the envelope under the spectrum decides.  The hand-over to the
// reference's sampler and the capped continuation run warp-wide too
// (cp_ceiling_warp, cp_trials_warp, and rounds of 32 capped trials).
static __device__ __noinline__ int cp_sample_v_learned_warp(const float o[MLP_OUT], float margin, int n, double a,
                                                            double eta, Draws& rng, double* v_out, uint32_t* rej,
                                                            Jtrip* jt) {
    const unsigned all = 0xffffffffu;
    const int lane = (int)(threadIdx.x & 31u);
    double sn = 2.0 * n * eta / (1.0 + a * a);
    double v_star = (1.0 + sn) / (2.0 + sn);
    // the trial round: lanes 0-15 draw their trial, the others take v*;
    // the spectrum is then evaluated at one call site by every lane (one
    // pass of the warp), f(v*) read from lane LEARNED_TRIALS
    Draws after_v = rng;
    int k = 0;
    double v = v_star, u = 0.0;
    Envelope e;
    float o_max = envelope_shape(o, &e);
    if (lane < LEARNED_TRIALS) {
        after_v.skip(3 * lane);
        v = envelope_draw(e, after_v, &k);
    }
    Draws after_u = after_v;
    if (lane < LEARNED_TRIALS) u = after_u.next();
    Jtrip tj;
    double f = cp_diff_partial_rate_j(n, a, eta, v, &tj);
    double f_star = __shfl_sync(all, f, LEARNED_TRIALS);
    if (!envelope_scale(&e, o_max, margin, f_star)) {
        // unusable envelope: the reference's sampler from the first draw
        return cp_trials_warp(n, a, eta, cp_ceiling_warp(n, a, eta), rng, v_out, rej, jt);
    }
    double g = e.scale * (double)e.w[k];
    bool viol = lane < LEARNED_TRIALS && f > g;
    bool acc = lane < LEARNED_TRIALS && !viol && u * g < f;
    unsigned m = __ballot_sync(all, viol || acc);
    if (m != 0u) {
        int j = __ffs(m) - 1;
        *rej += (uint32_t)j;
        if (__shfl_sync(all, (int)viol, j)) {
            // the envelope is under the spectrum: the reference's sampler takes over
            rng = shfl_draws(after_v, j);
            return cp_trials_warp(n, a, eta, cp_ceiling_warp(n, a, eta), rng, v_out, rej, jt);
        }
        rng = shfl_draws(after_u, j);
        *v_out = __shfl_sync(all, v, j);
        *jt = shfl_jtrip(tj, j);
        return 0;
    }
    rng = shfl_draws(after_u, LEARNED_TRIALS - 1);
    *rej += LEARNED_TRIALS;
    // cp_sample_v_capped: rejection under min(envelope, ceiling)
    double ceil = cp_ceiling_warp(n, a, eta);
    unsigned capped = envelope_cap(&e, ceil);
    Draws r = rng;
    for (int it0 = 0; it0 < r.cap; it0 += 32) {
        Draws my_r = r;
        my_r.skip(3 * lane);
        int kb;
        double vb = envelope_draw(e, my_r, &kb);
        Jtrip tb;
        double fb = cp_diff_partial_rate_j(n, a, eta, vb, &tb);
        double gb = e.scale * (double)e.w[kb];
        int dec = 0;  // 1: accepted under the cap; 2: envelope under the spectrum; 3: accepted
        if (fb > gb) {
            dec = (capped & (1u << kb)) ? 1 : 2;
        } else if (my_r.next() * gb < fb) {
            dec = 3;
        }
        unsigned mb = __ballot_sync(all, it0 + lane < r.cap && dec != 0);
        if (mb != 0u) {
            int j = __ffs(mb) - 1;
            rng = shfl_draws(my_r, j);
            *rej += (uint32_t)(it0 + j);
            if (__shfl_sync(all, dec, j) == 2) return cp_trials_warp(n, a, eta, ceil, rng, v_out, rej, jt);
            *v_out = __shfl_sync(all, vb, j);
            *jt = shfl_jtrip(tb, j);
            return 0;
        }
        r = shfl_draws(my_r, 31);
    }
    rng = r;
    *rej += (uint32_t)r.cap;
    return 4;  // PTG_ERR_REJECTION_CAP
}

// The learned CP emission sampler: the harmonic by the table inversion
// (the same draw as cp_sample), v from the learned envelope with the exact
// accept/reject against the spectrum (ptg_mlp.cuh) from harmonic
// mlp.min_harmonic up and with the reference's sampler below it, then
// cp_finish.  On this lane alone.
static __device__ __noinline__ int cp_sample_learned_lane(const MlpParams& mlp, const NlcTables& t, double a, double eta,
                                                          Draws& rng, int* n_out, double* s_out, double* theta_out,
                                                          d3* sv_out, uint32_t* rej) {
    int n = cp_invert(t, a, eta, rng.next());
    if (n < 1) n = 1;
    double v = 0.0;
    Jtrip jt;
    int st;
    if (n < mlp.min_harmonic) {
        // a low harmonic: the reference's ceiling costs less than the network
        st = cp_sample_v(n, a, eta, rng, &v, rej, &jt);
    } else {
        float x[MLP_IN], o[MLP_OUT];
        mlp_features(a, eta, n, x);
        mlp_forward_lane(mlp, x, o);
        LearnedCounts lc{0, 0, 0, 0};
        st = cp_sample_v_learned(o, mlp.margin, n, a, eta, rng, &v, rej, &lc, &jt);
    }
    if (st == 0) cp_finish_j(n, a, eta, v, jt, rng, s_out, theta_out, sv_out);
    *n_out = n;
    return st;
}

// The same by the 32 lanes of a converged warp, with the same draws and
// results, from the network staged in shared memory (mlp_stage); `sh` is
// the warp's scratch.
static __device__ __noinline__ int cp_sample_learned_warp(const MlpShared& net, const MlpParams& mlp,
                                                          const NlcTables& t, float* sh, double a, double eta,
                                                          Draws& rng, int* n_out, double* s_out, double* theta_out,
                                                          d3* sv_out, uint32_t* rej) {
    int n = cp_invert_warp(t, a, eta, rng.next());
    if (n < 1) n = 1;
    double v = 0.0;
    Jtrip jt;
    int st;
    if (n < mlp.min_harmonic) {
        st = cp_trials_warp(n, a, eta, cp_ceiling_warp(n, a, eta), rng, &v, rej, &jt);
    } else {
        float x[MLP_IN], o[MLP_OUT];
        mlp_features(a, eta, n, x);
        mlp_forward_warp(net, x, o, sh);
        st = cp_sample_v_learned_warp(o, mlp.margin, n, a, eta, rng, &v, rej, &jt);
    }
    if (st == 0) cp_finish_j(n, a, eta, v, jt, rng, s_out, theta_out, sv_out);
    *n_out = n;
    return st;
}

// The quantum emission rate in FP32 where it certainly applies (the table,
// or the bound below the table's smallest amplitude), from a^2 = u.u - 1
// and eta; false elsewhere.  `circular` selects the CP rate at the rms
// amplitude or the LP rate at the peak amplitude a sqrt 2.
__device__ __forceinline__ bool emission_rate32(const LmaTables& t, bool circular, double a2, double eta, float* r32) {
    // a^2 at or below zero: the rounding of u.u - 1 where <a^2> is below
    // about 1e-7 (u^0 ~ 3e4 in the pulse's wings).  The rate is then that of
    // a = 0 (nonlinear_compton/mod.rs:22-27), which is zero in every branch
    // for 0 < eta < 2, so the step cannot emit.
    if (a2 <= 0.0 && eta > 0.0 && eta < 2.0) {
        *r32 = 0.0f;
        return true;
    }
    float ln_a = 0.5f * logf((float)a2);
    if (circular)
        return rate32_cp(t.nlc_cp_rate32, ln_a, eta, r32) ||
               rate32_small_a(t.nlc_cp_small32, ln_a, (float)PTG_NLC_CP_MIN_0, a2, eta, r32);
    float ln_pk = ln_a + 0.34657359f;  // ln sqrt 2
    return rate32_lp(t.nlc_lp_rate32, ln_pk, eta, r32) ||
           rate32_small_a(t.nlc_lp_small32, ln_pk, (float)PTG_NLC_LP_MIN_0, 2.0 * a2, eta, r32);
}

// plane_wave.rs:251-282 / focused_laser.rs:260-281 with
// nonlinear_compton::probability (mod.rs:19-47) and generate (mod.rs:58-138).
// `dbw` is this lane's DoubleBessel workspace (linear polarisation only).
// Returns a ptg status (0 = ok).
static __device__ __noinline__ int lma_radiate(const FieldParams& f, const LmaTables& t, const DbWork& dbw,
                                               const MlpParams& mlp, d4 r, d4 u, double dt, Draws& rng, bool classical,
                                               bool* emitted, d4* k_out, d4* u_prime, d3* pol, double* a_eff,
                                               double* chi, double* absorption, uint32_t* rej,
                                               LpDefer* dfr = nullptr) {
    *emitted = false;
    double chirp = 1.0;
    if (f.model == M_PLANE_WAVE && f.chirp_b != 0.0) {
        chirp = 1.0 + 2.0 * f.chirp_b * phase_of(f, r);
        if (chirp < 0.0 && lma_a_sqd(f, r) > 0.0) return 3;  // PTG_ERR_SANITY
    }
    double width = 1.0;
    if (f.bandwidth != 0.0) {
        width = 1.0 + f.bandwidth * std_normal(rng);
        if (!(width > 0.0)) return 3;
    }
    double kk = SPEED_OF_LIGHT * COMPTON_TIME * f.k * chirp * width;
    d4 kappa = d4{kk, 0.0, 0.0, kk};
    double a2 = dot4(u, u) - 1.0;
    double eta = dot4(kappa, u);
    // the event draw, then the FP32 bound on the probability: a draw well
    // above it is a step without an emission (see PROB32_MARGIN); ln a is
    // taken in FP32 from a^2 (within 1e-7 of ln of the FP64 a)
    double u_event = rng.next();
    if (!classical) {
        float r32;
        bool in32 = emission_rate32(t, f.circular, a2, eta, &r32);
        if (in32) {
            float p32 = (float)(ALPHA_FINE / COMPTON_TIME) * r32 * ((float)dt / (float)u.t);
            if (u_event > (double)p32 * (1.0 + PROB32_MARGIN)) return 0;
        }
    }
    double aq = a2 >= 0.0 ? sqrt(a2) : 0.0;
    double dphi = dt * eta / (COMPTON_TIME * u.t);
    NlcTables nt = nlc_view(t);
    double rate;
    bool ok;
    if (f.circular)
        ok = classical ? cp_classical_rate(nt, aq, eta, &rate) : cp_rate(nt, aq, eta, &rate);
    else
        ok = classical ? lp_classical_rate(nt, aq * SQRT_2, eta, &rate) : lp_rate(nt, aq * SQRT_2, eta, &rate);
    if (!ok) return 2;  // PTG_ERR_OUT_OF_TABLE
    double prob = ALPHA_FINE * rate * dphi / eta;
    if (u_event < prob) {
        int n;
        double s, cphi;
        d3 sv;
        int st;
        if (f.circular && !classical && dfr != nullptr) {
            // the CP sampler (the reference's, or the learned proposal when
            // it is on), carried out by the whole warp
            if (dfr->pend == 2) {
                n = dfr->n, s = dfr->s, cphi = dfr->theta, sv = dfr->sv, st = dfr->status;
                *rej += dfr->rej;
                rng = dfr->rng;
                dfr->pend = 0;
            } else {
                dfr->rng = rng;
                dfr->a = aq;
                dfr->eta = eta;
                dfr->circular = 1;
                dfr->pend = 1;
                return LMA_DEFERRED;
            }
        } else if (f.circular && !classical && mlp.enabled) {
            st = cp_sample_learned_lane(mlp, nt, aq, eta, rng, &n, &s, &cphi, &sv, rej);
        } else if (f.circular)
            st = classical ? cp_classical_sample(nt, aq, eta, rng, &n, &s, &cphi, &sv, rej)
                           : cp_sample(nt, aq, eta, rng, &n, &s, &cphi, &sv, rej);
        else if (classical)
            st = lp_classical_sample(nt, dbw, aq * SQRT_2, eta, rng, &n, &s, &cphi, &sv, rej);
        else if (dfr == nullptr)
            st = lp_sample(nt, dbw, aq * SQRT_2, eta, rng, &n, &s, &cphi, &sv, rej);
        else if (dfr->pend == 2) {
            n = dfr->n, s = dfr->s, cphi = dfr->theta, sv = dfr->sv, st = dfr->status;
            *rej += dfr->rej;
            rng = dfr->rng;
            dfr->pend = 0;
        } else {
            dfr->rng = rng;
            dfr->a = aq * SQRT_2;
            dfr->eta = eta;
            dfr->circular = 0;
            dfr->pend = 1;
            return LMA_DEFERRED;
        }
        if (st != 0) return st;
        d4 k;
        st = nlc_kinematics(kappa, u, aq, eta, n, s, cphi, sv, f.pol_angle, classical, &k, pol);
        if (st != 0) return st;
        *k_out = k;
        *u_prime = d4{u.t + n * kappa.t - k.t, u.x + n * kappa.x - k.x, u.y + n * kappa.y - k.y, u.z + n * kappa.z - k.z};
        // the local amplitude, needed only for the photon's record
        double a = sqrt(lma_asq(f, r));
        *a_eff = a;
        *chi = a * dot4(u, kappa);
        *absorption = n * kappa.t;
        *emitted = true;
    }
    return 0;
}

// pair_creation/mod.rs:21-42 (LP): probability and Stokes update, peak
// amplitude a sqrt 2 for the tables
static __device__ __noinline__ bool lp_bw_probability(const LmaTables& t, d4 ell, d4 sv_in, d4 k, double a, double dt,
                                                      double pol_angle, double* prob, d4* sv_out) {
    double eta = dot4(k, ell);
    StokesBasis bs = lma_stokes_basis(ell);
    d3 g0 = stokes_rotate_cs(mk3(sv_in.x, sv_in.y, sv_in.z), bs.c2, bs.s2);
    d4 sv = stokes_rotate_by(d4{sv_in.t, g0.x, g0.y, g0.z}, pol_angle);
    double dphi = eta * dt / (COMPTON_TIME * ell.t);
    double f[2];
    if (!lpp_rates(t.bw_lp_total, t.bw_lp_mid_total, a * SQRT_2, eta, f)) return false;
    double f0 = f[0], f1 = f[1];
    double c = ALPHA_FINE * dphi / eta;
    double p = c * (0.5 * ((f0 + f1) + sv.x * (f0 - f1)));
    double p_avg = c * (0.5 * (f0 + f1));
    double delta = c * (0.5 * (f0 - f1));
    d4 o = d4{sv.t, (sv.x * (1.0 - p_avg) - delta) / (1.0 - p), sv.y * (1.0 - p_avg) / (1.0 - p),
              sv.z * (1.0 - p_avg) / (1.0 - p)};
    o = stokes_rotate_by(o, -pol_angle);
    d3 g = stokes_rotate_cs(mk3(o.x, o.y, o.z), bs.c2, -bs.s2);
    *sv_out = d4{o.t, g.x, g.y, g.z};
    *prob = p;
    return true;
}

// pair_creation/mod.rs:49-110 (LP)
static __device__ __noinline__ int lp_bw_generate(const LmaTables& t, const DbWork& w, d4 ell, d4 sv_in, d4 k, double a,
                                                  double pol_angle, Draws& rng, int* n_out, d4* q_out, uint32_t* rej) {
    double eta = dot4(k, ell);
    d4 sv = stokes_rotate_by(stokes_in_lma_basis(sv_in, ell), pol_angle);
    int n;
    double s, cphi;
    int st = lpp_sample(t.bw_lp_cdf, t.bw_lp_mid_cdf, t.bw_lp_mid_total, w, a * SQRT_2, eta, sv.x, sv.y, rng, &n, &s,
                        &cphi, rej);
    if (st != 0) return st;
    *n_out = n;
    return bw_kinematics(ell, k, a, pol_angle, n, s, cphi, q_out);
}

// plane_wave.rs:284-316 / focused_laser.rs:283-306 with
// pair_creation::probability and generate (pair_creation/mod.rs:21-110).
static __device__ __noinline__ int lma_pair_create(const FieldParams& f, const LmaTables& t, const DbWork& dbw, d4 r,
                                                   d4 ell, d4 pol, double dt, Draws& rng, double rate_increase,
                                                   double* prob, d4* pol_new, bool* created, d4* ue, d4* up,
                                                   double* frac, double* a_eff, double* chi, double* absorption,
                                                   uint32_t* rej, BwDefer* bdf = nullptr) {
    *prob = 0.0;
    *pol_new = pol;
    *created = false;
    double a = sqrt(lma_asq(f, r));
    double chirp = 1.0;
    if (f.model == M_PLANE_WAVE) {
        chirp = 1.0 + 2.0 * f.chirp_b * phase_of(f, r);
        if (chirp < 0.0 && a > 0.0) return 3;
    }
    double kk = SPEED_OF_LIGHT * COMPTON_TIME * f.k * chirp;
    d4 kappa = d4{kk, 0.0, 0.0, kk};
    if (f.circular) {
        int ok = bw_probability(t.bw_cp_total, ell, pol, kappa, a, dt, f.pol_angle, prob, pol_new, rate_increase, bdf,
                                t.bw_cp_nodes);
        if (ok == BW_DEFERRED) return LMA_DEFERRED;  // the step repeats once the warp has summed
        if (!ok) return 2;
    } else if (!lp_bw_probability(t, ell, pol, kappa, a, dt, f.pol_angle, prob, pol_new)) {
        return 2;
    }
    double ri = (*prob * rate_increase > 0.1) ? 0.1 / *prob : rate_increase;
    if (rng.next() < *prob * ri) {
        int n;
        d4 q;
        int st = f.circular ? bw_generate(t.bw_cp_total, ell, pol, kappa, a, f.pol_angle, rng, &n, &q, rej, bdf)
                            : lp_bw_generate(t, dbw, ell, pol, kappa, a, f.pol_angle, rng, &n, &q, rej);
        if (st == BW_DEFERRED) return LMA_DEFERRED;  // the step repeats once the warp has sampled the harmonic
        if (st != 0) return st;
        *ue = d4{ell.t + n * kappa.t - q.t, ell.x + n * kappa.x - q.x, ell.y + n * kappa.y - q.y, ell.z + n * kappa.z - q.z};
        *up = q;
        *frac = 1.0 / ri;
        *a_eff = a;
        *chi = a * dot4(ell, kappa);
        *absorption = n * kappa.t;
        *created = true;
    }
    return 0;
}

}  // namespace ptg
