// Learned proposal for the CP nonlinear-Compton energy sampler.
//
// The reference samples v = s / s_max at harmonic n by rejection under a
// flat ceiling that costs 32 evaluations of the spectrum
// (nonlinear_compton/cp/mod.rs:42-70) before the first trial.  Here a small
// MLP (six features of a, eta and n; 4 layers of width 64, SiLU; BF16
// weights, FP32 accumulation) predicts, for 16 equal bins of v, an upper
// envelope of ln f(v) relative to ln f at v* = (1 + s_n) / (2 + s_n).  The
// sampler draws a bin in proportion to the envelope, v uniformly inside it,
// and accepts with probability f(v) / g(v) against the exact spectrum f,
// so accepted v follow f exactly wherever g >= f.  A proposal with f > g
// (the envelope under the spectrum) is detected and the emission is handed
// to the reference's own sampler, as is one that finds no acceptance within
// a fixed number of trials.
#pragma once
#include <cuda_bf16.h>

#include "ptg_nlc.cuh"

namespace ptg {

enum { MLP_IN = 6, MLP_H = 64, MLP_OUT = 16, MLP_IN_PAD = 16 };

// Lowest training target (ln of the envelope relative to f(v*)).
constexpr float MLP_TARGET_FLOOR = -24.0f;

// Device view of the network: row-major [out][in] BF16 weights (input of
// layer 0 padded to 16), FP32 biases.
struct MlpParams {
    const __nv_bfloat16 *w0, *w1, *w2, *w3;  // [64][16], [64][64], [64][64], [16][64]
    const float *b0, *b1, *b2, *b3;          // [64], [64], [64], [16]
    float margin;                            // ln of the envelope's safety factor
    int enabled;
    int min_harmonic;  // the collision kernels propose v with the network from this harmonic up
};

// Inputs, each scaled to about [-1, 1] over a in [0.05, 20], eta in
// [1e-3, 2], n in [1, ~5e4]: ln a, ln eta, ln n, ln s_n (s_n = 2 n eta /
// (1 + a^2), which maps v to the Bessel argument), v*, and
// ln(n / (1 + a^2)^{3/2}), which sets how sharply J_n peaks in v.  In
// FP32 (the network is BF16): the same function makes the training
// samples' inputs and the samplers'.
__host__ __device__ __forceinline__ void mlp_features(double a, double eta, int n, float x[MLP_IN]) {
    float af = (float)a, ef = (float)eta, nf = (float)n;
    float ln_a = logf(af), ln_n = logf(nf), ln_1a2 = log1pf(af * af);
    float sn = 2.0f * nf * ef / (1.0f + af * af);
    x[0] = ln_a * (1.0f / 3.0f);
    x[1] = (logf(ef) + 3.1f) * (1.0f / 3.8f);
    x[2] = ln_n * (1.0f / 6.0f) - 1.0f;
    x[3] = logf(sn) * (1.0f / 6.0f);
    x[4] = 2.0f * (1.0f + sn) / (2.0f + sn) - 2.0f;
    x[5] = (ln_n - 1.5f * ln_1a2) * (1.0f / 6.0f);
}

// SiLU with the fast FP32 exponential and division (the network only
// shapes a proposal; both are within a few ulp)
__device__ __forceinline__ float silu(float z) { return __fdividef(z, 1.0f + __expf(-z)); }

// One lane's forward pass in FP32 (CUDA cores); used inside the collision
// kernels, where emissions arrive one lane at a time.
static __device__ __noinline__ void mlp_forward_lane(const MlpParams& m, const float x[MLP_IN], float out[MLP_OUT]) {
    float h0[MLP_H], h1[MLP_H];
    for (int o = 0; o < MLP_H; ++o) {
        float z = m.b0[o];
        for (int i = 0; i < MLP_IN; ++i) z += __bfloat162float(m.w0[o * MLP_IN_PAD + i]) * x[i];
        h0[o] = silu(z);
    }
    for (int o = 0; o < MLP_H; ++o) {
        float z = m.b1[o];
        for (int i = 0; i < MLP_H; ++i) z += __bfloat162float(m.w1[o * MLP_H + i]) * h0[i];
        h1[o] = silu(z);
    }
    for (int o = 0; o < MLP_H; ++o) {
        float z = m.b2[o];
        for (int i = 0; i < MLP_H; ++i) z += __bfloat162float(m.w2[o * MLP_H + i]) * h1[i];
        h0[o] = silu(z);
    }
    for (int o = 0; o < MLP_OUT; ++o) {
        float z = m.b3[o];
        for (int i = 0; i < MLP_H; ++i) z += __bfloat162float(m.w3[o * MLP_H + i]) * h0[i];
        out[o] = z;
    }
}

// The network staged in a block's shared memory for the warp forward pass
// (mlp_forward_warp): hidden layers input-major, with units l and l + 32
// of input i packed in one word (low and high BF16), so that for each input
// the 32 lanes read 32 consecutive words; the output layer input-major.
struct MlpShared {
    uint32_t w0[MLP_IN][32];
    uint32_t w1[MLP_H][32];
    uint32_t w2[MLP_H][32];
    __nv_bfloat16 w3[MLP_H][MLP_OUT];
    float b0[MLP_H], b1[MLP_H], b2[MLP_H], b3[MLP_OUT];
};

__device__ __forceinline__ uint32_t bf16_bits(__nv_bfloat16 v) { return (uint32_t)__bfloat16_as_ushort(v); }
// the two BF16 of a packed word as FP32 (exact, as __bfloat162float)
__device__ __forceinline__ float bf16_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t w) { return __uint_as_float(w & 0xffff0000u); }

// The block's staged network (one per block, shared by every call site).
__device__ __forceinline__ MlpShared* mlp_smem() {
    __shared__ MlpShared s_net;
    return &s_net;
}

// Copies the network into `s`: every thread of the block, then a barrier.
__device__ __forceinline__ void mlp_stage(const MlpParams& m, MlpShared* s) {
    for (int t = threadIdx.x; t < MLP_H * 32; t += blockDim.x) {
        int i = t >> 5, l = t & 31;
        if (i < MLP_IN)
            s->w0[i][l] = bf16_bits(m.w0[l * MLP_IN_PAD + i]) | (bf16_bits(m.w0[(l + 32) * MLP_IN_PAD + i]) << 16);
        s->w1[i][l] = bf16_bits(m.w1[l * MLP_H + i]) | (bf16_bits(m.w1[(l + 32) * MLP_H + i]) << 16);
        s->w2[i][l] = bf16_bits(m.w2[l * MLP_H + i]) | (bf16_bits(m.w2[(l + 32) * MLP_H + i]) << 16);
    }
    for (int t = threadIdx.x; t < MLP_H * MLP_OUT; t += blockDim.x) {
        int i = t / MLP_OUT, o = t % MLP_OUT;
        s->w3[i][o] = m.w3[o * MLP_H + i];
    }
    for (int t = threadIdx.x; t < MLP_H; t += blockDim.x) {
        s->b0[t] = m.b0[t];
        s->b1[t] = m.b1[t];
        s->b2[t] = m.b2[t];
        if (t < MLP_OUT) s->b3[t] = m.b3[t];
    }
    __syncthreads();
}

// Parameter vector (FP32 master copy, gradients, Adam moments).
enum : int {
    P_W0 = 0,
    P_W1 = P_W0 + MLP_H * MLP_IN_PAD,
    P_W2 = P_W1 + MLP_H * MLP_H,
    P_W3 = P_W2 + MLP_H * MLP_H,
    P_B0 = P_W3 + MLP_OUT * MLP_H,
    P_B1 = P_B0 + MLP_H,
    P_B2 = P_B1 + MLP_H,
    P_B3 = P_B2 + MLP_H,
    P_TOTAL = P_B3 + MLP_OUT
};

// Weights as the kernels read them: BF16, row-major [out][in] and the
// transposes [in][out] for the backward products.
struct MlpDev {
    __nv_bfloat16 *w0, *w1, *w2, *w3;
    __nv_bfloat16 *t1, *t2, *t3;  // W1^T [64][64], W2^T [64][64], W3^T [64][16]
    const float* p;               // FP32 master (biases read from here)
};

// Counters of the learned sampler.
struct LearnedCounts {
    uint32_t evals;      // spectrum evaluations
    uint32_t trials;     // proposals
    uint32_t fallbacks;  // envelope violations (the reference's sampler took over)
    uint32_t exhausted;  // no acceptance within LEARNED_TRIALS (the capped envelope took over)
};

// Proposals under the learned envelope alone before the sampler also
// computes the reference's ceiling C and continues under min(envelope, C).
// A capped run of independent trials followed by a valid sampler still
// returns v distributed as f, so the cap costs nothing in exactness; it
// bounds the work where the learned envelope is loose.
constexpr int LEARNED_TRIALS = 16;

// Lowest harmonic at which the collision kernels propose v with the network
// (ptg_mlp_min_harmonic); below it the reference's ceiling costs less.
constexpr int MLP_MIN_HARMONIC_DEFAULT = 1;

// The learned envelope of one emission: bin heights scale * w[k], w <= 1.
struct Envelope {
    double scale;
    float w[MLP_OUT];
    float total;
};

// The envelope's shape from the network's outputs o (ln heights relative
// to f(v*)): relative heights w and their total.  Returns max o.
__device__ __forceinline__ float envelope_shape(const float* o, Envelope* e) {
    float o_max = -HUGE_VALF;
    for (int q = 0; q < MLP_OUT; ++q) o_max = fmaxf(o_max, o[q]);
    e->total = 0.0f;
    for (int q = 0; q < MLP_OUT; ++q) {
        e->w[q] = __expf(o[q] - o_max);
        e->total += e->w[q];
    }
    return o_max;
}

// Its scale from f(v*).  Returns false when the envelope is unusable.
__device__ __forceinline__ bool envelope_scale(Envelope* e, float o_max, float margin, double f_star) {
    e->scale = f_star * exp((double)o_max + (double)margin);
    return f_star > 0.0 && isfinite(e->scale) && e->total > 0.0f;
}

// Both, from o and f(v*).
__device__ __forceinline__ bool envelope_from(const float* o, float margin, double f_star, Envelope* e) {
    return envelope_scale(e, envelope_shape(o, e), margin, f_star);
}

// The envelope capped at the flat ceiling c: heights min(scale * w, c);
// bit k of the result is set where the cap applies.
__device__ __forceinline__ unsigned envelope_cap(Envelope* e, double c) {
    double h[MLP_OUT], h_max = 0.0;
    unsigned capped = 0;
    for (int q = 0; q < MLP_OUT; ++q) {
        double v = e->scale * (double)e->w[q];
        if (v >= c) {
            v = c;
            capped |= 1u << q;
        }
        h[q] = v;
        h_max = fmax(h_max, v);
    }
    e->total = 0.0f;
    for (int q = 0; q < MLP_OUT; ++q) {
        e->w[q] = (float)(h[q] / h_max);
        e->total += e->w[q];
    }
    e->scale = h_max;
    return capped;
}

// A bin in proportion to the envelope's heights, and v uniformly in it.
__device__ __forceinline__ double envelope_draw(const Envelope& e, Draws& rng, int* bin) {
    float r = (float)rng.next() * e.total;
    int k = 0;
    float c = e.w[0];
    while (k < MLP_OUT - 1 && c <= r) c += e.w[++k];
    *bin = k;
    return ((double)k + rng.next()) * (1.0 / MLP_OUT);
}

// The reference's sampler taking over one emission; counts its spectrum
// evaluations (the 32-point ceiling and one per trial).
static __device__ __noinline__ int cp_hand_over(int n, double a, double eta, Draws& rng, double* v_out,
                                                uint32_t* rej, LearnedCounts* c, Jtrip* jt = nullptr) {
    uint32_t before = *rej;
    int st = cp_sample_v(n, a, eta, rng, v_out, rej, jt);
    c->evals += 32u + (*rej - before) + 1u;
    return st;
}

// After LEARNED_TRIALS rejections: the reference's ceiling c, then
// rejection under min(envelope, c).  Where the cap applies and f exceeds
// it, the reference's own rule (accept when u <= f / c) accepts; where the
// learned height applies and f exceeds it, the envelope is under the
// spectrum and the reference's sampler takes over with the same c.
static __device__ __noinline__ int cp_sample_v_capped(Envelope e, int n, double a, double eta, Draws& rng,
                                                      double* v_out, uint32_t* rej, LearnedCounts* c,
                                                      Jtrip* jt = nullptr) {
    double ceil = cp_ceiling(n, a, eta);
    c->evals += 32u;
    unsigned capped = envelope_cap(&e, ceil);
    for (int it = 0; it < rng.cap; ++it) {
        int k;
        double v = envelope_draw(e, rng, &k);
        Jtrip tj;
        double f = cp_diff_partial_rate_j(n, a, eta, v, &tj);
        c->evals += 1;
        double g = e.scale * (double)e.w[k];
        if (f > g) {
            if (capped & (1u << k)) {
                *v_out = v;
                if (jt) *jt = tj;
                *rej += it;
                return 0;
            }
            c->fallbacks += 1;
            *rej += it;
            uint32_t before = *rej;
            int st = cp_sample_v_under(n, a, eta, ceil, rng, v_out, rej, jt);
            c->evals += (*rej - before) + 1u;
            return st;
        }
        if (rng.next() * g < f) {
            *v_out = v;
            if (jt) *jt = tj;
            *rej += it;
            return 0;
        }
    }
    *rej += rng.cap;
    return 4;  // PTG_ERR_REJECTION_CAP
}

// v at harmonic n from the learned envelope `o` (16 log-heights relative
// to ln f(v*)).  Returns a ptg status.
static __device__ __noinline__ int cp_sample_v_learned(const float o[MLP_OUT], float margin, int n, double a, double eta,
                                                       Draws& rng, double* v_out, uint32_t* rej, LearnedCounts* c,
                                                       Jtrip* jt = nullptr) {
    double sn = 2.0 * n * eta / (1.0 + a * a);
    double v_star = (1.0 + sn) / (2.0 + sn);
    Jtrip jstar;
    double f_star = cp_diff_partial_rate_j(n, a, eta, v_star, &jstar);  // as the warp sampler evaluates it
    c->evals += 1;
    Envelope e;
    if (!envelope_from(o, margin, f_star, &e)) {
        c->fallbacks += 1;
        return cp_hand_over(n, a, eta, rng, v_out, rej, c, jt);
    }
    for (int it = 0; it < LEARNED_TRIALS; ++it) {
        int k;
        double v = envelope_draw(e, rng, &k);
        Jtrip tj;
        double f = cp_diff_partial_rate_j(n, a, eta, v, &tj);
        c->evals += 1;
        c->trials += 1;
        double g = e.scale * (double)e.w[k];
        if (f > g) {
            // the envelope is under the spectrum here
            c->fallbacks += 1;
            *rej += it;
            return cp_hand_over(n, a, eta, rng, v_out, rej, c, jt);
        }
        if (rng.next() * g < f) {
            *v_out = v;
            if (jt) *jt = tj;
            *rej += it;
            return 0;
        }
    }
    *rej += LEARNED_TRIALS;
    c->exhausted += 1;
    return cp_sample_v_capped(e, n, a, eta, rng, v_out, rej, c, jt);
}

}  // namespace ptg
