// Learned proposal for the CP nonlinear-Compton energy sampler.
//
// The reference samples v = s / s_max at harmonic n by rejection under a
// flat ceiling that costs 32 evaluations of the spectrum
// (nonlinear_compton/cp/mod.rs:42-70) before the first trial.  Here a small
// MLP (inputs ln a, ln eta, ln n; 4 layers of width 64, SiLU; BF16 weights,
// FP32 accumulation) predicts, for 16 equal bins of v, an upper envelope of
// ln f(v) relative to ln f at v* = (1 + s_n) / (2 + s_n).  The sampler draws
// a bin in proportion to the envelope, v uniformly inside it, and accepts
// with probability f(v) / g(v) against the exact spectrum f, so accepted v
// follow f exactly wherever g >= f.  A proposal with f > g (the envelope
// under the spectrum) is detected and the emission falls back to the
// reference's own sampler, so the distribution stays the reference's.
#pragma once
#include <cuda_bf16.h>

#include "ptg_nlc.cuh"

namespace ptg {

enum { MLP_IN = 3, MLP_H = 64, MLP_OUT = 16, MLP_IN_PAD = 16 };

// Device view of the network: row-major [out][in] BF16 weights (input of
// layer 0 padded to 16), FP32 biases.
struct MlpParams {
    const __nv_bfloat16 *w0, *w1, *w2, *w3;  // [64][16], [64][64], [64][64], [16][64]
    const float *b0, *b1, *b2, *b3;          // [64], [64], [64], [16]
    float margin;                            // ln of the envelope's safety factor
    int enabled;
};

// Normalised inputs: ln a in [ln 0.05, ln 20], ln eta in [ln 1e-3, ln 2],
// ln n in [0, ~12].
__host__ __device__ __forceinline__ void mlp_features(double a, double eta, int n, float x[3]) {
    x[0] = (float)(log(a) / 3.0);
    x[1] = (float)((log(eta) + 3.1) / 3.8);
    x[2] = (float)(log((double)n) / 6.0 - 1.0);
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }

// One lane's forward pass in FP32 (CUDA cores); used inside the collision
// kernels, where emissions arrive one lane at a time.
static __device__ __noinline__ void mlp_forward_lane(const MlpParams& m, const float x[3], float out[MLP_OUT]) {
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
    uint32_t fallbacks;  // envelope violations (fell back to the reference sampler)
};

// v at harmonic n from the learned envelope `o` (16 log-heights relative
// to ln f(v*)).  Falls back to cp_sample_v on a violation.  Returns a ptg
// status.
static __device__ __noinline__ int cp_sample_v_learned(const float o[MLP_OUT], float margin, int n, double a, double eta,
                                                       Draws& rng, double* v_out, uint32_t* rej, LearnedCounts* c) {
    double sn = 2.0 * n * eta / (1.0 + a * a);
    double v_star = (1.0 + sn) / (2.0 + sn);
    double f_star = cp_diff_partial_rate(n, a, eta, v_star);
    c->evals += 1;
    double base = log(f_star);
    if (!(f_star > 0.0) || !isfinite(base)) {
        c->fallbacks += 1;
        return cp_sample_v(n, a, eta, rng, v_out, rej);
    }
    double w[MLP_OUT], cum[MLP_OUT];
    double acc = 0.0;
    for (int k = 0; k < MLP_OUT; ++k) {
        w[k] = exp((double)o[k] + (double)margin);
        acc += w[k];
        cum[k] = acc;
    }
    for (int it = 0; it < REJECTION_CAP; ++it) {
        double u1 = rng.next() * acc;
        int k = 0;
        while (k < MLP_OUT - 1 && cum[k] <= u1) ++k;
        double v = ((double)k + rng.next()) * (1.0 / MLP_OUT);
        double f = cp_diff_partial_rate(n, a, eta, v);
        c->evals += 1;
        c->trials += 1;
        double g = exp(base) * w[k];
        if (f > g) {
            // the envelope is under the spectrum here: use the reference's sampler
            c->fallbacks += 1;
            *rej += it;
            return cp_sample_v(n, a, eta, rng, v_out, rej);
        }
        if (rng.next() * g < f) {
            *v_out = v;
            *rej += it;
            return 0;
        }
    }
    *rej += REJECTION_CAP;
    return 4;
}

}  // namespace ptg
