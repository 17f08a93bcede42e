// Training and batched inference of the learned CP proposal (ptg_mlp.cuh)
// on the tensor cores: BF16 operands, FP32 accumulation, warp-level
// mma.sync m16n8k16.  A warp carries 16 rows through the network; the
// accumulator fragments of one layer are, two n-tiles at a time, exactly
// the A fragments of the next layer, so activations never leave registers
// in the forward pass.  Weight gradients (dW = dZ^T H) take their
// transposed operands from shared memory.
//
// Also here: the training-data generator (table sampler draws of a, eta,
// n, one exact spectrum value per sample) and the sampler benchmark
// (plain reference sampler vs learned proposal, same a, eta, n).
#include <cuda_bf16.h>

#include <algorithm>

#include "ptg_launch.h"
#include "ptg_lma.cuh"
#include "ptg_mlp.cuh"

namespace ptg {

// One training sample: the network's inputs, the bin of v, the target
// (largest sampled ln f in the bin, relative to ln f(v*)).
struct MlpSample {
    float x[MLP_IN];
    int bin;
    float t;
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16(float d[4], const uint32_t a[4], const uint32_t b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// B fragment (k = 2t..2t+1 and 2t+8..2t+9, n = g) of a K x N operand whose
// element (k, n) is W[n * ld + k] (row-major [N][K], consecutive k).
__device__ __forceinline__ void load_b(const __nv_bfloat16* W, int ld, int kb, int nb, uint32_t b[2]) {
    int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const __nv_bfloat16* p = W + (size_t)(nb + g) * ld + kb + 2 * t;
    b[0] = *reinterpret_cast<const uint32_t*>(p);
    b[1] = *reinterpret_cast<const uint32_t*>(p + 8);
}

// Dense layer on a warp's 16 rows: z[ntile][4] = A . W^T + bias, A given as
// ktiles x 4 fragments.
template <int KT, int NT>
__device__ __forceinline__ void dense(const uint32_t a[KT][4], const __nv_bfloat16* W, int ld, const float* bias,
                                      float z[NT][4]) {
    int lane = threadIdx.x & 31, t = lane & 3;
    for (int nt = 0; nt < NT; ++nt) {
        float b0 = bias[nt * 8 + 2 * t], b1 = bias[nt * 8 + 2 * t + 1];
        z[nt][0] = b0, z[nt][1] = b1, z[nt][2] = b0, z[nt][3] = b1;
        for (int kt = 0; kt < KT; ++kt) {
            uint32_t b[2];
            load_b(W, ld, kt * 16, nt * 8, b);
            mma_bf16(z[nt], a[kt], b);
        }
    }
}

// Accumulator tiles (pairs of n-tiles) as the next layer's A fragments.
template <int NT>
__device__ __forceinline__ void to_a(const float h[NT][4], uint32_t a[NT / 2][4]) {
    for (int k = 0; k < NT / 2; ++k) {
        a[k][0] = pack_bf16(h[2 * k][0], h[2 * k][1]);
        a[k][1] = pack_bf16(h[2 * k][2], h[2 * k][3]);
        a[k][2] = pack_bf16(h[2 * k + 1][0], h[2 * k + 1][1]);
        a[k][3] = pack_bf16(h[2 * k + 1][2], h[2 * k + 1][3]);
    }
}

__device__ __forceinline__ void input_a(const float x[2][MLP_IN], uint32_t a[1][4]) {
    // 16 x 16 input tile, columns 0..MLP_IN-1 used (all below 8): this
    // lane holds columns 2t, 2t+1 of rows g (x[0]) and g + 8 (x[1])
    static_assert(MLP_IN <= 8, "the inputs fill the first half of the K tile");
    int t = threadIdx.x & 3;
    float c[2][2];
    for (int h = 0; h < 2; ++h)
        for (int q = 0; q < 2; ++q) {
            float v = 0.0f;
            for (int i = 0; i < MLP_IN; ++i) v = (2 * t + q == i) ? x[h][i] : v;
            c[h][q] = v;
        }
    a[0][0] = pack_bf16(c[0][0], c[0][1]);
    a[0][1] = pack_bf16(c[1][0], c[1][1]);
    a[0][2] = 0u;
    a[0][3] = 0u;
}

template <int NT>
__device__ __forceinline__ void silu_tiles(const float z[NT][4], float h[NT][4]) {
    for (int n = 0; n < NT; ++n)
        for (int q = 0; q < 4; ++q) h[n][q] = silu(z[n][q]);
}

__device__ __forceinline__ float dsilu(float z) {
    float s = __frcp_rn(1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

// Forward pass of a warp's 16 rows; keeps the pre-activations for backward.
struct WarpFwd {
    float z0[8][4], z1[8][4], z2[8][4], o[2][4];
};

__device__ __forceinline__ void warp_forward(const MlpDev& m, const float x[2][MLP_IN], WarpFwd& f) {
    uint32_t a0[1][4], a1[4][4];
    input_a(x, a0);
    dense<1, 8>(a0, m.w0, MLP_IN_PAD, m.p + P_B0, f.z0);
    float h[8][4];
    silu_tiles<8>(f.z0, h);
    to_a<8>(h, a1);
    dense<4, 8>(a1, m.w1, MLP_H, m.p + P_B1, f.z1);
    silu_tiles<8>(f.z1, h);
    to_a<8>(h, a1);
    dense<4, 8>(a1, m.w2, MLP_H, m.p + P_B2, f.z2);
    silu_tiles<8>(f.z2, h);
    to_a<8>(h, a1);
    dense<4, 2>(a1, m.w3, MLP_H, m.p + P_B3, f.o);
}

// Batched inference.  The weights are first packed in fragment order
// (k_mlp_pack): for every (k tile, n tile) of a layer, each lane's two
// 32-bit B fragments side by side, so that a warp reads a tile with one
// 8-byte load per lane, all 256 bytes contiguous.  Each block stages the
// packed weights (20 KB) and the biases in shared memory once and its warps
// then run 16-row tiles in a grid-stride loop.  The products and their
// order are those of warp_forward, so the outputs are the same bit for bit.
enum : int {
    PK_L0 = 0,                   // 1 x 8 tiles
    PK_L1 = PK_L0 + 1 * 8 * 32,  // 4 x 8 tiles
    PK_L2 = PK_L1 + 4 * 8 * 32,  // 4 x 8 tiles
    PK_L3 = PK_L2 + 4 * 8 * 32,  // 4 x 2 tiles
    PK_TOTAL = PK_L3 + 4 * 2 * 32
};

__global__ void k_mlp_pack(MlpDev m, uint2* packed) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= PK_TOTAL) return;
    int lane = idx & 31, tile = idx >> 5;
    const __nv_bfloat16* W;
    int ld, nt_count, local;
    if (idx < PK_L1) {
        W = m.w0, ld = MLP_IN_PAD, nt_count = 8, local = tile;
    } else if (idx < PK_L2) {
        W = m.w1, ld = MLP_H, nt_count = 8, local = tile - PK_L1 / 32;
    } else if (idx < PK_L3) {
        W = m.w2, ld = MLP_H, nt_count = 8, local = tile - PK_L2 / 32;
    } else {
        W = m.w3, ld = MLP_H, nt_count = 2, local = tile - PK_L3 / 32;
    }
    int kt = local / nt_count, nt = local % nt_count;
    int g = lane >> 2, t = lane & 3;
    const __nv_bfloat16* p = W + (size_t)(nt * 8 + g) * ld + kt * 16 + 2 * t;
    packed[idx] = make_uint2(*reinterpret_cast<const uint32_t*>(p), *reinterpret_cast<const uint32_t*>(p + 8));
}

template <int KT, int NT>
__device__ __forceinline__ void dense_packed(const uint32_t a[KT][4], const uint2* w, const float* bias,
                                             float z[NT][4]) {
    int lane = threadIdx.x & 31, t = lane & 3;
    for (int nt = 0; nt < NT; ++nt) {
        float b0 = bias[nt * 8 + 2 * t], b1 = bias[nt * 8 + 2 * t + 1];
        z[nt][0] = b0, z[nt][1] = b1, z[nt][2] = b0, z[nt][3] = b1;
        for (int kt = 0; kt < KT; ++kt) {
            uint2 f = w[(kt * NT + nt) * 32 + lane];
            uint32_t b[2] = {f.x, f.y};
            mma_bf16(z[nt], a[kt], b);
        }
    }
}

__global__ void __launch_bounds__(256) k_mlp_infer(const uint2* packed, const float* params,
                                                   const float* x_in /* [n][MLP_IN] */, unsigned long long n,
                                                   float* out) {
    __shared__ uint2 w[PK_TOTAL];
    __shared__ float bias[3 * MLP_H + MLP_OUT];  // b0, b1, b2, b3 (contiguous in the master vector)
    for (int k = threadIdx.x; k < PK_TOTAL; k += blockDim.x) w[k] = packed[k];
    for (int k = threadIdx.x; k < 3 * MLP_H + MLP_OUT; k += blockDim.x) bias[k] = params[P_B0 + k];
    __syncthreads();
    int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    unsigned long long warps = (unsigned long long)gridDim.x * (blockDim.x >> 5);
    unsigned long long tiles = (n + 15) / 16;
    for (unsigned long long tile = blockIdx.x * (unsigned long long)(blockDim.x >> 5) + (threadIdx.x >> 5);
         tile < tiles; tile += warps) {
        unsigned long long r0 = tile * 16;
        float x[2][MLP_IN];
        for (int h = 0; h < 2; ++h) {
            unsigned long long r = r0 + g + 8 * h;
            for (int i = 0; i < MLP_IN; ++i) x[h][i] = r < n ? x_in[MLP_IN * r + i] : 0.0f;
        }
        uint32_t a0[1][4], a1[4][4];
        float z[8][4], h8[8][4], o[2][4];
        input_a(x, a0);
        dense_packed<1, 8>(a0, w + PK_L0, bias, z);
        silu_tiles<8>(z, h8);
        to_a<8>(h8, a1);
        dense_packed<4, 8>(a1, w + PK_L1, bias + MLP_H, z);
        silu_tiles<8>(z, h8);
        to_a<8>(h8, a1);
        dense_packed<4, 8>(a1, w + PK_L2, bias + 2 * MLP_H, z);
        silu_tiles<8>(z, h8);
        to_a<8>(h8, a1);
        dense_packed<4, 2>(a1, w + PK_L3, bias + 3 * MLP_H, o);
        for (int nt = 0; nt < 2; ++nt)
            for (int h = 0; h < 2; ++h) {
                unsigned long long r = r0 + g + 8 * h;
                if (r < n) {
                    out[r * 16 + nt * 8 + 2 * t] = o[nt][2 * h];
                    out[r * 16 + nt * 8 + 2 * t + 1] = o[nt][2 * h + 1];
                }
            }
    }
}

// Shared-memory staging for the weight gradients of one warp.
struct WarpStage {
    __nv_bfloat16 d[16][72];  // dZ (or dO) rows x out, padded
    __nv_bfloat16 h[16][72];  // the layer's input rows x in, padded
};

// dW[out][in] += sum over the warp's 16 rows of d[row][out] * h[row][in],
// M = out (mt tiles of 16), N = in (nt tiles of 8), K = 16 rows; added
// into the block's shared accumulator.
__device__ __forceinline__ void grad_w(const WarpStage& s, int m_tiles, int n_tiles, float* acc, int ld) {
    int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    for (int mt = 0; mt < m_tiles; ++mt) {
        uint32_t a[4];
        // A[m = out][k = row] = d[row][out]
        auto A = [&](int m, int k) { return s.d[k][mt * 16 + m]; };
        __nv_bfloat162 p;
        p.x = A(g, 2 * t), p.y = A(g, 2 * t + 1);
        a[0] = *reinterpret_cast<uint32_t*>(&p);
        p.x = A(g + 8, 2 * t), p.y = A(g + 8, 2 * t + 1);
        a[1] = *reinterpret_cast<uint32_t*>(&p);
        p.x = A(g, 2 * t + 8), p.y = A(g, 2 * t + 9);
        a[2] = *reinterpret_cast<uint32_t*>(&p);
        p.x = A(g + 8, 2 * t + 8), p.y = A(g + 8, 2 * t + 9);
        a[3] = *reinterpret_cast<uint32_t*>(&p);
        for (int nt = 0; nt < n_tiles; ++nt) {
            uint32_t b[2];
            // B[k = row][n = in] = h[row][in]
            p.x = s.h[2 * t][nt * 8 + g], p.y = s.h[2 * t + 1][nt * 8 + g];
            b[0] = *reinterpret_cast<uint32_t*>(&p);
            p.x = s.h[2 * t + 8][nt * 8 + g], p.y = s.h[2 * t + 9][nt * 8 + g];
            b[1] = *reinterpret_cast<uint32_t*>(&p);
            float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            mma_bf16(c, a, b);
            int row = mt * 16 + g, col = nt * 8 + 2 * t;
            atomicAdd(&acc[row * ld + col], c[0]);
            atomicAdd(&acc[row * ld + col + 1], c[1]);
            atomicAdd(&acc[(row + 8) * ld + col], c[2]);
            atomicAdd(&acc[(row + 8) * ld + col + 1], c[3]);
        }
    }
}

// Accumulator-layout tiles (rows g, g + 8) into the stage's row matrix.
template <int NT>
__device__ __forceinline__ void stage_rows(const float v[NT][4], __nv_bfloat16 (*dst)[72]) {
    int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    for (int nt = 0; nt < NT; ++nt) {
        dst[g][nt * 8 + 2 * t] = __float2bfloat16(v[nt][0]);
        dst[g][nt * 8 + 2 * t + 1] = __float2bfloat16(v[nt][1]);
        dst[g + 8][nt * 8 + 2 * t] = __float2bfloat16(v[nt][2]);
        dst[g + 8][nt * 8 + 2 * t + 1] = __float2bfloat16(v[nt][3]);
    }
}

// Bias gradient: column sums of accumulator tiles over the warp's rows.
template <int NT>
__device__ __forceinline__ void grad_b(const float d[NT][4], float* acc) {
    int lane = threadIdx.x & 31, t = lane & 3;
    for (int nt = 0; nt < NT; ++nt)
        for (int q = 0; q < 2; ++q) {
            float v = d[nt][q] + d[nt][q + 2];
            for (int off = 4; off < 32; off <<= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            if (lane < 4) atomicAdd(&acc[nt * 8 + 2 * t + q], v);
        }
}

// One optimisation step's gradients over `rows` samples starting at `first`
// (pinball loss at quantile tau on ln f - ln f(v*), averaged): each block
// covers a contiguous share and writes its partial gradient to
// partial[block][P_TOTAL]; loss_out[block] gets its loss sum.
__global__ void __launch_bounds__(128) k_mlp_grad(MlpDev m, const MlpSample* data, unsigned long long first,
                                                  int rows, float tau, float* partial, float* loss_out) {
    extern __shared__ float smem[];  // P_TOTAL gradient accumulators, then 4 warp stages
    float* acc = smem;
    WarpStage* stage = reinterpret_cast<WarpStage*>(smem + ((P_TOTAL + 3) / 4) * 4);
    __shared__ float loss_s;
    for (int i = threadIdx.x; i < P_TOTAL; i += blockDim.x) acc[i] = 0.0f;
    if (threadIdx.x == 0) loss_s = 0.0f;
    __syncthreads();
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    int per_block = (rows + gridDim.x - 1) / gridDim.x;
    per_block = (per_block + 63) / 64 * 64;
    int b0r = blockIdx.x * per_block;
    int b1r = min(rows, b0r + per_block);
    WarpStage& s = stage[warp];
    float inv_rows = 1.0f / (float)rows;
    float loss = 0.0f;
    for (int r0 = b0r + warp * 16; r0 < b1r; r0 += 64) {
        float x[2][MLP_IN];
        int bin[2];
        float tgt[2];
        bool ok[2];
        for (int h = 0; h < 2; ++h) {
            int r = r0 + g + 8 * h;
            ok[h] = r < b1r;
            MlpSample smp{};
            smp.bin = -1;
            if (ok[h]) smp = data[first + r];
            for (int i = 0; i < MLP_IN; ++i) x[h][i] = smp.x[i];
            bin[h] = smp.bin;
            tgt[h] = smp.t;
            if (smp.bin < 0 || !(smp.t == smp.t)) ok[h] = false;
        }
        WarpFwd f;
        warp_forward(m, x, f);
        // pinball loss on the sampled bin only
        float d_o[2][4];
        for (int nt = 0; nt < 2; ++nt)
            for (int q = 0; q < 4; ++q) {
                int h = q >> 1, col = nt * 8 + 2 * t + (q & 1);
                float d = 0.0f;
                if (ok[h] && col == bin[h]) {
                    float res = tgt[h] - f.o[nt][q];
                    loss += res > 0.0f ? tau * res : (tau - 1.0f) * res;
                    d = (res > 0.0f ? -tau : 1.0f - tau) * inv_rows;
                }
                d_o[nt][q] = d;
            }
        // layer 3: dW3 = dO^T h2, db3, dH2 = dO W3
        float h2[8][4];
        silu_tiles<8>(f.z2, h2);
        __syncwarp();
        stage_rows<2>(d_o, s.d);
        stage_rows<8>(h2, s.h);
        __syncwarp();
        grad_w(s, 1, 8, acc + P_W3, MLP_H);
        grad_b<2>(d_o, acc + P_B3);
        uint32_t ad[4][4];
        {
            uint32_t a_o[1][4];
            to_a<2>(d_o, a_o);
            float dh[8][4];
            for (int nt = 0; nt < 8; ++nt) {
                dh[nt][0] = dh[nt][1] = dh[nt][2] = dh[nt][3] = 0.0f;
                uint32_t b[2];
                load_b(m.t3, MLP_OUT, 0, nt * 8, b);
                mma_bf16(dh[nt], a_o[0], b);
                for (int q = 0; q < 4; ++q) dh[nt][q] *= dsilu(f.z2[nt][q]);
            }
            // dZ2 in dh: layer 2 gradients, then dH1 = dZ2 W2
            float h1[8][4];
            silu_tiles<8>(f.z1, h1);
            __syncwarp();
            stage_rows<8>(dh, s.d);
            stage_rows<8>(h1, s.h);
            __syncwarp();
            grad_w(s, 4, 8, acc + P_W2, MLP_H);
            grad_b<8>(dh, acc + P_B2);
            to_a<8>(dh, ad);
        }
        {
            float dh[8][4];
            for (int nt = 0; nt < 8; ++nt) {
                dh[nt][0] = dh[nt][1] = dh[nt][2] = dh[nt][3] = 0.0f;
                for (int kt = 0; kt < 4; ++kt) {
                    uint32_t b[2];
                    load_b(m.t2, MLP_H, kt * 16, nt * 8, b);
                    mma_bf16(dh[nt], ad[kt], b);
                }
                for (int q = 0; q < 4; ++q) dh[nt][q] *= dsilu(f.z1[nt][q]);
            }
            float h0[8][4];
            silu_tiles<8>(f.z0, h0);
            __syncwarp();
            stage_rows<8>(dh, s.d);
            stage_rows<8>(h0, s.h);
            __syncwarp();
            grad_w(s, 4, 8, acc + P_W1, MLP_H);
            grad_b<8>(dh, acc + P_B1);
            to_a<8>(dh, ad);
        }
        {
            float dh[8][4];
            for (int nt = 0; nt < 8; ++nt) {
                dh[nt][0] = dh[nt][1] = dh[nt][2] = dh[nt][3] = 0.0f;
                for (int kt = 0; kt < 4; ++kt) {
                    uint32_t b[2];
                    load_b(m.t1, MLP_H, kt * 16, nt * 8, b);
                    mma_bf16(dh[nt], ad[kt], b);
                }
                for (int q = 0; q < 4; ++q) dh[nt][q] *= dsilu(f.z0[nt][q]);
            }
            // layer 0: input x padded to 16 columns
            __syncwarp();
            stage_rows<8>(dh, s.d);
            for (int h = 0; h < 2; ++h)
                for (int c = 0; c < 16; c += 4) {
                    // lanes write the 16 x 16 input tile of their rows
                    int col = c + t;
                    float v = 0.0f;
                    for (int i = 0; i < MLP_IN; ++i) v = col == i ? x[h][i] : v;
                    s.h[g + 8 * h][col] = __float2bfloat16(v);
                }
            __syncwarp();
            grad_w(s, 4, 2, acc + P_W0, MLP_IN_PAD);
            grad_b<8>(dh, acc + P_B0);
        }
    }
    for (int off = 16; off > 0; off >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, off);
    if (lane == 0) atomicAdd(&loss_s, loss);
    __syncthreads();
    float* out = partial + (size_t)blockIdx.x * P_TOTAL;
    for (int i = threadIdx.x; i < P_TOTAL; i += blockDim.x) out[i] = acc[i];
    if (threadIdx.x == 0) loss_out[blockIdx.x] = loss_s;
}

// Sum of the blocks' partial gradients, Adam step on the FP32 master, and
// the BF16 copies (row-major and transposed) the other kernels read.
__global__ void k_mlp_adam(float* p, float* mom, float* vel, const float* partial, int nblocks, float lr, float b1,
                           float b2, float eps, int step, MlpDev m) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P_TOTAL) return;
    // padding columns of layer 0 stay zero
    if (i < P_W1 && (i % MLP_IN_PAD) >= MLP_IN) return;
    float g = 0.0f;
    for (int b = 0; b < nblocks; ++b) g += partial[(size_t)b * P_TOTAL + i];
    float mo = b1 * mom[i] + (1.0f - b1) * g;
    float ve = b2 * vel[i] + (1.0f - b2) * g * g;
    mom[i] = mo;
    vel[i] = ve;
    float mh = mo / (1.0f - powf(b1, (float)step)), vh = ve / (1.0f - powf(b2, (float)step));
    float w = p[i] - lr * mh / (sqrtf(vh) + eps);
    p[i] = w;
    __nv_bfloat16 wb = __float2bfloat16(w);
    if (i < P_W1) {
        m.w0[i] = wb;
    } else if (i < P_W2) {
        int k = i - P_W1, o = k / MLP_H, c = k % MLP_H;
        m.w1[k] = wb;
        m.t1[c * MLP_H + o] = wb;
    } else if (i < P_W3) {
        int k = i - P_W2, o = k / MLP_H, c = k % MLP_H;
        m.w2[k] = wb;
        m.t2[c * MLP_H + o] = wb;
    } else if (i < P_B0) {
        int k = i - P_W3, o = k / MLP_H, c = k % MLP_H;
        m.w3[k] = wb;
        m.t3[c * MLP_OUT + o] = wb;
    }
}

// BF16 copies from the FP32 master (after initialisation or a load).
__global__ void k_mlp_sync(const float* p, MlpDev m) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P_B0) return;
    __nv_bfloat16 wb = __float2bfloat16(p[i]);
    if (i < P_W1) {
        m.w0[i] = wb;
    } else if (i < P_W2) {
        int k = i - P_W1, o = k / MLP_H, c = k % MLP_H;
        m.w1[k] = wb;
        m.t1[c * MLP_H + o] = wb;
    } else if (i < P_W3) {
        int k = i - P_W2, o = k / MLP_H, c = k % MLP_H;
        m.w2[k] = wb;
        m.t2[c * MLP_H + o] = wb;
    } else {
        int k = i - P_W3, o = k / MLP_H, c = k % MLP_H;
        m.w3[k] = wb;
        m.t3[c * MLP_OUT + o] = wb;
    }
}

// Draws of the table sampler for training and benchmarking: (a, eta)
// log-uniform over [a_lo, a_hi] x [eta_lo, eta_hi], n by the CP harmonic
// CDF; one bin of v and the exact spectrum's largest sampled value in it
// per sample.
__device__ __forceinline__ void draw_point(Draws& rng, double a_lo, double a_hi, double e_lo, double e_hi, double* a,
                                           double* eta) {
    *a = exp(log(a_lo) + (log(a_hi) - log(a_lo)) * rng.next());
    *eta = exp(log(e_lo) + (log(e_hi) - log(e_lo)) * rng.next());
}

__global__ void k_mlp_data(const LmaTables* t, unsigned long long n, unsigned long long seed, double a_lo, double a_hi,
                           double e_lo, double e_hi, MlpSample* out) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    Draws rng;
    rng.begin(seed, mix64(i + 0x5851F42D4C957F2Dull), 0);
    double a, eta;
    draw_point(rng, a_lo, a_hi, e_lo, e_hi, &a, &eta);
    NlcTables nt = nlc_view(*t);
    int nh = cp_invert(nt, a, eta, rng.next());
    if (nh < 1) nh = 1;
    double sn = 2.0 * nh * eta / (1.0 + a * a);
    double v_star = (1.0 + sn) / (2.0 + sn);
    double base = log(cp_diff_partial_rate(nh, a, eta, v_star));
    // the target is the largest of f at the bin's two edges and at two
    // uniform interior points, so that a high quantile of it tracks the
    // bin's maximum
    int bin = min((int)(rng.next() * MLP_OUT), MLP_OUT - 1);
    double lo = fmax((double)bin / MLP_OUT, 1e-9), hi = fmin((double)(bin + 1) / MLP_OUT, 1.0 - 1e-9);
    double f = fmax(cp_diff_partial_rate(nh, a, eta, lo), cp_diff_partial_rate(nh, a, eta, hi));
    for (int q = 0; q < 2; ++q) f = fmax(f, cp_diff_partial_rate(nh, a, eta, lo + (hi - lo) * rng.next()));
    MlpSample s;
    mlp_features(a, eta, nh, s.x);
    s.bin = bin;
    // bins far under the peak carry no proposals: their targets are
    // floored, which keeps the envelope above the spectrum there and the
    // regression's range to the part of the spectrum that matters
    double tv = fmax(log(f) - base, (double)MLP_TARGET_FLOOR);
    s.t = (f > 0.0 && isfinite(base)) ? (float)tv : (isfinite(base) ? MLP_TARGET_FLOOR : __int_as_float(0x7fc00000));
    out[i] = s;
}

// ---------------------------------------------------- sampler benchmark --
// Emission i draws (a, eta) and the harmonic n from its own stream, so both
// methods see the same (a, eta, n) per index.
__device__ __forceinline__ void bench_point(const NlcTables& nt, unsigned long long i, unsigned long long seed,
                                            double a_lo, double a_hi, double e_lo, double e_hi, double* a, double* eta,
                                            int* nh) {
    Draws pt;
    pt.begin(seed, mix64(i + 0x2545F4914F6CDD1Dull), 0);
    draw_point(pt, a_lo, a_hi, e_lo, e_hi, a, eta);
    *nh = max(cp_invert(nt, *a, *eta, pt.next()), 1);
}

// One emission's point, kept between the learned path's passes.
struct BenchPoint {
    double a, eta;
    int n, pad;
};

// The first pass, shared by both samplers: the point of every emission, and
// the network's inputs for it.
__global__ void k_sampler_features(const LmaTables* t, unsigned long long n, unsigned long long seed, double a_lo,
                                   double a_hi, double e_lo, double e_hi, float* x_out, BenchPoint* pts) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    NlcTables nt = nlc_view(*t);
    double a, eta;
    int nh;
    bench_point(nt, i, seed, a_lo, a_hi, e_lo, e_hi, &a, &eta, &nh);
    mlp_features(a, eta, nh, x_out + MLP_IN * i);
    pts[i] = BenchPoint{a, eta, nh, 0};
}

// Both samplers as one state machine per lane, so that every lane of a warp
// evaluates the spectrum at the same instruction on every pass of a single
// loop: a lane that finishes an emission takes the next one from a global
// counter (warp-aggregated) instead of idling while the other lanes of its
// warp finish theirs.  The cost per emission is heavy-tailed (from two to
// thousands of spectrum evaluations); without this the slowest lane sets
// every warp's time.  Per emission and method the draws and decisions are
// those of cp_sample_v (plain) and cp_sample_v_learned (learned, with the
// capped continuation of cp_sample_v_capped).  fallback_out: bits 0-1 =
// 0; 1 = the learned envelope under the spectrum, the reference's sampler
// took over; 2 = no acceptance within LEARNED_TRIALS, the capped envelope
// took over; 3 = 2 and then 1.  Bits 2-31: proposals drawn from the
// learned (or capped) envelope.
enum : int { SB_IDLE, SB_DONE, SB_CEIL, SB_TRIAL, SB_STAR, SB_LTRIAL, SB_MTRIAL };

template <bool LEARNED>
__global__ void __launch_bounds__(128) k_sampler_run(const LmaTables* t, unsigned long long n, unsigned long long seed,
                                                     double a_lo, double a_hi, double e_lo, double e_hi,
                                                     const float* env, const BenchPoint* pts, float margin,
                                                     unsigned long long* counter, double* v_out, unsigned* evals_out,
                                                     unsigned* fallback_out, int* status_out) {
    NlcTables nt = nlc_view(*t);
    const unsigned FULL = 0xffffffffu;
    int lane = threadIdx.x & 31;
    int phase = SB_IDLE;
    unsigned long long i = 0;
    double a = 0.0, eta = 0.0, mx = 0.0, v = 0.0, u = 0.0;
    int nh = 1, k = 0, bin = 0;
    unsigned evals = 0, fb = 0, trials = 0, capped = 0;
    Envelope e{};
    Draws rng;
    for (;;) {
        // new emissions for idle lanes
        unsigned idle = __ballot_sync(FULL, phase == SB_IDLE);
        if (idle) {
            int leader = __ffs(idle) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(idle));
            base = __shfl_sync(FULL, base, leader);
            if (phase == SB_IDLE) {
                i = base + __popc(idle & ((1u << lane) - 1u));
                if (i >= n) {
                    phase = SB_DONE;
                } else {
                    BenchPoint p = pts[i];
                    a = p.a, eta = p.eta, nh = p.n;
                    rng.begin(seed ^ 0x9E3779B97F4A7C15ull, mix64(i), LEARNED ? 2 : 1);
                    evals = fb = trials = 0;
                    k = 0;
                    mx = -HUGE_VAL;
                    phase = LEARNED ? SB_STAR : SB_CEIL;
                }
            }
        }
        if (__all_sync(FULL, phase == SB_DONE)) break;
        // the point this lane evaluates on this pass
        if (phase == SB_CEIL) {
            v = cp_ceiling_point(nh, a, eta, k);
        } else if (phase == SB_TRIAL) {
            v = rng.next();
            u = rng.next();
        } else if (phase == SB_STAR) {
            double sn = 2.0 * nh * eta / (1.0 + a * a);
            v = (1.0 + sn) / (2.0 + sn);
        } else if (phase == SB_LTRIAL || phase == SB_MTRIAL) {
            v = envelope_draw(e, rng, &bin);
        }
        double f = 0.0;
        if (phase != SB_DONE) {
            f = cp_diff_partial_rate(nh, a, eta, v);
            evals += 1;
        }
        // transitions
        int st = -1;  // >= 0: the emission ends with this status
        if (phase == SB_CEIL) {
            mx = fmax(mx, f);
            if (++k == 32) {
                mx *= 1.2;
                k = 0;
                if (fb == 2) {
                    capped = envelope_cap(&e, mx);
                    phase = SB_MTRIAL;
                } else {
                    phase = SB_TRIAL;
                }
            }
        } else if (phase == SB_TRIAL) {
            if (u <= f / mx) {
                st = 0;
            } else if (++k == REJECTION_CAP) {
                st = 4;  // PTG_ERR_REJECTION_CAP
            }
        } else if (phase == SB_STAR) {
            if (envelope_from(env + MLP_OUT * i, margin, f, &e)) {
                phase = SB_LTRIAL;
            } else {
                fb = 1;
                phase = SB_CEIL;
            }
        } else if (phase == SB_LTRIAL) {
            double g = e.scale * (double)e.w[bin];
            trials += 1;
            if (f > g) {
                fb = 1;  // the envelope is under the spectrum: hand over
                phase = SB_CEIL;
            } else if (rng.next() * g < f) {
                st = 0;
            } else if (trials == LEARNED_TRIALS) {
                fb = 2;
                phase = SB_CEIL;
            }
        } else if (phase == SB_MTRIAL) {
            double g = e.scale * (double)e.w[bin];
            trials += 1;
            if (f > g) {
                if (capped & (1u << bin)) {
                    st = 0;  // over the reference's own ceiling: its rule accepts
                } else {
                    fb = 3;
                    k = 0;
                    phase = SB_TRIAL;
                }
            } else if (rng.next() * g < f) {
                st = 0;
            } else if (++k == REJECTION_CAP) {
                st = 4;
            }
        }
        if (st >= 0) {
            v_out[i] = st == 0 ? v : -1.0;
            evals_out[i] = evals;
            if (fallback_out) fallback_out[i] = fb | (min(trials, 0x3FFFFFFFu) << 2);
            status_out[i] = st;
            phase = SB_IDLE;
        }
    }
}

// ------------------------------------------------------------ launchers --
size_t mlp_packed_bytes() { return sizeof(uint2) * PK_TOTAL; }

cudaError_t launch_mlp_infer(const MlpDev& m, void* packed, const float* x, unsigned long long n, float* out,
                             cudaStream_t s) {
    k_mlp_pack<<<(PK_TOTAL + 255) / 256, 256, 0, s>>>(m, (uint2*)packed);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    unsigned long long tiles = (n + 15) / 16;
    unsigned long long blocks = std::min<unsigned long long>((tiles + 7) / 8, 4ull * (unsigned long long)std::max(sms, 1));
    k_mlp_infer<<<(unsigned)std::max<unsigned long long>(blocks, 1), 256, 0, s>>>((const uint2*)packed, m.p, x, n, out);
    return cudaGetLastError();
}

cudaError_t launch_mlp_grad(const MlpDev& m, const void* data, unsigned long long first, int rows, float tau,
                            float* partial, float* loss, int blocks, cudaStream_t s) {
    size_t smem = sizeof(float) * ((P_TOTAL + 3) / 4) * 4 + 4 * sizeof(WarpStage);
    static bool configured = false;  // one device per process uses this path
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    k_mlp_grad<<<blocks, 128, smem, s>>>(m, (const MlpSample*)data, first, rows, tau, partial, loss);
    return cudaGetLastError();
}

cudaError_t launch_mlp_adam(float* p, float* mom, float* vel, const float* partial, int nblocks, float lr, int step,
                            const MlpDev& m, cudaStream_t s) {
    k_mlp_adam<<<(P_TOTAL + 255) / 256, 256, 0, s>>>(p, mom, vel, partial, nblocks, lr, 0.9f, 0.999f, 1e-8f, step, m);
    return cudaGetLastError();
}

cudaError_t launch_mlp_sync(const float* p, const MlpDev& m, cudaStream_t s) {
    k_mlp_sync<<<(P_B0 + 255) / 256, 256, 0, s>>>(p, m);
    return cudaGetLastError();
}

cudaError_t launch_mlp_data(const LmaTables* t, unsigned long long n, unsigned long long seed, double a_lo,
                            double a_hi, double e_lo, double e_hi, void* out, cudaStream_t s) {
    k_mlp_data<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(t, n, seed, a_lo, a_hi, e_lo, e_hi, (MlpSample*)out);
    return cudaGetLastError();
}

size_t sampler_point_bytes() { return sizeof(BenchPoint); }

cudaError_t launch_sampler_features(const LmaTables* t, unsigned long long n, unsigned long long seed, double a_lo,
                                    double a_hi, double e_lo, double e_hi, float* x_out, void* pts, cudaStream_t s) {
    k_sampler_features<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(t, n, seed, a_lo, a_hi, e_lo, e_hi, x_out,
                                                                   (BenchPoint*)pts);
    return cudaGetLastError();
}

cudaError_t launch_sampler_run(const LmaTables* t, unsigned long long n, unsigned long long seed, double a_lo,
                               double a_hi, double e_lo, double e_hi, int learned, const float* env, const void* pts,
                               float margin, unsigned long long* counter, double* v_out, unsigned* evals,
                               unsigned* fallbacks, int* status, cudaStream_t s) {
    if (!pts || (learned && !env)) return cudaErrorInvalidValue;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = learned ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sampler_run<true>, 128, 0)
                            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sampler_run<false>, 128, 0);
    if (e != cudaSuccess) return e;
    // persistent grid: one wave of resident blocks, no more lanes than work
    unsigned long long blocks = (unsigned long long)max(sms, 1) * (unsigned long long)max(per_sm, 1);
    blocks = std::min(blocks, (n + 127) / 128);
    e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    const BenchPoint* p = (const BenchPoint*)pts;
    if (learned)
        k_sampler_run<true><<<(unsigned)blocks, 128, 0, s>>>(t, n, seed, a_lo, a_hi, e_lo, e_hi, env, p, margin,
                                                             counter, v_out, evals, fallbacks, status);
    else
        k_sampler_run<false><<<(unsigned)blocks, 128, 0, s>>>(t, n, seed, a_lo, a_hi, e_lo, e_hi, env, p, margin,
                                                              counter, v_out, evals, fallbacks, status);
    return cudaGetLastError();
}

int mlp_param_count() { return P_TOTAL; }
size_t mlp_sample_bytes() { return sizeof(MlpSample); }

}  // namespace ptg
