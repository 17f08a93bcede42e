// Oracle (test infrastructure only): the counter-based random streams that
// the GPU kernels use, restated on the CPU so that the oracle can replay a
// particle with exactly the same draws as the device.
//
// The reference draws from one sequential Xoshiro256** per MPI rank
// (src/main.rs:1036-1040); no reference test pins that stream, so
// per-particle replay needs a stream both sides can regenerate.  Scheme:
//   Philox4x32-10 (Salmon et al., "Parallel random numbers: as easy as
//   1, 2, 3", SC'11), key = 64-bit run seed, counter =
//   (step, block, stream_lo, stream_hi).
//   A particle's stream id is fixed at creation; its step counter restarts
//   at 0 and the block counter restarts at 0 every step.  Each block yields
//   two 53-bit uniforms u = ((w0 << 21) | (w1 >> 11)) * 2^-53 in [0, 1).
//   Secondaries take child_stream(parent, step, slot).
#pragma once
#include <cstdint>

namespace orc {

inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)M0 * c[0];
        uint64_t p1 = (uint64_t)M1 * c[2];
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c[1] ^ k0;
        uint32_t n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
        k0 += W0;
        k1 += W1;
    }
}

inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

inline uint64_t primary_stream(uint64_t global_index) {
    return mix64(global_index + 0x9E3779B97F4A7C15ull);
}

inline uint64_t child_stream(uint64_t parent, uint32_t step, uint32_t slot) {
    uint64_t tag = ((uint64_t)step << 2) | (uint64_t)slot;
    return mix64(parent + 0x9E3779B97F4A7C15ull * (tag + 1));
}

struct DrawStream {
    uint64_t seed = 0, stream = 0;
    uint32_t step = 0, block = 0;
    uint32_t w[4] = {0, 0, 0, 0};
    int pos = 4;

    void begin_step(uint32_t s) {
        step = s;
        block = 0;
        pos = 4;
    }
    double next() {
        if (pos >= 4) {
            w[0] = step;
            w[1] = block;
            w[2] = (uint32_t)stream;
            w[3] = (uint32_t)(stream >> 32);
            philox4x32_10(w, (uint32_t)seed, (uint32_t)(seed >> 32));
            ++block;
            pos = 0;
        }
        uint64_t m = ((uint64_t)w[pos] << 21) | (uint64_t)(w[pos + 1] >> 11);
        pos += 2;
        return (double)m * (1.0 / 9007199254740992.0);
    }
};

}  // namespace orc
