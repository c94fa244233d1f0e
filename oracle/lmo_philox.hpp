// Oracle (test infrastructure only): Philox4x32-10 counter-based generator.
//
// Restates the published algorithm of Salmon, Moraes, Dror & Shaw, "Parallel random numbers:
// as easy as 1, 2, 3" (SC 2011): 10 rounds of two 32x32->64 multiplies with the paper's
// multipliers and Weyl key increments. The GPU path keys its per-path stream the same way, so an
// oracle path and a GPU path consume identical uniforms:
//   key     = (seed, 0x6c6d6770 "lmgp")
//   counter = (4*vertex + slot/4, path_lo, path_hi, 0)
//   uniform = (word[slot%4] >> 8) * 2^-24, in [0, 1)
#pragma once
#include <cstdint>

namespace lmo {

struct Philox4 { uint32_t v[4]; };

inline Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    for (int r = 0; r < 10; r++) {
        const uint64_t p0 = uint64_t(M0) * c0;
        const uint64_t p1 = uint64_t(M1) * c2;
        const uint32_t hi0 = uint32_t(p0 >> 32), lo0 = uint32_t(p0);
        const uint32_t hi1 = uint32_t(p1 >> 32), lo1 = uint32_t(p1);
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += W0; k1 += W1;
    }
    return Philox4{{c0, c1, c2, c3}};
}

inline float philox_uniform(uint32_t seed, uint64_t path, uint32_t vertex, uint32_t slot) {
    const Philox4 r = philox4x32_10(vertex * 4u + (slot >> 2), uint32_t(path), uint32_t(path >> 32), 0u, seed, 0x6c6d6770u);
    return float(r.v[slot & 3u] >> 8) * (1.0f / 16777216.0f);
}

}  // namespace lmo
