// Oracle-side random stream (test infrastructure only; never linked into the
// product library).
//
// The reference draws every random number from a thread-local mt19937 with a
// non-deterministic seed (source/math/random.cpp:10-19), so two runs of the
// reference never agree.  For parity work every path sample instead owns a
// counter-based stream:
//
//   key   = path_key(seed, scene, pixel, sample)
//   x_i   = splitmix64_finalize(key + (i + 1) * 0x9E3779B97F4A7C15)
//   u_i   = (x_i >> 40) * 2^-24            in [0, 1 - 2^-24]
//
// i.e. the SplitMix64 generator (Steele, Lea & Flood, OOPSLA 2014) seeded with
// the path key.  The CUDA library implements the same published recurrence in
// its own code; the reference harness interposes cadise::Random with this
// stream, and the CPU restatement consumes it in the reference's order, so a
// path sample can be replayed bit-for-bit on all three.
#pragma once

#include <cstdint>

namespace oracle_rng {

inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

inline uint64_t path_key(uint64_t seed, uint32_t scene, uint32_t pixel, uint32_t sample) {
    const uint64_t s = mix64(seed ^ (0xD1B54A32D192ED03ull * (uint64_t(scene) + 1)));
    return mix64(s ^ ((uint64_t(sample) << 32) | uint64_t(pixel)));
}

inline uint64_t draw_bits(uint64_t key, uint32_t index) {
    return mix64(key + (uint64_t(index) + 1) * 0x9E3779B97F4A7C15ull);
}

inline float draw_float(uint64_t key, uint32_t index) {
    return float(uint32_t(draw_bits(key, index) >> 40)) * (1.0f / 16777216.0f);
}

// Stateful view used by the harness and the CPU restatement.
struct Stream {
    uint64_t key = 0;
    uint32_t counter = 0;
    float next() { return draw_float(key, counter++); }
};

}  // namespace oracle_rng
