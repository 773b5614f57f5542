// gi_host.h -- pieces shared by the host-side translation units.
#pragma once
#include <cstdint>

namespace gi_host {

// splitmix64 (Steele, Lea, Flood 2014; Vigna's public-domain constants):
// a counter-based generator whose stream is fixed by the seed alone.
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
    // Uniform double in [0, 1) with 53 random bits.
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

}  // namespace gi_host
