// Counter-based random numbers: Philox4x32-10 (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11).  Every draw of the
// PIC step is a pure function of (seed, species, particle id, step, draw index),
// so results do not depend on thread scheduling or particle order.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define MAG_HD __host__ __device__ __forceinline__
#else
#define MAG_HD inline
#endif

namespace mag {

struct U4 {
    uint32_t x, y, z, w;
};

MAG_HD void mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo)
{
    uint64_t p = (uint64_t)a * (uint64_t)b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
}

MAG_HD U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1)
{
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(M0, c.x, hi0, lo0);
        mulhilo32(M1, c.z, hi1, lo1);
        c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += W0;
        k1 += W1;
    }
    return c;
}

// Stream tags keep the draw families of one particle disjoint.
enum : uint32_t {
    TAG_COLLIDE_TEST = 0,
    TAG_COLLIDE = 1,
    TAG_LOAD = 2,
    TAG_PARTNER = 3,
    TAG_MULTICOLL = 4,
    TAG_TTD = 5,
    TAG_SOURCE_INIT = 6,  // source box particles: initial positions and velocities
    TAG_SOURCE = 7,       // source box particles: collision test and scatter of a step
    TAG_SOURCE_TILE = 8   // source box particles: the tile of each copy of a step
};

// Draw block 'k' (4 words) of particle 'id' at 'step' for species 'sp'.
MAG_HD U4 draw(uint64_t seed, uint32_t sp, uint32_t id, uint64_t step, uint32_t tag, uint32_t k)
{
    U4 c{id, (uint32_t)step, (uint32_t)(step >> 32), (tag << 24) ^ k};
    return philox4x32_10(c, (uint32_t)seed ^ (sp * 0x85EBCA6Bu), (uint32_t)(seed >> 32));
}

// Per-step collision test: one 32-bit uniform per (seed, species, particle id,
// step), from the 64-bit finaliser of SplitMix64 (Steele, Lea, Flood, "Fast
// splittable pseudorandom number generators", OOPSLA 2014) applied to the
// stream position seed + (id * 2^32 + step) * golden gamma.  Two 64-bit
// multiplies instead of the ten rounds of Philox; the rarer draws of the
// collisions themselves stay on Philox.
MAG_HD uint32_t collision_test_u32(uint64_t seed, uint32_t sp, uint32_t id, uint64_t step)
{
    uint64_t z = (seed ^ ((uint64_t)sp << 56)) + (((uint64_t)id << 32) ^ step) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (uint32_t)(z >> 32);
}

// uniform in [0,1) with 24 random bits (float) / 53 random bits (double)
MAG_HD float u01f(uint32_t a) { return (float)(a >> 8) * (1.0f / 16777216.0f); }
MAG_HD double u01d(uint32_t a, uint32_t b)
{
    return (double)(((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6)) * (1.0 / 9007199254740992.0);
}
// uniform in (0,1] (for logarithms)
MAG_HD double u01d_open0(uint32_t a, uint32_t b) { return 1.0 - u01d(a, b); }

}  // namespace mag
