// Philox4x32-10 counter-based generator (Salmon et al., SC'11), device side.
//
// Round multipliers 0xD2511F53 / 0xCD9E8D57, Weyl key increments
// 0x9E3779B9 / 0xBB67AE85.  The key schedule depends only on the seed, so the
// FP32 walk precomputes the ten round keys once per launch (PhiloxKeys) and the
// hot loop spends two wide multiplies and two three-input XORs per round.
#pragma once
#include <cstdint>

namespace mcw {

constexpr uint32_t kPhiloxM0 = 0xD2511F53u;
constexpr uint32_t kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u;
constexpr uint32_t kPhiloxW1 = 0xBB67AE85u;

struct PhiloxKeys {
    uint32_t k0[10];
    uint32_t k1[10];
};

__host__ __device__ inline PhiloxKeys philox_schedule(uint64_t seed) {
    PhiloxKeys s;
    uint32_t a = (uint32_t)seed, b = (uint32_t)(seed >> 32);
    for (int r = 0; r < 10; ++r) {
        s.k0[r] = a;
        s.k1[r] = b;
        a += kPhiloxW0;
        b += kPhiloxW1;
    }
    return s;
}

__device__ __forceinline__ uint4 philox_round(uint4 c, uint32_t k0, uint32_t k1) {
    // each 32 x 32 -> 64-bit product as one wide multiply
    const uint64_t p0 = (uint64_t)kPhiloxM0 * c.x;
    const uint64_t p1 = (uint64_t)kPhiloxM1 * c.z;
    return make_uint4((uint32_t)(p1 >> 32) ^ c.y ^ k0, (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.w ^ k1,
                      (uint32_t)p0);
}

// Philox with a precomputed key schedule.
__device__ __forceinline__ uint4 philox10(uint4 c, const PhiloxKeys &ks) {
#pragma unroll
    for (int r = 0; r < 10; ++r) c = philox_round(c, ks.k0[r], ks.k1[r]);
    return c;
}

// Philox keyed directly by the 64-bit seed (replay kernel).
__device__ __forceinline__ uint4 philox10_seed(uint4 c, uint64_t seed) {
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        c = philox_round(c, k0, k1);
        k0 += kPhiloxW0;
        k1 += kPhiloxW1;
    }
    return c;
}

// Uniform in [2^-24, 1 - 2^-24] from the top 23 bits of w: the float
// 1.m (m = w >> 9) minus (1 - 2^-24).  Exact (Sterbenz), never 0 or 1.
__device__ __forceinline__ float u01_f32(uint32_t w) {
    return __uint_as_float(0x3F800000u | (w >> 9)) - 0.99999994f;
}

// Uniform double in [2^-53, 1 - 2^-53] from a 64-bit word: ((w >> 12) + 0.5) * 2^-52.
__device__ __forceinline__ double u01_f64(uint64_t w) {
    return ((double)(w >> 12) + 0.5) * 0x1p-52;
}

}  // namespace mcw
