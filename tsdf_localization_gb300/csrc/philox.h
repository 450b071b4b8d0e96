// Counter-based random numbers for the device: Philox4x64 with 10 rounds
// (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
// SC 2011), with the paper's multipliers and Weyl increments.  Every consumer
// keys it with (seed, its stream constant) and counts with its own indices, so
// draws are independent across particles and reproducible per seed.
#pragma once

#include <stdint.h>

namespace tsdfl {

constexpr unsigned long long kStreamMotion = 0x6D6F74696F6E0001ull;
constexpr unsigned long long kStreamWheel = 0x776865656C000001ull;
constexpr unsigned long long kStreamResidual = 0x7265736964000001ull;
constexpr unsigned long long kStreamMetropolis = 0x6D6574726F000001ull;
constexpr unsigned long long kStreamRejection = 0x72656A6563000001ull;

#ifdef __CUDACC__

__device__ __forceinline__ void philox4x64_10(unsigned long long c[4], unsigned long long k0, unsigned long long k1)
{
    const unsigned long long m0 = 0xD2E7470EE14C6C93ull, m1 = 0xCA5A826395121157ull;
    const unsigned long long w0 = 0x9E3779B97F4A7C15ull, w1 = 0xBB67AE8584CAA73Bull;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const unsigned long long lo0 = m0 * c[0], hi0 = __umul64hi(m0, c[0]);
        const unsigned long long lo1 = m1 * c[2], hi1 = __umul64hi(m1, c[2]);
        const unsigned long long n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
        k0 += w0;
        k1 += w1;
    }
}

// [0, 1) with 53 random bits.
__device__ __forceinline__ double u01_double(unsigned long long x) { return (double)(x >> 11) * 0x1.0p-53; }
// [0, 1) with 24 random bits.
__device__ __forceinline__ float u01_float(unsigned long long x) { return (float)(x >> 40) * 0x1.0p-24f; }
// An index in [0, n): the high word of x * n.
__device__ __forceinline__ uint32_t uniform_index(unsigned long long x, uint32_t n)
{
    return (uint32_t)__umul64hi(x, (unsigned long long)n);
}

#endif

}  // namespace tsdfl
