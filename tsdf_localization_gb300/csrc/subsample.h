// Seeded per-particle scan subsampling (no counterpart in the reference, whose
// evaluator scores every reduced point for every particle): particle i of a
// call keeps K of the N points, one from each of K strata of consecutive scan
// indices.  Stratum k is [b_k, b_{k+1}) with b_k = floor(k N / K); the point
// taken is b_k + floor(u * n_k / 2^32), n_k = b_{k+1} - b_k and u the upper 32
// bits of the k-th output of a SplitMix64 generator (Steele, Lea and Flood,
// OOPSLA 2014) whose state starts at mix(seed ^ mix(i)):
//   state_k = mix(seed ^ mix(i)) + (k + 1) * 0x9E3779B97F4A7C15,  u = mix(state_k) >> 32.
// Every point is kept with probability K / N, the K kept points are distinct,
// cover the whole scan, and differ from particle to particle and from seed to
// seed.  Shared by the host (tests, docs) and the kernels.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define TSDFL_SUB_HD __host__ __device__ __forceinline__
#else
#define TSDFL_SUB_HD inline
#endif

namespace tsdfl {

constexpr uint64_t kGoldenGamma = 0x9E3779B97F4A7C15ull;

TSDFL_SUB_HD uint64_t sub_mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// The generator's starting state for particle i.
TSDFL_SUB_HD uint64_t sub_particle_state(uint64_t seed, uint64_t i)
{
    return sub_mix64(seed ^ sub_mix64(i));
}

// Scan index of the k-th kept point (0 <= k < K <= N) of the particle whose
// starting state is st.
TSDFL_SUB_HD uint32_t sub_point(uint64_t st, uint32_t N, uint32_t K, uint32_t k)
{
    const uint32_t b0 = (uint32_t)(((uint64_t)k * N) / K);
    const uint32_t b1 = (uint32_t)(((uint64_t)(k + 1) * N) / K);
    const uint32_t u = (uint32_t)(sub_mix64(st + (uint64_t)(k + 1) * kGoldenGamma) >> 32);
    return b0 + (uint32_t)(((uint64_t)u * (b1 - b0)) >> 32);
}

}  // namespace tsdfl
