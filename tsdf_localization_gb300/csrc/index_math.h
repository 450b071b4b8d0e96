// Slot index of CudaSubVoxelMap::getIndex (cuda_sub_voxel_map.tcc:50-137) for
// map offsets that are finite and below 2^22 in magnitude, in plain signed
// integer arithmetic.  Shared by the device kernels (second tier behind the
// branch-free fast path) and by the host-side checks against the oracle.
//
// The reference converts float offsets to size_t; its x86-64 build gives, per
// axis with offset o and resolution res <= 1:
//   o >= 0       brick coordinate trunc(o), sub-voxel index trunc((o - trunc(o)) / res)
//   -1 < o < 0   brick coordinate 0, sub-voxel index -trunc(|o| / res) (wraps mod 2^64)
//   o <= -1      the coarse bound check passes (2^64 / res converts to 0), the
//                brick coordinate wraps to -trunc(|o|) and the sub-voxel index
//                becomes 2^63, which cancels mod 2^64 when an even number of
//                such terms (weighted by 1, sub_dim, sub_dim^2) add up.
// All sums are mod 2^64 in the reference, i.e. signed 64-bit arithmetic here.
#pragma once

#include <stdint.h>

#include "tsdfl_internal.h"

#if defined(__CUDACC__)
#define TSDFL_HD __host__ __device__ __forceinline__
#else
#define TSDFL_HD inline
#endif

namespace tsdfl {

constexpr uint32_t kIdxMiss = 0xffffffffu;   // getEntry returns the init value
constexpr uint32_t kIdxSlow = 0xfffffffeu;   // outside this function's domain

TSDFL_HD float div_rn(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}

TSDFL_HD uint32_t bits_of(float f)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    union { float f; uint32_t u; } v;
    v.f = f;
    return v.u;
#endif
}

struct AxisIdx {
    int64_t m;   // brick coordinate
    int64_t q;   // sub-voxel index (when !big)
    int big;     // sub-voxel index is 2^63
};

// Returns 0 = handled (a), 1 = the coarse bound check fails (miss), 2 = slow.
TSDFL_HD int axis_index(float o, uint32_t lim_bits, float res, AxisIdx& a)
{
    if (lim_bits == 0) return 1;   // not even brick 0 passes the coarse check on this axis
    const float mag = o < 0.0f ? -o : o;
    if (!(mag < 4194304.0f)) return 2;   // NaN, inf, huge
    if (o >= 0.0f) {
        if (bits_of(o) >= lim_bits) return 1;   // trunc(o) above the last brick that passes
        const int64_t mi = (int64_t)o;          // truncation
        const float s = o - (float)mi;          // exact
        a.m = mi;
        a.q = (int64_t)div_rn(s, res);
        a.big = 0;
        return 0;
    }
    const int64_t mi = (int64_t)mag;
    if (mi == 0) {
        a.m = 0;
        a.q = -(int64_t)div_rn(mag, res);
        a.big = 0;
        return 0;
    }
    if (!(res <= 1.0f)) return 2;   // the wrapped coarse check then depends on res
    a.m = -mi;
    a.q = 0;
    a.big = 1;
    return 0;
}

// Slot index for offsets (ox, oy, oz) = point - map min, kIdxMiss on a miss,
// kIdxSlow when an offset is NaN, infinite or at least 2^22 in magnitude.
TSDFL_HD uint32_t slot_index_tier2(const MapView& m, const int32_t* grid_occ, float ox, float oy, float oz)
{
    AxisIdx ax, ay, az;
    const int rx = axis_index(ox, m.lim_x, m.res, ax);
    const int ry = axis_index(oy, m.lim_y, m.res, ay);
    const int rz = axis_index(oz, m.lim_z, m.res, az);
    if (rx == 2 || ry == 2 || rz == 2) return kIdxSlow;
    if (rx == 1 || ry == 1 || rz == 1) return kIdxMiss;
    const int64_t up = ax.m + ay.m * (int64_t)m.up_dim_x64 + az.m * (int64_t)m.up_dim_2_64;
    if ((uint64_t)up >= m.grid_occ_size64) return kIdxMiss;
    const int32_t base = grid_occ[up];
    if (base < 0) return kIdxMiss;
    const int64_t S = (int64_t)m.sub_dim64, S2 = (int64_t)m.sub_dim_2_64;
    const int64_t parity = (ax.big ? 1 : 0) + (ay.big ? S : 0) + (az.big ? S2 : 0);
    if (parity & 1) return kIdxMiss;   // an odd number of 2^63 terms: the index is >= 2^63
    const int64_t idx = (int64_t)base + (ax.big ? 0 : ax.q) + (ay.big ? 0 : ay.q * S) + (az.big ? 0 : az.q * S2);
    if ((uint64_t)idx >= m.data_size64) return kIdxMiss;
    return (uint32_t)idx;
}

#if defined(__CUDACC__)
// Slot index of a map-frame point with the exact reference semantics,
// kMissIndex on a miss: fast path for offsets in [0, mmax + 1) on all axes,
// the signed second tier for other finite offsets, the full 64-bit emulation
// (slot_index_slow) for NaN, infinite and huge offsets.
static __device__ __forceinline__ uint32_t slot_index(const MapView& m, float x, float y, float z)
{
    float ox = __fsub_rn(x, m.min_x), oy = __fsub_rn(y, m.min_y), oz = __fsub_rn(z, m.min_z);
    bool fast = __float_as_uint(ox) < m.lim_x && __float_as_uint(oy) < m.lim_y && __float_as_uint(oz) < m.lim_z;
    if (!fast) {
        uint32_t r = slot_index_tier2(m, m.grid_occ, ox, oy, oz);
        return r == kIdxSlow ? slot_index_slow(m, x, y, z) : r;
    }
    int32_t mx = __float2int_rz(ox), my = __float2int_rz(oy), mz = __float2int_rz(oz);
    uint32_t up = (uint32_t)mx + (uint32_t)my * m.up_dim_x + (uint32_t)mz * m.up_dim_2;
    if (up >= m.grid_occ_size) return kMissIndex;
    int32_t base = __ldg(m.grid_occ + up);
    if (base < 0) return kMissIndex;
    float sx = __fsub_rn(ox, (float)mx), sy = __fsub_rn(oy, (float)my), sz = __fsub_rn(oz, (float)mz);
    uint32_t qx = (uint32_t)__float2int_rz(__fdiv_rn(sx, m.res));
    uint32_t qy = (uint32_t)__float2int_rz(__fdiv_rn(sy, m.res));
    uint32_t qz = (uint32_t)__float2int_rz(__fdiv_rn(sz, m.res));
    uint32_t idx = (uint32_t)base + qx + qy * m.sub_dim + qz * m.sub_dim_2;
    return idx < m.data_size ? idx : kMissIndex;
}
#endif

}  // namespace tsdfl
