// Sensor-update kernels for sm_103a: pose build, scan staging, per-particle
// scoring, normalisation / mean pose, systematic resampling, map re-layout.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <vector>

#include "index_math.h"
#include "subsample.h"
#include "tsdfl_internal.h"

namespace tsdfl {

std::atomic<unsigned long long> g_launches{0};

namespace {

constexpr int kLutBytes = ((kNumCodes * 8 + 15) / 16) * 16;
constexpr int kLutFBytes = ((kNumCodes * 4 + 15) / 16) * 16;

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// 1-D bulk copy global -> this CTA's shared memory, completing on bar
// (cp.async.bulk; src, dst 16-byte aligned, bytes a multiple of 16).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}

// Bounded wait: gives up after ~2^22 polls (try_wait itself suspends for a
// while each time), so a copy that never lands cannot hang the GPU.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t phase)
{
    for (uint32_t i = 0; i < (1u << 22); ++i)
        if (mbar_try_wait(bar, phase)) return true;
    return false;
}

// Stages n floats of three arrays into shared memory with bulk copies; every
// thread of the block must call it.  Returns false (and raises status) when
// the copies did not complete in time.
__device__ bool stage_xyz(float* xs, float* ys, float* zs, const float* gx, const float* gy, const float* gz,
                          int npad, uint64_t* bar, int32_t* status)
{
    if (threadIdx.x == 0) mbar_init(bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t bytes = (uint32_t)npad * 4u;
        mbar_expect_tx(bar, 3u * bytes);
        bulk_g2s(xs, gx, bytes, bar);
        bulk_g2s(ys, gy, bytes, bar);
        bulk_g2s(zs, gz, bytes, bar);
    }
    bool ok = mbar_wait_bounded(bar, 0);
    if (!ok) ok = mbar_wait_bounded(bar, 0);   // give copies in flight a second bound
    if (!ok && threadIdx.x == 0) atomicExch(status, TSDFL_ERR_TIMEOUT);
    return __syncthreads_and(ok ? 1 : 0) != 0;
}

__device__ __forceinline__ long long warp_sum_ll(long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ uint32_t warp_sum_u32(uint32_t v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// First statement of every kernel of the update and resampling chain, which
// the launchers start with programmatic dependent launch: the grid may be
// scheduled while the previous kernel in the stream is still running, so it
// waits here until that kernel has completed and its writes are visible, then
// lets its own successor be scheduled once all of its CTAs have started (the
// successor waits in turn).  Both instructions do nothing for a grid launched
// without the attribute.
__device__ __forceinline__ void chain_enter()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Element-wise min (x, y) / max (z, w) over the warp; NaN entries are ignored.
__device__ __forceinline__ float4 warp_extent(float4 e)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        e.x = fminf(e.x, __shfl_xor_sync(0xffffffffu, e.x, o));
        e.y = fminf(e.y, __shfl_xor_sync(0xffffffffu, e.y, o));
        e.z = fmaxf(e.z, __shfl_xor_sync(0xffffffffu, e.z, o));
        e.w = fmaxf(e.w, __shfl_xor_sync(0xffffffffu, e.w, o));
    }
    return e;
}

__device__ __forceinline__ double warp_sum_d(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Code of the slot a point falls in (kCodeMiss when getIndex misses): the
// generic kernel's view of a map with the compact layout, read through the
// brick table.
__device__ __forceinline__ uint32_t dense_code(const MapView& m, float x, float y, float z)
{
    uint32_t idx = slot_index(m, x, y, z);
    return idx == kMissIndex ? (uint32_t)kCodeMiss : (uint32_t)__ldg(m.codes + idx);
}

// Spread clouds' particle order: 2^kCellBits x 2^kCellBits cells (below).
constexpr int kCellBits = 6;
constexpr int kCellBins = 1 << (2 * kCellBits);

struct PointParams {
    const float* points;  // N x 3
    int N, npad, npairs;
    const float* particles;  // P x 7 (the cloud's extent is taken from a sample)
    int P;
    float max_range_sq, c_in, c_out;
    const float* code_values;  // kNumCodes floats (device)
    int shift;                 // fixed-point scale 2^shift
};

// Spatial order of the pair layout: the tiled kernels walk the scan in chunks
// of consecutive points with every particle at once, so the order decides how
// much of the map a chunk touches across the cloud; exact fixed-point sums make
// the result independent of it.  A compact cloud (tracking) gathers least with
// chunks that are compact in the sensor frame: azimuth sector, then range band
// (0.5 m).  A cloud spread over the map (global localisation, any yaw) gathers
// least with chunks of one height band (1 m), whose hits stay in one layer of
// the map whatever the particle's position and yaw: height, sector, then range
// band (2 m).  The cloud counts as spread when its x or y extent exceeds
// kWideCloud.
constexpr int kSortSectors = 16;
constexpr int kSortBins = 2048;
constexpr float kWideCloud = 10.0f;   // metres
constexpr int kPrepThreads = 1024;
constexpr int kBinCache = 16384;    // points whose bin the staging keeps in shared memory
static_assert(kSortBins == 2 * kPrepThreads, "two bins per thread in the scan");

// Sector of the diamond angle (|y| / (|x| + |y|) per quadrant, counter-clockwise
// from +x: monotone in the azimuth, no trigonometry), with the range band and,
// for a spread cloud, the height band.
__device__ __forceinline__ int spatial_bin(float x, float y, float z, bool wide)
{
    const float r1 = fabsf(x) + fabsf(y);
    if (!(r1 < 1e30f) || !(fabsf(z) < 1e30f)) return kSortBins - 1;   // NaN / huge: last
    const float t = r1 > 0.0f ? __fdividef(fabsf(y), r1) : 0.0f;
    const float a = x >= 0.0f ? (y >= 0.0f ? t : 4.0f - t) : (y >= 0.0f ? 2.0f - t : 2.0f + t);   // [0, 4]
    const int s = min((int)(a * (0.25f * kSortSectors)), kSortSectors - 1);
    const float r = sqrtf(x * x + y * y);
    if (!wide) return s * 128 + (int)fminf(r * 2.0f, 127.0f);   // 16 sectors x 128 bands of 0.5 m
    const int zb = (int)fminf(fmaxf(floorf(z) + 4.0f, 0.0f), 7.0f);   // [-4, 4) m in 1 m bands
    return (zb * kSortSectors + s) * 16 + (int)fminf(r * 0.5f, 15.0f);   // x 16 bands of 2 m
}

// Scan staging: AoS points -> SoA (padded with zeros to npad), the per-point
// score constant of tsdf_evaluator.cpp:56-65 and the number of points inside
// max_range; the pair layout of the tiled kernels in spatial order (a counting
// sort by spatial_bin; perm records each position's scan index); also the
// likelihood tables for this scan.  Block 0 of pose_prepare_kernel, beside the
// pose blocks.  Which order suits the cloud (compact or spread) is decided on
// the x / y extent of a sample of at most kExtentSample particles, and the
// particle order's cells span that extent (clamped at its edges); both only
// decide how fast the scoring runs, never what it returns.
constexpr int kExtentSample = 4096;

__device__ __forceinline__ void prepare_points_block(const PointParams& p, const EvalBuffers& b)
{
    __shared__ int warp_counts[32];
    __shared__ int bins[kSortBins];
    __shared__ uint16_t sbin[kBinCache];
    __shared__ float4 s_ext[32];
    __shared__ int s_wide;
    if (threadIdx.x == 0) *b.status = 0;
    for (int c = threadIdx.x; c < kCellBins; c += blockDim.x) b.phist[c] = 0;   // the particle order's histogram
    {   // the cloud's x / y extent from a sample of the particles
        const float inf = __int_as_float(0x7f800000);
        float4 e = make_float4(inf, inf, -inf, -inf);
        const int n_s = min(p.P, kExtentSample), stride = max(1, p.P / kExtentSample);
        for (int k = threadIdx.x; k < n_s; k += blockDim.x) {
            const float* q = p.particles + 7 * (size_t)k * (size_t)stride;
            const float x = q[0], y = q[1];
            e = make_float4(fminf(e.x, x), fminf(e.y, y), fmaxf(e.z, x), fmaxf(e.w, y));
        }
        e = warp_extent(e);
        if ((threadIdx.x & 31) == 0) s_ext[threadIdx.x >> 5] = e;
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
                const float4 v = s_ext[w];
                e = make_float4(fminf(e.x, v.x), fminf(e.y, v.y), fmaxf(e.z, v.z), fmaxf(e.w, v.w));
            }
            s_wide = fmaxf(e.z - e.x, e.w - e.y) > kWideCloud ? 1 : 0;   // no particles: -inf
            b.counts[2] = s_wide;   // the particles are put in spatial order too
            b.cloud_ext[0] = e;
        }
    }
    for (int i = threadIdx.x; i < kSortBins; i += blockDim.x) bins[i] = 0;
    __syncthreads();
    const bool wide = s_wide != 0;
    int in = 0;
#pragma unroll 4
    for (int j = threadIdx.x; j < p.npad; j += blockDim.x) {
        float x = 0, y = 0, z = 0, c = 0;
        if (j < p.N) {
            x = __ldg(p.points + 3 * j);
            y = __ldg(p.points + 3 * j + 1);
            z = __ldg(p.points + 3 * j + 2);
            float sq = __fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z));
            bool inr = sq < p.max_range_sq;
            c = inr ? p.c_in : p.c_out;
            in += inr ? 1 : 0;
            const int bin = spatial_bin(x, y, z, wide);
            atomicAdd(&bins[bin], 1);
            if (j < kBinCache) sbin[j] = (uint16_t)bin;
        }
        ((float*)b.xs)[j] = x;
        ((float*)b.ys)[j] = y;
        ((float*)b.zs)[j] = z;
        ((float*)b.cs)[j] = c;
    }
    __syncthreads();   // counts complete; this block's SoA stores visible to it
    {   // exclusive scan of the bin counts, two bins per thread
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const int c0 = bins[2 * threadIdx.x], c1 = bins[2 * threadIdx.x + 1];
        int v = c0 + c1;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += t;
        }
        if (lane == 31) warp_counts[warp] = v;
        __syncthreads();
        if (warp == 0) {
            int w = lane < (int)(blockDim.x >> 5) ? warp_counts[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += t;
            }
            warp_counts[lane] = w;   // inclusive over warps
        }
        __syncthreads();
        const int before = (warp ? warp_counts[warp - 1] : 0) + v - c0 - c1;
        bins[2 * threadIdx.x] = before;
        bins[2 * threadIdx.x + 1] = before + c0;
    }
    __syncthreads();
    // pair layout of the fast kernel: in every block of 64 positions, lane l of
    // a warp takes positions 64*blk + l and 64*blk + 32 + l
    for (int j = threadIdx.x; j < p.N; j += blockDim.x) {
        const float x = b.xs[j], y = b.ys[j], z = b.zs[j];
        const int q = atomicAdd(&bins[j < kBinCache ? (int)sbin[j] : spatial_bin(x, y, z, wide)], 1);
        const int pair = (q >> 6) * 32 + (q & 31), half = (q >> 5) & 1;
        float* xy = reinterpret_cast<float*>(b.pxy + pair);
        xy[half] = x;
        xy[2 + half] = y;
        reinterpret_cast<float*>(b.pz + pair)[half] = z;
        b.perm[q] = j;
    }
    for (int q = p.N + threadIdx.x; q < 2 * p.npairs; q += blockDim.x) {   // padding positions
        const int pair = (q >> 6) * 32 + (q & 31), half = (q >> 5) & 1;
        float* xy = reinterpret_cast<float*>(b.pxy + pair);
        xy[half] = 0.0f;
        xy[2 + half] = 0.0f;
        reinterpret_cast<float*>(b.pz + pair)[half] = 0.0f;
        b.perm[q] = 0;   // never read: padding lanes record no debug code
    }
    for (int c = threadIdx.x; c < kNumCodes; c += blockDim.x) {
        float v = p.code_values[c];
        b.lut_f[c] = v;
        b.lut_fx[c] = __double2ll_rn(ldexp((double)v, p.shift));
    }
    in = (int)warp_sum_u32((uint32_t)in);
    if ((threadIdx.x & 31) == 0) warp_counts[threadIdx.x >> 5] = in;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += warp_counts[w];
        b.counts[0] = t;
    }
}

// Spatial order of a spread cloud's particles (global localisation): 64 x 64
// cells over the particles' x / y extent, numbered along a Morton curve; a
// counting sort puts the particles in cell order.  The tiled kernel then walks
// regions of consecutive particles, so that at any time the grid scores
// particles from one part of the map and the gathers stay in the L2.  The
// order within a cell depends on the atomics, which changes nothing: every
// particle's sums are exact integers written to its own index.
constexpr int kCellScanThreads = 1024;
static_assert(kCellBins == 4 * kCellScanThreads, "four bins per thread in the scan");

__device__ __forceinline__ uint32_t morton2(uint32_t x, uint32_t y)
{
    uint32_t m = 0;
#pragma unroll
    for (int k = 0; k < kCellBits; ++k) m |= (((x >> k) & 1u) << (2 * k)) | (((y >> k) & 1u) << (2 * k + 1));
    return m;
}

__global__ void particle_cells_kernel(const float* particles, int P, EvalBuffers b)
{
    chain_enter();
    if (b.counts[2] == 0) return;   // a compact cloud keeps its order
    const float4 e = b.cloud_ext[0];
    const float n = (float)(1 << kCellBits);
    const float sx = n / fmaxf(e.z - e.x, 1e-3f), sy = n / fmaxf(e.w - e.y, 1e-3f);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
        const float x = particles[7 * (size_t)i], y = particles[7 * (size_t)i + 1];
        // fmaxf / fminf also send NaN positions to cell 0
        const uint32_t cx = (uint32_t)fminf(fmaxf((x - e.x) * sx, 0.0f), n - 1.0f);
        const uint32_t cy = (uint32_t)fminf(fmaxf((y - e.y) * sy, 0.0f), n - 1.0f);
        const uint32_t key = morton2(cx, cy);
        b.pkeys[i] = key;
        atomicAdd(&b.phist[key], 1);
    }
}

__global__ void __launch_bounds__(kCellScanThreads) particle_scan_kernel(EvalBuffers b)
{
    chain_enter();
    if (b.counts[2] == 0) return;
    __shared__ int warp_sums[kCellScanThreads / 32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    int c[4], v = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        c[k] = b.phist[4 * t + k];
        v += c[k];
    }
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int w = warp_sums[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += u;
        }
        warp_sums[lane] = w;   // inclusive over warps
    }
    __syncthreads();
    int run = (warp ? warp_sums[warp - 1] : 0) + incl - v;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        b.phist[4 * t + k] = run;
        run += c[k];
    }
}

__global__ void particle_scatter_kernel(int P, EvalBuffers b)
{
    chain_enter();
    if (b.counts[2] == 0) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
        const int q = atomicAdd(&b.phist[b.pkeys[i]], 1);
        b.order[q] = (uint32_t)i;
    }
}

struct Tf16 {
    float v[16];
};

// Laser pose of every particle (tsdf_evaluator.cpp:102-147): trig in double,
// rounded to float (the correctly rounded sin/cos), products and sums in the
// reference's order without contraction.  Three lanes per particle, ten
// particles a warp (lanes 30 and 31 idle): lane 3p + k forms the sine and
// cosine of angle k (roll, pitch, yaw), the three exchange them by shuffles,
// and lane 3p + r forms row r of the 3 x 4 laser pose, so the FP64 latency of
// the three sincos is spread over three lanes.  Also zeros in the scoring
// sums, so no memset breaks the chain of kernels.  `blk` numbers the pose
// blocks of pose_prepare_kernel.
__device__ __forceinline__ void pose_block(int blk, const float* particles, int P, const Tf16& tf, float* pose12,
                                           float* trig6, long long* sum_fx, uint32_t* hits)
{
    const int lane = threadIdx.x & 31;
    const int slot = lane / 3, k = lane - 3 * slot;
    const int i = (blk * (kPoseThreads / 32) + (int)(threadIdx.x >> 5)) * kPoseSlots + slot;
    const bool active = slot < kPoseSlots && i < P;
    if (active && k == 0) {   // the tiled kernel's per-particle sums start at zero
        sum_fx[i] = 0;
        hits[i] = 0;
    }
    const float* p = particles + 7 * (size_t)(active ? i : 0);
    double sd, cd;
    sincos((double)p[3 + (k < 3 ? k : 0)], &sd, &cd);
    const float sv = (float)sd, cv = (float)cd;
    const int base = 3 * slot;
    auto from = [&](float v, int j) { return __shfl_sync(0xffffffffu, v, min(base + j, 31)); };
    const float sin_alpha = from(sv, 0), cos_alpha = from(cv, 0);
    const float sin_beta = from(sv, 1), cos_beta = from(cv, 1);
    const float sin_gamma = from(sv, 2), cos_gamma = from(cv, 2);
    if (!active) return;
    float a[4];   // row k of the particle's transform
    if (k == 0) {
        a[0] = __fmul_rn(cos_beta, cos_gamma);
        a[1] = __fsub_rn(__fmul_rn(__fmul_rn(sin_alpha, sin_beta), cos_gamma), __fmul_rn(cos_alpha, sin_gamma));
        a[2] = __fadd_rn(__fmul_rn(__fmul_rn(cos_alpha, sin_beta), cos_gamma), __fmul_rn(sin_alpha, sin_gamma));
        a[3] = p[0];
    } else if (k == 1) {
        a[0] = __fmul_rn(cos_beta, sin_gamma);
        a[1] = __fadd_rn(__fmul_rn(__fmul_rn(sin_alpha, sin_beta), sin_gamma), __fmul_rn(cos_alpha, cos_gamma));
        a[2] = __fsub_rn(__fmul_rn(__fmul_rn(cos_alpha, sin_beta), sin_gamma), __fmul_rn(sin_alpha, cos_gamma));
        a[3] = p[1];
    } else {
        a[0] = -sin_beta;
        a[1] = __fmul_rn(sin_alpha, cos_beta);
        a[2] = __fmul_rn(cos_alpha, cos_beta);
        a[3] = p[2];
    }
    const float* f = tf.v;
    float o[4];
#pragma unroll
    for (int c = 0; c < 3; ++c)
        o[c] = __fadd_rn(__fadd_rn(__fmul_rn(a[0], f[c]), __fmul_rn(a[1], f[4 + c])), __fmul_rn(a[2], f[8 + c]));
    o[3] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(a[0], f[3]), __fmul_rn(a[1], f[7])), __fmul_rn(a[2], f[11])), a[3]);
    reinterpret_cast<float4*>(pose12 + 12 * (size_t)i)[k] = make_float4(o[0], o[1], o[2], o[3]);
    float* tg = trig6 + 6 * (size_t)i;
    tg[2 * k] = sv;
    tg[2 * k + 1] = cv;
}

// First kernel of an update: block 0 stages the scan (prepare_points_block),
// the others form the laser poses (pose_block); the two parts share no data,
// so they run side by side.
__global__ void __launch_bounds__(kPoseThreads) pose_prepare_kernel(Tf16 tf, PointParams p, EvalBuffers b)
{
    chain_enter();
    if (blockIdx.x == 0) prepare_points_block(p, b);
    else pose_block((int)blockIdx.x - 1, p.particles, p.P, tf, b.pose12, b.trig6, b.sum_fx, b.hits);
}

struct EvalParams {
    MapView m;
    const float4* pxy;
    const float2* pz;
    const int32_t* perm;   // scan index of each pair-layout point (debug rows)
    const float* pose12;
    const float* xs;
    const float* ys;
    const float* zs;
    const float* cs;
    const long long* lut_fx;
    const float* lut_f;
    long long* sum_fx;   // exact mode, code storage
    double* sum_f64;     // exact mode, float storage
    float* raw;          // serial mode
    uint32_t* hits;
    uint32_t* dbg;       // optional: P x N_total slot index (brick) / code (dense)
    const uint32_t* order;   // spatial order of the particles (used when *sched != 0)
    const int32_t* sched;    // the staging kernel's spread-cloud flag (null: original order)
    int32_t* status;
    int P;
    int n0, n1;          // point range of this pass
    int n_total;
    int first_pass;
    float a_hit;
};

// Exact mode: one warp per particle, lanes stride over the scan (neighbouring
// lanes take neighbouring scan points, so their map gathers fall close
// together).  Likelihood values are summed in 64-bit fixed point, which is
// exact and independent of order; the weight is formed from the sum afterwards.
template <bool DENSE, int ST>
__global__ void __launch_bounds__(1024, 1) eval_exact_kernel(EvalParams p)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint64_t bar;
    long long* lut = reinterpret_cast<long long*>(smem);
    const int n = p.n1 - p.n0;
    const int npad = (n + 3) & ~3;
    float* xs = reinterpret_cast<float*>(smem + kLutBytes);
    float* ys = xs + npad;
    float* zs = ys + npad;
    for (int c = threadIdx.x; c < kNumCodes; c += blockDim.x) lut[c] = p.lut_fx[c];
    if (!stage_xyz(xs, ys, zs, p.xs + p.n0, p.ys + p.n0, p.zs + p.n0, npad, &bar, p.status)) return;

    const int lane = threadIdx.x & 31;
    const int warps = (blockDim.x >> 5) * gridDim.x;
    const MapView& m = p.m;
    for (int pi = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); pi < p.P; pi += warps) {
        float t[12];
        const float4* src = reinterpret_cast<const float4*>(p.pose12 + 12 * (size_t)pi);
        float4 a = __ldg(src), b4 = __ldg(src + 1), c4 = __ldg(src + 2);
        t[0] = a.x; t[1] = a.y; t[2] = a.z; t[3] = a.w;
        t[4] = b4.x; t[5] = b4.y; t[6] = b4.z; t[7] = b4.w;
        t[8] = c4.x; t[9] = c4.y; t[10] = c4.z; t[11] = c4.w;
        long long acc = 0;
        double accd = 0.0;
        uint32_t h = 0;
        for (int j = lane; j < n; j += 32) {
            float tx, ty, tz;
            transform_point(t, xs[j], ys[j], zs[j], tx, ty, tz);
            if (DENSE) {
                uint32_t code = dense_code(m, tx, ty, tz);
                h += code != (uint32_t)kCodeMiss ? 1u : 0u;
                acc += lut[code];
                if (p.dbg) p.dbg[(size_t)pi * p.n_total + p.n0 + j] = code;
            } else {
                uint32_t idx = slot_index(m, tx, ty, tz);
                if (ST == 1) {
                    float v = idx != kMissIndex ? __ldg(m.data + idx) : m.init_value;
                    accd += (double)v;
                } else if (ST == 2) {
                    float v = idx != kMissIndex ? __half2float(__ushort_as_half(__ldg(m.h16 + idx))) : m.init_value;
                    accd += (double)v;
                } else {
                    uint32_t code = idx != kMissIndex ? (uint32_t)__ldg(m.codes + idx) : (uint32_t)kCodeInit;
                    acc += lut[code];
                }
                h += idx != kMissIndex ? 1u : 0u;
                if (p.dbg) p.dbg[(size_t)pi * p.n_total + p.n0 + j] = idx;
            }
        }
        h = warp_sum_u32(h);
        if (ST != 0) accd = warp_sum_d(accd);
        else acc = warp_sum_ll(acc);
        if (lane == 0) {
            if (ST != 0) p.sum_f64[pi] = p.first_pass ? accd : p.sum_f64[pi] + accd;
            else p.sum_fx[pi] = p.first_pass ? acc : p.sum_fx[pi] + acc;
            p.hits[pi] = p.first_pass ? h : p.hits[pi] + h;
        }
    }
}

// ---------------------------------------------------------------- tiled kernel

typedef unsigned long long f2_t;   // two floats in one 64-bit register pair

__device__ __forceinline__ f2_t pk(float a, float b)
{
    f2_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk(f2_t v, float& a, float& b)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
// Packed additions: ptxas fuses a packed multiply feeding a packed add into an
// FMA even with explicit .rn, so products that feed additions stay scalar
// (__fmul_rn is never contracted).  mul2 is used only where its product is the
// addend of an FMA, which no contraction can absorb.
__device__ __forceinline__ f2_t add2(f2_t a, f2_t b)
{
    f2_t r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2_t add2_rz(f2_t a, f2_t b)
{
    f2_t r;
    asm("add.rz.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2_t sub2(f2_t a, f2_t b)
{
    f2_t r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2_t and2(f2_t a, f2_t b)
{
    f2_t r;
    asm("and.b64 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2_t mul2(f2_t a, f2_t b)
{
    f2_t r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2_t fma2_rn(f2_t a, f2_t b, f2_t c)
{
    f2_t r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
__device__ __forceinline__ f2_t fma2_rz(f2_t a, f2_t b, f2_t c)
{
    f2_t r;
    asm("fma.rz.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

__device__ __forceinline__ f2_t or2(f2_t a, f2_t b)
{
    f2_t r;
    asm("or.b64 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}

constexpr uint32_t kMagic = 0x4B000000u;     // bits of 2^23

// Code of a point the fast path does not cover: finite offsets go through the
// signed second tier, NaN / infinite / huge ones through the 64-bit emulation.
__device__ __forceinline__ uint32_t slow_code(const MapView& m, float x, float y, float z)
{
    const float ox = __fsub_rn(x, m.min_x), oy = __fsub_rn(y, m.min_y), oz = __fsub_rn(z, m.min_z);
    uint32_t idx = slot_index_tier2(m, m.grid_occ, ox, oy, oz);
    if (idx == kIdxSlow) idx = slot_index_slow(m, x, y, z);
    return idx == kMissIndex ? (uint32_t)kCodeMiss : (uint32_t)__ldg(m.codes + idx);
}

// Likelihood table entry in shared memory: the fixed-point value of a code.
// Entries 8 bytes apart spread a warp's random reads over 16 bank pairs (a
// 16-byte entry with the hit flag beside it left 8 and cost more shared-memory
// wavefronts than the hit compare saves).
struct __align__(8) LutEntry {
    long long v;
};
constexpr int kLutTableBytes = ((kNumCodes * 8 + 15) / 16) * 16;

// Branch-free fast path of one lookup, from the packed pipeline's outputs: the
// offsets' float bits (x, y) and value (z), upb = kMagic + brick index and
// slb = bits(1.5 * 2^23) + sub-voxel offset.  Returns the gathered code: the slot's, or
// a sentinel's -- kCodeMiss (fast, but the brick is outside the grid or not
// allocated), kCodeLater (the exact slow tiers decide: offset outside
// [0, mmax + 1) on x or y, outside (-1, mmax + 1) on z; `slow` is set) or
// kCodeNone (a padding point, valid false).
// LAY: where the brick's rank comes from -- kLayBitmap: the shared-memory
// bitmap `occ`; kLayHash: the sparse brick hash (allocated bricks only, for
// maps whose bitmap does not fit shared memory); kLayTable: the brick table
// grid_occ (the reference's own); kLayGrid: no rank, the grid layout's codes
// of every brick of the bounding box are addressed by the brick index.
constexpr int kLayTable = 0, kLayBitmap = 1, kLayHash = 2, kLayGrid = 3;

template <int LAY>
__device__ __forceinline__ uint32_t fast_code(const MapView& m, const unsigned char* occ, uint32_t ox_b,
                                              uint32_t oy_b, float oz, uint32_t upb, uint32_t slb, bool valid,
                                              bool& slow)
{
    const bool fast = ox_b < m.lim_x && oy_b < m.lim_y && oz > m.zlo && oz < m.zhi;
    slow = valid && !fast;
    const bool inside = valid && fast && upb < m.upb_lim;
    uint32_t idx;
    bool ok;
    if (LAY == kLayHash) {
        // open addressing, linear probing: every key lies within hash_probes
        // slots of its home, and every run of keys ends at an empty slot within
        // that bound (measured when the table is built)
        const uint32_t up = upb - kMagic;
        uint32_t rank = 0;
        bool found = false;
        if (inside) {
            const uint32_t h = (up * 0x9E3779B1u) >> m.hash_shift;
            for (uint32_t t = 0; t < m.hash_probes; ++t) {
                const uint2 e = __ldg(m.hash + ((h + t) & m.hash_mask));
                if (e.x == up) {
                    rank = e.y;
                    found = true;
                    break;
                }
                if (e.x == kHashEmpty) break;
            }
        }
        ok = found;
        idx = rank * m.sub_dim_3 + slb;
    } else if (LAY == kLayGrid) {
        // every brick of the bounding box is stored: a miss is a miss code there
        const uint32_t up = upb - kMagic;
        ok = inside;
        idx = (up + min(up, m.grid_uxy1)) * m.sub_dim_3 + slb;
    } else if (LAY == kLayBitmap) {
        // the masked offset stays inside the staged table whatever upb is
        const uint2 wb = *reinterpret_cast<const uint2*>(occ + ((upb >> 2) & m.occ_mask));
        const uint32_t v = __funnelshift_r(wb.x, 0u, upb);   // word >> (brick & 31)
        ok = inside && (v & 1u) != 0u;
        idx = (wb.y - (uint32_t)__popc(v)) * m.sub_dim_3 + slb;
    } else {
        const int32_t base = __ldg(m.grid_occ + (inside ? upb - kMagic : 0u));
        ok = inside && base >= 0;
        idx = (uint32_t)base + slb;
    }
    if (LAY == kLayGrid) {
        const uint32_t sent = valid ? (fast ? m.gsent_miss : m.gsent_later) : m.gsent_none;
        return __ldg(reinterpret_cast<const uint16_t*>(m.grid_b + 2ull * (ok ? idx : sent)));
    }
    const uint32_t sent = valid ? (fast ? m.sent_miss : m.sent_later) : m.sent_none;
    return __ldg(reinterpret_cast<const uint16_t*>(m.codes_b + 2ull * (ok ? idx : sent)));
}

// Constants of the packed index pipeline, each a pair of equal floats.
struct PipeConsts {
    f2_t NMX, NMY, NMZ;       // the map's min corner
    f2_t MAG, MAG15;          // 2^23, 1.5 * 2^23
    f2_t INV, INVLO;          // sub-voxel multiplier terms
    f2_t UX, UXY, SD, SD2;    // up_dim_x, up_dim_x * up_dim_y, sub_dim, sub_dim^2
    f2_t NZ;                  // -0
};

__device__ __forceinline__ PipeConsts pipe_consts(const MapView& m)
{
    PipeConsts c;
    c.NMX = pk(m.min_x, m.min_x);
    c.NMY = pk(m.min_y, m.min_y);
    c.NMZ = pk(m.min_z, m.min_z);
    c.MAG = pk(8388608.0f, 8388608.0f);
    c.MAG15 = pk(12582912.0f, 12582912.0f);
    c.INV = pk(m.sub_inv, m.sub_inv);
    c.INVLO = pk(m.sub_inv_lo, m.sub_inv_lo);
    c.UX = pk(m.up_dim_x_f, m.up_dim_x_f);
    c.UXY = pk(m.up_dim_2_f, m.up_dim_2_f);
    c.SD = pk(m.sub_dim_f, m.sub_dim_f);
    c.SD2 = pk(m.sub_dim_2_f, m.sub_dim_2_f);
    c.NZ = pk(m.neg_zero, m.neg_zero);
    return c;
}

// A laser pose (3 x 4, row-major) as pairs: both halves of R[k] hold entry k
// for a pose shared by the pair's two lookups, or entry k of two poses.
struct PosePairs {
    f2_t R[12];
};

__device__ __forceinline__ PosePairs pose_pairs(const float* pose12)
{
    const float4* src = reinterpret_cast<const float4*>(pose12);
    const float4 a = __ldg(src), b = __ldg(src + 1), c = __ldg(src + 2);
    PosePairs r;
    r.R[0] = pk(a.x, a.x); r.R[1] = pk(a.y, a.y); r.R[2] = pk(a.z, a.z); r.R[3] = pk(a.w, a.w);
    r.R[4] = pk(b.x, b.x); r.R[5] = pk(b.y, b.y); r.R[6] = pk(b.z, b.z); r.R[7] = pk(b.w, b.w);
    r.R[8] = pk(c.x, c.x); r.R[9] = pk(c.y, c.y); r.R[10] = pk(c.z, c.z); r.R[11] = pk(c.w, c.w);
    return r;
}

// Transform and fast-path lookup of two sensor-frame points (X, Y, Z pairs):
// the gathered codes k0, k1, whether the exact slow tiers must decide them
// (s0, s1), and the transformed points (for the deferral).  v0 / v1: the
// lookup is a real point (false: padding, kCodeNone).
template <int LAY, bool TWO, bool MIN0>
__device__ __forceinline__ void pair_lookup(const MapView& m, const unsigned char* occ, const PosePairs& P,
                                            const PipeConsts& K, f2_t X, f2_t Y, f2_t Z, bool v0, bool v1,
                                            uint32_t& k0, uint32_t& k1, bool& s0, bool& s1, f2_t& TX, f2_t& TY,
                                            f2_t& TZ)
{
    const f2_t ABS = 0x7fffffff7fffffffull, SGN = 0x8000000080000000ull;
    // tsdf_evaluator.cpp:44-46: ((r0 x + r1 y) + r2 z) + r3, every product and
    // sum rounded (products as FMAs with a -0 addend)
    TX = add2(add2(add2(fma2_rn(P.R[0], X, K.NZ), fma2_rn(P.R[1], Y, K.NZ)), fma2_rn(P.R[2], Z, K.NZ)), P.R[3]);
    TY = add2(add2(add2(fma2_rn(P.R[4], X, K.NZ), fma2_rn(P.R[5], Y, K.NZ)), fma2_rn(P.R[6], Z, K.NZ)), P.R[7]);
    TZ = add2(add2(add2(fma2_rn(P.R[8], X, K.NZ), fma2_rn(P.R[9], Y, K.NZ)), fma2_rn(P.R[10], Z, K.NZ)), P.R[11]);
    // offsets from the map's min corner (cuda_sub_voxel_map.tcc:52-54)
    const f2_t OX = MIN0 ? TX : sub2(TX, K.NMX), OY = MIN0 ? TY : sub2(TY, K.NMY);
    const f2_t OZ = MIN0 ? TZ : sub2(TZ, K.NMZ);
    const f2_t AZ = and2(OZ, ABS);   // |oz|: below the map, brick 0 and a negative sub-voxel index
    // 2^23 + trunc(o), trunc(o) and s = o - trunc(o), all exact
    const f2_t MX = add2_rz(OX, K.MAG), MY = add2_rz(OY, K.MAG), MZ = add2_rz(AZ, K.MAG);
    const f2_t FY = sub2(MY, K.MAG), FZ = sub2(MZ, K.MAG);
    const f2_t SX = sub2(OX, sub2(MX, K.MAG)), SY = sub2(OY, FY), SZ = sub2(AZ, FZ);
    f2_t CX, CY, CZ;   // 1.5 2^23 + sub-voxel index q
    if (TWO) {         // trunc(fl(s * hi + fl(s * lo)))
        CX = add2_rz(fma2_rn(SX, K.INV, mul2(SX, K.INVLO)), K.MAG15);
        CY = add2_rz(fma2_rn(SY, K.INV, mul2(SY, K.INVLO)), K.MAG15);
        CZ = add2_rz(fma2_rn(SZ, K.INV, mul2(SZ, K.INVLO)), K.MAG15);
    } else {           // floor(s * inv), the product unrounded
        CX = fma2_rz(SX, K.INV, K.MAG15);
        CY = fma2_rz(SY, K.INV, K.MAG15);
        CZ = fma2_rz(SZ, K.INV, K.MAG15);
    }
    // qz takes the sign of oz; slot and brick offsets as exact float sums
    const f2_t QY = sub2(CY, K.MAG15), QZ = or2(sub2(CZ, K.MAG15), and2(OZ, SGN));
    const f2_t SLB = fma2_rn(QZ, K.SD2, fma2_rn(QY, K.SD, CX));   // 1.5 2^23 + qx + qy S + qz S^2
    const f2_t UPB = fma2_rn(FZ, K.UXY, fma2_rn(FY, K.UX, MX));   // 2^23 + mx + my Ux + mz Ux Uy
    float ox0, ox1, oy0, oy1, oz0, oz1, u0, u1, l0, l1;
    upk(OX, ox0, ox1); upk(OY, oy0, oy1); upk(OZ, oz0, oz1); upk(UPB, u0, u1); upk(SLB, l0, l1);
    k0 = fast_code<LAY>(m, occ, __float_as_uint(ox0), __float_as_uint(oy0), oz0, __float_as_uint(u0),
                        __float_as_uint(l0), v0, s0);
    k1 = fast_code<LAY>(m, occ, __float_as_uint(ox1), __float_as_uint(oy1), oz1, __float_as_uint(u1),
                        __float_as_uint(l1), v1, s1);
}

#ifndef TSDFL_TILED_THREADS
#define TSDFL_TILED_THREADS 768
#endif
constexpr int kTiledThreads = TSDFL_TILED_THREADS;
constexpr int kTiledWarps = kTiledThreads / 32;
constexpr int kRing = 64;   // deferred lookups per warp (transformed point + scan index)
constexpr uint32_t kDbgSlow = 0x10000u;   // debug code flag: decided by the exact slow tiers

// Appends the lanes with `slow` set to the warp's ring of deferred lookups.
__device__ __forceinline__ void defer(float4* ring, uint32_t head, uint32_t& tail, bool slow, float tx, float ty,
                                      float tz, int j, int lane)
{
    const unsigned mask = __ballot_sync(0xffffffffu, slow);
    if (mask == 0u) return;
    const uint32_t pos = tail + (uint32_t)__popc(mask & ((1u << lane) - 1u));
    if (slow) ring[pos & (kRing - 1)] = make_float4(tx, ty, tz, __int_as_float(j));
    tail += (uint32_t)__popc(mask);
    __syncwarp();
}

struct Partial {
    long long acc;
    uint32_t hits;
};

// Scores `count` (<= 32) deferred lookups from the ring, one per lane, through
// the exact second tier / 64-bit emulation.  The map view is read from a
// shared-memory copy so that no kernel parameter's address escapes.
__device__ __noinline__ Partial drain(const MapView* m, const LutEntry* lut, const float4* ring, uint32_t head,
                                      int count, int lane, uint32_t* dbg_row, const int32_t* perm)
{
    Partial r{0, 0u};
    if (lane < count) {
        const float4 e = ring[(head + (uint32_t)lane) & (kRing - 1)];
        const uint32_t code = slow_code(*m, e.x, e.y, e.z);
        r.acc = lut[code].v;
        r.hits = code <= (uint32_t)kCodeInit ? 1u : 0u;
        if (dbg_row) dbg_row[perm[__float_as_int(e.w)]] = code | kDbgSlow;
    }
    __syncwarp();
    return r;
}

constexpr int kTiledChunk = 1024;     // scan points per work item
constexpr int kTiledGroup = 4;        // particles per work item
constexpr int kSpreadChunk = 1024;    // scan points per work item, spread clouds
constexpr int kRegionGroups = 1024;   // particle groups per region, spread clouds

struct TiledParams {
    EvalParams e;
    int chunk;          // points per work item (multiple of 64)
    int group;          // particles per work item
    int groups;         // particle groups
    int items;          // chunks * groups
};

// Exact mode, tiled.  The pass's scan points are staged once per CTA (bulk
// copies into shared memory, pair layout); then every warp walks its share of
// the (point chunk, particle group) work items in chunk-major order -- item k
// belongs to warp k mod W of the W warps of the grid -- so all SMs score the
// same part of the scan at a time and its map footprint stays in L2, with no
// block-wide barrier after staging.  Each lane scores two points per step:
// every floating-point operation of the transform and of the index is one
// packed f32x2 instruction for both points (products as FMAs with a -0 addend,
// which round exactly like the reference's products), and the brick and
// sub-voxel offsets are formed as exact float sums whose bits are the biased
// integers, so the integer work per lookup is the rank, the address and the
// bounds.  Likelihood codes are summed in 64-bit fixed point and added to the
// particle's total with an integer atomic: exact and independent of order, so
// results equal eval_exact_kernel's bit for bit.
// One work item of the tiled scoring: the points [c0, c0 + chunk_pts) of the
// staged pass (pair layout in sxy/spz) against the particles of group grp.
// Sums go to p.sum_fx / p.hits with one integer atomic per particle.
// TWO: the sub-voxel index needs the two-term multiplier (sub_fast 1);
// DBG: per-point codes are written to the debug buffer; MIN0: the map's min
// corner is the origin, so offsets are the transformed coordinates.
// PAIRED: the step loop unrolled by two, so each warp has the gathers of two
// steps in flight (compact clouds: 2.464 -> 2.415 ms at 100k x 8,192; spread
// clouds, whose gathers go to DRAM, lose 6 % with it and keep one step).
template <int LAY, bool TWO, bool DBG, bool MIN0, bool PAIRED = false>
__device__ __forceinline__ void tiled_item(const EvalParams& p, const MapView& m, const MapView* s_map,
                                           const unsigned char* occ, const float4* sxy, const float2* spz,
                                           const LutEntry* lut, float4* ring, int n, int chunk_pts, int group,
                                           int chunk, int grp, int lane, const uint32_t* order = nullptr)
{
    const PipeConsts K = pipe_consts(m);
    uint32_t head = 0, tail = 0;
    const int c0 = chunk * chunk_pts;
    const int cn = min(chunk_pts, n - c0);
    const int b0 = c0 >> 6, nblk = (cn + 63) >> 6, nfull = cn >> 6;
    for (int k = 0; k < group; ++k) {
        const int q = grp * group + k;
        if (q >= p.P) break;
        const int pi = order ? (int)order[q] : q;   // the particle at position q
        const PosePairs R = pose_pairs(p.pose12 + 12 * (size_t)pi);
        long long acc = 0;
        uint32_t hits = 0;
        // debug rows are indexed by scan index: perm maps the pass's pair-layout
        // positions back to it
        uint32_t* dbg_row = DBG ? p.dbg + (size_t)pi * p.n_total : nullptr;
        const int32_t* perm = DBG ? p.perm + p.n0 : nullptr;
        // one step: the two points of block blk held by this lane (the
        // chunk's partial last block masks its padding points)
        auto step = [&](int blk, bool partial) {
            const float4 xy = sxy[(b0 + blk) * 32 + lane];
            const float2 zz = spz[(b0 + blk) * 32 + lane];
            uint32_t k0, k1;
            bool s0, s1;
            f2_t TX, TY, TZ;
            pair_lookup<LAY, TWO, MIN0>(m, occ, R, K, pk(xy.x, xy.y), pk(xy.z, xy.w), pk(zz.x, zz.y),
                                          !partial || 64 * blk + lane < cn, !partial || 64 * blk + 32 + lane < cn,
                                          k0, k1, s0, s1, TX, TY, TZ);
            // lanes the fast path cannot decide are deferred to the warp's ring and
            // scored 32 at a time (kCodeLater contributes nothing here), so no warp
            // diverges into the slow tiers; at most 31 entries wait between steps,
            // so each append of <= 32 fits the ring
            if (__any_sync(0xffffffffu, s0 || s1)) {
                float tx, ty, tz, u;
                upk(TX, tx, u); upk(TY, ty, u); upk(TZ, tz, u);
                defer(ring, head, tail, s0, tx, ty, tz, c0 + 64 * blk + lane, lane);
                if (tail - head >= 32) {
                    const Partial d = drain(s_map, lut, ring, head, 32, lane, dbg_row, perm);
                    acc += d.acc;
                    hits += d.hits;
                    head += 32;
                }
                upk(TX, u, tx); upk(TY, u, ty); upk(TZ, u, tz);
                defer(ring, head, tail, s1, tx, ty, tz, c0 + 64 * blk + 32 + lane, lane);
                if (tail - head >= 32) {
                    const Partial d = drain(s_map, lut, ring, head, 32, lane, dbg_row, perm);
                    acc += d.acc;
                    hits += d.hits;
                    head += 32;
                }
            }
            if (DBG) {
                const int j = c0 + 64 * blk + lane;
                if (k0 < (uint32_t)kCodeNone) dbg_row[perm[j]] = k0;
                if (k1 < (uint32_t)kCodeNone) dbg_row[perm[j + 32]] = k1;
            }
            const LutEntry e0 = lut[k0], e1 = lut[k1];
            acc += e0.v + e1.v;
            hits += (k0 <= (uint32_t)kCodeInit ? 1u : 0u) + (k1 <= (uint32_t)kCodeInit ? 1u : 0u);
        };
        if constexpr (PAIRED) {
#pragma unroll 2
            for (int blk = 0; blk < nfull; ++blk) step(blk, false);
        } else {
            for (int blk = 0; blk < nfull; ++blk) step(blk, false);
        }
        if (nfull < nblk) step(nfull, true);
        if (tail != head) {
            const Partial d = drain(s_map, lut, ring, head, (int)(tail - head), lane, dbg_row, perm);
            acc += d.acc;
            hits += d.hits;
            head = tail;
        }
        acc = warp_sum_ll(acc);
        hits = warp_sum_u32(hits);
        if (lane == 0) {
            atomicAdd(reinterpret_cast<unsigned long long*>(p.sum_fx + pi), (unsigned long long)acc);
            atomicAdd(p.hits + pi, hits);
        }
    }
}

// Shared memory of the tiled kernels: the likelihood table, the brick bitmap
// (compact layout), then the staged pass and the deferral rings.
__device__ __forceinline__ void fill_lut(LutEntry* lut, const long long* lut_fx)
{
    for (int c = threadIdx.x; c < kNumCodes; c += blockDim.x) {
        LutEntry e;
        e.v = lut_fx[c];
        lut[c] = e;
    }
}

// CLOUD: which clouds this instantiation scores -- kCloudAny either kind, on
// the staging kernel's flag (compact or spread); kCloudCompact and
// kCloudSpread return at once for the other kind, so that the two launched
// back to back score any cloud.  The compact one walks with the paired step
// loop, which costs the spread walk 3 % when both run in one kernel; each
// keeps both walks in its code, since the compiler's choices for the compact
// walk measured slower without the other one beside it.
constexpr int kCloudAny = 0, kCloudCompact = 1, kCloudSpread = 2;

template <int LAY, bool TWO, bool DBG, bool MIN0, int CLOUD>
__global__ void __launch_bounds__(kTiledThreads, 1) eval_tiled_kernel(TiledParams tp)
{
    chain_enter();
    if (CLOUD != kCloudAny && (*tp.e.sched != 0) != (CLOUD == kCloudSpread)) return;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint64_t bar;
    __shared__ MapView s_map;   // the map view the slow tiers read
    const EvalParams& p = tp.e;
    const MapView& m = p.m;
    LutEntry* lut = reinterpret_cast<LutEntry*>(smem);
    const int n = p.n1 - p.n0;
    const int npairs = ((n + 63) >> 6) * 32;
    if (threadIdx.x == 0) s_map = m;
    const uint32_t occ_bytes = LAY == kLayBitmap ? m.occ_bytes : 0u;
    unsigned char* occ = smem + kLutTableBytes;
    float4* sxy = reinterpret_cast<float4*>(occ + occ_bytes);
    float2* spz = reinterpret_cast<float2*>(sxy + npairs);
    fill_lut(lut, p.lut_fx);
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_expect_tx(&bar, (uint32_t)npairs * 24u + occ_bytes);
        bulk_g2s(sxy, p.pxy + p.n0 / 2, (uint32_t)npairs * 16u, &bar);
        bulk_g2s(spz, p.pz + p.n0 / 2, (uint32_t)npairs * 8u, &bar);
        if (occ_bytes) bulk_g2s(occ, m.occ, occ_bytes, &bar);
    }
    bool staged = mbar_wait_bounded(&bar, 0);
    if (!staged) staged = mbar_wait_bounded(&bar, 0);   // give copies in flight a second bound
    if (!staged && threadIdx.x == 0) atomicExch(p.status, TSDFL_ERR_TIMEOUT);
    if (__syncthreads_and(staged ? 1 : 0) == 0) return;

    const int lane = threadIdx.x & 31;
    float4* ring = reinterpret_cast<float4*>(spz + npairs) + (threadIdx.x >> 5) * kRing;
    const int gwarp = blockIdx.x * kTiledWarps + (threadIdx.x >> 5);
    const int nwarps = gridDim.x * kTiledWarps;
    if (*p.sched) {
        // spread cloud: the particles in spatial order, walked region by region
        // (kRegionGroups groups of neighbouring particles, all chunks, chunk-major
        // within the region), so that the grid's gathers at any time fall in one
        // part of the map
        const int chunk_pts = kSpreadChunk;
        const int chunks = (n + chunk_pts - 1) / chunk_pts, items = chunks * tp.groups;
        const int per_region = chunks * kRegionGroups;
        for (int item = gwarp; item < items; item += nwarps) {
            const int r = item / per_region, rem = item - r * per_region;
            const int g0 = r * kRegionGroups, rg = min(kRegionGroups, tp.groups - g0);
            const int chunk = rem / rg, grp = g0 + (rem - chunk * rg);
            tiled_item<LAY, TWO, DBG, MIN0>(p, m, &s_map, occ, sxy, spz, lut, ring, n, chunk_pts, tp.group, chunk,
                                            grp, lane, p.order);
        }
        return;
    }
    for (int item = gwarp; item < tp.items; item += nwarps) {
        const int chunk = item / tp.groups, grp = item - chunk * tp.groups;
        tiled_item<LAY, TWO, DBG, MIN0, CLOUD == kCloudCompact>(p, m, &s_map, occ, sxy, spz, lut, ring, n, tp.chunk,
                                                                tp.group, chunk, grp, lane);
    }
}

// Seeded per-particle scan subsampling (subsample.h): one warp per particle
// scores the particle's K kept points, two per lane per step, through the same
// packed pipeline as the tiled kernel, reading the scan from the SoA arrays the
// staging kernel wrote (scan order, L1-resident for scans of a few thousand
// points).  Per particle: the fixed-point likelihood sum, the hits and the
// number of kept points within max_range (its weight's range term), written
// directly (one warp owns the particle).
struct SubParams {
    EvalParams e;
    int K;
    unsigned long long seed;
    uint32_t* nin;
    float c_in;
};

template <bool DENSE, bool TWO, bool MIN0>
__global__ void __launch_bounds__(kTiledThreads, 1) eval_subsample_kernel(SubParams sp)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint64_t bar;
    __shared__ MapView s_map;   // the map view the slow tiers read
    const EvalParams& p = sp.e;
    const MapView& m = p.m;
    LutEntry* lut = reinterpret_cast<LutEntry*>(smem);
    const uint32_t occ_bytes = DENSE ? m.occ_bytes : 0u;
    unsigned char* occ = smem + kLutTableBytes;
    float4* rings = reinterpret_cast<float4*>(occ + occ_bytes);
    if (threadIdx.x == 0) s_map = m;
    fill_lut(lut, p.lut_fx);
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    bool staged = true;
    if (occ_bytes) {
        if (threadIdx.x == 0) {
            mbar_expect_tx(&bar, occ_bytes);
            bulk_g2s(occ, m.occ, occ_bytes, &bar);
        }
        staged = mbar_wait_bounded(&bar, 0);
        if (!staged) staged = mbar_wait_bounded(&bar, 0);   // give the copy in flight a second bound
    }
    if (!staged && threadIdx.x == 0) atomicExch(p.status, TSDFL_ERR_TIMEOUT);
    if (__syncthreads_and(staged ? 1 : 0) == 0) return;

    const int lane = threadIdx.x & 31;
    float4* ring = rings + (threadIdx.x >> 5) * kRing;
    const PipeConsts K = pipe_consts(m);
    const uint32_t N = (uint32_t)p.n_total, Ks = (uint32_t)sp.K;
    const int gwarp = blockIdx.x * kTiledWarps + (threadIdx.x >> 5);
    const int nwarps = gridDim.x * kTiledWarps;
    const bool ordered = p.sched && *p.sched;
    for (int q = gwarp; q < p.P; q += nwarps) {
        const int pi = ordered ? (int)p.order[q] : q;   // neighbouring warps take neighbouring particles
        const PosePairs R = pose_pairs(p.pose12 + 12 * (size_t)pi);
        const uint64_t st = sub_particle_state(sp.seed, (uint64_t)pi);
        long long acc = 0;
        uint32_t hits = 0, nin = 0, head = 0, tail = 0;
        for (uint32_t base = 0; base < Ks; base += 64) {   // the same trip count on every lane
            const uint32_t ka = base + (uint32_t)lane, kb = ka + 32u;
            const bool va = ka < Ks, vb = kb < Ks;
            const uint32_t ja = sub_point(st, N, Ks, va ? ka : 0u), jb = sub_point(st, N, Ks, vb ? kb : 0u);
            const float xa = __ldg(p.xs + ja), ya = __ldg(p.ys + ja), za = __ldg(p.zs + ja);
            const float xb = __ldg(p.xs + jb), yb = __ldg(p.ys + jb), zb = __ldg(p.zs + jb);
            nin += (va && __ldg(p.cs + ja) == sp.c_in ? 1u : 0u) + (vb && __ldg(p.cs + jb) == sp.c_in ? 1u : 0u);
            uint32_t k0, k1;
            bool s0, s1;
            f2_t TX, TY, TZ;
            pair_lookup<DENSE ? kLayBitmap : kLayTable, TWO, MIN0>(m, occ, R, K, pk(xa, xb), pk(ya, yb), pk(za, zb),
                                                                   va, vb, k0, k1, s0, s1, TX, TY, TZ);
            if (__any_sync(0xffffffffu, s0 || s1)) {
                float tx, ty, tz, u;
                upk(TX, tx, u); upk(TY, ty, u); upk(TZ, tz, u);
                defer(ring, head, tail, s0, tx, ty, tz, (int)ja, lane);
                if (tail - head >= 32) {
                    const Partial d = drain(&s_map, lut, ring, head, 32, lane, nullptr, nullptr);
                    acc += d.acc;
                    hits += d.hits;
                    head += 32;
                }
                upk(TX, u, tx); upk(TY, u, ty); upk(TZ, u, tz);
                defer(ring, head, tail, s1, tx, ty, tz, (int)jb, lane);
                if (tail - head >= 32) {
                    const Partial d = drain(&s_map, lut, ring, head, 32, lane, nullptr, nullptr);
                    acc += d.acc;
                    hits += d.hits;
                    head += 32;
                }
            }
            const LutEntry e0 = lut[k0], e1 = lut[k1];
            acc += e0.v + e1.v;
            hits += (k0 <= (uint32_t)kCodeInit ? 1u : 0u) + (k1 <= (uint32_t)kCodeInit ? 1u : 0u);
        }
        if (tail != head) {
            const Partial d = drain(&s_map, lut, ring, head, (int)(tail - head), lane, nullptr, nullptr);
            acc += d.acc;
            hits += d.hits;
        }
        acc = warp_sum_ll(acc);
        hits = warp_sum_u32(hits);
        nin = warp_sum_u32(nin);
        if (lane == 0) {
            p.sum_fx[pi] = acc;
            p.hits[pi] = hits;
            sp.nin[pi] = nin;
        }
    }
}

// Work items per batch of the persistent multi-filter launch: the CTA's warps
// take them one at a time from a shared counter, so uneven items even out
// before the CTA's next barrier.
constexpr int kBatchDepth = 8;
constexpr int kBatchItems = kTiledWarps * kBatchDepth;

struct BatchSeg {
    EvalParams e;
    int chunk, group, groups, items;
    int dense, two;
    uint32_t first_batch;
};

// Many filters in one persistent launch (one per map-layout kind present:
// compact or brick table, one- or two-term sub-voxel multiplier -- the same
// specialisations as eval_tiled_kernel).  The work queue is the filters'
// (filter, pass) segments one after another, each cut into batches of
// kBatchItems (point chunk, particle group) items.  A CTA takes the next batch
// with one atomic, its warps take the batch's items from a shared counter;
// when the batch belongs to another
// segment than the one staged, the CTA stages that segment (the filter's code
// LUT, its map's occupancy bitmap, the pass's scan points) before its warps
// score the items.  Per-item scoring is eval_tiled_kernel's, so every filter's
// sums equal its single-filter sums bit for bit.
template <bool DENSE, bool TWO, bool MIN0>
__global__ void __launch_bounds__(kTiledThreads, 1) eval_batch_kernel(const BatchSeg* __restrict__ segs, int nseg,
                                                                      uint32_t total_batches, uint32_t* counter,
                                                                      int32_t* status)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint64_t bar;
    __shared__ BatchSeg s_seg;
    __shared__ uint32_t s_batch;
    __shared__ uint32_t s_next;
    __shared__ int s_segi;
    LutEntry* lut = reinterpret_cast<LutEntry*>(smem);
    unsigned char* occ = smem + kLutTableBytes;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    int cur = -1;
    uint32_t phase = 0;
    float4* sxy = nullptr;
    float2* spz = nullptr;
    float4* ring = nullptr;
    int n = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            const uint32_t b = atomicAdd(counter, 1u);
            int lo = 0, hi = nseg - 1;   // last segment whose first batch is <= b
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (segs[mid].first_batch <= b) lo = mid;
                else hi = mid - 1;
            }
            s_batch = b;
            s_segi = lo;
            s_next = 0;
        }
        __syncthreads();
        const uint32_t b = s_batch;
        const int segi = s_segi;
        if (b >= total_batches) break;
        if (segi != cur) {
            if (threadIdx.x == 0) s_seg = segs[segi];
            __syncthreads();
            const EvalParams& p = s_seg.e;
            n = p.n1 - p.n0;
            const int npairs = ((n + 63) >> 6) * 32;
            const uint32_t occ_bytes = DENSE ? p.m.occ_bytes : 0u;
            sxy = reinterpret_cast<float4*>(occ + occ_bytes);
            spz = reinterpret_cast<float2*>(sxy + npairs);
            ring = reinterpret_cast<float4*>(spz + npairs) + warp * kRing;
            fill_lut(lut, p.lut_fx);
            if (threadIdx.x == 0) {
                mbar_expect_tx(&bar, (uint32_t)npairs * 24u + occ_bytes);
                bulk_g2s(sxy, p.pxy + p.n0 / 2, (uint32_t)npairs * 16u, &bar);
                bulk_g2s(spz, p.pz + p.n0 / 2, (uint32_t)npairs * 8u, &bar);
                if (occ_bytes) bulk_g2s(occ, p.m.occ, occ_bytes, &bar);
            }
            bool staged = mbar_wait_bounded(&bar, phase);
            if (!staged) staged = mbar_wait_bounded(&bar, phase);   // give copies in flight a second bound
            phase ^= 1u;
            if (!staged && threadIdx.x == 0) atomicExch(status, TSDFL_ERR_TIMEOUT);
            if (__syncthreads_and(staged ? 1 : 0) == 0) return;
            cur = segi;
        }
        const int base = (int)(b - s_seg.first_batch) * kBatchItems;
        for (;;) {
            uint32_t j = 0;
            if (lane == 0) j = atomicAdd(&s_next, 1u);
            j = __shfl_sync(0xffffffffu, j, 0);
            const int item = base + (int)j;
            if (j >= (uint32_t)kBatchItems || item >= s_seg.items) break;
            const EvalParams& p = s_seg.e;
            const int chunk = item / s_seg.groups, grp = item - chunk * s_seg.groups;
            tiled_item<DENSE ? kLayBitmap : kLayTable, TWO, false, MIN0>(p, p.m, &p.m, occ, sxy, spz, lut, ring, n,
                                                                          s_seg.chunk, s_seg.group, chunk, grp,
                                                                          lane);
        }
        __syncthreads();   // every warp is done with s_batch and the staged segment
    }
}

// Serial mode: one thread per particle runs evaluatePose's loop
// (tsdf_evaluator.cpp:38-68) in scan order with float sums, reproducing the
// reference's un-normalised weight bit for bit.
template <bool F32>
__global__ void __launch_bounds__(256) eval_serial_kernel(EvalParams p)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint64_t bar;
    float* lut = reinterpret_cast<float*>(smem);
    const int n = p.n1 - p.n0;
    const int npad = (n + 3) & ~3;
    float* xs = reinterpret_cast<float*>(smem + kLutFBytes);
    float* ys = xs + npad;
    float* zs = ys + npad;
    float* cs = zs + npad;
    for (int c = threadIdx.x; c < kNumCodes; c += blockDim.x) lut[c] = p.lut_f[c];
    for (int j = threadIdx.x; j < n; j += blockDim.x) cs[j] = p.cs[p.n0 + j];
    if (!stage_xyz(xs, ys, zs, p.xs + p.n0, p.ys + p.n0, p.zs + p.n0, npad, &bar, p.status)) return;
    int pi = blockIdx.x * blockDim.x + threadIdx.x;
    if (pi >= p.P) return;
    float t[12];
    for (int k = 0; k < 12; ++k) t[k] = p.pose12[12 * (size_t)pi + k];
    const MapView& m = p.m;
    float sum = p.first_pass ? 0.0f : p.raw[pi];
    uint32_t h = p.first_pass ? 0u : p.hits[pi];
    for (int j = 0; j < n; ++j) {
        float tx, ty, tz;
        transform_point(t, xs[j], ys[j], zs[j], tx, ty, tz);
        uint32_t idx = slot_index(m, tx, ty, tz);
        float v;
        if (F32) v = idx != kMissIndex ? m.data[idx] : m.init_value;
        else v = lut[idx != kMissIndex ? (uint32_t)m.codes[idx] : (uint32_t)kCodeInit];
        h += idx != kMissIndex ? 1u : 0u;
        if (p.dbg) p.dbg[(size_t)pi * p.n_total + p.n0 + j] = idx;
        v = __fadd_rn(__fmul_rn(p.a_hit, v), cs[j]);
        sum = __fadd_rn(sum, v);
    }
    p.raw[pi] = sum;
    p.hits[pi] = h;
}

constexpr int kNormBlocks = 256;
constexpr int kNormThreads = 256;
constexpr int kNormSums = 10;

struct NormParams {
    int P;
    int mode;            // 0 fixed point, 1 double sums, 2 serial raw
    int shift;
    double a_hit, c_in, c_out;
    int n_points;        // points every particle scored
    const uint32_t* nin; // per-particle points within max_range (subsampled scans), else null
};

// The block's sums of ten values per thread (blockDim.x == kNormThreads), in a
// fixed order: the values go to shared memory, 160 threads add sixteen each,
// ten threads add those sixteen partial sums.  Few FP64 instructions: a
// warp-shuffle tree would spend five FP64 additions a warp for every sum, and
// GB300's FP64 pipe is narrow.  Valid in threads 0..9 (out[k]).
constexpr int kNormSumsParts = 16;
static_assert(kNormSums * kNormSumsParts <= kNormThreads && kNormThreads % kNormSumsParts == 0,
              "the block's threads cover the partial sums");
__device__ __forceinline__ double block_sums10(const double (&acc)[kNormSums], double (*red)[kNormThreads],
                                               double (*red2)[kNormSumsParts])
{
    for (int k = 0; k < kNormSums; ++k) red[k][threadIdx.x] = acc[k];
    __syncthreads();
    if (threadIdx.x < kNormSums * kNormSumsParts) {
        const int k = threadIdx.x / kNormSumsParts, part = threadIdx.x % kNormSumsParts;
        double v = 0.0;
        for (int j = 0; j < kNormThreads / kNormSumsParts; ++j) v += red[k][part + kNormSumsParts * j];
        red2[k][part] = v;
    }
    __syncthreads();
    double v = 0.0;
    if (threadIdx.x < kNormSums)
        for (int j = 0; j < kNormSumsParts; ++j) v += red2[threadIdx.x][j];
    return v;
}

// Forms each particle's un-normalised weight from its likelihood sum and
// accumulates, in double and in a fixed order, the weight sum and the
// weighted pose sums of tsdf_evaluator.cpp:198-217.
__global__ void norm_partial_kernel(NormParams q, EvalBuffers b, const double* sum_f64)
{
    chain_enter();
    double acc[kNormSums];
    for (int k = 0; k < kNormSums; ++k) acc[k] = 0.0;
    const double n_in_all = (double)b.counts[0];
    const double scale = ldexp(1.0, -q.shift);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < q.P; i += gridDim.x * blockDim.x) {
        const double n_in = q.nin ? (double)q.nin[i] : n_in_all;
        const double n_out = (double)q.n_points - n_in;
        float raw;
        if (q.mode == 2) {
            raw = b.raw[i];
        } else {
            double sl = q.mode == 0 ? (double)b.sum_fx[i] * scale : sum_f64[i];
            raw = (float)(q.a_hit * sl + n_in * q.c_in + n_out * q.c_out);
            b.raw[i] = raw;
        }
        double w = (double)raw;
        const float* pp = b.particles + 7 * (size_t)i;
        const float* tg = b.trig6 + 6 * (size_t)i;
        acc[0] += w;
        acc[1] += (double)pp[0] * w;
        acc[2] += (double)pp[1] * w;
        acc[3] += (double)pp[2] * w;
        acc[4] += (double)tg[0] * w;
        acc[5] += (double)tg[1] * w;
        acc[6] += (double)tg[2] * w;
        acc[7] += (double)tg[3] * w;
        acc[8] += (double)tg[4] * w;
        acc[9] += (double)tg[5] * w;
    }
    __shared__ double red[kNormSums][kNormThreads];
    __shared__ double red2[kNormSums][kNormSumsParts];
    const double v = block_sums10(acc, red, red2);
    if (threadIdx.x < kNormSums) b.partials[blockIdx.x * kNormSums + threadIdx.x] = v;
}

// Final weight sum, the "No particle is valid!" check (tsdf_evaluator.cpp:159)
// and the mean pose with circular means of the angles (:219-221).  One block
// of kNormBlocks threads: thread t takes block t's partial sums (nb blocks ran),
// then a fixed reduction tree (so the result does not depend on timing); the
// position and the three angles are formed by four threads side by side.
__global__ void __launch_bounds__(kNormBlocks) norm_final_kernel(EvalBuffers b, float* pose_out, int nb)
{
    chain_enter();
    static_assert(kNormBlocks == kNormThreads, "one partial per thread");
    __shared__ double red[kNormSums][kNormThreads];
    __shared__ double red2[kNormSums][kNormSumsParts];
    __shared__ double s[kNormSums];
    const int t = threadIdx.x;
    double acc[kNormSums];
    for (int k = 0; k < kNormSums; ++k) acc[k] = t < nb ? b.partials[t * kNormSums + k] : 0.0;
    const double v = block_sums10(acc, red, red2);
    if (t < kNormSums) {
        s[t] = v;
        b.sums[t] = v;
    }
    __syncthreads();
    if (t >= 4) return;
    const bool degenerate = !((float)s[0] != 0.0f) || !isfinite(s[0]);
    if (t == 0) {
        b.weight_sum_f[0] = (float)s[0];
        if (degenerate) atomicExch(b.status, TSDFL_ERR_DEGENERATE);
    }
    if (degenerate || !pose_out) return;
    const double inv = 1.0 / s[0];
    if (t == 0) {
        pose_out[0] = (float)(s[1] * inv);
        pose_out[1] = (float)(s[2] * inv);
        pose_out[2] = (float)(s[3] * inv);
    } else {
        pose_out[2 + t] = (float)atan2(s[2 + 2 * t] * inv, s[3 + 2 * t] * inv);
    }
}

// particles[i].second = raw / weight_sum (tsdf_evaluator.cpp:203), skipped when
// the sum was degenerate so the caller's particles stay untouched.
// Also the last step of an evaluation: thread 0 carries its device status into
// the sticky status word (when one is given and still clear).
__device__ __forceinline__ void fold_status(const int32_t* ev, int32_t* sticky)
{
    if (sticky && blockIdx.x == 0 && threadIdx.x == 0) {
        const int v = *ev;
        if (v && *sticky == 0) *sticky = v;
    }
}

__global__ void normalize_kernel(int P, EvalBuffers b, float* particles_out, int32_t* sticky)
{
    chain_enter();
    fold_status(b.status, sticky);
    if (*b.status == TSDFL_ERR_DEGENERATE) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    particles_out[7 * (size_t)i + 6] = __fdiv_rn(b.raw[i], b.weight_sum_f[0]);
}

// Log-domain normalisation (TSDFL_NORM_LOG), after norm_partial/final have
// formed the raw weights: the largest raw weight (positive floats order like
// their bits: one atomicMax), then sum_i exp(ln raw_i - ln max) in double
// (block partials in a fixed order), LSE, and w_i = exp(ln raw_i - LSE).
__global__ void log_max_kernel(int P, EvalBuffers b)
{
    uint32_t mx = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
        const float r = b.raw[i];
        if (r > 0.0f) mx = max(mx, __float_as_uint(r));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0 && mx) atomicMax(reinterpret_cast<unsigned int*>(b.counts + 1), mx);
}

__global__ void log_sum_kernel(int P, EvalBuffers b)
{
    const double lm = log((double)__uint_as_float((uint32_t)b.counts[1]));
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
        const float r = b.raw[i];
        if (r > 0.0f) acc += exp(log((double)r) - lm);
    }
    __shared__ double red[kNormThreads / 32];
    acc = warp_sum_d(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.0;
        for (int w = 0; w < kNormThreads / 32; ++w) v += red[w];
        b.partials[blockIdx.x] = v;
    }
}

__global__ void __launch_bounds__(kNormBlocks) log_final_kernel(EvalBuffers b)
{
    __shared__ double red[kNormBlocks / 32];
    const double v = warp_sum_d(b.partials[threadIdx.x]);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < kNormBlocks / 32; ++w) s += red[w];
        b.sums[10] = log((double)__uint_as_float((uint32_t)b.counts[1])) + log(s);   // LSE
    }
}

__global__ void normalize_log_kernel(int P, EvalBuffers b, float* particles_out, int32_t* sticky)
{
    fold_status(b.status, sticky);
    if (*b.status == TSDFL_ERR_DEGENERATE) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const float r = b.raw[i];
    particles_out[7 * (size_t)i + 6] = r > 0.0f ? (float)exp(log((double)r) - b.sums[10]) : 0.0f;
}

// ---------------------------------------------------------------- resampling

constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr int kMaxSegments = 1024;
constexpr int kSumsThreads = 1024;
constexpr int kSumsItems = 4;
constexpr int kSumsChunk = kSumsThreads * kSumsItems;   // a whole number of scan tiles
static_assert(kSumsChunk % kScanTile == 0, "chunks of the double sums are made of scan tiles");
static_assert(kSumsThreads == 1024, "the double sums scan one aggregate per warp in one warp");
constexpr int kNoBinade = 0x7fffffff;

// One chunk of kSumsChunk weights in the fallback's double sums (below).
struct SumsChunk {
    unsigned long long R0;   // the chunk's increment in units 2^(b-52), for a start of even parity
    unsigned long long P;    // the sum before the chunk in those units (par set)
    int b;                   // binade of every serial sum the chunk touches, or kNoBinade
    int delta;               // increment for an odd start minus R0 (+-1 at the first tie, else 0)
    int ok;                  // no weight reaches 2^(b+1): R0 and delta hold
    int par;                 // the chunk's sums are written by resample_chunk_write_kernel
};

struct Segment {
    double u_start;   // exact float value
    double delta;     // exact float step
    long long j0;     // index of the first value
    long long n;      // number of values
};

struct ResampleWs {
    long long* cdf;         // M: inclusive fixed-point prefix within the tile
    long long* tile_sums;   // tiles
    long long* tile_off;    // tiles (exclusive)
    Segment* segs;          // kMaxSegments
    int* nseg;
    int* exact_ok;          // 1 when the parallel path reproduces the serial one
    long long* total;
    int* serial;            // 1 when only the literal loop reproduces it
    double* sums;           // M serial double prefix sums (aliases cdf; used when !exact_ok)
    const float* u0p;       // the draw in device memory (replaces u0 when set)
    double* tile_dsum;      // tiles: double sum of each scan tile's weights (any order)
    SumsChunk* chunks;      // ceil(M / kSumsChunk)
};

// Weight as an exact multiple of 2^-52 (its value in those units), or -1 when
// it is negative, not finite, not a multiple, or too large.
__device__ __forceinline__ long long weight_fx52(float w)
{
    uint32_t bits = __float_as_uint(w);
    if (bits == 0u || bits == 0x80000000u) return 0;
    if (bits >> 31) return -1;
    uint32_t e = (bits >> 23) & 0xffu;
    if (e == 0xffu) return -1;
    long long mant = e ? (long long)((bits & 0x7fffffu) | 0x800000u) : (long long)(bits & 0x7fffffu);
    int E = e ? (int)e - 150 : -149;
    int sh = E + 52;
    if (sh >= 0) {
        if (sh > 36) return -1;
        return mant << sh;
    }
    if (sh <= -63) return -1;
    if (mant & ((1ll << -sh) - 1)) return -1;
    return mant >> -sh;
}

// Tile-local inclusive scan of the fixed-point weights (exact integers).
// Also the tile's double sum of the weights for the fallback below, and
// *ws.serial for a negative or non-finite weight (only the literal loop
// reproduces those).
__global__ void resample_scan_kernel(const float* w, int stride, int M, ResampleWs ws)
{
    chain_enter();
    __shared__ long long warp_tot[kScanThreads / 32];
    __shared__ double warp_d[kScanThreads / 32];
    __shared__ int bad, wild;
    if (threadIdx.x == 0) bad = wild = 0;
    __syncthreads();
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    long long v[kScanItems];
    long long run = 0;
    double dsum = 0.0;
    for (int k = 0; k < kScanItems; ++k) {
        int i = base + k;
        long long f = 0;
        if (i < M) {
            const float x = w[(size_t)i * stride];
            f = weight_fx52(x);
            if (f < 0) { bad = 1; f = 0; }
            if (!(x >= 0.0f) || !(x < INFINITY)) wild = 1;
            else dsum += (double)x;
        }
        run += f;
        v[k] = run;
    }
    {
        const double d = warp_sum_d(dsum);
        if ((threadIdx.x & 31) == 0) warp_d[threadIdx.x >> 5] = d;
    }
    // inclusive scan of per-thread totals across the block
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    long long x = run;
    for (int o = 1; o < 32; o <<= 1) {
        long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    long long woff = 0;
    for (int k = 0; k < warp; ++k) woff += warp_tot[k];
    long long excl = woff + x - run;
    for (int k = 0; k < kScanItems; ++k) {
        int i = base + k;
        if (i < M) ws.cdf[i] = excl + v[k];
    }
    if (threadIdx.x == kScanThreads - 1) ws.tile_sums[blockIdx.x] = excl + run;
    if (threadIdx.x == 0) {
        double d = 0.0;
        for (int k = 0; k < kScanThreads / 32; ++k) d += warp_d[k];
        ws.tile_dsum[blockIdx.x] = d;
    }
    __syncthreads();
    if (threadIdx.x == 0 && bad) atomicExch(ws.exact_ok, 0);
    if (threadIdx.x == 0 && wild) atomicExch(ws.serial, 1);
}

// 2^k for -1022 <= k <= 1023, exactly.
__device__ __forceinline__ double pow2(int k)
{
    return __longlong_as_double((long long)(k + 1023) << 52);
}

// V * 2^(b-52) for V in [2^52, 2^53): the double's bits directly.
__device__ __forceinline__ double binade_value(unsigned long long V, int b)
{
    return __longlong_as_double((long long)(((unsigned long long)(b + 1023) << 52) | (V - (1ull << 52))));
}

// Builds the piecewise-arithmetic description of the reference's float draw
// sequence U_{k+1} = (float)((double)U_k + 1.0/M) (novel_resampling.h:59-63)
// for all draws below s_total: inside one binade of float the step is constant
// except near its top, where single steps are taken literally.  False when it
// cannot (a step that would depend on the parity of U, a draw that stops
// advancing, more than kMaxSegments pieces).  Scalings by powers of two only.
__device__ bool build_segments(int M, float u0, double s_total, ResampleWs ws)
{
    bool ok = true;
    const double inv_m = 1.0 / (double)M;
    // 1/M = Mi 2^(Ei - 52): the binade arithmetic below is integer work on the
    // doubles' bits (one lane walks the binades; GB300's FP64 pipe is narrow)
    const unsigned long long ib = (unsigned long long)__double_as_longlong(inv_m);
    const unsigned long long Mi = (ib & ((1ull << 52) - 1ull)) | (1ull << 52);
    const int Ei = (int)((ib >> 52) & 0x7ff) - 1023;
    const unsigned long long kHalf29 = 1ull << 28, kMask29 = (1ull << 29) - 1ull, kTop = 1ull << 53;
    double U = (double)u0;
    long long j = 0;
    int ns = 0;
    if (!(s_total >= 0.0) || !(s_total < INFINITY)) {   // no sum of non-negative finite weights
        *ws.nseg = 0;
        return false;
    }
    // the draws' and the sums' doubles are compared on their bits (a sum here
    // is >= +0, and a double >= +0 orders like its bits as a signed integer)
    const long long s_bits = __double_as_longlong(s_total);
    const long long kFltMinBits = 0x3810000000000000ll;   // 2^-126, the smallest normal float
    for (int iter = 0; __double_as_longlong(U) < s_bits; ++iter) {
        if (ns == kMaxSegments || iter > 4 * kMaxSegments) { ok = false; break; }
        bool regular = false;
        long long cnt = 0;
        int e = 0;
        unsigned long long Ui = 0, D = 0;
        double delta = 0.0;
        if (__double_as_longlong(U) >= kFltMinBits) {   // normal float: binade [2^e, 2^(e+1))
            const unsigned long long ub = (unsigned long long)__double_as_longlong(U);
            e = (int)((ub >> 52) & 0x7ff) - 1023;
            Ui = (ub & ((1ull << 52) - 1ull)) | (1ull << 52);   // U in units g = 2^(e-52)
            // Y = rint(inv_m / g): (double)U + inv_m = U + Y g while inside the binade
            const int sh = Ei - e;
            unsigned long long Y = 0, low;   // low: Y's bits below the float ulp u = 2^29 g
            bool big = false;                // Y >= 2^53: the first step leaves the binade
            if (sh >= 0) {
                low = sh >= 29 ? 0ull : (Mi & ((1ull << (29 - sh)) - 1ull)) << sh;
                if (sh >= 11) {
                    big = true;
                } else {
                    Y = Mi << sh;
                    big = Y >= kTop;
                }
            } else {
                const int n = -sh;
                if (n < 64) {   // round half to even
                    const unsigned long long q = Mi >> n, rem = Mi & ((1ull << n) - 1ull), half = 1ull << (n - 1);
                    Y = q + ((rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull);
                }
                low = Y & kMask29;
            }
            if (low == kHalf29) { ok = false; break; }   // step would depend on the parity of U
            if (!big) {
                // delta = rint(Y g / u) u = R 2^29 g
                const unsigned long long R = (Y >> 29) + (low > kHalf29 ? 1ull : 0ull);
                if (R == 0) { ok = false; break; }        // U would stop advancing
                D = R << 29;
                {   // delta = R 2^(e-23), built from its bits (R < 2^25)
                    const int lz = __clzll((long long)R);
                    delta = __longlong_as_double(((long long)(63 - lz + e - 23 + 1023) << 52) |
                                                 (long long)((R << (lz - 11)) & ((1ull << 52) - 1ull)));
                }
                // values U + i delta below top = 2^(e+1) - Y g take the regular step
                const unsigned long long T = kTop - Y;
                if (Ui < T) {
                    const unsigned long long num = (T - Ui + D - 1ull) >> 29;   // below 2^24
                    cnt = (long long)((uint32_t)num / (uint32_t)R);
                    regular = cnt > 0;
                }
            }
        }
        if (regular) {
            ws.segs[ns].u_start = U;
            ws.segs[ns].delta = delta;
            ws.segs[ns].j0 = j;
            ws.segs[ns].n = cnt;
            ++ns;
            j += cnt;
            const unsigned long long V = Ui + (unsigned long long)cnt * D;   // at most 2^53 (a float value)
            U = V >= kTop ? pow2(e + 1) : binade_value(V, e);
        } else {
            ws.segs[ns].u_start = U;
            ws.segs[ns].delta = 0.0;
            ws.segs[ns].j0 = j;
            ws.segs[ns].n = 1;
            ++ns;
            j += 1;
            double next = (double)(float)(U + inv_m);
            if (!(next > U)) { ok = false; break; }   // U stopped advancing
            U = next;
        }
    }
    *ws.nseg = ns;
    return ok;
}

// Builds the piecewise-arithmetic description of the reference's float draw
// sequence U_{k+1} = (float)((double)U_k + 1.0/M) (novel_resampling.h:59-63):
// inside one binade of float the step is constant except near its top, where
// single steps are taken literally.  One warp: the lanes form the tiles'
// prefix offsets, lane 0 walks the binades (scalings by powers of two only).
__global__ void resample_segments_kernel(int M, float u0, int tiles, ResampleWs ws)
{
    chain_enter();
    if (ws.u0p) u0 = *ws.u0p;
    const int lane = threadIdx.x & 31;
    if (threadIdx.x >= 32 || blockIdx.x != 0) return;
    const int per = (tiles + 31) / 32, t0 = min(tiles, lane * per), t1 = min(tiles, t0 + per);
    long long loc = 0;
    for (int t = t0; t < t1; ++t) loc += ws.tile_sums[t];
    long long x = loc;   // inclusive scan over the lanes (exact integers)
    for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    long long off = x - loc;
    for (int t = t0; t < t1; ++t) {
        ws.tile_off[t] = off;
        off += ws.tile_sums[t];
    }
    const long long acc = __shfl_sync(0xffffffffu, x, 31);
    if (lane != 0) return;
    *ws.total = acc;
    if (acc >= (1ll << 53)) *ws.exact_ok = 0;   // partial sums >= 2 may round in the serial double sum
    if (!*ws.exact_ok) { *ws.nseg = 0; return; }
    if (!build_segments(M, u0, ldexp((double)acc, -52), ws)) *ws.exact_ok = 0;
}

// Number of draws U_j below s (the count the serial loop has emitted once its
// running sum reaches s).
__device__ long long count_below(const Segment* seg, int ns, double s)
{
    int lo = 0, hi = ns;   // first segment with u_start >= s
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (seg[mid].u_start < s) lo = mid + 1;
        else hi = mid;
    }
    if (lo == 0) return 0;
    const Segment& g = seg[lo - 1];
    if (g.delta == 0.0) return g.j0 + 1;
    long long i = (long long)((s - g.u_start) / g.delta);
    if (i < 0) i = 0;
    while (i > 0 && g.u_start + (double)(i - 1) * g.delta >= s) --i;
    while (i < g.n && g.u_start + (double)i * g.delta < s) ++i;
    if (i > g.n) i = g.n;
    return g.j0 + i;
}

// count_below for s = c_fx 2^-52 (0 <= c_fx < 2^53), with integer operations
// only (the FP64 pipe is narrow): positive doubles order like their bits, and
// the draws of a regular segment are (A + k R) u with u = 2^(e-23) the float
// ulp of its binade, A = u_start / u, R = delta / u, so the count of those
// below s is ceil((ceil(s / u) - A) / R), clamped to [0, n].
__device__ __forceinline__ long long count_below_fx(const Segment* seg, int ns, long long c_fx)
{
    constexpr unsigned long long kM52 = (1ull << 52) - 1ull;
    long long sb = 0;   // bits of the double c_fx 2^-52 (exact)
    if (c_fx > 0) {
        const int lz = __clzll(c_fx);   // at least 11
        sb = ((long long)(63 - lz - 52 + 1023) << 52) | (long long)(((unsigned long long)c_fx << (lz - 11)) & kM52);
    }
    int lo = 0, hi = ns;   // first segment with u_start >= s
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__double_as_longlong(seg[mid].u_start) < sb) lo = mid + 1;
        else hi = mid;
    }
    if (lo == 0) return 0;
    const Segment& g = seg[lo - 1];
    const unsigned long long db = (unsigned long long)__double_as_longlong(g.delta);
    if (db == 0ull) return g.j0 + 1;
    const unsigned long long ub = (unsigned long long)__double_as_longlong(g.u_start);
    const int e = (int)((ub >> 52) & 0x7ff) - 1023, ed = (int)((db >> 52) & 0x7ff) - 1023;
    const unsigned long long A = ((ub & kM52) | (1ull << 52)) >> 29;
    const unsigned long long R = ((db & kM52) | (1ull << 52)) >> (e + 29 - ed);
    const unsigned long long L = A + (unsigned long long)g.n * R;   // the segment's end, below 2^50
    const int t = -29 - e;   // s / u = c_fx 2^t
    unsigned long long S;    // ceil(s / u), or L when it is at least L
    if (t >= 0) {
        S = (t >= 50 || ((unsigned long long)c_fx >> (63 - t)) != 0ull) ? L : (unsigned long long)c_fx << t;
        if (S > L) S = L;
    } else {
        const int n = -t;
        S = n >= 63 ? 1ull : ((unsigned long long)c_fx + (1ull << n) - 1ull) >> n;
    }
    if (S >= L) return g.j0 + g.n;
    if (S <= A) return g.j0;
    return g.j0 + (long long)((S - A + R - 1ull) / R);
}

// Particle m receives the draws in [cdf_{m-1}, cdf_m) (novel_resampling.h:52-68):
// writes their indices and, when asked, copies of the particle.
__global__ void resample_assign_kernel(const float* particles, int M, float* out, uint32_t* idx_out, long long cap,
                                       uint32_t* count_out, ResampleWs ws, int32_t* status)
{
    chain_enter();
    __shared__ Segment seg[kMaxSegments];
    if (!*ws.exact_ok) return;
    const int ns = *ws.nseg;
    for (int k = threadIdx.x; k < ns; k += blockDim.x) seg[k] = ws.segs[k];
    __syncthreads();
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    const long long c_hi_fx = ws.cdf[m] + ws.tile_off[m / kScanTile];
    long long c_lo_fx = 0;
    if (m > 0) c_lo_fx = ws.cdf[m - 1] + ws.tile_off[(m - 1) / kScanTile];
    long long lo = count_below_fx(seg, ns, c_lo_fx);
    long long hi = count_below_fx(seg, ns, c_hi_fx);
    if (m == M - 1) {
        *count_out = (uint32_t)hi;
        if (hi > cap) atomicExch(status, TSDFL_ERR_CAPACITY);
    }
    for (long long j = lo; j < hi && j < cap; ++j) {
        if (idx_out) idx_out[j] = (uint32_t)m;
        if (out) {
            const float* src = particles + 7 * (size_t)m;
            float* dst = out + 7 * (size_t)j;
            for (int k = 0; k < 7; ++k) dst[k] = src[k];
        }
    }
}

constexpr int kChainTile = 2048;
constexpr int kChainThreads = 512;

// Fallback of the parallel systematic path for weights that are not exact
// multiples of 2^-52 (tiny or huge) but non-negative and finite: the serial
// double sums s_m = s_{m-1} + w_m of the reference loop (novel_resampling.h:
// 53-56), formed in parallel.  While the sum stays in one binade [2^b, 2^(b+1))
// every result is a multiple of u = 2^(b-52), so s_k = s_{k-1} + r_k u with
// r_k = floor(w_k / u) + [frac > 1/2] -- independent of s -- except at ties
// (frac == 1/2), which round to the even multiple.  The sum after a tie is
// always even, so the parity before a tie is that of the last tie (or the
// binade's start) XOR the low bits of the increments since: a segmented XOR
// scan.  Where the exact sum leaves the binade (or a weight reaches 2^(b+1))
// one ordinary double addition is made and the scan restarts; that happens
// about once per binade.
// The weights are cut into chunks of kSumsChunk.  Approximate double sums of
// the scan tiles tell which chunks keep every serial sum they touch inside one
// binade with a margin far above the sums' rounding (all but a few: a chunk
// per binade the running sum crosses).  Such a chunk's increment depends on
// the sum before it only through that sum's parity, at the chunk's first tie,
// so it is formed for both parities by one block per chunk
// (resample_chunk_transfer_kernel); one block then chains the chunks' starts,
// walking the others weight by weight (resample_sums_kernel), after which one
// block per chunk writes the chained chunks' sums (resample_chunk_write_kernel).
// The chain verifies each transfer it applies (the start in the chunk's binade,
// the end below the binade's top), so the margin only decides speed, never the
// result.  Negative or non-finite weights set *ws.serial: only the literal loop
// reproduces them.  With s monotone, the draws each particle emits then follow
// from the draw segments in parallel (resample_fallback_assign_kernel).
// One weight in units u = 2^(b-52) of the running sum's binade [2^b, 2^(b+1)),
// from the float's bits alone (integer shifts, no FP64 operation): q =
// floor(w / u), whether the remainder is exactly half a unit (a tie) or above
// it, and whether w >= 2^(b+1).
struct FloatSplit {
    unsigned long long q;
    bool tie, above, big;
};

__device__ __forceinline__ FloatSplit split_weight(float w, int b)
{
    FloatSplit o{0ull, false, false, false};
    const uint32_t bits = __float_as_uint(w);
    int ex = (int)((bits >> 23) & 0xffu);
    unsigned long long man = bits & 0x7fffffu;
    if (man == 0ull && ex == 0) return o;   // +0
    if (ex) man |= 0x800000ull;
    else ex = 1;                            // subnormal: man * 2^-149
    // w = man * 2^(ex - 150); big: w >= 2^(b+1)
    if (man >= 0x800000ull) {
        o.big = ex - 127 >= b + 1;
    } else {
        const int k = b + 1 + 149;          // man >= 2^k
        o.big = k <= 0 ? true : (k >= 23 ? false : man >= (1ull << k));
    }
    if (o.big) return o;
    const int sh = ex - 150 + 52 - b;       // w / u = man * 2^sh
    if (sh >= 0) {
        o.q = man << sh;                    // below 2^53: w < 2^(b+1)
    } else {
        const int n = -sh;
        if (n >= 64) return o;              // far below half a unit
        o.q = n >= 32 ? 0ull : man >> n;
        const unsigned long long rem = n >= 32 ? man : man & ((1ull << n) - 1ull);
        const unsigned long long half = 1ull << (n - 1);
        o.tie = rem == half;
        o.above = rem > half;
    }
    return o;
}


// The binade of a positive normal double, and its value in units 2^(b-52).
__device__ __forceinline__ int binade_of(double s)
{
    return (int)((__double_as_longlong(s) >> 52) & 0x7ff) - 1023;
}
__device__ __forceinline__ unsigned long long binade_units(double s)
{
    return ((unsigned long long)__double_as_longlong(s) & ((1ull << 52) - 1ull)) | (1ull << 52);
}

struct ParityPrefix {   // segmented XOR: the parity state after a run of items
    uint32_t reset;     // a tie occurred in the run: the parity restarted at 0 there
    uint32_t x;         // XOR of the increments' low bits since the start or the last tie
};

__device__ __forceinline__ ParityPrefix parity_combine(ParityPrefix a, ParityPrefix b)
{
    return b.reset ? b : ParityPrefix{a.reset, a.x ^ b.x};
}

// The increments of the staged weights sw[pos, t) in units 2^(b-52) for a
// running sum of parity p0 before item pos.  Thread k of the block's
// kSumsThreads takes items pos + kSumsItems k + j; incl[j] is the sum of the
// increments up to and including its item j.  Increments of weights that
// reach 2^(b+1) are 0 (big set); increments are clamped at 2^53 (where the
// sum leaves the binade anyway).  The block's threads all call it; red_par and
// red_sum are read after the call returns, so the caller synchronises before
// calling again.
struct BinadeRun {
    unsigned long long q[kSumsItems], r[kSumsItems], incl[kSumsItems];
    bool tie[kSumsItems], big[kSumsItems], valid[kSumsItems];
};

__device__ __forceinline__ void binade_increments(const float* sw, int pos, int t, int b, uint32_t p0, BinadeRun& x,
                                                  ParityPrefix* red_par, unsigned long long* red_sum)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned long long LIM = 1ull << 53;
    ParityPrefix agg{0u, 0u};
    for (int j = 0; j < kSumsItems; ++j) {
        const int i = pos + kSumsItems * tid + j;
        x.valid[j] = i < t;
        x.q[j] = 0;
        x.r[j] = 0;
        x.tie[j] = false;
        x.big[j] = false;
        if (x.valid[j]) {
            const FloatSplit f = split_weight(sw[i], b);
            x.big[j] = f.big;
            if (!f.big) {
                x.q[j] = f.q;
                x.tie[j] = f.tie;
                x.r[j] = f.q + (f.above ? 1ull : 0ull);
            }
        }
        agg = parity_combine(agg, x.tie[j] ? ParityPrefix{1u, 0u} : ParityPrefix{0u, (uint32_t)(x.r[j] & 1)});
    }
    // exclusive segmented-XOR scan of the threads' aggregates
    ParityPrefix px = agg;
    for (int o = 1; o < 32; o <<= 1) {
        ParityPrefix y{__shfl_up_sync(0xffffffffu, px.reset, o), __shfl_up_sync(0xffffffffu, px.x, o)};
        if (lane >= o) px = parity_combine(y, px);
    }
    if (lane == 31) red_par[warp] = px;
    __syncthreads();
    // the warps' aggregates before this warp: every warp scans the 32 of them
    ParityPrefix wx = red_par[lane];
    for (int o = 1; o < 32; o <<= 1) {
        ParityPrefix y{__shfl_up_sync(0xffffffffu, wx.reset, o), __shfl_up_sync(0xffffffffu, wx.x, o)};
        if (lane >= o) wx = parity_combine(y, wx);
    }
    ParityPrefix before{__shfl_sync(0xffffffffu, wx.reset, (warp + 31) & 31),
                        __shfl_sync(0xffffffffu, wx.x, (warp + 31) & 31)};
    if (warp == 0) before = ParityPrefix{0u, 0u};
    {
        ParityPrefix y{__shfl_up_sync(0xffffffffu, px.reset, 1), __shfl_up_sync(0xffffffffu, px.x, 1)};
        if (lane > 0) before = parity_combine(before, y);
    }
    uint32_t par = before.reset ? before.x : (p0 & 1u) ^ before.x;   // parity before the first item
    unsigned long long tsum = 0;
    for (int j = 0; j < kSumsItems; ++j) {
        if (x.tie[j]) {   // round half to even: +1 when the sum before plus q is odd
            x.r[j] = x.q[j] + ((par ^ (uint32_t)(x.q[j] & 1)) & 1u);
            par = 0u;
        } else {
            par ^= (uint32_t)(x.r[j] & 1);
        }
        if (x.r[j] > LIM) x.r[j] = LIM;
        tsum += x.r[j];
    }
    // exclusive sum scan of the threads' increments
    unsigned long long xs = tsum;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, xs, o);
        if (lane >= o) xs += y;
    }
    if (lane == 31) red_sum[warp] = xs;
    __syncthreads();
    unsigned long long ws_ = red_sum[lane];
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, ws_, o);
        if (lane >= o) ws_ += y;
    }
    const unsigned long long wbefore = __shfl_sync(0xffffffffu, ws_, (warp + 31) & 31);
    unsigned long long run = xs - tsum + (warp ? wbefore : 0ull);
    for (int j = 0; j < kSumsItems; ++j) {
        run += x.r[j];
        x.incl[j] = run;
    }
}

__device__ __forceinline__ double block_sum_d(double v, double* red)
{
    v = warp_sum_d(v);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
    __syncthreads();
    return t;
}

// Stages chunk c's weights in shared memory; returns its length.
__device__ __forceinline__ int stage_chunk(const float* __restrict__ w, int stride, int M, int c, float* sw)
{
    const int c0 = c * kSumsChunk, t = min(kSumsChunk, M - c0);
    for (int i = threadIdx.x; i < t; i += blockDim.x) sw[i] = w[(size_t)(c0 + i) * stride];
    return t;
}

// One block per chunk: the chunk's binade (the serial sums' bounds from the
// tiles' double sums, widened by far more than their rounding), and for a
// chunk inside one binade its increment R0 from an even start and the change
// delta for an odd one.
__global__ void __launch_bounds__(kSumsThreads) resample_chunk_transfer_kernel(const float* __restrict__ w,
                                                                               int stride, int M, ResampleWs ws)
{
    chain_enter();
    __shared__ float sw[kSumsChunk];
    __shared__ unsigned long long red_sum[kSumsThreads / 32];
    __shared__ ParityPrefix red_par[kSumsThreads / 32];
    __shared__ double red_d[kSumsThreads / 32];
    __shared__ int s_b, s_first, s_big;
    if (*ws.exact_ok || *ws.serial) return;
    const int c = blockIdx.x, tid = threadIdx.x;
    constexpr int kTilesPerChunk = kSumsChunk / kScanTile;
    const int tiles = (M + kScanTile - 1) / kScanTile;
    const int t0 = c * kTilesPerChunk, t1 = min(t0 + kTilesPerChunk, tiles);
    double a = 0.0, e = 0.0;
    for (int i = tid; i < t0; i += kSumsThreads) a += ws.tile_dsum[i];
    for (int i = t0 + tid; i < t1; i += kSumsThreads) e += ws.tile_dsum[i];
    a = block_sum_d(a, red_d);
    e = block_sum_d(e, red_d);
    if (tid == 0) {
        // |serial - approximate| <= (M + tiles + 2 kScanTile) 2^-53 relative: widen by 4x that
        const double eps = ((double)M + (double)tiles + 2.0 * kScanTile) * 0x1p-51;
        const double lo = a * (1.0 - eps), hi = (a + e) * (1.0 + eps);
        int b = kNoBinade;
        if (a > 0.0 && lo > 0.0 && binade_of(lo) == binade_of(hi)) b = binade_of(lo);
        s_b = b;
        s_first = kSumsChunk;
        s_big = 0;
        SumsChunk& k = ws.chunks[c];
        k.b = b;
        k.ok = 0;
        k.par = 0;
        k.delta = 0;
        k.R0 = 0;
        k.P = 0;
    }
    __syncthreads();
    const int b = s_b;
    if (b == kNoBinade) return;
    const int t = stage_chunk(w, stride, M, c, sw);
    __syncthreads();
    BinadeRun x;
    binade_increments(sw, 0, t, b, 0u, x, red_par, red_sum);
    bool big = false;
    for (int j = 0; j < kSumsItems; ++j) {
        big |= x.big[j];
        if (x.tie[j]) atomicMin(&s_first, kSumsItems * tid + j);
    }
    if (big) s_big = 1;
    __syncthreads();
    SumsChunk& k = ws.chunks[c];
    for (int j = 0; j < kSumsItems; ++j)   // r(odd start) - r(even start) at the first tie
        if (kSumsItems * tid + j == s_first) k.delta = x.r[j] == x.q[j] ? 1 : -1;
    if (tid == kSumsThreads - 1) {
        k.R0 = x.incl[kSumsItems - 1];
        k.ok = s_big ? 0 : 1;
    }
}

__device__ void systematic_chain_block(const float* __restrict__ w, int stride, int M, float u0,
                                       uint32_t* __restrict__ cnt, uint32_t* __restrict__ off,
                                       unsigned long long* total, int* err);

// The chain: one block walks the chunks in order, applying the transfers of
// chunks inside one binade (thread 0, checked) and forming the others' sums
// weight by weight; then thread 0 describes the draws below the total as
// segments.  Where only the literal loop reproduces the reference (*ws.serial:
// set by the scan for negative or non-finite weights, or here when the draws
// cannot be described), the block walks that instead.
__device__ void serial_sums_block(const float* __restrict__ w, int stride, int M, float u0, ResampleWs ws)
{
    __shared__ float sw[kSumsChunk];
    __shared__ unsigned long long red_sum[kSumsThreads / 32];
    __shared__ ParityPrefix red_par[kSumsThreads / 32];
    __shared__ double s_s, s_prev;
    __shared__ int s_pos, s_e, s_c;
    const int tid = threadIdx.x;
    const int chunks = (M + kSumsChunk - 1) / kSumsChunk;
    const unsigned long long LIM = 1ull << 53;
    if (tid == 0) {
        s_s = 0.0;
        s_c = 0;
    }
    __syncthreads();
    for (;;) {
        if (tid == 0) {   // chunks inside one binade: only their starts
            int c = s_c;
            double sum = s_s;
            for (; c < chunks; ++c) {
                SumsChunk& k = ws.chunks[c];
                if (k.b == kNoBinade || !k.ok || !(sum > 0.0) || binade_of(sum) != k.b) break;
                const unsigned long long P = binade_units(sum);
                const unsigned long long E = P + k.R0 + ((P & 1ull) ? (unsigned long long)(long long)k.delta : 0ull);
                if (E >= LIM) break;
                k.P = P;
                k.par = 1;
                sum = binade_value(E, k.b);
            }
            s_c = c;
            s_s = sum;
        }
        __syncthreads();
        const int c = s_c;
        if (c >= chunks) break;
        const int c0 = c * kSumsChunk;
        const int t = stage_chunk(w, stride, M, c, sw);
        if (tid == 0) s_pos = 0;
        __syncthreads();
        for (int guard = 0; guard <= kSumsChunk; ++guard) {   // one pass per event: at most t + 1
            const int pos = s_pos;
            if (pos >= t) break;
            const double s = s_s;
            if (tid == 0) s_e = t;
            __syncthreads();
            if (s == 0.0) {   // leading zero weights keep the sum 0; the first positive one is the sum
                for (int i = pos + tid; i < t; i += kSumsThreads)
                    if (sw[i] > 0.0f) atomicMin(&s_e, i);
                __syncthreads();
                const int z = s_e;
                for (int i = pos + tid; i < z; i += kSumsThreads) ws.sums[c0 + i] = 0.0;
                if (tid == 0) {
                    if (z < t) {
                        s_s = (double)sw[z];
                        ws.sums[c0 + z] = s_s;
                    }
                    s_pos = z < t ? z + 1 : t;
                }
                __syncthreads();
                continue;
            }
            const int b = binade_of(s);   // s in [2^b, 2^(b+1))
            const unsigned long long P0 = binade_units(s);
            BinadeRun x;
            binade_increments(sw, pos, t, b, (uint32_t)(P0 & 1ull), x, red_par, red_sum);
            for (int j = 0; j < kSumsItems; ++j) {
                const int i = pos + kSumsItems * tid + j;
                const unsigned long long before = x.incl[j] - x.r[j];
                if (x.valid[j] && (x.big[j] || P0 + before + x.q[j] >= LIM)) atomicMin(&s_e, i);   // leaves the binade
            }
            __syncthreads();
            const int e = s_e;
            for (int j = 0; j < kSumsItems; ++j) {   // below e every sum stays in the binade
                const int i = pos + kSumsItems * tid + j;
                if (i < e) ws.sums[c0 + i] = binade_value(P0 + x.incl[j], b);
                if (i == e - 1) s_prev = binade_value(P0 + x.incl[j], b);
            }
            __syncthreads();
            if (tid == 0) {
                const double prev = e > pos ? s_prev : s;
                if (e < t) {
                    const double nx = prev + (double)sw[e];   // one ordinary double addition
                    ws.sums[c0 + e] = nx;
                    s_s = nx;
                    s_pos = e + 1;
                } else {
                    s_s = prev;
                    s_pos = t;
                }
            }
            __syncthreads();
        }
        if (tid == 0) s_c = c + 1;
        __syncthreads();
    }
    if (tid == 0 && !build_segments(M, u0, s_s, ws)) *ws.serial = 1;   // s_s: the total
    __syncthreads();
}

__global__ void __launch_bounds__(kSumsThreads) resample_sums_kernel(const float* __restrict__ w, int stride, int M,
                                                                     float u0, ResampleWs ws, uint32_t* cnt,
                                                                     uint32_t* off, unsigned long long* total,
                                                                     int* err)
{
    chain_enter();
    if (*ws.exact_ok) return;
    if (ws.u0p) u0 = *ws.u0p;
    if (!*ws.serial) serial_sums_block(w, stride, M, u0, ws);
    if (*ws.serial) systematic_chain_block(w, stride, M, u0, cnt, off, total, err);
}

// One block per chained chunk: its sums from the start the chain gave it.
__global__ void __launch_bounds__(kSumsThreads) resample_chunk_write_kernel(const float* __restrict__ w, int stride,
                                                                            int M, ResampleWs ws)
{
    chain_enter();
    __shared__ float sw[kSumsChunk];
    __shared__ unsigned long long red_sum[kSumsThreads / 32];
    __shared__ ParityPrefix red_par[kSumsThreads / 32];
    if (*ws.exact_ok || *ws.serial) return;
    const int c = blockIdx.x;
    const SumsChunk k = ws.chunks[c];
    if (!k.par) return;
    const int t = stage_chunk(w, stride, M, c, sw);
    __syncthreads();
    BinadeRun x;
    binade_increments(sw, 0, t, k.b, (uint32_t)(k.P & 1ull), x, red_par, red_sum);
    const int c0 = c * kSumsChunk;
    for (int j = 0; j < kSumsItems; ++j) {
        const int i = kSumsItems * threadIdx.x + j;
        if (x.valid[j]) ws.sums[c0 + i] = binade_value(k.P + x.incl[j], k.b);
    }
}

__device__ void scatter_block(const float* particles, int M, const uint32_t* cnt, const uint32_t* off,
                              const unsigned long long* total, const int* err, float* out, uint32_t* idx_out,
                              long long cap, uint32_t* count_out, int32_t* status);

// The fallbacks' assignment: from the literal loop's counts and offsets
// (*ws.serial), else particle m receives the draws in [s_{m-1}, s_m) of the
// serial double sums.
__global__ void resample_fallback_assign_kernel(const float* particles, int M, float* out, uint32_t* idx_out,
                                                long long cap, uint32_t* count_out, ResampleWs ws, int32_t* status,
                                                const uint32_t* cnt, const uint32_t* off,
                                                const unsigned long long* total, const int* err)
{
    chain_enter();
    __shared__ Segment seg[kMaxSegments];
    if (*ws.exact_ok) return;
    if (*ws.serial) {
        scatter_block(particles, M, cnt, off, total, err, out, idx_out, cap, count_out, status);
        return;
    }
    const int ns = *ws.nseg;
    for (int k = threadIdx.x; k < ns; k += blockDim.x) seg[k] = ws.segs[k];
    __syncthreads();
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    const long long lo = m > 0 ? count_below(seg, ns, ws.sums[m - 1]) : 0;
    const long long hi = count_below(seg, ns, ws.sums[m]);
    if (m == M - 1) {
        *count_out = (uint32_t)hi;
        if (hi > cap) atomicExch(status, TSDFL_ERR_CAPACITY);
    }
    for (long long j = lo; j < hi && j < cap; ++j) {
        if (idx_out) idx_out[j] = (uint32_t)m;
        if (out) {
            const float* src = particles + 7 * (size_t)m;
            float* dst = out + 7 * (size_t)j;
            for (int k = 0; k < 7; ++k) dst[k] = src[k];
        }
    }
}

__global__ void set_flags_kernel(int* exact_ok, int* serial, int* err)
{
    chain_enter();
    *exact_ok = 1;
    *serial = 0;
    *err = 0;
}

// SystematicResampler's loop (novel_resampling.h:41-72) literally, for the
// weights the parallel path cannot reproduce exactly (negative, tiny or huge):
// one thread walks it over tiles of weights the block stages in shared memory,
// writing every particle's count and exclusive offset; the copies are made in
// parallel afterwards.  A draw that stops advancing or a count beyond 4M + 16
// (the reference would never finish) stops the walk and sets *err.  Run by
// resample_sums_kernel's block when *ws.serial is set (neither parallel form
// applies).
__device__ void systematic_chain_block(const float* __restrict__ w, int stride, int M, float u0,
                                       uint32_t* __restrict__ cnt, uint32_t* __restrict__ off,
                                       unsigned long long* total, int* err)
{
    __shared__ float sw[kChainTile];
    __shared__ uint32_t sc[kChainTile], so[kChainTile];
    __shared__ int s_stop;
    const double inv_m = 1.0 / (double)M;
    float u = u0;
    double s = 0.0;
    unsigned long long n = 0;
    if (threadIdx.x == 0) s_stop = 0;
    for (int base = 0; base < M; base += kChainTile) {
        const int t = min(kChainTile, M - base);
        for (int i = threadIdx.x; i < t; i += blockDim.x) sw[i] = w[(size_t)(base + i) * stride];
        __syncthreads();
        if (threadIdx.x == 0) {
            bool stop = false;   // kept in a register: the loop reads no shared flag
#pragma unroll 4
            for (int i = 0; i < t; ++i) {
                uint32_t k = 0;
                s += (double)sw[i];
                while (s > (double)u) {
                    ++k;
                    const float next = (float)((double)u + inv_m);
                    if (next == u || n + k > 4ull * (unsigned long long)M + 16ull) {   // would never finish
                        stop = true;
                        break;
                    }
                    u = next;
                }
                sc[i] = k;
                so[i] = (uint32_t)n;
                n += k;
                if (n >= (1ull << 31)) stop = true;   // offsets stay 32-bit
                if (stop) break;
            }
            *total = n;
            s_stop = stop ? 1 : 0;
        }
        __syncthreads();
        if (s_stop) {
            if (threadIdx.x == 0) *err = 1;
            return;
        }
        for (int i = threadIdx.x; i < t; i += blockDim.x) {
            cnt[base + i] = sc[i];
            off[base + i] = so[i];
        }
        __syncthreads();
    }
}

// ResidualSystematicResampler::resample (novel_resampling.h:76-104) for
// weights w >= 0 with (float)M * w < 2^22 - 1 (others stop it with *err): one
// thread walks the draw chain -- temp = (float)M w - u; o = floor(temp) + 1,
// the reference's (size_t)(temp + 1.0); u = (float)o - temp -- over tiles of
// (float)M w staged in shared memory, four dependent float additions a
// particle and nothing else; the block then turns the counts into offsets with
// a scan.
__global__ void __launch_bounds__(kChainThreads) residual_chain_kernel(const float* __restrict__ w, int stride,
                                                                       int M, float u0, uint32_t* __restrict__ cnt,
                                                                       uint32_t* __restrict__ off,
                                                                       unsigned long long* total, int* err)
{
    static_assert(kChainTile == 4 * kChainThreads, "four counts per thread in the scan");
    __shared__ float sc[kChainTile];   // (float)M * w, then the counts
    __shared__ uint32_t warp_tot[kChainThreads / 32];
    __shared__ uint32_t s_base;
    const float Mf = (float)M;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float u = u0;
    if (threadIdx.x == 0) s_base = 0u;
    for (int base = 0; base < M; base += kChainTile) {
        const int t = min(kChainTile, M - base);
        bool bad = false;
        for (int i = threadIdx.x; i < t; i += blockDim.x) {
            const float x = w[(size_t)(base + i) * stride];
            const float c = __fmul_rn(Mf, x);
            bad |= !(x >= 0.0f) || !(c < 4194303.0f);
            sc[i] = c;
        }
        if (__syncthreads_or(bad ? 1 : 0)) {
            if (threadIdx.x == 0) {
                *err = 1;
                *total = s_base;
            }
            return;
        }
        if (threadIdx.x == 0) {
            // 32 products to registers at a time, so that only the chain is serial
            int i = 0;
            for (; i + 32 <= t; i += 32) {
                float v[32];
#pragma unroll
                for (int k = 0; k < 32; ++k) v[k] = sc[i + k];
#pragma unroll
                for (int k = 0; k < 32; ++k) {
                    const float temp = __fsub_rn(v[k], u);
                    // floor(temp) + 1 for -1 <= temp < 2^22: rounding temp + 1.5 * 2^23 down
                    // lands on an integer (unit spacing there), so both steps are exact
                    const float of = __fsub_rn(__fadd_rd(temp, 12582912.0f), 12582911.0f);
                    u = __fsub_rn(of, temp);
                    v[k] = of;
                }
#pragma unroll
                for (int k = 0; k < 32; ++k) sc[i + k] = v[k];
            }
            for (; i < t; ++i) {
                const float temp = __fsub_rn(sc[i], u);
                const float of = __fsub_rn(__fadd_rd(temp, 12582912.0f), 12582911.0f);
                u = __fsub_rn(of, temp);
                sc[i] = of;
            }
        }
        __syncthreads();
        // exclusive offsets of this tile's counts, four per thread
        uint32_t v[4], run = 0;
        for (int k = 0; k < 4; ++k) {
            const int i = 4 * threadIdx.x + k;
            v[k] = i < t ? (uint32_t)sc[i] : 0u;
            run += v[k];
        }
        uint32_t x = run;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[warp] = x;
        __syncthreads();
        uint32_t woff = 0, tile_total = 0;
        for (int k = 0; k < kChainThreads / 32; ++k) {
            if (k < warp) woff += warp_tot[k];
            tile_total += warp_tot[k];
        }
        uint32_t o = s_base + woff + x - run;
        for (int k = 0; k < 4; ++k) {
            const int i = 4 * threadIdx.x + k;
            if (i < t) {
                cnt[base + i] = v[k];
                off[base + i] = o;
            }
            o += v[k];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            s_base += tile_total;
            if (s_base >= (1u << 31)) *err = 1;   // offsets stay 32-bit
        }
        __syncthreads();
        if (*err) {
            if (threadIdx.x == 0) *total = s_base;
            return;
        }
    }
    if (threadIdx.x == 0) *total = s_base;
}

// Copies particle m (7 floats) to its cnt[m] output slots below cap, or writes
// its index there; thread 0 reports the count (and the chain's failure).
__device__ void scatter_block(const float* particles, int M, const uint32_t* cnt, const uint32_t* off,
                              const unsigned long long* total, const int* err, float* out, uint32_t* idx_out,
                              long long cap, uint32_t* count_out, int32_t* status)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (*err) {
        if (m == 0) {
            *count_out = (uint32_t)*total;
            atomicExch(status, TSDFL_ERR_UNSUPPORTED);
        }
        return;
    }
    if (m == 0) {
        *count_out = (uint32_t)*total;
        if ((long long)*total > cap) atomicExch(status, TSDFL_ERR_CAPACITY);
    }
    if (m >= M) return;
    const long long o = off[m];
    for (long long j = o; j < o + (long long)cnt[m] && j < cap; ++j) {
        if (idx_out) idx_out[j] = (uint32_t)m;
        if (out) {
            const float* src = particles + 7 * (size_t)m;
            float* dst = out + 7 * (size_t)j;
            for (int k = 0; k < 7; ++k) dst[k] = src[k];
        }
    }
}

__global__ void resample_scatter_kernel(const float* particles, int M, const uint32_t* cnt, const uint32_t* off,
                                        const unsigned long long* total, const int* err, float* out,
                                        uint32_t* idx_out, long long cap, uint32_t* count_out, int32_t* status)
{
    scatter_block(particles, M, cnt, off, total, err, out, idx_out, cap, count_out, status);
}

__global__ void set_int_kernel(int* p, int v) { *p = v; }

// Best particle of mcl_3d.cpp:382-394: the first index with the largest weight
// above 0 (strict comparison from max_value = 0).  Keys (weight bits, ~index)
// order positive floats by value and equal weights by the lower index.
__global__ void best_particle_kernel(const float* particles, int M, unsigned long long* key)
{
    unsigned long long best = 0ull;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
        const float w = particles[7 * (size_t)i + 6];
        if (w > 0.0f) {
            const unsigned long long k = ((unsigned long long)__float_as_uint(w) << 32) | (0xffffffffu - (uint32_t)i);
            best = k > best ? k : best;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long y = __shfl_xor_sync(0xffffffffu, best, o);
        best = y > best ? y : best;
    }
    if ((threadIdx.x & 31) == 0 && best) atomicMax(key, best);
}

__global__ void best_index_kernel(const unsigned long long* key, uint32_t* index_out)
{
    const unsigned long long k = *key;
    *index_out = k ? 0xffffffffu - (uint32_t)(k & 0xffffffffu) : 0xffffffffu;
}

// ------------------------------------------------------------- map layouts

__global__ void halves_kernel(const uint16_t* codes, const float* values, const float* data, size_t n,
                              uint16_t* h16)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float v = codes ? values[codes[i]] : data[i];
        h16[i] = __half_as_ushort(__float2half_rn(v));
    }
}

// Grid layout: output brick j of the bounding box order with skirts -- for
// j < 2 up_dim_2 brick j / 2 of the lowest layer (odd j) behind its skirt (even
// j), beyond that brick j - up_dim_2 -- copied from the code array, whose
// leading miss brick is what the skirt of the first allocated brick reads.
__global__ void grid_fill_kernel(const uint16_t* codes, const int32_t* grid_occ, uint64_t uxy, uint64_t s3,
                                 uint64_t n, uint16_t* grid)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t j = i / s3, t = i - j * s3;
        const bool low = j < 2 * uxy;
        const uint64_t up = low ? j >> 1 : j - uxy;
        const bool skirt = low && (j & 1) == 0;
        const int32_t base = grid_occ[up];
        grid[i] = base < 0 ? (uint16_t)kCodeMiss : codes[(int64_t)base + (int64_t)t - (skirt ? (int64_t)s3 : 0)];
    }
}

__global__ void codes_from_floats_kernel(const float* data, size_t n, const float* values, float init_value,
                                         uint16_t* codes, int32_t* fail)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float v = data[i];
        uint32_t vb = __float_as_uint(v);
        int code = -1;
        if (vb == __float_as_uint(init_value)) {
            code = kCodeInit;
        } else {
            // likelihood values decrease with |tsdf|: binary search, then exact match
            int lo = 0, hi = kCodeInit - 1;
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (values[mid] > v) lo = mid + 1;
                else hi = mid;
            }
            for (int c = max(0, lo - 2); c <= min(kCodeInit - 1, lo + 2); ++c)
                if (__float_as_uint(values[c]) == vb) { code = c; break; }
        }
        if (code < 0) {
            atomicExch(fail, 1);
            code = kCodeInit;
        }
        codes[i] = (uint16_t)code;
    }
}


int check(cudaError_t e)
{
    return e == cudaSuccess ? TSDFL_OK : TSDFL_ERR_DEVICE;
}

}  // namespace

// ------------------------------------------------------------------ launchers

// Launches a kernel of the update / resampling chain with programmatic
// dependent launch (the kernel opens with chain_enter()), so its launch
// overlaps the end of the previous kernel instead of following it.
template <typename... Params, typename... Args>
void launch_chained(void (*kernel)(Params...), unsigned grid, unsigned block, size_t smem, cudaStream_t s,
                    Args... args)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, args...);
}

int launch_pose_prepare(const float* tf, const float* particles, int P, const float* points, int N, int npad,
                        float max_range_sq, float c_in, float c_out, const float* code_values, int shift,
                        const EvalBuffers& b, cudaStream_t s)
{
    Tf16 t;
    for (int k = 0; k < 16; ++k) t.v[k] = tf[k];
    PointParams p{points, N, npad, 32 * ((N + 63) / 64), particles, P, max_range_sq, c_in, c_out, code_values,
                  shift};
    launch_chained(pose_prepare_kernel, (unsigned)(1 + pose_blocks((size_t)(P > 0 ? P : 0))), kPoseThreads, 0, s,
                   t, p, b);
    g_launches += 1;
    return check(cudaGetLastError());
}

int launch_particle_order(const float* particles, int P, const EvalBuffers& b, cudaStream_t s)
{
    if (P <= 0) return TSDFL_OK;
    // the cell histogram was cleared by pose_prepare_kernel
    const unsigned blocks = (unsigned)std::min((P + 255) / 256, 4096);
    launch_chained(particle_cells_kernel, blocks, 256, 0, s, particles, P, b);
    launch_chained(particle_scan_kernel, 1, kCellScanThreads, 0, s, b);
    launch_chained(particle_scatter_kernel, blocks, 256, 0, s, P, b);
    g_launches += 3;
    return check(cudaGetLastError());
}

size_t eval_smem_bytes(bool serial, int n)
{
    int npad = (n + 3) & ~3;
    return serial ? (size_t)kLutFBytes + 4ull * npad * 4 : (size_t)kLutBytes + 3ull * npad * 4;
}

using TiledKernel = void (*)(TiledParams);

// The debug instantiation decides the cloud at run time; the production ones
// come in a compact and a spread kind (cloud 1 / 2).
template <int LAY, bool TWO>
TiledKernel pick_tiled_2(bool dbg, bool min0, int cloud)
{
    if (dbg) return min0 ? eval_tiled_kernel<LAY, TWO, true, true, kCloudAny>
                         : eval_tiled_kernel<LAY, TWO, true, false, kCloudAny>;
    if (cloud == kCloudSpread)
        return min0 ? eval_tiled_kernel<LAY, TWO, false, true, kCloudSpread>
                    : eval_tiled_kernel<LAY, TWO, false, false, kCloudSpread>;
    return min0 ? eval_tiled_kernel<LAY, TWO, false, true, kCloudCompact>
                : eval_tiled_kernel<LAY, TWO, false, false, kCloudCompact>;
}

template <int LAY>
TiledKernel pick_tiled_1(bool two, bool dbg, bool min0, int cloud)
{
    return two ? pick_tiled_2<LAY, true>(dbg, min0, cloud) : pick_tiled_2<LAY, false>(dbg, min0, cloud);
}

TiledKernel pick_tiled(int lay, bool two, bool dbg, bool min0, int cloud)
{
    switch (lay) {
    case kLayBitmap: return pick_tiled_1<kLayBitmap>(two, dbg, min0, cloud);
    case kLayHash: return pick_tiled_1<kLayHash>(two, dbg, min0, cloud);
    case kLayGrid: return pick_tiled_1<kLayGrid>(two, dbg, min0, cloud);
    default: return pick_tiled_1<kLayTable>(two, dbg, min0, cloud);
    }
}

size_t tiled_smem_bytes(const MapView& m, bool dense, int n)
{
    return (size_t)kLutTableBytes + (dense ? (size_t)m.occ_bytes : 0) + (size_t)(32 * ((n + 63) / 64)) * 24 +
           sizeof(float4) * kRing * kTiledWarps;
}

int tiled_warps_per_cta() { return kTiledWarps; }

int tiled_pass_points(const MapView& m, bool dense)
{
    const size_t budget = 227 * 1024 - 1024;   // dynamic shared memory left beside the static part
    size_t fixed = tiled_smem_bytes(m, dense, 0);
    if (fixed >= budget) return 0;
    size_t pts = (budget - fixed) / 12 / 64 * 64;
    return (int)(pts < (size_t)kMaxPassPoints ? pts : (size_t)kMaxPassPoints);
}

int launch_eval_pass(const MapView& m, float a_hit, int P, int n0, int n1, int n_total, bool first, bool serial,
                     bool dense, bool generic, const EvalBuffers& b, double* sum_f64, int sm_count, cudaStream_t s)
{
    EvalParams p;
    p.m = m;
    p.pose12 = b.pose12;
    p.xs = b.xs; p.ys = b.ys; p.zs = b.zs; p.cs = b.cs;
    p.pxy = b.pxy; p.pz = b.pz; p.perm = b.perm;
    p.lut_fx = b.lut_fx;
    p.lut_f = b.lut_f;
    p.sum_fx = b.sum_fx;
    p.sum_f64 = sum_f64;
    p.raw = b.raw;
    p.hits = b.hits;
    p.dbg = b.dbg_index;
    p.order = b.order;
    p.sched = b.counts + 2;
    p.status = b.status;
    p.P = P; p.n0 = n0; p.n1 = n1; p.n_total = n_total; p.first_pass = first ? 1 : 0;
    p.a_hit = a_hit;
    size_t smem = eval_smem_bytes(serial, n1 - n0);
    const bool f32 = m.storage != 0;   // value slots (float or half) rather than codes
    if (serial) {
        auto k = f32 ? eval_serial_kernel<true> : eval_serial_kernel<false>;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k<<<(P + 255) / 256, 256, smem, s>>>(p);
        g_launches += 1;
    } else if (!f32 && m.tiled && !generic) {
        // one launch covers the whole scan; sums are accumulated with atomics
        TiledParams tp;
        tp.e = p;
        tp.chunk = kTiledChunk;
        tp.group = kTiledGroup;
        // small filters: smaller work items (fewer particles, then fewer points)
        // until the grid has about two per warp; the sums are exact integers,
        // so the shape changes no result
        auto items_of = [&](int chunk, int group) {
            return (long long)((n1 - n0 + chunk - 1) / chunk) * (long long)((P + group - 1) / group);
        };
        const long long want = 2ll * sm_count * kTiledWarps;
        while (items_of(tp.chunk, tp.group) < want && (tp.group > 1 || tp.chunk > 256)) {
            if (tp.group > 1) tp.group /= 2;
            else tp.chunk /= 2;
        }
        tp.groups = (P + tp.group - 1) / tp.group;
        tp.items = ((n1 - n0 + tp.chunk - 1) / tp.chunk) * tp.groups;
        // sub_fast 2: floor(s * sub_inv) is the sub-voxel index; 1: the two-term multiplier
        const bool two = m.sub_fast == 1, dbg = p.dbg != nullptr;
        // the slot: from the brick index alone on the grid layout; else the brick
        // rank from the shared-memory bitmap, the sparse brick hash when the map
        // has one, or the brick table
        const int lay = m.grid_b ? kLayGrid : (dense ? kLayBitmap : (m.hash ? kLayHash : kLayTable));
        size_t tsmem = tiled_smem_bytes(m, dense, n1 - n0);
        // pose_prepare_kernel cleared sum_fx and hits before the first pass
        int blocks = sm_count;
        int need = (tp.items + kTiledWarps - 1) / kTiledWarps;
        if (need < blocks) blocks = need > 0 ? need : 1;
        // the debug kernel scores either kind of cloud; otherwise the compact
        // and the spread kernel run back to back, the one not meant for the
        // staging kernel's choice returning at once
        const int clouds[2] = {dbg ? kCloudAny : kCloudCompact, kCloudSpread};
        for (int ci = 0; ci < (dbg ? 1 : 2); ++ci) {
            auto k = pick_tiled(lay, two, dbg, m.min0 != 0, clouds[ci]);
            cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsmem);
            launch_chained(k, (unsigned)blocks, kTiledThreads, tsmem, s, tp);
            g_launches += 1;
        }
    } else {
        auto k = dense && !f32 ? eval_exact_kernel<true, 0>
                               : (m.storage == 2 ? eval_exact_kernel<false, 2>
                                                 : (f32 ? eval_exact_kernel<false, 1> : eval_exact_kernel<false, 0>));
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int blocks = sm_count;
        int need = (P + 31) / 32;
        if (need < blocks) blocks = need > 0 ? need : 1;
        k<<<blocks, 1024, smem, s>>>(p);
        g_launches += 1;
    }
    return check(cudaGetLastError());
}

template <bool DENSE, bool TWO>
void (*pick_sub_2(bool min0))(SubParams)
{
    return min0 ? eval_subsample_kernel<DENSE, TWO, true> : eval_subsample_kernel<DENSE, TWO, false>;
}

int launch_eval_subsample(const MapView& m, float a_hit, int P, int N, int K, unsigned long long seed, float c_in,
                          const EvalBuffers& b, int sm_count, cudaStream_t s)
{
    if (!m.tiled || m.storage != 0) return TSDFL_ERR_UNSUPPORTED;
    SubParams sp;
    EvalParams& p = sp.e;
    p = EvalParams{};
    p.m = m;
    p.pose12 = b.pose12;
    p.xs = b.xs; p.ys = b.ys; p.zs = b.zs; p.cs = b.cs;
    p.lut_fx = b.lut_fx;
    p.sum_fx = b.sum_fx;
    p.hits = b.hits;
    p.order = b.order;
    p.sched = b.counts + 2;
    p.status = b.status;
    p.P = P; p.n0 = 0; p.n1 = N; p.n_total = N; p.first_pass = 1;
    p.a_hit = a_hit;
    sp.K = K;
    sp.seed = seed;
    sp.nin = b.nin;
    sp.c_in = c_in;
    const bool dense = m.occ_bytes != 0, two = m.sub_fast == 1;
    auto k = dense ? (two ? pick_sub_2<true, true>(m.min0 != 0) : pick_sub_2<true, false>(m.min0 != 0))
                   : (two ? pick_sub_2<false, true>(m.min0 != 0) : pick_sub_2<false, false>(m.min0 != 0));
    const size_t smem = (size_t)kLutTableBytes + (dense ? (size_t)m.occ_bytes : 0) + sizeof(float4) * kRing * kTiledWarps;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int blocks = sm_count;
    const int need = (P + kTiledWarps - 1) / kTiledWarps;
    if (need < blocks) blocks = need > 0 ? need : 1;
    k<<<blocks, kTiledThreads, smem, s>>>(sp);
    g_launches += 1;
    return check(cudaGetLastError());
}

size_t batch_seg_bytes() { return sizeof(BatchSeg); }

uint32_t build_batch_segs(const BatchSegSpec* specs, int nseg, int chunk, int group, void* host_out,
                          BatchKinds* kinds)
{
    BatchSeg* out = static_cast<BatchSeg*>(host_out);
    // within a kind, the segments of one map follow each other, so that the L2
    // holds one map's footprint at a time
    std::vector<int> order(nseg);
    for (int i = 0; i < nseg; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return reinterpret_cast<uintptr_t>(specs[a].m.codes) < reinterpret_cast<uintptr_t>(specs[b].m.codes);
    });
    uint32_t total = 0;
    int o = 0;
    for (int kind = 0; kind < 8; ++kind) {   // bit 2: min at the origin, bit 1: compact, bit 0: two-term
        kinds->first[kind] = o;
        kinds->count[kind] = 0;
        uint32_t batches = 0;
        for (int oi = 0; oi < nseg; ++oi) {
            const BatchSegSpec& sp = specs[order[oi]];
            const int k = (sp.m.min0 ? 4 : 0) + (sp.dense ? 2 : 0) + (sp.m.sub_fast == 1 ? 1 : 0);
            if (k != kind) continue;
            const EvalBuffers& b = sp.b;
            BatchSeg g{};
            EvalParams& p = g.e;
            p.m = sp.m;
            p.pose12 = b.pose12;
            p.xs = b.xs; p.ys = b.ys; p.zs = b.zs; p.cs = b.cs;
            p.pxy = b.pxy; p.pz = b.pz; p.perm = b.perm;
            p.lut_fx = b.lut_fx;
            p.lut_f = b.lut_f;
            p.sum_fx = b.sum_fx;
            p.hits = b.hits;
            p.status = b.status;
            p.P = sp.P; p.n0 = sp.n0; p.n1 = sp.n1; p.n_total = sp.n_total; p.first_pass = sp.n0 == 0 ? 1 : 0;
            p.a_hit = sp.a_hit;
            g.chunk = chunk;
            g.group = group;
            g.groups = (sp.P + group - 1) / group;
            g.items = ((sp.n1 - sp.n0 + chunk - 1) / chunk) * g.groups;
            g.dense = sp.dense ? 1 : 0;
            g.two = sp.m.sub_fast == 1 ? 1 : 0;
            g.first_batch = batches;
            batches += (uint32_t)((g.items + kBatchItems - 1) / kBatchItems);
            out[o++] = g;
            kinds->count[kind]++;
        }
        kinds->batches[kind] = batches;
        total += batches;
    }
    return total;
}

size_t batch_smem_bytes() { return 227 * 1024 - 1024; }

int launch_eval_batch(const void* d_segs, const BatchKinds& kinds, uint32_t* counter, int32_t* status,
                      int sm_count, cudaStream_t s)
{
    const BatchSeg* segs = static_cast<const BatchSeg*>(d_segs);
    const size_t smem = batch_smem_bytes();
    using BatchKernel = void (*)(const BatchSeg*, int, uint32_t, uint32_t*, int32_t*);
    static const BatchKernel kKinds[8] = {
        eval_batch_kernel<false, false, false>, eval_batch_kernel<false, true, false>,
        eval_batch_kernel<true, false, false>,  eval_batch_kernel<true, true, false>,
        eval_batch_kernel<false, false, true>,  eval_batch_kernel<false, true, true>,
        eval_batch_kernel<true, false, true>,   eval_batch_kernel<true, true, true>};
    for (int kind = 0; kind < 8; ++kind) {
        if (kinds.count[kind] == 0 || kinds.batches[kind] == 0) continue;
        auto k = kKinds[kind];
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaMemsetAsync(counter, 0, sizeof(uint32_t), s);
        unsigned blocks = (unsigned)sm_count;
        if (kinds.batches[kind] < blocks) blocks = kinds.batches[kind];
        k<<<blocks, kTiledThreads, smem, s>>>(segs + kinds.first[kind], kinds.count[kind], kinds.batches[kind],
                                              counter, status);
        g_launches += 1;
    }
    return check(cudaGetLastError());
}

int launch_norm(int P, int mode, int shift, double a_hit, double c_in, double c_out, int n_points,
                const double* sum_f64, float* particles_out, float* pose_out, const EvalBuffers& b, cudaStream_t s,
                int32_t* sticky, const uint32_t* nin, bool log_domain)
{
    // one block per kNormThreads particles, at most kNormBlocks: the block count
    // depends on P alone, so the sums' order does too
    const int nb = std::max(1, std::min(kNormBlocks, (P + kNormThreads - 1) / kNormThreads));
    NormParams q{P, mode, shift, a_hit, c_in, c_out, n_points, nin};
    launch_chained(norm_partial_kernel, (unsigned)nb, kNormThreads, 0, s, q, b, sum_f64);
    launch_chained(norm_final_kernel, 1, kNormBlocks, 0, s, b, pose_out, nb);
    g_launches += 2;
    if (P > 0 && log_domain) {
        cudaMemsetAsync(b.counts + 1, 0, sizeof(int32_t), s);
        log_max_kernel<<<kNormBlocks, kNormThreads, 0, s>>>(P, b);
        log_sum_kernel<<<kNormBlocks, kNormThreads, 0, s>>>(P, b);
        log_final_kernel<<<1, kNormBlocks, 0, s>>>(b);
        normalize_log_kernel<<<(P + 255) / 256, 256, 0, s>>>(P, b, particles_out, sticky);
        g_launches += 4;
    } else if (P > 0) {
        launch_chained(normalize_kernel, (unsigned)((P + 255) / 256), 256, 0, s, P, b, particles_out, sticky);
        g_launches += 1;
    }
    return check(cudaGetLastError());
}

size_t resample_workspace_bytes(size_t M)
{
    size_t tiles = (M + kScanTile - 1) / kScanTile + 1;
    size_t chunks = (M + kSumsChunk - 1) / kSumsChunk + 1;
    // flags: 16 + 16 + 8 + 4 + 4 <= 64
    return 8 * (M + 3 * tiles) + sizeof(Segment) * kMaxSegments + 64 + sizeof(SumsChunk) * chunks;
}

int launch_resample_impl(const float* particles, const float* w, int stride, size_t M, float u0, float* out,
                         uint32_t* idx_out, size_t cap, uint32_t* count_out, void* workspace, int32_t* status,
                         cudaStream_t s, const float* u0p)
{
    size_t tiles = (M + kScanTile - 1) / kScanTile;
    char* p = static_cast<char*>(workspace);
    ResampleWs ws;
    ws.cdf = reinterpret_cast<long long*>(p); p += 8 * M;
    ws.tile_sums = reinterpret_cast<long long*>(p); p += 8 * (tiles + 1);
    ws.tile_off = reinterpret_cast<long long*>(p); p += 8 * (tiles + 1);
    ws.segs = reinterpret_cast<Segment*>(p); p += sizeof(Segment) * kMaxSegments;
    ws.nseg = reinterpret_cast<int*>(p); p += 16;
    ws.exact_ok = reinterpret_cast<int*>(p); p += 16;
    ws.total = reinterpret_cast<long long*>(p); p += 8;
    int* err = reinterpret_cast<int*>(p); p += 4;
    ws.serial = reinterpret_cast<int*>(p); p += 4;
    ws.tile_dsum = reinterpret_cast<double*>(p); p += 8 * (tiles + 1);
    ws.chunks = reinterpret_cast<SumsChunk*>(p);
    ws.sums = reinterpret_cast<double*>(ws.cdf);
    ws.u0p = u0p;
    const unsigned chunks = (unsigned)((M + kSumsChunk - 1) / kSumsChunk);
    // the literal loop reuses the prefix-sum array for counts and offsets
    uint32_t* cnt = reinterpret_cast<uint32_t*>(ws.cdf);
    uint32_t* off = cnt + M;
    unsigned long long* total = reinterpret_cast<unsigned long long*>(ws.total);
    const unsigned blocks = (unsigned)((M + 255) / 256);
    launch_chained(set_flags_kernel, 1, 1, 0, s, ws.exact_ok, ws.serial, err);
    launch_chained(resample_scan_kernel, (unsigned)tiles, kScanThreads, 0, s, w, stride, (int)M, ws);
    launch_chained(resample_segments_kernel, 1, 32, 0, s, (int)M, u0, (int)tiles, ws);
    launch_chained(resample_assign_kernel, blocks, 256, 0, s, particles, (int)M, out, idx_out, (long long)cap,
                   count_out, ws, status);
    // exact fallbacks: serial double sums + parallel assignment, else the literal loop
    launch_chained(resample_chunk_transfer_kernel, chunks ? chunks : 1u, kSumsThreads, 0, s, w, stride, (int)M, ws);
    launch_chained(resample_sums_kernel, 1, kSumsThreads, 0, s, w, stride, (int)M, u0, ws, cnt, off, total, err);
    launch_chained(resample_chunk_write_kernel, chunks ? chunks : 1u, kSumsThreads, 0, s, w, stride, (int)M, ws);
    launch_chained(resample_fallback_assign_kernel, blocks, 256, 0, s, particles, (int)M, out, idx_out,
                   (long long)cap, count_out, ws, status, (const uint32_t*)cnt, (const uint32_t*)off,
                   (const unsigned long long*)total, (const int*)err);
    g_launches += 8;
    return check(cudaGetLastError());
}

int launch_resample_residual(const float* particles, const float* w, int stride, size_t M, float u0, float* out,
                             uint32_t* idx_out, size_t cap, uint32_t* count_out, void* workspace, int32_t* status,
                             cudaStream_t s)
{
    char* p = static_cast<char*>(workspace);
    uint32_t* cnt = reinterpret_cast<uint32_t*>(p);
    uint32_t* off = cnt + M;
    unsigned long long* total = reinterpret_cast<unsigned long long*>(p + ((8 * M + 15) / 16) * 16);
    int* err = reinterpret_cast<int*>(total + 1);
    set_int_kernel<<<1, 1, 0, s>>>(err, 0);
    residual_chain_kernel<<<1, kChainThreads, 0, s>>>(w, stride, (int)M, u0, cnt, off, total, err);
    resample_scatter_kernel<<<(unsigned)((M + 255) / 256), 256, 0, s>>>(particles, (int)M, cnt, off, total, err,
                                                                         out, idx_out, (long long)cap, count_out,
                                                                         status);
    g_launches += 3;
    return check(cudaGetLastError());
}

int launch_best_particle(const float* particles, size_t M, unsigned long long* key, uint32_t* index_out, int sm_count,
                         cudaStream_t s)
{
    cudaMemsetAsync(key, 0, sizeof(unsigned long long), s);
    unsigned blocks = (unsigned)((M + 255) / 256);
    if (blocks > (unsigned)(4 * sm_count)) blocks = (unsigned)(4 * sm_count);
    if (blocks == 0) blocks = 1;
    best_particle_kernel<<<blocks, 256, 0, s>>>(particles, (int)M, key);
    best_index_kernel<<<1, 1, 0, s>>>(key, index_out);
    g_launches += 2;
    return check(cudaGetLastError());
}

int launch_codes_from_floats(const float* data, size_t n, const float* code_values, float init_value,
                             uint16_t* codes, int32_t* fail, cudaStream_t s)
{
    if (n) codes_from_floats_kernel<<<1024, 256, 0, s>>>(data, n, code_values, init_value, codes, fail);
    return check(cudaGetLastError());
}

int launch_grid_fill(const uint16_t* codes, const int32_t* grid_occ, uint64_t up_dim_2, uint64_t sub_dim_3,
                     uint64_t n, uint16_t* grid, cudaStream_t s)
{
    if (n) grid_fill_kernel<<<4096, 256, 0, s>>>(codes, grid_occ, up_dim_2, sub_dim_3, n, grid);
    return check(cudaGetLastError());
}

int launch_halves(const uint16_t* codes, const float* code_values, const float* data, size_t n, uint16_t* h16,
                  cudaStream_t s)
{
    if (n) halves_kernel<<<1024, 256, 0, s>>>(codes, code_values, data, n, h16);
    return check(cudaGetLastError());
}


}  // namespace tsdfl
