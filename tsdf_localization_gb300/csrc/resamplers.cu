// The reference's other resamplers on the device.  Each emits exactly M
// particles; their random draws come from the caller (the reference's own
// sequence, drawn on the host in its order: the output is then the reference's
// bit for bit) or from Philox4x64-10 keyed by the seed (philox.h).
//
//   WheelResampler       (wheel_resampler.cpp:6-33)  float running sums, first
//                        sum >= the draw; no such sum: the particle stays
//   ResidualResampler    (novel_resampling.h:9-35)   random particles, each
//                        copied ceil(M * w) times until M are emitted
//   MetropolisResampler  (novel_resampling.h:106-143) B proposals per output,
//                        accepted against particle 0's weight (the reference
//                        binds particle_k once, to particle 0)
//   RejectionResampler   (novel_resampling.h:146-187) proposals until
//                        u <= w_j / max w
#include <stdint.h>

#include <atomic>

#include "philox.h"
#include "tsdfl_internal.h"

namespace tsdfl {

extern std::atomic<unsigned long long> g_launches;

namespace {

constexpr int kWheelTile = 2048;
constexpr int kWheelThreads = 512;
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;

int check(cudaError_t e) { return e == cudaSuccess ? TSDFL_OK : TSDFL_ERR_DEVICE; }

__device__ __forceinline__ void gather(const float* particles, uint32_t src, size_t dst, float* out,
                                       uint32_t* idx_out)
{
    if (idx_out) idx_out[dst] = src;
    if (out) {
        const float* a = particles + 7 * (size_t)src;
        float* b = out + 7 * dst;
#pragma unroll
        for (int k = 0; k < 7; ++k) b[k] = a[k];
    }
}

// ------------------------------------------------------------------ wheel

// wheel_resampler.cpp:22-30: weight_sum += w_m in float, in particle order.
// One thread walks the sums over weights staged in shared memory (only the
// additions chain); the block then forms their running maximum R_m with
// fmaxf, which skips NaN (a NaN sum stays NaN, so R stops growing at the first
// one).  The first m with draw <= sum_m is the first m with draw <= R_m, so a
// binary search over R finds it.
__global__ void __launch_bounds__(kWheelThreads) wheel_sums_kernel(const float* __restrict__ w, int stride,
                                                                   uint32_t M, float* __restrict__ R)
{
    static_assert(kWheelTile == 4 * kWheelThreads, "four sums per thread in the running maximum");
    __shared__ float sw[kWheelTile];
    __shared__ float sr[kWheelTile];
    __shared__ float warp_max[kWheelThreads / 32];
    __shared__ float s_carry;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float s = 0.0f;
    if (threadIdx.x == 0) s_carry = -INFINITY;
    for (uint32_t base = 0; base < M; base += kWheelTile) {
        const uint32_t t = min((uint32_t)kWheelTile, M - base);
        for (uint32_t i = threadIdx.x; i < kWheelTile; i += blockDim.x)
            sw[i] = i < t ? w[(size_t)(base + i) * stride] : 0.0f;
        __syncthreads();
        if (threadIdx.x == 0) {
            // 32 weights to registers at a time (one load latency per 32 additions)
            for (uint32_t i = 0; i < t; i += 32) {
                float v[32];
#pragma unroll
                for (int k = 0; k < 32; ++k) v[k] = sw[i + k];
#pragma unroll
                for (int k = 0; k < 32; ++k) {
                    s = __fadd_rn(s, v[k]);
                    v[k] = s;
                }
#pragma unroll
                for (int k = 0; k < 32; ++k) sr[i + k] = v[k];
            }
        }
        __syncthreads();
        // running maximum of this tile's sums, four per thread, from the carry
        float m[4], run = -INFINITY;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t i = 4 * threadIdx.x + k;
            run = fmaxf(run, i < t ? sr[i] : -INFINITY);
            m[k] = run;
        }
        float x = run;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x = fmaxf(x, y);
        }
        if (lane == 31) warp_max[warp] = x;
        __syncthreads();
        float before = s_carry, tile_max = s_carry;
        for (int k = 0; k < kWheelThreads / 32; ++k) {
            if (k < warp) before = fmaxf(before, warp_max[k]);
            tile_max = fmaxf(tile_max, warp_max[k]);
        }
        const float xprev = __shfl_up_sync(0xffffffffu, x, 1);
        if (lane > 0) before = fmaxf(before, xprev);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t i = 4 * threadIdx.x + k;
            if (i < t) R[base + i] = fmaxf(before, m[k]);
        }
        __syncthreads();
        if (threadIdx.x == 0) s_carry = tile_max;
        __syncthreads();
    }
}

__global__ void wheel_assign_kernel(const float* particles, const float* __restrict__ R, uint32_t M,
                                    const double* draws, unsigned long long seed, float* out, uint32_t* idx_out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M) return;
    double u;
    if (draws) {
        u = draws[i];
    } else {
        unsigned long long c[4] = {i, 0, 0, 0};
        philox4x64_10(c, seed, kStreamWheel);
        u = u01_double(c[0]);
    }
    const float r = (float)u;   // FLOAT_T random_value = uniform_distribution(...)
    uint32_t lo = 0, hi = M;
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (r <= R[mid]) hi = mid;
        else lo = mid + 1;
    }
    gather(particles, lo < M ? lo : i, i, out, idx_out);
}

// --------------------------------------------------------------- residual

// Draw j picks particle r_j, which ResidualResampler copies
// count_j = #{index : (float)index < insertions} times, insertions =
// min(fl(w * (float)M), left) (novel_resampling.h:22-30).  With
// c_j = ceil(fl(w * M)) (0 for a non-positive product, M for NaN or anything
// above M) and C_j their inclusive sums, output p takes r_j for the first j
// with C_j > p: the cap on the last draw only cuts at M.
__global__ void residual_counts_kernel(const float* __restrict__ w, int stride, uint32_t M, const uint32_t* draws,
                                       uint32_t K, unsigned long long seed, uint32_t* __restrict__ r,
                                       unsigned long long* __restrict__ c, int32_t* status)
{
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;   // draws 4q .. 4q+3
    if (4ull * q >= K) return;
    unsigned long long words[4] = {q, 0, 0, 0};
    if (!draws) philox4x64_10(words, seed, kStreamResidual);
    const float Mf = (float)M;
    for (int k = 0; k < 4; ++k) {
        const uint32_t j = 4 * q + k;
        if (j >= K) break;
        uint32_t ri = draws ? draws[j] : uniform_index(words[k], M);
        unsigned long long cnt = 0;
        if (ri >= M) {
            atomicExch(status, TSDFL_ERR_INVALID_ARG);
            ri = 0;
        } else {
            const float e = __fmul_rn(w[(size_t)ri * stride], Mf);
            if (!(e <= Mf)) cnt = M;
            else if (e > 0.0f) cnt = (unsigned long long)ceilf(e);
        }
        r[j] = ri;
        c[j] = cnt;
    }
}

// Inclusive sums of c[0..K) in place: per-tile sums (kScanTile values a
// block), one block scanning the tile sums, each tile rescanned from its offset.
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ unsigned long long block_exclusive(unsigned long long v, unsigned long long* warp_tot,
                                                              unsigned long long& total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    __syncthreads();
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    unsigned long long off = 0;
    total = 0;
    for (int k = 0; k < kScanThreads / 32; ++k) {
        if (k < warp) off += warp_tot[k];
        total += warp_tot[k];
    }
    return off + x - v;
}

__global__ void __launch_bounds__(kScanThreads) tile_sums_u64_kernel(const unsigned long long* __restrict__ c,
                                                                     uint32_t K, unsigned long long* tile_sum)
{
    __shared__ unsigned long long warp_tot[kScanThreads / 32];
    const uint32_t base = blockIdx.x * kScanTile;
    unsigned long long run = 0;
    for (int k = 0; k < kScanItems; ++k) {
        const uint32_t i = base + kScanItems * threadIdx.x + k;
        run += i < K ? c[i] : 0;
    }
    unsigned long long total;
    block_exclusive(run, warp_tot, total);
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

// Exclusive prefix of tile_sum[0..tiles) in place (one block).
__global__ void __launch_bounds__(kScanThreads) scan_tile_sums_kernel(unsigned long long* tile_sum, uint32_t tiles)
{
    __shared__ unsigned long long warp_tot[kScanThreads / 32];
    __shared__ unsigned long long s_base;
    if (threadIdx.x == 0) s_base = 0;
    for (uint32_t base = 0; base < tiles; base += kScanThreads) {
        const uint32_t t = base + threadIdx.x;
        const unsigned long long v = t < tiles ? tile_sum[t] : 0;
        unsigned long long total;
        const unsigned long long ex = block_exclusive(v, warp_tot, total);
        if (t < tiles) tile_sum[t] = s_base + ex;
        __syncthreads();
        if (threadIdx.x == 0) s_base += total;
    }
}

__global__ void __launch_bounds__(kScanThreads) tile_rescan_u64_kernel(unsigned long long* c, uint32_t K,
                                                                       const unsigned long long* tile_off)
{
    __shared__ unsigned long long warp_tot[kScanThreads / 32];
    const uint32_t base = blockIdx.x * kScanTile;
    unsigned long long v[kScanItems], run = 0;
    for (int k = 0; k < kScanItems; ++k) {
        const uint32_t i = base + kScanItems * threadIdx.x + k;
        v[k] = i < K ? c[i] : 0;
        run += v[k];
    }
    unsigned long long total;
    unsigned long long off = tile_off[blockIdx.x] + block_exclusive(run, warp_tot, total);
    for (int k = 0; k < kScanItems; ++k) {
        const uint32_t i = base + kScanItems * threadIdx.x + k;
        off += v[k];
        if (i < K) c[i] = off;
    }
}

__global__ void residual_assign_kernel(const float* particles, uint32_t M, const uint32_t* __restrict__ r,
                                       const unsigned long long* __restrict__ C, uint32_t K, float* out,
                                       uint32_t* idx_out, int32_t* status)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= M) return;
    if (C[K - 1] < M) {   // the draws ran out before M particles were emitted (an invalid draw reported first stays)
        if (p == 0) atomicCAS(status, 0, TSDFL_ERR_UNSUPPORTED);
        return;
    }
    uint32_t lo = 0, hi = K - 1;
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (C[mid] > p) hi = mid;
        else lo = mid + 1;
    }
    gather(particles, r[lo], p, out, idx_out);
}

// ------------------------------------------------------------- metropolis

__global__ void metropolis_kernel(const float* particles, const float* __restrict__ w, int stride, uint32_t M,
                                  uint32_t steps, const float* u_draws, const uint32_t* j_draws,
                                  unsigned long long seed, float* out, uint32_t* idx_out, int32_t* status)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M) return;
    const float w0 = w[0];   // particle_k stays bound to particle 0 (novel_resampling.h:122)
    uint32_t k = 0;
    unsigned long long words[4] = {0, 0, 0, 0};
    for (uint32_t n = 0; n < steps; ++n) {
        float u;
        uint32_t j;
        if (u_draws) {
            u = u_draws[(size_t)i * steps + n];
            j = j_draws[(size_t)i * steps + n];
            if (j >= M) {
                atomicExch(status, TSDFL_ERR_INVALID_ARG);
                continue;
            }
        } else {
            if ((n & 1) == 0) {
                words[0] = i;
                words[1] = n >> 1;
                words[2] = 0;
                words[3] = 0;
                philox4x64_10(words, seed, kStreamMetropolis);
            }
            u = u01_float(words[2 * (n & 1)]);
            j = uniform_index(words[2 * (n & 1) + 1], M);
        }
        if (u <= __fdiv_rn(w[(size_t)j * stride], w0)) k = j;
    }
    gather(particles, k, i, out, idx_out);
}

// -------------------------------------------------------------- rejection

// sup_w = max(0.0, max w) as the reference's double loop forms it
// (novel_resampling.h:158-168): positive floats order like their bits.
__global__ void max_weight_kernel(const float* __restrict__ w, int stride, uint32_t M, unsigned int* bits)
{
    unsigned int best = 0;
    for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
        const float x = w[(size_t)m * stride];
        if (x > 0.0f) best = max(best, __float_as_uint(x));
    }
    for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0 && best) atomicMax(bits, best);
}

__global__ void rejection_kernel(const float* particles, const float* __restrict__ w, int stride, uint32_t M,
                                 const unsigned int* sup_bits, unsigned long long seed, uint32_t max_rounds,
                                 float* out, uint32_t* idx_out, int32_t* status)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M) return;
    const double sup = (double)__uint_as_float(*sup_bits);
    uint32_t j = i;
    unsigned long long c[4] = {i, 0, 0, 0};
    philox4x64_10(c, seed, kStreamRejection);
    float u = u01_float(c[0]);
    for (uint32_t t = 1; (double)u > __ddiv_rn((double)w[(size_t)j * stride], sup); ++t) {
        if (t > max_rounds) {   // the reference would keep drawing
            atomicExch(status, TSDFL_ERR_UNSUPPORTED);
            break;
        }
        c[0] = i;
        c[1] = t;
        c[2] = 0;
        c[3] = 0;
        philox4x64_10(c, seed, kStreamRejection);
        j = uniform_index(c[0], M);
        u = u01_float(c[1]);
    }
    gather(particles, j, i, out, idx_out);
}

}  // namespace

size_t resamplers_workspace_bytes(size_t M, size_t K)
{
    auto a = [](size_t v) { return (v + 255) / 256 * 256; };
    const size_t wheel = a(4 * M);
    const size_t residual = a(4 * K) + a(8 * K) + a(8 * ((K + 4095) / 4096 + 1));
    return (wheel > residual ? wheel : residual) + 256;
}

int launch_resample_wheel(const float* particles, const float* w, int stride, size_t M, const double* draws,
                          uint64_t seed, float* out, uint32_t* idx_out, void* ws, cudaStream_t s)
{
    if (M == 0) return TSDFL_OK;
    float* R = static_cast<float*>(ws);
    wheel_sums_kernel<<<1, kWheelThreads, 0, s>>>(w, stride, (uint32_t)M, R);
    wheel_assign_kernel<<<(unsigned)((M + 255) / 256), 256, 0, s>>>(particles, R, (uint32_t)M, draws, seed, out,
                                                                     idx_out);
    g_launches += 2;
    return check(cudaGetLastError());
}

int launch_resample_residual_random(const float* particles, const float* w, int stride, size_t M,
                                    const uint32_t* draws, size_t K, uint64_t seed, float* out, uint32_t* idx_out,
                                    void* ws, int32_t* status, cudaStream_t s)
{
    if (M == 0) return TSDFL_OK;
    auto a = [](size_t v) { return (v + 255) / 256 * 256; };
    uint32_t* r = static_cast<uint32_t*>(ws);
    unsigned long long* C = reinterpret_cast<unsigned long long*>(static_cast<char*>(ws) + a(4 * K));
    unsigned long long* tile = reinterpret_cast<unsigned long long*>(static_cast<char*>(ws) + a(4 * K) + a(8 * K));
    const size_t quads = (K + 3) / 4;
    const unsigned tiles = (unsigned)((K + kScanTile - 1) / kScanTile);
    residual_counts_kernel<<<(unsigned)((quads + 255) / 256), 256, 0, s>>>(w, stride, (uint32_t)M, draws,
                                                                          (uint32_t)K, seed, r, C, status);
    tile_sums_u64_kernel<<<tiles, kScanThreads, 0, s>>>(C, (uint32_t)K, tile);
    scan_tile_sums_kernel<<<1, kScanThreads, 0, s>>>(tile, tiles);
    tile_rescan_u64_kernel<<<tiles, kScanThreads, 0, s>>>(C, (uint32_t)K, tile);
    residual_assign_kernel<<<(unsigned)((M + 255) / 256), 256, 0, s>>>(particles, (uint32_t)M, r, C, (uint32_t)K,
                                                                        out, idx_out, status);
    g_launches += 5;
    return check(cudaGetLastError());
}

int launch_resample_metropolis(const float* particles, const float* w, int stride, size_t M, uint32_t steps,
                               const float* u_draws, const uint32_t* j_draws, uint64_t seed, float* out,
                               uint32_t* idx_out, int32_t* status, cudaStream_t s)
{
    if (M == 0) return TSDFL_OK;
    metropolis_kernel<<<(unsigned)((M + 255) / 256), 256, 0, s>>>(particles, w, stride, (uint32_t)M, steps, u_draws,
                                                                   j_draws, seed, out, idx_out, status);
    g_launches += 1;
    return check(cudaGetLastError());
}

int launch_resample_rejection(const float* particles, const float* w, int stride, size_t M, uint64_t seed,
                              uint32_t max_rounds, float* out, uint32_t* idx_out, void* ws, int32_t* status,
                              int sm_count, cudaStream_t s)
{
    if (M == 0) return TSDFL_OK;
    unsigned int* bits = static_cast<unsigned int*>(ws);
    cudaMemsetAsync(bits, 0, sizeof(unsigned int), s);
    unsigned blocks = (unsigned)((M + 255) / 256);
    if (blocks > (unsigned)(4 * sm_count)) blocks = (unsigned)(4 * sm_count);
    max_weight_kernel<<<blocks, 256, 0, s>>>(w, stride, (uint32_t)M, bits);
    rejection_kernel<<<(unsigned)((M + 255) / 256), 256, 0, s>>>(particles, w, stride, (uint32_t)M, bits, seed,
                                                                  max_rounds, out, idx_out, status);
    g_launches += 2;
    return check(cudaGetLastError());
}

}  // namespace tsdfl
