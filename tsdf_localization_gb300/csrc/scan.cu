// Scan reduction on the device: the pre-processing TSDFEvaluator::evaluateParticles
// applies to a PointCloud2 before scoring (tsdf_evaluator.cpp:304-376).
//
//   1. points with sqrt(x*x + y*y + z*z) < 1 (float) are dropped;
//   2. the k-th kept point gets index k and the ring field of cloud point k
//      (the reference advances its ring iterator only for kept points,
//      :319-332), or its own ring with TSDFL_SCAN_OWN_RING;
//   3. per axis the cell centre floor(v / cell) * cell + cell / 2 (float);
//   4. of the points sharing (ring, centre) the one with the smallest index
//      stays (unordered_set::insert keeps the first, :328); a NaN centre never
//      equals another, so such points always stay;
//   5. the survivors are written ring by ring (0..63), by index within a ring
//      (:339-373), as their original float x, y, z.
//
// Layout: the cloud stays in its PointCloud2 byte layout (point_step bytes per
// point, x, y, z as consecutive floats at x_offset as iter_x[0..2] reads them,
// ring as int16 at ring_offset).  One tile = 256 consecutive cloud points = one
// block of 256 threads.  The (ring, centre) set is
// an open-addressing hash table of 128-bit keys claimed with one 128-bit CAS
// (empty = all ones; a key's high word holds the ring, < 64), load <= 1/2, with
// the smallest index per key kept by atomicMin.
//
// Kernels (one stream, in order):
//   scan_keep_kernel    kept points per tile; clears the hash table
//   scan_tiles_kernel   exclusive prefix of the tile counts (one block)
//   scan_insert_kernel  index k, ring, centre; inserts (ring, centre) -> min k
//   scan_winner_kernel  survivors (the key's minimum is the point's k); per-tile
//                       survivors per ring
//   scan_rings_kernel   output offset of every (ring, tile) within its ring (a block per ring)
//   scan_write_kernel   ring starts; stable multi-split by ring: writes the survivors' x, y, z
#include <stdint.h>

#include <atomic>

#include "tsdfl_internal.h"

namespace tsdfl {

extern std::atomic<unsigned long long> g_launches;

namespace {

constexpr int kScanRings = 64;
constexpr int kScanBlock = 256;
constexpr int kScanRounds = 1;
constexpr int kScanTilePts = kScanBlock * kScanRounds;
constexpr int kScanWarps = kScanBlock / 32;
constexpr uint32_t kNotKept = 0xffffffffu;
constexpr uint32_t kAlwaysStays = 0xfffffffeu;   // NaN centre: never merged
constexpr int kMaxProbeRounds = 1 << 30;         // the table is never more than half full

struct alignas(16) ScanKey {
    unsigned long long hi, lo;
};

struct ScanParams {
    const uint8_t* cloud;
    uint32_t n;
    uint32_t step, off_x, off_ring;
    int aligned4;    // x, y, z are 4-byte aligned in every point
    int aligned2;    // ring is 2-byte aligned in every point
    int own_ring;
    float cell, half;
    uint32_t tiles;
    unsigned long long table_mask;
    ScanKey* keys;
    uint32_t* vals;
    uint32_t* tile_cnt;   // tiles + 1: kept per tile, then its exclusive prefix; [tiles] = total
    uint32_t* kk;         // n: kept index k, kNotKept
    uint32_t* slot;       // n: hash slot, kAlwaysStays
    int8_t* ring8;        // n: ring of kept points (-1 otherwise); after the winner pass: survivors only
    uint32_t* hist;       // kScanRings x tiles: survivors per (ring, tile), then their offsets
    uint32_t* ring_base;  // kScanRings: survivors of each ring
    float* out;
    unsigned long long cap;
    uint32_t* count;
    int32_t* status;
};

__device__ __forceinline__ uint32_t ld_u32(const uint8_t* p, bool aligned)
{
    if (aligned) return *reinterpret_cast<const uint32_t*>(p);
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

__device__ __forceinline__ int ld_i16(const uint8_t* p, bool aligned)
{
    if (aligned) return *reinterpret_cast<const int16_t*>(p);
    return (int)(int16_t)(uint16_t)((uint32_t)p[0] | ((uint32_t)p[1] << 8));
}

__device__ __forceinline__ void load_xyz(const ScanParams& p, uint32_t i, float& x, float& y, float& z)
{
    const uint8_t* q = p.cloud + (size_t)i * p.step + p.off_x;
    x = __uint_as_float(ld_u32(q, p.aligned4));
    y = __uint_as_float(ld_u32(q + 4, p.aligned4));
    z = __uint_as_float(ld_u32(q + 8, p.aligned4));
}

// tsdf_evaluator.cpp:313-321: the float range test (no contraction).
__device__ __forceinline__ bool kept(float x, float y, float z)
{
    const float s = __fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z));
    return !(sqrtf(s) < 1.0f);
}

// tsdf_evaluator.cpp:323-325 in float: floor(v / cell) * cell + cell / 2.
__device__ __forceinline__ float centre(float v, float cell, float half)
{
    return __fadd_rn(__fmul_rn(floorf(__fdiv_rn(v, cell)), cell), half);
}

__device__ __forceinline__ unsigned long long mix(const ScanKey& k)
{
    unsigned long long h = k.hi * 0x9E3779B97F4A7C15ull ^ (k.lo + 0x632BE59BD9B4E019ull) * 0xC2B2AE3D27D4EB4Full;
    h ^= h >> 31;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 29;
    return h;
}

// Exclusive rank of f among the block's threads and the block total (kScanBlock
// threads; s_warp holds kScanWarps words).  Every thread must call it.
__device__ __forceinline__ uint32_t block_rank(bool f, uint32_t* s_warp, uint32_t& total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned b = __ballot_sync(0xffffffffu, f);
    __syncthreads();   // s_warp of the previous call has been read
    if (lane == 0) s_warp[w] = __popc(b);
    __syncthreads();
    uint32_t before = 0;
    total = 0;
#pragma unroll
    for (int v = 0; v < kScanWarps; ++v) {
        const uint32_t c = s_warp[v];
        before += v < w ? c : 0;
        total += c;
    }
    return before + __popc(b & ((1u << lane) - 1u));
}

__global__ void __launch_bounds__(kScanBlock) scan_keep_kernel(ScanParams p)
{
    __shared__ uint32_t s_warp[kScanWarps];
    // clear the hash table (grid-stride)
    const unsigned long long slots = p.table_mask + 1;
    for (unsigned long long s = (unsigned long long)blockIdx.x * kScanBlock + threadIdx.x; s < slots;
         s += (unsigned long long)gridDim.x * kScanBlock) {
        p.keys[s] = ScanKey{~0ull, ~0ull};
        p.vals[s] = 0xffffffffu;
    }
    const uint32_t t0 = blockIdx.x * kScanTilePts;
    uint32_t sum = 0;
    for (int r = 0; r < kScanRounds; ++r) {
        const uint32_t i = t0 + r * kScanBlock + threadIdx.x;
        bool f = false;
        if (i < p.n) {
            float x, y, z;
            load_xyz(p, i, x, y, z);
            f = kept(x, y, z);
        }
        uint32_t tot;
        block_rank(f, s_warp, tot);
        sum += tot;
    }
    if (threadIdx.x == 0) p.tile_cnt[blockIdx.x] = sum;
}

// Exclusive prefix of tile_cnt[0..tiles) in place; tile_cnt[tiles] = total.
__global__ void __launch_bounds__(1024) scan_tiles_kernel(ScanParams p)
{
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_run;
    if (threadIdx.x == 0) s_run = 0;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (uint32_t base = 0; base < p.tiles; base += 1024) {
        const uint32_t t = base + threadIdx.x;
        const uint32_t v = t < p.tiles ? p.tile_cnt[t] : 0;
        uint32_t inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += u;
        }
        __syncthreads();
        if (lane == 31) s_warp[w] = inc;
        __syncthreads();
        uint32_t before = s_run, total = 0;
        for (int q = 0; q < 32; ++q) {
            before += q < w ? s_warp[q] : 0;
            total += s_warp[q];
        }
        if (t < p.tiles) p.tile_cnt[t] = before + inc - v;
        __syncthreads();
        if (threadIdx.x == 0) s_run += total;
    }
    __syncthreads();
    if (threadIdx.x == 0) p.tile_cnt[p.tiles] = s_run;
}

__global__ void __launch_bounds__(kScanBlock) scan_insert_kernel(ScanParams p)
{
    __shared__ uint32_t s_warp[kScanWarps];
    const uint32_t t0 = blockIdx.x * kScanTilePts;
    uint32_t k_base = p.tile_cnt[blockIdx.x];
    for (int r = 0; r < kScanRounds; ++r) {
        const uint32_t i = t0 + r * kScanBlock + threadIdx.x;
        float x = 0, y = 0, z = 0;
        bool f = false;
        if (i < p.n) {
            load_xyz(p, i, x, y, z);
            f = kept(x, y, z);
        }
        uint32_t tot;
        const uint32_t k = k_base + block_rank(f, s_warp, tot);
        k_base += tot;
        if (i >= p.n) continue;
        if (!f) {
            p.kk[i] = kNotKept;
            p.ring8[i] = -1;
            continue;
        }
        const uint32_t rsrc = p.own_ring ? i : k;
        const int ring = ld_i16(p.cloud + (size_t)rsrc * p.step + p.off_ring, p.aligned2);
        p.kk[i] = k;
        if (ring < 0 || ring >= kScanRings) {
            // the reference indexes past its 64 ring lists here; reported, point dropped
            p.ring8[i] = -1;
            atomicExch(p.status, TSDFL_ERR_INVALID_ARG);
            continue;
        }
        p.ring8[i] = (int8_t)ring;
        const float cx = centre(x, p.cell, p.half), cy = centre(y, p.cell, p.half), cz = centre(z, p.cell, p.half);
        if (cx != cx || cy != cy || cz != cz) {
            p.slot[i] = kAlwaysStays;
            continue;
        }
        const ScanKey key{((unsigned long long)ring << 32) | __float_as_uint(cx),
                          ((unsigned long long)__float_as_uint(cy) << 32) | __float_as_uint(cz)};
        unsigned long long s = mix(key) & p.table_mask;
        bool placed = false;
        for (int probe = 0; probe < kMaxProbeRounds && (unsigned long long)probe <= p.table_mask; ++probe) {
            ScanKey old = atomicCAS(&p.keys[s], ScanKey{~0ull, ~0ull}, key);
            if ((old.hi == ~0ull && old.lo == ~0ull) || (old.hi == key.hi && old.lo == key.lo)) {
                atomicMin(&p.vals[s], k);
                placed = true;
                break;
            }
            s = (s + 1) & p.table_mask;
        }
        if (!placed) {
            p.slot[i] = kAlwaysStays;
            atomicExch(p.status, TSDFL_ERR_CAPACITY);
            continue;
        }
        p.slot[i] = (uint32_t)s;
    }
}

__global__ void __launch_bounds__(kScanBlock) scan_winner_kernel(ScanParams p)
{
    __shared__ uint32_t s_hist[kScanRings];
    if (threadIdx.x < kScanRings) s_hist[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t t0 = blockIdx.x * kScanTilePts;
    for (int r = 0; r < kScanRounds; ++r) {
        const uint32_t i = t0 + r * kScanBlock + threadIdx.x;
        if (i >= p.n) break;
        const int ring = p.ring8[i];
        if (ring < 0) continue;
        const uint32_t s = p.slot[i];
        const bool stays = s == kAlwaysStays || p.vals[s] == p.kk[i];
        if (stays) atomicAdd(&s_hist[ring], 1u);
        else p.ring8[i] = -1;
    }
    __syncthreads();
    if (threadIdx.x < kScanRings) p.hist[(size_t)threadIdx.x * p.tiles + blockIdx.x] = s_hist[threadIdx.x];
}

// One block per ring: hist[ring][tile] -> first output position of the
// tile's survivors of that ring relative to the ring's start; ring_total[ring].
__global__ void __launch_bounds__(kScanBlock) scan_rings_kernel(ScanParams p)
{
    __shared__ uint32_t s_warp[kScanWarps];
    __shared__ uint32_t s_run;
    const int ring = blockIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t* h = p.hist + (size_t)ring * p.tiles;
    if (threadIdx.x == 0) s_run = 0;
    for (uint32_t base = 0; base < p.tiles; base += kScanBlock) {
        const uint32_t t = base + threadIdx.x;
        const uint32_t v = t < p.tiles ? h[t] : 0;
        uint32_t inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += u;
        }
        __syncthreads();   // s_run and s_warp of the previous chunk have been read
        if (lane == 31) s_warp[w] = inc;
        __syncthreads();
        uint32_t before = s_run, total = 0;
#pragma unroll
        for (int q = 0; q < kScanWarps; ++q) {
            before += q < w ? s_warp[q] : 0;
            total += s_warp[q];
        }
        if (t < p.tiles) h[t] = before + inc - v;
        __syncthreads();
        if (threadIdx.x == 0) s_run += total;
    }
    __syncthreads();
    if (threadIdx.x == 0) p.ring_base[ring] = s_run;   // the ring's total; scan_write_kernel scans them
}

__global__ void __launch_bounds__(kScanBlock) scan_write_kernel(ScanParams p)
{
    __shared__ uint32_t s_cnt[kScanWarps][kScanRings];
    __shared__ uint32_t s_run[kScanRings];
    __shared__ uint32_t s_off[kScanRings];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x < kScanRings) s_off[threadIdx.x] = p.ring_base[threadIdx.x];
    __syncthreads();
    if (threadIdx.x == 0) {   // the rings' starts: exclusive prefix of their totals
        uint32_t run = 0;
        for (int r = 0; r < kScanRings; ++r) {
            const uint32_t c = s_off[r];
            s_off[r] = run;
            run += c;
        }
        if (blockIdx.x == 0) {
            *p.count = run;
            if (run > p.cap) atomicExch(p.status, TSDFL_ERR_CAPACITY);
        }
    }
    __syncthreads();
    if (threadIdx.x < kScanRings) {
        s_run[threadIdx.x] = 0;
        s_off[threadIdx.x] += p.hist[(size_t)threadIdx.x * p.tiles + blockIdx.x];
    }
    const uint32_t t0 = blockIdx.x * kScanTilePts;
    for (int r = 0; r < kScanRounds; ++r) {
        const uint32_t i = t0 + r * kScanBlock + threadIdx.x;
        const int ring = i < p.n ? p.ring8[i] : -1;
        // peers: the lanes of this warp with the same surviving ring
        const unsigned peers = __match_any_sync(0xffffffffu, ring >= 0 ? ring : kScanRings + lane);
        const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
        __syncthreads();   // the previous round's offsets have been read
        for (int e = threadIdx.x; e < kScanWarps * kScanRings; e += kScanBlock) (&s_cnt[0][0])[e] = 0;
        __syncthreads();
        if (ring >= 0 && rank == 0) s_cnt[w][ring] = __popc(peers);
        __syncthreads();
        if (threadIdx.x < kScanRings) {
            uint32_t run = s_run[threadIdx.x];
#pragma unroll
            for (int v = 0; v < kScanWarps; ++v) {
                const uint32_t c = s_cnt[v][threadIdx.x];
                s_cnt[v][threadIdx.x] = run;
                run += c;
            }
            s_run[threadIdx.x] = run;
        }
        __syncthreads();
        if (ring >= 0) {
            const unsigned long long pos = (unsigned long long)s_off[ring] + s_cnt[w][ring] + rank;
            if (pos < p.cap) {
                const uint8_t* q = p.cloud + (size_t)i * p.step + p.off_x;
                uint32_t* o = reinterpret_cast<uint32_t*>(p.out + 3 * pos);
                o[0] = ld_u32(q, p.aligned4);
                o[1] = ld_u32(q + 4, p.aligned4);
                o[2] = ld_u32(q + 8, p.aligned4);
            }
        }
    }
}

int check(cudaError_t e) { return e == cudaSuccess ? TSDFL_OK : TSDFL_ERR_DEVICE; }

size_t table_slots(size_t n)
{
    size_t s = 1024;
    while (s < 2 * n) s <<= 1;
    return s;
}

}  // namespace

size_t scan_workspace_bytes(size_t n)
{
    const size_t tiles = (n + kScanTilePts - 1) / kScanTilePts;
    const size_t slots = table_slots(n);
    auto a = [](size_t v) { return (v + 255) / 256 * 256; };
    return a(16 * slots) + a(4 * slots) + a(4 * (tiles + 1)) + a(4 * n) + a(4 * n) + a(n) +
           a(4 * kScanRings * (tiles ? tiles : 1)) + a(4 * kScanRings);
}

int launch_reduce_scan(const uint8_t* cloud, size_t n, uint32_t step, uint32_t off_x, uint32_t off_ring, float cell,
                       bool own_ring, float* out, size_t cap, uint32_t* count, void* workspace, int32_t* status,
                       cudaStream_t s)
{
    if (n == 0) {
        cudaMemsetAsync(count, 0, sizeof(uint32_t), s);
        return check(cudaGetLastError());
    }
    const size_t tiles = (n + kScanTilePts - 1) / kScanTilePts;
    const size_t slots = table_slots(n);
    auto a = [](size_t v) { return (v + 255) / 256 * 256; };
    char* w = static_cast<char*>(workspace);
    ScanParams p{};
    p.cloud = cloud;
    p.n = (uint32_t)n;
    p.step = step;
    p.off_x = off_x;
    p.off_ring = off_ring;
    const uintptr_t base = reinterpret_cast<uintptr_t>(cloud);
    p.aligned4 = (base % 4 == 0 && step % 4 == 0 && off_x % 4 == 0) ? 1 : 0;
    p.aligned2 = (base % 2 == 0 && step % 2 == 0 && off_ring % 2 == 0) ? 1 : 0;
    p.own_ring = own_ring ? 1 : 0;
    p.cell = cell;
    p.half = cell / 2;
    p.tiles = (uint32_t)tiles;
    p.table_mask = slots - 1;
    p.keys = reinterpret_cast<ScanKey*>(w); w += a(16 * slots);
    p.vals = reinterpret_cast<uint32_t*>(w); w += a(4 * slots);
    p.tile_cnt = reinterpret_cast<uint32_t*>(w); w += a(4 * (tiles + 1));
    p.kk = reinterpret_cast<uint32_t*>(w); w += a(4 * n);
    p.slot = reinterpret_cast<uint32_t*>(w); w += a(4 * n);
    p.ring8 = reinterpret_cast<int8_t*>(w); w += a(n);
    p.hist = reinterpret_cast<uint32_t*>(w); w += a(4 * kScanRings * tiles);
    p.ring_base = reinterpret_cast<uint32_t*>(w);
    p.out = out;
    p.cap = cap;
    p.count = count;
    p.status = status;
    const unsigned g = (unsigned)tiles;
    scan_keep_kernel<<<g, kScanBlock, 0, s>>>(p);
    scan_tiles_kernel<<<1, 1024, 0, s>>>(p);
    scan_insert_kernel<<<g, kScanBlock, 0, s>>>(p);
    scan_winner_kernel<<<g, kScanBlock, 0, s>>>(p);
    scan_rings_kernel<<<kScanRings, kScanBlock, 0, s>>>(p);
    scan_write_kernel<<<g, kScanBlock, 0, s>>>(p);
    g_launches += 6;
    return check(cudaGetLastError());
}

}  // namespace tsdfl
