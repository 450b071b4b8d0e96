// Internal declarations shared by the host API and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "map_host.h"
#include "tsdfl.h"

namespace tsdfl {

// Slot codes: 0..599 = likelihood of |tsdf| in mm (map_util.h:124-127),
// 600 = init value (allocated slot never written), 601 = unallocated brick in
// the dense layout (a miss).
constexpr int kCodeInit = 600;
constexpr int kCodeMiss = 601;
constexpr int kCodeNone = 602;   // no point (padding): no hit, contributes 0
constexpr int kCodeLater = 603;  // scored later by the exact slow tiers: no hit, contributes 0 here
constexpr int kNumCodes = 604;
constexpr uint32_t kMissIndex = 0xffffffffu;

// Largest scan a single evaluation pass stages in shared memory (3 floats per
// point); longer scans are evaluated in several passes over point ranges.
constexpr int kMaxPassPoints = 16384;

// Fast-path bound on a map offset (metres): below it float->integer conversions
// are exact and cannot wrap.
constexpr float kFastOffsetLimit = 4194304.0f;


// Everything a kernel needs to look a point up in one map, passed by value
// (kernel parameters live in the constant bank).
struct MapView {
    float min_x, min_y, min_z;
    float res;
    float init_value;
    // fast path (non-negative offsets below kFastOffsetLimit)
    int32_t mmax_x, mmax_y, mmax_z;   // trunc(offset) passes the coarse bound check iff <= mmax
    uint32_t up_dim_x, up_dim_2, grid_occ_size;
    uint32_t sub_dim, sub_dim_2, sub_dim_3;
    uint32_t data_size;
    // full semantics (slow path)
    uint64_t dim_x, dim_y, dim_z;
    uint64_t up_dim_x64, up_dim_2_64, grid_occ_size64;
    uint64_t sub_dim64, sub_dim_2_64, data_size64;
    const int32_t* grid_occ;
    const uint16_t* codes;    // 16-bit slot codes (storage 0)
    const float* data;        // float slots (storage 1)
    const uint16_t* h16;      // half-precision slot values, IEEE bits (storage 2)
    const uint16_t* dense;    // non-null when the compact layout (occ) is built; equals codes
    int32_t storage;          // 0 = codes, 1 = float, 2 = half
    // Division-free sub-voxel index q = trunc(fl(s / res)) for s in [0, 1),
    // verified on the host (every threshold of q; monotone in s):
    // sub_fast = 2: q == floor(s * sub_inv) (exact product);
    // sub_fast = 1: q == trunc(fl(s * sub_inv + fl(s * sub_inv_lo))) (one FMA);
    // 0: neither (generic kernel).
    int32_t sub_fast;
    float sub_inv, sub_inv_lo;
    uint32_t lim_x, lim_y, lim_z;  // float bits of min(mmax + 1, 2^22) per axis
    // Code arrays: the reference's slots in its data order (bricks in linear
    // brick order, sub_dim^3 slots each, x fastest), preceded by one brick of
    // kCodeMiss -- what getIndex's wrapped 64-bit sum reads below slot 0 is a
    // miss -- and followed by kSentinels codes.  A brick of rank r (r allocated
    // bricks before it) starts at r * sub_dim^3, so a slot index is
    // r * sub_dim^3 + sub with sub in [-sub_dim^3, sub_dim^3).
    // Compact layout (TSDFL_MAP_DENSE): the brick's rank comes from a bitmap of
    // the brick grid staged in shared memory instead of a grid_occ gather.  occ
    // holds pairs {word w, allocated bricks in words 0..w}; bit (up & 31) of
    // word up >> 5 is set when brick up is allocated; the pairs are zero-padded
    // to occ_bytes (a power of two), so any index masked by occ_mask reads
    // inside the staged table.  rank = incl[w] - popc(word >> (up & 31)) for an
    // allocated brick.
    const uint32_t* occ;
    uint32_t occ_bytes;            // staged bytes (power of two), 0 without the compact layout
    uint32_t occ_mask;             // (occ_bytes - 1) & ~7
    // Sparse brick hash (TSDFL_MAP_HASH, or TSDFL_MAP_DENSE on maps whose bitmap
    // does not fit shared memory): {brick index, rank} of the allocated bricks
    // only, open addressing with linear probing from slot
    // (brick * 0x9E3779B1) >> hash_shift; empty slots hold kHashEmpty; every key
    // sits within hash_probes slots of its home and every run of keys ends
    // within that bound.
    const uint2* hash;
    uint32_t hash_mask, hash_shift, hash_probes;
    // Both code arrays end in kSentinels extra entries {kCodeMiss, kCodeLater,
    // kCodeNone, kCodeNone}: the fast path gathers a lookup that falls outside
    // the allocated slots from there, so every gather yields the final code.
    uint32_t codes_sent;           // index of the first sentinel in codes
    // Tiled fast path (eval_tiled_kernel, eval_batch_kernel), verified on the
    // host: brick indices below 2^23 and sub-voxel indices below sub_dim, so
    // that with float offsets o the packed pipeline forms
    //   bits(2^23 + trunc(ox) + trunc(oy) up_dim_x + trunc(|oz|) up_dim_2) = kMagic + brick
    //   bits(1.5 2^23 + qx + qy sub_dim +- qz sub_dim^2)                    = kMagic15 + sub
    // exactly (every term an integer below 2^22).  Gathers address
    // codes_b + 2 (r sub_dim^3 + bits(...)), codes_b = codes - 2 kMagic15 (bytes).
    int32_t tiled;                 // 1 when the conditions hold
    int32_t min0;                  // the map's min corner is (0, 0, 0): offsets are the coordinates
    float up_dim_x_f, up_dim_2_f, sub_dim_f, sub_dim_2_f;
    float zlo, zhi;                // fast z offsets: zlo < oz < zhi
    float neg_zero;                // -0.0f: the addend of exact products formed by FMA
    uint32_t upb_lim;              // kMagic + grid_occ_size
    uint32_t sent_miss, sent_later, sent_none;   // sentinels in the biased index
    unsigned long long codes_b;
    // Grid layout (TSDFL_MAP_GRID): the codes of every brick of the bounding
    // box in brick order, so no rank is needed.  Brick up starts at
    // (up + min(up, up_dim_2 - 1) + 1) sub_dim^3: a brick of the lowest layer
    // (up < up_dim_2) sits behind a skirt of sub_dim^3 codes holding what the
    // reference reads at its negative sub-voxel offsets (the tail of the
    // previous allocated brick, or misses), every other brick directly behind
    // its predecessor.  Unallocated bricks and skirts hold kCodeMiss; the
    // kSentinels codes follow the last brick.  Gathers address
    // grid_b + 2 ((up + min(up, grid_uxy1)) sub_dim^3 + bits(...)),
    // grid_b = grid + 2 (sub_dim^3 - kMagic15) (bytes); grid_b is 0 without it.
    unsigned long long grid_b;
    uint32_t grid_uxy1;            // up_dim_2 - 1
    uint32_t gsent_miss, gsent_later, gsent_none;   // sentinels in the grid's biased index
};

constexpr int kSentinels = 4;

// pose_prepare_kernel: blocks of kPoseThreads; in the pose blocks three lanes
// per particle, kPoseSlots particles a warp.
constexpr int kPoseThreads = 1024;
constexpr int kPoseSlots = 10;
constexpr int kPoseParticlesPerBlock = (kPoseThreads / 32) * kPoseSlots;
inline size_t pose_blocks(size_t P) { return (P + kPoseParticlesPerBlock - 1) / kPoseParticlesPerBlock; }
constexpr uint32_t kHashEmpty = 0xffffffffu;

#ifdef __CUDACC__

// float -> size_t as the reference's x86-64 build converts it (cvttss2si):
// in-range values truncate, negatives wrap modulo 2^64, out-of-range values give
// 2^63 (below 2^63) or 0 (at or above 2^64).
static __device__ __forceinline__ uint64_t f2u_x86(float v)
{
    const float two63 = 9223372036854775808.0f;
    if (v != v) return 0x8000000000000000ull;
    if (v < two63) {
        if (v >= -two63) return (uint64_t)__float2ll_rz(v);
        return 0x8000000000000000ull;
    }
    float w = __fsub_rn(v, two63);
    if (w < two63) return ((uint64_t)__float2ll_rz(w)) ^ 0x8000000000000000ull;
    return 0;
}

// CudaSubVoxelMap::getIndex (cuda_sub_voxel_map.tcc:50-137) with every
// conversion of the reference's x86-64 build: used for offsets the fast path
// does not cover.  Returns the slot index, or kMissIndex when it is not below
// data_size (getEntry then returns the init value, :139-157).
static __device__ __noinline__ uint32_t slot_index_slow(const MapView& m, float x, float y, float z)
{
    uint64_t gx = f2u_x86(__fsub_rn(x, m.min_x));
    uint64_t gy = f2u_x86(__fsub_rn(y, m.min_y));
    uint64_t gz = f2u_x86(__fsub_rn(z, m.min_z));
    gx = f2u_x86(__fdiv_rn(__ull2float_rn(gx), m.res));
    gy = f2u_x86(__fdiv_rn(__ull2float_rn(gy), m.res));
    gz = f2u_x86(__fdiv_rn(__ull2float_rn(gz), m.res));
    if (gx >= m.dim_x || gy >= m.dim_y || gz >= m.dim_z) return kMissIndex;
    float ox = __fsub_rn(x, m.min_x), oy = __fsub_rn(y, m.min_y), oz = __fsub_rn(z, m.min_z);
    uint64_t ux = f2u_x86(ox), uy = f2u_x86(oy), uz = f2u_x86(oz);
    float sx = __fsub_rn(ox, __ull2float_rn(ux));
    float sy = __fsub_rn(oy, __ull2float_rn(uy));
    float sz = __fsub_rn(oz, __ull2float_rn(uz));
    uint64_t up = ux + uy * m.up_dim_x64 + uz * m.up_dim_2_64;
    if (up >= m.grid_occ_size64) return kMissIndex;
    int32_t base = m.grid_occ[up];
    if (base < 0) return kMissIndex;
    uint64_t qx = f2u_x86(__fdiv_rn(sx, m.res));
    uint64_t qy = f2u_x86(__fdiv_rn(sy, m.res));
    uint64_t qz = f2u_x86(__fdiv_rn(sz, m.res));
    uint64_t idx = (uint64_t)(int64_t)base + qx + qy * m.sub_dim64 + qz * m.sub_dim_2_64;
    return idx < m.data_size64 ? (uint32_t)idx : kMissIndex;
}

// Transform of one scan point by a laser pose (tsdf_evaluator.cpp:44-46) with
// the reference's rounding order and no contraction into FMA.
static __device__ __forceinline__ void transform_point(const float* t, float x, float y, float z, float& tx, float& ty,
                                                float& tz)
{
    tx = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(t[0], x), __fmul_rn(t[1], y)), __fmul_rn(t[2], z)), t[3]);
    ty = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(t[4], x), __fmul_rn(t[5], y)), __fmul_rn(t[6], z)), t[7]);
    tz = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(t[8], x), __fmul_rn(t[9], y)), __fmul_rn(t[10], z)), t[11]);
}

#endif  // __CUDACC__

// Kernel launchers (kernels.cu)
struct EvalBuffers {
    const float* particles;  // P x 7
    const float* xs;         // N (padded to 4)
    const float* ys;
    const float* zs;
    const float* cs;         // per-point score constant (a_range*inv_max_range or a_max)
    float4* pxy;             // point pairs (x_a, x_b, y_a, y_b) per 64-point block, spatial order
    float2* pz;              // point pairs (z_a, z_b)
    int32_t* perm;           // scan index of each point of the pair layout
    float* pose12;           // P x 12 laser poses
    float* trig6;            // P x 6: sin/cos of roll, pitch, yaw
    long long* sum_fx;       // P: fixed-point likelihood sums
    float* raw;              // P: un-normalised weights
    uint32_t* hits;          // P
    uint32_t* nin;           // P: kept points within max_range (subsampled scans)
    long long* lut_fx;       // kNumCodes fixed-point likelihoods
    float* lut_f;            // kNumCodes float likelihoods
    int32_t* counts;         // [0] = points in range
    double* partials;        // reduction partials
    double* sums;            // [0] weight sum, [1..9] pose sums
    float* weight_sum_f;     // [1]
    int32_t* status;         // per-evaluation device status word
    uint32_t* dbg_index;     // optional P x N
    // Spread clouds (global localisation): the particles in spatial order --
    // counts[2] is set by the staging kernel when the cloud is spread, then
    // order[q] is the particle at position q of a Morton order of 64 x 64
    // cells over the cloud's x / y extent (cloud_ext).
    uint32_t* order;         // P
    uint32_t* pkeys;         // P: each particle's cell
    int32_t* phist;          // kCellBins: cell counts, then offsets
    float4* cloud_ext;       // [1]: min x, min y, max x, max y of the particles
};

// First kernel of an update: the particles' laser poses (tf: the sensor's
// 4 x 4 transform) beside the scan staging (pair layout in spatial order,
// likelihood tables, per-point constants); also clears the scoring sums.
int launch_pose_prepare(const float* tf, const float* particles, int P, const float* points, int N, int npad,
                        float max_range_sq, float c_in, float c_out, const float* code_values, int shift,
                        const EvalBuffers& b, cudaStream_t s);
// Runs after launch_pose_prepare: orders the particles of a spread cloud by
// cell (b.order); for a compact cloud its kernels return at once.
int launch_particle_order(const float* particles, int P, const EvalBuffers& b, cudaStream_t s);
size_t eval_smem_bytes(bool serial, int n);
// Scan points one pass of the tiled kernel stages (0: the kernel cannot hold
// this map's occupancy bitmap beside any points).
int tiled_pass_points(const MapView& m, bool dense);
// Warps per CTA of the tiled scoring kernel (one CTA per SM).
int tiled_warps_per_cta();
int launch_eval_pass(const MapView& m, float a_hit, int P, int n0, int n1, int n_total, bool first, bool serial,
                     bool dense, bool generic, const EvalBuffers& b, double* sum_f64, int sm_count, cudaStream_t s);
// nin: per-particle points within max_range when the particles scored
// different point subsets (n_points each), else null (the scan's count).
// log_domain: weights from ln raw - LSE in double (TSDFL_NORM_LOG).
// sticky: where the evaluation's device status is carried at its end (the
// context's or the filter's sticky word).
int launch_norm(int P, int mode, int shift, double a_hit, double c_in, double c_out, int n_points,
                const double* sum_f64, float* particles_out, float* pose_out, const EvalBuffers& b, cudaStream_t s,
                int32_t* sticky, const uint32_t* nin = nullptr, bool log_domain = false);
// Seeded per-particle subsampling (subsample.h): K of the N staged points per
// particle, exact fixed-point sums, hits and in-range counts into b.sum_fx,
// b.hits, b.nin.  Needs a map on the tiled path (TSDFL_ERR_UNSUPPORTED else).
int launch_eval_subsample(const MapView& m, float a_hit, int P, int N, int K, unsigned long long seed, float c_in,
                          const EvalBuffers& b, int sm_count, cudaStream_t s);

// Many filters' scoring in one persistent launch (eval_batch_kernel).  One
// segment per (filter, pass) of a filter whose map takes the tiled path.
struct BatchSegSpec {
    MapView m;
    float a_hit;
    int P, n0, n1, n_total;
    bool dense;
    EvalBuffers b;
};
// The segments of each map-layout kind (bit 2: min corner at the origin, bit 1:
// compact layout, bit 0: two-term sub-voxel multiplier) form one queue and one
// persistent launch.
struct BatchKinds {
    int first[8], count[8];
    uint32_t batches[8];
};
size_t batch_seg_bytes();
// Writes nseg segment records (nseg * batch_seg_bytes() bytes at host_out),
// grouped by kind, with work items of `chunk` points x `group` particles;
// returns the number of batches over all kinds.
uint32_t build_batch_segs(const BatchSegSpec* specs, int nseg, int chunk, int group, void* host_out,
                          BatchKinds* kinds);
int launch_eval_batch(const void* d_segs, const BatchKinds& kinds, uint32_t* counter, int32_t* status, int sm_count,
                      cudaStream_t s);
size_t resample_workspace_bytes(size_t M);
// u0p (optional): the draw read from device memory when the kernels run.
int launch_resample_impl(const float* particles, const float* w, int stride, size_t M, float u0, float* out,
                         uint32_t* idx_out, size_t cap, uint32_t* count_out, void* workspace, int32_t* status,
                         cudaStream_t s, const float* u0p = nullptr);
// ResidualSystematicResampler on the device; workspace: resample_workspace_bytes(M).
int launch_resample_residual(const float* particles, const float* w, int stride, size_t M, float u0, float* out,
                             uint32_t* idx_out, size_t cap, uint32_t* count_out, void* workspace, int32_t* status,
                             cudaStream_t s);
int launch_best_particle(const float* particles, size_t M, unsigned long long* key, uint32_t* index_out, int sm_count,
                         cudaStream_t s);
int launch_codes_from_floats(const float* data, size_t n, const float* code_values, float init_value,
                             uint16_t* codes, int32_t* fail, cudaStream_t s);
// Grid layout (MapView::grid_b): n = (grid_occ_size + up_dim_2) sub_dim_3 codes
// from the code array (with its leading miss brick) and the brick table.
int launch_grid_fill(const uint16_t* codes, const int32_t* grid_occ, uint64_t up_dim_2, uint64_t sub_dim_3,
                     uint64_t n, uint16_t* grid, cudaStream_t s);
// Half-precision slot values (round to nearest): from codes through the
// code -> value table, or from float slots when codes is null.
int launch_halves(const uint16_t* codes, const float* code_values, const float* data, size_t n, uint16_t* h16,
                  cudaStream_t s);

// Scan reduction of a PointCloud2 (scan.cu); workspace: scan_workspace_bytes(n).
size_t scan_workspace_bytes(size_t n);
int launch_reduce_scan(const uint8_t* cloud, size_t n, uint32_t step, uint32_t off_x, uint32_t off_ring, float cell,
                       bool own_ring, float* out, size_t cap, uint32_t* count, void* workspace, int32_t* status,
                       cudaStream_t s);

// Motion update (motion.cu): draws from the generator when draws is null.
int launch_motion(float* particles, size_t P, const double mean[6], const double stddev[6], uint64_t seed,
                  uint64_t step, const double* draws, double* draws_out, cudaStream_t s);

// Particles as geometry_msgs::Pose records (7 doubles each) (motion.cu).
int launch_pose_array(const float* particles, size_t P, double* poses, cudaStream_t s);

// The reference's other resamplers (resamplers.cu).  K: residual draws.
size_t resamplers_workspace_bytes(size_t M, size_t K);
int launch_resample_wheel(const float* particles, const float* w, int stride, size_t M, const double* draws,
                          uint64_t seed, float* out, uint32_t* idx_out, void* ws, cudaStream_t s);
int launch_resample_residual_random(const float* particles, const float* w, int stride, size_t M,
                                    const uint32_t* draws, size_t K, uint64_t seed, float* out, uint32_t* idx_out,
                                    void* ws, int32_t* status, cudaStream_t s);
int launch_resample_metropolis(const float* particles, const float* w, int stride, size_t M, uint32_t steps,
                               const float* u_draws, const uint32_t* j_draws, uint64_t seed, float* out,
                               uint32_t* idx_out, int32_t* status, cudaStream_t s);
int launch_resample_rejection(const float* particles, const float* w, int stride, size_t M, uint64_t seed,
                              uint32_t max_rounds, float* out, uint32_t* idx_out, void* ws, int32_t* status,
                              int sm_count, cudaStream_t s);

}  // namespace tsdfl
