// C ABI of the GB300 sensor update: contexts, maps, evaluation, resampling.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <mutex>
#include <new>
#include <algorithm>
#include <vector>
#include <unordered_map>
#include <deque>
#include <chrono>

#include "map_host.h"
#include "tsdfl.h"
#include "tsdfl_internal.h"
#include "subsample.h"

namespace tsdfl {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

}  // namespace tsdfl

using namespace tsdfl;

#define CUDA_TRY(expr)                                                                          \
    do {                                                                                        \
        cudaError_t _e = (expr);                                                                \
        if (_e != cudaSuccess) {                                                                \
            set_error("%s: %s (%s)", __func__, cudaGetErrorString(_e), #expr);                  \
            return _e == cudaErrorMemoryAllocation ? TSDFL_ERR_OUT_OF_MEMORY : TSDFL_ERR_DEVICE; \
        }                                                                                       \
    } while (0)

namespace {

constexpr int kSerialPassPoints = 8192;

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace

namespace tsdfl {
extern std::atomic<unsigned long long> g_launches;
}

struct tsdfl_ctx {
    bool timing = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool timed = false;
    int device = 0;
    int sm_count = 0;
    cudaStream_t own = nullptr;
    cudaStream_t stream = nullptr;
    size_t cap_P = 0, cap_N = 0;
    void* ws = nullptr;          // per-evaluation workspace
    size_t ws_bytes = 0;
    void* rs_ws = nullptr;       // resampling workspace
    size_t rs_bytes = 0;
    void* scan_ws = nullptr;     // scan reduction workspace
    size_t scan_bytes = 0;
    void* aux_ws = nullptr;      // workspace of the other resamplers
    size_t aux_bytes = 0;
    void* io = nullptr;          // device copies of host inputs (host API)
    size_t io_bytes = 0;
    int32_t* status = nullptr;   // [0] sticky status, [1] per-evaluation status
    int32_t* h_status = nullptr; // pinned
    float* h_pose = nullptr;     // pinned, 8 floats
    uint32_t* h_count = nullptr; // pinned
    EvalBuffers buf{};
    double* sum_f64 = nullptr;
};

struct tsdfl_map {
    int device = 0;
    tsdfl_map_coef coef{};
    MapView view{};
    int32_t* grid_occ = nullptr;
    uint16_t* codes = nullptr;    // the reference's slots (codes_base + miss brick)
    uint16_t* codes_base = nullptr;   // the allocation: one brick of kCodeMiss, the slots, the sentinels
    uint64_t codes_pre = 0;       // codes in front of the slots (sub_dim^3, or 0 for huge bricks)
    float* data = nullptr;
    uint16_t* h16 = nullptr;      // TSDFL_MAP_F16: half-precision slot values
    uint32_t* occ = nullptr;      // compact layout (TSDFL_MAP_DENSE): brick bitmap and prefix counts
    uint32_t occ_bytes = 0;
    uint2* hash = nullptr;        // sparse brick hash (TSDFL_MAP_HASH, or DENSE with a bitmap too large)
    uint16_t* grid = nullptr;     // grid layout (TSDFL_MAP_GRID): every brick of the bounding box
    uint64_t grid_codes = 0;      // codes in grid before the sentinels
    uint32_t hash_slots = 0, hash_probes = 0;
    float* values = nullptr;      // kNumCodes likelihood values (device)
    float max_value = 0;
    uint64_t bricks = 0;
    uint64_t bytes = 0;
};

namespace {

int set_device(int dev)
{
    CUDA_TRY(cudaSetDevice(dev));
    return TSDFL_OK;
}

// Layout of one evaluation's workspace for nP particles and nN points: the
// bytes it takes, and (base non-null) the buffers carved from base.
size_t eval_layout(size_t nP, size_t nN, char* base, EvalBuffers* e, double** sum_f64)
{
    if (nP < 1) nP = 1;
    if (nN < 4) nN = 4;
    size_t npad = align_up(nN, 4);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off = align_up(off + bytes, 256);
        return o;
    };
    size_t o_pose = take(sizeof(float) * 12 * nP);
    size_t o_trig = take(sizeof(float) * 6 * nP);
    size_t o_fx = take(sizeof(long long) * nP);
    size_t o_f64 = take(sizeof(double) * nP);
    size_t o_raw = take(sizeof(float) * nP);
    size_t o_hits = take(sizeof(uint32_t) * nP);
    size_t o_nin = take(sizeof(uint32_t) * nP);
    size_t o_xs = take(sizeof(float) * npad);
    size_t o_ys = take(sizeof(float) * npad);
    size_t o_zs = take(sizeof(float) * npad);
    size_t o_cs = take(sizeof(float) * npad);
    size_t npairs = 32 * ((nN + 63) / 64);
    size_t o_pxy = take(sizeof(float) * 4 * npairs);
    size_t o_pz = take(sizeof(float) * 2 * npairs);
    size_t o_perm = take(sizeof(int32_t) * 2 * npairs);
    size_t o_lfx = take(sizeof(long long) * kNumCodes);
    size_t o_lf = take(sizeof(float) * kNumCodes);
    size_t o_cnt = take(sizeof(int32_t) * 16);
    size_t o_part = take(sizeof(double) * 256 * 10);
    size_t o_sums = take(sizeof(double) * 16);
    size_t o_wsf = take(sizeof(float) * 4);
    size_t o_st = take(sizeof(int32_t) * 4);
    size_t o_ord = take(sizeof(uint32_t) * nP);
    size_t o_pk = take(sizeof(uint32_t) * nP);
    size_t o_ph = take(sizeof(int32_t) * 4096);
    size_t o_ce = take(sizeof(float) * 4);
    if (base) {
        char* b = base;
        e->pose12 = reinterpret_cast<float*>(b + o_pose);
        e->trig6 = reinterpret_cast<float*>(b + o_trig);
        e->sum_fx = reinterpret_cast<long long*>(b + o_fx);
        *sum_f64 = reinterpret_cast<double*>(b + o_f64);
        e->raw = reinterpret_cast<float*>(b + o_raw);
        e->hits = reinterpret_cast<uint32_t*>(b + o_hits);
        e->nin = reinterpret_cast<uint32_t*>(b + o_nin);
        e->xs = reinterpret_cast<float*>(b + o_xs);
        e->ys = reinterpret_cast<float*>(b + o_ys);
        e->zs = reinterpret_cast<float*>(b + o_zs);
        e->cs = reinterpret_cast<float*>(b + o_cs);
        e->pxy = reinterpret_cast<float4*>(b + o_pxy);
        e->pz = reinterpret_cast<float2*>(b + o_pz);
        e->perm = reinterpret_cast<int32_t*>(b + o_perm);
        e->lut_fx = reinterpret_cast<long long*>(b + o_lfx);
        e->lut_f = reinterpret_cast<float*>(b + o_lf);
        e->counts = reinterpret_cast<int32_t*>(b + o_cnt);
        e->partials = reinterpret_cast<double*>(b + o_part);
        e->sums = reinterpret_cast<double*>(b + o_sums);
        e->weight_sum_f = reinterpret_cast<float*>(b + o_wsf);
        e->status = reinterpret_cast<int32_t*>(b + o_st);
        e->order = reinterpret_cast<uint32_t*>(b + o_ord);
        e->pkeys = reinterpret_cast<uint32_t*>(b + o_pk);
        e->phist = reinterpret_cast<int32_t*>(b + o_ph);
        e->cloud_ext = reinterpret_cast<float4*>(b + o_ce);
    }
    return off;
}

// Carves the per-evaluation workspace for P particles and N points.
int ensure_workspace(tsdfl_ctx* c, size_t P, size_t N)
{
    if (P <= c->cap_P && N <= c->cap_N && c->ws) return TSDFL_OK;
    // grow by at least a quarter, so that counts that drift upwards (the
    // systematic resampler's) do not reallocate on every new maximum
    size_t nP = P > c->cap_P ? std::max(P, c->cap_P + c->cap_P / 4) : c->cap_P;
    size_t nN = N > c->cap_N ? std::max(N, c->cap_N + c->cap_N / 4) : c->cap_N;
    if (nP < 1) nP = 1;
    if (nN < 4) nN = 4;
    size_t total = eval_layout(nP, nN, nullptr, nullptr, nullptr);
    void* ws = nullptr;
    CUDA_TRY(cudaMalloc(&ws, total));
    if (c->ws) cudaFree(c->ws);
    c->ws = ws;
    c->ws_bytes = total;
    eval_layout(nP, nN, static_cast<char*>(ws), &c->buf, &c->sum_f64);
    c->buf.status = c->status + 1;
    c->cap_P = nP;
    c->cap_N = nN;
    return TSDFL_OK;
}

int ensure_resample_ws(tsdfl_ctx* c, size_t M)
{
    size_t need = resample_workspace_bytes(M);
    if (need <= c->rs_bytes) return TSDFL_OK;
    need = std::max(need, c->rs_bytes + c->rs_bytes / 4);
    void* p = nullptr;
    CUDA_TRY(cudaMalloc(&p, need));
    if (c->rs_ws) cudaFree(c->rs_ws);
    c->rs_ws = p;
    c->rs_bytes = need;
    return TSDFL_OK;
}

int ensure_scan_ws(tsdfl_ctx* c, size_t n)
{
    size_t need = scan_workspace_bytes(n);
    if (need <= c->scan_bytes) return TSDFL_OK;
    void* p = nullptr;
    CUDA_TRY(cudaMalloc(&p, need));
    if (c->scan_ws) cudaFree(c->scan_ws);
    c->scan_ws = p;
    c->scan_bytes = need;
    return TSDFL_OK;
}

int ensure_aux_ws(tsdfl_ctx* c, size_t need)
{
    if (need <= c->aux_bytes) return TSDFL_OK;
    void* p = nullptr;
    CUDA_TRY(cudaMalloc(&p, need));
    if (c->aux_ws) cudaFree(c->aux_ws);
    c->aux_ws = p;
    c->aux_bytes = need;
    return TSDFL_OK;
}

// Arguments of the scan reduction (tsdfl_reduce_scan*).
int check_scan_args(const char* fn, size_t n, uint32_t step, uint32_t x_offset, uint32_t ring_offset, float cell,
                    uint32_t flags)
{
    if (n >= (1ull << 31)) {
        set_error("%s: at most 2^31-1 cloud points", fn);
        return TSDFL_ERR_UNSUPPORTED;
    }
    if ((uint64_t)x_offset + 12 > step || (uint64_t)ring_offset + 2 > step) {
        set_error("%s: x, y, z (12 bytes at x_offset) and ring (2 bytes) must lie inside point_step", fn);
        return TSDFL_ERR_INVALID_ARG;
    }
    if (!(cell > 0.0f) || !std::isfinite(cell)) {
        set_error("%s: cell must be positive and finite", fn);
        return TSDFL_ERR_INVALID_ARG;
    }
    if (flags & ~TSDFL_SCAN_OWN_RING) {
        set_error("%s: unknown flags", fn);
        return TSDFL_ERR_INVALID_ARG;
    }
    return TSDFL_OK;
}

int ensure_io(tsdfl_ctx* c, size_t bytes)
{
    if (bytes <= c->io_bytes) return TSDFL_OK;
    bytes = std::max(bytes, c->io_bytes + c->io_bytes / 4);
    void* p = nullptr;
    CUDA_TRY(cudaMalloc(&p, bytes));
    if (c->io) cudaFree(c->io);
    c->io = p;
    c->io_bytes = bytes;
    return TSDFL_OK;
}

int validate_coef(const tsdfl_map_coef* c)
{
    if (!c) return TSDFL_ERR_INVALID_ARG;
    if (!(c->resolution > 0.0f) || !std::isfinite(c->resolution)) {
        set_error("map: resolution must be positive");
        return TSDFL_ERR_INVALID_ARG;
    }
    if (c->grid_occ_size != c->up_dim_x * c->up_dim_y * c->up_dim_z || c->up_dim_2 != c->up_dim_x * c->up_dim_y ||
        c->sub_dim_2 != c->sub_dim * c->sub_dim) {
        set_error("map: inconsistent coefficients");
        return TSDFL_ERR_INVALID_ARG;
    }
    const uint64_t sub3 = c->sub_dim * c->sub_dim * c->sub_dim;
    if (c->grid_occ_size >= (1ull << 31) || c->data_size + 4 * sub3 >= (1ull << 31) || c->sub_dim > 1024 ||
        c->up_dim_x >= (1u << 22) || c->up_dim_y >= (1u << 22) || c->up_dim_z >= (1u << 22)) {
        set_error("map: too large for 32-bit slot indices");
        return TSDFL_ERR_UNSUPPORTED;
    }
    return TSDFL_OK;
}

// The kSentinels codes after the last slot of a code array (MapView::codes_sent).
cudaError_t write_sentinels(uint16_t* arr, size_t at, cudaStream_t s)
{
    static const uint16_t kSent[kSentinels] = {(uint16_t)kCodeMiss, (uint16_t)kCodeLater, (uint16_t)kCodeNone,
                                               (uint16_t)kCodeNone};
    return cudaMemcpyAsync(arr + at, kSent, sizeof(kSent), cudaMemcpyHostToDevice, s);
}

// The code array of a map: one brick of kCodeMiss in front of the n slots (what
// a slot index below 0 reads: getIndex's wrapped 64-bit sum is a miss there),
// the sentinels behind them.  Sets m->codes_base, m->codes_pre and m->codes.
cudaError_t alloc_codes(tsdfl_map* m, size_t n, cudaStream_t s)
{
    const uint64_t S3 = m->coef.sub_dim * m->coef.sub_dim_2;
    const uint64_t pre = S3 <= (1ull << 21) ? S3 : 0;
    cudaError_t e = cudaMalloc(&m->codes_base, sizeof(uint16_t) * (pre + n + kSentinels));
    if (e != cudaSuccess) {
        m->codes_base = nullptr;
        return e;
    }
    m->codes_pre = pre;
    m->codes = m->codes_base + pre;
    if (pre) {
        std::vector<uint16_t> miss(pre, (uint16_t)kCodeMiss);
        e = cudaMemcpy(m->codes_base, miss.data(), sizeof(uint16_t) * pre, cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = write_sentinels(m->codes, n, s);
    return e;
}

void free_codes(tsdfl_map* m)
{
    cudaFree(m->codes_base);
    m->codes_base = nullptr;
    m->codes = nullptr;
    m->codes_pre = 0;
}

// Largest sub-voxel index trunc(fl(s / res)) over floats s in [0, 1).
uint64_t max_sub_index(float res)
{
    float below_one;
    const uint32_t b = 0x3F7FFFFFu;
    std::memcpy(&below_one, &b, 4);
    return f2u_x86_host(below_one / res);
}

void fill_view(tsdfl_map* m)
{
    const tsdfl_map_coef& c = m->coef;
    MapView& v = m->view;
    v.min_x = c.min_x; v.min_y = c.min_y; v.min_z = c.min_z;
    v.res = c.resolution;
    v.init_value = c.init_value;
    v.mmax_x = coarse_mmax(c.dim_x, c.resolution);
    v.mmax_y = coarse_mmax(c.dim_y, c.resolution);
    v.mmax_z = coarse_mmax(c.dim_z, c.resolution);
    v.up_dim_x = (uint32_t)c.up_dim_x;
    v.up_dim_2 = (uint32_t)c.up_dim_2;
    v.grid_occ_size = (uint32_t)c.grid_occ_size;
    v.sub_dim = (uint32_t)c.sub_dim;
    v.sub_dim_2 = (uint32_t)c.sub_dim_2;
    v.sub_dim_3 = (uint32_t)(c.sub_dim * c.sub_dim_2);
    v.data_size = (uint32_t)c.data_size;
    v.dim_x = c.dim_x; v.dim_y = c.dim_y; v.dim_z = c.dim_z;
    v.up_dim_x64 = c.up_dim_x;
    v.up_dim_2_64 = c.up_dim_2;
    v.grid_occ_size64 = c.grid_occ_size;
    v.sub_dim64 = c.sub_dim;
    v.sub_dim_2_64 = c.sub_dim_2;
    v.data_size64 = c.data_size;
    v.grid_occ = m->grid_occ;
    v.codes = m->codes;
    v.data = m->data;
    v.h16 = m->h16;
    v.dense = m->occ ? m->codes : nullptr;
    v.storage = m->h16 ? 2 : (m->codes ? 0 : 1);
    v.sub_fast = sub_index_mult(c.resolution, c.sub_dim, &v.sub_inv, &v.sub_inv_lo);
    auto lim = [](int32_t mmax) {
        float f = (float)std::min<int64_t>((int64_t)mmax + 1, 4194304);
        if (mmax < 0) f = 0.0f;
        uint32_t b;
        std::memcpy(&b, &f, 4);
        return b;
    };
    v.lim_x = lim(v.mmax_x);
    v.lim_y = lim(v.mmax_y);
    v.lim_z = lim(v.mmax_z);
    v.occ = m->occ;
    v.occ_bytes = m->occ_bytes;
    v.occ_mask = m->occ_bytes ? (m->occ_bytes - 1u) & ~7u : 0u;
    v.hash = m->hash;
    v.hash_mask = m->hash_slots ? m->hash_slots - 1u : 0u;
    v.hash_shift = 32u;
    for (uint32_t sz = m->hash_slots; sz > 1u; sz >>= 1) v.hash_shift -= 1u;
    v.hash_probes = m->hash_probes;
    v.codes_sent = (uint32_t)c.data_size;
    // tiled fast path: the packed pipeline's float sums are exact integers
    // (largest brick index a fast lookup forms below 2^23, sub-voxel offsets
    // within +-sub_dim^3 <= 2^21) and every sub-voxel index stays inside its
    // brick, so slot indices land in [r S^3 - S^3, r S^3 + S^3)
    const uint64_t S3 = c.sub_dim * c.sub_dim_2;
    auto fmax_trunc = [&](int32_t mmax) { return mmax < 0 ? 0ull : (uint64_t)std::min<int64_t>(mmax, 4194303); };
    const uint64_t up_max = fmax_trunc(v.mmax_x) + fmax_trunc(v.mmax_y) * c.up_dim_x + fmax_trunc(v.mmax_z) * c.up_dim_2;
    v.tiled = v.sub_fast != 0 && m->codes != nullptr && m->codes_pre == S3 && S3 <= (1ull << 21) && up_max < (1ull << 23) &&
              c.grid_occ_size < (1ull << 23) && max_sub_index(c.resolution) < c.sub_dim ? 1 : 0;
    v.min0 = c.min_x == 0.0f && c.min_y == 0.0f && c.min_z == 0.0f && !std::signbit(c.min_x) &&
             !std::signbit(c.min_y) && !std::signbit(c.min_z) ? 1 : 0;
    v.up_dim_x_f = (float)c.up_dim_x;
    v.up_dim_2_f = (float)c.up_dim_2;
    v.sub_dim_f = (float)c.sub_dim;
    v.sub_dim_2_f = (float)c.sub_dim_2;
    // -1 < oz < mmax_z + 1: points just below the map take brick layer 0 and a
    // negative sub-voxel index (an empty range when not even layer 0 passes)
    v.zhi = v.mmax_z < 0 ? 0.0f : (float)std::min<int64_t>((int64_t)v.mmax_z + 1, 4194304);
    v.zlo = v.mmax_z < 0 ? 0.0f : -1.0f;
    v.neg_zero = -0.0f;
    const uint32_t kMag = 0x4B000000u, kMag15 = 0x4B400000u;
    v.upb_lim = kMag + (uint32_t)std::min<uint64_t>(c.grid_occ_size, 1ull << 23);
    v.sent_miss = (uint32_t)c.data_size + kMag15;
    v.sent_later = v.sent_miss + 1u;
    v.sent_none = v.sent_miss + 2u;
    v.codes_b = (unsigned long long)(uintptr_t)m->codes - 2ull * kMag15;
    v.grid_uxy1 = c.up_dim_2 ? (uint32_t)(c.up_dim_2 - 1) : 0u;
    v.grid_b = 0;
    v.gsent_miss = v.gsent_later = v.gsent_none = 0;
    if (m->grid) {
        v.grid_b = (unsigned long long)(uintptr_t)m->grid + 2ull * S3 - 2ull * kMag15;
        v.gsent_miss = (uint32_t)(m->grid_codes - S3) + kMag15;
        v.gsent_later = v.gsent_miss + 1u;
        v.gsent_none = v.gsent_miss + 2u;
    }
}



// Grid layout (TSDFL_MAP_GRID): the codes of every brick of the bounding box,
// so the tiled kernel addresses a slot by the brick index alone.  A lookup
// with a negative sub-voxel offset (oz in (-1, 0), the lowest layer only) reads
// the skirt in front of its brick, which holds what the reference's index
// reads there: the tail of the previous allocated brick.  Built under the
// compact layout's conditions; the biased 32-bit index must stay below 2^32,
// which the 2^31-code limit leaves room for.
int build_grid(tsdfl_map* m, cudaStream_t s)
{
    const tsdfl_map_coef& c = m->coef;
    const uint64_t S3 = c.sub_dim * c.sub_dim_2;
    if (max_sub_index(c.resolution) >= c.sub_dim || !m->codes || m->codes_pre != S3 || c.grid_occ_size == 0 ||
        c.grid_occ_size >= (1ull << 23))
        return TSDFL_OK;
    const uint64_t n = (c.grid_occ_size + c.up_dim_2) * S3;
    if (n >= (1ull << 31)) return TSDFL_OK;
    CUDA_TRY(cudaMalloc(&m->grid, sizeof(uint16_t) * (n + kSentinels)));
    int rc = launch_grid_fill(m->codes, m->grid_occ, c.up_dim_2, S3, n, m->grid, s);
    if (rc) return rc;
    CUDA_TRY(write_sentinels(m->grid, n, s));
    m->grid_codes = n;
    m->bytes += sizeof(uint16_t) * (n + kSentinels);
    return TSDFL_OK;
}

// Compact layout (TSDFL_MAP_DENSE): the code array itself, with the brick's
// rank read from a bitmap of the brick grid staged in shared memory instead of
// a grid_occ gather.  Built when every sub-voxel index stays inside its brick
// and the bitmap (pairs {word, allocated bricks up to and including it},
// zero-padded to a power of two) fits the tiled kernels' staging.
int build_compact(tsdfl_map* m, const int32_t* go)
{
    const tsdfl_map_coef& c = m->coef;
    const uint64_t gos = c.grid_occ_size;
    if (max_sub_index(c.resolution) >= c.sub_dim || !m->codes || m->codes_pre != c.sub_dim * c.sub_dim_2)
        return TSDFL_OK;   // brick table only
    const uint64_t words = (gos + 31) / 32;
    uint64_t bytes = 16;
    while (bytes < 8 * words) bytes *= 2;
    if (bytes > (1u << 17)) return TSDFL_OK;
    std::vector<uint32_t> occ(bytes / 4, 0u);
    for (uint64_t up = 0; up < gos; ++up)
        if (go[up] >= 0) occ[2 * (up / 32)] |= 1u << (up % 32);
    uint32_t run = 0;
    for (uint64_t w = 0; w < words; ++w) {
        run += (uint32_t)__builtin_popcount(occ[2 * w]);
        occ[2 * w + 1] = run;
    }
    CUDA_TRY(cudaMalloc(&m->occ, bytes));
    CUDA_TRY(cudaMemcpy(m->occ, occ.data(), bytes, cudaMemcpyHostToDevice));
    m->occ_bytes = (uint32_t)bytes;
    m->bytes += bytes;
    return TSDFL_OK;
}

// Sparse brick hash: {brick index, rank} of every allocated brick in a table
// of 2^k >= 2n slots, linear probing from (brick * 0x9E3779B1) >> (32 - k).
// hash_probes bounds both a key's distance from its home and the run a miss
// walks to the empty slot that ends it.
int build_hash(tsdfl_map* m, const int32_t* go)
{
    const tsdfl_map_coef& c = m->coef;
    if (!m->codes || m->codes_pre != c.sub_dim * c.sub_dim_2) return TSDFL_OK;
    uint64_t n = 0;
    for (uint64_t up = 0; up < c.grid_occ_size; ++up) n += go[up] >= 0 ? 1 : 0;
    uint32_t k = 4;
    while ((1ull << k) < 2 * n) ++k;
    if (k > 30) return TSDFL_OK;
    const uint32_t slots = 1u << k, mask = slots - 1u;
    std::vector<uint2> table(slots, make_uint2(kHashEmpty, 0u));
    uint32_t longest = 0, rank = 0;
    for (uint64_t up = 0; up < c.grid_occ_size; ++up) {
        if (go[up] < 0) continue;
        const uint32_t key = (uint32_t)up;
        const uint32_t h = (uint32_t)(key * 0x9E3779B1u) >> (32 - k);
        uint32_t t = 0;
        while (table[(h + t) & mask].x != kHashEmpty) ++t;
        table[(h + t) & mask] = make_uint2(key, rank++);
        longest = std::max(longest, t);
    }
    uint32_t run = 0, longest_run = 0;   // occupied slots in a row, around the wrap
    for (uint32_t i = 0; i < 2 * slots; ++i) {
        run = table[i & mask].x == kHashEmpty ? 0 : run + 1;
        longest_run = std::max(longest_run, run);
    }
    CUDA_TRY(cudaMalloc(&m->hash, sizeof(uint2) * slots));
    CUDA_TRY(cudaMemcpy(m->hash, table.data(), sizeof(uint2) * slots, cudaMemcpyHostToDevice));
    m->hash_slots = slots;
    m->hash_probes = std::max(longest, longest_run) + 1;
    m->bytes += sizeof(uint2) * slots;
    return TSDFL_OK;
}

// grid_occ: the caller's brick table (host)
int finish_map(tsdfl_ctx* ctx, tsdfl_map* m, const int32_t* grid_occ, uint32_t flags)
{
    if (flags & TSDFL_MAP_F16) {   // half-precision values replace the codes or float slots
        const size_t n = m->coef.data_size;
        CUDA_TRY(cudaMalloc(&m->h16, sizeof(uint16_t) * (n ? n : 1)));
        int rc = launch_halves(m->codes, m->values, m->data, n, m->h16, ctx->stream);
        if (rc) return rc;
        CUDA_TRY(cudaStreamSynchronize(ctx->stream));
        m->bytes -= m->codes ? sizeof(uint16_t) * (m->codes_pre + n) : sizeof(float) * n;
        m->bytes += sizeof(uint16_t) * n;
        free_codes(m);
        cudaFree(m->data);
        m->data = nullptr;
        fill_view(m);
        return TSDFL_OK;
    }
    if ((flags & TSDFL_MAP_GRID) && m->codes) {
        int rc = build_grid(m, ctx->stream);
        if (rc) return rc;
    }
    if ((flags & TSDFL_MAP_HASH) && m->codes) {
        int rc = build_hash(m, grid_occ);
        if (rc) return rc;
    } else if ((flags & TSDFL_MAP_DENSE) && m->codes) {
        int rc = build_compact(m, grid_occ);
        if (rc) return rc;
        if (!m->occ) {   // the bitmap does not fit shared memory: index the bricks in a hash
            rc = build_hash(m, grid_occ);
            if (rc) return rc;
        }
    }
    fill_view(m);
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return TSDFL_OK;
}

void destroy_map(tsdfl_map* m)
{
    if (!m) return;
    cudaSetDevice(m->device);
    cudaFree(m->grid_occ);
    cudaFree(m->codes_base);
    cudaFree(m->data);
    cudaFree(m->h16);
    cudaFree(m->occ);
    cudaFree(m->hash);
    cudaFree(m->grid);
    cudaFree(m->values);
    delete m;
}

// Map allocations shared by both create entry points.
int map_common(tsdfl_ctx* ctx, const tsdfl_map_coef* coef, const int32_t* grid_occ, float sigma, tsdfl_map* m)
{
    m->device = ctx->device;
    m->coef = *coef;
    float vals[kNumCodes];
    code_values(sigma, coef->init_value, vals);
    m->max_value = 0;
    for (int k = 0; k < kNumCodes; ++k) m->max_value = std::fmax(m->max_value, std::fabs(vals[k]));
    CUDA_TRY(cudaMalloc(&m->values, sizeof(vals)));
    CUDA_TRY(cudaMemcpyAsync(m->values, vals, sizeof(vals), cudaMemcpyHostToDevice, ctx->stream));
    size_t go = sizeof(int32_t) * (coef->grid_occ_size ? coef->grid_occ_size : 1);
    CUDA_TRY(cudaMalloc(&m->grid_occ, go));
    if (coef->grid_occ_size)
        CUDA_TRY(cudaMemcpyAsync(m->grid_occ, grid_occ, sizeof(int32_t) * coef->grid_occ_size,
                                 cudaMemcpyHostToDevice, ctx->stream));
    m->bytes = sizeof(vals) + go;
    m->bricks = 0;
    for (uint64_t i = 0; i < coef->grid_occ_size; ++i) m->bricks += grid_occ[i] >= 0;
    return TSDFL_OK;
}

int run_eval(tsdfl_ctx* c, const tsdfl_map* map, const tsdfl_model* mdl, float* d_particles, size_t P,
             const float* d_points, size_t N, const float tf[16], uint32_t flags, float* d_pose, uint32_t* d_dbg)
{
    int rc = ensure_workspace(c, P, N);
    if (rc) return rc;
    EvalBuffers b = c->buf;
    b.particles = d_particles;
    b.dbg_index = d_dbg;
    const bool serial = (flags & TSDFL_SUM_SERIAL) != 0;
    if (serial && map->view.storage == 2) {
        set_error("evaluate: serial sums need code or float slots (the map holds half-precision values)");
        return TSDFL_ERR_UNSUPPORTED;
    }
    const float inv_max_range = (float)(1.0 / (double)mdl->max_range);
    const float max_range_sq = mdl->max_range * mdl->max_range;
    const float c_in = mdl->a_range * inv_max_range;
    const float c_out = mdl->a_max;
    // fixed-point scale: sums of N values below max_value stay below 2^62
    int shift = 40;
    {
        double bound = std::fmax((double)map->max_value, 1e-30) * (double)(N + 1);
        int need = (int)std::ceil(std::log2(bound));
        if (62 - need < shift) shift = 62 - need;
    }
    const int npad = (int)align_up(N, 4);
    cudaStream_t s = c->stream;
    rc = launch_pose_prepare(tf, d_particles, (int)P, d_points, (int)N, npad, max_range_sq, c_in, c_out, map->values,
                             shift, b, s);
    if (rc) return rc;
    rc = launch_particle_order(d_particles, (int)P, b, s);
    if (rc) return rc;
    const bool tiled = !serial && map->view.storage == 0 && map->view.tiled && !(flags & TSDFL_EVAL_GENERIC);
    bool dense = map->occ != nullptr && !(tiled && map->grid);   // the grid layout needs no bitmap
    size_t pass = serial ? kSerialPassPoints : (size_t)kMaxPassPoints;
    if (tiled) {
        int tp = tiled_pass_points(map->view, dense);
        if (tp < 1024 && dense) {   // the rank tables crowd out the scan: use the brick table instead
            dense = false;
            tp = tiled_pass_points(map->view, false);
        }
        pass = (size_t)tp;
    }
    if (c->timing) CUDA_TRY(cudaEventRecord(c->ev0, s));
    for (size_t n0 = 0; n0 < N; n0 += pass) {
        size_t n1 = n0 + pass < N ? n0 + pass : N;
        rc = launch_eval_pass(map->view, mdl->a_hit, (int)P, (int)n0, (int)n1, (int)N, n0 == 0, serial,
                              dense && !serial, (flags & TSDFL_EVAL_GENERIC) != 0, b, c->sum_f64, c->sm_count, s);
        if (rc) return rc;
    }
    if (c->timing) {
        CUDA_TRY(cudaEventRecord(c->ev1, s));
        c->timed = true;
    }
    const int mode = serial ? 2 : (map->view.storage != 0 ? 1 : 0);
    return launch_norm((int)P, mode, shift, (double)mdl->a_hit, (double)c_in, (double)c_out, (int)N, c->sum_f64,
                       d_particles, d_pose, b, s, c->status, nullptr, (flags & TSDFL_NORM_LOG) != 0);
}

// Seeded per-particle subsampling: K of the N points per particle
// (subsample.h), exact fixed-point sums, per-particle range terms.
int run_eval_sub(tsdfl_ctx* c, const tsdfl_map* map, const tsdfl_model* mdl, float* d_particles, size_t P,
                 const float* d_points, size_t N, const float tf[16], size_t K, uint64_t seed, float* d_pose)
{
    if (!map->view.tiled || map->view.storage != 0) {
        set_error("tsdfl_evaluate_subsampled: the map has no tiled fast path (float slots or an unsupported "
                  "resolution)");
        return TSDFL_ERR_UNSUPPORTED;
    }
    int rc = ensure_workspace(c, P, N);
    if (rc) return rc;
    EvalBuffers b = c->buf;
    b.particles = d_particles;
    b.dbg_index = nullptr;
    const float inv_max_range = (float)(1.0 / (double)mdl->max_range);
    const float max_range_sq = mdl->max_range * mdl->max_range;
    const float c_in = mdl->a_range * inv_max_range;
    const float c_out = mdl->a_max;
    int shift = 40;
    {
        double bound = std::fmax((double)map->max_value, 1e-30) * (double)(K + 1);
        int need = (int)std::ceil(std::log2(bound));
        if (62 - need < shift) shift = 62 - need;
    }
    const int npad = (int)align_up(N, 4);
    cudaStream_t s = c->stream;
    rc = launch_pose_prepare(tf, d_particles, (int)P, d_points, (int)N, npad, max_range_sq, c_in, c_out, map->values,
                             shift, b, s);
    if (rc) return rc;
    rc = launch_particle_order(d_particles, (int)P, b, s);
    if (rc) return rc;
    if (c->timing) CUDA_TRY(cudaEventRecord(c->ev0, s));
    rc = launch_eval_subsample(map->view, mdl->a_hit, (int)P, (int)N, (int)K, seed, c_in, b, c->sm_count, s);
    if (rc) return rc;
    if (c->timing) {
        CUDA_TRY(cudaEventRecord(c->ev1, s));
        c->timed = true;
    }
    return launch_norm((int)P, 0, shift, (double)mdl->a_hit, (double)c_in, (double)c_out, (int)K, c->sum_f64,
                       d_particles, d_pose, b, s, c->status, b.nin);
}

int check_sub_args(const char* fn, size_t P, size_t N, size_t K)
{
    if (K == 0 || K > N) {
        set_error("%s: need 0 < K <= N (K = %zu, N = %zu)", fn, K, N);
        return TSDFL_ERR_INVALID_ARG;
    }
    if (P >= (1ull << 31) || N >= (1ull << 31)) {
        set_error("%s: too many particles or points", fn);
        return TSDFL_ERR_UNSUPPORTED;
    }
    return TSDFL_OK;
}

int check_model(const tsdfl_model* mdl)
{
    if (!mdl || !(mdl->max_range > 0.0f)) {
        set_error("model: max_range must be positive");
        return TSDFL_ERR_INVALID_ARG;
    }
    return TSDFL_OK;
}

}  // namespace

extern "C" {

const char* tsdfl_last_error(void) { return g_err; }
const char* tsdfl_version(void) { return "tsdfl 0.1 (sm_103a)"; }

int tsdfl_ctx_create(int device, tsdfl_ctx** out)
{
    if (!out) return TSDFL_ERR_INVALID_ARG;
    *out = nullptr;
    int rc = set_device(device);
    if (rc) return rc;
    auto* c = new (std::nothrow) tsdfl_ctx;
    if (!c) return TSDFL_ERR_OUT_OF_MEMORY;
    c->device = device;
    cudaError_t e = cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&c->status, sizeof(int32_t) * 4);
    if (e == cudaSuccess) e = cudaMemset(c->status, 0, sizeof(int32_t) * 4);
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_status, sizeof(int32_t) * 4);
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_pose, sizeof(float) * 8);
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_count, sizeof(uint32_t) * 4);
    if (e != cudaSuccess) {
        set_error("tsdfl_ctx_create: %s", cudaGetErrorString(e));
        tsdfl_ctx_destroy(c);
        return e == cudaErrorMemoryAllocation ? TSDFL_ERR_OUT_OF_MEMORY : TSDFL_ERR_DEVICE;
    }
    c->stream = c->own;
    *out = c;
    return TSDFL_OK;
}

int tsdfl_ctx_destroy(tsdfl_ctx* c)
{
    if (!c) return TSDFL_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    cudaFree(c->ws);
    cudaFree(c->rs_ws);
    cudaFree(c->scan_ws);
    cudaFree(c->aux_ws);
    cudaFree(c->io);
    cudaFree(c->status);
    cudaFreeHost(c->h_status);
    cudaFreeHost(c->h_pose);
    cudaFreeHost(c->h_count);
    if (c->own) cudaStreamDestroy(c->own);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    delete c;
    return TSDFL_OK;
}

int tsdfl_ctx_set_stream(tsdfl_ctx* c, void* stream)
{
    if (!c) return TSDFL_ERR_INVALID_ARG;
    c->stream = stream ? static_cast<cudaStream_t>(stream) : c->own;
    return TSDFL_OK;
}

void* tsdfl_ctx_stream(tsdfl_ctx* c) { return c ? (void*)c->stream : nullptr; }

int tsdfl_ctx_set_timing(tsdfl_ctx* c, int enable)
{
    if (!c) return TSDFL_ERR_INVALID_ARG;
    int rc = set_device(c->device);
    if (rc) return rc;
    if (enable && !c->ev0) {
        CUDA_TRY(cudaEventCreate(&c->ev0));
        CUDA_TRY(cudaEventCreate(&c->ev1));
    }
    c->timing = enable != 0;
    c->timed = false;
    return TSDFL_OK;
}

int tsdfl_ctx_last_timing(tsdfl_ctx* c, float* eval_kernel_ms)
{
    if (!c || !eval_kernel_ms) return TSDFL_ERR_INVALID_ARG;
    if (!c->timed) {
        set_error("tsdfl_ctx_last_timing: no timed evaluation");
        return TSDFL_ERR_INVALID_ARG;
    }
    CUDA_TRY(cudaEventSynchronize(c->ev1));
    CUDA_TRY(cudaEventElapsedTime(eval_kernel_ms, c->ev0, c->ev1));
    return TSDFL_OK;
}

uint64_t tsdfl_launch_count(void) { return (uint64_t)g_launches.load(); }

int tsdfl_ctx_workspace_bytes(const tsdfl_ctx* c, size_t* eval_bytes, size_t* resample_bytes)
{
    if (!c) return TSDFL_ERR_INVALID_ARG;
    if (eval_bytes) *eval_bytes = c->ws_bytes;
    if (resample_bytes) *resample_bytes = c->rs_bytes;
    return TSDFL_OK;
}

int tsdfl_ctx_sync(tsdfl_ctx* c)
{
    if (!c) return TSDFL_ERR_INVALID_ARG;
    int rc = set_device(c->device);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(c->h_status, c->status, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaMemsetAsync(c->status, 0, sizeof(int32_t), c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    int st = c->h_status[0];
    if (st == TSDFL_ERR_DEGENERATE) set_error("No particle is valid!");
    else if (st == TSDFL_ERR_TIMEOUT) set_error("a device wait timed out");
    else if (st == TSDFL_ERR_CAPACITY) set_error("output capacity exceeded");
    else if (st == TSDFL_ERR_INVALID_ARG) set_error("invalid device input (a scan ring outside [0, 64))");
    else if (st) set_error("device status %d", st);
    return st;
}

int tsdfl_ctx_reserve(tsdfl_ctx* c, size_t P, size_t N)
{
    if (!c) return TSDFL_ERR_INVALID_ARG;
    int rc = set_device(c->device);
    if (rc) return rc;
    rc = ensure_workspace(c, P, N);
    if (rc) return rc;
    return ensure_resample_ws(c, P);
}

int tsdfl_map_create(tsdfl_ctx* ctx, const tsdfl_map_coef* coef, const int32_t* grid_occ, const float* data,
                     float sigma, uint32_t flags, tsdfl_map** out)
{
    if (!ctx || !out || !coef || (coef->grid_occ_size && !grid_occ) || (coef->data_size && !data)) {
        set_error("tsdfl_map_create: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    *out = nullptr;
    int rc = validate_coef(coef);
    if (rc) return rc;
    rc = set_device(ctx->device);
    if (rc) return rc;
    auto* m = new tsdfl_map;
    rc = map_common(ctx, coef, grid_occ, sigma, m);
    if (rc) { destroy_map(m); return rc; }
    size_t n = coef->data_size;
    cudaError_t e = cudaMalloc(&m->data, sizeof(float) * (n ? n : 1));
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(m->data, data, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) {
        set_error("tsdfl_map_create: %s", cudaGetErrorString(e));
        destroy_map(m);
        return e == cudaErrorMemoryAllocation ? TSDFL_ERR_OUT_OF_MEMORY : TSDFL_ERR_DEVICE;
    }
    bool use_codes = !(flags & TSDFL_MAP_FORCE_F32);
    if (use_codes) {
        int32_t* fail = ctx->status + 2;
        e = alloc_codes(m, n, ctx->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(fail, 0, sizeof(int32_t), ctx->stream);
        if (e == cudaSuccess) {
            rc = launch_codes_from_floats(m->data, n, m->values, coef->init_value, m->codes, fail, ctx->stream);
            if (rc) { destroy_map(m); return rc; }
            e = cudaMemcpyAsync(ctx->h_status + 2, fail, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) {
            set_error("tsdfl_map_create: %s", cudaGetErrorString(e));
            destroy_map(m);
            return TSDFL_ERR_DEVICE;
        }
        if (ctx->h_status[2]) free_codes(m);   // some slot is not a likelihood value of this sigma: keep floats
    }
    if (m->codes) {
        cudaFree(m->data);
        m->data = nullptr;
        m->bytes += sizeof(uint16_t) * (m->codes_pre + n);
    } else {
        m->bytes += sizeof(float) * n;
    }
    rc = finish_map(ctx, m, grid_occ, flags);
    if (rc) { destroy_map(m); return rc; }
    *out = m;
    return TSDFL_OK;
}

int tsdfl_map_create_codes(tsdfl_ctx* ctx, const tsdfl_map_coef* coef, const int32_t* grid_occ,
                           const uint16_t* codes, float sigma, uint32_t flags, tsdfl_map** out)
{
    if (!ctx || !out || !coef || (coef->grid_occ_size && !grid_occ) || (coef->data_size && !codes)) {
        set_error("tsdfl_map_create_codes: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    *out = nullptr;
    int rc = validate_coef(coef);
    if (rc) return rc;
    rc = set_device(ctx->device);
    if (rc) return rc;
    auto* m = new tsdfl_map;
    rc = map_common(ctx, coef, grid_occ, sigma, m);
    if (rc) { destroy_map(m); return rc; }
    size_t n = coef->data_size;
    cudaError_t e = alloc_codes(m, n, ctx->stream);
    if (e == cudaSuccess && n)
        e = cudaMemcpyAsync(m->codes, codes, sizeof(uint16_t) * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) {
        set_error("tsdfl_map_create_codes: %s", cudaGetErrorString(e));
        destroy_map(m);
        return e == cudaErrorMemoryAllocation ? TSDFL_ERR_OUT_OF_MEMORY : TSDFL_ERR_DEVICE;
    }
    m->bytes += sizeof(uint16_t) * (m->codes_pre + n);
    rc = finish_map(ctx, m, grid_occ, flags);
    if (rc) { destroy_map(m); return rc; }
    *out = m;
    return TSDFL_OK;
}

int tsdfl_map_destroy(tsdfl_map* m)
{
    destroy_map(m);
    return TSDFL_OK;
}

int tsdfl_map_get_info(const tsdfl_map* m, tsdfl_map_info* info)
{
    if (!m || !info) return TSDFL_ERR_INVALID_ARG;
    info->grid_occ_size = m->coef.grid_occ_size;
    info->data_size = m->coef.data_size;
    info->bricks = m->bricks;
    info->device_bytes = m->bytes;
    info->storage = m->h16 ? 2 : (m->codes ? 0 : 1);
    info->dense = m->grid ? 3 : (m->occ ? 1 : (m->hash ? 2 : 0));
    info->fast_index = m->view.tiled ? m->view.sub_fast : 0;
    info->reserved = 0;
    return TSDFL_OK;
}

int tsdfl_evaluate_device(tsdfl_ctx* c, const tsdfl_map* map, const tsdfl_model* mdl, float* d_particles, size_t P,
                          const float* d_points, size_t N, const float tf[16], uint32_t flags, float* d_pose_out)
{
    if (!c || !map || !tf || (P && !d_particles) || (N && !d_points)) {
        set_error("tsdfl_evaluate_device: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    int rc = check_model(mdl);
    if (rc) return rc;
    if (N == 0) return TSDFL_OK;
    if (P == 0) {
        set_error("No particle is valid!");
        return TSDFL_ERR_DEGENERATE;
    }
    if (P >= (1ull << 31) || N >= (1ull << 31)) {
        set_error("tsdfl_evaluate_device: too many particles or points");
        return TSDFL_ERR_UNSUPPORTED;
    }
    rc = set_device(c->device);
    if (rc) return rc;
    return run_eval(c, map, mdl, d_particles, P, d_points, N, tf, flags, d_pose_out, nullptr);
}

int tsdfl_evaluate_debug(tsdfl_ctx* c, const tsdfl_map* map, const tsdfl_model* mdl, float* particles, size_t P,
                         const float* points, size_t N, const float tf[16], uint32_t flags, float pose_out[6],
                         tsdfl_eval_debug* dbg)
{
    if (!c || !map || !tf || (P && !particles) || (N && !points)) {
        set_error("tsdfl_evaluate: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    int rc = check_model(mdl);
    if (rc) return rc;
    if (N == 0) return TSDFL_OK;
    if (P == 0) {
        set_error("No particle is valid!");
        return TSDFL_ERR_DEGENERATE;
    }
    if (P >= (1ull << 31) || N >= (1ull << 31)) {
        set_error("tsdfl_evaluate: too many particles or points");
        return TSDFL_ERR_UNSUPPORTED;
    }
    rc = set_device(c->device);
    if (rc) return rc;
    const bool want_idx = dbg && dbg->voxel_index;
    size_t part_b = align_up(sizeof(float) * 7 * P, 256);
    size_t pts_b = align_up(sizeof(float) * 3 * N, 256);
    size_t pose_b = 256;
    size_t idx_b = want_idx ? align_up(sizeof(uint32_t) * P * N, 256) : 0;
    rc = ensure_io(c, part_b + pts_b + pose_b + idx_b);
    if (rc) return rc;
    char* io = static_cast<char*>(c->io);
    float* d_part = reinterpret_cast<float*>(io);
    float* d_pts = reinterpret_cast<float*>(io + part_b);
    float* d_pose = reinterpret_cast<float*>(io + part_b + pts_b);
    uint32_t* d_idx = want_idx ? reinterpret_cast<uint32_t*>(io + part_b + pts_b + pose_b) : nullptr;
    cudaStream_t s = c->stream;
    CUDA_TRY(cudaMemcpyAsync(d_part, particles, sizeof(float) * 7 * P, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(d_pts, points, sizeof(float) * 3 * N, cudaMemcpyHostToDevice, s));
    rc = run_eval(c, map, mdl, d_part, P, d_pts, N, tf, flags, d_pose, d_idx);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(particles, d_part, sizeof(float) * 7 * P, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaMemcpyAsync(c->h_pose, d_pose, sizeof(float) * 6, cudaMemcpyDeviceToHost, s));
    if (dbg) {
        if (dbg->raw_weights)
            CUDA_TRY(cudaMemcpyAsync(dbg->raw_weights, c->buf.raw, sizeof(float) * P, cudaMemcpyDeviceToHost, s));
        if (dbg->hits)
            CUDA_TRY(cudaMemcpyAsync(dbg->hits, c->buf.hits, sizeof(uint32_t) * P, cudaMemcpyDeviceToHost, s));
        if (dbg->laser_pose)
            CUDA_TRY(cudaMemcpyAsync(dbg->laser_pose, c->buf.pose12, sizeof(float) * 12 * P, cudaMemcpyDeviceToHost, s));
        if (want_idx)
            CUDA_TRY(cudaMemcpyAsync(dbg->voxel_index, d_idx, sizeof(uint32_t) * P * N, cudaMemcpyDeviceToHost, s));
        CUDA_TRY(cudaMemcpyAsync(&dbg->weight_sum, c->buf.sums, sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    int st = tsdfl_ctx_sync(c);
    if (st) return st;
    if (pose_out) std::memcpy(pose_out, c->h_pose, sizeof(float) * 6);
    return TSDFL_OK;
}

int tsdfl_evaluate(tsdfl_ctx* c, const tsdfl_map* map, const tsdfl_model* mdl, float* particles, size_t P,
                   const float* points, size_t N, const float tf[16], uint32_t flags, float pose_out[6])
{
    return tsdfl_evaluate_debug(c, map, mdl, particles, P, points, N, tf, flags, pose_out, nullptr);
}

int tsdfl_evaluate_subsampled_device(tsdfl_ctx* c, const tsdfl_map* map, const tsdfl_model* mdl, float* d_particles,
                                     size_t P, const float* d_points, size_t N, const float tf[16], size_t K,
                                     uint64_t seed, float* d_pose_out)
{
    if (!c || !map || !tf || (P && !d_particles) || (N && !d_points)) {
        set_error("tsdfl_evaluate_subsampled_device: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    int rc = check_model(mdl);
    if (rc) return rc;
    if (N == 0) return TSDFL_OK;
    if (P == 0) {
        set_error("No particle is valid!");
        return TSDFL_ERR_DEGENERATE;
    }
    rc = check_sub_args("tsdfl_evaluate_subsampled_device", P, N, K);
    if (rc) return rc;
    rc = set_device(c->device);
    if (rc) return rc;
    return run_eval_sub(c, map, mdl, d_particles, P, d_points, N, tf, K, seed, d_pose_out);
}

int tsdfl_evaluate_subsampled(tsdfl_ctx* c, const tsdfl_map* map, const tsdfl_model* mdl, float* particles, size_t P,
                              const float* points, size_t N, const float tf[16], size_t K, uint64_t seed,
                              float pose_out[6], float* raw_out, uint32_t* hits_out)
{
    if (!c || !map || !tf || (P && !particles) || (N && !points)) {
        set_error("tsdfl_evaluate_subsampled: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    int rc = check_model(mdl);
    if (rc) return rc;
    if (N == 0) return TSDFL_OK;
    if (P == 0) {
        set_error("No particle is valid!");
        return TSDFL_ERR_DEGENERATE;
    }
    rc = check_sub_args("tsdfl_evaluate_subsampled", P, N, K);
    if (rc) return rc;
    rc = set_device(c->device);
    if (rc) return rc;
    size_t part_b = align_up(sizeof(float) * 7 * P, 256);
    size_t pts_b = align_up(sizeof(float) * 3 * N, 256);
    rc = ensure_io(c, part_b + pts_b + 256);
    if (rc) return rc;
    char* io = static_cast<char*>(c->io);
    float* d_part = reinterpret_cast<float*>(io);
    float* d_pts = reinterpret_cast<float*>(io + part_b);
    float* d_pose = reinterpret_cast<float*>(io + part_b + pts_b);
    cudaStream_t s = c->stream;
    CUDA_TRY(cudaMemcpyAsync(d_part, particles, sizeof(float) * 7 * P, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(d_pts, points, sizeof(float) * 3 * N, cudaMemcpyHostToDevice, s));
    rc = run_eval_sub(c, map, mdl, d_part, P, d_pts, N, tf, K, seed, d_pose);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(particles, d_part, sizeof(float) * 7 * P, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaMemcpyAsync(c->h_pose, d_pose, sizeof(float) * 6, cudaMemcpyDeviceToHost, s));
    if (raw_out) CUDA_TRY(cudaMemcpyAsync(raw_out, c->buf.raw, sizeof(float) * P, cudaMemcpyDeviceToHost, s));
    if (hits_out) CUDA_TRY(cudaMemcpyAsync(hits_out, c->buf.hits, sizeof(uint32_t) * P, cudaMemcpyDeviceToHost, s));
    int st = tsdfl_ctx_sync(c);
    if (st) return st;
    if (pose_out) std::memcpy(pose_out, c->h_pose, sizeof(float) * 6);
    return TSDFL_OK;
}

uint32_t tsdfl_subsample_index(uint64_t seed, uint64_t particle, uint32_t N, uint32_t K, uint32_t k)
{
    if (K == 0 || K > N || k >= K) return 0xffffffffu;
    return sub_point(sub_particle_state(seed, particle), N, K, k);
}

// Host forms of the systematic resampler: the M weights are every stride-th
// float of src starting at src[offset] (stride 1: a weight array; stride 7,
// offset 6: the particle cloud).  The whole source is copied in one transfer.
int resample_systematic_host(tsdfl_ctx* c, const char* fn, const float* src, size_t stride, size_t offset, size_t M,
                             float u0, uint32_t* idx_out, size_t cap, size_t* count_out)
{
    if (!c || (M && !src) || (cap && !idx_out) || !count_out) {
        set_error("%s: invalid argument", fn);
        return TSDFL_ERR_INVALID_ARG;
    }
    *count_out = 0;
    if (M == 0) return TSDFL_OK;
    if (M >= (1ull << 24)) {
        set_error("%s: at most 2^24-1 particles", fn);
        return TSDFL_ERR_UNSUPPORTED;
    }
    int rc = set_device(c->device);
    if (rc) return rc;
    rc = ensure_resample_ws(c, M);
    if (rc) return rc;
    size_t w_b = align_up(sizeof(float) * stride * M, 256);
    size_t i_b = align_up(sizeof(uint32_t) * (cap ? cap : 1), 256);
    rc = ensure_io(c, w_b + i_b + 256);
    if (rc) return rc;
    char* io = static_cast<char*>(c->io);
    float* d_src = reinterpret_cast<float*>(io);
    uint32_t* d_idx = reinterpret_cast<uint32_t*>(io + w_b);
    uint32_t* d_cnt = reinterpret_cast<uint32_t*>(io + w_b + i_b);
    cudaStream_t s = c->stream;
    CUDA_TRY(cudaMemcpyAsync(d_src, src, sizeof(float) * stride * M, cudaMemcpyHostToDevice, s));
    rc = launch_resample_impl(nullptr, d_src + offset, (int)stride, M, u0, nullptr, d_idx, cap, d_cnt, c->rs_ws,
                              c->status, s);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(c->h_count, d_cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    if (cap) CUDA_TRY(cudaMemcpyAsync(idx_out, d_idx, sizeof(uint32_t) * cap, cudaMemcpyDeviceToHost, s));
    int st = tsdfl_ctx_sync(c);
    *count_out = c->h_count[0];
    return st;
}

int tsdfl_resample_systematic(tsdfl_ctx* c, const float* weights, size_t M, float u0, uint32_t* idx_out, size_t cap,
                              size_t* count_out)
{
    return resample_systematic_host(c, "tsdfl_resample_systematic", weights, 1, 0, M, u0, idx_out, cap, count_out);
}

int tsdfl_resample_systematic_particles(tsdfl_ctx* c, const float* particles, size_t M, float u0, uint32_t* idx_out,
                                        size_t cap, size_t* count_out)
{
    return resample_systematic_host(c, "tsdfl_resample_systematic_particles", particles, 7, 6, M, u0, idx_out, cap,
                                    count_out);
}

int tsdfl_resample_systematic_device(tsdfl_ctx* c, const float* d_particles, size_t M, float u0,
                                     float* d_particles_out, size_t cap, uint32_t* d_count)
{
    if (!c || (M && !d_particles) || !d_particles_out || !d_count) {
        set_error("tsdfl_resample_systematic_device: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    if (M == 0) return TSDFL_OK;
    if (M >= (1ull << 24)) {
        set_error("tsdfl_resample_systematic_device: at most 2^24-1 particles");
        return TSDFL_ERR_UNSUPPORTED;
    }
    int rc = set_device(c->device);
    if (rc) return rc;
    rc = ensure_resample_ws(c, M);
    if (rc) return rc;
    return launch_resample_impl(d_particles, d_particles + 6, 7, M, u0, d_particles_out, nullptr, cap, d_count,
                                c->rs_ws, c->status, c->stream);
}

int tsdfl_resample_residual_systematic(tsdfl_ctx* c, const float* weights, size_t M, float u0, uint32_t* idx_out,
                                       size_t cap, size_t* count_out)
{
    if (!c || (M && !weights) || (cap && !idx_out) || !count_out) {
        set_error("tsdfl_resample_residual_systematic: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    *count_out = 0;
    if (M == 0) return TSDFL_OK;
    if (M >= (1ull << 24)) {
        set_error("tsdfl_resample_residual_systematic: at most 2^24-1 particles");
        return TSDFL_ERR_UNSUPPORTED;
    }
    int rc = set_device(c->device);
    if (rc) return rc;
    rc = ensure_resample_ws(c, M);
    if (rc) return rc;
    size_t w_b = align_up(sizeof(float) * M, 256);
    size_t i_b = align_up(sizeof(uint32_t) * (cap ? cap : 1), 256);
    rc = ensure_io(c, w_b + i_b + 256);
    if (rc) return rc;
    char* io = static_cast<char*>(c->io);
    float* d_w = reinterpret_cast<float*>(io);
    uint32_t* d_idx = reinterpret_cast<uint32_t*>(io + w_b);
    uint32_t* d_cnt = reinterpret_cast<uint32_t*>(io + w_b + i_b);
    cudaStream_t s = c->stream;
    CUDA_TRY(cudaMemcpyAsync(d_w, weights, sizeof(float) * M, cudaMemcpyHostToDevice, s));
    rc = launch_resample_residual(nullptr, d_w, 1, M, u0, nullptr, d_idx, cap, d_cnt, c->rs_ws, c->status, s);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(c->h_count, d_cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    if (cap) CUDA_TRY(cudaMemcpyAsync(idx_out, d_idx, sizeof(uint32_t) * cap, cudaMemcpyDeviceToHost, s));
    int st = tsdfl_ctx_sync(c);
    *count_out = c->h_count[0];
    if (st == TSDFL_ERR_UNSUPPORTED)
        set_error("tsdfl_resample_residual_systematic: negative or non-finite weights, or a particle count of 2^24");
    return st;
}

int tsdfl_resample_residual_systematic_device(tsdfl_ctx* c, const float* d_particles, size_t M, float u0,
                                              float* d_particles_out, size_t cap, uint32_t* d_count)
{
    if (!c || (M && !d_particles) || !d_particles_out || !d_count) {
        set_error("tsdfl_resample_residual_systematic_device: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    if (M == 0) return TSDFL_OK;
    if (M >= (1ull << 24)) {
        set_error("tsdfl_resample_residual_systematic_device: at most 2^24-1 particles");
        return TSDFL_ERR_UNSUPPORTED;
    }
    int rc = set_device(c->device);
    if (rc) return rc;
    rc = ensure_resample_ws(c, M);
    if (rc) return rc;
    return launch_resample_residual(d_particles, d_particles + 6, 7, M, u0, d_particles_out, nullptr, cap, d_count,
                                    c->rs_ws, c->status, c->stream);
}

int tsdfl_best_particle_device(tsdfl_ctx* c, const float* d_particles, size_t M, uint32_t* d_index)
{
    if (!c || (M && !d_particles) || !d_index) {
        set_error("tsdfl_best_particle_device: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    if (M >= (1ull << 31)) {
        set_error("tsdfl_best_particle_device: too many particles");
        return TSDFL_ERR_UNSUPPORTED;
    }
    int rc = set_device(c->device);
    if (rc) return rc;
    // status words 2-3 hold the 64-bit reduction key
    return launch_best_particle(d_particles, M, reinterpret_cast<unsigned long long*>(c->status + 2), d_index,
                                c->sm_count, c->stream);
}

int tsdfl_reduce_scan_device(tsdfl_ctx* c, const void* d_cloud, size_t n, uint32_t step, uint32_t x_offset,
                             uint32_t ring_offset, float cell, uint32_t flags, float* d_points_out, size_t cap,
                             uint32_t* d_count)
{
    if (!c || (n && !d_cloud) || (cap && !d_points_out) || !d_count) {
        set_error("tsdfl_reduce_scan_device: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    int rc = check_scan_args("tsdfl_reduce_scan_device", n, step, x_offset, ring_offset, cell, flags);
    if (rc) return rc;
    rc = set_device(c->device);
    if (rc) return rc;
    rc = ensure_scan_ws(c, n);
    if (rc) return rc;
    return launch_reduce_scan(static_cast<const uint8_t*>(d_cloud), n, step, x_offset, ring_offset, cell,
                              (flags & TSDFL_SCAN_OWN_RING) != 0, d_points_out, cap, d_count, c->scan_ws, c->status,
                              c->stream);
}

int tsdfl_reduce_scan(tsdfl_ctx* c, const void* cloud, size_t n, uint32_t step, uint32_t x_offset,
                      uint32_t ring_offset, float cell, uint32_t flags, float* points_out, size_t cap,
                      size_t* count_out)
{
    if (!c || (n && !cloud) || (cap && !points_out) || !count_out) {
        set_error("tsdfl_reduce_scan: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    *count_out = 0;
    int rc = check_scan_args("tsdfl_reduce_scan", n, step, x_offset, ring_offset, cell, flags);
    if (rc) return rc;
    if (n == 0) return TSDFL_OK;
    rc = set_device(c->device);
    if (rc) return rc;
    rc = ensure_scan_ws(c, n);
    if (rc) return rc;
    const size_t cloud_b = align_up((size_t)step * n, 256);
    const size_t out_b = align_up(sizeof(float) * 3 * (cap ? cap : 1), 256);
    rc = ensure_io(c, cloud_b + out_b + 256);
    if (rc) return rc;
    char* io = static_cast<char*>(c->io);
    uint8_t* d_cloud = reinterpret_cast<uint8_t*>(io);
    float* d_out = reinterpret_cast<float*>(io + cloud_b);
    uint32_t* d_cnt = reinterpret_cast<uint32_t*>(io + cloud_b + out_b);
    cudaStream_t s = c->stream;
    CUDA_TRY(cudaMemcpyAsync(d_cloud, cloud, (size_t)step * n, cudaMemcpyHostToDevice, s));
    rc = launch_reduce_scan(d_cloud, n, step, x_offset, ring_offset, cell, (flags & TSDFL_SCAN_OWN_RING) != 0, d_out,
                            cap, d_cnt, c->scan_ws, c->status, s);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(c->h_count, d_cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    int st = tsdfl_ctx_sync(c);
    *count_out = c->h_count[0];
    if (st && st != TSDFL_ERR_CAPACITY) return st;
    size_t m = *count_out < cap ? *count_out : cap;
    if (m) {
        CUDA_TRY(cudaMemcpyAsync(points_out, d_out, sizeof(float) * 3 * m, cudaMemcpyDeviceToHost, s));
        CUDA_TRY(cudaStreamSynchronize(s));
    }
    return st;
}

int tsdfl_evaluate_cloud(tsdfl_ctx* c, const tsdfl_map* map, const tsdfl_model* mdl, float* particles, size_t P,
                         const void* cloud, size_t n, uint32_t step, uint32_t x_offset, uint32_t ring_offset,
                         float cell, uint32_t scan_flags, const float tf[16], uint32_t flags, float pose_out[6],
                         size_t* n_reduced)
{
    if (n_reduced) *n_reduced = 0;
    if (!c || !map || !tf || (P && !particles) || (n && !cloud)) {
        set_error("tsdfl_evaluate_cloud: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    int rc = check_model(mdl);
    if (rc) return rc;
    rc = check_scan_args("tsdfl_evaluate_cloud", n, step, x_offset, ring_offset, cell, scan_flags);
    if (rc) return rc;
    if (n == 0) return TSDFL_OK;
    if (P >= (1ull << 31)) {
        set_error("tsdfl_evaluate_cloud: too many particles");
        return TSDFL_ERR_UNSUPPORTED;
    }
    rc = set_device(c->device);
    if (rc) return rc;
    rc = ensure_scan_ws(c, n);
    if (rc) return rc;
    const size_t part_b = align_up(sizeof(float) * 7 * (P ? P : 1), 256);
    const size_t cloud_b = align_up((size_t)step * n, 256);
    const size_t pts_b = align_up(sizeof(float) * 3 * n, 256);
    rc = ensure_io(c, part_b + cloud_b + pts_b + 512);
    if (rc) return rc;
    char* io = static_cast<char*>(c->io);
    float* d_part = reinterpret_cast<float*>(io);
    uint8_t* d_cloud = reinterpret_cast<uint8_t*>(io + part_b);
    float* d_pts = reinterpret_cast<float*>(io + part_b + cloud_b);
    uint32_t* d_cnt = reinterpret_cast<uint32_t*>(io + part_b + cloud_b + pts_b);
    float* d_pose = reinterpret_cast<float*>(io + part_b + cloud_b + pts_b + 256);
    cudaStream_t s = c->stream;
    CUDA_TRY(cudaMemcpyAsync(d_cloud, cloud, (size_t)step * n, cudaMemcpyHostToDevice, s));
    if (P) CUDA_TRY(cudaMemcpyAsync(d_part, particles, sizeof(float) * 7 * P, cudaMemcpyHostToDevice, s));
    rc = launch_reduce_scan(d_cloud, n, step, x_offset, ring_offset, cell, (scan_flags & TSDFL_SCAN_OWN_RING) != 0,
                            d_pts, n, d_cnt, c->scan_ws, c->status, s);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(c->h_count, d_cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    int st = tsdfl_ctx_sync(c);
    if (st) return st;
    const size_t N = c->h_count[0];
    if (n_reduced) *n_reduced = N;
    if (N == 0) return TSDFL_OK;
    if (P == 0) {
        set_error("No particle is valid!");
        return TSDFL_ERR_DEGENERATE;
    }
    rc = run_eval(c, map, mdl, d_part, P, d_pts, N, tf, flags, d_pose, nullptr);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(particles, d_part, sizeof(float) * 7 * P, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaMemcpyAsync(c->h_pose, d_pose, sizeof(float) * 6, cudaMemcpyDeviceToHost, s));
    st = tsdfl_ctx_sync(c);
    if (st) return st;
    if (pose_out) std::memcpy(pose_out, c->h_pose, sizeof(float) * 6);
    return TSDFL_OK;
}

// ------------------------------------------------ batched filters

struct tsdfl_batch {
    tsdfl_ctx* ctx = nullptr;
    std::vector<tsdfl_filter> f;
    struct Per {
        EvalBuffers b{};
        double* sum_f64 = nullptr;
        void* rs_ws = nullptr;
        int shift = 40;
        int npad = 4;
        bool tiled = false;
        bool dense = false;
        bool big = false;            // scored by the single-filter kernel, not the persistent queue
        size_t pass = 0;
        int32_t* sticky = nullptr;   // where device errors of this filter go (null: the context's status)
    };
    std::vector<Per> per;
    cudaStream_t stream = nullptr;   // null: the context's stream
    void* ws = nullptr;
    void* d_segs = nullptr;
    std::vector<BatchSegSpec> specs;
    uint32_t batches = 0;
    BatchKinds kinds{};
    uint32_t* d_counter = nullptr;
    int chunk = 1024, group = 4;
    cudaGraphExec_t exec = nullptr;
};

namespace {

int batch_build_segments(tsdfl_batch* B, void* pinned = nullptr)
{
    std::vector<char> host;
    char* h = static_cast<char*>(pinned);
    if (!h) {
        host.resize(B->specs.size() * batch_seg_bytes() + 1);
        h = host.data();
    }
    B->batches = build_batch_segs(B->specs.data(), (int)B->specs.size(), B->chunk, B->group, h, &B->kinds);
    if (B->specs.empty()) return TSDFL_OK;
    if (pinned)
        CUDA_TRY(cudaMemcpyAsync(B->d_segs, h, B->specs.size() * batch_seg_bytes(), cudaMemcpyHostToDevice,
                                 B->stream));
    else
        CUDA_TRY(cudaMemcpy(B->d_segs, h, B->specs.size() * batch_seg_bytes(), cudaMemcpyHostToDevice));
    return TSDFL_OK;
}

// Per-filter settings that depend on the filter's map and scan size.  A filter
// whose first pass alone makes about two of the single-filter kernel's work
// items per warp of the GPU is scored by that kernel (it fills the GPU by
// itself, and measured faster per lookup than the persistent queue); the
// queue takes the others, which alone would leave most SMs idle.
void per_configure(tsdfl_batch::Per& q, const tsdfl_filter& F, int sm_count)
{
    q.b.particles = F.d_particles;
    q.npad = (int)align_up(F.N, 4);
    double bound = std::fmax((double)F.map->max_value, 1e-30) * (double)(F.N + 1);
    int need = (int)std::ceil(std::log2(bound));
    q.shift = 62 - need < 40 ? 62 - need : 40;
    const MapView& m = F.map->view;
    q.dense = F.map->occ != nullptr;
    q.tiled = m.storage == 0 && m.tiled != 0;
    if (q.tiled) {
        int tp = tiled_pass_points(m, q.dense);
        if (tp < 1024 && q.dense) {
            q.dense = false;
            tp = tiled_pass_points(m, false);
        }
        if (tp < 64) q.tiled = false;
        q.pass = (size_t)(tp > 0 ? tp : kMaxPassPoints);
    }
    if (!q.tiled) q.pass = (size_t)kMaxPassPoints;
    q.big = false;
    if (q.tiled && F.N) {
        const size_t n1 = F.N < q.pass ? F.N : q.pass;
        const unsigned long long items = (unsigned long long)((n1 + 1023) / 1024) * ((F.P + 3) / 4);
        q.big = items >= 2ull * (unsigned long long)sm_count * (unsigned long long)tiled_warps_per_cta();
    }
}

// The persistent launch's segments of filter i (one per pass).
void append_specs(tsdfl_batch* B, size_t i)
{
    const tsdfl_filter& F = B->f[i];
    const tsdfl_batch::Per& q = B->per[i];
    if (!q.tiled || q.big || !F.N) return;
    for (size_t n0 = 0; n0 < F.N; n0 += q.pass) {
        BatchSegSpec sp;
        sp.m = F.map->view;
        sp.a_hit = F.model.a_hit;
        sp.P = (int)F.P;
        sp.n0 = (int)n0;
        sp.n1 = (int)(n0 + q.pass < F.N ? n0 + q.pass : F.N);
        sp.n_total = (int)F.N;
        sp.dense = q.dense;
        sp.b = q.b;
        B->specs.push_back(sp);
    }
}

cudaStream_t batch_stream(const tsdfl_batch* B) { return B->stream ? B->stream : B->ctx->stream; }

// Scoring of every filter: the persistent launch, the filters that fill the
// GPU by themselves with the single-filter kernel (in their particle order for
// a spread cloud), then the filters neither takes.
int batch_score(tsdfl_batch* B, cudaStream_t s)
{
    tsdfl_ctx* c = B->ctx;
    for (size_t i = 0; i < B->f.size(); ++i) {
        if (!B->per[i].tiled || B->per[i].big || B->f[i].N == 0) continue;
        CUDA_TRY(cudaMemsetAsync(B->per[i].b.sum_fx, 0, sizeof(long long) * B->f[i].P, s));
        CUDA_TRY(cudaMemsetAsync(B->per[i].b.hits, 0, sizeof(uint32_t) * B->f[i].P, s));
    }
    int rc = launch_eval_batch(B->d_segs, B->kinds, B->d_counter, c->status, c->sm_count, s);
    if (rc) return rc;
    for (size_t i = 0; i < B->f.size(); ++i) {   // pose_prepare_kernel cleared their sums
        const tsdfl_filter& F = B->f[i];
        const tsdfl_batch::Per& q = B->per[i];
        if (!q.big || F.N == 0) continue;
        rc = launch_particle_order(F.d_particles, (int)F.P, q.b, s);
        if (rc) return rc;
        for (size_t n0 = 0; n0 < F.N; n0 += q.pass) {
            size_t n1 = n0 + q.pass < F.N ? n0 + q.pass : F.N;
            rc = launch_eval_pass(F.map->view, F.model.a_hit, (int)F.P, (int)n0, (int)n1, (int)F.N, n0 == 0, false,
                                  q.dense, false, q.b, q.sum_f64, c->sm_count, s);
            if (rc) return rc;
        }
    }
    for (size_t i = 0; i < B->f.size(); ++i) {
        const tsdfl_filter& F = B->f[i];
        const tsdfl_batch::Per& q = B->per[i];
        if (q.tiled || F.N == 0) continue;
        for (size_t n0 = 0; n0 < F.N; n0 += q.pass) {
            size_t n1 = n0 + q.pass < F.N ? n0 + q.pass : F.N;
            rc = launch_eval_pass(F.map->view, F.model.a_hit, (int)F.P, (int)n0, (int)n1, (int)F.N, n0 == 0, false,
                                  q.dense, true, q.b, q.sum_f64, c->sm_count, s);
            if (rc) return rc;
        }
    }
    return TSDFL_OK;
}

int batch_record(tsdfl_batch* B)
{
    tsdfl_ctx* c = B->ctx;
    cudaStream_t s = batch_stream(B);
    for (size_t i = 0; i < B->f.size(); ++i) {
        const tsdfl_filter& F = B->f[i];
        tsdfl_batch::Per& q = B->per[i];
        if (F.N == 0) continue;
        const float inv_max_range = (float)(1.0 / (double)F.model.max_range);
        const float c_in = F.model.a_range * inv_max_range;
        int rc = launch_pose_prepare(F.tf, F.d_particles, (int)F.P, F.d_points, (int)F.N, q.npad,
                                     F.model.max_range * F.model.max_range, c_in, F.model.a_max, F.map->values,
                                     q.shift, q.b, s);
        if (rc) return rc;
    }
    int rc = batch_score(B, s);
    if (rc) return rc;
    for (size_t i = 0; i < B->f.size(); ++i) {
        const tsdfl_filter& F = B->f[i];
        tsdfl_batch::Per& q = B->per[i];
        if (F.N == 0) continue;
        const float inv_max_range = (float)(1.0 / (double)F.model.max_range);
        const float c_in = F.model.a_range * inv_max_range;
        const int mode = F.map->view.storage != 0 ? 1 : 0;
        int32_t* sticky = q.sticky ? q.sticky : c->status;
        rc = launch_norm((int)F.P, mode, q.shift, (double)F.model.a_hit, (double)c_in, (double)F.model.a_max,
                         (int)F.N, q.sum_f64, F.d_particles, F.d_pose_out, q.b, s, sticky);
        if (rc) return rc;
        if (F.d_u0 && F.d_resampled && F.P)
            rc = launch_resample_impl(F.d_particles, F.d_particles + 6, 7, F.P, 0.0f, F.d_resampled, nullptr,
                                      F.resample_cap, F.d_count, q.rs_ws, sticky, s, F.d_u0);
        if (rc) return rc;
    }
    return TSDFL_OK;
}

}  // namespace

int tsdfl_batch_create(tsdfl_ctx* c, const tsdfl_filter* filters, size_t n, uint32_t flags, tsdfl_batch** out)
{
    if (!c || !out || (n && !filters)) {
        set_error("tsdfl_batch_create: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    *out = nullptr;
    if (flags != 0) {
        set_error("tsdfl_batch_create: batches use exact sums (flags 0)");
        return TSDFL_ERR_INVALID_ARG;
    }
    for (size_t i = 0; i < n; ++i) {
        const tsdfl_filter& F = filters[i];
        if (!F.map || (F.P && !F.d_particles) || (F.N && !F.d_points) ||
            (F.d_u0 && (!F.d_resampled || !F.d_count))) {
            set_error("tsdfl_batch_create: filter %zu: invalid argument", i);
            return TSDFL_ERR_INVALID_ARG;
        }
        int rc = check_model(&F.model);
        if (rc) return rc;
        if (F.N && F.P == 0) {
            set_error("tsdfl_batch_create: filter %zu: no particles", i);
            return TSDFL_ERR_DEGENERATE;
        }
        if (F.P >= (1ull << 24) || F.N >= (1ull << 31)) {
            set_error("tsdfl_batch_create: filter %zu: too many particles or points", i);
            return TSDFL_ERR_UNSUPPORTED;
        }
        if (F.map->device != c->device) {
            set_error("tsdfl_batch_create: filter %zu: map on another device", i);
            return TSDFL_ERR_INVALID_ARG;
        }
    }
    int rc = set_device(c->device);
    if (rc) return rc;
    auto* B = new (std::nothrow) tsdfl_batch;
    if (!B) return TSDFL_ERR_OUT_OF_MEMORY;
    B->ctx = c;
    B->f.assign(filters, filters + n);
    B->per.resize(n);
    std::vector<size_t> eval_off(n), rs_off(n);
    size_t total = 0;
    for (size_t i = 0; i < n; ++i) {
        eval_off[i] = total;
        total = align_up(total + eval_layout(B->f[i].P, B->f[i].N, nullptr, nullptr, nullptr), 256);
        rs_off[i] = total;
        total = align_up(total + resample_workspace_bytes(B->f[i].P ? B->f[i].P : 1), 256);
    }
    cudaError_t e = cudaMalloc(&B->ws, total ? total : 256);
    if (e == cudaSuccess) e = cudaMalloc(&B->d_counter, 256);
    if (e == cudaSuccess) e = cudaMalloc(&B->d_segs, (2 * n + 1) * batch_seg_bytes() + 256);
    if (e != cudaSuccess) {
        set_error("tsdfl_batch_create: %s", cudaGetErrorString(e));
        tsdfl_batch_destroy(B);
        return e == cudaErrorMemoryAllocation ? TSDFL_ERR_OUT_OF_MEMORY : TSDFL_ERR_DEVICE;
    }
    char* base = static_cast<char*>(B->ws);
    for (size_t i = 0; i < n; ++i) {
        tsdfl_filter& F = B->f[i];
        tsdfl_batch::Per& q = B->per[i];
        eval_layout(F.P, F.N, base + eval_off[i], &q.b, &q.sum_f64);
        q.rs_ws = base + rs_off[i];
        per_configure(q, F, c->sm_count);
        append_specs(B, i);
    }
    if (B->specs.size() > 2 * n + 1) {   // more passes than the segment buffer holds: grow it
        cudaFree(B->d_segs);
        if (cudaMalloc(&B->d_segs, B->specs.size() * batch_seg_bytes() + 256) != cudaSuccess) {
            set_error("tsdfl_batch_create: out of memory");
            tsdfl_batch_destroy(B);
            return TSDFL_ERR_OUT_OF_MEMORY;
        }
    }
    rc = batch_build_segments(B);
    if (rc) {
        tsdfl_batch_destroy(B);
        return rc;
    }
    *out = B;
    return TSDFL_OK;
}

int tsdfl_batch_destroy(tsdfl_batch* B)
{
    if (!B) return TSDFL_OK;
    cudaSetDevice(B->ctx->device);
    if (B->ctx->stream) cudaStreamSynchronize(B->ctx->stream);
    if (B->exec) cudaGraphExecDestroy(B->exec);
    cudaFree(B->ws);
    cudaFree(B->d_counter);
    cudaFree(B->d_segs);
    delete B;
    return TSDFL_OK;
}

int tsdfl_batch_run(tsdfl_batch* B)
{
    if (!B) return TSDFL_ERR_INVALID_ARG;
    int rc = set_device(B->ctx->device);
    if (rc) return rc;
    if (B->exec) {
        CUDA_TRY(cudaGraphLaunch(B->exec, B->ctx->stream));
        g_launches += 1;
        return TSDFL_OK;
    }
    return batch_record(B);
}

int tsdfl_batch_capture(tsdfl_batch* B)
{
    if (!B) return TSDFL_ERR_INVALID_ARG;
    int rc = set_device(B->ctx->device);
    if (rc) return rc;
    if (B->exec) {
        cudaGraphExecDestroy(B->exec);
        B->exec = nullptr;
    }
    cudaStream_t s = B->ctx->stream;
    cudaGraph_t g = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
    rc = batch_record(B);
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) {
        set_error("tsdfl_batch_capture: %s", cudaGetErrorString(e));
        return TSDFL_ERR_DEVICE;
    }
    e = cudaGraphInstantiate(&B->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        B->exec = nullptr;
        set_error("tsdfl_batch_capture: %s", cudaGetErrorString(e));
        return TSDFL_ERR_DEVICE;
    }
    return TSDFL_OK;
}

int tsdfl_batch_set_tiles(tsdfl_batch* B, int chunk, int group)
{
    if (!B || chunk < 64 || chunk % 64 || group < 1 || group > 64) {
        set_error("tsdfl_batch_set_tiles: chunk must be a positive multiple of 64, group in [1, 64]");
        return TSDFL_ERR_INVALID_ARG;
    }
    int rc = set_device(B->ctx->device);
    if (rc) return rc;
    CUDA_TRY(cudaStreamSynchronize(B->ctx->stream));   // the segment table is read by queued work
    B->chunk = chunk;
    B->group = group;
    rc = batch_build_segments(B);
    if (rc) return rc;
    if (B->exec) return tsdfl_batch_capture(B);   // the graph holds the old batch count
    return TSDFL_OK;
}

int tsdfl_batch_autotune(tsdfl_batch* B, int* chunk_out, int* group_out, float* best_ms)
{
    if (!B) return TSDFL_ERR_INVALID_ARG;
    int rc = set_device(B->ctx->device);
    if (rc) return rc;
    cudaStream_t s = B->ctx->stream;
    const bool had_graph = B->exec != nullptr;
    static const int shapes[][2] = {{1024, 4}, {512, 4}, {2048, 4}, {1024, 2}, {1024, 8}, {512, 8}, {2048, 2}};
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    // the points and poses the scoring reads
    const int keep_chunk = B->chunk, keep_group = B->group;
    cudaGraphExec_t keep_exec = B->exec;
    B->exec = nullptr;
    rc = batch_record(B);
    float best = 1e30f;
    int bc = keep_chunk, bg = keep_group;
    for (const auto& sh : shapes) {
        if (rc) break;
        CUDA_TRY(cudaStreamSynchronize(s));
        B->chunk = sh[0];
        B->group = sh[1];
        rc = batch_build_segments(B);
        if (rc) break;
        float t = 0;
        for (int rep = 0; rep < 3 && !rc; ++rep) {
            cudaEventRecord(e0, s);
            rc = batch_score(B, s);
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0) t += ms;   // the first is a warm-up
        }
        if (!rc && t / 2 < best) {
            best = t / 2;
            bc = sh[0];
            bg = sh[1];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    B->exec = keep_exec;
    B->chunk = bc;
    B->group = bg;
    int rc2 = batch_build_segments(B);
    if (!rc) rc = rc2;
    if (!rc && had_graph) rc = tsdfl_batch_capture(B);
    if (chunk_out) *chunk_out = bc;
    if (group_out) *group_out = bg;
    if (best_ms) *best_ms = best;
    return rc ? rc : tsdfl_ctx_sync(B->ctx);
}

int tsdfl_batch_hits(tsdfl_batch* B, size_t i, uint32_t* hits)
{
    if (!B || i >= B->f.size() || (B->f[i].P && !hits)) {
        set_error("tsdfl_batch_hits: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    int rc = set_device(B->ctx->device);
    if (rc) return rc;
    if (B->f[i].P)
        CUDA_TRY(cudaMemcpyAsync(hits, B->per[i].b.hits, sizeof(uint32_t) * B->f[i].P, cudaMemcpyDeviceToHost,
                                 B->ctx->stream));
    return tsdfl_ctx_sync(B->ctx);
}

int tsdfl_batch_info(const tsdfl_batch* B, uint32_t* segments, uint32_t* batches, uint32_t* outside)
{
    if (!B) return TSDFL_ERR_INVALID_ARG;
    if (segments) *segments = (uint32_t)B->specs.size();
    if (batches) *batches = B->batches;
    if (outside) {
        uint32_t o = 0;
        for (size_t i = 0; i < B->f.size(); ++i) o += (!B->per[i].tiled && B->f[i].N) ? 1u : 0u;
        *outside = o;
    }
    return TSDFL_OK;
}

int tsdfl_batch_single(const tsdfl_batch* B, uint32_t* single)
{
    if (!B || !single) return TSDFL_ERR_INVALID_ARG;
    uint32_t n = 0;
    for (size_t i = 0; i < B->f.size(); ++i) n += (B->per[i].big && B->f[i].N) ? 1u : 0u;
    *single = n;
    return TSDFL_OK;
}

// ------------------------------------------------ served sessions

struct tsdfl_server {
    tsdfl_ctx* ctx = nullptr;
    tsdfl_server_config cfg{};
    size_t used = 0;
    struct Request {
        uint32_t session;
        uint64_t ticket;
        std::vector<float> points;
        std::chrono::steady_clock::time_point t_submit;
        uint64_t pp;
    };
    struct Session {
        bool open = false;
        const tsdfl_map* map = nullptr;
        tsdfl_model model{};
        float tf[16];
        uint64_t seed = 0, step = 0;
        size_t P = 0, cap = 0;
        void* mem = nullptr;
        size_t bytes = 0;
        float* parts[2] = {nullptr, nullptr};
        int cur = 0;
        tsdfl_batch::Per per;
        bool busy = false;
        std::deque<Request> queue;
    };
    struct Result {
        float pose[6];
        double latency_ms;
        int status;
    };
    struct Slot {
        cudaStream_t stream = nullptr;
        cudaEvent_t done = nullptr;
        tsdfl_batch batch;
        std::vector<Request> reqs;
        void* d_mem = nullptr;    // points, draws, poses, counts, statuses
        float* d_points = nullptr;
        float* d_u0 = nullptr;
        float* d_pose = nullptr;
        uint32_t* d_count = nullptr;
        int32_t* d_status = nullptr;
        void* h_mem = nullptr;    // pinned mirror
        float* h_points = nullptr;
        float* h_u0 = nullptr;
        float* h_pose = nullptr;
        uint32_t* h_count = nullptr;
        int32_t* h_status = nullptr;
        void* h_segs = nullptr;   // pinned segment records
        size_t seg_cap = 0;
        bool busy = false;
        std::chrono::steady_clock::time_point t_launch;
        uint64_t pp = 0;
    };
    std::vector<Session> sessions;
    Slot slots[2];
    std::unordered_map<uint64_t, Result> results;
    uint64_t next_ticket = 1;
    uint64_t queued_pp = 0, inflight_pp = 0;
    double rate = 2.0e11;   // particle*points per second, refined from finished batches
    uint64_t accepted = 0, refused = 0, published = 0, launched = 0;
};

namespace {

uint64_t splitmix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

size_t session_bytes(size_t cap, size_t max_points)
{
    return align_up(2 * sizeof(float) * 7 * cap, 256) + align_up(eval_layout(cap, max_points, nullptr, nullptr, nullptr), 256) +
           align_up(resample_workspace_bytes(cap), 256) + 256;
}

// Returns requests [from, end) of the slot to the front of their sessions'
// queues, in order (updates that were not launched).
void server_requeue(tsdfl_server* S, tsdfl_server::Slot& sl, size_t from = 0)
{
    for (size_t r = sl.reqs.size(); r-- > from;) {
        tsdfl_server::Session& se = S->sessions[sl.reqs[r].session];
        se.busy = false;
        se.queue.push_front(std::move(sl.reqs[r]));
    }
    sl.reqs.resize(from);
}

// Publishes the slot's requests as failed with `status` (updates that cannot
// be launched however often they are tried); the sessions stay as they were.
void server_fail(tsdfl_server* S, tsdfl_server::Slot& sl, int status)
{
    const auto now = std::chrono::steady_clock::now();
    for (auto& q : sl.reqs) {
        tsdfl_server::Session& se = S->sessions[q.session];
        se.busy = false;
        tsdfl_server::Result res{};
        res.status = status;
        res.latency_ms = std::chrono::duration<double, std::milli>(now - q.t_submit).count();
        S->results[q.ticket] = res;
        S->queued_pp -= q.pp;
        S->published += 1;
    }
    sl.reqs.clear();
}

int server_launch(tsdfl_server* S, int k);

// Launches every queued update of an idle session as one batch on slot k.  A
// launch that failed for want of device memory goes back to the queues (the
// memory may free up); any other failure would repeat on every attempt, so its
// updates are published with the error status and the server moves on.
int server_dispatch(tsdfl_server* S, int k)
{
    tsdfl_server::Slot& sl = S->slots[k];
    const int rc = server_launch(S, k);
    if (rc && !sl.busy) {
        if (rc == TSDFL_ERR_OUT_OF_MEMORY) server_requeue(S, sl);
        else server_fail(S, sl, rc);
    }
    return rc;
}

int server_launch(tsdfl_server* S, int k)
{
    tsdfl_server::Slot& sl = S->slots[k];
    sl.reqs.clear();
    for (size_t i = 0; i < S->sessions.size() && sl.reqs.size() < S->cfg.max_sessions; ++i) {
        tsdfl_server::Session& se = S->sessions[i];
        if (!se.open || se.busy || se.queue.empty()) continue;
        sl.reqs.push_back(std::move(se.queue.front()));
        se.queue.pop_front();
        se.busy = true;
    }
    if (sl.reqs.empty()) return TSDFL_OK;
    tsdfl_batch& B = sl.batch;
    B.f.clear();
    B.per.clear();
    B.specs.clear();
    size_t n = sl.reqs.size();
    sl.pp = 0;
    for (size_t r = 0; r < n; ++r) {
        const tsdfl_server::Request& q = sl.reqs[r];
        tsdfl_server::Session& se = S->sessions[q.session];
        const size_t N = q.points.size() / 3;
        std::memcpy(sl.h_points + 3 * S->cfg.max_points * r, q.points.data(), sizeof(float) * 3 * N);
        sl.h_u0[r] = tsdfl_server_draw(se.seed, se.step, se.P);
        tsdfl_filter F{};
        F.map = se.map;
        F.model = se.model;
        std::memcpy(F.tf, se.tf, sizeof(F.tf));
        F.d_particles = se.parts[se.cur];
        F.P = se.P;
        F.d_points = sl.d_points + 3 * S->cfg.max_points * r;
        F.N = N;
        F.d_pose_out = sl.d_pose + 8 * r;
        F.d_u0 = sl.d_u0 + r;
        F.d_resampled = se.parts[se.cur ^ 1];
        F.resample_cap = se.cap;
        F.d_count = sl.d_count + r;
        B.f.push_back(F);
        tsdfl_batch::Per pq = se.per;
        per_configure(pq, F, B.ctx->sm_count);
        pq.sticky = sl.d_status + r;
        B.per.push_back(pq);
        const size_t before = B.specs.size();
        append_specs(&B, r);
        if (B.specs.size() > sl.seg_cap) {
            // more scan passes than the slot's tables hold (the tables are sized
            // for max_sessions scans of max_points, so this is a safeguard):
            // this and the later updates wait for the next batch
            B.specs.resize(before);
            B.f.pop_back();
            B.per.pop_back();
            if (r == 0) {   // this update alone does not fit: it fails, the others wait
                server_requeue(S, sl, 1);
                set_error("tsdfl_server_poll: one scan has more passes than a batch holds");
                return TSDFL_ERR_UNSUPPORTED;
            }
            server_requeue(S, sl, r);
            n = r;
            break;
        }
        sl.pp += (uint64_t)se.P * N;
    }
    cudaStream_t s = sl.stream;
    CUDA_TRY(cudaMemsetAsync(sl.d_status, 0, sizeof(int32_t) * n, s));
    for (size_t r = 0; r < n; ++r)   // the scans sit at max_points strides
        CUDA_TRY(cudaMemcpyAsync(sl.d_points + 3 * S->cfg.max_points * r, sl.h_points + 3 * S->cfg.max_points * r,
                                 sizeof(float) * B.f[r].N * 3, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(sl.d_u0, sl.h_u0, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    int rc = batch_build_segments(&B, sl.h_segs);
    if (rc) return rc;
    rc = batch_record(&B);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(sl.h_pose, sl.d_pose, sizeof(float) * 8 * n, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaMemcpyAsync(sl.h_count, sl.d_count, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaMemcpyAsync(sl.h_status, sl.d_status, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaEventRecord(sl.done, s));
    sl.busy = true;
    sl.t_launch = std::chrono::steady_clock::now();
    S->queued_pp -= sl.pp;
    S->inflight_pp += sl.pp;
    S->launched += 1;
    return TSDFL_OK;
}

// Publishes the updates of slot k once its batch is done; false while it runs.
bool server_collect(tsdfl_server* S, int k, size_t* completed)
{
    tsdfl_server::Slot& sl = S->slots[k];
    if (!sl.busy || cudaEventQuery(sl.done) != cudaSuccess) return false;
    const auto now = std::chrono::steady_clock::now();
    for (size_t r = 0; r < sl.reqs.size(); ++r) {
        const tsdfl_server::Request& q = sl.reqs[r];
        tsdfl_server::Session& se = S->sessions[q.session];
        tsdfl_server::Result res;
        std::memcpy(res.pose, sl.h_pose + 8 * r, sizeof(res.pose));
        res.status = sl.h_status[r];
        res.latency_ms = std::chrono::duration<double, std::milli>(now - q.t_submit).count();
        const uint32_t cnt = sl.h_count[r];
        if (res.status == TSDFL_OK || res.status == TSDFL_ERR_CAPACITY) {
            se.P = cnt < se.cap ? cnt : se.cap;
            se.cur ^= 1;
        }
        se.step += 1;
        se.busy = false;
        S->results[q.ticket] = res;
        S->published += 1;
        if (completed) *completed += 1;
    }
    const double secs = std::chrono::duration<double>(now - sl.t_launch).count();
    if (secs > 0 && sl.pp > 0) S->rate = 0.8 * S->rate + 0.2 * ((double)sl.pp / secs);
    S->inflight_pp -= sl.pp;
    sl.busy = false;
    sl.reqs.clear();
    return true;
}

}  // namespace

float tsdfl_server_draw(uint64_t seed, uint64_t k, size_t P)
{
    const double u = (double)(splitmix64(seed + k * 0x9E3779B97F4A7C15ull) >> 11) * 0x1.0p-53;
    return (float)(u / (double)(P ? P : 1));
}

int tsdfl_server_create(tsdfl_ctx* c, const tsdfl_server_config* cfg, tsdfl_server** out)
{
    if (!c || !cfg || !out || cfg->max_sessions == 0 || cfg->max_points == 0) {
        set_error("tsdfl_server_create: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    *out = nullptr;
    int rc = set_device(c->device);
    if (rc) return rc;
    auto* S = new (std::nothrow) tsdfl_server;
    if (!S) return TSDFL_ERR_OUT_OF_MEMORY;
    S->ctx = c;
    S->cfg = *cfg;
    if (S->cfg.max_queue == 0) S->cfg.max_queue = 4;
    const size_t ns = cfg->max_sessions, np = cfg->max_points;
    // a scan of max_points needs at most ceil(max_points / 1024) + 1 passes
    // (every tiled pass holds at least 1,024 points), so a batch of
    // max_sessions scans always fits the segment tables
    const size_t passes = (np + 1023) / 1024 + 1;
    for (auto& sl : S->slots) {
        sl.seg_cap = ns * passes + 8;
        const size_t pts_b = align_up(sizeof(float) * 3 * np * ns, 256);
        const size_t u0_b = align_up(sizeof(float) * ns, 256), pose_b = align_up(sizeof(float) * 8 * ns, 256);
        const size_t cnt_b = align_up(sizeof(uint32_t) * ns, 256), st_b = align_up(sizeof(int32_t) * ns, 256);
        const size_t total = pts_b + u0_b + pose_b + cnt_b + st_b;
        cudaError_t e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaMalloc(&sl.d_mem, total);
        if (e == cudaSuccess) e = cudaMallocHost(&sl.h_mem, total);
        if (e == cudaSuccess) e = cudaMalloc(&sl.batch.d_segs, sl.seg_cap * batch_seg_bytes());
        if (e == cudaSuccess) e = cudaMallocHost(&sl.h_segs, sl.seg_cap * batch_seg_bytes());
        if (e == cudaSuccess) e = cudaMalloc(&sl.batch.d_counter, 256);
        if (e != cudaSuccess) {
            set_error("tsdfl_server_create: %s", cudaGetErrorString(e));
            tsdfl_server_destroy(S);
            return e == cudaErrorMemoryAllocation ? TSDFL_ERR_OUT_OF_MEMORY : TSDFL_ERR_DEVICE;
        }
        char* d = static_cast<char*>(sl.d_mem);
        char* h = static_cast<char*>(sl.h_mem);
        sl.d_points = reinterpret_cast<float*>(d);
        sl.h_points = reinterpret_cast<float*>(h);
        sl.d_u0 = reinterpret_cast<float*>(d + pts_b);
        sl.h_u0 = reinterpret_cast<float*>(h + pts_b);
        sl.d_pose = reinterpret_cast<float*>(d + pts_b + u0_b);
        sl.h_pose = reinterpret_cast<float*>(h + pts_b + u0_b);
        sl.d_count = reinterpret_cast<uint32_t*>(d + pts_b + u0_b + pose_b);
        sl.h_count = reinterpret_cast<uint32_t*>(h + pts_b + u0_b + pose_b);
        sl.d_status = reinterpret_cast<int32_t*>(d + pts_b + u0_b + pose_b + cnt_b);
        sl.h_status = reinterpret_cast<int32_t*>(h + pts_b + u0_b + pose_b + cnt_b);
        sl.batch.ctx = c;
        sl.batch.stream = sl.stream;
        S->used += total + 2 * sl.seg_cap * batch_seg_bytes();
    }
    if (S->used > cfg->hbm_budget) {
        set_error("tsdfl_server_create: the dispatch buffers alone exceed the budget");
        tsdfl_server_destroy(S);
        return TSDFL_ERR_OUT_OF_MEMORY;
    }
    *out = S;
    return TSDFL_OK;
}

int tsdfl_server_destroy(tsdfl_server* S)
{
    if (!S) return TSDFL_OK;
    cudaSetDevice(S->ctx->device);
    for (auto& sl : S->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.done) cudaEventDestroy(sl.done);
        cudaFree(sl.d_mem);
        cudaFreeHost(sl.h_mem);
        cudaFree(sl.batch.d_segs);
        cudaFreeHost(sl.h_segs);
        cudaFree(sl.batch.d_counter);
        sl.batch.d_segs = nullptr;
        sl.batch.d_counter = nullptr;
        if (sl.stream) cudaStreamDestroy(sl.stream);
    }
    for (auto& se : S->sessions) cudaFree(se.mem);
    delete S;
    return TSDFL_OK;
}

int tsdfl_session_open(tsdfl_server* S, const tsdfl_map* map, const float* particles, size_t P, const float tf[16],
                       const tsdfl_model* model, uint64_t seed, uint32_t* session)
{
    if (!S || !map || !tf || !session || (P && !particles) || P == 0) {
        set_error("tsdfl_session_open: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    int rc = check_model(model);
    if (rc) return rc;
    if (P >= (1ull << 23)) {
        set_error("tsdfl_session_open: too many particles");
        return TSDFL_ERR_UNSUPPORTED;
    }
    size_t open = 0;
    for (auto& se : S->sessions) open += se.open ? 1 : 0;
    if (open >= S->cfg.max_sessions) {
        set_error("tsdfl_session_open: the server holds max_sessions sessions");
        return TSDFL_ERR_CAPACITY;
    }
    const size_t cap = 2 * P + 16;
    const size_t bytes = session_bytes(cap, S->cfg.max_points);
    if (S->used + bytes > S->cfg.hbm_budget) {
        set_error("tsdfl_session_open: the device memory budget cannot hold the session");
        return TSDFL_ERR_OUT_OF_MEMORY;
    }
    rc = set_device(S->ctx->device);
    if (rc) return rc;
    void* mem = nullptr;
    CUDA_TRY(cudaMalloc(&mem, bytes));
    tsdfl_server::Session se;
    se.open = true;
    se.map = map;
    se.model = *model;
    std::memcpy(se.tf, tf, sizeof(se.tf));
    se.seed = seed;
    se.P = P;
    se.cap = cap;
    se.mem = mem;
    se.bytes = bytes;
    char* b = static_cast<char*>(mem);
    se.parts[0] = reinterpret_cast<float*>(b);
    se.parts[1] = reinterpret_cast<float*>(b + sizeof(float) * 7 * cap);
    char* ev = b + align_up(2 * sizeof(float) * 7 * cap, 256);
    const size_t ev_b = align_up(eval_layout(cap, S->cfg.max_points, nullptr, nullptr, nullptr), 256);
    eval_layout(cap, S->cfg.max_points, ev, &se.per.b, &se.per.sum_f64);
    se.per.rs_ws = ev + ev_b;
    CUDA_TRY(cudaMemcpy(se.parts[0], particles, sizeof(float) * 7 * P, cudaMemcpyHostToDevice));
    S->used += bytes;
    uint32_t id = (uint32_t)S->sessions.size();
    for (uint32_t i = 0; i < S->sessions.size(); ++i)
        if (!S->sessions[i].open && !S->sessions[i].busy) {
            id = i;
            break;
        }
    if (id == S->sessions.size()) S->sessions.push_back(std::move(se));
    else S->sessions[id] = std::move(se);
    *session = id;
    return TSDFL_OK;
}

int tsdfl_session_close(tsdfl_server* S, uint32_t id)
{
    if (!S || id >= S->sessions.size() || !S->sessions[id].open) {
        set_error("tsdfl_session_close: invalid session");
        return TSDFL_ERR_INVALID_ARG;
    }
    tsdfl_server::Session& se = S->sessions[id];
    if (se.busy) {   // its batch must finish before the memory goes
        for (auto& sl : S->slots)
            if (sl.busy) CUDA_TRY(cudaStreamSynchronize(sl.stream));
        size_t done = 0;
        for (int k = 0; k < 2; ++k) server_collect(S, k, &done);
    }
    for (auto& q : se.queue) S->queued_pp -= q.pp;
    se.queue.clear();
    cudaFree(se.mem);
    S->used -= se.bytes;
    se.mem = nullptr;
    se.open = false;
    return TSDFL_OK;
}

int tsdfl_session_submit(tsdfl_server* S, uint32_t id, const float* points, size_t N, uint64_t* ticket)
{
    if (!S || id >= S->sessions.size() || !S->sessions[id].open || (N && !points) || !ticket) {
        set_error("tsdfl_session_submit: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    tsdfl_server::Session& se = S->sessions[id];
    if (N > S->cfg.max_points) {
        set_error("tsdfl_session_submit: more than max_points points");
        return TSDFL_ERR_INVALID_ARG;
    }
    const uint64_t pp = (uint64_t)se.P * N;
    const double wait_ms = 1e3 * (double)(S->queued_pp + S->inflight_pp + pp) / S->rate;
    if (se.queue.size() >= S->cfg.max_queue || (S->cfg.max_wait_ms > 0 && wait_ms > S->cfg.max_wait_ms)) {
        S->refused += 1;
        set_error("tsdfl_session_submit: refused (session queue full or the server over its admission bound)");
        return TSDFL_ERR_CAPACITY;
    }
    tsdfl_server::Request q;
    q.session = id;
    q.ticket = S->next_ticket++;
    q.points.assign(points, points + 3 * N);
    q.t_submit = std::chrono::steady_clock::now();
    q.pp = pp;
    se.queue.push_back(std::move(q));
    S->queued_pp += pp;
    S->accepted += 1;
    *ticket = S->next_ticket - 1;
    return TSDFL_OK;
}

int tsdfl_server_poll(tsdfl_server* S, size_t* completed)
{
    if (!S) return TSDFL_ERR_INVALID_ARG;
    if (completed) *completed = 0;
    int rc = set_device(S->ctx->device);
    if (rc) return rc;
    for (int k = 0; k < 2; ++k) server_collect(S, k, completed);
    int first = TSDFL_OK;
    for (int k = 0; k < 2; ++k) {   // a failed dispatch on one slot does not hold up the other
        if (S->slots[k].busy) continue;
        rc = server_dispatch(S, k);
        if (rc && first == TSDFL_OK) first = rc;
    }
    return first;
}

int tsdfl_server_result(tsdfl_server* S, uint64_t ticket, float pose[6], double* latency_ms, int* status)
{
    if (!S) return TSDFL_ERR_INVALID_ARG;
    auto it = S->results.find(ticket);
    if (it == S->results.end()) {
        set_error("tsdfl_server_result: ticket not published");
        return TSDFL_ERR_INVALID_ARG;
    }
    if (pose) std::memcpy(pose, it->second.pose, sizeof(float) * 6);
    if (latency_ms) *latency_ms = it->second.latency_ms;
    if (status) *status = it->second.status;
    S->results.erase(it);
    return TSDFL_OK;
}

int tsdfl_session_particles(tsdfl_server* S, uint32_t id, float* out, size_t cap, size_t* count)
{
    if (!S || id >= S->sessions.size() || !S->sessions[id].open || !count) {
        set_error("tsdfl_session_particles: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    tsdfl_server::Session& se = S->sessions[id];
    *count = se.P;
    if (se.busy) {
        set_error("tsdfl_session_particles: an update of the session is on the device");
        return TSDFL_ERR_CAPACITY;
    }
    int rc = set_device(S->ctx->device);
    if (rc) return rc;
    const size_t m = se.P < cap ? se.P : cap;
    if (m) CUDA_TRY(cudaMemcpy(out, se.parts[se.cur], sizeof(float) * 7 * m, cudaMemcpyDeviceToHost));
    return TSDFL_OK;
}

int tsdfl_server_stats(const tsdfl_server* S, uint64_t* accepted, uint64_t* refused, uint64_t* published,
                       uint64_t* batches, double* rate)
{
    if (!S) return TSDFL_ERR_INVALID_ARG;
    if (accepted) *accepted = S->accepted;
    if (refused) *refused = S->refused;
    if (published) *published = S->published;
    if (batches) *batches = S->launched;
    if (rate) *rate = S->rate;
    return TSDFL_OK;
}

// ------------------------------------------------ the reference's other resamplers

namespace {

enum class Rs { Wheel, Residual, Metropolis, Rejection };

struct RsCall {
    Rs kind;
    size_t M;
    const void* draws;      // wheel: double[M]; residual: uint32[n_draws]; metropolis: float[M*steps]
    const void* draws2;     // metropolis: uint32[M*steps]
    size_t n_draws;
    uint32_t steps;
    uint64_t seed;
};

constexpr uint32_t kRejectionRounds = 1u << 20;

size_t residual_draws(const RsCall& r) { return r.draws ? r.n_draws : 4 * r.M + 4096; }

int rs_launch(tsdfl_ctx* c, const RsCall& r, const float* particles, const float* w, int stride, float* out,
              uint32_t* idx_out)
{
    const size_t K = r.kind == Rs::Residual ? residual_draws(r) : 0;
    int rc = ensure_aux_ws(c, resamplers_workspace_bytes(r.M, K));
    if (rc) return rc;
    cudaStream_t s = c->stream;
    switch (r.kind) {
    case Rs::Wheel:
        return launch_resample_wheel(particles, w, stride, r.M, static_cast<const double*>(r.draws), r.seed, out,
                                     idx_out, c->aux_ws, s);
    case Rs::Residual:
        return launch_resample_residual_random(particles, w, stride, r.M, static_cast<const uint32_t*>(r.draws), K,
                                               r.seed, out, idx_out, c->aux_ws, c->status, s);
    case Rs::Metropolis:
        return launch_resample_metropolis(particles, w, stride, r.M, r.steps, static_cast<const float*>(r.draws),
                                          static_cast<const uint32_t*>(r.draws2), r.seed, out, idx_out, c->status,
                                          s);
    case Rs::Rejection:
        return launch_resample_rejection(particles, w, stride, r.M, r.seed, kRejectionRounds, out, idx_out,
                                         c->aux_ws, c->status, c->sm_count, s);
    }
    return TSDFL_ERR_INVALID_ARG;
}

int rs_check(const char* fn, tsdfl_ctx* c, const RsCall& r, bool have_in, bool have_out)
{
    if (!c || (r.M && (!have_in || !have_out))) {
        set_error("%s: invalid argument", fn);
        return TSDFL_ERR_INVALID_ARG;
    }
    if (r.M >= (1ull << 31)) {
        set_error("%s: too many particles", fn);
        return TSDFL_ERR_UNSUPPORTED;
    }
    if (r.kind == Rs::Residual && r.draws && r.M && r.n_draws == 0) {
        set_error("%s: no draws", fn);
        return TSDFL_ERR_INVALID_ARG;
    }
    if (r.kind == Rs::Residual && residual_draws(r) >= (1ull << 32)) {
        set_error("%s: too many draws", fn);
        return TSDFL_ERR_UNSUPPORTED;
    }
    if (r.kind == Rs::Metropolis && (!r.draws) != (!r.draws2)) {
        set_error("%s: give both draw arrays or neither", fn);
        return TSDFL_ERR_INVALID_ARG;
    }
    if (r.kind == Rs::Metropolis && (uint64_t)r.M * r.steps >= (1ull << 40)) {
        set_error("%s: too many draws", fn);
        return TSDFL_ERR_UNSUPPORTED;
    }
    return set_device(c->device);
}

const char* rs_message(int st)
{
    if (st == TSDFL_ERR_UNSUPPORTED) return "the draws ran out before every particle was emitted";
    if (st == TSDFL_ERR_INVALID_ARG) return "a drawn particle index is not below M";
    return nullptr;
}

int rs_host(const char* fn, tsdfl_ctx* c, const RsCall& r, const float* weights, uint32_t* idx_out)
{
    int rc = rs_check(fn, c, r, weights != nullptr, idx_out != nullptr);
    if (rc || r.M == 0) return rc;
    size_t db = 0, db2 = 0;
    if (r.draws) {
        if (r.kind == Rs::Wheel) db = sizeof(double) * r.M;
        if (r.kind == Rs::Residual) db = sizeof(uint32_t) * r.n_draws;
        if (r.kind == Rs::Metropolis) {
            db = sizeof(float) * r.M * r.steps;
            db2 = sizeof(uint32_t) * r.M * r.steps;
        }
    }
    const size_t w_b = align_up(sizeof(float) * r.M, 256), i_b = align_up(sizeof(uint32_t) * r.M, 256);
    const size_t d_b = align_up(db, 256), d2_b = align_up(db2, 256);
    rc = ensure_io(c, w_b + i_b + d_b + d2_b);
    if (rc) return rc;
    char* io = static_cast<char*>(c->io);
    float* d_w = reinterpret_cast<float*>(io);
    uint32_t* d_idx = reinterpret_cast<uint32_t*>(io + w_b);
    void* d_dr = db ? io + w_b + i_b : nullptr;
    void* d_dr2 = db2 ? io + w_b + i_b + d_b : nullptr;
    cudaStream_t s = c->stream;
    CUDA_TRY(cudaMemcpyAsync(d_w, weights, sizeof(float) * r.M, cudaMemcpyHostToDevice, s));
    if (db) CUDA_TRY(cudaMemcpyAsync(d_dr, r.draws, db, cudaMemcpyHostToDevice, s));
    if (db2) CUDA_TRY(cudaMemcpyAsync(d_dr2, r.draws2, db2, cudaMemcpyHostToDevice, s));
    RsCall dr = r;
    dr.draws = d_dr;
    dr.draws2 = d_dr2;
    rc = rs_launch(c, dr, nullptr, d_w, 1, nullptr, d_idx);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(idx_out, d_idx, sizeof(uint32_t) * r.M, cudaMemcpyDeviceToHost, s));
    int st = tsdfl_ctx_sync(c);
    if (st && rs_message(st)) set_error("%s: %s", fn, rs_message(st));
    return st;
}

int rs_device(const char* fn, tsdfl_ctx* c, const RsCall& r, const float* d_particles, float* d_out)
{
    int rc = rs_check(fn, c, r, d_particles != nullptr, d_out != nullptr);
    if (rc || r.M == 0) return rc;
    return rs_launch(c, r, d_particles, d_particles + 6, 7, d_out, nullptr);
}

}  // namespace

int tsdfl_resample_wheel(tsdfl_ctx* c, const float* weights, size_t M, const double* draws, uint64_t seed,
                         uint32_t* idx_out)
{
    return rs_host("tsdfl_resample_wheel", c, RsCall{Rs::Wheel, M, draws, nullptr, 0, 0, seed}, weights, idx_out);
}

int tsdfl_resample_wheel_device(tsdfl_ctx* c, const float* d_particles, size_t M, const double* d_draws,
                                uint64_t seed, float* d_out)
{
    return rs_device("tsdfl_resample_wheel_device", c, RsCall{Rs::Wheel, M, d_draws, nullptr, 0, 0, seed},
                     d_particles, d_out);
}

int tsdfl_resample_residual(tsdfl_ctx* c, const float* weights, size_t M, const uint32_t* draws, size_t n_draws,
                            uint64_t seed, uint32_t* idx_out)
{
    return rs_host("tsdfl_resample_residual", c, RsCall{Rs::Residual, M, draws, nullptr, n_draws, 0, seed}, weights,
                   idx_out);
}

int tsdfl_resample_residual_device(tsdfl_ctx* c, const float* d_particles, size_t M, const uint32_t* d_draws,
                                   size_t n_draws, uint64_t seed, float* d_out)
{
    return rs_device("tsdfl_resample_residual_device", c,
                     RsCall{Rs::Residual, M, d_draws, nullptr, n_draws, 0, seed}, d_particles, d_out);
}

int tsdfl_resample_metropolis(tsdfl_ctx* c, const float* weights, size_t M, uint32_t steps, const float* u_draws,
                              const uint32_t* j_draws, uint64_t seed, uint32_t* idx_out)
{
    return rs_host("tsdfl_resample_metropolis", c, RsCall{Rs::Metropolis, M, u_draws, j_draws, 0, steps, seed},
                   weights, idx_out);
}

int tsdfl_resample_metropolis_device(tsdfl_ctx* c, const float* d_particles, size_t M, uint32_t steps,
                                     const float* d_u_draws, const uint32_t* d_j_draws, uint64_t seed, float* d_out)
{
    return rs_device("tsdfl_resample_metropolis_device", c,
                     RsCall{Rs::Metropolis, M, d_u_draws, d_j_draws, 0, steps, seed}, d_particles, d_out);
}

int tsdfl_resample_rejection(tsdfl_ctx* c, const float* weights, size_t M, uint64_t seed, uint32_t* idx_out)
{
    return rs_host("tsdfl_resample_rejection", c, RsCall{Rs::Rejection, M, nullptr, nullptr, 0, 0, seed}, weights,
                   idx_out);
}

int tsdfl_resample_rejection_device(tsdfl_ctx* c, const float* d_particles, size_t M, uint64_t seed, float* d_out)
{
    return rs_device("tsdfl_resample_rejection_device", c, RsCall{Rs::Rejection, M, nullptr, nullptr, 0, 0, seed},
                     d_particles, d_out);
}

int tsdfl_pose_array_device(tsdfl_ctx* c, const float* d_particles, size_t P, double* d_poses)
{
    if (!c || (P && (!d_particles || !d_poses))) {
        set_error("tsdfl_pose_array_device: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    if (P >= (1ull << 32)) {
        set_error("tsdfl_pose_array_device: too many particles");
        return TSDFL_ERR_UNSUPPORTED;
    }
    int rc = set_device(c->device);
    if (rc) return rc;
    return launch_pose_array(d_particles, P, d_poses, c->stream);
}

int tsdfl_pose_array(tsdfl_ctx* c, const float* particles, size_t P, double* poses)
{
    if (!c || (P && (!particles || !poses))) {
        set_error("tsdfl_pose_array: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    if (P == 0) return TSDFL_OK;
    if (P >= (1ull << 32)) {
        set_error("tsdfl_pose_array: too many particles");
        return TSDFL_ERR_UNSUPPORTED;
    }
    int rc = set_device(c->device);
    if (rc) return rc;
    const size_t part_b = align_up(sizeof(float) * 7 * P, 256);
    rc = ensure_io(c, part_b + sizeof(double) * 7 * P);
    if (rc) return rc;
    char* io = static_cast<char*>(c->io);
    float* d_part = reinterpret_cast<float*>(io);
    double* d_poses = reinterpret_cast<double*>(io + part_b);
    cudaStream_t s = c->stream;
    CUDA_TRY(cudaMemcpyAsync(d_part, particles, sizeof(float) * 7 * P, cudaMemcpyHostToDevice, s));
    rc = launch_pose_array(d_part, P, d_poses, s);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(poses, d_poses, sizeof(double) * 7 * P, cudaMemcpyDeviceToHost, s));
    return tsdfl_ctx_sync(c);
}

int tsdfl_motion_update_device(tsdfl_ctx* c, float* d_particles, size_t P, const tsdfl_motion* m, uint64_t seed,
                               uint64_t step, double* d_draws_out)
{
    if (!c || !m || (P && !d_particles)) {
        set_error("tsdfl_motion_update_device: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    if (P >= (1ull << 32)) {
        set_error("tsdfl_motion_update_device: too many particles");
        return TSDFL_ERR_UNSUPPORTED;
    }
    int rc = set_device(c->device);
    if (rc) return rc;
    return launch_motion(d_particles, P, m->mean, m->stddev, seed, step, nullptr, d_draws_out, c->stream);
}

int tsdfl_motion_apply_device(tsdfl_ctx* c, float* d_particles, size_t P, const double* d_draws)
{
    if (!c || (P && (!d_particles || !d_draws))) {
        set_error("tsdfl_motion_apply_device: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    if (P >= (1ull << 32)) {
        set_error("tsdfl_motion_apply_device: too many particles");
        return TSDFL_ERR_UNSUPPORTED;
    }
    int rc = set_device(c->device);
    if (rc) return rc;
    return launch_motion(d_particles, P, nullptr, nullptr, 0, 0, d_draws, nullptr, c->stream);
}

namespace {

int motion_host(tsdfl_ctx* c, float* particles, size_t P, const tsdfl_motion* m, uint64_t seed, uint64_t step,
                const double* draws, const char* fn)
{
    if (!c || (P && !particles) || (!m && !draws && P)) {
        set_error("%s: invalid argument", fn);
        return TSDFL_ERR_INVALID_ARG;
    }
    if (P == 0) return TSDFL_OK;
    if (P >= (1ull << 32)) {
        set_error("%s: too many particles", fn);
        return TSDFL_ERR_UNSUPPORTED;
    }
    int rc = set_device(c->device);
    if (rc) return rc;
    const size_t part_b = align_up(sizeof(float) * 7 * P, 256);
    const size_t draw_b = draws ? align_up(sizeof(double) * 6 * P, 256) : 0;
    rc = ensure_io(c, part_b + draw_b);
    if (rc) return rc;
    char* io = static_cast<char*>(c->io);
    float* d_part = reinterpret_cast<float*>(io);
    double* d_draws = draws ? reinterpret_cast<double*>(io + part_b) : nullptr;
    cudaStream_t s = c->stream;
    CUDA_TRY(cudaMemcpyAsync(d_part, particles, sizeof(float) * 7 * P, cudaMemcpyHostToDevice, s));
    if (draws) CUDA_TRY(cudaMemcpyAsync(d_draws, draws, sizeof(double) * 6 * P, cudaMemcpyHostToDevice, s));
    rc = draws ? launch_motion(d_part, P, nullptr, nullptr, 0, 0, d_draws, nullptr, s)
               : launch_motion(d_part, P, m->mean, m->stddev, seed, step, nullptr, nullptr, s);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(particles, d_part, sizeof(float) * 7 * P, cudaMemcpyDeviceToHost, s));
    return tsdfl_ctx_sync(c);
}

}  // namespace

int tsdfl_motion_update(tsdfl_ctx* c, float* particles, size_t P, const tsdfl_motion* m, uint64_t seed,
                        uint64_t step)
{
    if (!m) {
        set_error("tsdfl_motion_update: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    return motion_host(c, particles, P, m, seed, step, nullptr, "tsdfl_motion_update");
}

int tsdfl_motion_apply(tsdfl_ctx* c, float* particles, size_t P, const double* draws)
{
    return motion_host(c, particles, P, nullptr, 0, 0, draws, "tsdfl_motion_apply");
}

}  // extern "C"

// ------------------------------------------------ resampling without allocation
//
// Some callers must not allocate device memory once their filter loop runs: a
// real-time localisation node whose update deadline cannot absorb cudaMalloc's
// device-wide synchronisation, or a host process whose device memory is owned
// by a fixed pool it cannot grow.  tsdfl_resample_systematic_static serves them
// with a scratch area compiled into this library (one per device, in the
// module's static device memory) instead of the context's growable workspace.

namespace {

constexpr size_t kStaticResampleParticles = size_t(1) << 18;   // largest M the static scratch holds
// Upper bound of resample_workspace_bytes(kStaticResampleParticles): the
// fixed-point prefix sums (8 bytes a particle), three tile tables, the
// segment table and the chunk table of the double sums, with headroom.
// Checked against the launcher's own figure on every call.
constexpr size_t kStaticResampleBytes = 8 * (kStaticResampleParticles + 3 * (kStaticResampleParticles / 256 + 2)) +
                                        64 * 1024;
constexpr int kStaticMaxDevices = 64;

static __device__ __align__(256) unsigned char g_resample_scratch[kStaticResampleBytes];

std::mutex g_static_mu;
void* g_static_ptr[kStaticMaxDevices] = {};
unsigned long long g_static_ctx[kStaticMaxDevices] = {};   // context id the address belongs to

// Unique id of the current context (cuCtxGetId through the runtime's driver
// entry points; ids are never reused within a process), 0 when unavailable.
unsigned long long current_context_id()
{
    typedef int (*GetCurrent)(void**);
    typedef int (*GetId)(void*, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrent>(f);
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetId>(f);
    }
    void* ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
    return id;
}

// Device address of this device's copy of g_resample_scratch, looked up with
// that device current (the caller has made it current) on the first call and
// again whenever the device's context has changed since (a cudaDeviceReset
// loads the module into a new context, where the array may sit elsewhere).
int static_scratch(int dev, void** out)
{
    if (dev < 0 || dev >= kStaticMaxDevices) {
        set_error("tsdfl_resample_systematic_static: device %d beyond the %d devices supported", dev,
                  kStaticMaxDevices);
        return TSDFL_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lock(g_static_mu);
    const unsigned long long ctx_id = current_context_id();
    if (!g_static_ptr[dev] || ctx_id != g_static_ctx[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_resample_scratch);
        if (e != cudaSuccess || !p) {
            set_error("tsdfl_resample_systematic_static: cudaGetSymbolAddress failed on device %d: %s", dev,
                      cudaGetErrorString(e));
            return TSDFL_ERR_DEVICE;
        }
        g_static_ptr[dev] = p;
        g_static_ctx[dev] = ctx_id;
    }
    *out = g_static_ptr[dev];
    return TSDFL_OK;
}

}  // namespace

extern "C" {

int tsdfl_resample_systematic_static(tsdfl_ctx* c, const float* d_particles, size_t M, float u0,
                                     float* d_particles_out, size_t cap, uint32_t* d_count)
{
    if (!c || (M && !d_particles) || !d_particles_out || !d_count) {
        set_error("tsdfl_resample_systematic_static: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    if (M == 0) return TSDFL_OK;
    if (M > kStaticResampleParticles || resample_workspace_bytes(M) > kStaticResampleBytes) {
        set_error("tsdfl_resample_systematic_static: %zu particles exceed the static scratch limit of %zu", M,
                  kStaticResampleParticles);
        return TSDFL_ERR_UNSUPPORTED;
    }
    int rc = set_device(c->device);
    if (rc) return rc;
    void* scratch = nullptr;
    rc = static_scratch(c->device, &scratch);
    if (rc) return rc;
    return launch_resample_impl(d_particles, d_particles + 6, 7, M, u0, d_particles_out, nullptr, cap, d_count,
                                scratch, c->status, c->stream);
}

}  // extern "C"
