// Likelihood-map construction from TSDF cells (host): the map createTSDFMap
// builds (include/tsdf_localization/map/map_util.h:17-154) on top of
// CudaSubVoxelMap::setData (include/tsdf_localization/cuda/cuda_sub_voxel_map.tcc:170-230),
// producing 16-bit slot codes instead of float slots.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <omp.h>

#include "map_host.h"
#include "tsdfl.h"

namespace tsdfl {

uint64_t f2u_x86_host(float v)
{
    const float two63 = 9223372036854775808.0f;
    if (v != v) return 0x8000000000000000ull;
    if (v < two63) {
        if (v >= -two63) return (uint64_t)(int64_t)v;
        return 0x8000000000000000ull;
    }
    float w = v - two63;
    if (w < two63) return ((uint64_t)(int64_t)w) ^ 0x8000000000000000ull;
    return 0;
}

// map_util.h:124-127 for |tsdf| = mm millimetres.
float likelihood_value(int mm, float sigma)
{
    const float sigma_quad = sigma * sigma;
    const float tsdf_value = (float)mm;
    double value = (double)tsdf_value * 0.001;
    value = (double)(expf((float)(-(value * value) / (double)sigma_quad / 2)) /
                     sqrtf((float)((double)(2 * sigma_quad) * M_PI)));
    value = value * value * value;
    return (float)value;
}

// map_util.h:68-71
float likelihood_init(float sigma)
{
    const float sigma_quad = sigma * sigma;
    float init = expf((float)(-(10.0 * 10.0) / (double)sigma_quad / 2)) / sqrtf((float)((double)(2 * sigma_quad) * M_PI));
    return init * init * init;
}

void code_values(float sigma, float init_value, float out[604])
{
    for (int c = 0; c < 600; ++c) out[c] = likelihood_value(c, sigma);
    out[600] = init_value;
    out[601] = init_value;
    out[602] = 0.0f;
    out[603] = 0.0f;
}

// CudaSubVoxelMap ctor (cuda_sub_voxel_map.tcc:4-48)
void coef_init(tsdfl_map_coef* c, const float mn[3], const float mx[3], float res, float init)
{
    std::memset(c, 0, sizeof(*c));
    c->dim_x = (uint64_t)std::ceil(std::fabs(mx[0] - mn[0]) / res);
    c->dim_y = (uint64_t)std::ceil(std::fabs(mx[1] - mn[1]) / res);
    c->dim_z = (uint64_t)std::ceil(std::fabs(mx[2] - mn[2]) / res);
    c->min_x = mn[0]; c->min_y = mn[1]; c->min_z = mn[2];
    c->max_x = mx[0]; c->max_y = mx[1]; c->max_z = mx[2];
    c->resolution = res;
    c->init_value = init;
    c->up_dim_x = (uint64_t)std::ceil((float)std::fabs(mx[0] - mn[0]) / 1.0f);
    c->up_dim_y = (uint64_t)std::ceil((float)std::fabs(mx[1] - mn[1]) / 1.0f);
    c->up_dim_z = (uint64_t)std::ceil((float)std::fabs(mx[2] - mn[2]) / 1.0f);
    c->up_dim_2 = c->up_dim_x * c->up_dim_y;
    c->sub_dim = (uint64_t)std::ceil(1.0f / res);
    c->sub_dim_2 = c->sub_dim * c->sub_dim;
    c->grid_occ_size = c->up_dim_x * c->up_dim_y * c->up_dim_z;
    c->data_size = 0;
}

// Brick (upper voxel) index of a position as setData computes it (:179-186).
static inline uint64_t brick_of(const tsdfl_map_coef& c, float x, float y, float z)
{
    uint64_t ux = f2u_x86_host((x - c.min_x) / 1.0f);
    uint64_t uy = f2u_x86_host((y - c.min_y) / 1.0f);
    uint64_t uz = f2u_x86_host((z - c.min_z) / 1.0f);
    return ux + uy * c.up_dim_x + uz * c.up_dim_x * c.up_dim_y;
}

uint64_t host_slot_index(const tsdfl_map_coef& c, const int32_t* grid_occ, float x, float y, float z)
{
    uint64_t gx = f2u_x86_host(x - c.min_x), gy = f2u_x86_host(y - c.min_y), gz = f2u_x86_host(z - c.min_z);
    gx = f2u_x86_host((float)gx / c.resolution);
    gy = f2u_x86_host((float)gy / c.resolution);
    gz = f2u_x86_host((float)gz / c.resolution);
    if (gx >= c.dim_x || gy >= c.dim_y || gz >= c.dim_z) return c.data_size;
    float ox = x - c.min_x, oy = y - c.min_y, oz = z - c.min_z;
    uint64_t ux = f2u_x86_host(ox / 1.0f), uy = f2u_x86_host(oy / 1.0f), uz = f2u_x86_host(oz / 1.0f);
    float sx = ox - (float)ux * 1.0f, sy = oy - (float)uy * 1.0f, sz = oz - (float)uz * 1.0f;
    uint64_t up = ux + uy * c.up_dim_x + uz * c.up_dim_2;
    if (up >= c.grid_occ_size) return c.data_size;
    int32_t base = grid_occ[up];
    if (base < 0) return c.data_size;
    uint64_t qx = f2u_x86_host(sx / c.resolution), qy = f2u_x86_host(sy / c.resolution),
             qz = f2u_x86_host(sz / c.resolution);
    return (uint64_t)(int64_t)base + qx + qy * c.sub_dim + qz * c.sub_dim_2;
}

int32_t coarse_mmax(uint64_t dim, float res)
{
    for (int64_t m = 0; m < 4194304; ++m) {
        float q = (float)m / res;
        if (f2u_x86_host(q) >= dim) return (int32_t)(m - 1);
    }
    return 4194304;
}

// Smallest non-negative float s (searched up to 2.0) for which pred(s) holds;
// pred must be monotone in s.  2.0 when it never holds below 2.
template <class Pred>
static float min_float_where(Pred pred)
{
    uint32_t lo = 0, hi;
    float two = 2.0f;
    std::memcpy(&hi, &two, 4);
    if (!pred(two)) return two;
    while (lo < hi) {   // float order == bit order for non-negative floats
        uint32_t mid = lo + (hi - lo) / 2;
        float f;
        std::memcpy(&f, &mid, 4);
        if (pred(f)) hi = mid;
        else lo = mid + 1;
    }
    float f;
    std::memcpy(&f, &lo, 4);
    return f;
}

int sub_index_mult(float res, uint64_t sub_dim, float* hi_out, float* lo_out)
{
    if (!(res > 0.0f) || !(res <= 1.0f) || sub_dim + 2 > 4096) return 0;
    const int K = (int)sub_dim + 1;
    // thr[k] = smallest float s >= 0 with trunc(s / res) >= k (2.0 when none below 2)
    std::vector<float> thr(K + 1, 2.0f);
    for (int k = 1; k <= K; ++k)
        thr[k] = min_float_where([&](float s) { return f2u_x86_host(s / res) >= (uint64_t)k; });
    auto bits_of = [](float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; };
    auto float_of = [](uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; };
    const float below_one = float_of(bits_of(1.0f) - 1);
    // q(s) and both candidate forms are non-decreasing in s, so they agree on
    // every float in [0, 1) iff they agree on both sides of every threshold.
    auto agrees = [&](auto idx) {
        for (int k = 1; k <= K; ++k) {
            if (thr[k] < 1.0f) {
                if (idx(thr[k]) < (uint64_t)k || idx(float_of(bits_of(thr[k]) - 1)) >= (uint64_t)k) return false;
            } else if (idx(below_one) >= (uint64_t)k) {
                return false;
            }
        }
        return true;
    };
    // one multiplier m: q == floor(s * m), the product taken exactly
    const float base = 1.0f / res;
    for (int d = 0; d <= 8192; ++d) {
        for (int sgn = -1; sgn <= 1; sgn += 2) {
            if (d == 0 && sgn > 0) continue;
            const float m = float_of(bits_of(base) + (uint32_t)(sgn * d));
            if (agrees([&](float s) { return (uint64_t)std::floor((double)s * (double)m); })) {
                *hi_out = m;
                *lo_out = 0.0f;
                return 2;
            }
        }
    }
    // two terms hi + lo ~ 1 / res to about 48 bits: q == trunc(fl(s * hi + fl(s * lo)));
    // |lo| << hi keeps the form monotone in s
    const double inv = 1.0 / (double)res;
    const float h0 = (float)inv;
    for (int da = 0; da <= 16; ++da) {
        for (int sa = -1; sa <= 1; sa += 2) {
            if (da == 0 && sa > 0) continue;
            const float hi = float_of(bits_of(h0) + (uint32_t)(sa * da));
            const float l0 = (float)(inv - (double)hi);
            for (int db = 0; db <= 16; ++db) {
                for (int sb = -1; sb <= 1; sb += 2) {
                    if (db == 0 && sb > 0) continue;
                    const float lo = l0 == 0.0f ? 0.0f : float_of(bits_of(l0) + (uint32_t)(sb * db));
                    if (!(std::fabs(lo) * 4.0f < hi)) continue;
                    if (agrees([&](float s) { return (uint64_t)std::fmaf(s, hi, s * lo); })) {
                        *hi_out = hi;
                        *lo_out = lo;
                        return 1;
                    }
                }
            }
        }
    }
    return 0;
}

}  // namespace tsdfl

using namespace tsdfl;

namespace {

struct Cell {  // one band cell of the TSDF, in reading order
    float x, y, z;
    uint16_t code;
};

// Cell position of map_util.h:111-120: (float)index * voxel_mm, times 0.001 in double.
inline float cell_pos(int idx, int voxel_mm)
{
    return (float)((double)((float)idx * (float)voxel_mm) * 0.001);
}

}  // namespace

extern "C" {

void tsdfl_free(void* p) { std::free(p); }

int tsdfl_code_values(float sigma, float init_value, float* out601)
{
    float v[604];
    code_values(sigma, init_value, v);
    std::memcpy(out601, v, sizeof(float) * 601);
    return TSDFL_OK;
}

int tsdfl_build_map_codes(const int32_t* chunk_pos, const uint32_t* chunks, size_t n_chunks, int edge, int voxel_mm,
                          float sigma, tsdfl_map_coef* coef, int32_t** grid_occ_out, uint16_t** codes_out,
                          float** free_xyz, size_t* n_free)
{
    if (!coef || !grid_occ_out || !codes_out || edge <= 0 || voxel_mm <= 0 || (n_chunks && (!chunk_pos || !chunks))) {
        set_error("tsdfl_build_map_codes: invalid argument");
        return TSDFL_ERR_INVALID_ARG;
    }
    // bounding box from the chunk coordinates, min and max starting at 0 (map_util.h:23-66)
    float mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
    for (size_t k = 0; k < n_chunks; ++k)
        for (int a = 0; a < 3; ++a) {
            int coord = chunk_pos[3 * k + a];
            if ((float)coord < mn[a]) mn[a] = (float)coord;
            if ((float)coord > mx[a]) mx[a] = (float)coord;
        }
    for (int a = 0; a < 3; ++a) {
        mn[a] = (float)((double)(mn[a] * (float)edge * (float)voxel_mm) * 0.001);
        mx[a] = (float)((double)((mx[a] * (float)edge + (float)edge) * (float)voxel_mm) * 0.001);
    }
    const float init = likelihood_init(sigma);
    coef_init(coef, mn, mx, (float)(voxel_mm * 0.001), init);
    if (coef->grid_occ_size >= (1ull << 31)) {
        set_error("tsdfl_build_map_codes: map has too many bricks");
        return TSDFL_ERR_UNSUPPORTED;
    }

    // band cells of every chunk, in chunk order then cell order (map_util.h:100-149)
    const size_t cells = (size_t)edge * edge * edge;
    std::vector<std::vector<Cell>> band(n_chunks);
    std::vector<std::vector<float>> freep(n_chunks);
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t k = 0; k < (int64_t)n_chunks; ++k) {
        const uint32_t* raw = chunks + (size_t)k * cells;
        const int32_t* cp = chunk_pos + 3 * k;
        auto& out = band[k];
        for (int i = 0; i < edge; ++i)
            for (int j = 0; j < edge; ++j)
                for (int l = 0; l < edge; ++l) {
                    uint32_t e = raw[(size_t)edge * edge * i + (size_t)edge * j + l];
                    int16_t val = (int16_t)(uint16_t)(e & 0xffffu);
                    int16_t wgt = (int16_t)(uint16_t)(e >> 16);
                    if (wgt == 0) continue;
                    float tsdf_value = (float)val;
                    float px = cell_pos(edge * cp[0] + i, voxel_mm);
                    float py = cell_pos(edge * cp[1] + j, voxel_mm);
                    float pz = cell_pos(edge * cp[2] + l, voxel_mm);
                    if (std::fabs(tsdf_value) < 600.0f) {
                        int av = val < 0 ? -(int)val : (int)val;
                        out.push_back({px, py, pz, (uint16_t)av});
                    } else if (free_xyz) {
                        freep[k].push_back(px);
                        freep[k].push_back(py);
                        freep[k].push_back(pz);
                    }
                }
    }
    // setData: mark bricks, offsets in linear brick order, fill with init
    int32_t* grid_occ = (int32_t*)std::malloc(sizeof(int32_t) * (coef->grid_occ_size + 1));
    for (uint64_t i = 0; i < coef->grid_occ_size; ++i) grid_occ[i] = -1;
    int overflow = 0;
#pragma omp parallel for schedule(dynamic, 8) reduction(| : overflow)
    for (int64_t k = 0; k < (int64_t)n_chunks; ++k)
        for (const Cell& c : band[k]) {
            uint64_t up = brick_of(*coef, c.x, c.y, c.z);
            if (up >= coef->grid_occ_size) overflow |= 1;
            else grid_occ[up] = 0;
        }
    if (overflow) {
        std::free(grid_occ);
        set_error("Upper voxel index overflow!");
        return TSDFL_ERR_INVALID_ARG;
    }
    const uint64_t sub3 = coef->sub_dim * coef->sub_dim * coef->sub_dim;
    uint64_t offset = 0;
    for (uint64_t i = 0; i < coef->grid_occ_size; ++i)
        if (grid_occ[i] >= 0) {
            grid_occ[i] = (int32_t)offset;
            offset += sub3;
        }
    if (offset >= (1ull << 31)) {
        std::free(grid_occ);
        set_error("tsdfl_build_map_codes: map has too many slots");
        return TSDFL_ERR_UNSUPPORTED;
    }
    coef->data_size = offset;
    uint16_t* codes = (uint16_t*)std::malloc(sizeof(uint16_t) * (offset + 1));
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)offset; ++i) codes[i] = 600;
    // slot of every band cell (parallel), then the writes in reading order so
    // that the last write wins where two cells share a slot, as in setEntry
    std::vector<std::vector<uint32_t>> slot(n_chunks);
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t k = 0; k < (int64_t)n_chunks; ++k) {
        slot[k].resize(band[k].size());
        for (size_t t = 0; t < band[k].size(); ++t) {
            const Cell& c = band[k][t];
            uint64_t idx = host_slot_index(*coef, grid_occ, c.x, c.y, c.z);
            slot[k][t] = idx < coef->data_size ? (uint32_t)idx : 0xffffffffu;
        }
    }
    for (size_t k = 0; k < n_chunks; ++k)
        for (size_t t = 0; t < band[k].size(); ++t)
            if (slot[k][t] != 0xffffffffu) codes[slot[k][t]] = band[k][t].code;
    if (free_xyz) {
        size_t nf = 0;
        for (auto& f : freep) nf += f.size() / 3;
        float* fp = (float*)std::malloc(sizeof(float) * 3 * (nf + 1));
        size_t o = 0;
        for (auto& f : freep) {
            std::memcpy(fp + o, f.data(), sizeof(float) * f.size());
            o += f.size();
        }
        *free_xyz = fp;
        if (n_free) *n_free = nf;
    }
    *grid_occ_out = grid_occ;
    *codes_out = codes;
    return TSDFL_OK;
}

}  // extern "C"
