// Compares the library's slot-index arithmetic (index_math.h: the signed
// second tier, and a host emulation of the division-free fast path) with the
// oracle's getIndex (oracle/tsdf_oracle.c) on random maps and points,
// including negative, out-of-bounds and special offsets.  Exit status 0 when
// every handled lookup matches; prints counts.
//
// "index_check exhaustive RES..." instead checks the division-free sub-voxel
// index against trunc(s / res) for every float s in [0, 1).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "index_math.h"
#include "map_host.h"

extern "C" {
#include "tsdf_oracle.h"
}

namespace tsdfl {
void set_error(const char*, ...) {}
}
using namespace tsdfl;

static uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
static float fof(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

// fl(x + m) rounded toward zero (add.rz), for x >= 0 (or any x with x + m > 0):
// the exact sum in double, then truncated to float
static float rz_add(float x, float m)
{
    const double d = (double)x + (double)m;
    float f = (float)d;
    if ((double)f > d) f = std::nextafter(f, 0.0f);
    return f;
}

// Division-free sub-voxel index: mode 2 floor of the exact product s * hi;
// mode 1 trunc(fl(fma(s, hi, fl(s * lo)))).
static int64_t fast_sub_index(int mode, float s, float hi, float lo)
{
    if (mode == 2) return (int64_t)std::floor((double)s * (double)hi);
    return (int64_t)std::fmaf(s, hi, s * lo);
}

static int exhaustive(int argc, char** argv)
{
    int fails = 0;
    for (int a = 2; a < argc; ++a) {
        const float res = (float)atof(argv[a]);
        const uint64_t sub_dim = (uint64_t)std::ceil(1.0f / res);
        float inv = 0.0f, lo = 0.0f;
        const int mode = sub_index_mult(res, sub_dim, &inv, &lo);
        long bad = 0;
        if (mode) {
#pragma omp parallel for reduction(+ : bad) schedule(static)
            for (long u = 0; u < (long)fbits(1.0f); ++u) {
                const float s = fof((uint32_t)u);
                const int64_t want = (int64_t)f2u_x86_host(s / res);
                if (fast_sub_index(mode, s, inv, lo) != want) ++bad;
            }
        }
        printf("exhaustive res=%g sub_dim=%llu mode=%d hi=%.9g lo=%.9g bad=%ld\n", res, (unsigned long long)sub_dim,
               mode, inv, lo, bad);
        if (bad || !mode) ++fails;
    }
    return fails ? 1 : 0;
}

int main(int argc, char** argv)
{
    if (argc > 1 && std::strcmp(argv[1], "exhaustive") == 0) return exhaustive(argc, argv);
    long n_points = argc > 1 ? atol(argv[1]) : 2000000;
    const float ress[] = {0.064f, 0.05f, 0.1f, 0.08f, 0.04f};
    const float mins[][3] = {{0, 0, 0}, {-4.096f, -8.192f, -4.096f}, {-10.0f, 3.2f, -0.3f}};
    std::mt19937_64 rng(12345);
    long bad = 0, handled = 0, slow = 0, fast_n = 0, fast_bad = 0;
    for (float res : ress)
        for (auto& mn0 : mins) {
            float mn[3] = {mn0[0], mn0[1], mn0[2]};
            float mx[3] = {mn[0] + 21.3f, mn[1] + 17.7f, mn[2] + 6.1f};
            orc_map_coef c;
            orc_map_coef_init(&c, mn, mx, res, 0.0f);
            std::vector<int32_t> go(c.grid_occ_size);
            int32_t off = 0;
            int32_t S3 = (int32_t)(c.sub_dim * c.sub_dim_2);
            for (auto& g : go) {
                g = (rng() % 3 == 0) ? -1 : off;
                if (g >= 0) off += S3;
            }
            c.data_size = (uint64_t)off;
            MapView v{};
            v.min_x = c.min_x; v.min_y = c.min_y; v.min_z = c.min_z;
            v.res = c.resolution;
            v.mmax_x = coarse_mmax(c.dim_x, res); v.mmax_y = coarse_mmax(c.dim_y, res); v.mmax_z = coarse_mmax(c.dim_z, res);
            auto lim = [](int32_t mm) { return mm < 0 ? 0u : fbits((float)std::min<int64_t>((int64_t)mm + 1, 4194304)); };
            v.lim_x = lim(v.mmax_x); v.lim_y = lim(v.mmax_y); v.lim_z = lim(v.mmax_z);
            v.up_dim_x = (uint32_t)c.up_dim_x; v.up_dim_2 = (uint32_t)c.up_dim_2; v.grid_occ_size = (uint32_t)c.grid_occ_size;
            v.sub_dim = (uint32_t)c.sub_dim; v.sub_dim_2 = (uint32_t)c.sub_dim_2; v.sub_dim_3 = (uint32_t)S3;
            v.data_size = (uint32_t)c.data_size;
            v.dim_x = c.dim_x; v.dim_y = c.dim_y; v.dim_z = c.dim_z;
            v.up_dim_x64 = c.up_dim_x; v.up_dim_2_64 = c.up_dim_2; v.grid_occ_size64 = c.grid_occ_size;
            v.sub_dim64 = c.sub_dim; v.sub_dim_2_64 = c.sub_dim_2; v.data_size64 = c.data_size;
            v.sub_fast = sub_index_mult(res, c.sub_dim, &v.sub_inv, &v.sub_inv_lo);
            // the tiled path's conditions and constants (fill_view): compact
            // bitmap pairs {word, allocated bricks up to and including it}
            const uint32_t v_lim_x = v.lim_x, v_lim_y = v.lim_y;
            const float zhi = v.mmax_z < 0 ? 0.0f : (float)std::min<int64_t>((int64_t)v.mmax_z + 1, 4194304);
            const float zlo = v.mmax_z < 0 ? 0.0f : -1.0f;
            float below_one = fof(0x3F7FFFFFu);
            const bool tiled = v.sub_fast != 0 && (uint64_t)S3 <= (1ull << 21) && c.grid_occ_size < (1ull << 22) &&
                               f2u_x86_host(below_one / res) < c.sub_dim;
            const uint64_t words = (c.grid_occ_size + 31) / 32;
            uint64_t occ_bytes = 16;
            while (occ_bytes < 8 * words) occ_bytes *= 2;
            const uint32_t occ_mask = (uint32_t)(occ_bytes - 1) & ~7u;
            std::vector<uint32_t> occ(occ_bytes / 4, 0u);
            for (uint64_t u = 0; u < c.grid_occ_size; ++u)
                if (go[u] >= 0) occ[2 * (u / 32)] |= 1u << (u % 32);
            for (uint64_t w = 0, run = 0; w < words; ++w) {
                run += (uint32_t)__builtin_popcount(occ[2 * w]);
                occ[2 * w + 1] = (uint32_t)run;
            }
            std::uniform_real_distribution<float> U(-3.5f, 25.0f);
            const float special[] = {-1.0f, -0.99999994f, -0.5f, -0.0f, 0.0f, 1e-30f, 0.99999994f, 1.0f, -2.0f, -1e-7f};
            for (long i = 0; i < n_points; ++i) {
                float o[3];
                for (int a = 0; a < 3; ++a) {
                    uint64_t r = rng();
                    if (r % 17 == 0) o[a] = special[(r >> 8) % 10];
                    else if (r % 17 == 1) o[a] = (float)((int)((r >> 8) % 30)) + ((r >> 40) % 2 ? -1e-6f : 1e-6f);
                    else o[a] = U(rng);
                }
                if (i % 1000 == 0) o[i / 1000 % 3] = (i / 3000) % 2 ? NAN : 1e20f;
                float x = mn[0] + o[0], y = mn[1] + o[1], z = mn[2] + o[2];
                // the offsets the device computes: point - min, rounded once
                float ox = x - mn[0], oy = y - mn[1], oz = z - mn[2];
                uint64_t ref = orc_get_index(&c, go.data(), x, y, z);
                uint32_t want = ref < c.data_size ? (uint32_t)ref : kIdxMiss;
                uint32_t t2 = slot_index_tier2(v, go.data(), ox, oy, oz);
                if (t2 == kIdxSlow) { ++slow; continue; }
                ++handled;
                if (t2 != want) {
                    if (bad < 10) printf("tier2 mismatch res=%g o=(%.9g %.9g %.9g) got %u want %u\n", res, ox, oy, oz, t2, want);
                    ++bad;
                }
                // the tiled kernels' packed pipeline, operation by operation (float
                // sums whose bits are the biased brick and sub-voxel offsets), for
                // both layouts: the bitmap rank (compact) and the brick table
                if (tiled) {
                    const bool fast = fbits(ox) < v_lim_x && fbits(oy) < v_lim_y && oz > zlo && oz < zhi;
                    if (!fast) goto next;
                    ++fast_n;
                    const float az = std::fabs(oz);
                    const float MX = rz_add(ox, 8388608.0f), MY = rz_add(oy, 8388608.0f), MZ = rz_add(az, 8388608.0f);
                    const float FY = MY - 8388608.0f, FZ = MZ - 8388608.0f;
                    const float SX = ox - (MX - 8388608.0f), SY = oy - FY, SZ = az - FZ;
                    auto cq = [&](float s_) {   // 1.5 2^23 + q(s)
                        if (v.sub_fast == 2) return 12582912.0f + (float)std::floor((double)s_ * (double)v.sub_inv);
                        return rz_add(std::fmaf(s_, v.sub_inv, s_ * v.sub_inv_lo), 12582912.0f);
                    };
                    const float CX = cq(SX), CY = cq(SY), CZ = cq(SZ);
                    const float QY = CY - 12582912.0f, QZ = std::copysign(CZ - 12582912.0f, oz);
                    const float SLB = std::fmaf(QZ, (float)c.sub_dim_2, std::fmaf(QY, (float)c.sub_dim, CX));
                    const float UPB = std::fmaf(FZ, (float)c.up_dim_2, std::fmaf(FY, (float)c.up_dim_x, MX));
                    const uint32_t upb = fbits(UPB), slb = fbits(SLB);
                    const bool inside = upb < 0x4B000000u + (uint32_t)c.grid_occ_size;
                    for (int layout = 0; layout < 2; ++layout) {
                        uint32_t idx;
                        bool ok;
                        if (layout == 0) {   // compact: rank from the bitmap
                            const uint32_t off = (upb >> 2) & occ_mask;
                            const uint32_t word = occ[off / 4], incl = occ[off / 4 + 1];
                            const uint32_t vv = word >> (upb & 31u);
                            ok = inside && (vv & 1u);
                            idx = (incl - (uint32_t)__builtin_popcount(vv)) * (uint32_t)S3 + slb;
                        } else {             // brick table
                            const int32_t base = go[inside ? upb - 0x4B000000u : 0u];
                            ok = inside && base >= 0;
                            idx = (uint32_t)base + slb;
                        }
                        // slot indices below 0 read the leading brick of misses
                        const int64_t slot = (int64_t)idx - 0x4B400000ll;
                        const uint32_t got = ok && slot >= 0 ? (uint32_t)slot : kIdxMiss;
                        if (got != want) {
                            if (fast_bad < 10)
                                printf("fast mismatch layout=%d res=%g o=(%.9g %.9g %.9g) got %u want %u\n", layout, res,
                                       ox, oy, oz, got, want);
                            ++fast_bad;
                        }
                    }
                }
            next:;
            }
        }
    printf("handled %ld slow %ld tier2_bad %ld fast %ld fast_bad %ld\n", handled, slow, bad, fast_n, fast_bad);
    return (bad || fast_bad) ? 1 : 0;
}
