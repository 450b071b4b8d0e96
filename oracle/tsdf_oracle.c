/*
 * TEST INFRASTRUCTURE ONLY -- NOT PART OF THE PRODUCT.
 *
 * CPU restatement of the uos/tsdf_localization sensor update (the oracle).
 * Every function cites the reference lines it restates.  Build flags (see
 * oracle/Makefile): -O2 -ffp-contract=off -fopenmp, no -march, no fast-math,
 * so float expressions round exactly as written on both x86-64 and aarch64.
 *
 * Two platform-dependent points of the reference are pinned here:
 *  - float -> size_t conversions are out of range for negative or huge map
 *    offsets; the reference's Release build on x86-64 gives the cvttss2si
 *    results, which orc_f2u_x86 reproduces with integer code.
 *  - sin/cos/atan2 of float arguments bind to the double-precision libm
 *    functions (the result rounded to float), i.e. the correctly rounded value.
 */
#include "tsdf_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#define TWO63F 9223372036854775808.0f
#define SIGN64 0x8000000000000000ull

uint64_t orc_f2u_x86(float v)
{
    if (v != v) return SIGN64;                        /* cvttss2si of NaN: integer indefinite */
    if (v < TWO63F) {
        if (v >= -TWO63F) return (uint64_t)(int64_t)v; /* truncation, two's complement wrap */
        return SIGN64;
    }
    float w = v - TWO63F;                             /* exact: both multiples of 2^40 */
    if (w < TWO63F) return ((uint64_t)(int64_t)w) ^ SIGN64;
    return 0;                                         /* indefinite ^ sign bit */
}

uint64_t orc_d2u_x86(double v)
{
    const double two63 = 9223372036854775808.0;
    if (v != v) return SIGN64;                        /* cvttsd2si of NaN: integer indefinite */
    if (v < two63) {
        if (v >= -two63) return (uint64_t)(int64_t)v;  /* truncation, two's complement wrap */
        return SIGN64;
    }
    double w = v - two63;                             /* exact for these magnitudes */
    if (w < two63) return ((uint64_t)(int64_t)w) ^ SIGN64;
    return 0;
}

/* cuda_sub_voxel_map.tcc:4-48 */
void orc_map_coef_init(orc_map_coef* c, const float mn[3], const float mx[3],
                       float resolution, float init_value)
{
    memset(c, 0, sizeof(*c));
    c->dim_x = (uint64_t)ceilf(fabsf(mx[0] - mn[0]) / resolution);
    c->dim_y = (uint64_t)ceilf(fabsf(mx[1] - mn[1]) / resolution);
    c->dim_z = (uint64_t)ceilf(fabsf(mx[2] - mn[2]) / resolution);
    c->min_x = mn[0]; c->min_y = mn[1]; c->min_z = mn[2];
    c->max_x = mx[0]; c->max_y = mx[1]; c->max_z = mx[2];
    c->resolution = resolution;
    c->init_value = init_value;
    c->up_dim_x = (uint64_t)ceilf(fabsf(mx[0] - mn[0]) / 1.0f);
    c->up_dim_y = (uint64_t)ceilf(fabsf(mx[1] - mn[1]) / 1.0f);
    c->up_dim_z = (uint64_t)ceilf(fabsf(mx[2] - mn[2]) / 1.0f);
    c->up_dim_2 = c->up_dim_x * c->up_dim_y;
    c->sub_dim = (uint64_t)ceilf(1.0f / resolution);
    c->sub_dim_2 = c->sub_dim * c->sub_dim;
    c->grid_occ_size = c->up_dim_x * c->up_dim_y * c->up_dim_z;
    c->data_size = 0;
}

/* cuda_sub_voxel_map.tcc:50-137 (track_reuse_ off, as on the evaluation path) */
uint64_t orc_get_index(const orc_map_coef* c, const int32_t* grid_occ, float x, float y, float z)
{
    uint64_t gx = orc_f2u_x86(x - c->min_x);
    uint64_t gy = orc_f2u_x86(y - c->min_y);
    uint64_t gz = orc_f2u_x86(z - c->min_z);
    gx = orc_f2u_x86((float)gx / c->resolution);
    gy = orc_f2u_x86((float)gy / c->resolution);
    gz = orc_f2u_x86((float)gz / c->resolution);
    if (gx >= c->dim_x || gy >= c->dim_y || gz >= c->dim_z) return c->data_size;

    float ox = x - c->min_x, oy = y - c->min_y, oz = z - c->min_z;
    uint64_t ux = orc_f2u_x86(ox / 1.0f);
    uint64_t uy = orc_f2u_x86(oy / 1.0f);
    uint64_t uz = orc_f2u_x86(oz / 1.0f);
    float sx = ox - (float)ux * 1.0f;
    float sy = oy - (float)uy * 1.0f;
    float sz = oz - (float)uz * 1.0f;
    uint64_t up = ux + uy * c->up_dim_x + uz * c->up_dim_2;
    if (up >= c->grid_occ_size) return c->data_size;
    int32_t base = grid_occ[up];
    if (base < 0) return c->data_size;
    uint64_t qx = orc_f2u_x86(sx / c->resolution);
    uint64_t qy = orc_f2u_x86(sy / c->resolution);
    uint64_t qz = orc_f2u_x86(sz / c->resolution);
    return (uint64_t)(int64_t)base + qx + qy * c->sub_dim + qz * c->sub_dim_2;
}

/* cuda_sub_voxel_map.tcc:139-157 */
float orc_get_entry(const orc_map_coef* c, const int32_t* grid_occ, const float* data,
                    float x, float y, float z)
{
    if (data == NULL || grid_occ == NULL) return c->init_value;
    uint64_t i = orc_get_index(c, grid_occ, x, y, z);
    return i < c->data_size ? data[i] : c->init_value;
}

/* cuda_sub_voxel_map.tcc:170-230 */
int orc_map_set_data(orc_map_coef* c, int32_t* grid_occ, const float* xyzv, size_t n,
                     float** data_out, size_t* skipped)
{
    *data_out = NULL;
    if (skipped) *skipped = 0;
    for (uint64_t i = 0; i < c->grid_occ_size; ++i) grid_occ[i] = -1;
    if (n == 0) return 0;
    for (size_t t = 0; t < n; ++t) {
        const float* cell = xyzv + 4 * t;
        uint64_t ux = orc_f2u_x86((cell[0] - c->min_x) / 1.0f);
        uint64_t uy = orc_f2u_x86((cell[1] - c->min_y) / 1.0f);
        uint64_t uz = orc_f2u_x86((cell[2] - c->min_z) / 1.0f);
        uint64_t up = ux + uy * c->up_dim_x + uz * c->up_dim_x * c->up_dim_y;
        if (up >= c->grid_occ_size) return -1; /* "Upper voxel index overflow!" */
        grid_occ[up] = 0;
    }
    int32_t offset = 0;
    int32_t sub_size = (int32_t)(c->sub_dim * c->sub_dim * c->sub_dim);
    for (uint64_t i = 0; i < c->grid_occ_size; ++i) {
        if (grid_occ[i] >= 0) { grid_occ[i] = offset; offset += sub_size; }
    }
    c->data_size = (uint64_t)offset;
    float* data = (float*)malloc(sizeof(float) * (c->data_size ? c->data_size : 1));
    for (uint64_t i = 0; i < c->data_size; ++i) data[i] = c->init_value;
    for (size_t t = 0; t < n; ++t) {
        const float* cell = xyzv + 4 * t;
        uint64_t i = orc_get_index(c, grid_occ, cell[0], cell[1], cell[2]);
        if (i < c->data_size) data[i] = cell[3];
        else if (skipped) ++*skipped;   /* the reference writes data_[data_size]: not reproduced */
    }
    *data_out = data;
    return 0;
}

static inline float trig_sin(float a) { return (float)sin((double)a); }
static inline float trig_cos(float a) { return (float)cos((double)a); }

/* tsdf_evaluator.cpp:102-147 */
void orc_particle_pose(const float p[7], const float tf[16], float tl[12])
{
    float alpha = p[3], beta = p[4], gamma = p[5];
    float sin_alpha = trig_sin(alpha), cos_alpha = trig_cos(alpha);
    float sin_beta = trig_sin(beta), cos_beta = trig_cos(beta);
    float sin_gamma = trig_sin(gamma), cos_gamma = trig_cos(gamma);
    float t[12];
    t[0] = cos_beta * cos_gamma;
    t[4] = cos_beta * sin_gamma;
    t[8] = -sin_beta;
    t[3] = p[0];
    t[1] = sin_alpha * sin_beta * cos_gamma - cos_alpha * sin_gamma;
    t[5] = sin_alpha * sin_beta * sin_gamma + cos_alpha * cos_gamma;
    t[9] = sin_alpha * cos_beta;
    t[7] = p[1];
    t[2] = cos_alpha * sin_beta * cos_gamma + sin_alpha * sin_gamma;
    t[6] = cos_alpha * sin_beta * sin_gamma - sin_alpha * cos_gamma;
    t[10] = cos_alpha * cos_beta;
    t[11] = p[2];
    for (int r = 0; r < 3; ++r) {
        const float* a = t + 4 * r;
        tl[4 * r + 0] = a[0] * tf[0] + a[1] * tf[4] + a[2] * tf[8];
        tl[4 * r + 1] = a[0] * tf[1] + a[1] * tf[5] + a[2] * tf[9];
        tl[4 * r + 2] = a[0] * tf[2] + a[1] * tf[6] + a[2] * tf[10];
        tl[4 * r + 3] = a[0] * tf[3] + a[1] * tf[7] + a[2] * tf[11] + a[3];
    }
}

/* tsdf_evaluator.cpp:78-245; the point loop is evaluatePose, :27-76 */
int orc_evaluate(const orc_map_coef* c, const int32_t* grid_occ, const float* data,
                 const orc_model* m, float* particles, size_t P,
                 const float* points, size_t N, const float tf[16],
                 float* raw_out, uint32_t* hits_out, uint64_t* idx_out,
                 double* sum64_out, float pose_out[6], int n_threads)
{
    const float a_hit = m->a_hit, a_range = m->a_range, a_max = m->a_max;
    const float inv_max_range = (float)(1.0 / (double)m->max_range);
    const float max_range_squared = m->max_range * m->max_range;
    const int have_map = (data != NULL && grid_occ != NULL);
    float* raw = (float*)malloc(sizeof(float) * (P ? P : 1));

    const int nt = n_threads > 0 ? n_threads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic) num_threads(nt)
    for (size_t i = 0; i < P; ++i) {
        float tl[12];
        orc_particle_pose(particles + 7 * i, tf, tl);
        float eval_sum = 0.0f;
        double sum64 = 0.0;
        uint32_t hits = 0;
        for (size_t j = 0; j < N; ++j) {
            float x = points[3 * j], y = points[3 * j + 1], z = points[3 * j + 2];
            float tx = tl[0] * x + tl[1] * y + tl[2] * z + tl[3];
            float ty = tl[4] * x + tl[5] * y + tl[6] * z + tl[7];
            float tz = tl[8] * x + tl[9] * y + tl[10] * z + tl[11];
            uint64_t idx = have_map ? orc_get_index(c, grid_occ, tx, ty, tz) : c->data_size;
            float value = c->init_value;
            if (idx < c->data_size) { value = data[idx]; ++hits; }
            if (idx_out) idx_out[i * N + j] = idx;
            float square_dist = x * x + y * y + z * z;
            if (square_dist < max_range_squared) value = a_hit * value + a_range * inv_max_range;
            else value = a_hit * value + a_max;
            eval_sum += value;
            sum64 += (double)value;
        }
        raw[i] = eval_sum;
        if (raw_out) raw_out[i] = eval_sum;
        if (hits_out) hits_out[i] = hits;
        if (sum64_out) sum64_out[i] = sum64;
    }

    float weight_sum = 0.0f;
    for (size_t i = 0; i < P; ++i) weight_sum += raw[i];
    if (weight_sum == 0.0f) { free(raw); return 1; }   /* "No particle is valid!" */

    float avg_x = 0, avg_y = 0, avg_z = 0;
    float sum_sin_roll = 0, sum_cos_roll = 0, sum_sin_pitch = 0, sum_cos_pitch = 0;
    float sum_sin_yaw = 0, sum_cos_yaw = 0;
    for (size_t i = 0; i < P; ++i) {
        float* p = particles + 7 * i;
        p[6] = raw[i] / weight_sum;
        avg_x += p[0] * p[6];
        avg_y += p[1] * p[6];
        avg_z += p[2] * p[6];
        sum_sin_roll = (float)((double)sum_sin_roll + sin((double)p[3]) * (double)p[6]);
        sum_cos_roll = (float)((double)sum_cos_roll + cos((double)p[3]) * (double)p[6]);
        sum_sin_pitch = (float)((double)sum_sin_pitch + sin((double)p[4]) * (double)p[6]);
        sum_cos_pitch = (float)((double)sum_cos_pitch + cos((double)p[4]) * (double)p[6]);
        sum_sin_yaw = (float)((double)sum_sin_yaw + sin((double)p[5]) * (double)p[6]);
        sum_cos_yaw = (float)((double)sum_cos_yaw + cos((double)p[5]) * (double)p[6]);
    }
    if (pose_out) {
        pose_out[0] = avg_x; pose_out[1] = avg_y; pose_out[2] = avg_z;
        pose_out[3] = (float)atan2((double)sum_sin_roll, (double)sum_cos_roll);
        pose_out[4] = (float)atan2((double)sum_sin_pitch, (double)sum_cos_pitch);
        pose_out[5] = (float)atan2((double)sum_sin_yaw, (double)sum_cos_yaw);
    }
    free(raw);
    return 0;
}

/* map_util.h:124-127 */
float orc_likelihood_value(int16_t tsdf_mm, float sigma)
{
    float sigma_quad = sigma * sigma;
    float tsdf_value = (float)tsdf_mm;
    double value = (double)tsdf_value * 0.001;
    value = (double)(expf((float)(-(value * value) / (double)sigma_quad / 2))
                     / sqrtf((float)((double)(2 * sigma_quad) * M_PI)));
    value = value * value * value;
    return (float)value;
}

/* map_util.h:68-71 */
float orc_likelihood_init(float sigma)
{
    float sigma_quad = sigma * sigma;
    float init = expf((float)(-(10.0 * 10.0) / (double)sigma_quad / 2))
                 / sqrtf((float)((double)(2 * sigma_quad) * M_PI));
    init = init * init * init;
    return init;
}

typedef struct { char name[48]; size_t index; } chunk_tag;

static int cmp_tag(const void* a, const void* b)
{
    return strcmp(((const chunk_tag*)a)->name, ((const chunk_tag*)b)->name);
}

/* map_util.h:17-151 up to the setData call (HighFive lists "/map" members in
 * increasing name order): the bounding box, the init value, the (x, y, z, value)
 * tuples of touched cells with |tsdf| < 600 and the free-space cells, in the
 * order the reference pushes them.  CH is the reference's CHUNK_SIZE. */
static void chunk_tuples(const int32_t* chunk_pos, const uint32_t* chunks, size_t n_chunks, int CH,
                         int voxel_mm, float sigma, float mn[3], float mx[3], float* init_out,
                         float** tuples_out, size_t* n_out, float** free_out, size_t* nf_out)
{
    mn[0] = mn[1] = mn[2] = 0.0f;
    mx[0] = mx[1] = mx[2] = 0.0f;
    for (size_t k = 0; k < n_chunks; ++k)
        for (int a = 0; a < 3; ++a) {
            int coord = chunk_pos[3 * k + a];
            if ((float)coord < mn[a]) mn[a] = (float)coord;
            if ((float)coord > mx[a]) mx[a] = (float)coord;
        }
    for (int a = 0; a < 3; ++a) {
        mn[a] = (float)((double)(mn[a] * (float)CH * (float)voxel_mm) * 0.001);
        mx[a] = (float)((double)((mx[a] * (float)CH + (float)CH) * (float)voxel_mm) * 0.001);
    }
    *init_out = orc_likelihood_init(sigma);

    float lut[600];
    for (int v = 0; v < 600; ++v) lut[v] = orc_likelihood_value((int16_t)v, sigma);

    chunk_tag* tags = (chunk_tag*)malloc(sizeof(chunk_tag) * (n_chunks ? n_chunks : 1));
    for (size_t k = 0; k < n_chunks; ++k) {
        snprintf(tags[k].name, sizeof(tags[k].name), "%d_%d_%d",
                 chunk_pos[3 * k], chunk_pos[3 * k + 1], chunk_pos[3 * k + 2]);
        tags[k].index = k;
    }
    qsort(tags, n_chunks, sizeof(chunk_tag), cmp_tag);

    size_t cap = 1 << 16, n = 0, fcap = 1 << 16, nf = 0;
    float* tuples = (float*)malloc(sizeof(float) * 4 * cap);
    float* freep = (float*)malloc(sizeof(float) * 3 * fcap);
    for (size_t t = 0; t < n_chunks; ++t) {
        size_t k = tags[t].index;
        const uint32_t* raw = chunks + (size_t)k * (size_t)(CH * CH * CH);
        const int32_t* cp = chunk_pos + 3 * k;
        for (int i = 0; i < CH; i++)
            for (int j = 0; j < CH; j++)
                for (int l = 0; l < CH; l++) {
                    uint32_t e = raw[CH * CH * i + CH * j + l];
                    int16_t val = (int16_t)(uint16_t)(e & 0xffffu);
                    int16_t wgt = (int16_t)(uint16_t)(e >> 16);
                    float tsdf_value = (float)val;
                    if (wgt == 0) continue;
                    int x = CH * cp[0] + i, y = CH * cp[1] + j, z = CH * cp[2] + l;
                    float px = (float)((double)((float)x * (float)voxel_mm) * 0.001);
                    float py = (float)((double)((float)y * (float)voxel_mm) * 0.001);
                    float pz = (float)((double)((float)z * (float)voxel_mm) * 0.001);
                    if (fabsf(tsdf_value) < 600.0f) {
                        if (n == cap) { cap *= 2; tuples = (float*)realloc(tuples, sizeof(float) * 4 * cap); }
                        int av = val < 0 ? -val : val;
                        tuples[4 * n] = px; tuples[4 * n + 1] = py; tuples[4 * n + 2] = pz;
                        tuples[4 * n + 3] = lut[av];
                        ++n;
                    } else {
                        if (nf == fcap) { fcap *= 2; freep = (float*)realloc(freep, sizeof(float) * 3 * fcap); }
                        freep[3 * nf] = px; freep[3 * nf + 1] = py; freep[3 * nf + 2] = pz;
                        ++nf;
                    }
                }
    }
    free(tags);
    *tuples_out = tuples;
    *n_out = n;
    *free_out = freep;
    *nf_out = nf;
}

size_t orc_chunk_tuples(const int32_t* chunk_pos, const uint32_t* chunks, size_t n_chunks, int edge,
                        int voxel_mm, float sigma, float mn[3], float mx[3], float* init_out,
                        float** tuples_out, float** free_xyz_out, size_t* n_free_out)
{
    size_t n = 0;
    chunk_tuples(chunk_pos, chunks, n_chunks, edge, voxel_mm, sigma, mn, mx, init_out, tuples_out, &n,
                 free_xyz_out, n_free_out);
    return n;
}

/* map_util.h:17-154: the tuples above, then the CudaSubVoxelMap ctor
 * (map_util.h:73) and setData (:151). */
int orc_build_map_from_chunks(const int32_t* chunk_pos, const uint32_t* chunks, size_t n_chunks, int edge,
                              int voxel_mm, float sigma, orc_map_coef* c, int32_t** grid_occ_out,
                              float** data_out, float** free_xyz_out, size_t* n_free_out)
{
    float mn[3], mx[3], init;
    float* tuples = NULL;
    size_t n = 0;
    chunk_tuples(chunk_pos, chunks, n_chunks, edge, voxel_mm, sigma, mn, mx, &init, &tuples, &n, free_xyz_out,
                 n_free_out);
    orc_map_coef_init(c, mn, mx, (float)(voxel_mm * 0.001), init);
    int32_t* grid_occ = (int32_t*)malloc(sizeof(int32_t) * (c->grid_occ_size ? c->grid_occ_size : 1));
    float* data = NULL;
    int rc = orc_map_set_data(c, grid_occ, tuples, n, &data, NULL);
    free(tuples);
    *grid_occ_out = grid_occ;
    *data_out = data;
    return rc;
}

/* novel_resampling.h:41-72 */
size_t orc_resample_systematic(const float* w, size_t M, float U0, uint32_t* idx_out, size_t cap)
{
    double inverse_M = 1.0 / (double)M;
    float U = U0;
    double s = 0.0;
    size_t n = 0;
    for (size_t m = 0; m < M; ++m) {
        s += (double)w[m];
        while (s > (double)U) {
            if (n < cap) idx_out[n] = (uint32_t)m;
            ++n;
            float next = (float)((double)U + inverse_M);
            if (next == U) return (size_t)-1;   /* the reference would loop forever */
            U = next;
        }
    }
    return n;
}

/* novel_resampling.h:76-104 */
size_t orc_resample_residual_systematic(const float* w, size_t M, float u0, uint32_t* idx_out, size_t cap)
{
    const float Mf = (float)M;                        /* size_t * float converts M to float */
    float u = u0;
    size_t n = 0;
    for (size_t m = 0; m < M; ++m) {
        float temp = Mf * w[m] - u;                   /* float product and difference */
        uint64_t o = orc_d2u_x86((double)temp + 1.0);
        if (o >= (1ull << 32)) return (size_t)-1;
        u = (float)o - temp;                          /* size_t - float: o converted to float */
        for (uint64_t k = 0; k < o; ++k) {
            if (n < cap) idx_out[n] = (uint32_t)m;
            ++n;
        }
    }
    return n;
}

/* tsdf_evaluator.cpp:300-376 */
typedef struct {
    int32_t ring, index;
    float cx, cy, cz;
    size_t src;
} orc_scan_pt;

static int orc_scan_key_cmp(const void* a, const void* b)
{
    const orc_scan_pt* p = (const orc_scan_pt*)a;
    const orc_scan_pt* q = (const orc_scan_pt*)b;
    uint32_t pb[3], qb[3];
    memcpy(&pb[0], &p->cx, 4); memcpy(&pb[1], &p->cy, 4); memcpy(&pb[2], &p->cz, 4);
    memcpy(&qb[0], &q->cx, 4); memcpy(&qb[1], &q->cy, 4); memcpy(&qb[2], &q->cz, 4);
    if (p->ring != q->ring) return p->ring < q->ring ? -1 : 1;
    for (int k = 0; k < 3; ++k)
        if (pb[k] != qb[k]) return pb[k] < qb[k] ? -1 : 1;
    return p->index < q->index ? -1 : (p->index > q->index ? 1 : 0);
}

static int orc_scan_out_cmp(const void* a, const void* b)
{
    const orc_scan_pt* p = (const orc_scan_pt*)a;
    const orc_scan_pt* q = (const orc_scan_pt*)b;
    if (p->ring != q->ring) return p->ring < q->ring ? -1 : 1;
    return p->index < q->index ? -1 : (p->index > q->index ? 1 : 0);
}

size_t orc_reduce_scan(const float* xyz, const int16_t* ring, size_t n, float cell, int own_ring, float* out,
                       size_t cap)
{
    const float half = cell / 2;
    orc_scan_pt* pts = (orc_scan_pt*)malloc(sizeof(orc_scan_pt) * (n ? n : 1));
    size_t k = 0;
    for (size_t i = 0; i < n; ++i) {
        const float x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
        const float dist = sqrtf(x * x + y * y + z * z);
        if (dist < 1.0) continue;
        orc_scan_pt p;
        p.ring = own_ring ? ring[i] : ring[k];   /* the ring iterator advances once per kept point */
        p.index = (int32_t)k;
        p.cx = floorf(x / cell) * cell + half;
        p.cy = floorf(y / cell) * cell + half;
        p.cz = floorf(z / cell) * cell + half;
        p.src = i;
        if (p.ring < 0 || p.ring >= 64) { free(pts); return (size_t)-1; }
        pts[k++] = p;
    }
    /* first (lowest index) of every (ring, centre); NaN centres never compare equal */
    qsort(pts, k, sizeof(orc_scan_pt), orc_scan_key_cmp);
    size_t m = 0;
    for (size_t t = 0; t < k; ++t) {
        int nan = pts[t].cx != pts[t].cx || pts[t].cy != pts[t].cy || pts[t].cz != pts[t].cz;
        if (t > 0 && !nan && pts[t].ring == pts[t - 1].ring && pts[t].cx == pts[t - 1].cx &&
            pts[t].cy == pts[t - 1].cy && pts[t].cz == pts[t - 1].cz)
            continue;
        pts[m++] = pts[t];
    }
    qsort(pts, m, sizeof(orc_scan_pt), orc_scan_out_cmp);
    for (size_t t = 0; t < m && t < cap; ++t) memcpy(out + 3 * t, xyz + 3 * pts[t].src, 12);
    free(pts);
    return m;
}

/* util.cpp:86-111, getAngleFromMat; unqualified fabs/atan2/asin/cos on floats
 * bind to the double functions in the reference's build. */
static void orc_angles_from_mat(const float m[16], float* roll, float* pitch, float* yaw)
{
    if (fabs((double)m[8]) >= 1) {
        *yaw = 0;
        double delta = atan2((double)m[9], (double)m[10]);
        *pitch = m[8] < 0 ? (float)(M_PI / 2.0) : (float)(-M_PI / 2.0);
        *roll = (float)delta;
    } else {
        *pitch = (float)(-asin((double)m[8]));
        *roll = (float)atan2((double)m[9] / cos((double)*pitch), (double)m[10] / cos((double)*pitch));
        *yaw = (float)atan2((double)m[4] / cos((double)*pitch), (double)m[0] / cos((double)*pitch));
    }
}

/* particle_cloud.cpp:530-614 */
void orc_motion_apply(float* particles, size_t P, const double* draws)
{
    for (size_t i = 0; i < P; ++i) {
        float* p = particles + 7 * i;
        const double* d = draws + 6 * i;
        float sr = (float)sin(d[3]), cr = (float)cos(d[3]);
        float sp = (float)sin(d[4]), cp = (float)cos(d[4]);
        float sy = (float)sin(d[5]), cy = (float)cos(d[5]);
        float o[16], q[16], t[16];
        o[0] = cp * cy;
        o[4] = cp * sy;
        o[8] = -sp;
        o[3] = (float)d[0];
        o[1] = sr * sp * cy - cr * sy;
        o[5] = sr * sp * sy + cr * cy;
        o[9] = sr * cp;
        o[7] = (float)d[1];
        o[2] = cr * sp * cy + sr * sy;
        o[6] = cr * sp * sy - sr * cy;
        o[10] = cr * cp;
        o[11] = (float)d[2];
        float sa = (float)sin((double)p[3]), ca = (float)cos((double)p[3]);
        float sb = (float)sin((double)p[4]), cb = (float)cos((double)p[4]);
        float sg = (float)sin((double)p[5]), cg = (float)cos((double)p[5]);
        q[0] = cb * cg;
        q[4] = cb * sg;
        q[8] = -sb;
        q[3] = 0;
        q[1] = sa * sb * cg - ca * sg;
        q[5] = sa * sb * sg + ca * cg;
        q[9] = sa * cb;
        q[7] = 0;
        q[2] = ca * sb * cg + sa * sg;
        q[6] = ca * sb * sg - sa * cg;
        q[10] = ca * cb;
        q[11] = 0;
        for (int r = 0; r < 3; ++r) {
            t[4 * r] = q[4 * r] * o[0] + q[4 * r + 1] * o[4] + q[4 * r + 2] * o[8];
            t[4 * r + 1] = q[4 * r] * o[1] + q[4 * r + 1] * o[5] + q[4 * r + 2] * o[9];
            t[4 * r + 2] = q[4 * r] * o[2] + q[4 * r + 1] * o[6] + q[4 * r + 2] * o[10];
            t[4 * r + 3] = q[4 * r] * o[3] + q[4 * r + 1] * o[7] + q[4 * r + 2] * o[11] + q[4 * r + 3];
        }
        float roll, pitch, yaw;
        orc_angles_from_mat(t, &roll, &pitch, &yaw);
        p[0] = p[0] + t[3];
        p[1] = p[1] + t[7];
        p[2] = p[2] + t[11];
        p[3] = roll;
        p[4] = pitch;
        p[5] = yaw;
    }
}

/* wheel_resampler.cpp:13-30 */
void orc_resample_wheel(const float* w, size_t M, const double* draws, uint32_t* idx)
{
    for (size_t i = 0; i < M; ++i) {
        float random_value = (float)draws[i];
        float weight_sum = 0.0f;
        idx[i] = (uint32_t)i;
        for (size_t m = 0; m < M; ++m) {
            weight_sum += w[m];
            if (random_value <= weight_sum) {
                idx[i] = (uint32_t)m;
                break;
            }
        }
    }
}

/* novel_resampling.h:14-31 */
size_t orc_resample_residual(const float* w, size_t M, const uint32_t* draws, size_t K, uint32_t* idx)
{
    size_t filled = 0, used = 0;
    while (filled < M) {
        if (used >= K) return (size_t)-1;
        size_t r = draws[used++];
        float expected = w[r] * (float)M;
        size_t left = M - filled;
        float insertions = expected <= (float)left ? expected : (float)left;
        for (size_t k = 0; (float)k < insertions; ++k) idx[filled++] = (uint32_t)r;
    }
    return used;
}

/* novel_resampling.h:118-139: particle_k stays particle 0 */
void orc_resample_metropolis(const float* w, size_t M, uint32_t steps, const float* u, const uint32_t* j,
                             uint32_t* idx)
{
    for (size_t i = 0; i < M; ++i) {
        size_t k = 0;
        for (uint32_t n = 0; n < steps; ++n) {
            float un = u[i * steps + n];
            uint32_t jn = j[i * steps + n];
            if (un <= w[jn] / w[0]) k = jn;
        }
        idx[i] = (uint32_t)k;
    }
}

/* novel_resampling.h:158-183 */
int orc_resample_rejection(const float* w, size_t M, orc_draw_u_fn du, orc_draw_j_fn dj, void* src,
                           uint32_t max_rounds, uint32_t* idx)
{
    double sup_w = 0.0;
    for (size_t m = 0; m < M; ++m)
        if (sup_w < w[m]) sup_w = w[m];
    int rc = 0;
    for (size_t i = 0; i < M; ++i) {
        size_t j = i;
        float u = du(src, i, 0);
        uint32_t t = 1;
        while (u > (w[j] / sup_w)) {
            if (t > max_rounds) {
                rc = -1;
                break;
            }
            j = dj(src, i, t);
            u = du(src, i, t);
            ++t;
        }
        idx[i] = (uint32_t)j;
    }
    return rc;
}

void orc_philox4x64_10(uint64_t c[4], uint64_t k0, uint64_t k1)
{
    const uint64_t m0 = 0xD2E7470EE14C6C93ull, m1 = 0xCA5A826395121157ull;
    const uint64_t w0 = 0x9E3779B97F4A7C15ull, w1 = 0xBB67AE8584CAA73Bull;
    for (int r = 0; r < 10; ++r) {
        unsigned __int128 p0 = (unsigned __int128)m0 * c[0], p1 = (unsigned __int128)m1 * c[2];
        uint64_t n0 = (uint64_t)(p1 >> 64) ^ c[1] ^ k0, n2 = (uint64_t)(p0 >> 64) ^ c[3] ^ k1;
        c[1] = (uint64_t)p1;
        c[3] = (uint64_t)p0;
        c[0] = n0;
        c[2] = n2;
        k0 += w0;
        k1 += w1;
    }
}

float orc_philox_u(void* src, size_t i, uint32_t t)
{
    const uint64_t* s = (const uint64_t*)src;
    uint64_t c[4] = {i, t, 0, 0};
    orc_philox4x64_10(c, s[0], s[1]);
    return (float)(c[t == 0 ? 0 : 1] >> 40) * 0x1.0p-24f;
}

uint32_t orc_philox_j(void* src, size_t i, uint32_t t)
{
    const uint64_t* s = (const uint64_t*)src;
    uint64_t c[4] = {i, t, 0, 0};
    orc_philox4x64_10(c, s[0], s[1]);
    return (uint32_t)(((unsigned __int128)c[0] * s[2]) >> 64);
}

/* mcl_3d.cpp:433-449 with tf2::Quaternion::setRPY's half-angle ZYX form */
void orc_pose_array(const float* particles, size_t P, double* poses)
{
    for (size_t i = 0; i < P; ++i) {
        const float* p = particles + 7 * i;
        double hr = (double)p[3] * 0.5, hp = (double)p[4] * 0.5, hy = (double)p[5] * 0.5;
        double sr = sin(hr), cr = cos(hr), sp = sin(hp), cp = cos(hp), sy = sin(hy), cy = cos(hy);
        double* o = poses + 7 * i;
        o[0] = p[0];
        o[1] = p[1];
        o[2] = p[2];
        o[3] = sr * cp * cy - cr * sp * sy;
        o[4] = cr * sp * cy + sr * cp * sy;
        o[5] = cr * cp * sy - sr * sp * cy;
        o[6] = cr * cp * cy + sr * sp * sy;
    }
}

/* Seeded per-particle subsampling (the library's own feature; the reference
 * scores every point): one point from each stratum [floor(k N / K),
 * floor((k+1) N / K)), picked by the upper 32 bits of the k-th output of a
 * SplitMix64 stream (Steele, Lea and Flood 2014) started at
 * mix(seed ^ mix(i)), scaled to the stratum by a 32x32 -> 64-bit product. */
static uint64_t orc_mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

void orc_subsample_indices(uint64_t seed, uint64_t i, uint32_t N, uint32_t K, uint32_t* out)
{
    const uint64_t state = orc_mix64(seed ^ orc_mix64(i));
    for (uint32_t k = 0; k < K; ++k) {
        const uint64_t lo = (uint64_t)k * N / K, hi = (uint64_t)(k + 1) * N / K;
        const uint64_t u = orc_mix64(state + (uint64_t)(k + 1) * 0x9E3779B97F4A7C15ull) >> 32;
        out[k] = (uint32_t)(lo + ((u * (hi - lo)) >> 32));
    }
}
