/*
 * TEST INFRASTRUCTURE ONLY -- NOT PART OF THE PRODUCT.
 *
 * CPU restatement ("the oracle") of the uos/tsdf_localization MCL sensor update
 * and systematic resampler.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load it; the CUDA library never
 * links or calls it.
 *
 * Parity pin: on x86-64 every function here is checked bit-for-bit against the
 * reference's own sources compiled verbatim (oracle/ref_driver.cpp built by
 * oracle/Makefile into oracle/_ref/).  The restatement is written so that it
 * gives the same bits on x86-64 and aarch64 (explicit x86 float->size_t
 * conversion semantics, no FP contraction, double-precision libm trig).
 */
#ifndef TSDF_ORACLE_H
#define TSDF_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same field order and types as CudaSubVoxelMap<float,float>::MapCoef
 * (include/tsdf_localization/cuda/cuda_sub_voxel_map.h:22-50). */
typedef struct orc_map_coef {
    uint64_t dim_x, dim_y, dim_z;
    float min_x, min_y, min_z;
    float max_x, max_y, max_z;
    float resolution;
    float init_value;
    uint64_t up_dim_x, up_dim_y, up_dim_z, up_dim_2;
    uint64_t sub_dim, sub_dim_2;
    uint64_t grid_occ_size, data_size;
} orc_map_coef;

/* Sensor-model parameters (TSDFEvaluator ctor, tsdf_evaluator.h:72-80). */
typedef struct orc_model {
    float a_hit, a_range, a_max, max_range;
} orc_model;

/* float -> size_t exactly as gcc emits it on x86-64 (cvttss2si based). */
uint64_t orc_f2u_x86(float v);

/* CudaSubVoxelMap ctor (cuda_sub_voxel_map.tcc:4-48). */
void orc_map_coef_init(orc_map_coef* c, const float mn[3], const float mx[3],
                       float resolution, float init_value);

/* CudaSubVoxelMap::setData (cuda_sub_voxel_map.tcc:170-230).  grid_occ must
 * hold grid_occ_size ints; *data_out is malloc'd (NULL when n == 0, as in the
 * reference where data_ stays nullptr).  Returns 0, or -1 on "Upper voxel index
 * overflow!".  Writes that the reference makes out of bounds (getIndex miss
 * inside setEntry) are skipped and counted in *skipped. */
int orc_map_set_data(orc_map_coef* c, int32_t* grid_occ, const float* xyzv, size_t n,
                     float** data_out, size_t* skipped);

/* CudaSubVoxelMap::getIndex / getEntry (cuda_sub_voxel_map.tcc:50-157). */
uint64_t orc_get_index(const orc_map_coef* c, const int32_t* grid_occ, float x, float y, float z);
float orc_get_entry(const orc_map_coef* c, const int32_t* grid_occ, const float* data,
                    float x, float y, float z);

/* Per-particle laser pose tf_laser[0..11] (tsdf_evaluator.cpp:102-147). */
void orc_particle_pose(const float particle7[7], const float tf[16], float out12[12]);

/* TSDFEvaluator::evaluate CPU path (tsdf_evaluator.cpp:78-245) with serial
 * per-particle sums (exactly as evaluatePose, :27-76) and a serial weight sum.
 * particles: AoS of 7 floats (x,y,z,roll,pitch,yaw,weight); weights are
 * overwritten with the normalised weight.  Optional outputs may be NULL:
 *   raw_out[P]     un-normalised weight (eval_sum of evaluatePose)
 *   hits_out[P]    number of points whose index < data_size
 *   idx_out[P*N]   voxel index per particle·point (data_size on a miss)
 *   sum64_out[P]   the same per-point scores accumulated in double
 *   pose_out[6]    x,y,z,roll,pitch,yaw of the weighted mean
 * n_threads <= 0 uses all OpenMP threads.  Returns 0, 1 when the weight sum is
 * zero ("No particle is valid!"). */
int orc_evaluate(const orc_map_coef* c, const int32_t* grid_occ, const float* data,
                 const orc_model* m, float* particles, size_t P,
                 const float* points, size_t N, const float tf[16],
                 float* raw_out, uint32_t* hits_out, uint64_t* idx_out,
                 double* sum64_out, float pose_out[6], int n_threads);

/* Likelihood value of one TSDF cell (map_util.h:124-127): |tsdf| in mm. */
float orc_likelihood_value(int16_t tsdf_mm, float sigma);
/* Value of untouched cells (map_util.h:68-71). */
float orc_likelihood_init(float sigma);

/* createTSDFMap (map_util.h:17-154) without HDF5.  chunk_pos: 3 ints per chunk
 * (chunk coordinates), chunks: n_chunks blocks of edge^3 uint32 raw TSDF values
 * (low int16 = value in mm, high int16 = weight, tsdf.h:11-33) in the order the
 * file lists them.  edge generalises the fixed CHUNK_SIZE (64, grid_map.h:18-19)
 * and voxel_mm the fixed 64 mm MAP_RESOLUTION (grid_map.h:21-22).
 * Outputs the map coef, a malloc'd grid_occ, a malloc'd data array and the
 * free-space point list (malloc'd xyz triples). */
int orc_build_map_from_chunks(const int32_t* chunk_pos, const uint32_t* chunks, size_t n_chunks, int edge,
                              int voxel_mm, float sigma, orc_map_coef* c, int32_t** grid_occ_out,
                              float** data_out, float** free_xyz_out, size_t* n_free_out);

/* The part of createTSDFMap before the map is made (map_util.h:17-147): the
 * bounding box mn/mx, the init value and the (x, y, z, value) tuples it hands
 * to setData, in push order (malloc'd, 4 floats each; returned count), plus the
 * free-space cells.  Feeding the tuples to the reference's own ctor + setData
 * gives the reference's map for the same chunks. */
size_t orc_chunk_tuples(const int32_t* chunk_pos, const uint32_t* chunks, size_t n_chunks, int edge,
                        int voxel_mm, float sigma, float mn[3], float mx[3], float* init_out,
                        float** tuples_out, float** free_xyz_out, size_t* n_free_out);

/* SystematicResampler::resample (novel_resampling.h:41-72) with the uniform
 * draw U0 supplied.  Writes up to cap source indices, returns the number of
 * particles the reference would emit, or (size_t)-1 if U stops advancing. */
size_t orc_resample_systematic(const float* w, size_t M, float U0, uint32_t* idx_out, size_t cap);

/* double -> size_t as the reference's x86-64 build converts it (cvttsd2si with
 * the 2^63 split), like orc_f2u_x86 for float. */
uint64_t orc_d2u_x86(double v);

/* ResidualSystematicResampler::resample (novel_resampling.h:76-104) with the
 * uniform draw u0 in [0, 1) supplied: particle m is emitted
 * o_m = (size_t)(temp + 1.0) times, temp = (float)M * w_m - u (float), and u
 * becomes (float)o_m - temp.  Writes up to cap source indices and returns the
 * number of particles the reference would emit, or (size_t)-1 when a count
 * reaches 2^32 (the reference would try to allocate it). */
size_t orc_resample_residual_systematic(const float* w, size_t M, float u0, uint32_t* idx_out, size_t cap);

/* The scan reduction of TSDFEvaluator::evaluateParticles
 * (tsdf_evaluator.cpp:300-376): points closer than 1 m (float sqrt of the float
 * sum of squares) are dropped; the k-th kept point takes ring[k] (the ring
 * iterator advances only for kept points) and index k; the first kept point of
 * every (ring, cell centre) stays, centre = floor(v / cell) * cell + cell / 2 in
 * float per axis; the survivors come out ring by ring (0..63), by index within a
 * ring, with their original coordinates.  Returns the number of survivors, or
 * (size_t)-1 for a ring outside [0, 64) (the reference indexes past its table).
 * own_ring != 0: every kept point takes its own ring instead. */
size_t orc_reduce_scan(const float* xyz, const int16_t* ring, size_t n, float cell, int own_ring, float* out,
                       size_t cap);

/* ParticleCloud::apply_model (particle_cloud.cpp:499-617) on given draws:
 * particles P x 7 floats updated in place, draws P x 6 doubles (dx, dy, dz,
 * roll, pitch, yaw), trig through the double overloads. */
void orc_motion_apply(float* particles, size_t P, const double* draws);

/* WheelResampler::resample (wheel_resampler.cpp:6-33), literally (O(M^2)):
 * idx[i] = source of output i for the draws (doubles in [0, 1)). */
void orc_resample_wheel(const float* w, size_t M, const double* draws, uint32_t* idx);
/* ResidualResampler::resample (novel_resampling.h:12-34) consuming draws[0..K)
 * (particle indices); returns the number consumed, or (size_t)-1 when they run out. */
size_t orc_resample_residual(const float* w, size_t M, const uint32_t* draws, size_t K, uint32_t* idx);
/* MetropolisResampler::resample (novel_resampling.h:113-142), steps proposals
 * per output, u and j draws output-major. */
void orc_resample_metropolis(const float* w, size_t M, uint32_t steps, const float* u, const uint32_t* j,
                             uint32_t* idx);
/* RejectionResampler::resample (novel_resampling.h:149-186) with draws taken
 * from callbacks in the reference's order (u for output i; then j, u per
 * proposal); t counts the proposals of output i (0 for its first u).  Returns 0,
 * or -1 when an output exceeds max_rounds proposals. */
typedef float (*orc_draw_u_fn)(void* src, size_t i, uint32_t t);
typedef uint32_t (*orc_draw_j_fn)(void* src, size_t i, uint32_t t);
int orc_resample_rejection(const float* w, size_t M, orc_draw_u_fn du, orc_draw_j_fn dj, void* src,
                           uint32_t max_rounds, uint32_t* idx);
/* mcl_3d.cpp:433-449: particles (P x 7 floats) as Pose records (P x 7
 * doubles: position, quaternion x, y, z, w of setRPY in double). */
void orc_pose_array(const float* particles, size_t P, double* poses);
/* Philox4x64-10 (Salmon et al., SC 2011) of one counter block. */
void orc_philox4x64_10(uint64_t c[4], uint64_t k0, uint64_t k1);
/* A draw source for orc_resample_rejection with the device's keying
 * (counter (i, t, 0, 0), key (seed, stream)): src points at two uint64 {seed, stream, M}. */
float orc_philox_u(void* src, size_t i, uint32_t t);
uint32_t orc_philox_j(void* src, size_t i, uint32_t t);

/* The library's seeded per-particle subsampling rule (no counterpart in the
 * reference): the K kept scan indices of particle i, out[K]. */
void orc_subsample_indices(uint64_t seed, uint64_t i, uint32_t N, uint32_t K, uint32_t* out);

#ifdef __cplusplus
}
#endif

#endif
