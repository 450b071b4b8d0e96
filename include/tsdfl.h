/*
 * tsdfl -- GB300-native MCL sensor update for TSDF maps (C ABI).
 *
 * Drop-in for the sensor-update path of uos/tsdf_localization:
 *   transform the scan by every particle's pose, look each point up in the
 *   likelihood map built from the TSDF, score, sum per particle, normalise,
 *   mean pose, systematic resampling.
 * Every entry point names the reference interface it replaces.  All functions
 * return a tsdfl status; tsdfl_last_error() gives the message of the last
 * failure on the calling thread.  Sizes are element counts.  Pointers named
 * d_* are device pointers; all other array pointers are host memory.
 */
#ifndef TSDFL_H
#define TSDFL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference throws std::runtime_error instead) ---- */
#define TSDFL_OK 0
#define TSDFL_ERR_INVALID_ARG 1
#define TSDFL_ERR_OUT_OF_MEMORY 2
#define TSDFL_ERR_DEGENERATE 3   /* weight sum 0 or not finite: "No particle is valid!" */
#define TSDFL_ERR_DEVICE 4       /* CUDA error (cudaCheck, cuda_util.cu:8-17) */
#define TSDFL_ERR_TIMEOUT 5      /* a bounded device wait ran out */
#define TSDFL_ERR_CAPACITY 6     /* an output buffer is too small */
#define TSDFL_ERR_UNSUPPORTED 7

/* Same field order, types and size (120 bytes on LP64) as
 * CudaSubVoxelMap<float,float>::MapCoef (include/tsdf_localization/cuda/
 * cuda_sub_voxel_map.h:22-50), so &map.coef() can be passed directly. */
typedef struct tsdfl_map_coef {
    uint64_t dim_x, dim_y, dim_z;
    float min_x, min_y, min_z;
    float max_x, max_y, max_z;
    float resolution;
    float init_value;
    uint64_t up_dim_x, up_dim_y, up_dim_z, up_dim_2;
    uint64_t sub_dim, sub_dim_2;
    uint64_t grid_occ_size, data_size;
} tsdfl_map_coef;

/* Sensor model of TSDFEvaluator / CudaEvaluator
 * (tsdf_evaluator.h:72-80, cuda_evaluator.h:112). */
typedef struct tsdfl_model {
    float a_hit, a_range, a_max, max_range;
} tsdfl_model;

typedef struct tsdfl_ctx tsdfl_ctx;
typedef struct tsdfl_map tsdfl_map;

const char* tsdfl_last_error(void);
const char* tsdfl_version(void);

/* ---- context: one device, one stream, a growable workspace ----
 * Replaces the device-buffer ownership of CudaEvaluator
 * (cuda_evaluator.cu:136-209, 239-261); unlike the reference, nothing is
 * process-global, so several maps and contexts can coexist. */
int tsdfl_ctx_create(int device, tsdfl_ctx** out);
int tsdfl_ctx_destroy(tsdfl_ctx* ctx);
/* Use the caller's cudaStream_t (NULL = the context's own stream). */
int tsdfl_ctx_set_stream(tsdfl_ctx* ctx, void* cuda_stream);
void* tsdfl_ctx_stream(tsdfl_ctx* ctx);
/* Waits for the stream and returns the status raised by device work since the
 * last sync (e.g. TSDFL_ERR_DEGENERATE from tsdfl_evaluate_device). */
int tsdfl_ctx_sync(tsdfl_ctx* ctx);
/* Pre-sizes the workspace for P particles and N points so that later calls
 * with at most as many allocate nothing. */
int tsdfl_ctx_reserve(tsdfl_ctx* ctx, size_t P, size_t N);

/* Device timing of the scoring kernels of the next evaluations (CUDA events
 * on the context stream) and the number of kernels this library launched in
 * the process so far. */
int tsdfl_ctx_set_timing(tsdfl_ctx* ctx, int enable);
int tsdfl_ctx_last_timing(tsdfl_ctx* ctx, float* eval_kernel_ms);
uint64_t tsdfl_launch_count(void);
/* Device bytes the context holds for evaluations and for resampling (each
 * grows on demand; either may be NULL). */
int tsdfl_ctx_workspace_bytes(const tsdfl_ctx* ctx, size_t* eval_bytes, size_t* resample_bytes);

/* ---- map ----
 * Uploads a built CudaSubVoxelMap<float,float> (coef(), rawGridOcc(),
 * rawData(); replaces the map upload in the CudaEvaluator ctor,
 * cuda_evaluator.cu:21-59).  When every slot equals one of the likelihood
 * values of createTSDFMap for `sigma` (map_util.h:68-71,124-127), slots are
 * stored as 16-bit codes, losslessly; otherwise as float.  flags: TSDFL_MAP_*. */
/* TSDFL_MAP_DENSE: also build the compact layout -- brick ranks from a bitmap
 * of the brick grid held in shared memory, read beside the slot codes (which
 * stay in the reference's data order) -- so the tiled kernel makes one map
 * gather per lookup instead of two.  Skipped (brick layout only) when a
 * sub-voxel index can reach sub_dim or the bitmap exceeds 128 KB.
 * TSDFL_MAP_F16: store every slot's likelihood value as an IEEE half instead
 * of a 16-bit code (the same 2 bytes a slot): values round to 11 significant
 * bits, so weights move by up to about 5e-4 relative -- an accuracy variant
 * scored by the generic kernel, not bit-exact with the reference. */
#define TSDFL_MAP_DENSE 1u
#define TSDFL_MAP_FORCE_F32 2u    /* keep float slots */
#define TSDFL_MAP_F16 4u
/* TSDFL_MAP_HASH: index the allocated bricks in a sparse hash ({brick, rank},
 * 8 bytes a slot at a load of at most 1/2) instead of the bitmap -- what
 * TSDFL_MAP_DENSE builds by itself when the bitmap of the brick grid would
 * exceed 128 KB (bounding boxes of more than 524,288 bricks of 1 m, mostly
 * empty).  The tiled kernel then reads the rank from this L2-resident table
 * instead of the brick table. */
#define TSDFL_MAP_HASH 8u
/* TSDFL_MAP_GRID: also store the codes of every brick of the bounding box in
 * brick order (unallocated bricks as misses; each brick of the lowest layer
 * behind a copy of what getIndex reads below its first slot, the tail of the
 * previous allocated brick), so the tiled kernel finds a slot from the brick
 * index alone, with no rank lookup.  Costs (bricks of the bounding box + bricks
 * of one layer) x sub_dim^3 x 2 bytes beside the code array.  Skipped under the
 * same conditions as the compact layout, or when the array would pass 2^31
 * codes. */
#define TSDFL_MAP_GRID 16u
int tsdfl_map_create(tsdfl_ctx* ctx, const tsdfl_map_coef* coef, const int32_t* grid_occ, const float* data,
                     float sigma, uint32_t flags, tsdfl_map** out);
/* Same map from 16-bit slot codes (code c < 600: likelihood of |tsdf| = c mm;
 * 600: the init value), as tsdfl_build_map_codes produces them. */
int tsdfl_map_create_codes(tsdfl_ctx* ctx, const tsdfl_map_coef* coef, const int32_t* grid_occ,
                           const uint16_t* codes, float sigma, uint32_t flags, tsdfl_map** out);
int tsdfl_map_destroy(tsdfl_map* map);

typedef struct tsdfl_map_info {
    uint64_t grid_occ_size, data_size, bricks;
    uint64_t device_bytes;     /* all device memory the map holds */
    int32_t storage;           /* 0 = 16-bit codes, 1 = float, 2 = half (TSDFL_MAP_F16) */
    int32_t dense;             /* brick rank index: 0 = brick table only, 1 = bitmap (compact layout),
                                  2 = sparse brick hash, 3 = none needed (TSDFL_MAP_GRID) */
    int32_t fast_index;        /* division-free slot indexing verified for this resolution */
    int32_t reserved;
} tsdfl_map_info;
int tsdfl_map_get_info(const tsdfl_map* map, tsdfl_map_info* info);

/* Likelihood-map construction of createTSDFMap (map_util.h:17-154) from TSDF
 * cells, without HDF5: n_chunks chunks of edge^3 raw cells (low int16 = value
 * in mm, high int16 = weight, tsdf.h:11-33; cell index edge*edge*i+edge*j+k),
 * chunk coordinates in chunk_pos (3 ints each), in the order the map file lists
 * them.  edge = 64 and voxel_mm = 64 give the reference's map exactly.
 * Outputs (malloc'd, free with tsdfl_free): grid_occ[coef.grid_occ_size],
 * slot codes[coef.data_size] and the free-space cell positions (xyz). */
int tsdfl_build_map_codes(const int32_t* chunk_pos, const uint32_t* chunks, size_t n_chunks, int edge,
                          int voxel_mm, float sigma, tsdfl_map_coef* coef, int32_t** grid_occ,
                          uint16_t** codes, float** free_xyz, size_t* n_free);
/* Reads a map file in the reference's HDF5 layout -- group "/map" with one
 * dataset of edge^3 raw cells per chunk, named "<x>_<y>_<z>" (GlobalMap,
 * global_map.cpp:12-170, written through HighFive; read by createTSDFMap,
 * map_util.h:17-113) -- without the HDF5 library.  Outputs the chunks in the
 * order createTSDFMap visits them (names in byte order) as tsdfl_build_map_codes
 * takes them: chunk_pos (3 ints per chunk) and chunks (n_chunks x edge^3 raw
 * cells), malloc'd (free with tsdfl_free).  Superblocks 0-3, object headers 1
 * and 2, symbol-table and compact groups, contiguous and compact 4-byte integer
 * datasets; other storage (dense groups, chunked or filtered datasets) gives
 * TSDFL_ERR_UNSUPPORTED, a malformed file TSDFL_ERR_INVALID_ARG. */
int tsdfl_read_map_h5(const char* path, int32_t** chunk_pos, uint32_t** chunks, size_t* n_chunks, int32_t* edge);
/* The float value of every code for sigma (601 entries: codes 0..600). */
int tsdfl_code_values(float sigma, float init_value, float* out601);
void tsdfl_free(void* p);

/* ---- sensor update ----
 * TSDFEvaluator::evaluate(particles, points, tf, use_cuda)
 * (tsdf_evaluator.cpp:78-245) / CudaEvaluator::evaluate
 * (cuda_evaluator.cu:118-428).
 * particles: P x 7 floats (x, y, z, roll, pitch, yaw, weight) -- the layout of
 *   struct Particle (particle.h:26-55); weights are overwritten with the
 *   normalised weights, as the reference does.
 * points: N x 3 floats (struct CudaPoint, cuda_evaluator.h:22-39).
 * tf: the 4x4 row-major sensor-to-base transform (tsdf_evaluator.cpp:271-284).
 * pose_out (optional): weighted mean x, y, z and circular-mean roll, pitch, yaw.
 * N == 0 returns TSDFL_OK and leaves everything untouched
 * (cuda_evaluator.cu:122-125).  Weight sum 0 -> TSDFL_ERR_DEGENERATE. */
#define TSDFL_SUM_EXACT 0u    /* order-independent fixed-point likelihood sums (default) */
#define TSDFL_SUM_SERIAL 1u   /* reference order float sums: raw weights bit-identical */
#define TSDFL_EVAL_GENERIC 4u /* exact sums with the generic (division-based) scoring kernel */
/* Normalise in the log domain: w_i = exp(ln raw_i - LSE), LSE = ln max_j raw_j
 * + ln sum_j exp(ln raw_j - ln max_j raw_j), all in double, instead of
 * raw_i / sum_j raw_j.  The same weights up to the final rounding for this
 * sensor model (raw weights are sums of bounded scores); for callers that
 * keep the reference's linear normalisation optional. */
#define TSDFL_NORM_LOG 8u
int tsdfl_evaluate(tsdfl_ctx* ctx, const tsdfl_map* map, const tsdfl_model* model, float* particles, size_t P,
                   const float* points, size_t N, const float tf[16], uint32_t flags, float pose_out[6]);

/* Per-particle diagnostics of one evaluation (host arrays, each optional):
 * raw weights (evaluatePose sums), hit counts (points whose slot index is
 * inside the map data), and for small cases the slot index of every
 * particle*point (0xffffffff on a miss).  Also returns the weight sum. */
typedef struct tsdfl_eval_debug {
    float* raw_weights;       /* [P] */
    uint32_t* hits;           /* [P] */
    uint32_t* voxel_index;    /* [P*N] */
    float* laser_pose;        /* [P*12] tf_laser of every particle */
    double weight_sum;
} tsdfl_eval_debug;
int tsdfl_evaluate_debug(tsdfl_ctx* ctx, const tsdfl_map* map, const tsdfl_model* model, float* particles,
                         size_t P, const float* points, size_t N, const float tf[16], uint32_t flags,
                         float pose_out[6], tsdfl_eval_debug* dbg);

/* Stream-ordered form on device buffers (no host synchronisation; errors that
 * only the device sees are reported by tsdfl_ctx_sync).  d_particles: P x 7
 * floats, updated in place with the normalised weights; d_points: N x 3;
 * d_pose_out: 6 floats or NULL.  Allocates only when the workspace must grow
 * (see tsdfl_ctx_reserve). */
int tsdfl_evaluate_device(tsdfl_ctx* ctx, const tsdfl_map* map, const tsdfl_model* model, float* d_particles,
                          size_t P, const float* d_points, size_t N, const float tf[16], uint32_t flags,
                          float* d_pose_out);

/* ---- systematic resampling ----
 * SystematicResampler::resample (novel_resampling.h:41-72) with its uniform
 * draw u0 in [0, 1/M) given.  Writes the source particle index of every
 * emitted particle (up to cap) and the count the reference emits, which is not
 * always M.  Bit-exact with the reference for the same weights and u0. */
int tsdfl_resample_systematic(tsdfl_ctx* ctx, const float* weights, size_t M, float u0, uint32_t* idx_out,
                              size_t cap, size_t* count_out);
/* The same on the particle cloud itself (M x 7 floats, the weight last), as
 * SystematicResampler::resample reads the weights from its particles
 * (novel_resampling.h:41-72): no weight array to gather on the host, the
 * cloud goes over in one copy. */
int tsdfl_resample_systematic_particles(tsdfl_ctx* ctx, const float* particles, size_t M, float u0,
                                        uint32_t* idx_out, size_t cap, size_t* count_out);
/* Device form: gathers the resampled particles (P x 7 floats) from d_particles
 * into d_particles_out (capacity cap particles) and writes the count to
 * *d_count (device).  Weights are the last field of every particle. */
int tsdfl_resample_systematic_device(tsdfl_ctx* ctx, const float* d_particles, size_t M, float u0,
                                     float* d_particles_out, size_t cap, uint32_t* d_count);

/* ---- residual systematic resampling ----
 * ResidualSystematicResampler::resample (novel_resampling.h:76-104), mcl_3d's
 * default resampler (mcl_3d.cpp:765), with its draw u0 in [0, 1) given:
 * particle m is emitted (size_t)(temp + 1.0) times, temp = (float)M * w_m - u,
 * u then becomes (float)count - temp.  Bit-exact with the reference for the
 * same weights and u0 (the float chain is walked in particle order by one
 * device thread; the copies are parallel).  Negative or non-finite weights, or
 * a particle count of 2^24, give TSDFL_ERR_UNSUPPORTED. */
int tsdfl_resample_residual_systematic(tsdfl_ctx* ctx, const float* weights, size_t M, float u0, uint32_t* idx_out,
                                       size_t cap, size_t* count_out);
int tsdfl_resample_residual_systematic_device(tsdfl_ctx* ctx, const float* d_particles, size_t M, float u0,
                                              float* d_particles_out, size_t cap, uint32_t* d_count);

/* ---- best particle ----
 * mcl_3d.cpp:382-394: the index of the first particle with the largest weight
 * above 0, written to *d_index (device; 0xFFFFFFFF when no weight is above 0,
 * where the reference would index with -1).  d_particles: M x 7 floats. */
int tsdfl_best_particle_device(tsdfl_ctx* ctx, const float* d_particles, size_t M, uint32_t* d_index);

/* ---- batched filters ----
 * No single call of the reference does this: many independent filters (each
 * one TSDFEvaluator::evaluate + SystematicResampler::resample, as the single
 * calls above) updated together.  Their scoring runs in ONE persistent launch
 * over a (filter, pass, point chunk, particle group) work queue; preparation,
 * normalisation and resampling are per-filter launches in the same stream.
 * The whole update can be captured once as a CUDA graph and replayed.  Every
 * filter's results are the same as its single-filter tsdfl_evaluate_device +
 * tsdfl_resample_systematic_device results (exact sums; same draws).  All
 * buffers are device buffers fixed at creation: write new particles, points
 * and draws into them between runs.  Exact sums only (flags 0). */
typedef struct tsdfl_batch tsdfl_batch;
typedef struct tsdfl_filter {
    const tsdfl_map* map;
    tsdfl_model model;
    float tf[16];             /* sensor-to-base transform, row-major */
    float* d_particles;       /* P x 7; weights overwritten with the normalised weights */
    size_t P;
    const float* d_points;    /* N x 3 */
    size_t N;
    float* d_pose_out;        /* 6 floats, or NULL */
    const float* d_u0;        /* systematic draw in [0, 1/P), read when the batch runs; NULL: no resampling */
    float* d_resampled;       /* resample_cap x 7 */
    size_t resample_cap;
    uint32_t* d_count;        /* particles the resampler emitted */
} tsdfl_filter;
int tsdfl_batch_create(tsdfl_ctx* ctx, const tsdfl_filter* filters, size_t n_filters, uint32_t flags,
                       tsdfl_batch** out);
int tsdfl_batch_destroy(tsdfl_batch* batch);
/* One update of every filter, stream-ordered on the context's stream (the
 * captured graph when there is one).  Device-side errors: tsdfl_ctx_sync. */
int tsdfl_batch_run(tsdfl_batch* batch);
/* Captures one update as a CUDA graph; later runs launch the graph. */
int tsdfl_batch_capture(tsdfl_batch* batch);
/* Work-item shape of the persistent scoring launch: chunk scan points (a
 * multiple of 64) x group particles.  Results do not depend on it. */
int tsdfl_batch_set_tiles(tsdfl_batch* batch, int chunk, int group);
/* Times the scoring launch for a set of shapes and keeps the fastest. */
int tsdfl_batch_autotune(tsdfl_batch* batch, int* chunk_out, int* group_out, float* best_ms);
/* Hit counts (points whose slot index is inside the map data) of filter i's
 * last update, P values copied to the host. */
int tsdfl_batch_hits(tsdfl_batch* batch, size_t i, uint32_t* hits);
/* Work in the persistent launch: segments, batches of work items, and the
 * filters scored outside it (maps without the tiled path). */
int tsdfl_batch_info(const tsdfl_batch* batch, uint32_t* segments, uint32_t* batches, uint32_t* outside);
/* Filters whose scans fill the GPU by themselves (about two of the
 * single-filter kernel's work items per warp): the batch's update scores them
 * with the single-filter kernel instead of the persistent launch, which
 * measured faster per lookup; results are the same either way. */
int tsdfl_batch_single(const tsdfl_batch* batch, uint32_t* single);

/* ---- served sessions ----
 * No counterpart in the reference (mcl_3d runs one filter per process).  A
 * request loop for many robots on one GPU: every session's particles, map and
 * random state stay on the device; scans are submitted as they arrive and
 * queued; tsdfl_server_poll publishes finished updates and, whenever one of
 * the two dispatch slots is free, launches every queued update of an idle
 * session as one batch (continuous batching: updates that arrive while others
 * run go out with the next batch, and two batches can be on the device at
 * once).  One update = tsdfl_evaluate + tsdfl_resample_systematic of the
 * session's particles, results identical to those single calls with the draw
 * tsdfl_server_draw gives (exact sums).  Admission: a session opens only if
 * its device memory fits the budget; a submission is refused when the work
 * queued before it would take longer than max_wait_ms at the measured rate. */
typedef struct tsdfl_server tsdfl_server;
typedef struct tsdfl_server_config {
    size_t hbm_budget;          /* bytes all sessions may hold on the device */
    size_t max_sessions;
    size_t max_points;          /* largest scan of one submission */
    double max_wait_ms;         /* refuse submissions expected to wait longer (0: never refuse) */
    uint32_t max_queue;         /* queued submissions per session (0: 4) */
} tsdfl_server_config;
int tsdfl_server_create(tsdfl_ctx* ctx, const tsdfl_server_config* cfg, tsdfl_server** out);
int tsdfl_server_destroy(tsdfl_server* server);
/* particles: P x 7 host floats; the session keeps at most 2P + 16 particles
 * (the systematic resampler's count drifts).  TSDFL_ERR_OUT_OF_MEMORY: the
 * budget cannot hold the session (refused). */
int tsdfl_session_open(tsdfl_server* server, const tsdfl_map* map, const float* particles, size_t P,
                       const float tf[16], const tsdfl_model* model, uint64_t seed, uint32_t* session);
int tsdfl_session_close(tsdfl_server* server, uint32_t session);
/* Queues one update with the scan points (N x 3 host floats, copied).  Refused
 * with TSDFL_ERR_CAPACITY when the session's queue is full or the admission
 * bound is exceeded. */
int tsdfl_session_submit(tsdfl_server* server, uint32_t session, const float* points, size_t N, uint64_t* ticket);
/* Non-blocking: publishes finished updates, launches queued ones; *completed
 * (optional) receives the number published by this call. */
int tsdfl_server_poll(tsdfl_server* server, size_t* completed);
/* The result of a published ticket (once): mean pose, latency from submission
 * to publication (host clock) and the update's status (TSDFL_OK, or e.g.
 * TSDFL_ERR_DEGENERATE).  TSDFL_ERR_INVALID_ARG while not yet published. */
int tsdfl_server_result(tsdfl_server* server, uint64_t ticket, float pose[6], double* latency_ms, int* status);
/* The session's current particles (count x 7 host floats). */
int tsdfl_session_particles(tsdfl_server* server, uint32_t session, float* out, size_t cap, size_t* count);
/* The systematic draw of a session's k-th update (k from 0) with P particles:
 * (float)(u / P), u = (splitmix64(seed + k * 0x9E3779B97F4A7C15) >> 11) * 2^-53. */
float tsdfl_server_draw(uint64_t seed, uint64_t k, size_t P);
/* Counters since creation: submissions accepted and refused, updates
 * published, batches launched, and the measured rate (particle*points/s). */
int tsdfl_server_stats(const tsdfl_server* server, uint64_t* accepted, uint64_t* refused, uint64_t* published,
                       uint64_t* batches, double* rate);

/* ---- the reference's other resamplers ----
 * WheelResampler (src/resampling/wheel_resampler.cpp:6-33), ResidualResampler
 * (novel_resampling.h:9-35), MetropolisResampler (:106-143) and
 * RejectionResampler (:146-187), all emitting exactly M particles.  Random
 * draws come from the caller -- the reference's own sequence drawn on the host
 * in its order, which makes the output the reference's bit for bit -- or, when
 * the draw pointer is NULL, from Philox4x64-10 on the device keyed by seed.
 * Host forms: weights[M] in, the source index of every output particle out
 * (idx_out[M]).  Device forms: M x 7 particles gathered into d_out.
 *
 * wheel: draws[M] doubles in [0, 1) (uniform_distribution(0.0, 1.0)); output
 *   i takes the first particle whose float running weight sum reaches
 *   (float)draw, and stays itself when none does.
 * residual: draws[n_draws] particle indices (uniform_int_distribution(0, M-1));
 *   each drawn particle is copied ceil(M * w) times until M are emitted.  Too
 *   few draws (or, generated, more than 4M + 4096 needed) -> TSDFL_ERR_UNSUPPORTED.
 * metropolis: `steps` proposals per output (the reference's sampling_steps, 50
 *   in mcl_3d.cpp:258); u_draws[M*steps] floats, j_draws[M*steps] indices, in
 *   the reference's order (output-major, u before j); acceptance u <= w_j / w_0
 *   (the reference keeps particle 0 as the comparison particle).
 * rejection: device draws only (how many the reference consumes depends on the
 *   outcomes); u <= w_j / max(0, max w) accepts; an output still rejecting after
 *   2^20 proposals stops with TSDFL_ERR_UNSUPPORTED. */
int tsdfl_resample_wheel(tsdfl_ctx* ctx, const float* weights, size_t M, const double* draws, uint64_t seed,
                         uint32_t* idx_out);
int tsdfl_resample_wheel_device(tsdfl_ctx* ctx, const float* d_particles, size_t M, const double* d_draws,
                                uint64_t seed, float* d_out);
int tsdfl_resample_residual(tsdfl_ctx* ctx, const float* weights, size_t M, const uint32_t* draws, size_t n_draws,
                            uint64_t seed, uint32_t* idx_out);
int tsdfl_resample_residual_device(tsdfl_ctx* ctx, const float* d_particles, size_t M, const uint32_t* d_draws,
                                   size_t n_draws, uint64_t seed, float* d_out);
int tsdfl_resample_metropolis(tsdfl_ctx* ctx, const float* weights, size_t M, uint32_t steps, const float* u_draws,
                              const uint32_t* j_draws, uint64_t seed, uint32_t* idx_out);
int tsdfl_resample_metropolis_device(tsdfl_ctx* ctx, const float* d_particles, size_t M, uint32_t steps,
                                     const float* d_u_draws, const uint32_t* d_j_draws, uint64_t seed,
                                     float* d_out);
int tsdfl_resample_rejection(tsdfl_ctx* ctx, const float* weights, size_t M, uint64_t seed, uint32_t* idx_out);
int tsdfl_resample_rejection_device(tsdfl_ctx* ctx, const float* d_particles, size_t M, uint64_t seed,
                                    float* d_out);

/* ---- scan reduction ----
 * The pre-processing of TSDFEvaluator::evaluateParticles
 * (tsdf_evaluator.cpp:304-376) on a PointCloud2's data: points closer than
 * 1 m are dropped; of the kept points sharing (ring, reduction cell centre)
 * the first stays; the survivors come out ring by ring (0..63), in cloud
 * order within a ring, as their original x, y, z (N x 3 floats, the points
 * argument of tsdfl_evaluate).  Same points in the same order as the reference.
 * cloud: n_points records of point_step bytes; x, y, z are consecutive floats
 *   at x_offset (iter_x[0..2], :313-315), the ring an int16 at ring_offset.
 * cell: reduction_cell_size (> 0), centre = floor(v / cell) * cell + cell / 2.
 * The k-th kept point takes the ring field of the k-th cloud point, as the
 * reference's ring iterator does (:319-332); TSDFL_SCAN_OWN_RING takes the
 * point's own ring instead.  A ring outside [0, 64) gives
 * TSDFL_ERR_INVALID_ARG (the reference indexes past its 64 ring lists).
 * Writes min(count, cap) points; count > cap gives TSDFL_ERR_CAPACITY with
 * *count_out still the full count. */
#define TSDFL_SCAN_OWN_RING 1u
int tsdfl_reduce_scan(tsdfl_ctx* ctx, const void* cloud, size_t n_points, uint32_t point_step, uint32_t x_offset,
                      uint32_t ring_offset, float cell, uint32_t flags, float* points_out, size_t cap,
                      size_t* count_out);
/* Device form: d_cloud and d_points_out on the device, the count written to
 * *d_count (device); stream-ordered, device-side errors by tsdfl_ctx_sync. */
int tsdfl_reduce_scan_device(tsdfl_ctx* ctx, const void* d_cloud, size_t n_points, uint32_t point_step,
                             uint32_t x_offset, uint32_t ring_offset, float cell, uint32_t flags,
                             float* d_points_out, size_t cap, uint32_t* d_count);
/* TSDFEvaluator::evaluateParticles (tsdf_evaluator.cpp:247-376) after its tf
 * lookup: the scan reduction above and tsdfl_evaluate on the reduced points,
 * with the cloud copied to the device once and the reduced points kept there.
 * scan_flags: TSDFL_SCAN_*; flags: TSDFL_SUM_* / TSDFL_EVAL_*.  *n_reduced
 * (optional) receives the number of reduced points. */
int tsdfl_evaluate_cloud(tsdfl_ctx* ctx, const tsdfl_map* map, const tsdfl_model* model, float* particles, size_t P,
                         const void* cloud, size_t n_points, uint32_t point_step, uint32_t x_offset,
                         uint32_t ring_offset, float cell, uint32_t scan_flags, const float tf[16], uint32_t flags,
                         float pose_out[6], size_t* n_reduced);

/* ---- motion update ----
 * ParticleCloud::apply_model (particle_cloud.cpp:499-617), the loop every
 * motion-update overload runs: each particle draws dx, dy, dz, roll, pitch,
 * yaw from N(mean[k], stddev[k]), composes the odometry transform with its
 * orientation and takes the translation and getAngleFromMat's angles
 * (util.cpp:86-111) as its new pose; weights are kept.  The composition is the
 * reference's bit for bit.  The draws cannot be: the reference pulls them from
 * one serial std::mt19937 through std::normal_distribution.
 * tsdfl_motion_update* draws them on the device (Philox4x64-10 keyed by seed,
 * counter (particle, block, step), Box-Muller in FP64: the same distribution,
 * independent per particle, reproducible per (seed, step));
 * tsdfl_motion_apply* takes them from the caller (P x 6 doubles), e.g. the
 * reference's own sequence drawn on the host. */
typedef struct tsdfl_motion {
    double mean[6];     /* dx, dy, dz, roll, pitch, yaw */
    double stddev[6];   /* the reference's second std::normal_distribution argument */
} tsdfl_motion;
#define TSDFL_MOTION_ODOM 0       /* motionUpdate(const nav_msgs::Odometry&) (:153-197): in = linear.x, angular.z */
#define TSDFL_MOTION_IMU 1        /* motionUpdate(const ImuAccumulator::Data&) (:335-378): in = linear_vel, angular_yaw */
#define TSDFL_MOTION_SCALE 2      /* motionUpdate(lin_scale, ang_scale) (:380-413) */
#define TSDFL_MOTION_SCALE_IMU 3  /* motionUpdate(lin_scale, imu) (:415-454): in = lin_scale, delta_roll, delta_pitch, delta_yaw */
#define TSDFL_MOTION_DELTA 4      /* motion_update (:456-497): in = dx, dy, dz, roll, pitch, yaw, lin_base_noise, ang_base_noise */
/* The distributions an overload sets up, with its own float/double
 * arithmetic; a = a_1 .. a_12 (setMotionParameters), time_diff in seconds. */
int tsdfl_motion_model(int kind, const float a[12], const double* in, size_t n_in, float time_diff,
                       tsdfl_motion* out);
/* Device forms, stream-ordered: d_particles P x 7 floats updated in place;
 * d_draws_out (optional) receives the generated draws (P x 6 doubles). */
int tsdfl_motion_update_device(tsdfl_ctx* ctx, float* d_particles, size_t P, const tsdfl_motion* motion,
                               uint64_t seed, uint64_t step, double* d_draws_out);
int tsdfl_motion_apply_device(tsdfl_ctx* ctx, float* d_particles, size_t P, const double* d_draws);
/* Host forms (particles and draws in host memory). */
int tsdfl_motion_update(tsdfl_ctx* ctx, float* particles, size_t P, const tsdfl_motion* motion, uint64_t seed,
                        uint64_t step);
int tsdfl_motion_apply(tsdfl_ctx* ctx, float* particles, size_t P, const double* draws);

/* ---- particle output ----
 * mcl_3d.cpp:429-449: every particle as a geometry_msgs::Pose -- position x,
 * y, z, then the quaternion x, y, z, w tf2::Quaternion::setRPY forms from its
 * roll, pitch, yaw (half angles, ZYX, in double) -- 7 doubles per particle, in
 * particle order, ready for a PoseArray.  Device form on device buffers; host
 * form copies P x 7 floats in and P x 7 doubles out. */
int tsdfl_pose_array_device(tsdfl_ctx* ctx, const float* d_particles, size_t P, double* d_poses);
int tsdfl_pose_array(tsdfl_ctx* ctx, const float* particles, size_t P, double* poses);

/* ---- seeded per-particle scan subsampling ----
 * No counterpart in the reference (its evaluator scores every reduced point
 * for every particle).  The sensor update of tsdfl_evaluate_device with each
 * particle scoring K of the N points: particle i keeps one point from each of
 * K strata of consecutive scan indices, [floor(k N / K), floor((k+1) N / K)),
 * chosen by a SplitMix64 stream seeded from (seed, i) -- tsdfl_subsample_index
 * gives the k-th kept scan index.  Weights, normalisation and mean pose as in
 * tsdfl_evaluate_device, each particle's range term counting its own kept
 * points.  Needs a code map on the tiled path (TSDFL_ERR_UNSUPPORTED
 * otherwise); 0 < K <= N.  The host form optionally returns the un-normalised
 * weights and hit counts. */
int tsdfl_evaluate_subsampled_device(tsdfl_ctx* ctx, const tsdfl_map* map, const tsdfl_model* model,
                                     float* d_particles, size_t P, const float* d_points, size_t N, const float tf[16],
                                     size_t K, uint64_t seed, float* d_pose_out);
int tsdfl_evaluate_subsampled(tsdfl_ctx* ctx, const tsdfl_map* map, const tsdfl_model* model, float* particles,
                              size_t P, const float* points, size_t N, const float tf[16], size_t K, uint64_t seed,
                              float pose_out[6], float* raw_out, uint32_t* hits_out);
/* Scan index of the k-th point particle `particle` keeps (0xffffffff for
 * arguments outside 0 <= k < K <= N). */
uint32_t tsdfl_subsample_index(uint64_t seed, uint64_t particle, uint32_t N, uint32_t K, uint32_t k);

/* No counterpart in the reference.  tsdfl_resample_systematic_device for
 * callers that must not allocate device memory while their filter runs: the
 * scratch is a fixed area compiled into the library (one per device, about
 * 2.2 MB) instead of the context's growable workspace, so M is limited to
 * 262144 particles (larger M: TSDFL_ERR_UNSUPPORTED, nothing launched).
 * Same arguments, results and error reporting as the device form.  The first
 * call on a device looks the scratch up (cudaGetSymbolAddress), and so does
 * the first call after the device's context changed (cudaDeviceReset): make
 * those calls before any stream capture.  Nothing in the scratch has to start
 * at zero.  Calls
 * whose work overlaps on one device (different streams or host threads with
 * no ordering between them) share the scratch and race: order them. */
int tsdfl_resample_systematic_static(tsdfl_ctx* ctx, const float* d_particles, size_t M, float u0,
                                     float* d_particles_out, size_t cap, uint32_t* d_count);

#ifdef __cplusplus
}
#endif

#endif
