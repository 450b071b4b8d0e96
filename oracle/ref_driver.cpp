// TEST INFRASTRUCTURE ONLY -- NOT PART OF THE PRODUCT.
//
// C entry points around the reference's own sources, compiled verbatim from
// the reference tree by tsdf_localization_gb300/_build.py (tier-A oracle):
//   include/tsdf_localization/cuda/cuda_sub_voxel_map.{h,tcc}  (map, getEntry)
//   src/evaluation/tsdf_evaluator.cpp                          (CPU sensor update, scan reduction)
//   src/evaluation/model/likelihood_evaluation.cpp             (linked by evaluate)
//   include/tsdf_localization/resampling/novel_resampling.h    (resamplers)
//   src/particle_cloud.cpp, src/util/util.cpp                  (motion model, getAngleFromMat)
// Used by the CPU tests to pin oracle/tsdf_oracle.c bit for bit, and as the
// timed CPU baseline where it can be built.
#include <tsdf_localization/evaluation/tsdf_evaluator.h>
#include <tsdf_localization/particle_cloud.h>
#include <tsdf_localization/resampling/novel_resampling.h>
#include <tsdf_localization/resampling/wheel_resampler.h>
#include <tsdf_localization/util/constant.h>

#include <omp.h>

#include <cstdint>
#include <cstring>
#include <memory>
#include <tuple>
#include <vector>

namespace tsdf_localization {

// TSDFEvaluator's ctor always builds a CudaEvaluator (tsdf_evaluator.h:78); its
// definitions live in CUDA sources (cuda_evaluator.cu) that the CPU path never
// calls, so inert definitions stand in for them here.
CudaEvaluator::CudaEvaluator(CudaSubVoxelMap<FLOAT_T, FLOAT_T>&, bool, FLOAT_T, FLOAT_T, FLOAT_T, FLOAT_T)
    : d_map_(nullptr), per_point_(false), d_grid_occ_(nullptr), d_data_(nullptr), d_particles_(nullptr),
      d_particles_ordered_(nullptr), particles_reserved_(0), d_points_(nullptr), d_points_ordered_(nullptr),
      points_reserved_(0), d_transform_(nullptr), d_new_weights_(nullptr), d_point_weights_(nullptr),
      point_weights_size_(0) {}
geometry_msgs::PoseWithCovariance CudaEvaluator::evaluate(std::vector<Particle>&, const sensor_msgs::PointCloud2&, FLOAT_T*)
{
    throw std::runtime_error("CUDA evaluator is not part of the oracle build");
}
geometry_msgs::PoseWithCovariance CudaEvaluator::evaluate(std::vector<Particle>&, const std::vector<CudaPoint>&, FLOAT_T*)
{
    throw std::runtime_error("CUDA evaluator is not part of the oracle build");
}
CudaEvaluator::~CudaEvaluator() {}

}  // namespace tsdf_localization

using namespace tsdf_localization;
using Map = CudaSubVoxelMap<FLOAT_T, FLOAT_T>;

namespace {

// Records what the reference's evaluatePose receives and returns, per particle,
// when the evaluation runs on one thread.
struct ProbeEvaluator : TSDFEvaluator {
    using TSDFEvaluator::TSDFEvaluator;
    mutable bool record = false;
    mutable std::vector<float> raw, poses;
    FLOAT_T evaluatePose(FLOAT_T* pose, const std::vector<CudaPoint> cloud, EvaluationModel& model) const override
    {
        FLOAT_T w = TSDFEvaluator::evaluatePose(pose, cloud, model);
        if (record) {
            raw.push_back(w);
            poses.insert(poses.end(), pose, pose + 12);
        }
        return w;
    }
};

// Captures the point list evaluateParticles hands to evaluate (its scan
// reduction, tsdf_evaluator.cpp:300-376) instead of scoring it.
struct ScanProbe : TSDFEvaluator {
    using TSDFEvaluator::TSDFEvaluator;
    std::vector<CudaPoint> captured;
    geometry_msgs::PoseWithCovariance evaluate(std::vector<Particle>&, const std::vector<CudaPoint>& points,
                                               FLOAT_T*, bool) override
    {
        captured = points;
        return geometry_msgs::PoseWithCovariance();
    }
};

struct SeededSystematic : SystematicResampler {
    explicit SeededSystematic(uint32_t seed) { m_generator_ptr.reset(new std::mt19937(seed)); }
};

struct SeededResidualSystematic : ResidualSystematicResampler {
    explicit SeededResidualSystematic(uint32_t seed) { m_generator_ptr.reset(new std::mt19937(seed)); }
};

struct SeededWheel : WheelResampler {
    explicit SeededWheel(uint32_t seed) { m_generator_ptr.reset(new std::mt19937(seed)); }
    uint32_t next() { return (*m_generator_ptr)(); }
};

struct SeededResidual : ResidualResampler {
    explicit SeededResidual(uint32_t seed) { m_generator_ptr.reset(new std::mt19937(seed)); }
    uint32_t next() { return (*m_generator_ptr)(); }
};

struct SeededMetropolis : MetropolisResampler {
    SeededMetropolis(size_t steps, uint32_t seed) : MetropolisResampler(steps)
    {
        m_generator_ptr.reset(new std::mt19937(seed));
    }
    uint32_t next() { return (*m_generator_ptr)(); }
};

struct SeededRejection : RejectionResampler {
    explicit SeededRejection(uint32_t seed) { m_generator_ptr.reset(new std::mt19937(seed)); }
    uint32_t next() { return (*m_generator_ptr)(); }
};

// The same generator and distributions as the reference's resamplers, drawn
// on demand in the order the caller asks for them.
struct DrawSource {
    std::mt19937 gen;
    std::uniform_real_distribution<FLOAT_T> u01{0.0, 1.0};
    std::uniform_int_distribution<size_t> index;
    DrawSource(uint32_t seed, size_t M) : gen(seed), index(0, M - 1) {}
};

// Runs a resampler on particles whose x holds their index; writes the indices.
template <class R>
size_t run_indexed(R& r, const float* w, size_t M, uint32_t* idx_out, size_t cap)
{
    ParticleCloud cloud;
    auto& v = cloud.particles();
    v.resize(M);
    for (size_t i = 0; i < M; ++i) {
        for (int k = 0; k < 6; ++k) v[i].first[k] = 0.0f;
        v[i].first[0] = (float)i;
        v[i].second = w[i];
    }
    r.resample(cloud);
    size_t n = cloud.particles().size();
    for (size_t i = 0; i < n && i < cap; ++i) idx_out[i] = (uint32_t)cloud.particles()[i].first[0];
    return n;
}

struct MapHandle {
    std::shared_ptr<Map> map;
};

}  // namespace

extern "C" {

void* ref_map_create(const float mn[3], const float mx[3], float res, float init, const float* xyzv, size_t n)
{
    auto h = new MapHandle;
    h->map = std::make_shared<Map>(mn[0], mn[1], mn[2], mx[0], mx[1], mx[2], res, init);
    std::vector<std::tuple<FLOAT_T, FLOAT_T, FLOAT_T, FLOAT_T>> data;
    data.reserve(n);
    for (size_t i = 0; i < n; ++i) data.emplace_back(xyzv[4 * i], xyzv[4 * i + 1], xyzv[4 * i + 2], xyzv[4 * i + 3]);
    try {
        h->map->setData(data);
    } catch (const std::exception&) {
        delete h;
        return nullptr;
    }
    return h;
}

// A reference map holding the given slots: built by the reference ctor from the
// coefficients' bounds, then its arrays replaced through the public raw-pointer
// accessors (cuda_sub_voxel_map.h:131-159, 309-312).
void* ref_map_from_slots(const void* coef_in, const int32_t* grid_occ, const float* data)
{
    Map::MapCoef c;
    std::memcpy(&c, coef_in, sizeof(c));
    auto h = new MapHandle;
    h->map = std::make_shared<Map>(c.min_x_, c.min_y_, c.min_z_, c.max_x_, c.max_y_, c.max_z_, c.resolution_,
                                   c.init_value_);
    if (h->map->coef().grid_occ_size_ != c.grid_occ_size_) {
        delete h;
        return nullptr;
    }
    std::memcpy(h->map->rawGridOcc(), grid_occ, sizeof(OCC_T) * c.grid_occ_size_);
    float* d = new float[c.data_size_ ? c.data_size_ : 1];
    std::memcpy(d, data, sizeof(float) * c.data_size_);
    *h->map->rawDataPtr() = d;
    h->map->coef().data_size_ = c.data_size_;
    return h;
}

void ref_map_destroy(void* h) { delete static_cast<MapHandle*>(h); }

void ref_map_coef(void* h, void* out)
{
    static_assert(sizeof(Map::MapCoef) == 120, "MapCoef layout");
    std::memcpy(out, &static_cast<MapHandle*>(h)->map->coef(), sizeof(Map::MapCoef));
}

const int32_t* ref_map_grid_occ(void* h) { return static_cast<MapHandle*>(h)->map->rawGridOcc(); }
const float* ref_map_data(void* h) { return static_cast<MapHandle*>(h)->map->rawData(); }

float ref_map_get_entry(void* h, float x, float y, float z)
{
    return static_cast<MapHandle*>(h)->map->getEntry(x, y, z);
}

// One TSDFEvaluator::evaluate(..., use_cuda=false).  particles: AoS 7 floats,
// weights overwritten with the normalised weight.  serial != 0 runs the OpenMP
// loops on one thread (deterministic weight sum) and records, per particle, the
// laser pose (12 floats) and the un-normalised weight.  Returns 0, or 1 on
// "No particle is valid!".
int ref_evaluate(void* h, const float model[4], float* particles, size_t P, const float* points, size_t N,
                 const float tf[16], float* raw_out, float* pose12_out, float pose_out[6], int serial)
{
    auto* mh = static_cast<MapHandle*>(h);
    ProbeEvaluator ev(mh->map, false, model[0], model[1], model[2], model[3]);
    std::vector<Particle> ps(P);
    for (size_t i = 0; i < P; ++i) {
        for (int k = 0; k < 6; ++k) ps[i].first[k] = particles[7 * i + k];
        ps[i].second = particles[7 * i + 6];
    }
    std::vector<CudaPoint> pts(N);
    for (size_t j = 0; j < N; ++j) pts[j] = CudaPoint(points[3 * j], points[3 * j + 1], points[3 * j + 2]);
    FLOAT_T tfm[16];
    std::memcpy(tfm, tf, sizeof(tfm));
    int old_levels = omp_get_max_active_levels();
    if (serial) {
        omp_set_max_active_levels(0);
        ev.record = true;
    }
    int rc = 0;
    geometry_msgs::PoseWithCovariance pose;
    try {
        pose = ev.evaluate(ps, pts, tfm, false);
    } catch (const std::runtime_error&) {
        rc = 1;
    }
    omp_set_max_active_levels(old_levels);
    if (rc) return rc;
    for (size_t i = 0; i < P; ++i) particles[7 * i + 6] = ps[i].second;
    if (serial) {
        if (raw_out) std::memcpy(raw_out, ev.raw.data(), sizeof(float) * ev.raw.size());
        if (pose12_out) std::memcpy(pose12_out, ev.poses.data(), sizeof(float) * ev.poses.size());
    }
    if (pose_out) {
        pose_out[0] = (float)pose.pose.position.x;
        pose_out[1] = (float)pose.pose.position.y;
        pose_out[2] = (float)pose.pose.position.z;
        for (int k = 0; k < 3; ++k) pose_out[3 + k] = (float)tf2::rpy_hook()[k];
    }
    return 0;
}

// The draw SystematicResampler makes first (novel_resampling.h:44-49).
float ref_draw_u0(uint32_t seed, size_t M)
{
    std::mt19937 g(seed);
    auto inverse_M = 1.0 / M;
    std::uniform_real_distribution<FLOAT_T> d(0.0, inverse_M);
    return d(g);
}

// SystematicResampler::resample on weights w with its generator seeded by seed;
// writes the source index of every emitted particle.  Returns the count.
size_t ref_resample_systematic(const float* w, size_t M, uint32_t seed, uint32_t* idx_out, size_t cap)
{
    ParticleCloud cloud;
    cloud.particles().resize(M);
    for (size_t i = 0; i < M; ++i) {
        for (int k = 0; k < 6; ++k) cloud.particles()[i].first[k] = 0;
        cloud.particles()[i].first[0] = (float)i;
        cloud.particles()[i].second = w[i];
    }
    SeededSystematic r(seed);
    r.resample(cloud);
    size_t n = cloud.particles().size();
    for (size_t i = 0; i < n && i < cap; ++i) idx_out[i] = (uint32_t)cloud.particles()[i].first[0];
    return n;
}

// ResidualSystematicResampler's draw u ~ U[0, 1) for a generator seeded by seed.
float ref_draw_u01(uint32_t seed)
{
    std::mt19937 g(seed);
    std::uniform_real_distribution<FLOAT_T> d(0.0, 1.0);
    return d(g);
}

// ResidualSystematicResampler::resample on weights w, generator seeded by seed.
size_t ref_resample_residual_systematic(const float* w, size_t M, uint32_t seed, uint32_t* idx_out, size_t cap)
{
    ParticleCloud cloud;
    cloud.particles().resize(M);
    for (size_t i = 0; i < M; ++i) {
        for (int k = 0; k < 6; ++k) cloud.particles()[i].first[k] = 0;
        cloud.particles()[i].first[0] = (float)i;
        cloud.particles()[i].second = w[i];
    }
    SeededResidualSystematic r(seed);
    r.resample(cloud);
    size_t n = cloud.particles().size();
    for (size_t i = 0; i < n && i < cap; ++i) idx_out[i] = (uint32_t)cloud.particles()[i].first[0];
    return n;
}

// TSDFEvaluator::evaluateParticles' scan reduction (ignore_tf) on a cloud with
// float fields x, y, z and a short field ring; writes the reduced points in the
// order evaluate receives them.  Returns their number.
size_t ref_reduce_scan(const float* xyz, const int16_t* ring, size_t n, float cell, float* out, size_t cap)
{
    auto map = std::make_shared<Map>(0.0f, 0.0f, 0.0f, 1.0f, 1.0f, 1.0f, 0.1f, 0.0f);
    ScanProbe ev(map, false, 0.9f, 0.1f, 0.0f, 100.0f, cell);
    sensor_msgs::PointCloud2 cloud;
    cloud.height = 1;
    cloud.width = (uint32_t)n;
    cloud.point_step = 16;
    cloud.row_step = 16 * (uint32_t)n;
    const char* names[4] = {"x", "y", "z", "ring"};
    for (int f = 0; f < 4; ++f) {
        sensor_msgs::PointField pf;
        pf.name = names[f];
        pf.offset = 4 * f;
        cloud.fields.push_back(pf);
    }
    cloud.data.resize(16 * n);
    for (size_t i = 0; i < n; ++i) {
        std::memcpy(&cloud.data[16 * i], xyz + 3 * i, 12);
        std::memcpy(&cloud.data[16 * i + 12], ring + i, 2);
    }
    ParticleCloud pc;
    ev.evaluateParticles(pc, cloud, "base", "scan", false, true);
    for (size_t i = 0; i < ev.captured.size() && i < cap; ++i) {
        out[3 * i] = ev.captured[i].x;
        out[3 * i + 1] = ev.captured[i].y;
        out[3 * i + 2] = ev.captured[i].z;
    }
    return ev.captured.size();
}

// The reference's other resamplers with generators seeded by seed (outputs as indices).
size_t ref_resample_wheel(const float* w, size_t M, uint32_t seed, uint32_t* idx_out, size_t cap)
{
    SeededWheel r(seed);
    return run_indexed(r, w, M, idx_out, cap);
}
size_t ref_resample_residual(const float* w, size_t M, uint32_t seed, uint32_t* idx_out, size_t cap)
{
    SeededResidual r(seed);
    return run_indexed(r, w, M, idx_out, cap);
}
size_t ref_resample_metropolis(const float* w, size_t M, uint32_t steps, uint32_t seed, uint32_t* idx_out,
                               size_t cap)
{
    SeededMetropolis r(steps, seed);
    return run_indexed(r, w, M, idx_out, cap);
}
size_t ref_resample_rejection(const float* w, size_t M, uint32_t seed, uint32_t* idx_out, size_t cap)
{
    SeededRejection r(seed);
    return run_indexed(r, w, M, idx_out, cap);
}

// The generator's next output after the seeded resampler ran (kind 0 wheel,
// 1 residual, 2 metropolis).
uint32_t ref_resample_next(int kind, const float* w, size_t M, uint32_t steps, uint32_t seed)
{
    std::vector<uint32_t> idx(M);
    if (kind == 0) {
        SeededWheel r(seed);
        run_indexed(r, w, M, idx.data(), M);
        return r.next();
    }
    if (kind == 1) {
        SeededResidual r(seed);
        run_indexed(r, w, M, idx.data(), M);
        return r.next();
    }
    SeededMetropolis r(steps, seed);
    run_indexed(r, w, M, idx.data(), M);
    return r.next();
}

// The draws those resamplers take from a generator seeded by seed, in their order.
void ref_draws_wheel(uint32_t seed, size_t M, double* out)
{
    std::mt19937 g(seed);
    std::uniform_real_distribution<> d(0.0, 1.0);
    for (size_t i = 0; i < M; ++i) out[i] = d(g);
}
void ref_draws_residual(uint32_t seed, size_t M, size_t K, uint32_t* out)
{
    std::mt19937 g(seed);
    std::uniform_int_distribution<size_t> d(0, M - 1);
    for (size_t k = 0; k < K; ++k) out[k] = (uint32_t)d(g);
}
void ref_draws_metropolis(uint32_t seed, size_t M, uint32_t steps, float* u, uint32_t* j)
{
    std::mt19937 g(seed);
    std::uniform_real_distribution<FLOAT_T> du(0.0, 1.0);
    std::uniform_int_distribution<size_t> dj(0, M - 1);
    for (size_t i = 0; i < (size_t)M * steps; ++i) {
        u[i] = du(g);
        j[i] = (uint32_t)dj(g);
    }
}
void* ref_draw_source_create(uint32_t seed, size_t M) { return new DrawSource(seed, M); }
void ref_draw_source_destroy(void* s) { delete static_cast<DrawSource*>(s); }
float ref_draw_source_u(void* s, size_t, uint32_t)
{
    auto* d = static_cast<DrawSource*>(s);
    return d->u01(d->gen);
}
uint32_t ref_draw_source_j(void* s, size_t, uint32_t)
{
    auto* d = static_cast<DrawSource*>(s);
    return (uint32_t)d->index(d->gen);
}

// ParticleCloud::motion_update (particle_cloud.cpp:456-497) with every noise
// parameter zero: each particle's draws are exactly (dx, dy, dz, roll, pitch,
// yaw), so apply_model's pose composition (:499-617) runs on known increments.
// particles: P x 7 floats, updated in place.
void ref_motion_update(float* particles, size_t P, const float delta[6])
{
    ParticleCloud pc;
    pc.setMotionParameters(0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0);
    auto& v = pc.particles();
    v.resize(P);
    for (size_t i = 0; i < P; ++i) {
        for (int k = 0; k < 6; ++k) v[i].first[k] = particles[7 * i + k];
        v[i].second = particles[7 * i + 6];
    }
    pc.motion_update(delta[0], delta[1], delta[2], delta[3], delta[4], delta[5], 0, 0);
    for (size_t i = 0; i < P; ++i) {
        for (int k = 0; k < 6; ++k) particles[7 * i + k] = pc.particles()[i].first[k];
        particles[7 * i + 6] = pc.particles()[i].second;
    }
}

int ref_omp_threads(void) { return (int)OMP_THREADS; }

}  // extern "C"
