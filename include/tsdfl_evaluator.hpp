/* C++ host side of libtsdfl: RAII handles, the sensor update and systematic
 * resampling on the caller's particle containers, and -- when compiled inside
 * tsdf_localization (define TSDFL_WITH_TSDF_LOCALIZATION after including its
 * headers) -- the drop-in plug-ins for its Evaluator and Resampler interfaces:
 *
 *   tsdf_localization::GpuTsdfEvaluator      replaces CudaEvaluator
 *       (include/tsdf_localization/cuda/cuda_evaluator.h:94-125)
 *   tsdf_localization::GpuSystematicResampler replaces SystematicResampler
 *       (include/tsdf_localization/resampling/novel_resampling.h:38-74)
 *   tsdf_localization::GpuResidualSystematicResampler replaces
 *       ResidualSystematicResampler (novel_resampling.h:76-104)
 *   tsdf_localization::gpu_reduce_scan replaces the scan reduction block of
 *       TSDFEvaluator::evaluateParticles (src/evaluation/tsdf_evaluator.cpp:304-374)
 *   tsdf_localization::GpuMotionModel replaces ParticleCloud's motion-update
 *       overloads (src/particle_cloud.cpp:153-617)
 *   tsdf_localization::GpuWheelResampler, GpuResidualResampler,
 *       GpuMetropolisResampler, GpuRejectionResampler replace the other
 *       resamplers mcl_3d selects (mcl_3d.cpp:246-261)
 *   tsdfl::Map::from_h5 replaces createTSDFMap's loading of the map file
 *       (include/tsdf_localization/map/map_util.h:17-154) without HDF5
 *
 * Errors surface as std::runtime_error carrying libtsdfl's message, as the
 * reference's evaluators throw them ("No particle is valid!" for a zero
 * weight sum). */
#ifndef TSDFL_EVALUATOR_HPP
#define TSDFL_EVALUATOR_HPP

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "tsdfl.h"

namespace tsdfl {

inline void check(int rc)
{
    if (rc != TSDFL_OK) throw std::runtime_error(tsdfl_last_error());
}

// One device with its stream and workspace.
class Context {
public:
    explicit Context(int device = 0) { check(tsdfl_ctx_create(device, &h_)); }
    ~Context() { tsdfl_ctx_destroy(h_); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    tsdfl_ctx* get() const { return h_; }
    void set_stream(void* cuda_stream) { check(tsdfl_ctx_set_stream(h_, cuda_stream)); }
    void sync() { check(tsdfl_ctx_sync(h_)); }

private:
    tsdfl_ctx* h_ = nullptr;
};

// A likelihood map on the device, from the reference's map contents: its
// MapCoef, brick table and float slots (CudaSubVoxelMap::coef(), rawGridOcc(),
// rawData()).  sigma is the likelihood's standard deviation the slots were made
// with (map_util.h:124-127); slots that are not likelihood values of it keep
// float storage.
class Map {
public:
    Map(Context& ctx, const tsdfl_map_coef& coef, const int32_t* grid_occ, const float* data, float sigma = 0.1f,
        uint32_t flags = 0)
    {
        check(tsdfl_map_create(ctx.get(), &coef, grid_occ, data, sigma, flags, &h_));
    }
    ~Map() { tsdfl_map_destroy(h_); }
    Map(const Map&) = delete;
    Map& operator=(const Map&) = delete;
    tsdfl_map* get() const { return h_; }

    // createTSDFMap(h5_filename, free_map, sigma) (map_util.h:17-154) from a map
    // file in the reference's HDF5 layout, read without the HDF5 library
    // (tsdfl_read_map_h5): the device map, and the free-space cells (x, y, z
    // per cell) when free_xyz is given.  voxel_mm is MAP_RESOLUTION (64).
    static std::unique_ptr<Map> from_h5(Context& ctx, const char* path, int voxel_mm = 64, float sigma = 0.1f,
                                        uint32_t flags = TSDFL_MAP_DENSE, std::vector<float>* free_xyz = nullptr)
    {
        int32_t* pos = nullptr;
        uint32_t* raw = nullptr;
        size_t n = 0;
        int32_t edge = 0;
        check(tsdfl_read_map_h5(path, &pos, &raw, &n, &edge));
        tsdfl_map_coef coef{};
        int32_t* grid_occ = nullptr;
        uint16_t* codes = nullptr;
        float* free_cells = nullptr;
        size_t n_free = 0;
        int rc = tsdfl_build_map_codes(pos, raw, n, edge, voxel_mm, sigma, &coef, &grid_occ, &codes,
                                       free_xyz ? &free_cells : nullptr, free_xyz ? &n_free : nullptr);
        tsdfl_free(pos);
        tsdfl_free(raw);
        std::unique_ptr<Map> m(new Map());
        if (rc == TSDFL_OK) rc = tsdfl_map_create_codes(ctx.get(), &coef, grid_occ, codes, sigma, flags, &m->h_);
        if (rc == TSDFL_OK && free_xyz) free_xyz->assign(free_cells, free_cells + 3 * n_free);
        tsdfl_free(grid_occ);
        tsdfl_free(codes);
        tsdfl_free(free_cells);
        check(rc);
        return m;
    }

private:
    Map() = default;
    tsdfl_map* h_ = nullptr;
};

struct Pose6 {
    float x = 0, y = 0, z = 0, roll = 0, pitch = 0, yaw = 0;
};

// The sensor update of TSDFEvaluator::evaluate (tsdf_evaluator.cpp:78-245) on
// any particle type with `float first[6]` (x, y, z, roll, pitch, yaw) and
// `float second` (the weight) -- tsdf_localization::Particle -- and any point
// type with float members x, y, z.  Writes the normalised weights into the
// particles and returns the weighted mean pose; an empty scan leaves the
// particles untouched and returns false.
class SensorUpdate {
public:
    SensorUpdate(Context& ctx, Map& map, float a_hit = 0.9f, float a_range = 0.1f, float a_max = 0.0f,
                 float max_range = 100.0f, uint32_t flags = TSDFL_SUM_EXACT)
        : ctx_(ctx), map_(map), flags_(flags)
    {
        model_.a_hit = a_hit;
        model_.a_range = a_range;
        model_.a_max = a_max;
        model_.max_range = max_range;
    }

    template <class ParticleT, class PointT>
    bool evaluate(std::vector<ParticleT>& particles, const std::vector<PointT>& points, const float tf[16],
                  Pose6* pose)
    {
        if (points.empty()) return false;
        parts_.resize(7 * particles.size());
        for (size_t i = 0; i < particles.size(); ++i) {
            for (int k = 0; k < 6; ++k) parts_[7 * i + k] = particles[i].first[k];
            parts_[7 * i + 6] = particles[i].second;
        }
        pts_.resize(3 * points.size());
        for (size_t j = 0; j < points.size(); ++j) {
            pts_[3 * j] = points[j].x;
            pts_[3 * j + 1] = points[j].y;
            pts_[3 * j + 2] = points[j].z;
        }
        float out[6];
        check(tsdfl_evaluate(ctx_.get(), map_.get(), &model_, parts_.data(), particles.size(), pts_.data(),
                             points.size(), tf, flags_, out));
        for (size_t i = 0; i < particles.size(); ++i) particles[i].second = parts_[7 * i + 6];
        if (pose) *pose = Pose6{out[0], out[1], out[2], out[3], out[4], out[5]};
        return true;
    }

    // The scan reduction (ScanReducer) and evaluate() in one call on a
    // PointCloud2's data; false when no point survives the reduction.
    template <class ParticleT>
    bool evaluate_cloud(std::vector<ParticleT>& particles, const void* data, size_t n_points, uint32_t point_step,
                        uint32_t x_offset, uint32_t ring_offset, float reduction_cell_size, uint32_t scan_flags,
                        const float tf[16], Pose6* pose, size_t* n_reduced = nullptr)
    {
        parts_.resize(7 * (particles.size() ? particles.size() : 1));
        for (size_t i = 0; i < particles.size(); ++i) {
            for (int k = 0; k < 6; ++k) parts_[7 * i + k] = particles[i].first[k];
            parts_[7 * i + 6] = particles[i].second;
        }
        float out[6];
        size_t m = 0;
        check(tsdfl_evaluate_cloud(ctx_.get(), map_.get(), &model_, parts_.data(), particles.size(), data, n_points,
                                   point_step, x_offset, ring_offset, reduction_cell_size, scan_flags, tf, flags_,
                                   out, &m));
        if (n_reduced) *n_reduced = m;
        if (m == 0) return false;
        for (size_t i = 0; i < particles.size(); ++i) particles[i].second = parts_[7 * i + 6];
        if (pose) *pose = Pose6{out[0], out[1], out[2], out[3], out[4], out[5]};
        return true;
    }

private:
    Context& ctx_;
    Map& map_;
    tsdfl_model model_{};
    uint32_t flags_;
    std::vector<float> parts_, pts_;
};

// SystematicResampler::resample (novel_resampling.h:41-72) for a given draw
// u0 in [0, 1/M): replaces `particles` by the reference's output sequence
// (bit-exact, including its particle count, which is not always M).
template <class ParticleT>
void resample_systematic(Context& ctx, std::vector<ParticleT>& particles, float u0)
{
    const size_t M = particles.size();
    if (M == 0) return;
    std::vector<uint32_t> idx(2 * M + 16);
    size_t count = 0;
    // the reference's Particle (pose floats, then the weight) is the M x 7
    // float cloud the particles form reads: pass it as it lies
    const char* p0 = reinterpret_cast<const char*>(particles.data());
    const bool cloud = std::is_same<decltype(particles[0].second), float>::value &&
                       sizeof(ParticleT) == 7 * sizeof(float) &&
                       reinterpret_cast<const char*>(&particles[0].second) - p0 == 6 * sizeof(float);
    std::vector<float> w;
    auto call = [&]() {
        if (cloud) {
            check(tsdfl_resample_systematic_particles(ctx.get(), reinterpret_cast<const float*>(p0), M, u0,
                                                      idx.data(), idx.size(), &count));
        } else {
            if (w.empty()) {
                w.resize(M);
                for (size_t i = 0; i < M; ++i) w[i] = particles[i].second;
            }
            check(tsdfl_resample_systematic(ctx.get(), w.data(), M, u0, idx.data(), idx.size(), &count));
        }
    };
    call();
    if (count > idx.size()) {   // more draws than the first guess held: ask again with room for all
        idx.resize(count);
        call();
    }
    std::vector<ParticleT> out;
    out.reserve(count);
    for (size_t k = 0; k < count; ++k) out.push_back(particles[idx[k]]);
    particles = std::move(out);
}

// ResidualSystematicResampler::resample (novel_resampling.h:76-104) for a given
// draw u0 in [0, 1): replaces `particles` by the reference's output sequence.
template <class ParticleT>
void resample_residual_systematic(Context& ctx, std::vector<ParticleT>& particles, float u0)
{
    const size_t M = particles.size();
    if (M == 0) return;
    std::vector<float> w(M);
    for (size_t i = 0; i < M; ++i) w[i] = particles[i].second;
    std::vector<uint32_t> idx(2 * M + 16);
    size_t count = 0;
    check(tsdfl_resample_residual_systematic(ctx.get(), w.data(), M, u0, idx.data(), idx.size(), &count));
    if (count > idx.size()) {
        idx.resize(count);
        check(tsdfl_resample_residual_systematic(ctx.get(), w.data(), M, u0, idx.data(), idx.size(), &count));
    }
    std::vector<ParticleT> out;
    out.reserve(count);
    for (size_t k = 0; k < count; ++k) out.push_back(particles[idx[k]]);
    particles = std::move(out);
}

// The reference's other resamplers (Wheel, Residual, Metropolis, Rejection) on
// a caller's particle vector.  With a generator, the draws are taken from it
// with the reference's distributions and in its order (Rejection excepted, see
// below), so the same generator state gives the reference's particles bit for
// bit and leaves the generator where the reference leaves it; without one, the
// device draws them from Philox keyed by seed.
namespace detail {
template <class ParticleT>
std::vector<float> weights_of(const std::vector<ParticleT>& particles)
{
    std::vector<float> w(particles.size());
    for (size_t i = 0; i < particles.size(); ++i) w[i] = particles[i].second;
    return w;
}
template <class ParticleT>
void take(std::vector<ParticleT>& particles, const std::vector<uint32_t>& idx)
{
    std::vector<ParticleT> out;
    out.reserve(idx.size());
    for (uint32_t k : idx) out.push_back(particles[k]);
    particles = std::move(out);
}
}  // namespace detail

// WheelResampler (wheel_resampler.cpp:6-33): one uniform_real_distribution<>
// draw per particle.
template <class ParticleT, class Generator>
void resample_wheel(Context& ctx, std::vector<ParticleT>& particles, Generator* gen, uint64_t seed = 0)
{
    const size_t M = particles.size();
    if (M == 0) return;
    const std::vector<float> w = detail::weights_of(particles);
    std::vector<double> draws;
    if (gen) {
        std::uniform_real_distribution<> d(0.0, 1.0);
        draws.resize(M);
        for (size_t i = 0; i < M; ++i) draws[i] = d(*gen);
    }
    std::vector<uint32_t> idx(M);
    check(tsdfl_resample_wheel(ctx.get(), w.data(), M, gen ? draws.data() : nullptr, seed, idx.data()));
    detail::take(particles, idx);
}

// ResidualResampler (novel_resampling.h:9-35): uniform_int_distribution
// draws, as many as the reference takes (counted on the host from the
// weights, novel_resampling.h:19-30), then the copies on the device.
template <class ParticleT, class Generator>
void resample_residual(Context& ctx, std::vector<ParticleT>& particles, Generator* gen, uint64_t seed = 0)
{
    const size_t M = particles.size();
    if (M == 0) return;
    const std::vector<float> w = detail::weights_of(particles);
    std::vector<uint32_t> draws;
    if (gen) {
        std::uniform_int_distribution<size_t> d(0, M - 1);
        size_t filled = 0;
        while (filled < M) {
            const size_t r = d(*gen);
            draws.push_back((uint32_t)r);
            const float expected = w[r] * M;
            const size_t left = M - filled;
            const float insertions = expected <= left ? expected : left;
            for (size_t k = 0; k < insertions; ++k) ++filled;
        }
    }
    std::vector<uint32_t> idx(M);
    check(tsdfl_resample_residual(ctx.get(), w.data(), M, gen ? draws.data() : nullptr, draws.size(), seed,
                                  idx.data()));
    detail::take(particles, idx);
}

// MetropolisResampler(steps) (novel_resampling.h:106-143): per output and
// step, a uniform_real_distribution<float> then a uniform_int_distribution draw.
template <class ParticleT, class Generator>
void resample_metropolis(Context& ctx, std::vector<ParticleT>& particles, uint32_t steps, Generator* gen,
                         uint64_t seed = 0)
{
    const size_t M = particles.size();
    if (M == 0) return;
    const std::vector<float> w = detail::weights_of(particles);
    std::vector<float> u;
    std::vector<uint32_t> j;
    if (gen) {
        std::uniform_real_distribution<float> du(0.0, 1.0);
        std::uniform_int_distribution<size_t> dj(0, M - 1);
        u.resize(M * steps);
        j.resize(M * steps);
        for (size_t k = 0; k < M * steps; ++k) {
            u[k] = du(*gen);
            j[k] = (uint32_t)dj(*gen);
        }
    }
    std::vector<uint32_t> idx(M);
    check(tsdfl_resample_metropolis(ctx.get(), w.data(), M, steps, gen ? u.data() : nullptr,
                                    gen ? j.data() : nullptr, seed, idx.data()));
    detail::take(particles, idx);
}

// RejectionResampler (novel_resampling.h:146-187) with device draws: how many
// draws the reference takes depends on its outcomes, so its sequence cannot
// be handed over in advance.
template <class ParticleT>
void resample_rejection(Context& ctx, std::vector<ParticleT>& particles, uint64_t seed)
{
    const size_t M = particles.size();
    if (M == 0) return;
    const std::vector<float> w = detail::weights_of(particles);
    std::vector<uint32_t> idx(M);
    check(tsdfl_resample_rejection(ctx.get(), w.data(), M, seed, idx.data()));
    detail::take(particles, idx);
}

// mcl_3d.cpp:429-449: the particles as Pose records (position, setRPY
// quaternion x, y, z, w), 7 doubles each.
template <class ParticleT>
std::vector<double> pose_array(Context& ctx, const std::vector<ParticleT>& particles)
{
    std::vector<float> p(7 * particles.size());
    for (size_t i = 0; i < particles.size(); ++i) {
        for (int k = 0; k < 6; ++k) p[7 * i + k] = particles[i].first[k];
        p[7 * i + 6] = particles[i].second;
    }
    std::vector<double> out(7 * particles.size());
    check(tsdfl_pose_array(ctx.get(), p.data(), particles.size(), out.data()));
    return out;
}

// The scan reduction of TSDFEvaluator::evaluateParticles
// (tsdf_evaluator.cpp:304-376) on the device: the points it hands to evaluate,
// in its order, from a PointCloud2's data.
class ScanReducer {
public:
    ScanReducer(Context& ctx, float reduction_cell_size = 0.064f, uint32_t flags = 0)
        : ctx_(ctx), cell_(reduction_cell_size), flags_(flags)
    {
    }

    float cell() const { return cell_; }
    uint32_t flags() const { return flags_; }

    // data: n_points records of point_step bytes, x, y, z floats at x_offset,
    // the ring an int16 at ring_offset.
    template <class PointT>
    std::vector<PointT> reduce(const void* data, size_t n_points, uint32_t point_step, uint32_t x_offset,
                               uint32_t ring_offset)
    {
        buf_.resize(3 * (n_points ? n_points : 1));
        size_t m = 0;
        check(tsdfl_reduce_scan(ctx_.get(), data, n_points, point_step, x_offset, ring_offset, cell_, flags_,
                                buf_.data(), n_points, &m));
        std::vector<PointT> out;
        out.reserve(m);
        for (size_t i = 0; i < m; ++i) {
            PointT p;
            p.x = buf_[3 * i];
            p.y = buf_[3 * i + 1];
            p.z = buf_[3 * i + 2];
            out.push_back(p);
        }
        return out;
    }

private:
    Context& ctx_;
    float cell_;
    uint32_t flags_;
    std::vector<float> buf_;
};

// ParticleCloud's motion model (particle_cloud.cpp:153-617) on the device.
// a_1 .. a_12 as setMotionParameters takes them (0.1 each by default).
class MotionModel {
public:
    explicit MotionModel(Context& ctx, uint64_t seed = 0) : ctx_(ctx), seed_(seed)
    {
        for (int k = 0; k < 12; ++k) a_[k] = 0.1f;
    }

    void setMotionParameters(float a1, float a2, float a3, float a4, float a5, float a6, float a7, float a8,
                             float a9, float a10, float a11, float a12)
    {
        const float v[12] = {a1, a2, a3, a4, a5, a6, a7, a8, a9, a10, a11, a12};
        for (int k = 0; k < 12; ++k) a_[k] = v[k];
    }

    // The distributions of an overload (TSDFL_MOTION_*), see tsdfl_motion_model.
    tsdfl_motion distributions(int kind, const double* in, size_t n_in, float time_diff) const
    {
        tsdfl_motion m;
        check(tsdfl_motion_model(kind, a_, in, n_in, time_diff, &m));
        return m;
    }

    // Device-drawn noise: one counter-based stream per call.
    template <class ParticleT>
    void update(std::vector<ParticleT>& particles, const tsdfl_motion& m)
    {
        to_floats(particles);
        check(tsdfl_motion_update(ctx_.get(), parts_.data(), particles.size(), &m, seed_, step_++));
        from_floats(particles);
    }

    // Noise from the caller's generator in the reference's order: six
    // std::normal_distribution<> objects, x, y, z, roll, pitch, yaw per
    // particle (particle_cloud.cpp:506-511), so a generator in the same state
    // gives the reference's particles bit for bit.
    template <class ParticleT, class Generator>
    void update_with(std::vector<ParticleT>& particles, const tsdfl_motion& m, Generator& gen)
    {
        std::normal_distribution<> dist[6] = {
            std::normal_distribution<>(m.mean[0], m.stddev[0]), std::normal_distribution<>(m.mean[1], m.stddev[1]),
            std::normal_distribution<>(m.mean[2], m.stddev[2]), std::normal_distribution<>(m.mean[3], m.stddev[3]),
            std::normal_distribution<>(m.mean[4], m.stddev[4]), std::normal_distribution<>(m.mean[5], m.stddev[5])};
        draws_.resize(6 * particles.size());
        for (size_t i = 0; i < particles.size(); ++i)
            for (int k = 0; k < 6; ++k) draws_[6 * i + k] = dist[k](gen);
        to_floats(particles);
        check(tsdfl_motion_apply(ctx_.get(), parts_.data(), particles.size(), draws_.data()));
        from_floats(particles);
    }

private:
    template <class ParticleT>
    void to_floats(const std::vector<ParticleT>& particles)
    {
        parts_.resize(7 * (particles.size() ? particles.size() : 1));
        for (size_t i = 0; i < particles.size(); ++i) {
            for (int k = 0; k < 6; ++k) parts_[7 * i + k] = particles[i].first[k];
            parts_[7 * i + 6] = particles[i].second;
        }
    }
    template <class ParticleT>
    void from_floats(std::vector<ParticleT>& particles) const
    {
        for (size_t i = 0; i < particles.size(); ++i)
            for (int k = 0; k < 6; ++k) particles[i].first[k] = parts_[7 * i + k];
    }

    Context& ctx_;
    uint64_t seed_;
    uint64_t step_ = 0;
    float a_[12];
    std::vector<float> parts_;
    std::vector<double> draws_;
};

// Cell-centre reduction of a scan as CudaEvaluator's point-cloud overload
// performs it (cuda_evaluator.cu:77-115): every point maps to the centre of its
// 0.064 m cell, each centre kept once.  Order does not matter downstream: the
// exact-mode sums do not depend on it.
template <class PointT>
std::vector<PointT> reduce_to_cells(const std::vector<PointT>& points)
{
    std::vector<PointT> c;
    c.reserve(points.size());
    for (const auto& p : points) {
        PointT q = p;
        q.x = static_cast<float>(std::floor(p.x / 0.064) * 0.064 + 0.032);
        q.y = static_cast<float>(std::floor(p.y / 0.064) * 0.064 + 0.032);
        q.z = static_cast<float>(std::floor(p.z / 0.064) * 0.064 + 0.032);
        c.push_back(q);
    }
    auto key = [](const PointT& a) {
        uint32_t k[3];
        std::memcpy(&k[0], &a.x, 4);
        std::memcpy(&k[1], &a.y, 4);
        std::memcpy(&k[2], &a.z, 4);
        return std::make_tuple(k[0], k[1], k[2]);
    };
    std::sort(c.begin(), c.end(), [&](const PointT& a, const PointT& b) { return key(a) < key(b); });
    c.erase(std::unique(c.begin(), c.end(),
                        [](const PointT& a, const PointT& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }),
            c.end());
    return c;
}

}  // namespace tsdfl

#ifdef TSDFL_WITH_TSDF_LOCALIZATION
#include <memory>

namespace tsdf_localization {

// Byte offset of a PointCloud2 field; a missing field throws as
// PointCloud2ConstIterator's constructor does.
inline uint32_t tsdfl_field_offset(const sensor_msgs::PointCloud2& cloud, const std::string& name)
{
    for (const auto& f : cloud.fields)
        if (f.name == name) return f.offset;
    throw std::runtime_error("Field " + name + " does not exist");
}

// The points TSDFEvaluator::evaluateParticles scores (its ordered_points,
// tsdf_evaluator.cpp:304-374), reduced on the device: same points, same order.
inline std::vector<CudaPoint> gpu_reduce_scan(tsdfl::ScanReducer& reducer, const sensor_msgs::PointCloud2& cloud)
{
    return reducer.reduce<CudaPoint>(cloud.data.data(), (size_t)cloud.width * cloud.height, cloud.point_step,
                                     tsdfl_field_offset(cloud, "x"), tsdfl_field_offset(cloud, "ring"));
}

// Drop-in for CudaEvaluator: same constructor arguments (per_point is accepted;
// both reference modes give the same weights here) and the same two evaluate
// overloads.  The map's slots are copied to the device once, here.
class GpuTsdfEvaluator : public Evaluator {
public:
    GpuTsdfEvaluator(CudaSubVoxelMap<FLOAT_T, FLOAT_T>& map, bool per_point = false, FLOAT_T a_hit = 0.9,
                     FLOAT_T a_range = 0.1, FLOAT_T a_max = 0.0, FLOAT_T max_range = 100.0, int device = 0,
                     float sigma = 0.1f)
        : ctx_(new tsdfl::Context(device)),
          map_(new tsdfl::Map(*ctx_, *reinterpret_cast<const tsdfl_map_coef*>(&map.coef()), map.rawGridOcc(),
                              map.rawData(), sigma)),
          update_(new tsdfl::SensorUpdate(*ctx_, *map_, a_hit, a_range, a_max, max_range))
    {
        static_assert(sizeof(tsdfl_map_coef) == sizeof(typename CudaSubVoxelMap<FLOAT_T, FLOAT_T>::MapCoef),
                      "MapCoef layout");
        (void)per_point;
    }

    geometry_msgs::PoseWithCovariance evaluate(std::vector<Particle>& particles,
                                               const sensor_msgs::PointCloud2& real_cloud,
                                               FLOAT_T tf_matrix[16]) override
    {
        sensor_msgs::PointCloud2ConstIterator<float> iter_x(real_cloud, "x");
        std::vector<CudaPoint> points;
        for (; iter_x != iter_x.end(); ++iter_x) points.push_back(CudaPoint(iter_x[0], iter_x[1], iter_x[2]));
        return evaluate(particles, tsdfl::reduce_to_cells(points), tf_matrix);
    }

    geometry_msgs::PoseWithCovariance evaluate(std::vector<Particle>& particles, const std::vector<CudaPoint>& points,
                                               FLOAT_T tf_matrix[16]) override
    {
        geometry_msgs::PoseWithCovariance out;
        tsdfl::Pose6 p;
        if (!update_->evaluate(particles, points, tf_matrix, &p)) return out;
        return to_msg(p);
    }

    // TSDFEvaluator::evaluateParticles after its tf lookup
    // (tsdf_evaluator.cpp:304-376): the scan reduction and the update in one
    // call, the reduced points staying on the device.
    geometry_msgs::PoseWithCovariance evaluateCloud(std::vector<Particle>& particles,
                                                    const sensor_msgs::PointCloud2& cloud, FLOAT_T tf_matrix[16],
                                                    FLOAT_T reduction_cell_size = 0.064, uint32_t scan_flags = 0)
    {
        geometry_msgs::PoseWithCovariance out;
        tsdfl::Pose6 p;
        if (!update_->evaluate_cloud(particles, cloud.data.data(), (size_t)cloud.width * cloud.height,
                                     cloud.point_step, tsdfl_field_offset(cloud, "x"),
                                     tsdfl_field_offset(cloud, "ring"), reduction_cell_size, scan_flags, tf_matrix,
                                     &p))
            return out;
        return to_msg(p);
    }

private:
    static geometry_msgs::PoseWithCovariance to_msg(const tsdfl::Pose6& p)
    {
        geometry_msgs::PoseWithCovariance out;
        out.pose.position.x = p.x;
        out.pose.position.y = p.y;
        out.pose.position.z = p.z;
        tf2::Quaternion q;   // as tsdf_evaluator.cpp:226-228 converts the mean pose
        q.setRPY(p.roll, p.pitch, p.yaw);
        tf2::convert(q, out.pose.orientation);
        return out;
    }

private:
    std::unique_ptr<tsdfl::Context> ctx_;
    std::unique_ptr<tsdfl::Map> map_;
    std::unique_ptr<tsdfl::SensorUpdate> update_;
};

// The particle cloud as the poses of mcl_3d's PoseArray (mcl_3d.cpp:429-449):
// pose_array.poses = gpu_particle_poses(ctx, particle_cloud_.particles()).
inline std::vector<geometry_msgs::Pose> gpu_particle_poses(tsdfl::Context& ctx, const std::vector<Particle>& particles)
{
    const std::vector<double> v = tsdfl::pose_array(ctx, particles);
    std::vector<geometry_msgs::Pose> poses(particles.size());
    for (size_t i = 0; i < particles.size(); ++i) {
        poses[i].position.x = v[7 * i];
        poses[i].position.y = v[7 * i + 1];
        poses[i].position.z = v[7 * i + 2];
        poses[i].orientation.x = v[7 * i + 3];
        poses[i].orientation.y = v[7 * i + 4];
        poses[i].orientation.z = v[7 * i + 5];
        poses[i].orientation.w = v[7 * i + 6];
    }
    return poses;
}

// Drop-ins for the other resamplers mcl_3d can select (mcl_3d.cpp:246-261).
// Wheel, Residual and Metropolis draw from the inherited generator in the
// reference's order (same generator state: same particles, generator left
// where the reference leaves it); Rejection seeds the device generator from it.
class GpuWheelResampler : public Resampler {
public:
    explicit GpuWheelResampler(int device = 0) : ctx_(new tsdfl::Context(device)) {}
    void resample(ParticleCloud& particle_cloud) override
    {
        tsdfl::resample_wheel(*ctx_, particle_cloud.particles(), m_generator_ptr.get());
    }

private:
    std::unique_ptr<tsdfl::Context> ctx_;
};

class GpuResidualResampler : public Resampler {
public:
    explicit GpuResidualResampler(int device = 0) : ctx_(new tsdfl::Context(device)) {}
    void resample(ParticleCloud& particle_cloud) override
    {
        tsdfl::resample_residual(*ctx_, particle_cloud.particles(), m_generator_ptr.get());
    }

private:
    std::unique_ptr<tsdfl::Context> ctx_;
};

class GpuMetropolisResampler : public Resampler {
public:
    explicit GpuMetropolisResampler(size_t sampling_steps, int device = 0)
        : ctx_(new tsdfl::Context(device)), steps_((uint32_t)sampling_steps)
    {
    }
    void resample(ParticleCloud& particle_cloud) override
    {
        tsdfl::resample_metropolis(*ctx_, particle_cloud.particles(), steps_, m_generator_ptr.get());
    }

private:
    std::unique_ptr<tsdfl::Context> ctx_;
    uint32_t steps_;
};

class GpuRejectionResampler : public Resampler {
public:
    explicit GpuRejectionResampler(int device = 0) : ctx_(new tsdfl::Context(device)) {}
    void resample(ParticleCloud& particle_cloud) override
    {
        const uint64_t seed = ((uint64_t)(*m_generator_ptr)() << 32) | (*m_generator_ptr)();
        tsdfl::resample_rejection(*ctx_, particle_cloud.particles(), seed);
    }

private:
    std::unique_ptr<tsdfl::Context> ctx_;
};

// Drop-in for ParticleCloud's motion-update overloads (particle_cloud.cpp:153-497):
// the same names and arguments, applied to a ParticleCloud's particles on the
// device.  It keeps what ParticleCloud keeps for them -- a_1 .. a_12, the time
// of the last update and the reference pose behind refDist / refAngle, with
// ParticleCloud's expressions, compiled in the caller's build -- so mcl_3d
// calls it where it called particle_cloud_.motionUpdate (mcl_3d.cpp:335-347)
// and reads refDist / refAngle / resetRef from it.  Noise is drawn on the
// device; with host_draws set it comes from an owned std::mt19937 seeded from
// std::random_device as ParticleCloud's is, in the reference's order.
class GpuMotionModel {
public:
    explicit GpuMotionModel(int device = 0, bool host_draws = false)
        : ctx_(new tsdfl::Context(device)), model_(*ctx_, std::random_device{}()), host_draws_(host_draws)
    {
        std::random_device rd{};
        gen_.seed(rd());
        ref_pose_.fill(0);
        m_last_time_ = ros::Time::now();
    }

    // ParticleCloud::initialize sets the time the first update measures from.
    void resetTime() { m_last_time_ = ros::Time::now(); }

    void setMotionParameters(FLOAT_T a_1, FLOAT_T a_2, FLOAT_T a_3, FLOAT_T a_4, FLOAT_T a_5, FLOAT_T a_6,
                             FLOAT_T a_7, FLOAT_T a_8, FLOAT_T a_9, FLOAT_T a_10, FLOAT_T a_11, FLOAT_T a_12)
    {
        model_.setMotionParameters(a_1, a_2, a_3, a_4, a_5, a_6, a_7, a_8, a_9, a_10, a_11, a_12);
    }

    void motionUpdate(ParticleCloud& cloud, const nav_msgs::Odometry& odom)
    {
        auto linear_velocity = odom.twist.twist.linear.x;
        auto angular_velocity = odom.twist.twist.angular.z;
        FLOAT_T time_diff = elapsed();
        ref_pose_[0] = ref_pose_[0] + linear_velocity * time_diff * cos(ref_pose_[5] + (angular_velocity / 2 * time_diff));
        ref_pose_[1] = ref_pose_[1] + linear_velocity * time_diff * sin(ref_pose_[5] + (angular_velocity / 2 * time_diff));
        ref_pose_[5] = ref_pose_[5] + angular_velocity * time_diff;
        const double in[2] = {linear_velocity, angular_velocity};
        run(cloud, model_.distributions(TSDFL_MOTION_ODOM, in, 2, time_diff));
    }

    void motionUpdate(ParticleCloud& cloud, const ImuAccumulator::Data& imu_data)
    {
        auto linear_velocity = imu_data.linear_vel;
        auto angular_velocity = imu_data.angular_yaw;
        FLOAT_T time_diff = elapsed();
        ref_pose_[0] = ref_pose_[0] + linear_velocity * time_diff * cos(ref_pose_[5] + (angular_velocity / 2 * time_diff));
        ref_pose_[1] = ref_pose_[1] + linear_velocity * time_diff * sin(ref_pose_[5] + (angular_velocity / 2 * time_diff));
        ref_pose_[5] = ref_pose_[5] + angular_velocity * time_diff;
        const double in[2] = {linear_velocity, angular_velocity};
        run(cloud, model_.distributions(TSDFL_MOTION_IMU, in, 2, time_diff));
    }

    void motionUpdate(ParticleCloud& cloud, FLOAT_T lin_scale, FLOAT_T ang_scale)
    {
        FLOAT_T time_diff = elapsed();
        const double in[2] = {lin_scale, ang_scale};
        run(cloud, model_.distributions(TSDFL_MOTION_SCALE, in, 2, time_diff));
    }

    void motionUpdate(ParticleCloud& cloud, FLOAT_T lin_scale, const ImuAccumulator::Data& imu_data)
    {
        FLOAT_T time_diff = elapsed();
        const double in[4] = {lin_scale, imu_data.delta_roll, imu_data.delta_pitch, imu_data.delta_yaw};
        run(cloud, model_.distributions(TSDFL_MOTION_SCALE_IMU, in, 4, time_diff));
    }

    void motion_update(ParticleCloud& cloud, FLOAT_T dx, FLOAT_T dy, FLOAT_T dz, FLOAT_T roll, FLOAT_T pitch,
                       FLOAT_T yaw, FLOAT_T lin_base_noise = 0, FLOAT_T ang_base_noise = 0)
    {
        elapsed();
        ref_pose_[0] = ref_pose_[0] + dx * cos(ref_pose_[5] + yaw);
        ref_pose_[1] = ref_pose_[1] + dx * sin(ref_pose_[5] + yaw);
        ref_pose_[5] = ref_pose_[5] + yaw;
        const double in[8] = {dx, dy, dz, roll, pitch, yaw, lin_base_noise, ang_base_noise};
        run(cloud, model_.distributions(TSDFL_MOTION_DELTA, in, 8, 0.0f));
    }

    const std::array<FLOAT_T, 6>& refPose() { return ref_pose_; }
    void resetRef() { ref_pose_.fill(0); }
    FLOAT_T refDist()
    {
        return std::sqrt(ref_pose_[0] * ref_pose_[0] + ref_pose_[1] * ref_pose_[1] + ref_pose_[2] * ref_pose_[2]);
    }
    FLOAT_T refAngle() { return std::fabs(ref_pose_[5]); }

private:
    FLOAT_T elapsed()
    {
        ros::Time current_time = ros::Time::now();
        FLOAT_T time_diff = (current_time - m_last_time_).toSec();
        m_last_time_ = current_time;
        return time_diff;
    }

    void run(ParticleCloud& cloud, const tsdfl_motion& m)
    {
        if (host_draws_) model_.update_with(cloud.particles(), m, gen_);
        else model_.update(cloud.particles(), m);
    }

    std::unique_ptr<tsdfl::Context> ctx_;
    tsdfl::MotionModel model_;
    bool host_draws_;
    std::mt19937 gen_;
    std::array<FLOAT_T, 6> ref_pose_;
    ros::Time m_last_time_;
};

// Drop-in for SystematicResampler: draws U ~ U[0, 1/M) from the inherited
// generator exactly as the reference does, then resamples on the device.
class GpuSystematicResampler : public Resampler {
public:
    explicit GpuSystematicResampler(int device = 0) : ctx_(new tsdfl::Context(device)) {}

    void resample(ParticleCloud& particle_cloud) override
    {
        auto inverse_M = 1.0 / particle_cloud.size();
        std::uniform_real_distribution<FLOAT_T> uniform_distribution(0.0, inverse_M);
        const float u0 = uniform_distribution(*m_generator_ptr);
        tsdfl::resample_systematic(*ctx_, particle_cloud.particles(), u0);
    }

private:
    std::unique_ptr<tsdfl::Context> ctx_;
};

// Drop-in for ResidualSystematicResampler (mcl_3d's default, mcl_3d.cpp:765):
// the same draw u ~ U[0, 1) from the inherited generator, then the device.
class GpuResidualSystematicResampler : public Resampler {
public:
    explicit GpuResidualSystematicResampler(int device = 0) : ctx_(new tsdfl::Context(device)) {}

    void resample(ParticleCloud& particle_cloud) override
    {
        std::uniform_real_distribution<FLOAT_T> uniform_distribution(0.0, 1.0);
        const float u = uniform_distribution(*m_generator_ptr);
        tsdfl::resample_residual_systematic(*ctx_, particle_cloud.particles(), u);
    }

private:
    std::unique_ptr<tsdfl::Context> ctx_;
};

}  // namespace tsdf_localization
#endif

#endif
