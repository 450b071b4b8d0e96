// Builds the drop-in plug-ins of include/tsdfl_evaluator.hpp against the
// reference's own headers (tsdf_localization's Evaluator, Resampler, Particle,
// CudaSubVoxelMap, compiled with the test shims for ROS) and links them with
// libtsdfl.  Run without a GPU, constructing them must raise std::runtime_error
// with libtsdfl's message; with a GPU, one update and one resample run.
#include <tsdf_localization/cuda/cuda_evaluator.h>
#include <tsdf_localization/resampling/novel_resampling.h>
#include <tsdf_localization/resampling/wheel_resampler.h>

#define TSDFL_WITH_TSDF_LOCALIZATION
#include "tsdfl_evaluator.hpp"

#include <cstdio>
#include <cstring>
#include <tuple>
#include <vector>

namespace tsdf_localization {
// The two ParticleCloud members the resampler touches (particle_cloud.cpp is
// not part of this build).
ParticleCloud::ParticleCloud() {}
Particle& ParticleCloud::operator[](unsigned int index) { return m_particles.at(index); }
std::size_t ParticleCloud::size() const { return m_particles.size(); }
}  // namespace tsdf_localization

int main()
{
    using namespace tsdf_localization;
    CudaSubVoxelMap<FLOAT_T, FLOAT_T> map(0.0f, 0.0f, 0.0f, 4.0f, 4.0f, 2.0f, 0.064f, 0.0f);
    std::vector<std::tuple<FLOAT_T, FLOAT_T, FLOAT_T, FLOAT_T>> slots{{1.0f, 1.0f, 1.0f, 2.0f}};
    map.setData(slots);
    int status = 0;
    try {
        GpuTsdfEvaluator ev(map, false, 0.9f, 0.1f, 0.0f, 100.0f, 0, 0.1f);
        std::vector<Particle> parts(3);
        for (int i = 0; i < 3; ++i) {
            for (int k = 0; k < 6; ++k) parts[i].first[k] = 0.0f;
            parts[i].second = 1.0f / 3.0f;
        }
        std::vector<CudaPoint> pts{CudaPoint(1.0f, 1.0f, 1.0f), CudaPoint(2.0f, 1.0f, 1.0f)};
        FLOAT_T tf[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
        geometry_msgs::PoseWithCovariance pose = ev.evaluate(parts, pts, tf);
        std::printf("evaluated w0=%.9g x=%.9g\n", parts[0].second, pose.pose.position.x);
        GpuSystematicResampler rs(0);
        ParticleCloud cloud;
        cloud.particles() = parts;
        rs.resample(cloud);
        std::printf("resampled %zu\n", cloud.size());
        GpuResidualSystematicResampler rr(0);
        rr.resample(cloud);
        std::printf("residual resampled %zu\n", cloud.size());
        // a PointCloud2 with the fields evaluateParticles reads
        sensor_msgs::PointCloud2 pc;
        pc.height = 1;
        pc.width = 3;
        pc.point_step = 16;
        const char* names[4] = {"x", "y", "z", "ring"};
        for (int f = 0; f < 4; ++f) {
            sensor_msgs::PointField field;
            field.name = names[f];
            field.offset = 4 * f;
            pc.fields.push_back(field);
        }
        const float xyz[3][3] = {{1.5f, 1.0f, 1.0f}, {1.5f, 1.0f, 1.0f}, {0.2f, 0.1f, 0.0f}};
        pc.data.resize(48);
        for (int i = 0; i < 3; ++i) {
            std::memcpy(&pc.data[16 * i], xyz[i], 12);
            const int16_t ring = 1;
            std::memcpy(&pc.data[16 * i + 12], &ring, 2);
        }
        tsdfl::Context sctx(0);
        tsdfl::ScanReducer reducer(sctx, 0.064f);
        std::vector<CudaPoint> reduced = gpu_reduce_scan(reducer, pc);
        std::printf("reduced %zu\n", reduced.size());
        pose = ev.evaluateCloud(parts, pc, tf, 0.064f);
        std::printf("cloud evaluated w0=%.9g\n", parts[0].second);
        GpuMotionModel motion(0);
        motion.setMotionParameters(0.1f, 0.1f, 0.1f, 0.1f, 0.1f, 0.1f, 0.1f, 0.1f, 0.1f, 0.1f, 0.1f, 0.1f);
        nav_msgs::Odometry odom;
        odom.twist.twist.linear.x = 0.5;
        odom.twist.twist.angular.z = 0.1;
        motion.motionUpdate(cloud, odom);
        motion.motion_update(cloud, 0.1f, 0.0f, 0.0f, 0.0f, 0.0f, 0.05f);
        std::printf("moved %zu, ref dist %.9g\n", cloud.size(), motion.refDist());
        GpuWheelResampler wheel(0);
        wheel.resample(cloud);
        GpuResidualResampler residual(0);
        residual.resample(cloud);
        GpuMetropolisResampler metropolis(50, 0);
        metropolis.resample(cloud);
        GpuRejectionResampler rejection(0);
        rejection.resample(cloud);
        std::printf("other resamplers %zu\n", cloud.size());
        std::vector<geometry_msgs::Pose> poses = gpu_particle_poses(sctx, cloud.particles());
        std::printf("poses %zu\n", poses.size());
    } catch (const std::runtime_error& e) {
        std::printf("runtime_error: %s\n", e.what());
        status = 0;
    }
    std::printf("dropin compiled\n");
    return status;
}
