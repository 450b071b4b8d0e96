// Drives the C++ host layer (include/tsdfl_evaluator.hpp) on its own particle
// and point types: reads a map (MapCoef bytes, brick table, float slots),
// particles (P x 7), points (N x 3), tf[16] and a draw u0 from files in the
// directory given as argv[1]; writes the normalised weights, the mean pose and
// the resampled particles back there.
#include "tsdfl_evaluator.hpp"

using tsdfl::check;

#include <cstdio>
#include <fstream>
#include <iterator>
#include <random>
#include <string>
#include <vector>

struct MyParticle {
    float first[6];
    float second;
};
struct MyPoint {
    float x, y, z;
};

template <class T>
static std::vector<T> load(const std::string& path)
{
    std::ifstream f(path, std::ios::binary);
    std::vector<char> b((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    std::vector<T> v(b.size() / sizeof(T));
    std::memcpy(v.data(), b.data(), v.size() * sizeof(T));
    return v;
}

template <class T>
static void save(const std::string& path, const T* p, size_t n)
{
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(p), (std::streamsize)(n * sizeof(*p)));
}

int main(int argc, char** argv)
{
    if (argc < 2) return 2;
    const std::string d = argv[1];
    auto coef_b = load<char>(d + "/coef.bin");
    tsdfl_map_coef coef;
    if (coef_b.size() != sizeof(coef)) return 3;
    std::memcpy(&coef, coef_b.data(), sizeof(coef));
    auto grid_occ = load<int32_t>(d + "/grid_occ.bin");
    auto data = load<float>(d + "/data.bin");
    auto pf = load<float>(d + "/particles.bin");
    auto qf = load<float>(d + "/points.bin");
    auto tf = load<float>(d + "/tf.bin");
    auto u0 = load<float>(d + "/u0.bin");
    std::vector<MyParticle> parts(pf.size() / 7);
    for (size_t i = 0; i < parts.size(); ++i) {
        for (int k = 0; k < 6; ++k) parts[i].first[k] = pf[7 * i + k];
        parts[i].second = pf[7 * i + 6];
    }
    std::vector<MyPoint> pts(qf.size() / 3);
    for (size_t j = 0; j < pts.size(); ++j) pts[j] = MyPoint{qf[3 * j], qf[3 * j + 1], qf[3 * j + 2]};
    try {
        tsdfl::Context ctx(0);
        tsdfl::Map map(ctx, coef, grid_occ.data(), data.data(), 0.1f);
        tsdfl::SensorUpdate upd(ctx, map);
        tsdfl::Pose6 pose;
        upd.evaluate(parts, pts, tf.data(), &pose);
        std::vector<float> w(parts.size());
        for (size_t i = 0; i < parts.size(); ++i) w[i] = parts[i].second;
        save(d + "/weights_out.bin", w.data(), w.size());
        save(d + "/pose_out.bin", &pose.x, 6);
        std::vector<MyParticle> parts_r = parts;
        tsdfl::resample_residual_systematic(ctx, parts_r, u0.at(1));
        std::vector<float> out_r(7 * parts_r.size());
        for (size_t i = 0; i < parts_r.size(); ++i) {
            for (int k = 0; k < 6; ++k) out_r[7 * i + k] = parts_r[i].first[k];
            out_r[7 * i + 6] = parts_r[i].second;
        }
        save(d + "/residual_out.bin", out_r.data(), out_r.size());
        tsdfl::resample_systematic(ctx, parts, u0.at(0));
        std::vector<float> out(7 * parts.size());
        for (size_t i = 0; i < parts.size(); ++i) {
            for (int k = 0; k < 6; ++k) out[7 * i + k] = parts[i].first[k];
            out[7 * i + 6] = parts[i].second;
        }
        save(d + "/resampled_out.bin", out.data(), out.size());
        // scan reduction of a PointCloud2-style record array (x, y, z, ring)
        auto cloud = load<char>(d + "/cloud.bin");
        const size_t n_cloud = cloud.size() / 16;
        tsdfl::ScanReducer reducer(ctx, 0.064f);
        std::vector<MyPoint> red = reducer.reduce<MyPoint>(cloud.data(), n_cloud, 16, 0, 12);
        save(d + "/reduced_out.bin", &red.data()->x, 3 * red.size());
        std::vector<MyParticle> parts_c(pf.size() / 7);
        for (size_t i = 0; i < parts_c.size(); ++i) {
            for (int k = 0; k < 6; ++k) parts_c[i].first[k] = pf[7 * i + k];
            parts_c[i].second = pf[7 * i + 6];
        }
        tsdfl::Pose6 pose_c;
        size_t n_red = 0;
        upd.evaluate_cloud(parts_c, cloud.data(), n_cloud, 16, 0, 12, 0.064f, 0, tf.data(), &pose_c, &n_red);
        std::vector<float> wc(parts_c.size());
        for (size_t i = 0; i < parts_c.size(); ++i) wc[i] = parts_c[i].second;
        save(d + "/cloud_weights_out.bin", wc.data(), wc.size());
        // motion model on given draws and on device-drawn noise
        auto draws = load<double>(d + "/draws.bin");
        std::vector<MyParticle> parts_m(pf.size() / 7);
        for (size_t i = 0; i < parts_m.size(); ++i) {
            for (int k = 0; k < 6; ++k) parts_m[i].first[k] = pf[7 * i + k];
            parts_m[i].second = pf[7 * i + 6];
        }
        tsdfl::MotionModel motion(ctx, 42);
        std::vector<float> pm(pf);
        check(tsdfl_motion_apply(ctx.get(), pm.data(), parts_m.size(), draws.data()));
        save(d + "/motion_apply_out.bin", pm.data(), pm.size());
        const double odom_in[2] = {0.6, -0.3};
        tsdfl_motion m = motion.distributions(TSDFL_MOTION_ODOM, odom_in, 2, 0.1f);
        motion.update(parts_m, m);   // step 0 of seed 42
        std::vector<float> out_m(7 * parts_m.size());
        for (size_t i = 0; i < parts_m.size(); ++i) {
            for (int k = 0; k < 6; ++k) out_m[7 * i + k] = parts_m[i].first[k];
            out_m[7 * i + 6] = parts_m[i].second;
        }
        save(d + "/motion_update_out.bin", out_m.data(), out_m.size());
        // the other resamplers with the reference's seeded generator
        auto ow = load<float>(d + "/others_w.bin");
        auto oseed = load<uint32_t>(d + "/others_seed.bin");
        auto run_other = [&](int kind) {
            std::vector<MyParticle> ps(ow.size());
            for (size_t i = 0; i < ps.size(); ++i) {
                for (int k = 0; k < 6; ++k) ps[i].first[k] = 0.0f;
                ps[i].first[0] = (float)i;
                ps[i].second = ow[i];
            }
            std::mt19937 gen(oseed.at(0));
            if (kind == 0) tsdfl::resample_wheel(ctx, ps, &gen);
            if (kind == 1) tsdfl::resample_residual(ctx, ps, &gen);
            if (kind == 2) tsdfl::resample_metropolis(ctx, ps, 10, &gen);
            std::vector<uint32_t> idx(ps.size());
            for (size_t i = 0; i < ps.size(); ++i) idx[i] = (uint32_t)ps[i].first[0];
            // the generator is where the reference leaves it: report its next output
            idx.push_back(gen());
            return idx;
        };
        for (int kind = 0; kind < 3; ++kind) {
            auto idx = run_other(kind);
            save(d + "/others_out_" + std::to_string(kind) + ".bin", idx.data(), idx.size());
        }
        bool threw = false;
        try {   // an empty cloud: the reference's "No particle is valid!"
            std::vector<MyParticle> none;
            upd.evaluate(none, pts, tf.data(), &pose);
        } catch (const std::runtime_error& e) {
            threw = std::string(e.what()).find("No particle is valid!") != std::string::npos;
        }
        std::printf("cxx core ok P=%zu N=%zu resampled=%zu reduced=%zu/%zu empty_cloud_throws=%d\n", w.size(),
                    pts.size(), parts.size(), red.size(), n_red, threw ? 1 : 0);
        return threw ? 0 : 4;
    } catch (const std::runtime_error& e) {
        std::printf("runtime_error: %s\n", e.what());
        return 1;
    }
}
