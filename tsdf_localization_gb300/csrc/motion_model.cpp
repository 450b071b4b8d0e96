// Host side of the motion update: the normal distributions each of
// ParticleCloud's motion-update overloads sets up (particle_cloud.cpp:153-497),
// with the overload's own arithmetic (double for the odometry message, float
// for the others), as (mean, standard deviation) per draw.
#include <cstddef>

#include "tsdfl.h"

extern "C" int tsdfl_motion_model(int kind, const float a[12], const double* in, size_t n_in, float time_diff,
                                  tsdfl_motion* out)
{
    if (!a || !out || (n_in && !in)) return TSDFL_ERR_INVALID_ARG;
    for (int k = 0; k < 6; ++k) out->mean[k] = out->stddev[k] = 0.0;
    switch (kind) {
    case TSDFL_MOTION_ODOM: {   // :153-197, twist fields are double
        if (n_in != 2) return TSDFL_ERR_INVALID_ARG;
        const double d = in[0] * (double)time_diff, d2 = d * d;
        const double th = in[1] * (double)time_diff, th2 = th * th;
        const double m[6] = {d, 0, 0, 0, 0, th};
        for (int k = 0; k < 6; ++k) {
            out->mean[k] = m[k];
            out->stddev[k] = (double)a[2 * k] * d2 + (double)a[2 * k + 1] * th2;
        }
        return TSDFL_OK;
    }
    case TSDFL_MOTION_IMU: {    // :335-378, ImuAccumulator::Data fields are float
        if (n_in != 2) return TSDFL_ERR_INVALID_ARG;
        const float d = (float)in[0] * time_diff, d2 = d * d;
        const float th = (float)in[1] * time_diff, th2 = th * th;
        const float m[6] = {d, 0, 0, 0, 0, th};
        for (int k = 0; k < 6; ++k) {
            out->mean[k] = m[k];
            out->stddev[k] = a[2 * k] * d2 + a[2 * k + 1] * th2;
        }
        return TSDFL_OK;
    }
    case TSDFL_MOTION_SCALE: {  // :380-413, zero means
        if (n_in != 2) return TSDFL_ERR_INVALID_ARG;
        const float d = (float)in[0] * time_diff, d2 = d * d;
        const float th = (float)in[1] * time_diff, th2 = th * th;
        for (int k = 0; k < 6; ++k) out->stddev[k] = a[2 * k] * d2 + a[2 * k + 1] * th2;
        return TSDFL_OK;
    }
    case TSDFL_MOTION_SCALE_IMU: {   // :415-454: in = lin_scale, delta_roll, delta_pitch, delta_yaw
        if (n_in != 4) return TSDFL_ERR_INVALID_ARG;
        const float d = (float)in[0] * time_diff, d2 = d * d;
        const float r = (float)in[1], r2 = r * r;
        const float p = (float)in[2], p2 = p * p;
        const float th = (float)in[3], th2 = th * th;
        for (int k = 0; k < 3; ++k) out->stddev[k] = a[2 * k] * d2 + a[2 * k + 1] * th2;
        out->mean[3] = r;
        out->stddev[3] = a[7] * r2;
        out->mean[4] = p;
        out->stddev[4] = a[9] * p2;
        out->mean[5] = th;
        out->stddev[5] = a[11] * th2;
        return TSDFL_OK;
    }
    case TSDFL_MOTION_DELTA: {  // :456-497: in = dx, dy, dz, roll, pitch, yaw, lin_base_noise, ang_base_noise
        if (n_in != 8) return TSDFL_ERR_INVALID_ARG;
        float v[8];
        for (int k = 0; k < 8; ++k) v[k] = (float)in[k];
        const float dx2 = v[0] * v[0], dy2 = v[1] * v[1], dz2 = v[2] * v[2];
        const float r2 = v[3] * v[3], p2 = v[4] * v[4], y2 = v[5] * v[5];
        const float lin = v[6], ang = v[7];
        const float sd[6] = {a[0] * dx2 + a[1] * y2 + lin, a[2] * dy2 + a[3] * y2 + lin, a[4] * dz2 + a[5] * y2 + lin,
                             a[6] * dx2 + a[7] * r2 + ang, a[8] * dx2 + a[9] * p2 + ang, a[10] * dx2 + a[11] * y2 + ang};
        for (int k = 0; k < 6; ++k) {
            out->mean[k] = v[k];
            out->stddev[k] = sd[k];
        }
        return TSDFL_OK;
    }
    default:
        return TSDFL_ERR_INVALID_ARG;
    }
}
