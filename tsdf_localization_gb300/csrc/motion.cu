// Motion update on the device: ParticleCloud::apply_model
// (particle_cloud.cpp:499-617; the same loop body as motionUpdate(odom),
// :153-333).  Every particle draws six increments dx, dy, dz, roll, pitch,
// yaw, builds the odometry transform from them, rotates it by the particle's
// orientation and takes the translation and getAngleFromMat's angles
// (util.cpp:86-111) as its new pose; the weight is kept.
//
// Draws: the reference pulls them from one serial mt19937 through
// std::normal_distribution, a sequence no parallel generator reproduces.  Here
// each particle's six normals come from a counter-based generator instead:
// Philox4x64-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC 2011) keyed by the seed, with the counter (particle index,
// block 0/1, step, 0), and Box-Muller pairs in FP64.  Callers that need the
// reference's own sequence draw it on the host and pass it in
// (tsdfl_motion_apply*): the pose composition is the reference's bit for bit.
//
// Arithmetic as the reference's x86-64 build does it: trig of the double draws
// in double rounded to float, trig of the float orientation through the
// double overloads, float products and sums with no contraction, float
// pitch re-used in double cos for roll and yaw.
#include <stdint.h>

#include <atomic>

#include "philox.h"
#include "tsdfl_internal.h"

namespace tsdfl {

extern std::atomic<unsigned long long> g_launches;

namespace {

constexpr int kMotionBlock = 256;

struct MotionParams {
    float* particles;        // P x 7, updated in place
    uint32_t P;
    double mean[6], stddev[6];
    unsigned long long key0, key1, step;
    const double* draws;     // P x 6 given draws, or null: generate
    double* draws_out;       // optional: the generated draws
};

// A standard normal pair from two 64-bit words: u1 in (0, 1], u2 in [0, 1),
// r = sqrt(-2 ln u1), (r cos 2 pi u2, r sin 2 pi u2).
__device__ __forceinline__ void box_muller(unsigned long long a, unsigned long long b, double& z0, double& z1)
{
    const double u1 = ((double)(a >> 11) + 1.0) * 0x1.0p-53;
    const double u2 = (double)(b >> 11) * 0x1.0p-53;
    const double r = sqrt(-2.0 * log(u1));
    double s, c;
    sincospi(2.0 * u2, &s, &c);
    z0 = r * c;
    z1 = r * s;
}

__device__ __forceinline__ float fsin_d(double v) { return (float)sin(v); }
__device__ __forceinline__ float fcos_d(double v) { return (float)cos(v); }

// util.cpp:86-111 with the double overloads of fabs, atan2, asin and cos.
__device__ __forceinline__ void angles_from_mat(const float* m, float& roll, float& pitch, float& yaw)
{
    if (fabs((double)m[8]) >= 1.0) {
        yaw = 0.0f;
        const double delta = atan2((double)m[9], (double)m[10]);
        pitch = m[8] < 0.0f ? (float)(3.14159265358979323846 / 2.0) : (float)(-3.14159265358979323846 / 2.0);
        roll = (float)delta;
    } else {
        pitch = (float)(-asin((double)m[8]));
        const double cp = cos((double)pitch);
        roll = (float)atan2(__ddiv_rn((double)m[9], cp), __ddiv_rn((double)m[10], cp));
        yaw = (float)atan2(__ddiv_rn((double)m[4], cp), __ddiv_rn((double)m[0], cp));
    }
}

__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }

// particle_cloud.cpp:530-614 for one particle and its draws d[6].
__device__ __forceinline__ void compose(float* p, const double d[6])
{
    const float sr = fsin_d(d[3]), cr = fcos_d(d[3]);
    const float sp = fsin_d(d[4]), cp = fcos_d(d[4]);
    const float sy = fsin_d(d[5]), cy = fcos_d(d[5]);
    float o[12];
    o[0] = mul(cp, cy);
    o[4] = mul(cp, sy);
    o[8] = -sp;
    o[3] = (float)d[0];
    o[1] = sub(mul(mul(sr, sp), cy), mul(cr, sy));
    o[5] = add(mul(mul(sr, sp), sy), mul(cr, cy));
    o[9] = mul(sr, cp);
    o[7] = (float)d[1];
    o[2] = add(mul(mul(cr, sp), cy), mul(sr, sy));
    o[6] = sub(mul(mul(cr, sp), sy), mul(sr, cy));
    o[10] = mul(cr, cp);
    o[11] = (float)d[2];

    const float sa = fsin_d((double)p[3]), ca = fcos_d((double)p[3]);
    const float sb = fsin_d((double)p[4]), cb = fcos_d((double)p[4]);
    const float sg = fsin_d((double)p[5]), cg = fcos_d((double)p[5]);
    float q[12];
    q[0] = mul(cb, cg);
    q[4] = mul(cb, sg);
    q[8] = -sb;
    q[3] = 0.0f;
    q[1] = sub(mul(mul(sa, sb), cg), mul(ca, sg));
    q[5] = add(mul(mul(sa, sb), sg), mul(ca, cg));
    q[9] = mul(sa, cb);
    q[7] = 0.0f;
    q[2] = add(mul(mul(ca, sb), cg), mul(sa, sg));
    q[6] = sub(mul(mul(ca, sb), sg), mul(sa, cg));
    q[10] = mul(ca, cb);
    q[11] = 0.0f;

    float t[12];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const float a0 = q[4 * r], a1 = q[4 * r + 1], a2 = q[4 * r + 2];
        t[4 * r] = add(add(mul(a0, o[0]), mul(a1, o[4])), mul(a2, o[8]));
        t[4 * r + 1] = add(add(mul(a0, o[1]), mul(a1, o[5])), mul(a2, o[9]));
        t[4 * r + 2] = add(add(mul(a0, o[2]), mul(a1, o[6])), mul(a2, o[10]));
        t[4 * r + 3] = add(add(add(mul(a0, o[3]), mul(a1, o[7])), mul(a2, o[11])), q[4 * r + 3]);
    }
    float m[16];
#pragma unroll
    for (int k = 0; k < 12; ++k) m[k] = t[k];
    float roll, pitch, yaw;
    angles_from_mat(m, roll, pitch, yaw);
    p[0] = add(p[0], t[3]);
    p[1] = add(p[1], t[7]);
    p[2] = add(p[2], t[11]);
    p[3] = roll;
    p[4] = pitch;
    p[5] = yaw;
}

__global__ void __launch_bounds__(kMotionBlock) motion_kernel(MotionParams mp)
{
    const uint32_t i = blockIdx.x * kMotionBlock + threadIdx.x;
    if (i >= mp.P) return;
    double d[6];
    if (mp.draws) {
#pragma unroll
        for (int k = 0; k < 6; ++k) d[k] = mp.draws[6 * (size_t)i + k];
    } else {
        unsigned long long c0[4] = {i, 0, mp.step, 0};
        unsigned long long c1[4] = {i, 1, mp.step, 0};
        philox4x64_10(c0, mp.key0, mp.key1);
        philox4x64_10(c1, mp.key0, mp.key1);
        double z[6];
        box_muller(c0[0], c0[1], z[0], z[1]);
        box_muller(c0[2], c0[3], z[2], z[3]);
        box_muller(c1[0], c1[1], z[4], z[5]);
#pragma unroll
        for (int k = 0; k < 6; ++k) d[k] = __dadd_rn(__dmul_rn(z[k], mp.stddev[k]), mp.mean[k]);
        if (mp.draws_out) {
#pragma unroll
            for (int k = 0; k < 6; ++k) mp.draws_out[6 * (size_t)i + k] = d[k];
        }
    }
    float p[7];
    float* src = mp.particles + 7 * (size_t)i;
#pragma unroll
    for (int k = 0; k < 7; ++k) p[k] = src[k];
    compose(p, d);
#pragma unroll
    for (int k = 0; k < 6; ++k) src[k] = p[k];
}

// mcl_3d.cpp:433-449: a particle as geometry_msgs::Pose (position, then the
// orientation quaternion x, y, z, w of tf2::Quaternion::setRPY(roll, pitch,
// yaw): half angles, ZYX composition, in double).
__global__ void pose_array_kernel(const float* __restrict__ particles, uint32_t P, double* __restrict__ poses)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const float* p = particles + 7 * (size_t)i;
    double sr, cr, sp, cp, sy, cy;
    sincos(__dmul_rn((double)p[3], 0.5), &sr, &cr);
    sincos(__dmul_rn((double)p[4], 0.5), &sp, &cp);
    sincos(__dmul_rn((double)p[5], 0.5), &sy, &cy);
    double* o = poses + 7 * (size_t)i;
    o[0] = p[0];
    o[1] = p[1];
    o[2] = p[2];
    o[3] = __dsub_rn(__dmul_rn(__dmul_rn(sr, cp), cy), __dmul_rn(__dmul_rn(cr, sp), sy));
    o[4] = __dadd_rn(__dmul_rn(__dmul_rn(cr, sp), cy), __dmul_rn(__dmul_rn(sr, cp), sy));
    o[5] = __dsub_rn(__dmul_rn(__dmul_rn(cr, cp), sy), __dmul_rn(__dmul_rn(sr, sp), cy));
    o[6] = __dadd_rn(__dmul_rn(__dmul_rn(cr, cp), cy), __dmul_rn(__dmul_rn(sr, sp), sy));
}

int check(cudaError_t e) { return e == cudaSuccess ? TSDFL_OK : TSDFL_ERR_DEVICE; }

}  // namespace

int launch_pose_array(const float* particles, size_t P, double* poses, cudaStream_t s)
{
    if (P == 0) return TSDFL_OK;
    pose_array_kernel<<<(unsigned)((P + 255) / 256), 256, 0, s>>>(particles, (uint32_t)P, poses);
    g_launches += 1;
    return check(cudaGetLastError());
}

int launch_motion(float* particles, size_t P, const double mean[6], const double stddev[6], uint64_t seed,
                  uint64_t step, const double* draws, double* draws_out, cudaStream_t s)
{
    if (P == 0) return TSDFL_OK;
    MotionParams mp{};
    mp.particles = particles;
    mp.P = (uint32_t)P;
    for (int k = 0; k < 6; ++k) {
        mp.mean[k] = mean ? mean[k] : 0.0;
        mp.stddev[k] = stddev ? stddev[k] : 0.0;
    }
    mp.key0 = seed;
    mp.key1 = kStreamMotion;
    mp.step = step;
    mp.draws = draws;
    mp.draws_out = draws_out;
    motion_kernel<<<(unsigned)((P + kMotionBlock - 1) / kMotionBlock), kMotionBlock, 0, s>>>(mp);
    g_launches += 1;
    return check(cudaGetLastError());
}

}  // namespace tsdfl
