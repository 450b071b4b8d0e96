"""The motion model's host arithmetic (tsdfl_motion_model, no GPU needed): the
(mean, stddev) of the six draws each ParticleCloud overload sets up
(particle_cloud.cpp:153-497), in double for the odometry message and in float
for the others, restated here in numpy with the same rounding."""
import ctypes as C

import numpy as np
import pytest

from tsdf_localization_gb300 import _native as N

F = np.float32


def model(kind, a, inputs, dt):
    x = np.ascontiguousarray(inputs, np.float64)
    m = N.Motion()
    rc = N.lib().tsdfl_motion_model(kind, np.ascontiguousarray(a, np.float32).ctypes.data, x.ctypes.data,
                                    x.shape[0], F(dt), C.byref(m))
    assert rc == N.TSDFL_OK
    return np.array(m.mean), np.array(m.stddev)


@pytest.fixture
def a():
    return (np.arange(1, 13) * 0.013 + 0.001).astype(np.float32)


def test_odom_in_double(a):
    lin, ang, dt = 0.731, -0.2917, F(0.1003)
    mean, sd = model(N.TSDFL_MOTION_ODOM, a, [lin, ang], dt)
    d = lin * float(dt)
    th = ang * float(dt)
    assert mean.tolist() == [d, 0, 0, 0, 0, th]
    want = [float(a[2 * k]) * (d * d) + float(a[2 * k + 1]) * (th * th) for k in range(6)]
    assert sd.tolist() == want


@pytest.mark.parametrize("kind", [N.TSDFL_MOTION_IMU, N.TSDFL_MOTION_SCALE])
def test_float_overloads(a, kind):
    v0, v1, dt = F(0.731), F(-0.2917), F(0.1003)
    mean, sd = model(kind, a, [float(v0), float(v1)], dt)
    d = F(v0 * dt)
    th = F(v1 * dt)
    want = [float(F(F(a[2 * k] * F(d * d)) + F(a[2 * k + 1] * F(th * th)))) for k in range(6)]
    assert sd.tolist() == want
    if kind == N.TSDFL_MOTION_IMU:
        assert mean.tolist() == [float(d), 0, 0, 0, 0, float(th)]
    else:
        assert mean.tolist() == [0.0] * 6


def test_scale_imu(a):
    ls, r, p, y, dt = F(1.3), F(0.02), F(-0.013), F(0.21), F(0.05)
    mean, sd = model(N.TSDFL_MOTION_SCALE_IMU, a, [float(ls), float(r), float(p), float(y)], dt)
    d = F(ls * dt)
    xyz = [float(F(F(a[2 * k] * F(d * d)) + F(a[2 * k + 1] * F(y * y)))) for k in range(3)]
    assert sd.tolist() == xyz + [float(F(a[7] * F(r * r))), float(F(a[9] * F(p * p))), float(F(a[11] * F(y * y)))]
    assert mean.tolist() == [0, 0, 0, float(r), float(p), float(y)]


def test_delta(a):
    v = np.array([0.3, -0.05, 0.01, 0.02, -0.01, 0.15, 0.001, 0.002], np.float32)
    mean, sd = model(N.TSDFL_MOTION_DELTA, a, v.astype(np.float64), 0.0)
    dx2, dy2, dz2, r2, p2, y2 = (F(x * x) for x in v[:6])
    lin, ang = v[6], v[7]
    t = lambda a1, s1, a2, s2, b: float(F(F(F(a1 * s1) + F(a2 * s2)) + b))  # noqa: E731
    want = [t(a[0], dx2, a[1], y2, lin), t(a[2], dy2, a[3], y2, lin), t(a[4], dz2, a[5], y2, lin),
            t(a[6], dx2, a[7], r2, ang), t(a[8], dx2, a[9], p2, ang), t(a[10], dx2, a[11], y2, ang)]
    assert sd.tolist() == want
    assert mean.tolist() == [float(x) for x in v[:6]]


def test_bad_arguments(a):
    m = N.Motion()
    x = np.zeros(3)
    assert N.lib().tsdfl_motion_model(N.TSDFL_MOTION_ODOM, a.ctypes.data, x.ctypes.data, 3, F(0.1),
                                      C.byref(m)) == N.TSDFL_ERR_INVALID_ARG
    assert N.lib().tsdfl_motion_model(9, a.ctypes.data, x.ctypes.data, 2, F(0.1),
                                      C.byref(m)) == N.TSDFL_ERR_INVALID_ARG
