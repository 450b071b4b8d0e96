"""Motion update on the GPU (tsdfl_motion_*) against the oracle and the
reference's recorded outputs: the pose composition bit for bit on given draws;
the device-drawn noise reproducible per (seed, step), equal to the oracle's
Philox4x64-10 + Box-Muller draws, with the requested mean and spread."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle_py as O
from tsdf_localization_gb300 import Context, MotionModel
from tsdf_localization_gb300 import _native as N

pytestmark = pytest.mark.gpu
GOLD = np.load(Path(__file__).resolve().parent / "golden" / "reference_cases.npz")
KEY1 = 0x6D6F74696F6E0001


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


def random_particles(P, seed):
    rng = np.random.default_rng(seed)
    p = np.zeros((P, 7), np.float32)
    p[:, :3] = rng.uniform(-80, 80, (P, 3))
    p[:, 3:6] = rng.uniform(-np.pi, np.pi, (P, 3))
    p[: P // 50, 4] = np.float32(np.pi / 2)
    p[P // 50: P // 25, 4] = -np.float32(np.pi / 2)
    p[:, 6] = rng.random(P)
    return p


def test_gpu_motion_matches_reference(ctx):
    parts = GOLD["motion/particles"]
    for d, want in zip(GOLD["motion/deltas"], GOLD["motion/moved"]):
        got = MotionModel(ctx).apply(parts.copy(), np.tile(d.astype(np.float64), (parts.shape[0], 1)))
        assert np.array_equal(got, want)


def test_gpu_motion_random_draws_match_oracle(ctx):
    P = 200_000
    parts = random_particles(P, 3)
    rng = np.random.default_rng(4)
    draws = rng.normal(0, [0.4, 0.1, 0.05, 0.08, 0.08, 0.6], (P, 6))
    draws[:100] = 0.0
    got = MotionModel(ctx).apply(parts.copy(), draws)
    assert np.array_equal(got, O.motion_apply(parts, draws))


def expected_draws(P, seed, step, mean, sd):
    i = np.arange(P, dtype=np.uint64)
    z = np.zeros(P, np.uint64)
    s = np.full(P, step, np.uint64)
    w0 = O.philox4x64_10([i, z, s, z], (seed, KEY1))
    w1 = O.philox4x64_10([i, np.ones(P, np.uint64), s, z], (seed, KEY1))

    def bm(a, b):
        u1 = ((a >> np.uint64(11)).astype(np.float64) + 1.0) * 2.0 ** -53
        u2 = (b >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
        r = np.sqrt(-2.0 * np.log(u1))
        return r * np.cos(2 * np.pi * u2), r * np.sin(2 * np.pi * u2)

    z0, z1 = bm(w0[0], w0[1])
    z2, z3 = bm(w0[2], w0[3])
    z4, z5 = bm(w1[0], w1[1])
    return np.stack([z0, z1, z2, z3, z4, z5], 1) * np.asarray(sd) + np.asarray(mean)


def test_gpu_motion_generated_draws(ctx):
    torch = pytest.importorskip("torch")
    P = 100_000
    parts = random_particles(P, 5)
    mm = MotionModel(ctx, seed=99)
    m = mm.distributions("odom", [0.8, -0.4], 0.1)
    d_part = torch.from_numpy(parts.copy()).cuda()
    d_draws = torch.zeros((P, 6), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    N.check(N.lib().tsdfl_motion_update_device(ctx.handle, C.c_void_p(d_part.data_ptr()), P, C.byref(m), 99, 7,
                                               C.c_void_p(d_draws.data_ptr())))
    ctx.sync()
    draws = d_draws.cpu().numpy()
    want = expected_draws(P, 99, 7, list(m.mean), list(m.stddev))
    assert np.allclose(draws, want, rtol=1e-12, atol=1e-15)
    # the composition on those draws is the oracle's
    assert np.array_equal(d_part.cpu().numpy(), O.motion_apply(parts, draws))
    # the host form with the same seed and step gives the same particles
    p2 = parts.copy()
    mm.update(p2, m, step=7)
    assert np.array_equal(p2, d_part.cpu().numpy())
    # another step gives other draws
    p3 = parts.copy()
    mm.update(p3, m, step=8)
    assert not np.array_equal(p3, p2)


def test_gpu_motion_noise_statistics(ctx):
    torch = pytest.importorskip("torch")
    P = 1 << 20
    mean = [0.3, -0.1, 0.02, 0.01, -0.02, 0.2]
    sd = [0.05, 0.02, 0.01, 0.004, 0.003, 0.03]
    m = N.Motion((C.c_double * 6)(*mean), (C.c_double * 6)(*sd))
    d_part = torch.zeros((P, 7), dtype=torch.float32, device="cuda")
    d_draws = torch.zeros((P, 6), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    N.check(N.lib().tsdfl_motion_update_device(ctx.handle, C.c_void_p(d_part.data_ptr()), P, C.byref(m), 1, 0,
                                               C.c_void_p(d_draws.data_ptr())))
    ctx.sync()
    d = d_draws.cpu().numpy()
    z = (d - np.asarray(mean)) / np.asarray(sd)
    assert np.all(np.abs(z.mean(0)) < 5 / np.sqrt(P))
    assert np.all(np.abs(z.std(0) - 1) < 5 / np.sqrt(2 * P))
    c = np.corrcoef(z.T)
    assert np.all(np.abs(c - np.eye(6)) < 5 / np.sqrt(P))
    assert abs(np.corrcoef(z[:-1, 0], z[1:, 0])[0, 1]) < 5 / np.sqrt(P)
    # particles at the origin with zero orientation move by the draws
    moved = d_part.cpu().numpy()
    assert np.array_equal(moved[:, 0], d[:, 0].astype(np.float32))


def test_gpu_motion_empty_and_errors(ctx):
    mm = MotionModel(ctx)
    empty = np.zeros((0, 7), np.float32)
    mm.apply(empty, np.zeros((0, 6)))
    m = mm.distributions("scale", [1.0, 1.0], 0.1)
    mm.update(empty, m)
    assert N.lib().tsdfl_motion_apply_device(ctx.handle, None, 5, None) == N.TSDFL_ERR_INVALID_ARG


def test_gpu_pose_array_matches_oracle(ctx):
    from tsdf_localization_gb300 import pose_array
    parts = random_particles(50_000, 12)
    got = pose_array(ctx, parts)
    want = O.pose_array(parts)
    assert np.array_equal(got[:, :3], want[:, :3])
    # double sin/cos of the device and of the host may differ in the last bit
    assert np.allclose(got[:, 3:], want[:, 3:], rtol=0, atol=1e-15)
    assert np.allclose(np.linalg.norm(got[:, 3:], axis=1), 1.0, atol=1e-12)
    assert pose_array(ctx, np.zeros((0, 7), np.float32)).shape == (0, 7)
