"""The reference's Wheel, Residual, Metropolis and Rejection resamplers on the
GPU: with the reference's own draws (recorded in tests/golden) the outputs are
the reference's bit for bit; with device draws they equal the oracle run on
the same Philox4x64-10 draws; the device forms gather the same particles."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle_py as O
from tsdf_localization_gb300 import (Context, MetropolisResampler, RejectionResampler, ResidualResampler,
                                     TsdflError, WheelResampler)
from tsdf_localization_gb300 import _native as N

pytestmark = pytest.mark.gpu
GOLD = np.load(Path(__file__).resolve().parent / "golden" / "reference_cases.npz")
OTHERS = sorted({k.split("/")[1] for k in GOLD.files if k.startswith("others/") and k.count("/") == 2})


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


def weights(kind, M, seed):
    rng = np.random.default_rng(seed)
    if kind == "uniform":
        return np.full(M, 1.0 / M, np.float32)
    if kind == "random":
        w = rng.random(M) ** 3
    elif kind == "sparse":
        w = np.where(rng.random(M) < 0.02, rng.random(M) + 0.01, 0.0)
        w[0] = 0.5
    else:   # unnormalised, summing to about 0.7
        return rng.uniform(0, 1.4 / M, M).astype(np.float32)
    return (w / w.sum()).astype(np.float32)


def philox_words(seed, stream, c0, c1):
    z = np.zeros(np.asarray(c0).shape, np.uint64)
    return O.philox4x64_10([np.asarray(c0, np.uint64), np.asarray(c1, np.uint64), z, z], (seed, O.STREAMS[stream]))


def index_of(word, M):
    return ((word.astype(object) * M) >> 64).astype(np.uint32)


def u01_float(word):
    return ((word >> np.uint64(40)).astype(np.float64) * 2.0 ** -24).astype(np.float32)


@pytest.mark.parametrize("wset", OTHERS)
def test_gpu_other_resamplers_match_reference(ctx, wset):
    g = lambda name: GOLD[f"others/{wset}/{name}"]  # noqa: E731
    w = g("weights")
    assert np.array_equal(WheelResampler(ctx).resample_indices(w, g("wheel_draws")), g("wheel"))
    assert np.array_equal(ResidualResampler(ctx).resample_indices(w, g("residual_draws")), g("residual"))
    steps = int(GOLD["others/steps"])
    assert np.array_equal(MetropolisResampler(ctx, steps).resample_indices(w, g("metropolis_u"), g("metropolis_j")),
                          g("metropolis"))


@pytest.mark.parametrize("kind", ["uniform", "random", "sparse", "unnormalised"])
def test_gpu_wheel_device_draws_match_oracle(ctx, kind):
    M, seed = 20_000, 17
    w = weights(kind, M, 1)
    draws = philox_words(seed, "wheel", np.arange(M), np.zeros(M))[0]
    u = (draws >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
    got = WheelResampler(ctx, seed).resample_indices(w)
    assert np.array_equal(got, O.resample_wheel(w, u))


@pytest.mark.parametrize("kind", ["uniform", "random", "sparse", "unnormalised"])
def test_gpu_residual_device_draws_match_oracle(ctx, kind):
    M, seed = 50_000, 5
    w = weights(kind, M, 2)
    K = 4 * M + 4096
    q = np.arange((K + 3) // 4)
    words = philox_words(seed, "residual", q, np.zeros_like(q))
    r = np.stack([index_of(x, M) for x in words], 1).reshape(-1)[:K]
    want, _ = O.resample_residual(w, r)
    assert np.array_equal(ResidualResampler(ctx, seed).resample_indices(w), want)


@pytest.mark.parametrize("kind", ["uniform", "random", "sparse"])
def test_gpu_metropolis_device_draws_match_oracle(ctx, kind):
    M, steps, seed = 4000, 50, 9
    w = weights(kind, M, 3)
    i = np.repeat(np.arange(M), steps // 2)
    h = np.tile(np.arange(steps // 2), M)
    words = philox_words(seed, "metropolis", i, h)
    u = np.stack([u01_float(words[0]), u01_float(words[2])], 1).reshape(-1)
    j = np.stack([index_of(words[1], M), index_of(words[3], M)], 1).reshape(-1)
    assert np.array_equal(MetropolisResampler(ctx, steps, seed).resample_indices(w), O.resample_metropolis(w, steps, u, j))


@pytest.mark.parametrize("kind", ["uniform", "random", "sparse", "unnormalised"])
def test_gpu_rejection_device_draws_match_oracle(ctx, kind):
    M, seed = 3000, 21
    w = weights(kind, M, 4)
    assert np.array_equal(RejectionResampler(ctx, seed).resample_indices(w), O.resample_rejection_philox(w, seed))


def test_gpu_other_resamplers_device_forms(ctx):
    torch = pytest.importorskip("torch")
    M = 30_000
    rng = np.random.default_rng(6)
    parts = rng.random((M, 7)).astype(np.float32)
    parts[:, 6] = weights("random", M, 7)
    d = torch.from_numpy(parts).cuda()
    out = torch.zeros_like(d)
    torch.cuda.synchronize()
    lib = N.lib()
    vp = C.c_void_p
    cases = [
        (lambda: lib.tsdfl_resample_wheel_device(ctx.handle, vp(d.data_ptr()), M, None, 3, vp(out.data_ptr())),
         WheelResampler(ctx, 3)),
        (lambda: lib.tsdfl_resample_residual_device(ctx.handle, vp(d.data_ptr()), M, None, 0, 3, vp(out.data_ptr())),
         ResidualResampler(ctx, 3)),
        (lambda: lib.tsdfl_resample_metropolis_device(ctx.handle, vp(d.data_ptr()), M, 50, None, None, 3,
                                                      vp(out.data_ptr())), MetropolisResampler(ctx, 50, 3)),
        (lambda: lib.tsdfl_resample_rejection_device(ctx.handle, vp(d.data_ptr()), M, 3, vp(out.data_ptr())),
         RejectionResampler(ctx, 3)),
    ]
    for call, host in cases:
        N.check(call())
        ctx.sync()
        assert np.array_equal(out.cpu().numpy(), parts[host.resample_indices(parts[:, 6])])


def test_gpu_other_resamplers_errors(ctx):
    w = weights("random", 100, 8)
    with pytest.raises(TsdflError) as e:
        ResidualResampler(ctx).resample_indices(w, np.zeros(5, np.uint32) + 3)   # too few draws
    assert e.value.code == N.TSDFL_ERR_UNSUPPORTED
    with pytest.raises(TsdflError) as e:
        ResidualResampler(ctx).resample_indices(w, np.full(500, 100, np.uint32))   # index == M
    assert e.value.code == N.TSDFL_ERR_INVALID_ARG
    with pytest.raises(TsdflError) as e:   # only u draws
        N.check(N.lib().tsdfl_resample_metropolis(ctx.handle, w.ctypes.data, 100, 5, np.zeros(500, np.float32).ctypes.data,
                                                  None, 0, np.zeros(100, np.uint32).ctypes.data))
    assert e.value.code == N.TSDFL_ERR_INVALID_ARG
    # every weight zero: the wheel keeps every particle, residual never fills
    z = np.zeros(64, np.float32)
    assert np.array_equal(WheelResampler(ctx).resample_indices(z), np.arange(64))
    with pytest.raises(TsdflError):
        ResidualResampler(ctx).resample_indices(z)
    # empty clouds
    for r in (WheelResampler(ctx), ResidualResampler(ctx), MetropolisResampler(ctx), RejectionResampler(ctx)):
        assert r.resample_indices(np.zeros(0, np.float32)).shape == (0,)
