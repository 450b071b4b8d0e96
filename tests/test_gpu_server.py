"""Served sessions (tsdfl_server): sessions over several maps with uneven
particle counts submit scans while earlier batches run; every update's pose
and the session's particles after it equal the single-filter calls
(tsdfl_evaluate_device + tsdfl_resample_systematic_device with the session's
draw) -- the same result alone and in the mix -- and admission refuses what
does not fit."""
import ctypes as C

import numpy as np
import pytest

from tsdf_localization_gb300 import Context, DeviceMap, LocalizationServer
from tsdf_localization_gb300 import _native as N
from tsdf_localization_gb300 import synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
vp = C.c_void_p


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def worlds(ctx):
    room = synth.room_workload(seed=1, n_particles=10, n_points=64)
    tunnel = synth.make_workload(synth.TUNNEL, 5, 100, 64, 10, 32, 1024, edge=16, reduce_cell=0.1)
    return [(room, DeviceMap(ctx, room.coef, room.grid_occ, codes=room.codes, dense=True)),
            (tunnel, DeviceMap(ctx, tunnel.coef, tunnel.grid_occ, codes=tunnel.codes, dense=True))]


def single_update(ctx, dm, particles, points, tf, u0):
    """One update through the single-filter device calls: (pose, new particles)."""
    P = particles.shape[0]
    d_part = torch.from_numpy(particles.copy()).cuda()
    d_pts = torch.from_numpy(np.ascontiguousarray(points, np.float32)).cuda()
    d_pose = torch.zeros(8, dtype=torch.float32, device="cuda")
    d_out = torch.zeros((2 * P + 16, 7), dtype=torch.float32, device="cuda")
    d_cnt = torch.zeros(4, dtype=torch.int32, device="cuda")
    model = N.Model(0.9, 0.1, 0.0, 100.0)
    t = np.ascontiguousarray(tf, np.float32).reshape(16)
    torch.cuda.synchronize()
    N.check(N.lib().tsdfl_evaluate_device(ctx.handle, dm.handle, C.byref(model), vp(d_part.data_ptr()), P,
                                          vp(d_pts.data_ptr()), points.shape[0], t.ctypes.data_as(vp), 0,
                                          vp(d_pose.data_ptr())))
    N.check(N.lib().tsdfl_resample_systematic_device(ctx.handle, vp(d_part.data_ptr()), P, u0, vp(d_out.data_ptr()),
                                                     2 * P + 16, vp(d_cnt.data_ptr())))
    ctx.sync()
    cnt = min(int(d_cnt[0].item()), 2 * P + 16)
    return d_pose.cpu().numpy()[:6], d_out.cpu().numpy()[:cnt]


def drain(srv, tickets):
    out = {}
    for _ in range(200000):
        srv.poll()
        for t in list(tickets):
            r = srv.result(t)
            if r is not None:
                out[t] = r
                tickets.remove(t)
        if not tickets:
            return out
    raise AssertionError("updates did not finish")


def test_gpu_server_results_equal_single_updates(ctx, worlds):
    rng = np.random.default_rng(3)
    srv = LocalizationServer(ctx, hbm_budget=8 << 30, max_sessions=12, max_points=12000, max_queue=4)
    sessions = []
    for i, P in enumerate([1500, 40_000, 333, 9000, 20_000, 64, 5000, 12_345]):
        wl, dm = worlds[i % 2]
        parts = synth.particles_gaussian(wl.true_pose, 0.3, np.deg2rad(5.0), P, 50 + i)
        sid = srv.open(dm, parts, wl.tf, seed=1000 + i)
        sessions.append({"sid": sid, "dm": dm, "wl": wl, "parts": parts, "seed": 1000 + i, "k": 0,
                         "scans": [], "tickets": []})
    # three rounds; in each round every session submits one or two scans, and
    # the server is polled between submissions so batches overlap arrivals
    for rnd in range(3):
        for s in sessions:
            for _ in range(1 + (rnd + s["sid"]) % 2):
                Nn = int(rng.integers(1, 12000))
                pts = rng.normal(0, 4, (Nn, 3)).astype(np.float32)
                t = srv.submit(s["sid"], pts)
                assert t is not None
                s["scans"].append(pts)
                s["tickets"].append(t)
                srv.poll()
    pending = [t for s in sessions for t in s["tickets"]]
    res = drain(srv, set(pending))
    for s in sessions:
        parts = s["parts"]
        for k, (pts, t) in enumerate(zip(s["scans"], s["tickets"])):
            u0 = LocalizationServer.draw(s["seed"], k, parts.shape[0])
            pose, parts = single_update(ctx, s["dm"], parts, pts, s["wl"].tf, u0)
            got_pose, lat, st = res[t]
            assert st == 0 and lat > 0
            assert np.array_equal(got_pose, pose)
        assert np.array_equal(srv.particles(s["sid"]), parts)
    st = srv.stats()
    assert st["published"] == len(pending) and st["batches"] >= 3
    srv.close()


def test_gpu_server_admission(ctx, worlds):
    wl, dm = worlds[0]
    parts = synth.particles_gaussian(wl.true_pose, 0.3, 0.1, 200_000, 1)
    srv = LocalizationServer(ctx, hbm_budget=32 << 20, max_sessions=4, max_points=4000, max_queue=1)
    with pytest.raises(Exception):   # 200k particles (about 64 MB of device state) do not fit 32 MB
        srv.open(dm, parts, wl.tf)
    sid = srv.open(dm, parts[:1000], wl.tf)
    pts = np.random.default_rng(0).normal(0, 4, (3000, 3)).astype(np.float32)
    assert srv.submit(sid, pts) is not None
    assert srv.submit(sid, pts) is None   # the session's queue holds one
    assert srv.stats()["refused"] == 1
    srv.close()
    srv = LocalizationServer(ctx, hbm_budget=8 << 30, max_sessions=4, max_points=4000, max_wait_ms=1e-6)
    sid = srv.open(dm, parts[:1000], wl.tf)
    assert srv.submit(sid, pts) is None   # any work would wait longer than the bound
    srv.close()


def test_gpu_server_long_scans_and_failed_update(ctx, worlds):
    """Scans of several shared-memory passes from every session in one batch,
    and one session whose update fails (all scores zero: "No particle is
    valid!"): that update is published with its error and the session keeps
    its particles; every other update equals the single-filter calls, and the
    server keeps serving all sessions afterwards."""
    rng = np.random.default_rng(9)
    srv = LocalizationServer(ctx, hbm_budget=8 << 30, max_sessions=6, max_points=40000, max_queue=2)
    sessions = []
    for i, P in enumerate([2000, 700, 5000, 1200, 3000]):
        wl, dm = worlds[i % 2]
        parts = synth.particles_gaussian(wl.true_pose, 0.3, np.deg2rad(5.0), P, 80 + i)
        sessions.append({"sid": srv.open(dm, parts, wl.tf, seed=70 + i), "dm": dm, "wl": wl, "parts": parts,
                         "seed": 70 + i})
    wl, dm = worlds[0]
    bad_parts = synth.particles_gaussian(wl.true_pose, 0.3, 0.1, 900, 99)
    bad = srv.open(dm, bad_parts, wl.tf, model=(0.0, 0.0, 0.0, 100.0), seed=5)
    for rnd in range(2):
        tickets = {}
        for s in sessions:
            pts = rng.normal(0, 4, (int(rng.integers(20000, 40001)), 3)).astype(np.float32)
            tickets[srv.submit(s["sid"], pts)] = (s, pts)
        tb = srv.submit(bad, rng.normal(0, 4, (25000, 3)).astype(np.float32))
        res = drain(srv, set(tickets) | {tb})
        assert res[tb][2] == N.TSDFL_ERR_DEGENERATE
        for t, (s, pts) in tickets.items():
            u0 = LocalizationServer.draw(s["seed"], rnd, s["parts"].shape[0])
            pose, s["parts"] = single_update(ctx, s["dm"], s["parts"], pts, s["wl"].tf, u0)
            got_pose, _, st = res[t]
            assert st == 0 and np.array_equal(got_pose, pose)
    for s in sessions:
        assert np.array_equal(srv.particles(s["sid"]), s["parts"])
    assert np.array_equal(srv.particles(bad), bad_parts)
    srv.close()
