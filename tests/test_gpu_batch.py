"""Batched filters (tsdfl_batch): many filters with uneven particle counts and
scan sizes over several maps, scored in one persistent launch (filters that
fill the GPU by themselves with the single-filter kernel), give every
filter exactly its single-filter results -- weights, mean pose, resampled
particles and counts, bit for bit -- eagerly, replayed from a captured CUDA
graph, and after the autotuner changed the work-item shape."""
import ctypes as C

import numpy as np
import pytest

from tsdf_localization_gb300 import Context, DeviceMap, FilterBatch
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
def maps(ctx):
    room = synth.room_workload(seed=1, n_particles=10, n_points=64)
    room5 = synth.make_workload(synth.ROOM, 4, 50, 64, 10, 16, 1024, edge=8)
    tunnel = synth.make_workload(synth.TUNNEL, 5, 100, 64, 10, 32, 1024, edge=16, reduce_cell=0.1)
    out = []
    for wl, dense in ((room, True), (room5, False), (tunnel, True), (room, False)):
        out.append((wl, DeviceMap(ctx, wl.coef, wl.grid_occ, codes=wl.codes, dense=dense)))
    # a float-slot map: scored outside the persistent launch
    out.append((room5, DeviceMap(ctx, room5.coef, room5.grid_occ, data=room5.float_data(), force_f32=True)))
    return out


def make_filters(maps, sizes, seed):
    rng = np.random.default_rng(seed)
    fs, keep = [], []
    for i, (P, Nn) in enumerate(sizes):
        wl, dm = maps[i % len(maps)]
        w = synth.World(synth.ROOM if "room" in wl.name else synth.TUNNEL, 3 + i)
        parts = synth.particles_gaussian(wl.true_pose, 0.3, np.deg2rad(5.0), P, seed + i)
        pts = rng.normal(0, 4, (Nn, 3)).astype(np.float32)
        d_part = torch.from_numpy(parts).cuda()
        d_pts = torch.from_numpy(pts).cuda()
        d_pose = torch.zeros(8, dtype=torch.float32, device="cuda")
        d_u0 = torch.tensor([np.float32(rng.random() / P)], dtype=torch.float32, device="cuda")
        d_out = torch.zeros((2 * P + 16, 7), dtype=torch.float32, device="cuda")
        d_cnt = torch.zeros(4, dtype=torch.int32, device="cuda")
        f = {"map": dm, "P": P, "N": Nn, "tf": wl.tf, "particles": d_part.data_ptr(), "points": d_pts.data_ptr(),
             "pose_out": d_pose.data_ptr(), "u0": d_u0.data_ptr(), "resampled": d_out.data_ptr(),
             "cap": 2 * P + 16, "count": d_cnt.data_ptr()}
        fs.append(f)
        # every device buffer stays referenced while the batch holds its address
        keep.append({"parts0": parts, "pts": pts, "d_pts": d_pts, "part": d_part, "pose": d_pose, "u0": d_u0, "out": d_out,
                     "cnt": d_cnt, "dm": dm, "tf": np.ascontiguousarray(wl.tf, np.float32)})
    return fs, keep


def single(ctx, k, P):
    """The same filter through the single-filter device calls."""
    d_part = torch.from_numpy(k["parts0"].copy()).cuda()
    d_pts = torch.from_numpy(k["pts"]).cuda()
    d_pose = torch.zeros(8, dtype=torch.float32, device="cuda")
    d_out = torch.zeros_like(k["out"])
    d_cnt = torch.zeros(4, dtype=torch.int32, device="cuda")
    model = N.Model(0.9, 0.1, 0.0, 100.0)
    torch.cuda.synchronize()
    N.check(N.lib().tsdfl_evaluate_device(ctx.handle, k["dm"].handle, C.byref(model), vp(d_part.data_ptr()), P,
                                          vp(d_pts.data_ptr()), k["pts"].shape[0], k["tf"].ctypes.data_as(vp), 0,
                                          vp(d_pose.data_ptr())))
    N.check(N.lib().tsdfl_resample_systematic_device(ctx.handle, vp(d_part.data_ptr()), P, float(k["u0"].item()),
                                                     vp(d_out.data_ptr()), d_out.shape[0], vp(d_cnt.data_ptr())))
    ctx.sync()
    return d_part.cpu().numpy(), d_pose.cpu().numpy()[:6], d_out.cpu().numpy(), int(d_cnt[0].item())


def check_same(ctx, keep, sizes):
    for k, (P, _) in zip(keep, sizes):
        w, pose, out, cnt = single(ctx, k, P)
        got_cnt = int(k["cnt"][0].item())
        assert np.array_equal(k["part"].cpu().numpy(), w)
        assert np.array_equal(k["pose"].cpu().numpy()[:6], pose)
        assert got_cnt == cnt
        assert np.array_equal(k["out"].cpu().numpy()[:cnt], out[:cnt])


SIZES = [(1000, 1000), (20_000, 5000), (333, 20_000), (4096, 64), (50_000, 2500), (777, 7777), (12_000, 300),
         (2000, 16_000), (9, 1), (60_000, 12_000)]


def test_gpu_batch_equals_single_filters(ctx, maps):
    fs, keep = make_filters(maps, SIZES, 10)
    b = FilterBatch(ctx, fs)
    info = b.info()
    # two float-slot filters outside the tiled path, two that fill the GPU by
    # themselves (single-filter kernel), the rest in the persistent launch
    assert info["outside"] == 2 and info["single"] == 2 and info["segments"] >= 6
    torch.cuda.synchronize()
    b.run()
    ctx.sync()
    check_same(ctx, keep, SIZES)
    b.close()


def test_gpu_batch_graph_replay_and_autotune(ctx, maps):
    fs, keep = make_filters(maps, SIZES[:6], 20)
    b = FilterBatch(ctx, fs)
    b.capture()
    rng = np.random.default_rng(5)
    for rep in range(3):
        for k, (P, _) in zip(keep, SIZES[:6]):   # new particles and draws between replays
            k["parts0"] = synth.particles_gaussian(np.zeros(6, np.float32) + rep, 0.3, 0.1, P, 100 * rep + P)
            k["part"].copy_(torch.from_numpy(k["parts0"]))
            k["u0"].fill_(float(np.float32(rng.random() / P)))
        torch.cuda.synchronize()
        b.run()
        ctx.sync()
        check_same(ctx, keep, SIZES[:6])
    chunk, group, ms = b.autotune()
    assert chunk % 64 == 0 and group >= 1 and ms > 0
    for k in keep:
        k["part"].copy_(torch.from_numpy(k["parts0"]))
    torch.cuda.synchronize()
    b.run()
    ctx.sync()
    check_same(ctx, keep, SIZES[:6])
    for shape in ((512, 8), (2048, 2), (64, 1)):
        b.set_tiles(*shape)
        for k in keep:
            k["part"].copy_(torch.from_numpy(k["parts0"]))
        torch.cuda.synchronize()
        b.run()
        ctx.sync()
        check_same(ctx, keep, SIZES[:6])
    b.close()


def test_gpu_batch_arguments(ctx, maps):
    with pytest.raises(Exception):
        FilterBatch(ctx, [{"map": maps[0][1], "P": 10, "N": 10, "tf": np.eye(4), "particles": 0, "points": 0}])
    b = FilterBatch(ctx, [])
    b.run()
    ctx.sync()
    b.close()
