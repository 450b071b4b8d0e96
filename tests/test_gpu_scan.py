"""Scan reduction on the GPU (tsdfl_reduce_scan*, tsdfl_evaluate_cloud) against
the reference's recorded outputs and the oracle: the same points in the same
order, bit for bit, for PointCloud2 layouts with aligned and unaligned fields,
both ring conventions, clouds of LiDAR size, and the error cases."""
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle_py as O
from tsdf_localization_gb300 import Context, DeviceMap, ScanReducer, TSDFEvaluator, TsdflError, pack_cloud
from tsdf_localization_gb300 import _native as N
from tsdf_localization_gb300 import synth

pytestmark = pytest.mark.gpu
GOLD = np.load(Path(__file__).resolve().parent / "golden" / "reference_cases.npz")
SCANS = sorted({k.rsplit("/", 1)[0] for k in GOLD.files if k.startswith("scan/")})


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


def lidar(rings, cols, seed, near=0.03):
    w = synth.World(synth.BUILDING, 2)
    xyz, ring = w.scan(np.array([50.5, 50.5, 2.2, 0, 0, 0.3], np.float32), rings, cols, sigma=0.02,
                       dropout=0.01, seed=seed)
    rng = np.random.default_rng(seed)
    close = rng.random(xyz.shape[0]) < near
    xyz[close] *= np.float32(0.05)
    return xyz, ring


@pytest.mark.parametrize("case", SCANS)
def test_gpu_scan_reduction_matches_reference(ctx, case):
    got = ScanReducer(ctx, float(GOLD[f"{case}/cell"])).reduce_xyz(GOLD[f"{case}/xyz"], GOLD[f"{case}/ring"])
    assert np.array_equal(got, GOLD[f"{case}/reduced"], equal_nan=True)


@pytest.mark.parametrize("layout", [(16, 0, 12), (22, 0, 16), (32, 4, 20), (48, 16, 33), (15, 1, 13), (15, 3, 0)])
@pytest.mark.parametrize("own_ring", [False, True])
def test_gpu_scan_reduction_layouts(ctx, layout, own_ring):
    step, xo, ro = layout
    xyz, ring = lidar(16, 1024, 7)
    blob = pack_cloud(xyz, ring, step, xo, ro)
    got = ScanReducer(ctx, 0.064, own_ring).reduce(blob, xyz.shape[0], step, xo, ro)
    assert np.array_equal(got, O.reduce_scan(xyz, ring, 0.064, own_ring), equal_nan=True)


@pytest.mark.parametrize("rings,cols,cell", [(64, 2048, 0.064), (64, 4096, 0.05), (32, 1800, 0.2)])
def test_gpu_scan_reduction_lidar_size(ctx, rings, cols, cell):
    xyz, ring = lidar(rings, cols, 11)
    got = ScanReducer(ctx, cell).reduce_xyz(xyz, ring)
    want = O.reduce_scan(xyz, ring, cell)
    assert got.shape == want.shape and np.array_equal(got, want, equal_nan=True)


def test_gpu_scan_reduction_duplicates_and_non_finite(ctx):
    rng = np.random.default_rng(5)
    n = 200_000
    xyz = (np.round(rng.normal(0, 4, (n, 3)) * 4) / 4).astype(np.float32)
    xyz[rng.random(n) < 0.02, 0] = np.nan
    xyz[rng.random(n) < 0.01, 2] = np.inf
    ring = rng.integers(0, 3, n).astype(np.int16)
    for own in (False, True):
        got = ScanReducer(ctx, 0.25, own).reduce_xyz(xyz, ring)
        assert np.array_equal(got, O.reduce_scan(xyz, ring, 0.25, own), equal_nan=True)


def test_gpu_scan_reduction_edges(ctx):
    red = ScanReducer(ctx, 0.064)
    assert red.reduce_xyz(np.zeros((0, 3), np.float32), np.zeros(0, np.int16)).shape == (0, 3)
    inside = np.full((5000, 3), 0.3, np.float32)
    assert red.reduce_xyz(inside, np.zeros(5000, np.int16)).shape == (0, 3)
    xyz, ring = lidar(16, 256, 3)
    bad = ring.copy()
    bad[100] = 64
    with pytest.raises(TsdflError) as e:
        red.reduce_xyz(xyz, bad)
    assert e.value.code == N.TSDFL_ERR_INVALID_ARG
    bad[100] = -1
    with pytest.raises(TsdflError):
        red.reduce_xyz(xyz, bad)
    # a ring outside [0, 64) that the iterator never reaches is harmless
    tail = ring.copy()
    tail[-1] = 99
    xyz_t = xyz.copy()
    xyz_t[0] = 0.0                      # one point dropped: the last ring field is never read
    assert np.array_equal(red.reduce_xyz(xyz_t, tail), O.reduce_scan(xyz_t, tail, 0.064), equal_nan=True)
    # capacity: the count is still reported
    blob = pack_cloud(xyz, ring)
    out = np.zeros((10, 3), np.float32)
    import ctypes as C
    cnt = C.c_size_t(0)
    rc = N.lib().tsdfl_reduce_scan(ctx.handle, blob.ctypes.data, xyz.shape[0], 16, 0, 12, 0.064, 0, out.ctypes.data,
                                   10, C.byref(cnt))
    want = O.reduce_scan(xyz, ring, 0.064)
    assert rc == N.TSDFL_ERR_CAPACITY and cnt.value == want.shape[0]
    assert np.array_equal(out, want[:10])
    # invalid arguments are refused before any launch
    for args in ((16, 8, 12, 0.064), (16, 0, 15, 0.064), (16, 0, 12, 0.0), (16, 0, 12, float("nan"))):
        rc = N.lib().tsdfl_reduce_scan(ctx.handle, blob.ctypes.data, xyz.shape[0], args[0], args[1], args[2],
                                       args[3], 0, out.ctypes.data, 10, C.byref(cnt))
        assert rc == N.TSDFL_ERR_INVALID_ARG


def test_gpu_scan_reduction_device_form(ctx):
    torch = pytest.importorskip("torch")
    import ctypes as C
    xyz, ring = lidar(64, 1024, 9)
    blob = torch.from_numpy(pack_cloud(xyz, ring, 22, 0, 16)).cuda()
    out = torch.zeros((xyz.shape[0], 3), dtype=torch.float32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    N.check(N.lib().tsdfl_reduce_scan_device(ctx.handle, C.c_void_p(blob.data_ptr()), xyz.shape[0], 22, 0, 16,
                                             0.064, 0, C.c_void_p(out.data_ptr()), xyz.shape[0],
                                             C.c_void_p(cnt.data_ptr())))
    ctx.sync()
    want = O.reduce_scan(xyz, ring, 0.064)
    m = int(cnt.item())
    assert m == want.shape[0]
    assert np.array_equal(out[:m].cpu().numpy(), want, equal_nan=True)


@pytest.mark.parametrize("serial", [False, True])
def test_gpu_evaluate_cloud_equals_evaluate_on_reduced_points(ctx, serial):
    wl = synth.room_workload(n_particles=2000, n_points=2048)
    dmap = DeviceMap(ctx, wl.coef, wl.grid_occ, codes=wl.codes)
    w = synth.World(synth.ROOM, 1)
    xyz, ring = w.scan(wl.true_pose, 16, 900, sigma=0.01, dropout=0.02, seed=4)
    ev = TSDFEvaluator(dmap, serial_sums=serial)
    p1 = wl.particles.copy()
    pose1, n_red = ev.evaluate_cloud(p1, pack_cloud(xyz, ring), xyz.shape[0], 16, wl.tf)
    pts = O.reduce_scan(xyz, ring, 0.064)
    assert n_red == pts.shape[0]
    p2 = wl.particles.copy()
    pose2 = ev.evaluate(p2, pts, wl.tf)
    assert np.array_equal(p1, p2)
    assert np.array_equal(pose1.as_array(), pose2.as_array())
