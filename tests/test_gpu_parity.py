"""GPU parity: the CUDA sensor update and resampler against the oracle.

Bit-exact: laser poses, voxel (slot) indices, hit counts, serial-mode raw
weights, resampled indices and counts.  Exact-mode weights (fixed-point
likelihood sums): |gpu - fp64| <= 1e-5 |fp64| and never farther from the fp64
sum than the reference-order float sum by more than that bound.
"""
import numpy as np
import pytest

from oracle import oracle_py as O
from tsdf_localization_gb300 import Context, DeviceMap, SystematicResampler, TSDFEvaluator, TsdflError, synth

pytestmark = pytest.mark.gpu

MISS = 0xFFFFFFFF
WEIGHT_RTOL = 1e-5


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def room():
    return synth.room_workload(seed=11, n_particles=600, n_points=2048)


@pytest.fixture(scope="module")
def room_oracle(room):
    return O.OracleMap(O.coef_from(room.coef), room.grid_occ, room.float_data())


def _oracle_eval(om, wl, particles=None, points=None, tf=None, model=(0.9, 0.1, 0.0, 100.0), want_idx=True):
    p = (wl.particles if particles is None else particles).copy()
    r = O.evaluate(om, p, wl.points if points is None else points, wl.tf if tf is None else tf, model,
                   want_idx=want_idx)
    r["particles"] = p
    return r


def _as_u32_index(idx, data_size):
    return np.where(idx < data_size, idx, MISS).astype(np.uint32)


def _fp64_normalised(sum64):
    return sum64 / sum64.sum()


def _fp64_pose(particles, sum64):
    """Weighted mean pose of tsdf_evaluator.cpp:198-221 in double precision."""
    w = _fp64_normalised(sum64)
    p = particles.astype(np.float64)
    xyz = (p[:, :3] * w[:, None]).sum(0)
    ang = [np.arctan2((np.sin(p[:, k]) * w).sum(), (np.cos(p[:, k]) * w).sum()) for k in (3, 4, 5)]
    return np.concatenate([xyz, ang])


def _check_normalised(gpu_w, ref_w, sum64):
    f64 = _fp64_normalised(sum64)
    err_gpu = np.abs(gpu_w.astype(np.float64) - f64)
    err_ref = np.abs(ref_w.astype(np.float64) - f64)
    assert np.all(err_gpu <= WEIGHT_RTOL * f64)
    assert np.all(err_gpu <= err_ref + WEIGHT_RTOL * f64)


def _codes_of(ref_idx, codes, data_size):
    hit = ref_idx < data_size
    return np.where(hit, codes[np.minimum(ref_idx, data_size - 1)], 601).astype(np.uint32)


@pytest.mark.parametrize("kernel", ["fast", "generic"])
@pytest.mark.parametrize("layout", ["brick", "dense", "grid"])
def test_exact_mode_matches_oracle(ctx, room, room_oracle, layout, kernel):
    dmap = DeviceMap(ctx, room.coef, room.grid_occ, codes=room.codes, dense=(layout == "dense"),
                     grid=(layout == "grid"))
    assert dmap.info()["fast_index"] in (1, 2)
    ev = TSDFEvaluator(dmap, generic=(kernel == "generic"))
    ref = _oracle_eval(room_oracle, room)
    p = room.particles.copy()
    d = ev.evaluate_debug(p, room.points, room.tf, voxel_index=True)
    if kernel == "fast":
        d["voxel_index"] &= 0xFFFF   # drop the slow-path flag of the tiled kernel
    assert np.array_equal(d["hits"], ref["hits"])
    if layout != "dense" and kernel == "generic":
        assert np.array_equal(d["voxel_index"], _as_u32_index(ref["voxel_index"], room.coef.data_size))
    else:  # these kernels report slot codes
        assert np.array_equal(d["voxel_index"], _codes_of(ref["voxel_index"], room.codes, room.coef.data_size))
    f64 = ref["sum64"]
    err_gpu = np.abs(d["raw"].astype(np.float64) - f64)
    err_ref = np.abs(ref["raw"].astype(np.float64) - f64)
    assert np.all(err_gpu <= WEIGHT_RTOL * np.abs(f64))
    assert np.all(err_gpu <= err_ref + WEIGHT_RTOL * np.abs(f64))
    _check_normalised(p[:, 6], ref["particles"][:, 6], f64)
    assert np.allclose(d["pose"], _fp64_pose(room.particles, f64), rtol=0, atol=2e-5)
    # inputs other than the weights untouched
    assert np.array_equal(p[:, :6], room.particles[:, :6])


@pytest.mark.parametrize("voxel_mm", [50, 32])
def test_fast_index_with_residual_correction(ctx, voxel_mm):
    """Resolutions whose sub-voxel multiplier can be one short (0.05 m, 0.032 m):
    the tiled kernel's FMA residual test, all three layouts, against the oracle's
    getIndex, including points in the (-1, 0) m band and outside the map."""
    wl = synth.make_workload(synth.ROOM, 13, voxel_mm, 1500, 96, 16, 512, edge=64, name="room@res")
    om = O.OracleMap(O.coef_from(wl.coef), wl.grid_occ, wl.float_data())
    rng = np.random.default_rng(voxel_mm)
    pts = np.concatenate([wl.points, rng.uniform(-1.0, 0.3, size=(200, 3)).astype(np.float32),
                          rng.uniform(-30, 30, size=(200, 3)).astype(np.float32)])
    ref = _oracle_eval(om, wl, points=pts)
    for dense, grid in ((False, False), (True, False), (False, True)):
        dmap = DeviceMap(ctx, wl.coef, wl.grid_occ, codes=wl.codes, dense=dense, grid=grid)
        assert dmap.info()["fast_index"] == 1
        d = TSDFEvaluator(dmap).evaluate_debug(wl.particles.copy(), pts, wl.tf, voxel_index=True)
        assert np.array_equal(d["hits"], ref["hits"])
        assert np.array_equal(d["voxel_index"] & 0xFFFF, _codes_of(ref["voxel_index"], wl.codes, wl.coef.data_size))
        assert np.allclose(d["raw"], ref["sum64"], rtol=WEIGHT_RTOL, atol=0)


def test_map_min_corner_off_origin(ctx, room):
    """A map whose min corner is not the origin (the tiled kernel subtracts it
    from every transformed point): the room's bricks moved to (-1.3, -0.7,
    -0.45) m with the particles, all layouts against the oracle, including
    points in the (-1, 0) m band below the moved floor."""
    from tsdf_localization_gb300 import _native as N
    shift = np.array([-1.3, -0.7, -0.45], np.float32)
    coef = N.MapCoef.from_buffer_copy(bytes(room.coef))
    coef.min_x, coef.min_y, coef.min_z = (float(v) for v in shift)
    coef.max_x, coef.max_y, coef.max_z = (float(np.float32(getattr(room.coef, k)) + v)
                                          for k, v in zip(("max_x", "max_y", "max_z"), shift))
    om = O.OracleMap(O.coef_from(coef), room.grid_occ, room.float_data())
    parts = room.particles.copy()
    parts[:, :3] += shift
    rng = np.random.default_rng(17)
    pts = np.concatenate([room.points, rng.uniform(-1.0, 0.3, size=(300, 3)).astype(np.float32) + shift])
    ref = O.evaluate(om, parts.copy(), pts, room.tf, want_idx=True)
    want = _codes_of(ref["voxel_index"], room.codes, coef.data_size)
    for dense, grid in ((False, False), (True, False), (False, True)):
        dmap = DeviceMap(ctx, coef, room.grid_occ, codes=room.codes, dense=dense, grid=grid)
        assert dmap.info()["fast_index"] in (1, 2)
        d = TSDFEvaluator(dmap).evaluate_debug(parts.copy(), pts, room.tf, voxel_index=True)
        assert np.array_equal(d["hits"], ref["hits"])
        assert np.array_equal(d["voxel_index"] & 0xFFFF, want)
        assert np.allclose(d["raw"], ref["sum64"], rtol=WEIGHT_RTOL, atol=0)


def test_fast_and_generic_kernels_identical(ctx, room):
    """Both exact-mode kernels give identical fixed-point sums, so identical weights."""
    for dense in (False, True):
        dmap = DeviceMap(ctx, room.coef, room.grid_occ, codes=room.codes, dense=dense)
        a = TSDFEvaluator(dmap).evaluate_debug(room.particles.copy(), room.points, room.tf)
        b = TSDFEvaluator(dmap, generic=True).evaluate_debug(room.particles.copy(), room.points, room.tf)
        assert np.array_equal(a["raw"], b["raw"]) and np.array_equal(a["hits"], b["hits"])


def test_serial_mode_bit_exact(ctx, room, room_oracle):
    dmap = DeviceMap(ctx, room.coef, room.grid_occ, codes=room.codes)
    ev = TSDFEvaluator(dmap, serial_sums=True)
    ref = _oracle_eval(room_oracle, room)
    p = room.particles.copy()
    d = ev.evaluate_debug(p, room.points, room.tf, voxel_index=True)
    assert np.array_equal(d["raw"], ref["raw"])
    assert np.array_equal(d["hits"], ref["hits"])
    assert np.array_equal(d["voxel_index"], _as_u32_index(ref["voxel_index"], room.coef.data_size))
    lp = np.stack([O.particle_pose(room.particles[i], room.tf) for i in range(room.particles.shape[0])])
    assert np.array_equal(d["laser_pose"], lp)
    f64 = _fp64_normalised(ref["sum64"])
    assert np.all(np.abs(p[:, 6] - f64) <= np.abs(ref["particles"][:, 6] - f64) + WEIGHT_RTOL * f64)


def test_float_slot_map(ctx, room, room_oracle):
    """A map uploaded as float slots (the CudaSubVoxelMap contents) converts to
    codes losslessly; forced float storage gives the same results."""
    for force in (False, True):
        dmap = DeviceMap(ctx, room.coef, room.grid_occ, data=room.float_data(), force_f32=force)
        assert dmap.info()["storage"] == (1 if force else 0)
        ev = TSDFEvaluator(dmap, serial_sums=True)
        ref = _oracle_eval(room_oracle, room, want_idx=False)
        d = ev.evaluate_debug(room.particles.copy(), room.points, room.tf)
        assert np.array_equal(d["raw"], ref["raw"])
        ev2 = TSDFEvaluator(dmap)
        d2 = ev2.evaluate_debug(room.particles.copy(), room.points, room.tf)
        assert np.array_equal(d2["hits"], ref["hits"])
        assert np.allclose(d2["raw"], ref["sum64"], rtol=WEIGHT_RTOL, atol=0)


def test_points_outside_map_and_negative_offsets(ctx, room, room_oracle):
    """Points far outside the map, at negative offsets and in the (-1, 0) m band
    where the reference's float->size_t conversions wrap."""
    rng = np.random.default_rng(5)
    pts = np.concatenate([
        rng.uniform(-40, 40, size=(700, 3)),
        rng.uniform(-1.0, 0.2, size=(300, 3)) + np.array([11.0, 11.0, -1.2]),
        np.array([[1e20, 0, 0], [-1e20, 0, 0], [0, 0, -3e19], [np.inf, 0, 0], [5, 5, 1e10]]),
    ]).astype(np.float32)
    parts = synth.particles_gaussian([0.3, 0.4, 0.2, 0, 0, 0], 0.6, 0.2, 64, 9)
    ref = _oracle_eval(room_oracle, room, particles=parts, points=pts)
    for dense, grid in ((False, False), (True, False), (False, True)):
        dmap = DeviceMap(ctx, room.coef, room.grid_occ, codes=room.codes, dense=dense, grid=grid)
        for serial, generic in ((True, False), (False, False), (False, True)):
            ev = TSDFEvaluator(dmap, serial_sums=serial, generic=generic)
            d = ev.evaluate_debug(parts.copy(), pts, room.tf, voxel_index=True)
            if not serial and not generic:
                d["voxel_index"] &= 0xFFFF
            assert np.array_equal(d["hits"], ref["hits"])
            if serial or (generic and not dense):
                assert np.array_equal(d["voxel_index"], _as_u32_index(ref["voxel_index"], room.coef.data_size))
            else:
                assert np.array_equal(d["voxel_index"], _codes_of(ref["voxel_index"], room.codes,
                                                                  room.coef.data_size))
            if serial:
                assert np.array_equal(d["raw"], ref["raw"])


def test_multi_pass_long_scan(ctx, room, room_oracle):
    """Scans longer than one shared-memory pass (16384 exact, 8192 serial)."""
    w = synth.World(synth.ROOM, 11)
    xyz, ring = w.scan(room.true_pose, 32, 1024, seed=3)
    pts = xyz[:20000]
    parts = room.particles[:40].copy()
    ref = _oracle_eval(room_oracle, room, particles=parts, points=pts, want_idx=False)
    dmap = DeviceMap(ctx, room.coef, room.grid_occ, codes=room.codes)
    d = TSDFEvaluator(dmap, serial_sums=True).evaluate_debug(parts.copy(), pts, room.tf)
    assert np.array_equal(d["raw"], ref["raw"])
    d2 = TSDFEvaluator(dmap).evaluate_debug(parts.copy(), pts, room.tf)
    assert np.array_equal(d2["hits"], ref["hits"])
    assert np.allclose(d2["raw"], ref["sum64"], rtol=WEIGHT_RTOL, atol=0)


@pytest.mark.parametrize("spread", ["compact", "wide"])
def test_scan_order_independent_of_point_order(ctx, room, room_oracle, spread):
    """The tiled kernels stage the scan in a spatial order chosen by the cloud's
    extent (azimuth sector and range for a compact cloud, height band first for
    one wider than 10 m): per-point codes still land at their scan index, the
    weights equal the oracle's, and permuting the input points changes nothing."""
    rng = np.random.default_rng(21)
    parts = room.particles[:256].copy()
    if spread == "wide":   # 16 m across in x and y, any yaw
        parts[:, 0] += rng.uniform(-8.0, 8.0, 256).astype(np.float32)
        parts[:, 1] += rng.uniform(-8.0, 8.0, 256).astype(np.float32)
        parts[:, 5] = rng.uniform(-np.pi, np.pi, 256).astype(np.float32)
    ref = _oracle_eval(room_oracle, room, particles=parts)
    dmap = DeviceMap(ctx, room.coef, room.grid_occ, codes=room.codes, dense=True)
    ev = TSDFEvaluator(dmap)
    d = ev.evaluate_debug(parts.copy(), room.points, room.tf, voxel_index=True)
    assert np.array_equal(d["hits"], ref["hits"])
    assert np.array_equal(d["voxel_index"] & 0xFFFF, _codes_of(ref["voxel_index"], room.codes, room.coef.data_size))
    assert np.allclose(d["raw"], ref["sum64"], rtol=WEIGHT_RTOL, atol=0)
    perm = rng.permutation(room.points.shape[0])
    e = ev.evaluate_debug(parts.copy(), room.points[perm], room.tf, voxel_index=True)
    assert np.array_equal(e["raw"], d["raw"]) and np.array_equal(e["hits"], d["hits"])
    assert np.array_equal(e["voxel_index"], d["voxel_index"][:, perm])


def test_empty_scan_leaves_particles(ctx, room):
    dmap = DeviceMap(ctx, room.coef, room.grid_occ, codes=room.codes)
    p = room.particles.copy()
    assert TSDFEvaluator(dmap).evaluate(p, np.zeros((0, 3), np.float32), room.tf) is None
    assert np.array_equal(p, room.particles)


def test_degenerate_weights_raise(ctx, room):
    """All scores zero -> "No particle is valid!" and particles untouched."""
    dmap = DeviceMap(ctx, room.coef, room.grid_occ, codes=room.codes)
    ev = TSDFEvaluator(dmap, a_hit=0.0, a_range=0.0, a_max=0.0)
    p = room.particles.copy()
    with pytest.raises(TsdflError, match="No particle is valid!"):
        ev.evaluate(p, room.points, room.tf)
    assert np.array_equal(p, room.particles)
    # the context stays usable
    p2 = room.particles.copy()
    TSDFEvaluator(dmap).evaluate(p2, room.points, room.tf)
    assert abs(float(p2[:, 6].astype(np.float64).sum()) - 1.0) < 1e-4


def test_out_of_range_points_and_model(ctx, room, room_oracle):
    """Points beyond max_range take a_max instead of a_range/max_range."""
    model = (0.7, 0.2, 0.05, 6.0)
    ref = _oracle_eval(room_oracle, room, model=model, want_idx=False)
    dmap = DeviceMap(ctx, room.coef, room.grid_occ, codes=room.codes)
    d = TSDFEvaluator(dmap, a_hit=0.7, a_range=0.2, a_max=0.05, max_range=6.0, serial_sums=True).evaluate_debug(
        room.particles.copy(), room.points, room.tf)
    assert np.array_equal(d["raw"], ref["raw"])
    d2 = TSDFEvaluator(dmap, a_hit=0.7, a_range=0.2, a_max=0.05, max_range=6.0).evaluate_debug(
        room.particles.copy(), room.points, room.tf)
    assert np.allclose(d2["raw"], ref["sum64"], rtol=WEIGHT_RTOL, atol=0)


def _random_weights(rng, m, kind):
    if kind == "uniform":
        w = np.full(m, 1.0 / m)
    elif kind == "random":
        w = rng.random(m)
    elif kind == "peaked":
        w = rng.random(m) ** 8
    elif kind == "one":
        w = np.zeros(m)
        w[rng.integers(m)] = 1.0
    elif kind == "tiny":   # weights below 2^-29: serial double sums on the device
        w = rng.random(m)
        w[: m // 3] = 1e-12
    elif kind == "negative":   # negative weights: the literal loop on the device
        w = rng.random(m)
        w[:: max(1, m // 5)] *= -0.01
    else:
        raise ValueError(kind)
    w = w / w.sum()
    return w.astype(np.float32)


@pytest.mark.parametrize("m", [1, 2, 7, 1000, 4096, 65537, 250000])
@pytest.mark.parametrize("kind", ["uniform", "random", "peaked", "one", "tiny", "negative"])
def test_resample_bit_exact(ctx, m, kind):
    rng = np.random.default_rng(m * 31 + len(kind))
    w = _random_weights(rng, m, kind)
    rs = SystematicResampler(ctx, seed=m)
    parts = rng.random((m, 7)).astype(np.float32)   # the same weights inside a particle cloud
    parts[:, 6] = w
    # u0 from 0 and subnormal values up to just below 1/M: the draws' segments
    # cross many float binades before the first regular step
    for u0 in (0.0, float(np.float32(1e-42)), float(np.float32(1e-30)), float(np.float32(0.5 / m)),
               float(np.nextafter(np.float32(1.0 / m), np.float32(0))), rs.draw(m)):
        got = rs.resample_indices(w, u0)
        exp = O.resample_systematic(w, u0)
        assert got.shape == exp.shape
        assert np.array_equal(got, exp)
        assert np.array_equal(rs.resample_particle_indices(parts, u0), exp)


@pytest.mark.parametrize("m", [1, 2, 7, 1000, 65537, 250000])
@pytest.mark.parametrize("kind", ["uniform", "random", "peaked", "one", "tiny"])
def test_residual_resample_bit_exact(ctx, m, kind):
    """ResidualSystematicResampler: indices and count equal the oracle's (pinned
    to the reference) for draws at both ends of [0, 1)."""
    from tsdf_localization_gb300 import ResidualSystematicResampler
    rng = np.random.default_rng(m * 17 + len(kind))
    w = _random_weights(rng, m, kind)
    rs = ResidualSystematicResampler(ctx, seed=m)
    for u0 in (0.0, 0.5, float(np.nextafter(np.float32(1.0), np.float32(0))), rs.draw()):
        got = rs.resample_indices(w, u0, cap=2 * m + 16)
        exp = O.resample_residual_systematic(w, u0, cap=2 * m + 16)
        assert np.array_equal(got, exp)


def test_residual_resample_device_form_and_errors(ctx):
    from tsdf_localization_gb300 import ResidualSystematicResampler
    from tsdf_localization_gb300 import _native as N
    import ctypes as C
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    m = 5000
    parts = rng.normal(size=(m, 7)).astype(np.float32)
    parts[:, 6] = _random_weights(rng, m, "random")
    u0 = 0.3125
    idx = ResidualSystematicResampler(ctx).resample_indices(parts[:, 6], u0)
    d_in = torch.from_numpy(parts).cuda()
    d_out = torch.zeros((2 * m + 16, 7), dtype=torch.float32, device="cuda")
    d_cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    N.check(N.lib().tsdfl_resample_residual_systematic_device(ctx.handle, C.c_void_p(d_in.data_ptr()), m,
                                                              np.float32(u0), C.c_void_p(d_out.data_ptr()),
                                                              2 * m + 16, C.c_void_p(d_cnt.data_ptr())))
    ctx.sync()
    n = int(d_cnt.item())
    assert n == idx.shape[0]
    assert np.array_equal(d_out[:n].cpu().numpy(), parts[idx])
    bad = parts[:, 6].copy()
    bad[10] = -1.0
    with pytest.raises(TsdflError):
        ResidualSystematicResampler(ctx).resample_indices(bad, u0)
    # the context stays usable
    assert np.array_equal(ResidualSystematicResampler(ctx).resample_indices(parts[:, 6], u0), idx)


def test_best_particle(ctx):
    """mcl_3d.cpp:382-394: first index of the largest weight above 0."""
    import ctypes as C
    from tsdf_localization_gb300 import _native as N
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(8)

    def best_gpu(parts):
        d_in = torch.from_numpy(np.ascontiguousarray(parts)).cuda()
        d_idx = torch.zeros(1, dtype=torch.int32, device="cuda")
        N.check(N.lib().tsdfl_best_particle_device(ctx.handle, C.c_void_p(d_in.data_ptr()), parts.shape[0],
                                                   C.c_void_p(d_idx.data_ptr())))
        ctx.sync()
        return int(d_idx.item()) & 0xFFFFFFFF

    def best_ref(w):
        best, idx = np.float32(0.0), -1
        for i, v in enumerate(w):
            if v > best:
                best, idx = v, i
        return idx & 0xFFFFFFFF

    for m, kind in [(1, "one"), (1000, "random"), (300001, "random"), (5000, "ties"), (64, "zero"), (100, "neg")]:
        parts = rng.normal(size=(m, 7)).astype(np.float32)
        w = rng.random(m).astype(np.float32)
        if kind == "ties":
            w[[17, 4000, 99]] = np.float32(2.0)
        elif kind == "zero":
            w[:] = 0.0
        elif kind == "neg":
            w = -w
            w[50] = np.float32(1e-30)
        parts[:, 6] = w
        assert best_gpu(parts) == best_ref(parts[:, 6])


def _sparse_room(seed=4):
    """The room at 0.064 m plus one chunk about 200 m away: the bounding box
    holds about 840,000 bricks, too many for the shared-memory bitmap, almost
    all of them empty."""
    from tsdf_localization_gb300 import build_map_codes
    wl = synth.make_workload(synth.ROOM, seed, 64, 2048, 600, 16, 1024, edge=16, name="room+far")
    pos, raw = synth.World(synth.ROOM, seed).tsdf_chunks(64, edge=16)
    busy = int(np.argmax((raw >> 16).astype(bool).sum(1)))
    pos = np.concatenate([pos, np.array([[195, 195, 19]], np.int32)])
    raw = np.concatenate([raw, raw[busy:busy + 1]])
    names = ["%d_%d_%d" % tuple(p) for p in pos]
    order = sorted(range(len(names)), key=lambda i: names[i].encode())
    coef, go, codes, _ = build_map_codes(pos[order], raw[order], 16, 64, 0.1, want_free=False)
    return wl, coef, go, codes


@pytest.mark.parametrize("case", ["sparse", "forced"])
def test_sparse_brick_hash(ctx, case):
    """The sparse brick hash: built by the compact layout on its own when the
    brick bitmap exceeds shared memory ("sparse"), or on request
    (TSDFL_MAP_HASH, "forced"); slot codes and hit counts equal the oracle's,
    the weights the brick-table kernel's, within 1e-5 of FP64."""
    from tsdf_localization_gb300.evaluator import code_values
    if case == "sparse":
        wl, coef, go, codes = _sparse_room()
        assert coef.grid_occ_size > 524_288
        dmap = DeviceMap(ctx, coef, go, codes=codes, dense=True)
    else:
        wl = synth.room_workload(seed=11, n_particles=600, n_points=2048)
        coef, go, codes = wl.coef, wl.grid_occ, wl.codes
        dmap = DeviceMap(ctx, coef, go, codes=codes, hash_index=True)
    info = dmap.info()
    assert info["dense"] == 2 and info["fast_index"] in (1, 2)
    vals = np.append(code_values(0.1, coef.init_value), np.float32(coef.init_value))
    om = O.OracleMap(O.coef_from(coef), go, vals[codes])
    rng = np.random.default_rng(3)
    pts = np.concatenate([wl.points, rng.uniform(-1.0, 0.3, size=(200, 3)).astype(np.float32)])
    ref = _oracle_eval(om, wl, points=pts)
    d = TSDFEvaluator(dmap).evaluate_debug(wl.particles.copy(), pts, wl.tf, voxel_index=True)
    assert np.array_equal(d["hits"], ref["hits"])
    assert np.array_equal(d["voxel_index"] & 0xFFFF, _codes_of(ref["voxel_index"], codes, coef.data_size))
    assert np.allclose(d["raw"], ref["sum64"], rtol=WEIGHT_RTOL, atol=0)
    brick = DeviceMap(ctx, coef, go, codes=codes)
    assert brick.info()["dense"] == 0
    e = TSDFEvaluator(brick).evaluate_debug(wl.particles.copy(), pts, wl.tf)
    assert np.array_equal(e["raw"], d["raw"]) and np.array_equal(e["hits"], d["hits"])
