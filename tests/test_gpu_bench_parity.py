"""GPU parity on the workloads the bench reports, against the oracle.

- the 100x100x10 m building at 0.05 m with 100,000 Gaussian particles x 8,192
  points (compact and grid layouts, two-term sub-voxel multiplier, points below the
  map's floor, the compact-cloud scan order): a particle sample against the
  oracle, and all 100,000 particles across the two scoring kernels;
- global localisation on the seed-3 building: 1,000,000 particles uniform over
  free space (any yaw, the spread-cloud scan order) x 2,048 points, a sample
  against the oracle; systematic resampling of the device's own normalised
  weights at 1M bit for bit, and at 1M with weights below 2^-29 (the
  binade-by-binade double sums); the variant where every particle scores 256
  of the points, chosen per particle and seed.

Bars (as in test_gpu_parity.py): slot codes and hit counts bit-exact; serial
raw weights bit-exact; exact-mode weights within 1e-5 of the FP64 sums and no
farther from them than the reference's float sums plus that bound; resampled
indices bit-exact.
"""
import numpy as np
import pytest

from oracle import oracle_py as O
from tsdf_localization_gb300 import Context, DeviceMap, SystematicResampler, TSDFEvaluator, synth

pytestmark = pytest.mark.gpu

WEIGHT_RTOL = 1e-5
SAMPLE = 4000


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def building():
    return synth.building_workload(seed=2, n_particles=100_000, n_points=8192)


@pytest.fixture(scope="module")
def global_wl():
    return synth.global_workload(seed=3, n_particles=1_000_000, n_points=2048)


def _codes_of(ref_idx, codes, data_size):
    hit = ref_idx < data_size
    return np.where(hit, codes[np.minimum(ref_idx, data_size - 1)], 601).astype(np.uint32)


def _check_against_oracle(ctx, wl, parts, serial_n):
    """Compact and grid layouts: tiled kernel (debug and production
    instantiations) and serial kernel against the oracle on the given
    particles."""
    om = O.OracleMap(O.coef_from(wl.coef), wl.grid_occ, wl.float_data())
    p_ref = parts.copy()
    ref = O.evaluate(om, p_ref, wl.points, wl.tf, want_idx=True)
    assert ref["rc"] == 0
    f64 = ref["sum64"]
    want_codes = _codes_of(ref["voxel_index"], wl.codes, wl.coef.data_size)
    err_ref = np.abs(ref["raw"].astype(np.float64) - f64)
    sub = parts[:serial_n].copy()
    ref_s = O.evaluate(om, sub.copy(), wl.points, wl.tf)
    out = {}
    for layout, want_dense in (("compact", 1), ("grid", 3)):
        dmap = DeviceMap(ctx, wl.coef, wl.grid_occ, codes=wl.codes, dense=layout == "compact",
                         grid=layout == "grid")
        info = dmap.info()
        assert info["dense"] == want_dense and info["fast_index"] in (1, 2)
        ev = TSDFEvaluator(dmap)
        p = parts.copy()
        d = ev.evaluate_debug(p, wl.points, wl.tf, voxel_index=True)
        assert np.array_equal(d["hits"], ref["hits"])
        assert np.array_equal(d["voxel_index"] & 0xFFFF, want_codes)
        err_gpu = np.abs(d["raw"].astype(np.float64) - f64)
        assert np.all(err_gpu <= WEIGHT_RTOL * f64)
        assert np.all(err_gpu <= err_ref + WEIGHT_RTOL * f64)
        w64 = f64 / f64.sum()
        assert np.all(np.abs(p[:, 6].astype(np.float64) - w64) <= WEIGHT_RTOL * w64)
        # the production (debug-free) instantiation gives the same sums
        p2 = parts.copy()
        d2 = ev.evaluate_debug(p2, wl.points, wl.tf)
        assert np.array_equal(d2["raw"], d["raw"]) and np.array_equal(d2["hits"], d["hits"])
        assert np.array_equal(p2[:, 6], p[:, 6])
        # serial mode: the reference's point-order float sums, bit for bit
        ds = TSDFEvaluator(dmap, serial_sums=True).evaluate_debug(sub.copy(), wl.points, wl.tf)
        assert np.array_equal(ds["raw"], ref_s["raw"])
        assert np.array_equal(ds["hits"], ref_s["hits"])
        if out:
            assert np.array_equal(d["raw"], out["raw"])   # both layouts: the same fixed-point sums
        out = {"max_rel": float((err_gpu / f64).max()), "ref_max_rel": float((err_ref / f64).max()),
               "hits": d["hits"], "raw": d["raw"]}
    return out


def test_building_sample_matches_oracle(ctx, building):
    """C2's map, scan and particle cloud: every 25th of the 100,000 particles."""
    parts = np.ascontiguousarray(building.particles[:: building.particles.shape[0] // SAMPLE][:SAMPLE])
    ext = parts[:, :2].max(0) - parts[:, :2].min(0)
    assert ext.max() < 10.0   # the compact-cloud scan order
    r = _check_against_oracle(ctx, building, parts, serial_n=500)
    assert r["max_rel"] <= 1e-6   # exact sums: far inside the bound
    assert r["hits"].mean() > 0.5 * building.points.shape[0]


def test_building_full_size_kernels_agree(ctx, building):
    """All 100,000 x 8,192: the tiled kernel on the compact and grid layouts and
    the generic kernel on the brick table give identical fixed-point sums (so
    identical weights and hit counts), and the weights sum to 1."""
    compact = DeviceMap(ctx, building.coef, building.grid_occ, codes=building.codes, dense=True)
    brick = DeviceMap(ctx, building.coef, building.grid_occ, codes=building.codes, dense=False)
    a = TSDFEvaluator(compact).evaluate_debug(building.particles.copy(), building.points, building.tf)
    pb = building.particles.copy()
    b = TSDFEvaluator(brick, generic=True).evaluate_debug(pb, building.points, building.tf)
    assert np.array_equal(a["raw"], b["raw"]) and np.array_equal(a["hits"], b["hits"])
    assert abs(float(pb[:, 6].astype(np.float64).sum()) - 1.0) < 1e-4
    del compact
    grid = DeviceMap(ctx, building.coef, building.grid_occ, codes=building.codes, grid=True)
    assert grid.info()["dense"] == 3
    g = TSDFEvaluator(grid).evaluate_debug(building.particles.copy(), building.points, building.tf)
    assert np.array_equal(g["raw"], b["raw"]) and np.array_equal(g["hits"], b["hits"])


def test_global_sample_matches_oracle(ctx, global_wl):
    """C3: uniform particles over the whole building (the spread-cloud order)."""
    parts = np.ascontiguousarray(global_wl.particles[:: global_wl.particles.shape[0] // SAMPLE][:SAMPLE])
    ext = parts[:, :2].max(0) - parts[:, :2].min(0)
    assert ext.max() > 10.0   # the spread-cloud scan order
    _check_against_oracle(ctx, global_wl, parts, serial_n=500)


def test_global_resample_of_device_weights(ctx, global_wl):
    """C3's step: all 1,000,000 particles scored, then systematic resampling of
    the device's normalised weights, bit for bit against the oracle."""
    dmap = DeviceMap(ctx, global_wl.coef, global_wl.grid_occ, codes=global_wl.codes, dense=True)
    p = global_wl.particles.copy()
    TSDFEvaluator(dmap).evaluate(p, global_wl.points, global_wl.tf)
    w = np.ascontiguousarray(p[:, 6])
    rs = SystematicResampler(ctx, seed=5)
    for u0 in (rs.draw(w.shape[0]), 0.0, float(np.float32(0.5e-6))):
        got = rs.resample_indices(w, u0)
        assert np.array_equal(got, O.resample_systematic(w, u0))


@pytest.mark.parametrize("kind", ["c3", "mixed"])
def test_resample_1m_tiny_weights(ctx, kind):
    """1,000,000 weights, most of them below 2^-29: the serial double sums round,
    and the device forms them binade by binade."""
    m = 1_000_000
    rng = np.random.default_rng(77 if kind == "c3" else 78)
    if kind == "c3":   # 999,000 misses and 1,000 particles on the surface
        w = np.ones(m)
        w[rng.choice(m, 1000, replace=False)] = 1e6 * (1 + rng.random(1000))
    else:
        w = rng.random(m)
        w[rng.random(m) < 0.6] *= 1e-5
    w = (w / w.sum()).astype(np.float32)
    assert (w < 2.0 ** -29).mean() > 0.5
    rs = SystematicResampler(ctx, seed=m)
    for u0 in (rs.draw(m), 0.0, float(np.nextafter(np.float32(1.0 / m), np.float32(0)))):
        got = rs.resample_indices(w, u0)
        exp = O.resample_systematic(w, u0)
        assert got.shape == exp.shape
        assert np.array_equal(got, exp)


@pytest.mark.parametrize("k", [256, 2048])
def test_global_subsampled_matches_oracle(ctx, global_wl, k):
    """C3's variant: every particle scores 256 of the 2,048 points, chosen per
    particle and seed (k = 2048 keeps every point: the full update's sums);
    hit counts bit-exact, weights within 1e-5 of FP64 and never farther from
    it than the reference-order float sums."""
    n = 2000
    parts = np.ascontiguousarray(global_wl.particles[:: global_wl.particles.shape[0] // n][:n])
    dmap = DeviceMap(ctx, global_wl.coef, global_wl.grid_occ, codes=global_wl.codes, dense=True)
    om = O.OracleMap(O.coef_from(global_wl.coef), global_wl.grid_occ, global_wl.float_data())
    seed = 20250
    ref = O.evaluate_subsampled(om, parts, global_wl.points, global_wl.tf, k, seed)
    p = parts.copy()
    pose, raw, hits = TSDFEvaluator(dmap).evaluate_subsampled(p, global_wl.points, global_wl.tf, k, seed, debug=True)
    assert np.array_equal(hits, ref["hits"])
    f64 = ref["sum64"]
    err_gpu = np.abs(raw.astype(np.float64) - f64)
    err_ref = np.abs(ref["raw"].astype(np.float64) - f64)
    assert np.all(err_gpu <= WEIGHT_RTOL * f64)
    assert np.all(err_gpu <= err_ref + WEIGHT_RTOL * f64)
    w64 = f64 / f64.sum()
    assert np.all(np.abs(p[:, 6].astype(np.float64) - w64) <= WEIGHT_RTOL * w64)
    if k == global_wl.points.shape[0]:   # every point kept: the full update's sums
        d = TSDFEvaluator(dmap).evaluate_debug(parts.copy(), global_wl.points, global_wl.tf)
        assert np.array_equal(d["raw"], raw) and np.array_equal(d["hits"], hits)
    # the device form gives the same weights
    import torch
    dp = torch.from_numpy(parts.copy()).cuda()
    dpts = torch.from_numpy(global_wl.points).cuda()
    dpose = torch.zeros(8, dtype=torch.float32, device="cuda")
    import ctypes as C
    from tsdf_localization_gb300 import _native as N
    tf = np.ascontiguousarray(global_wl.tf, np.float32)
    model = N.Model(0.9, 0.1, 0.0, 100.0)
    torch.cuda.synchronize()
    N.check(N.lib().tsdfl_evaluate_subsampled_device(ctx.handle, dmap.handle, C.byref(model),
                                                     C.c_void_p(dp.data_ptr()), n, C.c_void_p(dpts.data_ptr()),
                                                     global_wl.points.shape[0], tf.ctypes.data_as(C.c_void_p), k,
                                                     seed, C.c_void_p(dpose.data_ptr())))
    ctx.sync()
    assert np.array_equal(dp.cpu().numpy()[:, 6], p[:, 6])
    assert np.array_equal(dpose.cpu().numpy()[:6], pose)


def test_building_f16_storage_accuracy(ctx, building):
    """The half-precision storage variant on C2's map: the same slots are hit
    (indices do not depend on storage), and the weights stay within the
    half-precision bound of FP64 -- an accuracy line, not the 1e-5 bar."""
    parts = np.ascontiguousarray(building.particles[:: building.particles.shape[0] // 1000][:1000])
    dmap = DeviceMap(ctx, building.coef, building.grid_occ, codes=building.codes, f16=True)
    assert dmap.info()["storage"] == 2
    om = O.OracleMap(O.coef_from(building.coef), building.grid_occ, building.float_data())
    ref = O.evaluate(om, parts.copy(), building.points, building.tf)
    p = parts.copy()
    d = TSDFEvaluator(dmap).evaluate_debug(p, building.points, building.tf)
    assert np.array_equal(d["hits"], ref["hits"])
    rel = np.abs(d["raw"].astype(np.float64) - ref["sum64"]) / ref["sum64"]
    assert rel.max() <= 2.0 ** -10
    assert rel.max() > 1e-7   # the rounding is visible: it is a different storage
    with pytest.raises(Exception):   # serial sums need exact slot values
        TSDFEvaluator(dmap, serial_sums=True).evaluate(parts.copy(), building.points, building.tf)


def test_building_log_domain_normaliser(ctx, building):
    """TSDFL_NORM_LOG on C2's sample: the log-sum-exp weights are the linear
    ones up to the final float rounding, and within 1e-5 of FP64."""
    parts = np.ascontiguousarray(building.particles[:: building.particles.shape[0] // 2000][:2000])
    dmap = DeviceMap(ctx, building.coef, building.grid_occ, codes=building.codes, dense=True)
    om = O.OracleMap(O.coef_from(building.coef), building.grid_occ, building.float_data())
    ref = O.evaluate(om, parts.copy(), building.points, building.tf)
    w64 = ref["sum64"] / ref["sum64"].sum()
    p_lin, p_log = parts.copy(), parts.copy()
    TSDFEvaluator(dmap).evaluate(p_lin, building.points, building.tf)
    pose = TSDFEvaluator(dmap, log_normalise=True).evaluate(p_log, building.points, building.tf)
    assert pose is not None
    assert np.all(np.abs(p_log[:, 6].astype(np.float64) - w64) <= WEIGHT_RTOL * w64)
    rel = np.abs(p_log[:, 6].astype(np.float64) - p_lin[:, 6]) / p_lin[:, 6]
    assert rel.max() <= 4 * 2.0 ** -24
