"""The oracle (CPU restatement) against the reference's own outputs recorded in
tests/golden/reference_cases.npz (made by tests/golden/make_golden.py from the
reference sources compiled here): map construction, getEntry, the serial
sensor update, laser poses and systematic resampling, bit for bit."""
import hashlib
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle_py as O

GOLD = np.load(Path(__file__).resolve().parent / "golden" / "reference_cases.npz")
MAPS = ["map_0064", "map_005"]
SETS = sorted({k.split("/")[1] for k in GOLD.files if k.startswith("resample/")})


def oracle_map(name):
    return O.OracleMap.from_tuples(GOLD[f"{name}/mn"], GOLD[f"{name}/mx"], float(GOLD[f"{name}/res"]), 0.0,
                                   GOLD[f"{name}/tuples"])


@pytest.mark.parametrize("name", MAPS)
def test_map_build_matches_reference(name):
    om = oracle_map(name)
    assert bytes(om.coef) == GOLD[f"{name}/coef"].tobytes()
    assert np.array_equal(om.grid_occ, GOLD[f"{name}/grid_occ"])
    assert hashlib.sha256(om.data.tobytes()).digest() == GOLD[f"{name}/data_sha256"].tobytes()
    assert np.array_equal(om.data[GOLD[f"{name}/data_sample_idx"]], GOLD[f"{name}/data_sample"])


@pytest.mark.parametrize("name", MAPS)
def test_get_entry_matches_reference(name):
    om = oracle_map(name)
    got = np.array([om.get_entry(*p) for p in GOLD[f"{name}/query"]], np.float32)
    assert np.array_equal(got, GOLD[f"{name}/entries"], equal_nan=True)


@pytest.mark.parametrize("name", MAPS)
def test_sensor_update_matches_reference(name):
    om = oracle_map(name)
    parts = GOLD[f"{name}/particles"].copy()
    r = O.evaluate(om, parts, GOLD[f"{name}/points"], GOLD[f"{name}/tf"])
    assert r["rc"] == 0
    assert np.array_equal(r["raw"], GOLD[f"{name}/raw"])
    assert np.array_equal(parts[:, 6], GOLD[f"{name}/weights"])
    lp = np.stack([O.particle_pose(p, GOLD[f"{name}/tf"]) for p in GOLD[f"{name}/particles"]])
    assert np.array_equal(lp, GOLD[f"{name}/laser_pose"])
    assert np.allclose(r["pose"], GOLD[f"{name}/pose"], rtol=0, atol=1e-6)


@pytest.mark.parametrize("wset", SETS)
def test_resample_matches_reference(wset):
    w = GOLD[f"resample/{wset}/weights"]
    got = O.resample_systematic(w, float(GOLD[f"resample/{wset}/u0"]))
    assert np.array_equal(got, GOLD[f"resample/{wset}/indices"])


@pytest.mark.skipif(not O.reference_available(), reason="reference not compiled on this machine")
def test_fixture_draws_match_reference_generator():
    for wset in SETS:
        assert np.float32(O.ref_draw_u0(int(GOLD[f"resample/{wset}/seed"]), GOLD[f"resample/{wset}/weights"].shape[0])) \
            == GOLD[f"resample/{wset}/u0"]


@pytest.mark.parametrize("wset", SETS)
def test_residual_resample_matches_reference(wset):
    w = GOLD[f"resample/{wset}/weights"]
    got = O.resample_residual_systematic(w, float(GOLD[f"residual/{wset}/u0"]))
    assert np.array_equal(got, GOLD[f"residual/{wset}/indices"])


@pytest.mark.skipif(not O.reference_available(), reason="reference not compiled on this machine")
def test_residual_resample_random_weights_match_reference():
    """Beyond the fixtures: 100 random weight vectors and seeds."""
    rng = np.random.default_rng(5)
    for _ in range(100):
        m = int(rng.integers(1, 2000))
        w = (lambda x: (x / x.sum()).astype(np.float32))(rng.random(m) ** 4 + 1e-9)
        seed = int(rng.integers(1, 2 ** 31))
        assert np.array_equal(O.resample_residual_systematic(w, O.ref_draw_u01(seed), cap=4 * m + 16),
                              O.ref_resample_residual_systematic(w, seed, cap=4 * m + 16))


SCANS = sorted({k.rsplit("/", 1)[0] for k in GOLD.files if k.startswith("scan/")})


@pytest.mark.parametrize("case", SCANS)
def test_scan_reduction_matches_reference(case):
    got = O.reduce_scan(GOLD[f"{case}/xyz"], GOLD[f"{case}/ring"], float(GOLD[f"{case}/cell"]))
    assert np.array_equal(got, GOLD[f"{case}/reduced"], equal_nan=True)


def test_scan_reduction_random_clouds_match_reference():
    if not O.reference_available():
        pytest.skip("the reference sources are not on this machine")
    rng = np.random.default_rng(21)
    for t in range(30):
        n = int(rng.integers(1, 3000))
        x = rng.normal(0, 3, (n, 3)).astype(np.float32)
        x[rng.random(n) < 0.05] = np.nan
        x[rng.random(n) < 0.1] *= np.float32(0.1)
        if t % 3 == 0:
            x = (np.round(x * 8) / 8).astype(np.float32)
        r = rng.integers(0, 64, n).astype(np.int16)
        cell = float(rng.choice([0.05, 0.064, 0.2]))
        assert np.array_equal(O.reduce_scan(x, r, cell), O.ref_reduce_scan(x, r, cell), equal_nan=True)


def test_scan_reduction_ring_skip_and_errors():
    # the k-th kept point takes the ring of the k-th cloud point
    xyz = np.array([[0.1, 0, 0], [2, 0, 0], [2, 0, 0]], np.float32)
    ring = np.array([5, 3, 63], np.int16)
    got = O.reduce_scan(xyz, ring, 0.1)         # kept: #1 -> ring 5, #2 -> ring 3 (different rings)
    assert got.shape == (2, 3)
    assert O.reduce_scan(xyz, ring, 0.1, own_ring=True).shape == (2, 3)
    ring2 = np.array([7, 7, 63], np.int16)      # both kept points get ring 7: one survives
    assert O.reduce_scan(xyz, ring2, 0.1).shape == (1, 3)
    assert O.reduce_scan(xyz, ring2, 0.1, own_ring=True).shape == (2, 3)
    with pytest.raises(ValueError):
        O.reduce_scan(xyz, np.array([64, 0, 0], np.int16), 0.1)
    assert O.reduce_scan(np.zeros((0, 3), np.float32), np.zeros(0, np.int16), 0.1).shape == (0, 3)


def test_motion_composition_matches_reference():
    parts, deltas, moved = GOLD["motion/particles"], GOLD["motion/deltas"], GOLD["motion/moved"]
    for d, want in zip(deltas, moved):
        got = O.motion_apply(parts, np.tile(d.astype(np.float64), (parts.shape[0], 1)))
        assert np.array_equal(got, want)


def test_motion_composition_random_matches_reference():
    if not O.reference_available():
        pytest.skip("the reference sources are not on this machine")
    rng = np.random.default_rng(23)
    P = 5000
    parts = np.zeros((P, 7), np.float32)
    parts[:, :3] = rng.uniform(-100, 100, (P, 3))
    parts[:, 3:6] = rng.uniform(-np.pi, np.pi, (P, 3))
    parts[:50, 4] = np.float32(np.pi / 2)
    parts[:, 6] = rng.random(P)
    for _ in range(15):
        d = rng.normal(0, [0.5, 0.2, 0.1, 0.1, 0.1, 0.5]).astype(np.float32)
        assert np.array_equal(O.motion_apply(parts, np.tile(d.astype(np.float64), (P, 1))),
                              O.ref_motion_update(parts, d))


def test_philox_restatement_matches_numpy():
    for key in ((0, 0), (12345, 0x6D6F74696F6E0001), (2 ** 64 - 1, 7)):
        g = np.random.Philox(key=np.array(key, np.uint64), counter=np.zeros(4, np.uint64))
        raw = g.random_raw(12)
        # numpy advances the counter before each block: blocks 1, 2, 3
        for b in range(3):
            got = O.philox4x64_10([np.uint64(b + 1), np.uint64(0), np.uint64(0), np.uint64(0)], key)
            assert [int(v) for v in got] == [int(v) for v in raw[4 * b:4 * b + 4]]


OTHERS = sorted({k.split("/")[1] for k in GOLD.files if k.startswith("others/") and k.count("/") == 2})


@pytest.mark.parametrize("wset", OTHERS)
def test_other_resamplers_match_reference(wset):
    g = lambda name: GOLD[f"others/{wset}/{name}"]  # noqa: E731
    w = g("weights")
    assert np.array_equal(O.resample_wheel(w, g("wheel_draws")), g("wheel"))
    idx, used = O.resample_residual(w, g("residual_draws"))
    assert np.array_equal(idx, g("residual")) and used == g("residual_draws").shape[0]
    assert np.array_equal(O.resample_metropolis(w, int(GOLD["others/steps"]), g("metropolis_u"), g("metropolis_j")),
                          g("metropolis"))
    assert np.array_equal(O.resample_rejection_arrays(w, g("rejection_u"), g("rejection_j")), g("rejection"))


def test_other_resamplers_random_weights_match_reference():
    if not O.reference_available():
        pytest.skip("the reference sources are not on this machine")
    rng = np.random.default_rng(31)
    for M in (1, 2, 50, 1500):
        for t in range(3):
            w = (rng.random(M) ** (1 + 4 * t)).astype(np.float32)
            if t == 1:
                w /= w.sum()
            seed = int(rng.integers(1, 2 ** 31))
            assert np.array_equal(O.ref_resample("wheel", w, seed), O.resample_wheel(w, O.ref_draws("wheel", seed, M)))
            assert np.array_equal(O.ref_resample("residual", w, seed),
                                  O.resample_residual(w, O.ref_draws("residual", seed, M, K=100 * M + 100))[0])
            u, j = O.ref_draws("metropolis", seed, M, steps=50)
            assert np.array_equal(O.ref_resample("metropolis", w, seed), O.resample_metropolis(w, 50, u, j))
            assert np.array_equal(O.ref_resample("rejection", w, seed), O.resample_rejection_reference_draws(w, seed))
