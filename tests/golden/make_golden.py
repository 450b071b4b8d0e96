"""Generates the golden fixtures in this directory from the reference's own
sources compiled here (oracle/_ref/libref.so, built by __graft_entry__.build()
when the reference tree is present).

Each case stores its inputs in full (map tuples, bounds, resolution, particles,
points, sensor transform, query points, weight vectors, generator seeds) and
what the reference computes from them: the map's coefficients and brick table
and a digest of its slots (CudaSubVoxelMap ctor + setData), getEntry at the
query points, TSDFEvaluator::evaluate's un-normalised and normalised weights,
laser poses and mean pose (serial, in point order), SystematicResampler's
and ResidualSystematicResampler's output indices for seeded draws, and the
point list TSDFEvaluator::evaluateParticles' scan reduction hands to evaluate
for a set of clouds (x, y, z, ring), and the particles ParticleCloud's motion
model produces from given increments (motion_update with zero noise), and the
Wheel, Residual, Metropolis and Rejection resamplers' outputs with the draws
they took from a seeded generator.

    python tests/golden/make_golden.py
"""
import hashlib
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle_py as O  # noqa: E402

OUT = Path(__file__).resolve().parent


def _pose_tf(rng):
    a, b, c = rng.uniform(-0.3, 0.3, 3)
    ca, sa, cb, sb, cc, sc = np.cos(a), np.sin(a), np.cos(b), np.sin(b), np.cos(c), np.sin(c)
    R = np.array([[cc * cb, cc * sb * sa - sc * ca, cc * sb * ca + sc * sa],
                  [sc * cb, sc * sb * sa + cc * ca, sc * sb * ca - cc * sa],
                  [-sb, cb * sa, cb * ca]])
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = rng.uniform(-0.2, 0.2, 3)
    return T.astype(np.float32).reshape(16)


def map_case(name, res, mn, mx, n_tuples, seed):
    rng = np.random.default_rng(seed)
    mn = np.asarray(mn, np.float32)
    mx = np.asarray(mx, np.float32)
    xyz = rng.uniform(mn, mx, size=(n_tuples, 3)).astype(np.float32)
    xyz[: n_tuples // 10] = xyz[n_tuples // 10: 2 * (n_tuples // 10)] + rng.normal(0, res / 4, (n_tuples // 10, 3))
    vals = rng.uniform(0.001, 63.0, n_tuples).astype(np.float32)
    tuples = np.concatenate([xyz, vals[:, None]], 1).astype(np.float32)
    rm = O.RefMap(mn, mx, res, 0.0, tuples)
    data = rm.data()
    centre = (mn + mx) / 2
    span = mx - mn
    q = np.concatenate([
        rng.uniform(mn - 1.5, mx + 1.5, size=(300, 3)),
        xyz[rng.choice(n_tuples, 200, replace=False)],
        mn + rng.uniform(-1.0, 0.3, size=(100, 3)),
        np.array([[np.nan, 0, 0], [1e20, 0, 0], [-1e20, 0, 0], [0, 0, np.inf]]) + mn,
    ]).astype(np.float32)
    entries = np.array([rm.get_entry(*p) for p in q], np.float32)
    P = 48
    parts = np.zeros((P, 7), np.float32)
    parts[:, :3] = centre + rng.normal(0, 0.3, (P, 3))
    parts[:, 3:6] = rng.normal(0, 0.08, (P, 3))
    parts[:, 5] += rng.uniform(-3.1, 3.1)
    parts[:, 6] = 1.0 / P
    dirs = rng.normal(size=(300, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    pts = (dirs * rng.uniform(0.3, 0.6 * span.min(), (300, 1))).astype(np.float32)
    pts[::37] *= 500.0   # beyond max_range and outside the map
    tf = _pose_tf(rng)
    p_ref = parts.copy()
    r = rm.evaluate(p_ref, pts, tf, serial=True)
    assert r["rc"] == 0
    return {
        f"{name}/tuples": tuples, f"{name}/mn": mn, f"{name}/mx": mx, f"{name}/res": np.float32(res),
        f"{name}/coef": np.frombuffer(bytes(rm.coef), np.uint8), f"{name}/grid_occ": rm.grid_occ(),
        f"{name}/data_sha256": np.frombuffer(hashlib.sha256(data.tobytes()).digest(), np.uint8),
        f"{name}/data_sample_idx": (idx := rng.choice(max(data.size, 1), 500)).astype(np.int64),
        f"{name}/data_sample": data[idx] if data.size else np.zeros(500, np.float32),
        f"{name}/query": q, f"{name}/entries": entries,
        f"{name}/particles": parts, f"{name}/points": pts, f"{name}/tf": tf,
        f"{name}/raw": r["raw"], f"{name}/weights": p_ref[:, 6].copy(), f"{name}/laser_pose": r["laser_pose"],
        f"{name}/pose": r["pose"],
    }


def resample_case(seed):
    rng = np.random.default_rng(seed)
    out = {}
    sets = {
        "uniform": np.full(1000, 1.0 / 1000, np.float32),
        "random": (lambda w: (w / w.sum()).astype(np.float32))(rng.random(2500) ** 3),
        "sparse": (lambda w: (w / w.sum()).astype(np.float32))(np.where(rng.random(3000) < 0.05, rng.random(3000), 0.0)),
        "tiny": (lambda w: (w / w.sum()).astype(np.float32))(np.exp(-rng.uniform(0, 40, 4000))),
        "unnormalised": rng.uniform(0.0, 2.0 / 700, 700).astype(np.float32),
    }
    for k, w in sets.items():
        s = int(rng.integers(1, 2 ** 31))
        out[f"resample/{k}/weights"] = w
        out[f"resample/{k}/seed"] = np.int64(s)
        out[f"resample/{k}/u0"] = np.float32(O.ref_draw_u0(s, w.shape[0]))
        out[f"resample/{k}/indices"] = O.ref_resample_systematic(w, s)
        s2 = int(rng.integers(1, 2 ** 31))
        out[f"residual/{k}/seed"] = np.int64(s2)
        out[f"residual/{k}/u0"] = np.float32(O.ref_draw_u01(s2))
        out[f"residual/{k}/indices"] = O.ref_resample_residual_systematic(w, s2)
    return out


def scan_cloud(kind, rng):
    """A cloud (xyz float32, ring int16) of one of several kinds."""
    if kind == "lidar":
        # 16 rings x 200 columns on walls 2-9 m away, some returns inside 1 m
        rings, cols = 16, 200
        el = np.deg2rad(np.linspace(-15, 15, rings))[:, None]
        az = np.linspace(-np.pi, np.pi, cols, endpoint=False)[None, :]
        r = rng.uniform(2.0, 9.0, (rings, cols))
        r[rng.random((rings, cols)) < 0.05] = rng.uniform(0.2, 1.2, 1)[0]
        xyz = np.stack([r * np.cos(el) * np.cos(az), r * np.cos(el) * np.sin(az), r * np.sin(el)], -1)
        ring = np.broadcast_to(np.arange(rings)[:, None], (rings, cols))
        # column-major order, as a spinning sensor emits it
        return xyz.transpose(1, 0, 2).reshape(-1, 3).astype(np.float32), ring.T.reshape(-1).astype(np.int16)
    if kind == "dense":
        # many points per cell and ring: the first per (ring, cell) survives
        d = rng.normal(0, 1, (2000, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        xyz = d * rng.uniform(1.0, 1.6, (2000, 1))
        xyz = (np.round(xyz * 4) / 4 + 0.025 + rng.uniform(-0.004, 0.004, xyz.shape)).astype(np.float32)
        return xyz, rng.integers(0, 2, 2000).astype(np.int16)
    if kind == "edge":
        # points at |p| ~ 1 m, non-finite values, large and negative coordinates
        n = 1500
        d = rng.normal(0, 1, (n, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        xyz = (d * rng.choice([0.9999999, 1.0, 1.0000001, 1.5, 40.0], (n, 1))).astype(np.float32)
        xyz[rng.random(n) < 0.03, 0] = np.nan
        xyz[rng.random(n) < 0.01, 1] = np.inf
        xyz[rng.random(n) < 0.01, 2] = -np.inf
        big = rng.random(n) < 0.05
        xyz[big] = rng.uniform(-3e6, 3e6, (big.sum(), 3)).astype(np.float32)
        xyz[:50] = xyz[50:100]            # exact duplicates of other points
        return xyz, rng.integers(0, 64, n).astype(np.int16)
    raise ValueError(kind)


def scan_case(seed):
    rng = np.random.default_rng(seed)
    out = {}
    for kind, cell in (("lidar", 0.064), ("lidar", 0.25), ("dense", 0.05), ("edge", 0.064), ("edge", 0.5)):
        xyz, ring = scan_cloud(kind, rng)
        key = f"scan/{kind}_{int(round(cell * 1000)):04d}"
        out[f"{key}/xyz"] = xyz
        out[f"{key}/ring"] = ring
        out[f"{key}/cell"] = np.float32(cell)
        out[f"{key}/reduced"] = O.ref_reduce_scan(xyz, ring, cell)
    return out


def motion_case(seed):
    rng = np.random.default_rng(seed)
    P = 600
    parts = np.zeros((P, 7), np.float32)
    parts[:, :3] = rng.uniform(-60, 60, (P, 3))
    parts[:, 3:5] = rng.uniform(-0.6, 0.6, (P, 2))
    parts[:, 5] = rng.uniform(-np.pi, np.pi, P)
    parts[:40, 4] = np.float32(np.pi / 2)       # getAngleFromMat's |m[8]| >= 1 branch
    parts[40:80, 4] = -np.float32(np.pi / 2)
    parts[:, 6] = rng.random(P)
    deltas = np.array([[0, 0, 0, 0, 0, 0],
                       [0.35, -0.02, 0.01, 0.004, -0.003, 0.12],
                       [-1.2, 0.4, -0.3, 0.3, -0.25, -2.9]], np.float32)
    out = {"motion/particles": parts, "motion/deltas": deltas}
    out["motion/moved"] = np.stack([O.ref_motion_update(parts, d) for d in deltas])
    return out


def other_resamplers_case(seed):
    rng = np.random.default_rng(seed)
    M, steps = 300, 10
    sets = {
        "random": (lambda w: (w / w.sum()).astype(np.float32))(rng.random(M) ** 3),
        "sparse": (lambda w: (w / w.sum()).astype(np.float32))(np.where(rng.random(M) < 0.1, rng.random(M) + 0.01,
                                                                        0.0)),
        "unnormalised": rng.uniform(0.0, 1.6 / M, M).astype(np.float32),
    }
    out = {}
    for k, w in sets.items():
        s = int(rng.integers(1, 2 ** 31))
        key = f"others/{k}"
        out[f"{key}/weights"] = w
        out[f"{key}/seed"] = np.int64(s)
        out[f"{key}/wheel_draws"] = O.ref_draws("wheel", s, M)
        out[f"{key}/wheel"] = O.ref_resample("wheel", w, s)
        draws = O.ref_draws("residual", s, M, K=50 * M)
        _, used = O.resample_residual(w, draws)
        out[f"{key}/residual_draws"] = draws[:used]
        out[f"{key}/residual"] = O.ref_resample("residual", w, s)
        u, j = O.ref_draws("metropolis", s, M, steps=steps)
        out[f"{key}/metropolis_u"], out[f"{key}/metropolis_j"] = u, j
        out[f"{key}/metropolis"] = O.ref_resample("metropolis", w, s, steps=steps)
        nu, nj, close = O.ref_rejection_draw_callables(s, M)
        idx, uu, jj = O.resample_rejection_arrays(w, nu, nj, record=True)
        close()
        out[f"{key}/rejection_u"], out[f"{key}/rejection_j"] = uu, jj
        out[f"{key}/rejection"] = O.ref_resample("rejection", w, s)
        assert np.array_equal(idx, out[f"{key}/rejection"])
        out[f"{key}/generator_next"] = np.array([O.ref_resample_next(kind, w, s, steps) for kind in range(3)],
                                                np.uint32)
    out["others/steps"] = np.int64(steps)
    return out


def main():
    if not O.reference_available():
        raise SystemExit("oracle/_ref/libref.so is not built: the reference tree is needed")
    fx = {}
    fx.update(map_case("map_0064", 0.064, (-1.3, -0.7, -0.45), (5.1, 4.3, 2.6), 6000, 11))
    fx.update(map_case("map_005", 0.05, (0.0, 0.0, 0.0), (4.2, 3.6, 2.2), 6000, 12))
    fx.update(resample_case(13))
    fx.update(scan_case(14))
    fx.update(motion_case(15))
    fx.update(other_resamplers_case(16))
    np.savez_compressed(OUT / "reference_cases.npz", **fx)
    print("wrote", OUT / "reference_cases.npz", (OUT / "reference_cases.npz").stat().st_size, "bytes")


if __name__ == "__main__":
    main()
