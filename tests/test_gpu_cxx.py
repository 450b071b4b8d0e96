"""The C++ host layer (include/tsdfl_evaluator.hpp) on the GPU: built with g++
against include/ and libtsdfl, run on the room workload, its weights, pose and
resampled particles equal the Python binding's and the oracle's."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle_py as O
from tsdf_localization_gb300 import (Context, DeviceMap, MotionModel, SystematicResampler, TSDFEvaluator, pack_cloud,
                                     synth)

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def test_cxx_host_layer_matches_python_and_oracle(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    lib_dir = ROOT / "tsdf_localization_gb300" / "_lib"
    exe = tmp_path / "cxx_core_check"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "native" / "cxx_core_check.cpp"), "-o", str(exe),
                    "-L", str(lib_dir), "-ltsdfl", f"-Wl,-rpath,{lib_dir}"], check=True)
    wl = synth.room_workload(seed=21, n_particles=700, n_points=1500)
    data = wl.float_data()
    u0 = np.float32(0.37 / wl.particles.shape[0])
    (tmp_path / "coef.bin").write_bytes(bytes(wl.coef))
    wl.grid_occ.astype(np.int32).tofile(tmp_path / "grid_occ.bin")
    data.astype(np.float32).tofile(tmp_path / "data.bin")
    wl.particles.astype(np.float32).tofile(tmp_path / "particles.bin")
    wl.points.astype(np.float32).tofile(tmp_path / "points.bin")
    np.asarray(wl.tf, np.float32).tofile(tmp_path / "tf.bin")
    u1 = np.float32(0.618)
    np.array([u0, u1], np.float32).tofile(tmp_path / "u0.bin")
    cxyz, cring = synth.World(synth.ROOM, 21).scan(wl.true_pose, 16, 700, sigma=0.01, dropout=0.02, seed=8)
    cxyz[::37] *= np.float32(0.1)       # some returns inside 1 m
    pack_cloud(cxyz, cring).tofile(tmp_path / "cloud.bin")
    draws = np.random.default_rng(3).normal(0, [0.3, 0.1, 0.05, 0.05, 0.05, 0.3], (wl.particles.shape[0], 6))
    draws.tofile(tmp_path / "draws.bin")
    gold = np.load(ROOT / "tests" / "golden" / "reference_cases.npz")
    gold["others/random/weights"].astype(np.float32).tofile(tmp_path / "others_w.bin")
    np.array([gold["others/random/seed"]], np.uint32).tofile(tmp_path / "others_seed.bin")
    res = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=300)
    print(res.stdout, res.stderr)
    assert res.returncode == 0, res.stdout + res.stderr
    w_cxx = np.fromfile(tmp_path / "weights_out.bin", np.float32)
    pose_cxx = np.fromfile(tmp_path / "pose_out.bin", np.float32)
    rs_cxx = np.fromfile(tmp_path / "resampled_out.bin", np.float32).reshape(-1, 7)
    rr_cxx = np.fromfile(tmp_path / "residual_out.bin", np.float32).reshape(-1, 7)

    ctx = Context(0)
    dmap = DeviceMap(ctx, wl.coef, wl.grid_occ, data=data)
    p = wl.particles.copy()
    pose = TSDFEvaluator(dmap).evaluate(p, wl.points, wl.tf)
    assert np.array_equal(w_cxx, p[:, 6])
    assert np.array_equal(pose_cxx, pose.as_array())
    idx = SystematicResampler(ctx).resample_indices(p[:, 6], float(u0))
    assert np.array_equal(rs_cxx, p[idx])

    om = O.OracleMap(O.coef_from(wl.coef), wl.grid_occ, data)
    ref = O.evaluate(om, wl.particles.copy(), wl.points, wl.tf)
    f64 = ref["sum64"] / ref["sum64"].sum()
    assert np.all(np.abs(w_cxx.astype(np.float64) - f64) <= 1e-5 * f64)
    assert np.array_equal(idx, O.resample_systematic(p[:, 6], float(u0)))
    ridx = O.resample_residual_systematic(p[:, 6], float(u1))
    assert np.array_equal(rr_cxx, p[ridx])

    red = np.fromfile(tmp_path / "reduced_out.bin", np.float32).reshape(-1, 3)
    want = O.reduce_scan(cxyz, cring, 0.064)
    assert np.array_equal(red, want)
    pc = wl.particles.copy()
    TSDFEvaluator(dmap).evaluate(pc, want, wl.tf)
    assert np.array_equal(np.fromfile(tmp_path / "cloud_weights_out.bin", np.float32), pc[:, 6])

    moved = np.fromfile(tmp_path / "motion_apply_out.bin", np.float32).reshape(-1, 7)
    assert np.array_equal(moved, O.motion_apply(wl.particles, draws))
    mm = MotionModel(ctx, seed=42)
    pm = wl.particles.copy()
    mm.update(pm, mm.distributions("odom", [0.6, -0.3], 0.1), step=0)
    assert np.array_equal(np.fromfile(tmp_path / "motion_update_out.bin", np.float32).reshape(-1, 7), pm)

    # Wheel, Residual, Metropolis from a seeded std::mt19937: the reference's particles
    for kind, name in enumerate(("wheel", "residual", "metropolis")):
        got = np.fromfile(tmp_path / f"others_out_{kind}.bin", np.uint32)
        assert np.array_equal(got[:-1], gold[f"others/random/{name}"])
        assert got[-1] == gold["others/random/generator_next"][kind]   # the generator left where the reference leaves it
