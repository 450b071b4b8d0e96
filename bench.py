"""Benchmark of the MCL sensor update: scored particle*points per second.

Workload (default): one filter of 100,000 particles (Gaussian, sigma 0.3 m / 5 deg)
x 8,192 scan points (64x2048 ray-cast, sigma 0.02 m, 1 % dropouts, reduced and
subsampled) in a seeded 100x100x10 m building mapped at 0.05 m.  One step = one
sensor update (transform, lookup, score, per-particle sum, normalisation, mean
pose) plus one systematic resampling, on the same particle poses every step as
the reference's own timing loop does (num_particles_eval.cpp:237-257).

Arms:
  default            libtsdfl on cuda (device-resident inputs) + e2e through the
                     host C ABI + roofline of the scoring kernel + CPU baseline
  --impl reference   the reference's CPU sensor update (its own sources where
                     they were compiled on this machine, else the CPU
                     restatement) on a bounded sample of the same workload
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "scored particle\u00b7points/s at 100k\u00d78k (vs plain); p50/p99 update latency served"
UNIT = "particle\u00b7points/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="building", choices=["building", "room", "global", "batch", "served"])
    ap.add_argument("--sessions", type=int, default=256, help="robots of the served workload")
    ap.add_argument("--seconds", type=float, default=3.0, help="arrival window of the served workload")
    ap.add_argument("--max-wait-ms", type=float, default=4.0, help="admission bound of the served workload")
    ap.add_argument("--filters", type=int, default=64, help="filters of the batch workload")
    ap.add_argument("--particles", type=int, default=None)
    ap.add_argument("--points", type=int, default=None)
    ap.add_argument("--layout", default="compact", choices=["compact", "grid", "brick"])
    ap.add_argument("--kernel", default="fast", choices=["fast", "generic"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-scan", action="store_true", help="skip the scan-reduction and motion side measurements")
    ap.add_argument("--no-sub", action="store_true",
                    help="skip the global-localisation, batched and served measurements of the default run")
    ap.add_argument("--batch-steps", type=int, default=20, help="graph replays timed by the batched measurement")
    ap.add_argument("--served-seconds", type=float, default=2.0, help="arrival window of the served measurement")
    return ap.parse_args()


def make_workload(args):
    from tsdf_localization_gb300 import synth
    if args.workload == "room":
        wl = synth.room_workload(seed=1, n_particles=args.particles or 1000, n_points=args.points or 2048)
    elif args.workload == "global":
        wl = synth.global_workload(seed=3, n_particles=args.particles or 1_000_000, n_points=args.points or 2048)
    else:
        wl = synth.building_workload(seed=2, n_particles=args.particles or 100_000, n_points=args.points or 8192)
    return wl


# DRAM bytes of one scoring launch from ncu captures of these exact workloads
# (dram__bytes_read.sum + dram__bytes_write.sum, single pass, full size;
# profiles/eval_tiled_kernel_building_20k_x_8192.md and
# profiles/eval_tiled_kernel_global_1m_x_2048.md)
MEASURED_TRAFFIC = {("building", 100_000, 8192, "compact", "fast"): 1.326252e9 + 0.054576e9,
                    ("global", 1_000_000, 2048, "compact", "fast"): 64.449552e9 + 0.189430e9}


def roofline_bytes(P: int, N: int, layout: str) -> float:
    """Algorithmic bytes of one scoring launch: per particle*point the map
    reads (brick layout: 4 B brick-table entry + 2 B slot code; compact layout:
    the 2 B slot code, its brick rank coming from shared memory), per particle
    56 B (pose in, weight, index, pose out), per point 12 B."""
    bpp = 2 if layout == "compact" else 6
    return float(bpp) * P * N + 56.0 * P + 12.0 * N


def measured_peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        fd, name = tempfile.mkstemp(prefix="tsdfl_clocks_", suffix=".csv")
        os.close(fd)
        self.path = Path(name)

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self) -> dict:
        if not self.proc or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "1"):
                    reasons.add(nm)
        try:
            self.path.unlink()
        except Exception:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(wl, target_s: float = 10.0) -> dict:
    """The reference CPU sensor update + resampling on a bounded particle sample."""
    from oracle import oracle_py as O
    kind = "reference" if O.reference_available() else "port"
    om = O.OracleMap(O.coef_from(wl.coef), wl.grid_occ, wl.float_data())
    N = wl.points.shape[0]
    if kind == "reference":
        rm = _reference_map(O, wl)
    P_s = min(wl.particles.shape[0], 512)
    rate = None
    while True:
        parts = wl.particles[:P_s].copy()
        t0 = time.perf_counter()
        if kind == "reference":
            r = rm.evaluate(parts, wl.points, wl.tf, serial=False)
            O.ref_resample_systematic(parts[:, 6], 1)
        else:
            r = O.evaluate(om, parts, wl.points, wl.tf)
            O.resample_systematic(parts[:, 6], float(np.float32(0.5 / P_s)))
        dt = time.perf_counter() - t0
        rate = P_s * N / dt
        if dt * 4 > target_s or P_s >= wl.particles.shape[0]:
            break
        P_s = min(wl.particles.shape[0], int(P_s * max(2.0, target_s / max(dt, 1e-3) / 2)))
    cores = os.cpu_count() or 1
    return {"value": rate, "unit": UNIT, "cores": cores, "kind": kind,
            "sample": f"{P_s} particles x {N} points, one update + resample, {dt:.2f} s"}, (P_s, kind, om,
                                                                                             rm if kind == "reference" else None)


def accuracy_vs_fp64(om, wl, dmap, n: int = 4000) -> dict:
    """Errors of the device's weights against FP64 on a particle sample (every
    (P/n)-th particle of the step): the oracle scores the same particles with
    per-particle sums in double; the reference's own float sums are reported
    beside ours.  Also whether hit counts agree and the mean pose's distance
    from the FP64 mean."""
    from oracle import oracle_py as O
    from tsdf_localization_gb300 import TSDFEvaluator
    P = wl.particles.shape[0]
    parts = np.ascontiguousarray(wl.particles[:: max(1, P // n)][:n])
    ref = O.evaluate(om, parts.copy(), wl.points, wl.tf)
    p = parts.copy()
    d = TSDFEvaluator(dmap).evaluate_debug(p, wl.points, wl.tf)
    f64 = ref["sum64"]
    w64 = f64 / f64.sum()
    rel = np.abs(d["raw"].astype(np.float64) - f64) / f64
    rel_ref = np.abs(ref["raw"].astype(np.float64) - f64) / f64
    rel_w = np.abs(p[:, 6].astype(np.float64) - w64) / w64
    q = parts.astype(np.float64)
    mean64 = np.concatenate([(q[:, :3] * w64[:, None]).sum(0),
                             [np.arctan2((np.sin(q[:, k]) * w64).sum(), (np.cos(q[:, k]) * w64).sum())
                              for k in (3, 4, 5)]])
    out = {"particles": int(parts.shape[0]), "points": int(wl.points.shape[0]),
           "max_rel_raw_weight": float(rel.max()), "max_rel_normalised_weight": float(rel_w.max()),
           "reference_float_sum_max_rel": float(rel_ref.max()),
           "hits_equal_oracle": bool(np.array_equal(d["hits"], ref["hits"])),
           "mean_pose_max_abs_err": float(np.abs(d["pose"].astype(np.float64) - mean64).max()),
           "tolerance": 1e-5}
    # the half-precision storage variant on the same sample (an accuracy line)
    from tsdf_localization_gb300 import DeviceMap
    hmap = DeviceMap(dmap.ctx, wl.coef, wl.grid_occ, codes=wl.codes, f16=True)
    ph = parts.copy()
    dh = TSDFEvaluator(hmap).evaluate_debug(ph, wl.points, wl.tf)
    hmap.close()
    pl = parts.copy()
    TSDFEvaluator(dmap, log_normalise=True).evaluate(pl, wl.points, wl.tf)
    out["log_domain_normaliser"] = {"max_rel_normalised_weight":
                                    float((np.abs(pl[:, 6].astype(np.float64) - w64) / w64).max())}
    out["f16_storage"] = {"max_rel_raw_weight": float((np.abs(dh["raw"].astype(np.float64) - f64) / f64).max()),
                          "max_rel_normalised_weight":
                              float((np.abs(ph[:, 6].astype(np.float64) - w64) / w64).max()),
                          "hits_equal_oracle": bool(np.array_equal(dh["hits"], ref["hits"]))}
    return out


def _reference_map(O, wl):
    """The map loaded into the reference's own CudaSubVoxelMap."""
    return O.RefMap.from_slots(wl.coef, wl.grid_occ, wl.float_data())


def scan_reduction_side(lib, ctx, stream, wl, device: str, with_cpu: bool, reps: int = 20) -> dict:
    """Times the scan reduction (evaluateParticles' pre-processing) on the raw
    64 x 2048 ray-cast cloud the workload's points come from: the device form
    replayed from a CUDA graph of `reps` calls (CUDA events on the context's
    stream, so host launch costs are excluded), the host form (pageable cloud
    in, points out) with a host clock, and the oracle on one host core."""
    import torch

    from tsdf_localization_gb300 import _native as N
    from tsdf_localization_gb300 import pack_cloud, synth
    xyz, ring = synth.World(synth.BUILDING, 2).scan(wl.true_pose, 64, 2048, dropout=0.01, seed=2)
    n = int(xyz.shape[0])
    blob_h = pack_cloud(xyz, ring)
    blob = torch.from_numpy(blob_h).to(device)
    out = torch.empty((n, 3), dtype=torch.float32, device=device)
    cnt = torch.zeros(1, dtype=torch.int32, device=device)
    vp = C.c_void_p
    torch.cuda.synchronize()

    def dev():
        N.check(lib.tsdfl_reduce_scan_device(ctx.handle, vp(blob.data_ptr()), n, 16, 0, 12, 0.05, 0,
                                             vp(out.data_ptr()), n, vp(cnt.data_ptr())))

    with torch.cuda.stream(stream):
        for _ in range(5):
            dev()
        ctx.sync()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream):
            for _ in range(reps):
                dev()
        for _ in range(3):
            graph.replay()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(10):
            graph.replay()
        e1.record(stream)
        e1.synchronize()
        ctx.sync()
    m = int(cnt.item())
    ho = np.empty((n, 3), np.float32)
    hc = C.c_size_t()
    tt = []
    for _ in range(20):
        t0 = time.perf_counter()
        N.check(lib.tsdfl_reduce_scan(ctx.handle, blob_h.ctypes.data_as(vp), n, 16, 0, 12, 0.05, 0,
                                      ho.ctypes.data_as(vp), n, C.byref(hc)))
        tt.append(time.perf_counter() - t0)
    res = {"cloud": "64x2048 ray-cast, building at 0.05 m, 16-byte records", "raw_points": n, "reduced_points": m,
           "cell_m": 0.05, "device_us": 1000.0 * e0.elapsed_time(e1) / (10 * reps),
           "host_api_us": 1e6 * float(np.median(tt)), "launches_per_call": 6}
    if with_cpu:
        from oracle import oracle_py as O
        t0 = time.perf_counter()
        ref = O.reduce_scan(xyz, ring, 0.05)
        res["cpu_oracle_ms"] = 1000.0 * (time.perf_counter() - t0)
        res["matches_oracle"] = bool(np.array_equal(ho[:hc.value], ref))
    return res


def tracking_side(lib, ctx, stream, wl, dmap, device: str, updates: int) -> dict:
    """Consecutive filter steps on the device -- motion update (ParticleCloud's
    lin_scale/ang_scale overload, 1 m/s and 0.5 rad/s scales over 0.1 s), sensor
    update, systematic resampling into the other particle buffer -- for a robot
    at rest at the workload's true pose; the mean pose's and the best
    particle's errors against the true pose after every update."""
    import torch

    from tsdf_localization_gb300 import MotionModel
    from tsdf_localization_gb300 import _native as N
    vp = C.c_void_p
    P0 = int(wl.particles.shape[0])
    cap = 2 * P0 + 16
    bufs = [torch.zeros((cap, 7), dtype=torch.float32, device=device) for _ in range(2)]
    bufs[0][:P0].copy_(torch.from_numpy(wl.particles))
    d_pose = torch.zeros(8, dtype=torch.float32, device=device)
    d_cnt = torch.zeros(4, dtype=torch.int32, device=device)
    d_best = torch.zeros(4, dtype=torch.int32, device=device)
    model = N.Model(0.9, 0.1, 0.0, 100.0)
    tf = np.ascontiguousarray(wl.tf, np.float32)
    mm = MotionModel(ctx, seed=77)
    motion = mm.distributions("scale", [1.0, 0.5], 0.1)
    Npts = int(wl.points.shape[0])
    d_pts = torch.from_numpy(wl.points).to(device)
    rng = np.random.default_rng(99)
    ctx.reserve(cap, Npts)
    true = np.asarray(wl.true_pose, np.float64)
    P, cur = P0, 0
    mean_err, best_err, yaw_err = [], [], []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for k in range(updates):
            d = bufs[cur]
            N.check(lib.tsdfl_motion_update_device(ctx.handle, vp(d.data_ptr()), P, C.byref(motion), 77, k, None))
            N.check(lib.tsdfl_evaluate_device(ctx.handle, dmap.handle, C.byref(model), vp(d.data_ptr()), P,
                                              vp(d_pts.data_ptr()), Npts, tf.ctypes.data_as(vp), 0,
                                              vp(d_pose.data_ptr())))
            N.check(lib.tsdfl_best_particle_device(ctx.handle, vp(d.data_ptr()), P, vp(d_best.data_ptr())))
            N.check(lib.tsdfl_resample_systematic_device(ctx.handle, vp(d.data_ptr()), P,
                                                         float(np.float32(rng.random() / P)),
                                                         vp(bufs[cur ^ 1].data_ptr()), cap, vp(d_cnt.data_ptr())))
            ctx.sync()
            pose = d_pose.cpu().numpy()[:6].astype(np.float64)
            bi = int(d_best[0].item()) & 0xFFFFFFFF
            b = d[min(bi, P - 1)].cpu().numpy().astype(np.float64)
            mean_err.append(float(np.linalg.norm(pose[:3] - true[:3])))
            best_err.append(float(np.linalg.norm(b[:3] - true[:3])))
            yaw_err.append(float(np.rad2deg(abs((pose[5] - true[5] + np.pi) % (2 * np.pi) - np.pi))))
            P = min(int(d_cnt[0].item()), cap)
            cur ^= 1
    secs = time.perf_counter() - t0
    marks = sorted({0, 1, 4, 9, updates // 2, updates - 1})
    return {"updates": updates, "particles": P0, "points": Npts,
            "step": "motion + sensor update + best particle + systematic resample, count read back",
            "ms_per_update": 1000.0 * secs / updates,
            "mean_position_error_m": {str(i + 1): mean_err[i] for i in marks if i < updates},
            "best_particle_error_m": {str(i + 1): best_err[i] for i in marks if i < updates},
            "mean_yaw_error_deg": {str(i + 1): yaw_err[i] for i in marks if i < updates}}


def motion_side(lib, ctx, stream, wl, device: str, with_cpu: bool, reps: int = 20) -> dict:
    """Times the motion update (ParticleCloud::apply_model with device-drawn
    noise, odometry 0.8 m/s, 0.2 rad/s, 0.1 s) on the workload's particles."""
    import torch

    from tsdf_localization_gb300 import MotionModel
    from tsdf_localization_gb300 import _native as N
    P = int(wl.particles.shape[0])
    mm = MotionModel(ctx)
    m = mm.distributions("odom", [0.8, 0.2], 0.1)
    d = torch.from_numpy(wl.particles.copy()).to(device)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for i in range(3):
            N.check(lib.tsdfl_motion_update_device(ctx.handle, C.c_void_p(d.data_ptr()), P, C.byref(m), 1, i, None))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(reps):
            N.check(lib.tsdfl_motion_update_device(ctx.handle, C.c_void_p(d.data_ptr()), P, C.byref(m), 1, 10 + i,
                                                   None))
        e1.record(stream)
        e1.synchronize()
        ctx.sync()
    res = {"particles": P, "device_us": 1000.0 * e0.elapsed_time(e1) / reps, "rng": "Philox4x64-10, Box-Muller FP64"}
    if with_cpu:
        from oracle import oracle_py as O
        draws = np.random.default_rng(0).normal(0, 0.01, (P, 6))
        t0 = time.perf_counter()
        O.motion_apply(wl.particles, draws)
        res["cpu_oracle_ms"] = 1000.0 * (time.perf_counter() - t0)
    return res


def batch_workload(n_filters: int, seed: int = 11, worlds=None, p_range=(1000, 200_000)):
    """64 independent filters over 4 seeded maps (room 20x20x4 m @0.05, the
    building @0.05, warehouse 200x80x15 m @0.1, tunnel 500x8x6 m @0.1);
    particle counts log-uniform in p_range ([1k, 200k]), scan sizes uniform in
    [1k, 16k] drawn from each map's reduced 64x2048 ray-cast scan, particles
    Gaussian (0.3 m, 5 deg) around each map's true pose."""
    from tsdf_localization_gb300 import synth
    if worlds is None:
        worlds = [
            synth.make_workload(synth.ROOM, 21, 50, 16000, 1, 64, 2048, dropout=0.01, edge=8, reduce_cell=0.05,
                                name="room20x20x4@0.05"),
            synth.building_workload(seed=2, n_particles=1, n_points=16000),
            synth.make_workload(synth.WAREHOUSE, 23, 100, 16000, 1, 64, 2048, dropout=0.01, edge=16,
                                reduce_cell=0.1, name="warehouse200x80x15@0.1"),
            synth.make_workload(synth.TUNNEL, 24, 100, 16000, 1, 64, 2048, dropout=0.01, edge=16, reduce_cell=0.1,
                                name="tunnel500x8x6@0.1"),
        ]
    rng = np.random.default_rng(seed)
    filters = []
    for i in range(n_filters):
        wl = worlds[i % 4]
        P = int(round(np.exp(rng.uniform(np.log(p_range[0]), np.log(p_range[1])))))
        N = int(rng.integers(1000, 16001))
        N = min(N, wl.points.shape[0])
        pts = wl.points[np.sort(rng.permutation(wl.points.shape[0])[:N])]
        parts = synth.particles_gaussian(wl.true_pose, 0.3, float(np.deg2rad(5.0)), P, seed * 1000 + i)
        filters.append((i % 4, parts, np.ascontiguousarray(pts, np.float32)))
    return worlds, filters


def plain_rate(ctx, stream, dev: str, flush) -> float:
    """The plain single-filter rate (particle*points/s) of one update plus
    systematic resampling at 100k particles x 8,192 points on the building map,
    L2 flushed before each of 5 timed repetitions (median)."""
    import torch

    from tsdf_localization_gb300 import DeviceMap
    from tsdf_localization_gb300 import _native as N
    from tsdf_localization_gb300 import synth
    lib = N.lib()
    wlp = synth.building_workload(seed=2, n_particles=100_000, n_points=8192)
    dmp = DeviceMap(ctx, wlp.coef, wlp.grid_occ, codes=wlp.codes, dense=True)
    model = N.Model(0.9, 0.1, 0.0, 100.0)
    tfp = np.ascontiguousarray(wlp.tf, np.float32)
    dp = torch.from_numpy(wlp.particles).to(dev)
    dq = torch.from_numpy(wlp.points).to(dev)
    dpo = torch.zeros(8, dtype=torch.float32, device=dev)
    dro = torch.zeros((200_016, 7), dtype=torch.float32, device=dev)
    dcn = torch.zeros(4, dtype=torch.int32, device=dev)
    vp = C.c_void_p
    torch.cuda.synchronize()
    pt = []
    with torch.cuda.stream(stream):
        for i in range(8):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            N.check(lib.tsdfl_evaluate_device(ctx.handle, dmp.handle, C.byref(model), vp(dp.data_ptr()), 100_000,
                                              vp(dq.data_ptr()), 8192, tfp.ctypes.data_as(vp), 0,
                                              vp(dpo.data_ptr())))
            N.check(lib.tsdfl_resample_systematic_device(ctx.handle, vp(dp.data_ptr()), 100_000,
                                                         float(np.float32(0.37 / 100_000)), vp(dro.data_ptr()),
                                                         200_016, vp(dcn.data_ptr())))
            e1.record(stream)
            e1.synchronize()
            if i >= 3:
                pt.append(e0.elapsed_time(e1))
        ctx.sync()
    return 100_000 * 8192 / (float(np.median(pt)) / 1000.0)


def served_measure(args, local: int, worlds, ctx, stream, maps, seconds: float) -> dict:
    """Served localization: robots over the four maps submit scans as Poisson
    arrivals (10-20 Hz each) to the native request loop for a fixed window;
    particle counts log-uniform in [5k, 500k] (2 % of the robots at 1M), scans
    uniform in [2k, 16k] points.  Returns the served aggregate rate, p50/p99
    latency of the published updates (submission to publication, host clock),
    and what admission refused."""
    from tsdf_localization_gb300 import LocalizationServer
    from tsdf_localization_gb300 import synth
    rng = np.random.default_rng(17 + local)
    srv = LocalizationServer(ctx, hbm_budget=150 << 30, max_sessions=args.sessions, max_points=16000,
                             max_wait_ms=args.max_wait_ms, max_queue=2)
    robots = []
    refused_open = 0
    for i in range(args.sessions):
        mi = i % 4
        wl = worlds[mi]
        P = 1_000_000 if rng.random() < 0.02 else int(round(np.exp(rng.uniform(np.log(5000), np.log(500_000)))))
        Nn = min(int(rng.integers(2000, 16001)), wl.points.shape[0])
        parts = synth.particles_gaussian(wl.true_pose, 0.3, float(np.deg2rad(5.0)), P, 7000 + i)
        try:
            sid = srv.open(maps[mi], parts, wl.tf, seed=9000 + i)
        except Exception:
            refused_open += 1
            continue
        start = int(rng.integers(0, wl.points.shape[0] - Nn + 1))
        robots.append({"sid": sid, "P": P, "N": Nn, "hz": float(rng.uniform(10, 20)),
                       "pts": np.ascontiguousarray(wl.points[start:start + Nn]), "next": 0.0})
    for r in robots:
        r["next"] = float(rng.exponential(1.0 / r["hz"]))
    # warm-up: one update per robot, not timed
    warm = [srv.submit(r["sid"], r["pts"]) for r in robots]
    pending = {t for t in warm if t is not None}
    while pending:
        srv.poll()
        for t in list(pending):
            if srv.result(t) is not None:
                pending.discard(t)
    base = srv.stats()
    offered_pp = served_pp = 0
    lat = []
    tickets = {}
    t0 = time.perf_counter()
    with ClockSampler(local) as clk:
        while True:
            now = time.perf_counter() - t0
            if now >= seconds:
                break
            for r in robots:
                while r["next"] <= now:
                    offered_pp += r["P"] * r["N"]
                    t = srv.submit(r["sid"], r["pts"])
                    if t is not None:
                        tickets[t] = r["P"] * r["N"]
                    r["next"] += float(rng.exponential(1.0 / r["hz"]))
            srv.poll()
            for t in list(tickets):
                res = srv.result(t)
                if res is not None:
                    lat.append(res[1])
                    served_pp += tickets.pop(t)
        window = time.perf_counter() - t0
        clocks = clk.summary()
    # drain what was admitted in the window (its latency counts, its work does not extend the window)
    t_drain = time.perf_counter()
    while tickets and time.perf_counter() - t_drain < 60:
        srv.poll()
        for t in list(tickets):
            res = srv.result(t)
            if res is not None:
                lat.append(res[1])
                tickets.pop(t)
    st = srv.stats()
    srv.close()
    Pv = np.array([r["P"] for r in robots])
    return {"workload": f"{args.sessions} served robots over room/building/warehouse/tunnel maps",
            "sessions_open": len(robots), "sessions_refused": refused_open,
            "particles_range": [int(Pv.min()), int(Pv.max())], "bursts_1M": int((Pv >= 1_000_000).sum()),
            "arrivals": "Poisson 10-20 Hz per robot", "window_s": window, "hbm_budget_gb": 150,
            "max_wait_ms": args.max_wait_ms,
            "form": "served: native request loop, continuous batching over two dispatch slots",
            "value": served_pp / window, "unit": UNIT,
            "offered_pp_per_s": offered_pp / window,
            "submitted": st["accepted"] - base["accepted"] + st["refused"] - base["refused"],
            "refused": st["refused"] - base["refused"], "published": len(lat),
            "batches": st["batches"] - base["batches"],
            "latency_ms": {"p50": float(np.percentile(lat, 50)) if lat else None,
                           "p99": float(np.percentile(lat, 99)) if lat else None},
            "clocks": clocks}


def run_served(args, rank: int, world: int, local: int) -> None:
    """--workload served: the served measurement as the bench's line, with the
    plain single-filter rate beside it."""
    import torch

    from tsdf_localization_gb300 import Context, DeviceMap
    dev = f"cuda:{local}"
    torch.cuda.set_device(local)
    worlds, _ = batch_workload(1)
    ctx = Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    maps = [DeviceMap(ctx, wl.coef, wl.grid_occ, codes=wl.codes, dense=True) for wl in worlds]
    sv = served_measure(args, local, worlds, ctx, stream, maps, args.seconds)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    plain = plain_rate(ctx, stream, dev, flush)
    if rank == 0:
        out = {"metric": METRIC, "value": sv["value"], "unit": UNIT, "n_gpus": world, "steps": sv["published"],
               "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f32", "data": "synthetic",
               "config": {k: sv[k] for k in ("workload", "sessions_open", "sessions_refused", "particles_range",
                                             "bursts_1M", "arrivals", "window_s", "hbm_budget_gb", "max_wait_ms",
                                             "form")} | {"parallelism": f"replicas x{world}"},
               "served": {"offered_pp_per_s": sv["offered_pp_per_s"], "served_pp_per_s": sv["value"],
                          "submitted": sv["submitted"], "refused": sv["refused"], "published": sv["published"],
                          "batches": sv["batches"]},
               "latency_ms": sv["latency_ms"], "vs_plain": sv["value"] / plain, "plain_value": plain,
               "roofline": None, "cpu_baseline": None, "e2e": None, "gpu_launches": None, "clocks": sv["clocks"]}
        print(json.dumps(out), flush=True)


def batch_measure(args, local: int, worlds, specs, ctx, stream, maps, flush) -> dict:
    """Batched uneven filters: one update of every filter per step (graph
    replay of prepare, the persistent scoring launch, normalise, resample),
    with new resampling draws written before each step.  Returns the rate, the
    step latencies, the autotuned tiles and the scoring launch's roofline."""
    import torch

    from tsdf_localization_gb300 import FilterBatch
    from tsdf_localization_gb300 import _native as N
    dev = f"cuda:{local}"
    keep, fs = [], []
    total_pp = 0
    for mi, parts, pts in specs:
        P, Nn = parts.shape[0], pts.shape[0]
        d_part = torch.from_numpy(parts).to(dev)
        d_pts = torch.from_numpy(pts).to(dev)
        d_pose = torch.zeros(8, dtype=torch.float32, device=dev)
        d_u0 = torch.zeros(1, dtype=torch.float32, device=dev)
        d_out = torch.zeros((2 * P + 16, 7), dtype=torch.float32, device=dev)
        d_cnt = torch.zeros(4, dtype=torch.int32, device=dev)
        keep.append((d_part, d_pts, d_pose, d_u0, d_out, d_cnt))
        fs.append({"map": maps[mi], "P": P, "N": Nn, "tf": worlds[mi].tf, "particles": d_part.data_ptr(),
                   "points": d_pts.data_ptr(), "pose_out": d_pose.data_ptr(), "u0": d_u0.data_ptr(),
                   "resampled": d_out.data_ptr(), "cap": 2 * P + 16, "count": d_cnt.data_ptr()})
        total_pp += P * Nn
    torch.cuda.synchronize()
    batch = FilterBatch(ctx, fs)
    info = batch.info()
    lib = N.lib()
    rng = np.random.default_rng(5 + local)
    u0_all = torch.zeros(len(fs), dtype=torch.float32).pin_memory()
    d_u0s = [k[3] for k in keep]
    Ps = np.array([f["P"] for f in fs], np.float64)

    def new_draws():
        u0_all.copy_(torch.from_numpy((rng.random(len(fs)) / Ps).astype(np.float32)))
        for i, d in enumerate(d_u0s):
            d.copy_(u0_all[i:i + 1], non_blocking=True)

    with torch.cuda.stream(stream):
        new_draws()
        batch.run()
        ctx.sync()
        chunk, group, score_ms = batch.autotune()
        batch.capture()
        for _ in range(args.warmup):
            new_draws()
            batch.run()
        ctx.sync()
        torch.cuda.synchronize()
        l0 = lib.tsdfl_launch_count()
        steps = args.batch_steps
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        with ClockSampler(local) as clk:
            for i in range(steps):
                flush.zero_()
                starts[i].record(stream)
                new_draws()
                batch.run()
                ends[i].record(stream)
                ends[i].synchronize()
            ctx.sync()
            torch.cuda.synchronize()
        launches = lib.tsdfl_launch_count() - l0
        clocks = clk.summary()
        # the same updates as one single-filter call pair per filter, one after
        # another on the stream (what the batch replaces)
        model = N.Model(0.9, 0.1, 0.0, 100.0)
        vp = C.c_void_p
        tfs = [np.ascontiguousarray(worlds[mi].tf, np.float32) for mi, _, _ in specs]

        def sequential():
            for f, t in zip(fs, tfs):
                N.check(lib.tsdfl_evaluate_device(ctx.handle, f["map"].handle, C.byref(model), vp(f["particles"]),
                                                  f["P"], vp(f["points"]), f["N"], t.ctypes.data_as(vp), 0,
                                                  vp(f["pose_out"])))
                N.check(lib.tsdfl_resample_systematic_device(ctx.handle, vp(f["particles"]), f["P"],
                                                             float(np.float32(0.5 / f["P"])), vp(f["resampled"]),
                                                             f["cap"], vp(f["count"])))

        sequential()
        ctx.sync()
        seq_ms = []
        for i in range(3):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sequential()
            e1.record(stream)
            e1.synchronize()
            seq_ms.append(e0.elapsed_time(e1))
        ctx.sync()
    batch.close()
    del keep
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    total_ms = float(np.sum(step_ms))
    peak, peak_src = measured_peaks()
    alg = 2.0 * total_pp + sum(56.0 * f["P"] + 12.0 * f["N"] for f in fs)
    achieved = alg / (score_ms / 1000.0) / 1e9
    Pv = np.array([f["P"] for f in fs])
    Nv = np.array([f["N"] for f in fs])
    return {"workload": f"{len(fs)} batched filters over room/building/warehouse/tunnel maps",
            "filters": len(fs), "particles_total": int(Pv.sum()), "particles_range": [int(Pv.min()), int(Pv.max())],
            "points_range": [int(Nv.min()), int(Nv.max())], "particle_points_per_step": int(total_pp),
            "layout": "compact", "tiles": [chunk, group], "segments": info["segments"],
            "work_batches": info["batches"],
            "form": "batched: one persistent scoring launch, graph-replayed update",
            "l2": "flushed (512 MB write) before every timed step",
            "steps": steps, "value": total_pp * steps / (total_ms / 1000.0), "unit": UNIT,
            "ms_per_step": total_ms / steps, "gpu_launches": int(launches),
            "sequential_single_filter_ms": float(np.median(seq_ms)),
            "vs_sequential": float(np.median(seq_ms)) / (total_ms / steps),
            "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99))},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None, "kernel": "eval_batch_kernel",
                         "kernel_ms": score_ms, "peak_source": peak_src, "algorithmic_bytes": alg},
            "clocks": clocks}


def run_batch(args, rank: int, world: int, local: int) -> None:
    """--workload batch: the batched measurement as the bench's line, with the
    plain single-filter rate beside it."""
    import torch

    from tsdf_localization_gb300 import Context, DeviceMap
    dev = f"cuda:{local}"
    torch.cuda.set_device(local)
    worlds, specs = batch_workload(args.filters)
    ctx = Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    maps = [DeviceMap(ctx, wl.coef, wl.grid_occ, codes=wl.codes, dense=True) for wl in worlds]
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    args.batch_steps = args.steps
    bm = batch_measure(args, local, worlds, specs, ctx, stream, maps, flush)
    total_ms = max_over_ranks(bm["ms_per_step"] * args.steps, device=dev)
    value = bm["particle_points_per_step"] * args.steps * world / (total_ms / 1000.0)
    plain = plain_rate(ctx, stream, dev, flush)
    if rank == 0:
        cfg = {k: bm[k] for k in ("workload", "filters", "particles_total", "particles_range", "points_range",
                                  "particle_points_per_step", "layout", "tiles", "segments", "work_batches", "form",
                                  "l2")}
        cfg["parallelism"] = f"replicas x{world}"
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": cfg,
               "vs_plain": value / plain, "plain_value": plain, "roofline": bm["roofline"],
               "cpu_baseline": None, "e2e": None, "gpu_launches": bm["gpu_launches"],
               "latency_ms": bm["latency_ms"], "clocks": bm["clocks"]}
        print(json.dumps(out), flush=True)


def global_measure(args, local: int, ctx, stream, flush, steps: int = 5, warmup: int = 3) -> dict:
    """Global localisation (1,000,000 particles uniform over the seed-3
    building's free space, any yaw, 2,048 points): update plus systematic
    resampling on the device, L2 flushed before every step; the scoring
    kernel's time and roofline."""
    import torch

    from tsdf_localization_gb300 import DeviceMap
    from tsdf_localization_gb300 import _native as N
    from tsdf_localization_gb300 import synth
    dev = f"cuda:{local}"
    lib = N.lib()
    wl = synth.global_workload(seed=3, n_particles=1_000_000, n_points=2048)
    P, Npts = int(wl.particles.shape[0]), int(wl.points.shape[0])
    dmap = DeviceMap(ctx, wl.coef, wl.grid_occ, codes=wl.codes, dense=True)
    model = N.Model(0.9, 0.1, 0.0, 100.0)
    tfp = np.ascontiguousarray(wl.tf, np.float32)
    d_part = torch.from_numpy(wl.particles).to(dev)
    d_pts = torch.from_numpy(wl.points).to(dev)
    cap = 2 * P + 16
    d_out = torch.empty((cap, 7), dtype=torch.float32, device=dev)
    d_cnt = torch.zeros(4, dtype=torch.int32, device=dev)
    d_pose = torch.zeros(8, dtype=torch.float32, device=dev)
    rng = np.random.default_rng(4321)
    vp = C.c_void_p
    ctx.reserve(P, Npts)

    def step():
        N.check(lib.tsdfl_evaluate_device(ctx.handle, dmap.handle, C.byref(model), vp(d_part.data_ptr()), P,
                                          vp(d_pts.data_ptr()), Npts, tfp.ctypes.data_as(vp), 0,
                                          vp(d_pose.data_ptr())))
        N.check(lib.tsdfl_resample_systematic_device(ctx.handle, vp(d_part.data_ptr()), P,
                                                     float(np.float32(rng.random() / P)), vp(d_out.data_ptr()), cap,
                                                     vp(d_cnt.data_ptr())))

    lib.tsdfl_ctx_set_timing(ctx.handle, 1)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            step()
        ctx.sync()
        ms, kms = [], []
        for _ in range(steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
            k = C.c_float()
            N.check(lib.tsdfl_ctx_last_timing(ctx.handle, C.byref(k)))
            kms.append(k.value)
        ctx.sync()
        # the variant where every particle scores 256 of the points, chosen per
        # particle and seed (tsdfl_evaluate_subsampled_device)
        K = 256
        ms_sub, kms_sub = [], []
        for i in range(warmup + steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            N.check(lib.tsdfl_evaluate_subsampled_device(ctx.handle, dmap.handle, C.byref(model),
                                                         vp(d_part.data_ptr()), P, vp(d_pts.data_ptr()), Npts,
                                                         tfp.ctypes.data_as(vp), K, 1000 + i, vp(d_pose.data_ptr())))
            N.check(lib.tsdfl_resample_systematic_device(ctx.handle, vp(d_part.data_ptr()), P,
                                                         float(np.float32(rng.random() / P)), vp(d_out.data_ptr()),
                                                         cap, vp(d_cnt.data_ptr())))
            e1.record(stream)
            e1.synchronize()
            if i >= warmup:
                ms_sub.append(e0.elapsed_time(e1))
                k = C.c_float()
                N.check(lib.tsdfl_ctx_last_timing(ctx.handle, C.byref(k)))
                kms_sub.append(k.value)
        ctx.sync()
    lib.tsdfl_ctx_set_timing(ctx.handle, 0)
    peak, peak_src = measured_peaks()
    kmed = float(np.median(kms))
    alg = roofline_bytes(P, Npts, "compact")
    dmap.close()
    sub = {"points_per_particle": K, "selection": "one point per stratum of N/K consecutive scan indices, "
                                                  "SplitMix64 per (seed, particle)",
           "value": P * K * steps / (float(np.sum(ms_sub)) / 1000.0), "unit": UNIT,
           "ms_per_step": float(np.mean(ms_sub)), "kernel_ms": float(np.median(kms_sub))}
    return {"workload": wl.name, "particles": P, "points": Npts, "steps": steps, "subsampled": sub,
            "step": "sensor update + normalise + mean pose + systematic resample (FP64 CDF)",
            "value": P * Npts * steps / (float(np.sum(ms)) / 1000.0), "unit": UNIT,
            "ms_per_step": float(np.mean(ms)),
            "roofline": {"bound": "hbm", "achieved": alg / (kmed / 1000.0) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": alg / (kmed / 1000.0) / 1e9 / peak,
                         "traffic": MEASURED_TRAFFIC.get(("global", P, Npts, "compact", "fast")),
                         "kernel": "eval_tiled_kernel", "kernel_ms": kmed, "peak_source": peak_src,
                         "algorithmic_bytes": alg}}


def sub_measurements(args, local: int, ctx, stream, flush, plain_value: float) -> dict:
    """The default run's side lines: global localisation, the batched filters
    and the served sessions, each with its rate against the plain line."""
    from tsdf_localization_gb300 import DeviceMap
    out = {}
    g = global_measure(args, local, ctx, stream, flush)
    g["vs_plain"] = g["value"] / plain_value
    out["global"] = g
    worlds, specs = batch_workload(args.filters)
    maps = [DeviceMap(ctx, wl.coef, wl.grid_occ, codes=wl.codes, dense=True) for wl in worlds]
    b = batch_measure(args, local, worlds, specs, ctx, stream, maps, flush)
    b["vs_plain"] = b["value"] / plain_value
    out["batch"] = b
    # small filters (1k-10k particles), where one filter alone leaves most SMs idle
    _, small = batch_workload(args.filters, seed=12, worlds=worlds, p_range=(1000, 10_000))
    bs = batch_measure(args, local, worlds, small, ctx, stream, maps, flush)
    bs["vs_plain"] = bs["value"] / plain_value
    out["batch_small"] = bs
    sv = served_measure(args, local, worlds, ctx, stream, maps, args.served_seconds)
    sv["vs_plain"] = sv["value"] / plain_value
    out["served"] = sv
    for m in maps:
        m.close()
    return out


def max_over_ranks(x: float, device=None) -> float:
    """The largest of every rank's x (all ranks get it); x itself without a
    process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference_arm(args, rank: int) -> None:
    if rank != 0:
        return
    wl = make_workload(args)
    base, (P_s, kind, om, rm) = cpu_baseline(wl, target_s=5.0)
    N = wl.points.shape[0]
    times = []
    for i in range(args.warmup + args.steps):
        parts = wl.particles[:P_s].copy()
        t0 = time.perf_counter()
        if kind == "reference":
            rm.evaluate(parts, wl.points, wl.tf, serial=False)
            from oracle import oracle_py as O
            O.ref_resample_systematic(parts[:, 6], 1 + i)
        else:
            from oracle import oracle_py as O
            O.evaluate(om, parts, wl.points, wl.tf)
            O.resample_systematic(parts[:, 6], float(np.float32(0.5 / P_s)))
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
    t = float(np.sum(times))
    value = P_s * N * len(times) / t
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * t / len(times),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": wl.name, "particles": int(wl.particles.shape[0]), "points": int(N),
                      "sample_particles": int(P_s)},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": base["cores"], "kind": kind,
                            "sample": f"{P_s} particles x {N} points per step"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference_arm(args, rank)
        return

    import torch
    import torch.distributed as dist

    from tsdf_localization_gb300 import Context, DeviceMap
    from tsdf_localization_gb300 import _native as N

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    if args.workload in ("batch", "served"):
        (run_batch if args.workload == "batch" else run_served)(args, rank, world, local)
        if world > 1:
            dist.destroy_process_group()
        return

    wl = make_workload(args)
    P = int(wl.particles.shape[0])
    Npts = int(wl.points.shape[0])
    lib = N.lib()
    ctx = Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    dmap = DeviceMap(ctx, wl.coef, wl.grid_occ, codes=wl.codes, dense=(args.layout == "compact"),
                     grid=(args.layout == "grid"))
    info = dmap.info()
    model = N.Model(0.9, 0.1, 0.0, 100.0)
    tf = np.ascontiguousarray(wl.tf, np.float32)
    tfp = tf.ctypes.data_as(C.c_void_p)
    cap = 2 * P + 16
    d_part = torch.from_numpy(wl.particles).to(f"cuda:{local}")
    d_pts = torch.from_numpy(wl.points).to(f"cuda:{local}")
    d_out = torch.empty((cap, 7), dtype=torch.float32, device=f"cuda:{local}")
    d_cnt = torch.zeros(4, dtype=torch.int32, device=f"cuda:{local}")
    d_pose = torch.zeros(8, dtype=torch.float32, device=f"cuda:{local}")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    ctx.reserve(P, Npts)
    rng = np.random.default_rng(1234 + rank)
    vp = C.c_void_p
    eflags = N.TSDFL_SUM_EXACT | (N.TSDFL_EVAL_GENERIC if args.kernel == "generic" else 0)

    def step():
        N.check(lib.tsdfl_evaluate_device(ctx.handle, dmap.handle, C.byref(model), vp(d_part.data_ptr()), P,
                                          vp(d_pts.data_ptr()), Npts, tfp, eflags, vp(d_pose.data_ptr())))
        u0 = float(np.float32(rng.random() / P))
        N.check(lib.tsdfl_resample_systematic_device(ctx.handle, vp(d_part.data_ptr()), P, u0,
                                                     vp(d_out.data_ptr()), cap, vp(d_cnt.data_ptr())))

    lib.tsdfl_ctx_set_timing(ctx.handle, 1)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
        ctx.sync()
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        l0 = lib.tsdfl_launch_count()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        kern_ms = []
        with ClockSampler(local) as clk:
            for i in range(args.steps):
                flush.zero_()                       # L2 flush outside the timed step
                starts[i].record(stream)
                step()
                ends[i].record(stream)
                ends[i].synchronize()
                k = C.c_float()
                N.check(lib.tsdfl_ctx_last_timing(ctx.handle, C.byref(k)))
                kern_ms.append(k.value)
            ctx.sync()
            torch.cuda.synchronize()
        launches = lib.tsdfl_launch_count() - l0
        clocks = clk.summary()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = max_over_ranks(float(np.sum(step_ms)), device=f"cuda:{local}")
    latency = {"p50": max_over_ranks(float(np.percentile(step_ms, 50)), device=f"cuda:{local}"),
               "p99": max_over_ranks(float(np.percentile(step_ms, 99)), device=f"cuda:{local}")}
    if world > 1:
        dist.barrier()
    value = P * Npts * args.steps * world / (total_ms / 1000.0)
    lib.tsdfl_ctx_set_timing(ctx.handle, 0)

    # roofline of the scoring kernel
    kmed = float(np.median(kern_ms))
    alg = roofline_bytes(P, Npts, args.layout)
    peak, peak_src = measured_peaks()
    achieved = alg / (kmed / 1000.0) / 1e9
    measured_traffic = MEASURED_TRAFFIC
    traffic = measured_traffic.get((args.workload, P, Npts, args.layout, args.kernel))
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "kernel": "eval_tiled_kernel" if (args.kernel == "fast" and info["fast_index"])
            else "eval_exact_kernel", "kernel_ms": kmed, "peak_source": peak_src,
            "algorithmic_bytes": alg,
            "traffic_gbs": traffic / (kmed / 1000.0) / 1e9 if traffic else None}

    # end to end through the host C ABI, pinned host buffers
    e2e = None
    if not args.no_e2e:
        h_part = torch.empty((P, 7), dtype=torch.float32).pin_memory().numpy()
        h_pts = torch.empty((Npts, 3), dtype=torch.float32).pin_memory().numpy()
        h_idx = torch.empty(cap, dtype=torch.int32).pin_memory().numpy()
        h_pts[:] = wl.points
        pose = np.zeros(6, np.float32)
        cnt = C.c_size_t()

        def e2e_inputs():
            # the step's input particle set, as the previous step left it in the
            # caller's buffer: staged before the timed region
            h_part[:] = wl.particles

        def e2e_step(i):
            # the evaluator's and the resampler's calls on the caller's particle cloud
            N.check(lib.tsdfl_evaluate(ctx.handle, dmap.handle, C.byref(model), h_part.ctypes.data_as(vp), P,
                                       h_pts.ctypes.data_as(vp), Npts, tfp, eflags, pose.ctypes.data_as(vp)))
            N.check(lib.tsdfl_resample_systematic_particles(ctx.handle, h_part.ctypes.data_as(vp), P,
                                                            np.float32(rng.random() / P), h_idx.ctypes.data_as(vp),
                                                            cap, C.byref(cnt)))
            return cnt.value

        with torch.cuda.stream(stream):
            for i in range(args.warmup):
                e2e_inputs()
                e2e_step(i)
            tt = []
            counts = []
            for i in range(args.steps):
                e2e_inputs()
                flush.zero_()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                counts.append(e2e_step(i))
                tt.append(time.perf_counter() - t0)
        e2e_s = float(np.sum(tt))
        h2d = 28 * P + 12 * Npts + 28 * P
        d2h = 28 * P + 4 * 6 + 4 + 4 * cap
        e2e = {"value": P * Npts * args.steps * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": 1000.0 * e2e_s / args.steps}

    base = None
    if rank == 0 and not args.no_cpu_baseline:
        base, (_, _, om, _) = cpu_baseline(wl)
        base["error_vs_fp64"] = accuracy_vs_fp64(om, wl, dmap)
        del om
    scan = motion = tracking = None
    if not args.no_scan:
        scan = scan_reduction_side(lib, ctx, stream, wl, f"cuda:{local}", rank == 0 and not args.no_cpu_baseline)
        motion = motion_side(lib, ctx, stream, wl, f"cuda:{local}", rank == 0 and not args.no_cpu_baseline)
        if args.workload in ("building", "global"):
            tracking = tracking_side(lib, ctx, stream, wl, dmap, f"cuda:{local}",
                                     100 if args.workload == "building" else 50)
    subs = {}
    if world == 1 and args.workload == "building" and not args.no_sub:
        subs = sub_measurements(args, local, ctx, stream, flush, value)

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
               "config": {"workload": wl.name, "particles": P, "points": Npts, "voxel_m": wl.voxel_mm / 1000.0,
                          "layout": args.layout, "kernel": args.kernel, "map_bricks": int(info["bricks"]),
                          "map_device_bytes": int(info["device_bytes"]), "sums": "exact fixed point",
                          "l2": "flushed (512 MB write) before every timed step",
                          "step": "sensor update + normalise + mean pose + systematic resample",
                          "form": "plain single filter", "parallelism": f"replicas x{world}"},
               "roofline": roof, "cpu_baseline": base, "e2e": e2e, "gpu_launches": int(launches),
               "latency_ms": latency, "clocks": clocks, "scan_reduction": scan,
               "motion_update": motion, "tracking": tracking, **subs}
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
