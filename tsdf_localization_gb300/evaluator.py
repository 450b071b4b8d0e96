"""Host-side mirror of the reference's sensor-update interface over libtsdfl.

    TSDFEvaluator(map, per_point, a_hit, a_range, a_max, max_range)
        .evaluate(particles, points, tf_matrix) -> mean pose
    SystematicResampler(seed).resample(particles) -> resampled particles

follow include/tsdf_localization/evaluation/tsdf_evaluator.h:72-114 and
include/tsdf_localization/resampling/novel_resampling.h:38-74: particles are a
(P, 7) float32 array (x, y, z, roll, pitch, yaw, weight) whose weights are
overwritten with the normalised weights; errors raise RuntimeError with the
reference's messages ("No particle is valid!").
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N


def _f32(a, shape_tail=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    if shape_tail is not None and (a.ndim != 2 or a.shape[1] != shape_tail):
        raise ValueError(f"expected an (n, {shape_tail}) array, got {a.shape}")
    return a


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Context:
    """One device and stream with the evaluation workspace (tsdfl_ctx)."""

    def __init__(self, device: int = 0):
        self._lib = N.lib()
        h = C.c_void_p()
        N.check(self._lib.tsdfl_ctx_create(device, C.byref(h)))
        self.handle = h
        self.device = device

    def close(self) -> None:
        if getattr(self, "handle", None):
            self._lib.tsdfl_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr: int | None) -> None:
        N.check(self._lib.tsdfl_ctx_set_stream(self.handle, C.c_void_p(stream_ptr or 0)))

    def sync(self) -> None:
        N.check(self._lib.tsdfl_ctx_sync(self.handle))

    def reserve(self, particles: int, points: int) -> None:
        N.check(self._lib.tsdfl_ctx_reserve(self.handle, particles, points))


class DeviceMap:
    """A likelihood map resident on the device (tsdfl_map).  dense=True also
    builds the compact layout (TSDFL_MAP_DENSE): one map gather per lookup.
    f16=True stores half-precision likelihood values instead (TSDFL_MAP_F16,
    an accuracy variant); hash_index=True indexes the allocated bricks in a
    sparse hash (TSDFL_MAP_HASH), which dense=True also builds for maps whose
    brick bitmap is too large for shared memory.  grid=True also stores the
    codes of every brick of the bounding box (TSDFL_MAP_GRID), which the tiled
    kernel addresses by brick index with no rank lookup."""

    def __init__(self, ctx: Context, coef: N.MapCoef, grid_occ: np.ndarray, data: np.ndarray | None = None,
                 codes: np.ndarray | None = None, sigma: float = 0.1, dense: bool = False, force_f32: bool = False,
                 f16: bool = False, hash_index: bool = False, grid: bool = False):
        self.ctx = ctx
        self.coef = coef
        lib = N.lib()
        go = np.ascontiguousarray(grid_occ, dtype=np.int32)
        flags = ((N.TSDFL_MAP_DENSE if dense else 0) | (N.TSDFL_MAP_FORCE_F32 if force_f32 else 0) |
                 (N.TSDFL_MAP_F16 if f16 else 0) | (N.TSDFL_MAP_HASH if hash_index else 0) |
                 (N.TSDFL_MAP_GRID if grid else 0))
        h = C.c_void_p()
        if codes is not None:
            cd = np.ascontiguousarray(codes, dtype=np.uint16)
            N.check(lib.tsdfl_map_create_codes(ctx.handle, C.byref(coef), _ptr(go), _ptr(cd), sigma, flags,
                                               C.byref(h)))
        else:
            d = np.ascontiguousarray(data, dtype=np.float32)
            N.check(lib.tsdfl_map_create(ctx.handle, C.byref(coef), _ptr(go), _ptr(d), sigma, flags, C.byref(h)))
        self.handle = h

    def info(self) -> dict:
        inf = N.MapInfo()
        N.check(N.lib().tsdfl_map_get_info(self.handle, C.byref(inf)))
        return {k: getattr(inf, k) for k, _ in N.MapInfo._fields_}

    def close(self) -> None:
        if getattr(self, "handle", None):
            N.lib().tsdfl_map_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class Pose:
    """Mean pose: position and roll/pitch/yaw (geometry_msgs::PoseWithCovariance
    carries the same as a quaternion, tsdf_evaluator.cpp:223-229)."""

    x: float
    y: float
    z: float
    roll: float
    pitch: float
    yaw: float

    def as_array(self) -> np.ndarray:
        return np.array([self.x, self.y, self.z, self.roll, self.pitch, self.yaw], dtype=np.float32)


class TSDFEvaluator:
    """GPU sensor update with the reference evaluator's constructor and call.

    per_point is accepted for signature compatibility; both reference modes
    give the same weights here (the per-point kernel's range test on the
    particle position, cuda_eval_particles.h:499, is not reproduced).
    """

    def __init__(self, device_map: DeviceMap, per_point: bool = False, a_hit: float = 0.9, a_range: float = 0.1,
                 a_max: float = 0.0, max_range: float = 100.0, serial_sums: bool = False, generic: bool = False,
                 log_normalise: bool = False):
        self.map = device_map
        self.ctx = device_map.ctx
        self.per_point = per_point
        self.model = N.Model(a_hit, a_range, a_max, max_range)
        self.flags = ((N.TSDFL_SUM_SERIAL if serial_sums else N.TSDFL_SUM_EXACT) |
                      (N.TSDFL_EVAL_GENERIC if generic else 0) | (N.TSDFL_NORM_LOG if log_normalise else 0))

    def evaluate(self, particles: np.ndarray, points: np.ndarray, tf_matrix) -> Pose | None:
        """Writes normalised weights into particles[:, 6]; returns the mean pose,
        or None for an empty scan (the reference returns a default pose)."""
        if not (isinstance(particles, np.ndarray) and particles.dtype == np.float32 and particles.flags.c_contiguous
                and particles.ndim == 2 and particles.shape[1] == 7):
            raise ValueError("particles must be a C-contiguous (P, 7) float32 array")
        pts = _f32(points, 3)
        tf = np.ascontiguousarray(np.asarray(tf_matrix, dtype=np.float32).reshape(16))
        if pts.shape[0] == 0:
            return None
        pose = np.zeros(6, dtype=np.float32)
        rc = N.lib().tsdfl_evaluate(self.ctx.handle, self.map.handle, C.byref(self.model), _ptr(particles),
                                    particles.shape[0], _ptr(pts), pts.shape[0], _ptr(tf), self.flags, _ptr(pose))
        N.check(rc)
        return Pose(*[float(v) for v in pose])

    def evaluate_cloud(self, particles: np.ndarray, cloud: np.ndarray, n_points: int, point_step: int, tf_matrix,
                       x_offset: int = 0, ring_offset: int = 12, reduction_cell_size: float = 0.064,
                       own_ring: bool = False):
        """TSDFEvaluator::evaluateParticles (tsdf_evaluator.cpp:247-376) after its
        tf lookup: reduces the PointCloud2 data on the GPU and scores the reduced
        points.  Returns (pose or None, number of reduced points)."""
        if not (isinstance(particles, np.ndarray) and particles.dtype == np.float32 and particles.flags.c_contiguous
                and particles.ndim == 2 and particles.shape[1] == 7):
            raise ValueError("particles must be a C-contiguous (P, 7) float32 array")
        blob = np.ascontiguousarray(cloud, np.uint8).reshape(-1)
        if blob.shape[0] < n_points * point_step:
            raise ValueError("cloud holds fewer than n_points * point_step bytes")
        tf = np.ascontiguousarray(np.asarray(tf_matrix, dtype=np.float32).reshape(16))
        pose = np.zeros(6, dtype=np.float32)
        nred = C.c_size_t(0)
        N.check(N.lib().tsdfl_evaluate_cloud(self.ctx.handle, self.map.handle, C.byref(self.model), _ptr(particles),
                                             particles.shape[0], _ptr(blob), n_points, point_step, x_offset,
                                             ring_offset, reduction_cell_size,
                                             N.TSDFL_SCAN_OWN_RING if own_ring else 0, _ptr(tf), self.flags,
                                             _ptr(pose), C.byref(nred)))
        if nred.value == 0:
            return None, 0
        return Pose(*[float(v) for v in pose]), nred.value

    def evaluate_subsampled(self, particles: np.ndarray, points: np.ndarray, tf_matrix, k: int, seed: int,
                            debug: bool = False):
        """evaluate() with every particle scoring k of the points, chosen per
        particle and seed (tsdfl_evaluate_subsampled): the mean pose, or with
        debug (pose, raw weights, hit counts)."""
        if not (isinstance(particles, np.ndarray) and particles.dtype == np.float32 and particles.flags.c_contiguous
                and particles.ndim == 2 and particles.shape[1] == 7):
            raise ValueError("particles must be a C-contiguous (P, 7) float32 array")
        pts = _f32(points, 3)
        tf = np.ascontiguousarray(np.asarray(tf_matrix, dtype=np.float32).reshape(16))
        P = particles.shape[0]
        pose = np.zeros(6, dtype=np.float32)
        raw = np.zeros(max(P, 1), np.float32)
        hits = np.zeros(max(P, 1), np.uint32)
        N.check(N.lib().tsdfl_evaluate_subsampled(self.ctx.handle, self.map.handle, C.byref(self.model),
                                                  _ptr(particles), P, _ptr(pts), pts.shape[0], _ptr(tf), int(k),
                                                  int(seed), _ptr(pose), _ptr(raw), _ptr(hits)))
        if debug:
            return pose, raw[:P], hits[:P]
        return Pose(*[float(v) for v in pose])

    def evaluate_debug(self, particles: np.ndarray, points: np.ndarray, tf_matrix, voxel_index: bool = False):
        """evaluate() plus per-particle raw weights, hit counts, laser poses and,
        for small cases, per particle*point: the slot index (serial sums, and
        the generic kernel on the brick layout) or the slot code (0..599 |tsdf|
        mm, 600 init, 601 miss) otherwise."""
        pts = _f32(points, 3)
        tf = np.ascontiguousarray(np.asarray(tf_matrix, dtype=np.float32).reshape(16))
        P, Nn = particles.shape[0], pts.shape[0]
        raw = np.zeros(P, np.float32)
        hits = np.zeros(P, np.uint32)
        lp = np.zeros((P, 12), np.float32)
        idx = np.zeros((P, Nn), np.uint32) if voxel_index else None
        dbg = N.EvalDebug(raw.ctypes.data, hits.ctypes.data, idx.ctypes.data if idx is not None else None,
                          lp.ctypes.data, 0.0)
        pose = np.zeros(6, dtype=np.float32)
        N.check(N.lib().tsdfl_evaluate_debug(self.ctx.handle, self.map.handle, C.byref(self.model), _ptr(particles),
                                             P, _ptr(pts), Nn, _ptr(tf), self.flags, _ptr(pose), C.byref(dbg)))
        return {"pose": pose, "raw": raw, "hits": hits, "laser_pose": lp, "voxel_index": idx,
                "weight_sum": dbg.weight_sum}


def pack_cloud(xyz: np.ndarray, ring: np.ndarray, point_step: int = 16, x_offset: int = 0,
               ring_offset: int = 12) -> np.ndarray:
    """PointCloud2 data bytes: per point x, y, z floats at x_offset and an int16
    ring at ring_offset, point_step bytes per point (other bytes zero)."""
    x = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
    r = np.ascontiguousarray(ring, np.int16).reshape(-1)
    if r.shape[0] != x.shape[0]:
        raise ValueError("xyz and ring differ in length")
    if x_offset + 12 > point_step or ring_offset + 2 > point_step:
        raise ValueError("fields must lie inside point_step")
    if ring_offset + 2 > x_offset and x_offset + 12 > ring_offset:
        raise ValueError("x, y, z and ring overlap")
    blob = np.zeros((x.shape[0], point_step), np.uint8)
    blob[:, x_offset:x_offset + 12] = x.view(np.uint8).reshape(-1, 12)
    blob[:, ring_offset:ring_offset + 2] = r.view(np.uint8).reshape(-1, 2)
    return blob.reshape(-1)


class ScanReducer:
    """The scan reduction of TSDFEvaluator::evaluateParticles
    (tsdf_evaluator.cpp:304-376) on the GPU: range filter (< 1 m dropped),
    first point per (ring, reduction cell), ring-major output in cloud order.
    own_ring=False follows the reference's ring iterator, which advances only
    for kept points (:319-332); True gives every point its own ring."""

    def __init__(self, ctx: Context, reduction_cell_size: float = 0.064, own_ring: bool = False):
        self.ctx = ctx
        self.cell = float(reduction_cell_size)
        self.flags = N.TSDFL_SCAN_OWN_RING if own_ring else 0

    def reduce(self, cloud: np.ndarray, n_points: int, point_step: int, x_offset: int = 0,
               ring_offset: int = 12) -> np.ndarray:
        """cloud: the PointCloud2 data (uint8, n_points * point_step bytes).
        Returns the reduced points as an (M, 3) float32 array."""
        blob = np.ascontiguousarray(cloud, np.uint8).reshape(-1)
        if blob.shape[0] < n_points * point_step:
            raise ValueError("cloud holds fewer than n_points * point_step bytes")
        out = np.zeros((max(n_points, 1), 3), np.float32)
        cnt = C.c_size_t(0)
        N.check(N.lib().tsdfl_reduce_scan(self.ctx.handle, _ptr(blob), n_points, point_step, x_offset, ring_offset,
                                          self.cell, self.flags, _ptr(out), out.shape[0], C.byref(cnt)))
        return out[:cnt.value].copy()

    def reduce_xyz(self, xyz: np.ndarray, ring: np.ndarray) -> np.ndarray:
        blob = pack_cloud(xyz, ring)
        return self.reduce(blob, blob.shape[0] // 16, 16, 0, 12)


class SystematicResampler:
    """SystematicResampler (novel_resampling.h:38-74) on the GPU.  The uniform
    draw U0 ~ U[0, 1/M) comes from a seeded numpy generator unless given."""

    def __init__(self, ctx: Context, seed: int | None = None):
        self.ctx = ctx
        self.rng = np.random.default_rng(seed)

    def draw(self, m: int) -> float:
        return float(np.float32(self.rng.random() * (1.0 / m)))

    def resample_indices(self, weights: np.ndarray, u0: float | None = None, cap: int | None = None) -> np.ndarray:
        w = np.ascontiguousarray(weights, dtype=np.float32)
        m = w.shape[0]
        if u0 is None:
            u0 = self.draw(m)
        cap = cap if cap is not None else 2 * m + 16
        out = np.zeros(max(cap, 1), np.uint32)
        cnt = C.c_size_t()
        N.check(N.lib().tsdfl_resample_systematic(self.ctx.handle, _ptr(w), m, np.float32(u0), _ptr(out), cap,
                                                  C.byref(cnt)))
        return out[: cnt.value]

    def resample_particle_indices(self, particles: np.ndarray, u0: float | None = None,
                                  cap: int | None = None) -> np.ndarray:
        """The same indices from the (M, 7) particle array itself (its last
        column holds the weights; tsdfl_resample_systematic_particles)."""
        p = np.ascontiguousarray(particles, dtype=np.float32)
        if p.ndim != 2 or p.shape[1] != 7:
            raise ValueError("particles must be an (M, 7) array")
        m = p.shape[0]
        if u0 is None:
            u0 = self.draw(m)
        cap = cap if cap is not None else 2 * m + 16
        out = np.zeros(max(cap, 1), np.uint32)
        cnt = C.c_size_t()
        N.check(N.lib().tsdfl_resample_systematic_particles(self.ctx.handle, _ptr(p), m, np.float32(u0), _ptr(out),
                                                            cap, C.byref(cnt)))
        return out[: cnt.value]

    def resample(self, particles: np.ndarray, u0: float | None = None) -> np.ndarray:
        idx = self.resample_particle_indices(particles, u0)
        return particles[idx].copy()


class ResidualSystematicResampler:
    """ResidualSystematicResampler (novel_resampling.h:76-104, mcl_3d's default)
    on the GPU.  The draw u0 ~ U[0, 1) comes from a seeded numpy generator
    unless given."""

    def __init__(self, ctx: Context, seed: int | None = None):
        self.ctx = ctx
        self.rng = np.random.default_rng(seed)

    def draw(self) -> float:
        return float(np.float32(self.rng.random()))

    def resample_indices(self, weights: np.ndarray, u0: float | None = None, cap: int | None = None) -> np.ndarray:
        w = np.ascontiguousarray(weights, dtype=np.float32)
        m = w.shape[0]
        if u0 is None:
            u0 = self.draw()
        cap = cap if cap is not None else 2 * m + 16
        out = np.zeros(max(cap, 1), np.uint32)
        cnt = C.c_size_t()
        N.check(N.lib().tsdfl_resample_residual_systematic(self.ctx.handle, _ptr(w), m, np.float32(u0), _ptr(out),
                                                           cap, C.byref(cnt)))
        return out[: cnt.value]

    def resample(self, particles: np.ndarray, u0: float | None = None) -> np.ndarray:
        idx = self.resample_indices(particles[:, 6], u0)
        return particles[idx].copy()


class _DrawnResampler:
    """Common host form of the reference's Wheel/Residual/Metropolis/Rejection
    resamplers: exactly M outputs; draws from the caller (the reference's
    own sequence gives its output bit for bit) or from the device generator."""

    def __init__(self, ctx: Context, seed: int = 0):
        self.ctx = ctx
        self.seed = int(seed)

    def resample(self, particles: np.ndarray, *draws) -> np.ndarray:
        return particles[self.resample_indices(particles[:, 6], *draws)]


class WheelResampler(_DrawnResampler):
    """WheelResampler (wheel_resampler.cpp:6-33); draws: M doubles in [0, 1)."""

    def resample_indices(self, weights: np.ndarray, draws: np.ndarray | None = None) -> np.ndarray:
        w = _f32(weights)
        d = None if draws is None else np.ascontiguousarray(draws, np.float64)
        if d is not None and d.shape != w.shape:
            raise ValueError("one draw per particle")
        out = np.zeros(w.shape[0], np.uint32)
        N.check(N.lib().tsdfl_resample_wheel(self.ctx.handle, _ptr(w), w.shape[0], _ptr(d), self.seed, _ptr(out)))
        return out


class ResidualResampler(_DrawnResampler):
    """ResidualResampler (novel_resampling.h:9-35); draws: particle indices."""

    def resample_indices(self, weights: np.ndarray, draws: np.ndarray | None = None) -> np.ndarray:
        w = _f32(weights)
        d = None if draws is None else np.ascontiguousarray(draws, np.uint32)
        out = np.zeros(w.shape[0], np.uint32)
        N.check(N.lib().tsdfl_resample_residual(self.ctx.handle, _ptr(w), w.shape[0], _ptr(d),
                                                0 if d is None else d.shape[0], self.seed, _ptr(out)))
        return out


class MetropolisResampler(_DrawnResampler):
    """MetropolisResampler(sampling_steps) (novel_resampling.h:106-143); draws:
    u (float) and j (index) arrays of M * steps, output-major."""

    def __init__(self, ctx: Context, sampling_steps: int = 50, seed: int = 0):
        super().__init__(ctx, seed)
        self.steps = int(sampling_steps)

    def resample_indices(self, weights: np.ndarray, u: np.ndarray | None = None,
                         j: np.ndarray | None = None) -> np.ndarray:
        w = _f32(weights)
        uu = None if u is None else np.ascontiguousarray(u, np.float32)
        jj = None if j is None else np.ascontiguousarray(j, np.uint32)
        out = np.zeros(w.shape[0], np.uint32)
        N.check(N.lib().tsdfl_resample_metropolis(self.ctx.handle, _ptr(w), w.shape[0], self.steps, _ptr(uu),
                                                  _ptr(jj), self.seed, _ptr(out)))
        return out


class RejectionResampler(_DrawnResampler):
    """RejectionResampler (novel_resampling.h:146-187); device draws only."""

    def resample_indices(self, weights: np.ndarray) -> np.ndarray:
        w = _f32(weights)
        out = np.zeros(w.shape[0], np.uint32)
        N.check(N.lib().tsdfl_resample_rejection(self.ctx.handle, _ptr(w), w.shape[0], self.seed, _ptr(out)))
        return out


class MotionModel:
    """ParticleCloud's motion update (particle_cloud.cpp:153-617) on the GPU.

    a = a_1 .. a_12 as setMotionParameters takes them (0.1 each by default,
    particle_cloud.h:59-70).  update() draws on the device from a counter-based
    generator keyed by the seed (one stream per step); apply() takes the draws
    (P x 6: dx, dy, dz, roll, pitch, yaw) from the caller.  Either way the pose
    composition is the reference's bit for bit."""

    KINDS = {"odom": N.TSDFL_MOTION_ODOM, "imu": N.TSDFL_MOTION_IMU, "scale": N.TSDFL_MOTION_SCALE,
             "scale_imu": N.TSDFL_MOTION_SCALE_IMU, "delta": N.TSDFL_MOTION_DELTA}

    def __init__(self, ctx: Context, a=(0.1,) * 12, seed: int = 0):
        self.ctx = ctx
        self.set_motion_parameters(*a)
        self.seed = int(seed)
        self.step = 0

    def set_motion_parameters(self, *a) -> None:
        if len(a) != 12:
            raise ValueError("12 motion parameters")
        self.a = np.asarray(a, np.float32)

    def distributions(self, kind: str, inputs, time_diff: float = 0.0) -> N.Motion:
        """(mean, stddev) of the six draws as the overload `kind` sets them up:
        odom (linear.x, angular.z), imu (linear_vel, angular_yaw), scale
        (lin_scale, ang_scale), scale_imu (lin_scale, delta_roll, delta_pitch,
        delta_yaw), delta (dx, dy, dz, roll, pitch, yaw, lin_base_noise,
        ang_base_noise)."""
        x = np.ascontiguousarray(inputs, np.float64)
        m = N.Motion()
        N.check(N.lib().tsdfl_motion_model(self.KINDS[kind], _ptr(self.a), _ptr(x), x.shape[0], time_diff,
                                           C.byref(m)))
        return m

    def update(self, particles: np.ndarray, motion: N.Motion, step: int | None = None) -> np.ndarray:
        """Moves particles (P, 7) float32 in place with device-drawn noise."""
        if step is None:
            step = self.step
            self.step += 1
        N.check(N.lib().tsdfl_motion_update(self.ctx.handle, _ptr(particles), particles.shape[0], C.byref(motion),
                                            self.seed, int(step)))
        return particles

    def apply(self, particles: np.ndarray, draws: np.ndarray) -> np.ndarray:
        d = np.ascontiguousarray(draws, np.float64)
        if d.shape != (particles.shape[0], 6):
            raise ValueError("draws must be (P, 6)")
        N.check(N.lib().tsdfl_motion_apply(self.ctx.handle, _ptr(particles), particles.shape[0], _ptr(d)))
        return particles


class FilterBatch:
    """Many independent filters updated together (tsdfl_batch): scoring in one
    persistent launch, optionally replayed from a captured CUDA graph.  Each
    filter is a dict of device buffers given as integer pointers -- particles
    (P x 7 float32), points (N x 3), pose_out (6 floats or 0), u0 (1 float or 0
    for no resampling), resampled (cap x 7), count (1 uint32) -- plus map
    (DeviceMap), P, N, cap, tf (16 floats) and model (a_hit, a_range, a_max,
    max_range)."""

    def __init__(self, ctx: Context, filters):
        self.ctx = ctx
        arr = (N.Filter * max(len(filters), 1))()
        self._maps = []
        for i, f in enumerate(filters):
            d = arr[i]
            d.map = f["map"].handle
            self._maps.append(f["map"])
            d.model = N.Model(*f.get("model", (0.9, 0.1, 0.0, 100.0)))
            tf = np.asarray(f["tf"], np.float32).reshape(16)
            for k in range(16):
                d.tf[k] = float(tf[k])
            d.d_particles = f["particles"]
            d.P = f["P"]
            d.d_points = f["points"]
            d.N = f["N"]
            d.d_pose_out = f.get("pose_out") or None
            d.d_u0 = f.get("u0") or None
            d.d_resampled = f.get("resampled") or None
            d.resample_cap = f.get("cap", 0)
            d.d_count = f.get("count") or None
        h = C.c_void_p()
        N.check(N.lib().tsdfl_batch_create(ctx.handle, arr, len(filters), 0, C.byref(h)))
        self.handle = h

    def run(self) -> None:
        N.check(N.lib().tsdfl_batch_run(self.handle))

    def capture(self) -> None:
        N.check(N.lib().tsdfl_batch_capture(self.handle))

    def set_tiles(self, chunk: int, group: int) -> None:
        N.check(N.lib().tsdfl_batch_set_tiles(self.handle, chunk, group))

    def autotune(self):
        c, g, t = C.c_int(), C.c_int(), C.c_float()
        N.check(N.lib().tsdfl_batch_autotune(self.handle, C.byref(c), C.byref(g), C.byref(t)))
        return c.value, g.value, t.value

    def hits(self, i: int, P: int) -> np.ndarray:
        out = np.zeros(P, np.uint32)
        N.check(N.lib().tsdfl_batch_hits(self.handle, i, _ptr(out)))
        return out

    def info(self):
        a, b, o = C.c_uint32(), C.c_uint32(), C.c_uint32()
        N.check(N.lib().tsdfl_batch_info(self.handle, C.byref(a), C.byref(b), C.byref(o)))
        n1 = C.c_uint32()
        N.check(N.lib().tsdfl_batch_single(self.handle, C.byref(n1)))
        return {"segments": a.value, "batches": b.value, "outside": o.value, "single": n1.value}

    def close(self) -> None:
        if getattr(self, "handle", None):
            N.lib().tsdfl_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LocalizationServer:
    """Served sessions (tsdfl_server): particles, map and draws of every
    session resident on the device; submissions queued and launched in
    continuous batches by poll()."""

    def __init__(self, ctx: Context, hbm_budget: int, max_sessions: int, max_points: int, max_wait_ms: float = 0.0,
                 max_queue: int = 4):
        self.ctx = ctx
        cfg = N.ServerConfig(int(hbm_budget), int(max_sessions), int(max_points), float(max_wait_ms), int(max_queue))
        h = C.c_void_p()
        N.check(N.lib().tsdfl_server_create(ctx.handle, C.byref(cfg), C.byref(h)))
        self.handle = h
        self._maps = []

    def open(self, device_map, particles: np.ndarray, tf, model=(0.9, 0.1, 0.0, 100.0), seed: int = 0) -> int:
        p = _f32(particles, 7)
        t = np.ascontiguousarray(np.asarray(tf, np.float32).reshape(16))
        sid = C.c_uint32()
        m = N.Model(*model)
        N.check(N.lib().tsdfl_session_open(self.handle, device_map.handle, _ptr(p), p.shape[0], _ptr(t), C.byref(m),
                                           int(seed), C.byref(sid)))
        self._maps.append(device_map)
        return sid.value

    def close_session(self, sid: int) -> None:
        N.check(N.lib().tsdfl_session_close(self.handle, sid))

    def submit(self, sid: int, points: np.ndarray):
        """The ticket, or None when the submission is refused."""
        pts = _f32(points, 3)
        t = C.c_uint64()
        rc = N.lib().tsdfl_session_submit(self.handle, sid, _ptr(pts), pts.shape[0], C.byref(t))
        if rc == N.TSDFL_ERR_CAPACITY:
            return None
        N.check(rc)
        return t.value

    def poll(self) -> int:
        n = C.c_size_t()
        N.check(N.lib().tsdfl_server_poll(self.handle, C.byref(n)))
        return n.value

    def result(self, ticket: int):
        """(pose (6,), latency ms, status), or None while not published."""
        pose = np.zeros(6, np.float32)
        lat = C.c_double()
        st = C.c_int()
        rc = N.lib().tsdfl_server_result(self.handle, ticket, _ptr(pose), C.byref(lat), C.byref(st))
        if rc != N.TSDFL_OK:
            return None
        return pose, lat.value, st.value

    def particles(self, sid: int) -> np.ndarray:
        cnt = C.c_size_t()
        N.lib().tsdfl_session_particles(self.handle, sid, None, 0, C.byref(cnt))
        out = np.zeros((max(cnt.value, 1), 7), np.float32)
        N.check(N.lib().tsdfl_session_particles(self.handle, sid, _ptr(out), out.shape[0], C.byref(cnt)))
        return out[:cnt.value]

    def stats(self) -> dict:
        a, r, p, b = C.c_uint64(), C.c_uint64(), C.c_uint64(), C.c_uint64()
        rate = C.c_double()
        N.check(N.lib().tsdfl_server_stats(self.handle, C.byref(a), C.byref(r), C.byref(p), C.byref(b),
                                           C.byref(rate)))
        return {"accepted": a.value, "refused": r.value, "published": p.value, "batches": b.value,
                "rate": rate.value}

    @staticmethod
    def draw(seed: int, k: int, P: int) -> float:
        return float(N.lib().tsdfl_server_draw(int(seed), int(k), int(P)))

    def close(self) -> None:
        if getattr(self, "handle", None):
            N.lib().tsdfl_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pose_array(ctx: Context, particles: np.ndarray) -> np.ndarray:
    """mcl_3d.cpp:429-449: the particles as geometry_msgs::Pose records, (P, 7)
    doubles: position, then the setRPY quaternion x, y, z, w."""
    p = _f32(particles, 7)
    out = np.zeros((p.shape[0], 7), np.float64)
    N.check(N.lib().tsdfl_pose_array(ctx.handle, _ptr(p), p.shape[0], _ptr(out)))
    return out


def code_values(sigma: float = 0.1, init_value: float = 0.0) -> np.ndarray:
    out = np.zeros(601, np.float32)
    N.check(N.lib().tsdfl_code_values(sigma, init_value, _ptr(out)))
    return out


def build_map_codes(chunk_pos: np.ndarray, chunks: np.ndarray, edge: int, voxel_mm: int, sigma: float = 0.1,
                    want_free: bool = True):
    """createTSDFMap's likelihood map from TSDF chunks (map_util.h:17-154):
    returns (coef, grid_occ, codes, free_xyz)."""
    lib = N.lib()
    pos = np.ascontiguousarray(chunk_pos, dtype=np.int32)
    raw = np.ascontiguousarray(chunks, dtype=np.uint32)
    n = pos.shape[0]
    coef = N.MapCoef()
    go = C.c_void_p()
    cd = C.c_void_p()
    fr = C.c_void_p()
    nf = C.c_size_t()
    N.check(lib.tsdfl_build_map_codes(_ptr(pos), _ptr(raw), n, edge, voxel_mm, sigma, C.byref(coef), C.byref(go),
                                      C.byref(cd), C.byref(fr) if want_free else None,
                                      C.byref(nf) if want_free else None))
    try:
        g = np.ctypeslib.as_array(C.cast(go, C.POINTER(C.c_int32)), (max(coef.grid_occ_size, 1),))
        grid_occ = g[: coef.grid_occ_size].copy()
        c = np.ctypeslib.as_array(C.cast(cd, C.POINTER(C.c_uint16)), (max(coef.data_size, 1),))
        codes = c[: coef.data_size].copy()
        free_xyz = np.zeros((0, 3), np.float32)
        if want_free and nf.value:
            f = np.ctypeslib.as_array(C.cast(fr, C.POINTER(C.c_float)), (nf.value * 3,))
            free_xyz = f.reshape(-1, 3).copy()
    finally:
        lib.tsdfl_free(go)
        lib.tsdfl_free(cd)
        if want_free:
            lib.tsdfl_free(fr)
    return coef, grid_occ, codes, free_xyz


def read_map_h5(path) -> tuple[np.ndarray, np.ndarray, int]:
    """The TSDF chunks of a map file in the reference's HDF5 layout (group
    "/map", one dataset of edge^3 raw cells per chunk named "<x>_<y>_<z>";
    global_map.cpp, map_util.h:17-113), read without the HDF5 library:
    (chunk_pos (n, 3) int32, chunks (n, edge^3) uint32, edge), in the order
    createTSDFMap visits them."""
    lib = N.lib()
    pos = C.c_void_p()
    raw = C.c_void_p()
    n = C.c_size_t()
    edge = C.c_int32()
    N.check(lib.tsdfl_read_map_h5(str(path).encode(), C.byref(pos), C.byref(raw), C.byref(n), C.byref(edge)))
    try:
        cells = edge.value ** 3
        k = n.value
        p = np.ctypeslib.as_array(C.cast(pos, C.POINTER(C.c_int32)), (max(k, 1) * 3,))[: 3 * k]
        r = np.ctypeslib.as_array(C.cast(raw, C.POINTER(C.c_uint32)), (max(k * cells, 1),))[: k * cells]
        return p.reshape(k, 3).copy(), r.reshape(k, cells).copy(), edge.value
    finally:
        lib.tsdfl_free(pos)
        lib.tsdfl_free(raw)


def load_map_h5(ctx: Context, path, voxel_mm: int = 64, sigma: float = 0.1, dense: bool = True):
    """createTSDFMap (map_util.h:17-154) from a map file: the device map and the
    free-space cell positions.  voxel_mm is the map's resolution in millimetres
    (MAP_RESOLUTION, 64 in the reference)."""
    chunk_pos, chunks, edge = read_map_h5(path)
    coef, grid_occ, codes, free_xyz = build_map_codes(chunk_pos, chunks, edge, voxel_mm, sigma)
    return DeviceMap(ctx, coef, grid_occ, codes=codes, sigma=sigma, dense=dense), free_xyz
