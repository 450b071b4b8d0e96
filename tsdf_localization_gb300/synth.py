"""Seeded synthetic workloads (worlds, TSDF chunks, scans, particle clouds).

The reference is measured on recorded maps and scans that are not available
here; these generators produce inputs with the same shapes and value ranges.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _native as N

ROOM, BUILDING, WAREHOUSE, TUNNEL = 0, 1, 2, 3


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class World:
    def __init__(self, kind: int, seed: int):
        self._lib = N.synth_lib()
        self.handle = self._lib.tsyn_world_create(kind, seed)
        if not self.handle:
            raise ValueError(f"unknown world kind {kind}")
        lo = np.zeros(3, np.float32)
        hi = np.zeros(3, np.float32)
        pose = np.zeros(6, np.float32)
        nb = C.c_int32()
        self._lib.tsyn_world_info(self.handle, _ptr(lo), _ptr(hi), _ptr(pose), C.byref(nb))
        self.lo, self.hi, self.pose, self.n_boxes = lo, hi, pose, nb.value
        self.kind, self.seed = kind, seed

    def __del__(self):
        if getattr(self, "handle", None):
            self._lib.tsyn_world_destroy(self.handle)
            self.handle = None

    def sdf(self, x: float, y: float, z: float) -> float:
        return self._lib.tsyn_world_sdf(self.handle, x, y, z)

    def tsdf_chunks(self, voxel_mm: int, edge: int = 64, band_m: float = 0.65):
        """TSDF band as (chunk_pos (n,3) int32, raw (n, edge^3) uint32)."""
        pos = C.c_void_p()
        raw = C.c_void_p()
        n = self._lib.tsyn_tsdf_chunks(self.handle, voxel_mm, edge, band_m, C.byref(pos), C.byref(raw))
        cells = edge ** 3
        try:
            p = np.ctypeslib.as_array(C.cast(pos, C.POINTER(C.c_int32)), (max(n, 1) * 3,))[: 3 * n]
            r = np.ctypeslib.as_array(C.cast(raw, C.POINTER(C.c_uint32)), (max(n, 1) * cells,))[: n * cells]
            return p.reshape(n, 3).copy(), r.reshape(n, cells).copy()
        finally:
            self._lib.tsyn_free(pos)
            self._lib.tsyn_free(raw)

    def scan(self, pose6, rings: int, cols: int, vmin_deg: float = -15.0, vmax_deg: float = 15.0,
             min_range: float = 0.3, max_range: float = 80.0, sigma: float = 0.02, dropout: float = 0.0,
             seed: int = 0):
        """Ray-cast scan in the sensor frame: (xyz (n,3) float32, ring (n,) int16)."""
        cap = rings * cols
        xyz = np.zeros((cap, 3), np.float32)
        ring = np.zeros(cap, np.int16)
        p6 = np.ascontiguousarray(pose6, dtype=np.float32)
        n = self._lib.tsyn_scan(self.handle, _ptr(p6), rings, cols, vmin_deg, vmax_deg, min_range, max_range,
                                sigma, dropout, seed, _ptr(xyz), _ptr(ring))
        return xyz[:n].copy(), ring[:n].copy()

    def particles_free_space(self, n: int, clearance: float, zlo: float, zhi: float, rp_max: float, seed: int):
        out = np.zeros((n, 7), np.float32)
        self._lib.tsyn_particles_free_space(self.handle, clearance, zlo, zhi, rp_max, n, seed, _ptr(out))
        return out


def reduce_scan(xyz: np.ndarray, ring: np.ndarray, cell: float = 0.064) -> np.ndarray:
    """Host scan reduction used to make synthetic workloads: one point per ring and
    cell as in tsdf_evaluator.cpp:304-376, with every point's own ring (the
    TSDFL_SCAN_OWN_RING form; the reference's ring iterator skips with the range
    filter)."""
    lib = N.synth_lib()
    x = np.ascontiguousarray(xyz, np.float32)
    r = np.ascontiguousarray(ring, np.int16)
    out = np.zeros_like(x)
    n = lib.tsyn_reduce_scan(_ptr(x), _ptr(r), x.shape[0], cell, _ptr(out))
    return out[:n].copy()


def subsample(xyz: np.ndarray, m: int, seed: int) -> np.ndarray:
    lib = N.synth_lib()
    x = np.ascontiguousarray(xyz, np.float32)
    if x.shape[0] <= m:
        return x.copy()
    out = np.zeros((m, 3), np.float32)
    lib.tsyn_subsample_ordered(_ptr(x), x.shape[0], m, seed, _ptr(out))
    return out


def particles_gaussian(center6, sigma_xyz: float, sigma_rpy: float, n: int, seed: int) -> np.ndarray:
    lib = N.synth_lib()
    c = np.ascontiguousarray(center6, np.float32)
    out = np.zeros((n, 7), np.float32)
    lib.tsyn_particles_gaussian(_ptr(c), sigma_xyz, sigma_rpy, n, seed, _ptr(out))
    return out


IDENTITY_TF = np.eye(4, dtype=np.float32).reshape(16)


def sensor_tf(z_offset: float = 0.0) -> np.ndarray:
    """Sensor-to-base transform: the scanner z_offset above the base frame."""
    t = np.eye(4, dtype=np.float32)
    t[2, 3] = z_offset
    return t.reshape(16)


@dataclass
class Workload:
    """One sensor-update input: map (reference representation), scan, particles."""

    name: str
    coef: N.MapCoef
    grid_occ: np.ndarray
    codes: np.ndarray
    points: np.ndarray
    particles: np.ndarray
    tf: np.ndarray
    true_pose: np.ndarray
    voxel_mm: int
    extra: dict = field(default_factory=dict)

    def float_data(self, sigma: float = 0.1) -> np.ndarray:
        """The map's float slots as the reference stores them."""
        from .evaluator import code_values
        vals = np.append(code_values(sigma, self.coef.init_value), np.float32(self.coef.init_value))
        return vals[self.codes]


def make_workload(kind: int, seed: int, voxel_mm: int, n_points: int, n_particles: int, rings: int, cols: int,
                  sigma_xyz: float = 0.3, sigma_rpy_deg: float = 5.0, noise: float = 0.02, dropout: float = 0.0,
                  reduce_cell: float = 0.064, edge: int = 64, sensor_height: float = 0.0, name: str = "") -> Workload:
    """World -> TSDF chunks -> likelihood map -> ray-cast scan -> reduced scan
    -> Gaussian particles around the true pose."""
    from .evaluator import build_map_codes
    w = World(kind, seed)
    chunk_pos, chunks = w.tsdf_chunks(voxel_mm, edge)
    coef, grid_occ, codes, free_xyz = build_map_codes(chunk_pos, chunks, edge, voxel_mm, 0.1, want_free=False)
    del chunks
    true = w.pose.copy()
    sensor_pose = true.copy()
    sensor_pose[2] += sensor_height
    xyz, ring = w.scan(sensor_pose, rings, cols, sigma=noise, dropout=dropout, seed=seed + 1)
    pts = reduce_scan(xyz, ring, reduce_cell)
    pts = subsample(pts, n_points, seed + 2)
    parts = particles_gaussian(true, sigma_xyz, np.deg2rad(sigma_rpy_deg), n_particles, seed + 3)
    return Workload(name or f"kind{kind}", coef, grid_occ, codes, pts, parts, sensor_tf(sensor_height), true,
                    voxel_mm, {"n_chunks": int(chunk_pos.shape[0]), "raw_points": int(xyz.shape[0])})


def room_workload(seed: int = 1, n_particles: int = 1000, n_points: int = 2048) -> Workload:
    """20x20x4 m room at 0.064 m in 64^3 chunks, 16x1024 scan reduced to
    n_points, particles with sigma 0.3 m / 5 deg."""
    return make_workload(ROOM, seed, 64, n_points, n_particles, 16, 1024, edge=64, name="room20x20x4@0.064")


def global_workload(seed: int = 3, n_particles: int = 1_000_000, n_points: int = 2048) -> Workload:
    """Global localisation in the 100x100x10 m building at 0.05 m: a 2,048-point
    scan (64x2048 ray-cast, 1 % dropouts) and particles uniform over free space
    (0.3 m clearance, sensor heights of the lower storey), yaw uniform, roll and
    pitch within +-3 deg."""
    wl = building_workload(seed=seed, n_particles=1, n_points=n_points)
    w = World(BUILDING, seed)
    z = float(wl.true_pose[2])
    parts = w.particles_free_space(n_particles, 0.3, z - 0.3, z + 0.3, float(np.deg2rad(3.0)), seed + 7)
    return Workload("building100x100x10@0.05/global", wl.coef, wl.grid_occ, wl.codes, wl.points, parts, wl.tf,
                    wl.true_pose, wl.voxel_mm, dict(wl.extra, global_particles=n_particles))


def building_workload(seed: int = 2, n_particles: int = 100_000, n_points: int = 8192) -> Workload:
    """100x100x10 m building at 0.05 m in sparse 8^3 bricks, 64x2048 scan with 1%
    dropouts reduced to n_points, particles with sigma 0.3 m / 5 deg."""
    return make_workload(BUILDING, seed, 50, n_points, n_particles, 64, 2048, dropout=0.01, edge=8,
                         reduce_cell=0.05, name="building100x100x10@0.05")
