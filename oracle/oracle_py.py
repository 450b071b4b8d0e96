"""TEST INFRASTRUCTURE ONLY: ctypes binding of the oracle libraries.

  oracle/_build/liboracle.so  CPU restatement of the reference sensor update
  oracle/_ref/libref.so       the reference's own CPU sources (where built)

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU baseline.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
P = C.c_void_p
SZ = C.c_size_t


class Coef(C.Structure):
    _fields_ = [
        ("dim_x", C.c_uint64), ("dim_y", C.c_uint64), ("dim_z", C.c_uint64),
        ("min_x", C.c_float), ("min_y", C.c_float), ("min_z", C.c_float),
        ("max_x", C.c_float), ("max_y", C.c_float), ("max_z", C.c_float),
        ("resolution", C.c_float), ("init_value", C.c_float),
        ("up_dim_x", C.c_uint64), ("up_dim_y", C.c_uint64), ("up_dim_z", C.c_uint64), ("up_dim_2", C.c_uint64),
        ("sub_dim", C.c_uint64), ("sub_dim_2", C.c_uint64),
        ("grid_occ_size", C.c_uint64), ("data_size", C.c_uint64),
    ]


class Model(C.Structure):
    _fields_ = [("a_hit", C.c_float), ("a_range", C.c_float), ("a_max", C.c_float), ("max_range", C.c_float)]


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def coef_from(src) -> Coef:
    """Copy of a MapCoef-like ctypes structure (same 120-byte layout)."""
    c = Coef()
    C.memmove(C.byref(c), C.byref(src), C.sizeof(Coef))
    return c


_orc = None
_ref = None


def oracle() -> C.CDLL:
    global _orc
    if _orc is None:
        path = HERE / "_build" / "liboracle.so"
        if not path.exists():
            raise ImportError("oracle/_build/liboracle.so is not built")
        L = C.CDLL(str(path))
        L.orc_f2u_x86.restype = C.c_uint64
        L.orc_f2u_x86.argtypes = [C.c_float]
        L.orc_map_coef_init.argtypes = [C.POINTER(Coef), P, P, C.c_float, C.c_float]
        L.orc_map_set_data.argtypes = [C.POINTER(Coef), P, P, SZ, C.POINTER(P), C.POINTER(SZ)]
        L.orc_get_index.restype = C.c_uint64
        L.orc_get_index.argtypes = [C.POINTER(Coef), P, C.c_float, C.c_float, C.c_float]
        L.orc_get_entry.restype = C.c_float
        L.orc_get_entry.argtypes = [C.POINTER(Coef), P, P, C.c_float, C.c_float, C.c_float]
        L.orc_particle_pose.argtypes = [P, P, P]
        L.orc_evaluate.argtypes = [C.POINTER(Coef), P, P, C.POINTER(Model), P, SZ, P, SZ, P, P, P, P, P, P, C.c_int]
        L.orc_likelihood_value.restype = C.c_float
        L.orc_likelihood_value.argtypes = [C.c_int16, C.c_float]
        L.orc_likelihood_init.restype = C.c_float
        L.orc_likelihood_init.argtypes = [C.c_float]
        L.orc_build_map_from_chunks.argtypes = [P, P, SZ, C.c_int, C.c_int, C.c_float, C.POINTER(Coef),
                                                C.POINTER(P), C.POINTER(P), C.POINTER(P), C.POINTER(SZ)]
        L.orc_chunk_tuples.restype = SZ
        L.orc_chunk_tuples.argtypes = [P, P, SZ, C.c_int, C.c_int, C.c_float, P, P, P, C.POINTER(P), C.POINTER(P),
                                       C.POINTER(SZ)]
        L.orc_resample_systematic.restype = SZ
        L.orc_resample_systematic.argtypes = [P, SZ, C.c_float, P, SZ]
        L.orc_resample_wheel.restype = None
        L.orc_resample_wheel.argtypes = [P, SZ, P, P]
        L.orc_resample_residual.restype = SZ
        L.orc_resample_residual.argtypes = [P, SZ, P, SZ, P]
        L.orc_resample_metropolis.restype = None
        L.orc_resample_metropolis.argtypes = [P, SZ, C.c_uint32, P, P, P]
        L.orc_resample_rejection.restype = C.c_int
        L.orc_resample_rejection.argtypes = [P, SZ, P, P, P, C.c_uint32, P]
        L.orc_pose_array.restype = None
        L.orc_pose_array.argtypes = [P, SZ, P]
        L.orc_motion_apply.restype = None
        L.orc_motion_apply.argtypes = [P, SZ, P]
        L.orc_reduce_scan.restype = SZ
        L.orc_reduce_scan.argtypes = [P, P, SZ, C.c_float, C.c_int, P, SZ]
        L.orc_subsample_indices.restype = None
        L.orc_subsample_indices.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32, P]
        L.orc_resample_residual_systematic.restype = SZ
        L.orc_resample_residual_systematic.argtypes = [P, SZ, C.c_float, P, SZ]
        _orc = L
    return _orc


def reference_available() -> bool:
    return (HERE / "_ref" / "libref.so").exists()


def reference() -> C.CDLL:
    global _ref
    if _ref is None:
        path = HERE / "_ref" / "libref.so"
        if not path.exists():
            raise ImportError("oracle/_ref/libref.so is not built (the reference tree is not on this machine)")
        L = C.CDLL(str(path))
        L.ref_map_create.restype = P
        L.ref_map_create.argtypes = [P, P, C.c_float, C.c_float, P, SZ]
        L.ref_map_destroy.argtypes = [P]
        L.ref_map_from_slots.restype = P
        L.ref_map_from_slots.argtypes = [P, P, P]
        L.ref_map_coef.argtypes = [P, P]
        L.ref_map_grid_occ.restype = P
        L.ref_map_grid_occ.argtypes = [P]
        L.ref_map_data.restype = P
        L.ref_map_data.argtypes = [P]
        L.ref_map_get_entry.restype = C.c_float
        L.ref_map_get_entry.argtypes = [P, C.c_float, C.c_float, C.c_float]
        L.ref_evaluate.restype = C.c_int
        L.ref_evaluate.argtypes = [P, P, P, SZ, P, SZ, P, P, P, P, C.c_int]
        L.ref_draw_u0.restype = C.c_float
        L.ref_draw_u0.argtypes = [C.c_uint32, SZ]
        L.ref_resample_systematic.restype = SZ
        L.ref_resample_systematic.argtypes = [P, SZ, C.c_uint32, P, SZ]
        L.ref_draw_u01.restype = C.c_float
        L.ref_draw_u01.argtypes = [C.c_uint32]
        L.ref_resample_residual_systematic.restype = SZ
        L.ref_resample_residual_systematic.argtypes = [P, SZ, C.c_uint32, P, SZ]
        for name in ("ref_resample_wheel", "ref_resample_residual", "ref_resample_rejection"):
            getattr(L, name).restype = SZ
            getattr(L, name).argtypes = [P, SZ, C.c_uint32, P, SZ]
        L.ref_resample_metropolis.restype = SZ
        L.ref_resample_metropolis.argtypes = [P, SZ, C.c_uint32, C.c_uint32, P, SZ]
        L.ref_resample_next.restype = C.c_uint32
        L.ref_resample_next.argtypes = [C.c_int, P, SZ, C.c_uint32, C.c_uint32]
        L.ref_draws_wheel.argtypes = [C.c_uint32, SZ, P]
        L.ref_draws_residual.argtypes = [C.c_uint32, SZ, SZ, P]
        L.ref_draws_metropolis.argtypes = [C.c_uint32, SZ, C.c_uint32, P, P]
        L.ref_draw_source_create.restype = P
        L.ref_draw_source_create.argtypes = [C.c_uint32, SZ]
        L.ref_draw_source_destroy.argtypes = [P]
        L.ref_motion_update.restype = None
        L.ref_motion_update.argtypes = [P, SZ, P]
        L.ref_reduce_scan.restype = SZ
        L.ref_reduce_scan.argtypes = [P, P, SZ, C.c_float, P, SZ]
        L.ref_omp_threads.restype = C.c_int
        _ref = L
    return _ref


# ------------------------------------------------------------------ restatement

class OracleMap:
    """A map in the reference's float-slot representation."""

    def __init__(self, coef: Coef, grid_occ: np.ndarray, data: np.ndarray):
        self.coef = coef
        self.grid_occ = np.ascontiguousarray(grid_occ, np.int32)
        self.data = np.ascontiguousarray(data, np.float32)

    @staticmethod
    def from_tuples(mn, mx, res: float, init: float, xyzv: np.ndarray) -> "OracleMap":
        L = oracle()
        c = Coef()
        L.orc_map_coef_init(C.byref(c), _ptr(np.asarray(mn, np.float32)), _ptr(np.asarray(mx, np.float32)), res,
                            init)
        go = np.zeros(max(c.grid_occ_size, 1), np.int32)
        t = np.ascontiguousarray(xyzv, np.float32)
        dp = P()
        skipped = SZ()
        rc = L.orc_map_set_data(C.byref(c), _ptr(go), _ptr(t), t.shape[0], C.byref(dp), C.byref(skipped))
        if rc != 0:
            raise RuntimeError("Upper voxel index overflow!")
        data = np.zeros(0, np.float32)
        if dp.value:
            data = np.ctypeslib.as_array(C.cast(dp, C.POINTER(C.c_float)), (max(c.data_size, 1),))[
                : c.data_size].copy()
            C.CDLL(None).free(dp)
        m = OracleMap(c, go[: c.grid_occ_size], data)
        m.skipped = skipped.value
        return m

    @staticmethod
    def from_chunks(chunk_pos: np.ndarray, chunks: np.ndarray, voxel_mm: int = 64, sigma: float = 0.1,
                    edge: int = 64):
        """createTSDFMap (map_util.h:17-154) on chunks of edge^3 cells (the
        reference's CHUNK_SIZE is 64): (map, free-space cells)."""
        L = oracle()
        c = Coef()
        go, dp, fp = P(), P(), P()
        nf = SZ()
        pos = np.ascontiguousarray(chunk_pos, np.int32)
        raw = np.ascontiguousarray(chunks, np.uint32)
        rc = L.orc_build_map_from_chunks(_ptr(pos), _ptr(raw), pos.shape[0], edge, voxel_mm, sigma, C.byref(c),
                                         C.byref(go), C.byref(dp), C.byref(fp), C.byref(nf))
        if rc != 0:
            raise RuntimeError("Upper voxel index overflow!")
        libc = C.CDLL(None)
        g = np.ctypeslib.as_array(C.cast(go, C.POINTER(C.c_int32)), (max(c.grid_occ_size, 1),))[
            : c.grid_occ_size].copy()
        d = np.zeros(0, np.float32)
        if dp.value:
            d = np.ctypeslib.as_array(C.cast(dp, C.POINTER(C.c_float)), (max(c.data_size, 1),))[: c.data_size].copy()
        f = np.ctypeslib.as_array(C.cast(fp, C.POINTER(C.c_float)), (max(nf.value, 1) * 3,))[
            : 3 * nf.value].reshape(-1, 3).copy()
        for p in (go, dp, fp):
            if p.value:
                libc.free(p)
        return OracleMap(c, g, d), f

    def get_index(self, x, y, z) -> int:
        return oracle().orc_get_index(C.byref(self.coef), _ptr(self.grid_occ), x, y, z)

    def get_entry(self, x, y, z) -> float:
        d = self.data if self.data.size else None
        return oracle().orc_get_entry(C.byref(self.coef), _ptr(self.grid_occ), _ptr(d), x, y, z)


def evaluate(m: OracleMap, particles: np.ndarray, points: np.ndarray, tf, model=(0.9, 0.1, 0.0, 100.0),
             want_idx: bool = False, threads: int = 0) -> dict:
    """TSDFEvaluator::evaluate CPU path; particles (P,7) float32 updated in place."""
    L = oracle()
    Pn, Nn = particles.shape[0], points.shape[0]
    pts = np.ascontiguousarray(points, np.float32)
    tfa = np.ascontiguousarray(np.asarray(tf, np.float32).reshape(16))
    raw = np.zeros(Pn, np.float32)
    hits = np.zeros(Pn, np.uint32)
    s64 = np.zeros(Pn, np.float64)
    idx = np.zeros((Pn, Nn), np.uint64) if want_idx else None
    pose = np.zeros(6, np.float32)
    mdl = Model(*model)
    d = m.data if m.data.size else None
    rc = L.orc_evaluate(C.byref(m.coef), _ptr(m.grid_occ), _ptr(d), C.byref(mdl), _ptr(particles), Pn, _ptr(pts),
                        Nn, _ptr(tfa), _ptr(raw), _ptr(hits), _ptr(idx), _ptr(s64), _ptr(pose), threads)
    return {"rc": rc, "raw": raw, "hits": hits, "sum64": s64, "voxel_index": idx, "pose": pose}


def subsample_indices(seed: int, i: int, N: int, K: int) -> np.ndarray:
    """The K scan indices particle i keeps under the library's seeded
    subsampling rule."""
    out = np.zeros(max(K, 1), np.uint32)
    oracle().orc_subsample_indices(seed, i, N, K, _ptr(out))
    return out[:K]


def evaluate_subsampled(m: OracleMap, particles: np.ndarray, points: np.ndarray, tf, K: int, seed: int,
                        model=(0.9, 0.1, 0.0, 100.0)) -> dict:
    """Every particle scored on its own K kept points (evaluatePose's loop per
    particle): raw float sums, hits and FP64 sums; weights normalised over the
    particles as TSDFEvaluator::evaluate does."""
    P, N = particles.shape[0], points.shape[0]
    raw = np.zeros(P, np.float32)
    hits = np.zeros(P, np.uint32)
    s64 = np.zeros(P, np.float64)
    pts = np.ascontiguousarray(points, np.float32)
    for i in range(P):
        idx = subsample_indices(seed, i, N, K)
        r = evaluate(m, np.ascontiguousarray(particles[i:i + 1]).copy(), pts[idx], tf, model, threads=1)
        raw[i], hits[i], s64[i] = r["raw"][0], r["hits"][0], r["sum64"][0]
    return {"raw": raw, "hits": hits, "sum64": s64}


def particle_pose(particle7, tf) -> np.ndarray:
    out = np.zeros(12, np.float32)
    oracle().orc_particle_pose(_ptr(np.ascontiguousarray(particle7, np.float32)),
                               _ptr(np.ascontiguousarray(np.asarray(tf, np.float32).reshape(16))), _ptr(out))
    return out


def resample_systematic(weights: np.ndarray, u0: float, cap: int | None = None) -> np.ndarray:
    w = np.ascontiguousarray(weights, np.float32)
    cap = cap if cap is not None else 2 * w.shape[0] + 16
    out = np.zeros(max(cap, 1), np.uint32)
    n = oracle().orc_resample_systematic(_ptr(w), w.shape[0], np.float32(u0), _ptr(out), cap)
    if n == (1 << 64) - 1:
        raise RuntimeError("U stopped advancing")
    return out[:n]


def resample_residual_systematic(weights: np.ndarray, u0: float, cap: int | None = None) -> np.ndarray:
    w = np.ascontiguousarray(weights, np.float32)
    cap = cap if cap is not None else 2 * w.shape[0] + 16
    out = np.zeros(max(cap, 1), np.uint32)
    n = oracle().orc_resample_residual_systematic(_ptr(w), w.shape[0], np.float32(u0), _ptr(out), cap)
    if n == (1 << 64) - 1:
        raise RuntimeError("a particle count reaches 2^32")
    return out[: min(n, cap)] if n > cap else out[:n]


def reduce_scan(xyz: np.ndarray, ring: np.ndarray, cell: float = 0.064, own_ring: bool = False) -> np.ndarray:
    """tsdf_evaluator.cpp:304-376: the reduced points, ring-major, cloud order."""
    x = np.ascontiguousarray(xyz, np.float32)
    r = np.ascontiguousarray(ring, np.int16)
    out = np.zeros((max(x.shape[0], 1), 3), np.float32)
    n = oracle().orc_reduce_scan(_ptr(x), _ptr(r), x.shape[0], np.float32(cell), int(own_ring), _ptr(out),
                                 out.shape[0])
    if n == (1 << 64) - 1:
        raise ValueError("ring outside [0, 64)")
    return out[:n].copy()


def pose_array(particles: np.ndarray) -> np.ndarray:
    """mcl_3d.cpp:433-449: (P, 7) doubles, position and setRPY quaternion (x, y, z, w)."""
    p = np.ascontiguousarray(particles, np.float32)
    out = np.zeros((p.shape[0], 7), np.float64)
    oracle().orc_pose_array(_ptr(p), p.shape[0], _ptr(out))
    return out


def motion_apply(particles: np.ndarray, draws: np.ndarray) -> np.ndarray:
    """particle_cloud.cpp:499-617 on given draws (P x 6 doubles); returns new particles."""
    p = np.ascontiguousarray(particles, np.float32).copy()
    d = np.ascontiguousarray(draws, np.float64)
    assert d.shape == (p.shape[0], 6)
    oracle().orc_motion_apply(_ptr(p), p.shape[0], _ptr(d))
    return p


def ref_motion_update(particles: np.ndarray, delta) -> np.ndarray:
    """The reference's ParticleCloud::motion_update with zero noise: every
    particle moves by exactly delta = (dx, dy, dz, roll, pitch, yaw) (floats)."""
    p = np.ascontiguousarray(particles, np.float32).copy()
    d = np.ascontiguousarray(delta, np.float32)
    reference().ref_motion_update(_ptr(p), p.shape[0], _ptr(d))
    return p


def resample_wheel(w: np.ndarray, draws: np.ndarray) -> np.ndarray:
    """WheelResampler on given draws (doubles in [0, 1)): source index per output."""
    w = np.ascontiguousarray(w, np.float32)
    d = np.ascontiguousarray(draws, np.float64)
    out = np.zeros(w.shape[0], np.uint32)
    oracle().orc_resample_wheel(_ptr(w), w.shape[0], _ptr(d), _ptr(out))
    return out


def resample_residual(w: np.ndarray, draws: np.ndarray):
    """ResidualResampler on given draws (particle indices): (indices, draws used)."""
    w = np.ascontiguousarray(w, np.float32)
    d = np.ascontiguousarray(draws, np.uint32)
    out = np.zeros(w.shape[0], np.uint32)
    used = oracle().orc_resample_residual(_ptr(w), w.shape[0], _ptr(d), d.shape[0], _ptr(out))
    if used == (1 << 64) - 1:
        raise ValueError("the draws ran out")
    return out, used


def resample_metropolis(w: np.ndarray, steps: int, u: np.ndarray, j: np.ndarray) -> np.ndarray:
    w = np.ascontiguousarray(w, np.float32)
    u = np.ascontiguousarray(u, np.float32)
    j = np.ascontiguousarray(j, np.uint32)
    out = np.zeros(w.shape[0], np.uint32)
    oracle().orc_resample_metropolis(_ptr(w), w.shape[0], steps, _ptr(u), _ptr(j), _ptr(out))
    return out


REJECTION_ROUNDS = 1 << 20
STREAMS = {"motion": 0x6D6F74696F6E0001, "wheel": 0x776865656C000001, "residual": 0x7265736964000001,
           "metropolis": 0x6D6574726F000001, "rejection": 0x72656A6563000001}


def resample_rejection_philox(w: np.ndarray, seed: int) -> np.ndarray:
    """RejectionResampler with the device's Philox draws (counter (i, t), key (seed, stream))."""
    w = np.ascontiguousarray(w, np.float32)
    src = np.array([seed, STREAMS["rejection"], w.shape[0]], np.uint64)
    out = np.zeros(w.shape[0], np.uint32)
    L = oracle()
    rc = L.orc_resample_rejection(_ptr(w), w.shape[0], C.cast(L.orc_philox_u, P), C.cast(L.orc_philox_j, P),
                                  _ptr(src), REJECTION_ROUNDS, _ptr(out))
    if rc:
        raise ValueError("an output exceeded the proposal limit")
    return out


def resample_rejection_reference_draws(w: np.ndarray, seed: int) -> np.ndarray:
    """The oracle's RejectionResampler drawing from the reference's own generator
    and distributions (seeded mt19937), in the reference's order."""
    w = np.ascontiguousarray(w, np.float32)
    R = reference()
    src = R.ref_draw_source_create(seed, w.shape[0])
    try:
        out = np.zeros(w.shape[0], np.uint32)
        rc = oracle().orc_resample_rejection(_ptr(w), w.shape[0], C.cast(R.ref_draw_source_u, P),
                                             C.cast(R.ref_draw_source_j, P), src, REJECTION_ROUNDS, _ptr(out))
        if rc:
            raise ValueError("an output exceeded the proposal limit")
        return out
    finally:
        R.ref_draw_source_destroy(src)


_DRAW_U = C.CFUNCTYPE(C.c_float, C.c_void_p, C.c_size_t, C.c_uint32)
_DRAW_J = C.CFUNCTYPE(C.c_uint32, C.c_void_p, C.c_size_t, C.c_uint32)


def resample_rejection_arrays(w: np.ndarray, u_seq, j_seq, record: bool = False):
    """The oracle's RejectionResampler consuming u and j draws from two sequences
    in order (the reference's consumption order).  With record=True the
    sequences are callables producing the next draw, and the draws consumed are
    returned alongside the indices."""
    w = np.ascontiguousarray(w, np.float32)
    used_u, used_j = [], []
    it_u = iter(u_seq) if not callable(u_seq) else None
    it_j = iter(j_seq) if not callable(j_seq) else None

    def du(_src, _i, _t):
        v = float(u_seq() if it_u is None else next(it_u))
        used_u.append(v)
        return v

    def dj(_src, _i, _t):
        v = int(j_seq() if it_j is None else next(it_j))
        used_j.append(v)
        return v

    fu, fj = _DRAW_U(du), _DRAW_J(dj)
    out = np.zeros(w.shape[0], np.uint32)
    rc = oracle().orc_resample_rejection(_ptr(w), w.shape[0], C.cast(fu, P), C.cast(fj, P), None,
                                         REJECTION_ROUNDS, _ptr(out))
    if rc:
        raise ValueError("an output exceeded the proposal limit")
    if record:
        return out, np.array(used_u, np.float32), np.array(used_j, np.uint32)
    return out


def ref_rejection_draw_callables(seed: int, M: int):
    """next-u and next-j callables over the reference's generator and distributions."""
    R = reference()
    src = R.ref_draw_source_create(seed, M)
    R.ref_draw_source_u.restype = C.c_float
    R.ref_draw_source_u.argtypes = [P, SZ, C.c_uint32]
    R.ref_draw_source_j.restype = C.c_uint32
    R.ref_draw_source_j.argtypes = [P, SZ, C.c_uint32]
    return (lambda: R.ref_draw_source_u(src, 0, 0)), (lambda: R.ref_draw_source_j(src, 0, 0)), \
        (lambda: R.ref_draw_source_destroy(src))


def ref_resample(kind: str, w: np.ndarray, seed: int, steps: int = 50) -> np.ndarray:
    """The reference's own Wheel/Residual/Metropolis/Rejection resampler, seeded."""
    w = np.ascontiguousarray(w, np.float32)
    out = np.zeros(w.shape[0], np.uint32)
    R = reference()
    if kind == "metropolis":
        n = R.ref_resample_metropolis(_ptr(w), w.shape[0], steps, seed, _ptr(out), out.shape[0])
    else:
        n = getattr(R, f"ref_resample_{kind}")(_ptr(w), w.shape[0], seed, _ptr(out), out.shape[0])
    assert n == w.shape[0]
    return out


def ref_resample_next(kind: int, w: np.ndarray, seed: int, steps: int = 50) -> int:
    """The seeded generator's next output after the reference's Wheel (0),
    Residual (1) or Metropolis (2) resampler ran."""
    w = np.ascontiguousarray(w, np.float32)
    return int(reference().ref_resample_next(kind, _ptr(w), w.shape[0], steps, seed))


def ref_draws(kind: str, seed: int, M: int, K: int = 0, steps: int = 50):
    """The draws the reference's resampler takes from mt19937(seed), in its order."""
    R = reference()
    if kind == "wheel":
        d = np.zeros(M, np.float64)
        R.ref_draws_wheel(seed, M, _ptr(d))
        return d
    if kind == "residual":
        d = np.zeros(K, np.uint32)
        R.ref_draws_residual(seed, M, K, _ptr(d))
        return d
    u = np.zeros(M * steps, np.float32)
    j = np.zeros(M * steps, np.uint32)
    R.ref_draws_metropolis(seed, M, steps, _ptr(u), _ptr(j))
    return u, j


PHILOX_M = (0xD2E7470EE14C6C93, 0xCA5A826395121157)
PHILOX_W = (0x9E3779B97F4A7C15, 0xBB67AE8584CAA73B)


def philox4x64_10(counter, key):
    """Philox4x64-10 (Salmon et al., SC 2011) of one counter block, vectorised
    over numpy uint64 arrays: counter 4 arrays, key 2 arrays or ints."""
    m64 = (1 << 64) - 1

    def as_int(v):
        a = np.asarray(v)
        return np.vectorize(int, otypes=[object])(a) if a.ndim else int(a)

    c = [as_int(v) for v in counter]
    k0, k1 = int(key[0]), int(key[1])
    for _ in range(10):
        p0 = c[0] * PHILOX_M[0]
        p1 = c[2] * PHILOX_M[1]
        c = [(p1 >> 64) ^ c[1] ^ k0, p1 & m64, (p0 >> 64) ^ c[3] ^ k1, p0 & m64]
        k0 = (k0 + PHILOX_W[0]) & m64
        k1 = (k1 + PHILOX_W[1]) & m64
    return [np.asarray(v, dtype=object).astype(np.uint64) for v in c]


def ref_reduce_scan(xyz: np.ndarray, ring: np.ndarray, cell: float = 0.064) -> np.ndarray:
    """The reference's own evaluateParticles reduction (oracle/_ref)."""
    x = np.ascontiguousarray(xyz, np.float32)
    r = np.ascontiguousarray(ring, np.int16)
    out = np.zeros((max(x.shape[0], 1), 3), np.float32)
    n = reference().ref_reduce_scan(_ptr(x), _ptr(r), x.shape[0], np.float32(cell), _ptr(out), out.shape[0])
    return out[:n].copy()


def chunk_tuples(chunk_pos: np.ndarray, chunks: np.ndarray, voxel_mm: int = 64, sigma: float = 0.1,
                 edge: int = 64) -> dict:
    """createTSDFMap up to its setData call (map_util.h:17-147): bounding box,
    init value, the (x, y, z, value) tuples in push order, free-space cells."""
    L = oracle()
    pos = np.ascontiguousarray(chunk_pos, np.int32)
    raw = np.ascontiguousarray(chunks, np.uint32)
    mn = np.zeros(3, np.float32)
    mx = np.zeros(3, np.float32)
    init = np.zeros(1, np.float32)
    tp, fp = P(), P()
    nf = SZ()
    n = L.orc_chunk_tuples(_ptr(pos), _ptr(raw), pos.shape[0], edge, voxel_mm, sigma, _ptr(mn), _ptr(mx),
                           _ptr(init), C.byref(tp), C.byref(fp), C.byref(nf))
    libc = C.CDLL(None)
    try:
        t = np.ctypeslib.as_array(C.cast(tp, C.POINTER(C.c_float)), (max(n, 1) * 4,))[: 4 * n].reshape(-1, 4).copy()
        f = np.ctypeslib.as_array(C.cast(fp, C.POINTER(C.c_float)), (max(nf.value, 1) * 3,))[
            : 3 * nf.value].reshape(-1, 3).copy()
    finally:
        for p in (tp, fp):
            if p.value:
                libc.free(p)
    return {"min": mn, "max": mx, "init": float(init[0]), "tuples": t, "free": f}


def likelihood_value(mm: int, sigma: float = 0.1) -> float:
    return oracle().orc_likelihood_value(mm, sigma)


def likelihood_init(sigma: float = 0.1) -> float:
    return oracle().orc_likelihood_init(sigma)


# ------------------------------------------------------------------ reference

class RefMap:
    """CudaSubVoxelMap<float,float> built by the reference's own ctor + setData."""

    @staticmethod
    def from_slots(coef, grid_occ: np.ndarray, data: np.ndarray) -> "RefMap":
        L = reference()
        self = RefMap.__new__(RefMap)
        c = coef_from(coef)
        go = np.ascontiguousarray(grid_occ, np.int32)
        d = np.ascontiguousarray(data, np.float32)
        self.h = L.ref_map_from_slots(C.byref(c), _ptr(go), _ptr(d))
        if not self.h:
            raise RuntimeError("reference map construction failed")
        self.coef = Coef()
        L.ref_map_coef(self.h, C.byref(self.coef))
        return self

    def __init__(self, mn, mx, res: float, init: float, xyzv: np.ndarray):
        L = reference()
        t = np.ascontiguousarray(xyzv, np.float32)
        self.h = L.ref_map_create(_ptr(np.asarray(mn, np.float32)), _ptr(np.asarray(mx, np.float32)), res, init,
                                  _ptr(t), t.shape[0])
        if not self.h:
            raise RuntimeError("Upper voxel index overflow!")
        self.coef = Coef()
        L.ref_map_coef(self.h, C.byref(self.coef))

    def __del__(self):
        if getattr(self, "h", None):
            reference().ref_map_destroy(self.h)
            self.h = None

    def grid_occ(self) -> np.ndarray:
        p = reference().ref_map_grid_occ(self.h)
        return np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_int32)), (max(self.coef.grid_occ_size, 1),))[
            : self.coef.grid_occ_size].copy()

    def data(self) -> np.ndarray:
        p = reference().ref_map_data(self.h)
        if not p:
            return np.zeros(0, np.float32)
        return np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_float)), (max(self.coef.data_size, 1),))[
            : self.coef.data_size].copy()

    def get_entry(self, x, y, z) -> float:
        return reference().ref_map_get_entry(self.h, x, y, z)

    def evaluate(self, particles: np.ndarray, points: np.ndarray, tf, model=(0.9, 0.1, 0.0, 100.0),
                 serial: bool = True) -> dict:
        L = reference()
        Pn = particles.shape[0]
        raw = np.zeros(Pn, np.float32)
        poses = np.zeros((Pn, 12), np.float32)
        pose = np.zeros(6, np.float32)
        mdl = np.asarray(model, np.float32)
        pts = np.ascontiguousarray(points, np.float32)
        tfa = np.ascontiguousarray(np.asarray(tf, np.float32).reshape(16))
        rc = L.ref_evaluate(self.h, _ptr(mdl), _ptr(particles), Pn, _ptr(pts), pts.shape[0], _ptr(tfa), _ptr(raw),
                            _ptr(poses), _ptr(pose), 1 if serial else 0)
        return {"rc": rc, "raw": raw, "laser_pose": poses, "pose": pose}


def ref_draw_u0(seed: int, m: int) -> float:
    return reference().ref_draw_u0(seed, m)


def ref_draw_u01(seed: int) -> float:
    return reference().ref_draw_u01(seed)


def ref_resample_residual_systematic(weights: np.ndarray, seed: int, cap: int | None = None) -> np.ndarray:
    w = np.ascontiguousarray(weights, np.float32)
    cap = cap if cap is not None else 2 * w.shape[0] + 16
    out = np.zeros(max(cap, 1), np.uint32)
    n = reference().ref_resample_residual_systematic(_ptr(w), w.shape[0], seed, _ptr(out), cap)
    return out[:n]


def ref_resample_systematic(weights: np.ndarray, seed: int, cap: int | None = None) -> np.ndarray:
    w = np.ascontiguousarray(weights, np.float32)
    cap = cap if cap is not None else 2 * w.shape[0] + 16
    out = np.zeros(max(cap, 1), np.uint32)
    n = reference().ref_resample_systematic(_ptr(w), w.shape[0], seed, _ptr(out), cap)
    return out[:n]
