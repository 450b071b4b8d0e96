"""ctypes binding of libtsdfl.so (include/tsdfl.h) and libtsdfl_synth.so.

The CUDA library is the product: nothing here computes; a missing library is
an ImportError, never a silent fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB_DIR = Path(__file__).resolve().parent / "_lib"

TSDFL_OK = 0
TSDFL_ERR_INVALID_ARG = 1
TSDFL_ERR_OUT_OF_MEMORY = 2
TSDFL_ERR_DEGENERATE = 3
TSDFL_ERR_DEVICE = 4
TSDFL_ERR_TIMEOUT = 5
TSDFL_ERR_CAPACITY = 6
TSDFL_ERR_UNSUPPORTED = 7

TSDFL_MAP_DENSE = 1
TSDFL_MAP_FORCE_F32 = 2
TSDFL_MAP_F16 = 4
TSDFL_MAP_HASH = 8
TSDFL_MAP_GRID = 16
TSDFL_SUM_EXACT = 0
TSDFL_SUM_SERIAL = 1
TSDFL_EVAL_GENERIC = 4
TSDFL_NORM_LOG = 8
TSDFL_SCAN_OWN_RING = 1
TSDFL_MOTION_ODOM, TSDFL_MOTION_IMU, TSDFL_MOTION_SCALE, TSDFL_MOTION_SCALE_IMU, TSDFL_MOTION_DELTA = range(5)


class MapCoef(C.Structure):
    """CudaSubVoxelMap<float,float>::MapCoef (cuda_sub_voxel_map.h:22-50)."""

    _fields_ = [
        ("dim_x", C.c_uint64), ("dim_y", C.c_uint64), ("dim_z", C.c_uint64),
        ("min_x", C.c_float), ("min_y", C.c_float), ("min_z", C.c_float),
        ("max_x", C.c_float), ("max_y", C.c_float), ("max_z", C.c_float),
        ("resolution", C.c_float), ("init_value", C.c_float),
        ("up_dim_x", C.c_uint64), ("up_dim_y", C.c_uint64), ("up_dim_z", C.c_uint64), ("up_dim_2", C.c_uint64),
        ("sub_dim", C.c_uint64), ("sub_dim_2", C.c_uint64),
        ("grid_occ_size", C.c_uint64), ("data_size", C.c_uint64),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


assert C.sizeof(MapCoef) == 120


class Model(C.Structure):
    _fields_ = [("a_hit", C.c_float), ("a_range", C.c_float), ("a_max", C.c_float), ("max_range", C.c_float)]


class MapInfo(C.Structure):
    _fields_ = [("grid_occ_size", C.c_uint64), ("data_size", C.c_uint64), ("bricks", C.c_uint64),
                ("device_bytes", C.c_uint64), ("storage", C.c_int32), ("dense", C.c_int32),
                ("fast_index", C.c_int32), ("reserved", C.c_int32)]


class Motion(C.Structure):
    _fields_ = [("mean", C.c_double * 6), ("stddev", C.c_double * 6)]


class Filter(C.Structure):
    _fields_ = [("map", C.c_void_p), ("model", Model), ("tf", C.c_float * 16), ("d_particles", C.c_void_p),
                ("P", C.c_size_t), ("d_points", C.c_void_p), ("N", C.c_size_t), ("d_pose_out", C.c_void_p),
                ("d_u0", C.c_void_p), ("d_resampled", C.c_void_p), ("resample_cap", C.c_size_t),
                ("d_count", C.c_void_p)]


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget", C.c_size_t), ("max_sessions", C.c_size_t), ("max_points", C.c_size_t),
                ("max_wait_ms", C.c_double), ("max_queue", C.c_uint32)]


class EvalDebug(C.Structure):
    _fields_ = [("raw_weights", C.c_void_p), ("hits", C.c_void_p), ("voxel_index", C.c_void_p),
                ("laser_pose", C.c_void_p), ("weight_sum", C.c_double)]


P = C.c_void_p
SZ = C.c_size_t
I = C.c_int
F = C.c_float
U32 = C.c_uint32

# (name, restype, argtypes) of every entry point include/tsdfl.h declares
SIGNATURES = [
    ("tsdfl_last_error", C.c_char_p, []),
    ("tsdfl_version", C.c_char_p, []),
    ("tsdfl_ctx_create", I, [I, C.POINTER(P)]),
    ("tsdfl_ctx_destroy", I, [P]),
    ("tsdfl_ctx_set_stream", I, [P, P]),
    ("tsdfl_ctx_stream", P, [P]),
    ("tsdfl_ctx_sync", I, [P]),
    ("tsdfl_ctx_reserve", I, [P, SZ, SZ]),
    ("tsdfl_ctx_set_timing", I, [P, I]),
    ("tsdfl_ctx_last_timing", I, [P, C.POINTER(F)]),
    ("tsdfl_launch_count", C.c_uint64, []),
    ("tsdfl_ctx_workspace_bytes", I, [P, C.POINTER(SZ), C.POINTER(SZ)]),
    ("tsdfl_map_create", I, [P, C.POINTER(MapCoef), P, P, F, C.c_uint32, C.POINTER(P)]),
    ("tsdfl_map_create_codes", I, [P, C.POINTER(MapCoef), P, P, F, C.c_uint32, C.POINTER(P)]),
    ("tsdfl_map_destroy", I, [P]),
    ("tsdfl_map_get_info", I, [P, C.POINTER(MapInfo)]),
    ("tsdfl_build_map_codes", I, [P, P, SZ, I, I, F, C.POINTER(MapCoef), C.POINTER(P), C.POINTER(P),
                                  C.POINTER(P), C.POINTER(SZ)]),
    ("tsdfl_code_values", I, [F, F, P]),
    ("tsdfl_read_map_h5", I, [C.c_char_p, C.POINTER(P), C.POINTER(P), C.POINTER(SZ), C.POINTER(C.c_int32)]),
    ("tsdfl_free", None, [P]),
    ("tsdfl_evaluate", I, [P, P, C.POINTER(Model), P, SZ, P, SZ, P, C.c_uint32, P]),
    ("tsdfl_evaluate_debug", I, [P, P, C.POINTER(Model), P, SZ, P, SZ, P, C.c_uint32, P, C.POINTER(EvalDebug)]),
    ("tsdfl_evaluate_device", I, [P, P, C.POINTER(Model), P, SZ, P, SZ, P, C.c_uint32, P]),
    ("tsdfl_resample_systematic", I, [P, P, SZ, F, P, SZ, C.POINTER(SZ)]),
    ("tsdfl_resample_systematic_particles", I, [P, P, SZ, F, P, SZ, C.POINTER(SZ)]),
    ("tsdfl_resample_systematic_device", I, [P, P, SZ, F, P, SZ, P]),
    ("tsdfl_resample_systematic_static", I, [P, P, SZ, F, P, SZ, P]),
    ("tsdfl_resample_residual_systematic", I, [P, P, SZ, F, P, SZ, P]),
    ("tsdfl_resample_residual_systematic_device", I, [P, P, SZ, F, P, SZ, P]),
    ("tsdfl_best_particle_device", I, [P, P, SZ, P]),
    ("tsdfl_reduce_scan", I, [P, P, SZ, U32, U32, U32, F, U32, P, SZ, C.POINTER(SZ)]),
    ("tsdfl_reduce_scan_device", I, [P, P, SZ, U32, U32, U32, F, U32, P, SZ, P]),
    ("tsdfl_resample_wheel", I, [P, P, SZ, P, C.c_uint64, P]),
    ("tsdfl_resample_wheel_device", I, [P, P, SZ, P, C.c_uint64, P]),
    ("tsdfl_resample_residual", I, [P, P, SZ, P, SZ, C.c_uint64, P]),
    ("tsdfl_resample_residual_device", I, [P, P, SZ, P, SZ, C.c_uint64, P]),
    ("tsdfl_resample_metropolis", I, [P, P, SZ, U32, P, P, C.c_uint64, P]),
    ("tsdfl_resample_metropolis_device", I, [P, P, SZ, U32, P, P, C.c_uint64, P]),
    ("tsdfl_resample_rejection", I, [P, P, SZ, C.c_uint64, P]),
    ("tsdfl_resample_rejection_device", I, [P, P, SZ, C.c_uint64, P]),
    ("tsdfl_batch_create", I, [P, C.POINTER(Filter), SZ, U32, C.POINTER(P)]),
    ("tsdfl_batch_destroy", I, [P]),
    ("tsdfl_batch_run", I, [P]),
    ("tsdfl_batch_capture", I, [P]),
    ("tsdfl_batch_set_tiles", I, [P, I, I]),
    ("tsdfl_batch_autotune", I, [P, C.POINTER(I), C.POINTER(I), C.POINTER(F)]),
    ("tsdfl_batch_hits", I, [P, SZ, P]),
    ("tsdfl_batch_info", I, [P, C.POINTER(U32), C.POINTER(U32), C.POINTER(U32)]),
    ("tsdfl_batch_single", I, [P, C.POINTER(U32)]),
    ("tsdfl_server_create", I, [P, C.POINTER(ServerConfig), C.POINTER(P)]),
    ("tsdfl_server_destroy", I, [P]),
    ("tsdfl_session_open", I, [P, P, P, SZ, P, C.POINTER(Model), C.c_uint64, C.POINTER(U32)]),
    ("tsdfl_session_close", I, [P, U32]),
    ("tsdfl_session_submit", I, [P, U32, P, SZ, C.POINTER(C.c_uint64)]),
    ("tsdfl_server_poll", I, [P, C.POINTER(SZ)]),
    ("tsdfl_server_result", I, [P, C.c_uint64, P, C.POINTER(C.c_double), C.POINTER(I)]),
    ("tsdfl_session_particles", I, [P, U32, P, SZ, C.POINTER(SZ)]),
    ("tsdfl_server_draw", F, [C.c_uint64, C.c_uint64, SZ]),
    ("tsdfl_server_stats", I, [P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                               C.POINTER(C.c_uint64), C.POINTER(C.c_double)]),
    ("tsdfl_pose_array_device", I, [P, P, SZ, P]),
    ("tsdfl_pose_array", I, [P, P, SZ, P]),
    ("tsdfl_motion_model", I, [I, P, P, SZ, F, C.POINTER(Motion)]),
    ("tsdfl_motion_update_device", I, [P, P, SZ, C.POINTER(Motion), C.c_uint64, C.c_uint64, P]),
    ("tsdfl_motion_apply_device", I, [P, P, SZ, P]),
    ("tsdfl_motion_update", I, [P, P, SZ, C.POINTER(Motion), C.c_uint64, C.c_uint64]),
    ("tsdfl_motion_apply", I, [P, P, SZ, P]),
    ("tsdfl_evaluate_cloud", I, [P, P, C.POINTER(Model), P, SZ, P, SZ, U32, U32, U32, F, U32, P, U32, P,
                                 C.POINTER(SZ)]),
    ("tsdfl_evaluate_subsampled_device", I, [P, P, C.POINTER(Model), P, SZ, P, SZ, P, SZ, C.c_uint64, P]),
    ("tsdfl_evaluate_subsampled", I, [P, P, C.POINTER(Model), P, SZ, P, SZ, P, SZ, C.c_uint64, P, P, P]),
    ("tsdfl_subsample_index", U32, [C.c_uint64, C.c_uint64, U32, U32, U32]),
]

SYNTH_SIGNATURES = [
    ("tsyn_world_create", P, [I, C.c_uint64]),
    ("tsyn_world_destroy", None, [P]),
    ("tsyn_world_info", None, [P, P, P, P, P]),
    ("tsyn_world_sdf", F, [P, F, F, F]),
    ("tsyn_free", None, [P]),
    ("tsyn_tsdf_chunks", SZ, [P, I, I, F, C.POINTER(P), C.POINTER(P)]),
    ("tsyn_scan", SZ, [P, P, I, I, F, F, F, F, F, F, C.c_uint64, P, P]),
    ("tsyn_reduce_scan", SZ, [P, P, SZ, F, P]),
    ("tsyn_subsample_ordered", None, [P, SZ, SZ, C.c_uint64, P]),
    ("tsyn_particles_gaussian", None, [P, F, F, SZ, C.c_uint64, P]),
    ("tsyn_particles_free_space", None, [P, F, F, F, F, SZ, C.c_uint64, P]),
]


def _load(path: Path, sigs) -> C.CDLL:
    if not path.exists():
        raise ImportError(f"{path.name} is not built: run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(path))
    for name, res, args in sigs:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


_lib = None
_synth = None


def lib() -> C.CDLL:
    """libtsdfl.so of this package, or the build named by TSDFL_LIBRARY."""
    global _lib
    if _lib is None:
        import os
        _lib = _load(Path(os.environ.get("TSDFL_LIBRARY", _LIB_DIR / "libtsdfl.so")), SIGNATURES)
    return _lib


def synth_lib() -> C.CDLL:
    global _synth
    if _synth is None:
        _synth = _load(_LIB_DIR / "libtsdfl_synth.so", SYNTH_SIGNATURES)
    return _synth


class TsdflError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


def check(rc: int) -> None:
    if rc != TSDFL_OK:
        msg = lib().tsdfl_last_error().decode(errors="replace")
        raise TsdflError(rc, msg or f"tsdfl error {rc}")
