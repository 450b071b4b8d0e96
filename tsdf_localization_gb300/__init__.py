"""GB300-native MCL sensor update for TSDF maps (uos/tsdf_localization hot path).

The compute lives in libtsdfl.so (hand-written CUDA for sm_103a behind the C
ABI in include/tsdfl.h); this package binds it for tests, benchmarks and Python
callers.  Build with `python -c "import __graft_entry__ as g; g.build()"`.
"""
from ._native import TsdflError
from .evaluator import (Context, DeviceMap, FilterBatch, LocalizationServer, MetropolisResampler, MotionModel, Pose, RejectionResampler,
                        ResidualResampler, ResidualSystematicResampler, ScanReducer, SystematicResampler,
                        TSDFEvaluator, WheelResampler, build_map_codes, code_values, load_map_h5, pack_cloud,
                        pose_array, read_map_h5)

__all__ = ["Context", "DeviceMap", "FilterBatch", "LocalizationServer", "MetropolisResampler", "MotionModel", "Pose", "RejectionResampler",
           "ResidualResampler", "ResidualSystematicResampler", "ScanReducer", "SystematicResampler", "TSDFEvaluator",
           "TsdflError", "WheelResampler", "build_map_codes", "code_values", "load_map_h5", "pack_cloud", "pose_array",
           "read_map_h5"]
