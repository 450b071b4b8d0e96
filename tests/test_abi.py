"""The C ABI: libtsdfl.so loads and exports every function include/tsdfl.h
declares, and the Python binding declares a signature for each of them."""
import ctypes as C
import re
from pathlib import Path

from tsdf_localization_gb300 import _native as N

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    text = (ROOT / "include" / "tsdfl.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tsdfl_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_entry_points():
    names = declared_functions()
    for must in ("tsdfl_ctx_create", "tsdfl_map_create", "tsdfl_evaluate", "tsdfl_evaluate_device",
                 "tsdfl_resample_systematic", "tsdfl_resample_systematic_device", "tsdfl_last_error"):
        assert must in names


def test_library_exports_every_declared_function():
    lib = C.CDLL(str(N._LIB_DIR / "libtsdfl.so"))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_function():
    bound = {name for name, _, _ in N.SIGNATURES}
    assert set(declared_functions()) <= bound, set(declared_functions()) - bound


def test_calls_without_a_device_fail_cleanly():
    """Argument checks run before any device work: invalid handles are
    rejected with an error code and a message, never a crash."""
    lib = N.lib()
    assert lib.tsdfl_evaluate(None, None, None, None, 0, None, 0, None, 0, None) == N.TSDFL_ERR_INVALID_ARG
    assert lib.tsdfl_last_error()
    assert lib.tsdfl_resample_systematic(None, None, 0, 0.0, None, 0, None) == N.TSDFL_ERR_INVALID_ARG
    assert lib.tsdfl_resample_systematic_particles(None, None, 0, 0.0, None, 0, None) == N.TSDFL_ERR_INVALID_ARG
    assert lib.tsdfl_version()
