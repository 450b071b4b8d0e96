"""The C++ drop-in plug-ins (include/tsdfl_evaluator.hpp) compile against the
reference's own Evaluator/Resampler headers and link with libtsdfl; without a
GPU they report the failure as std::runtime_error, as the reference does."""
import subprocess
from pathlib import Path

import pytest

from oracle.build import REFERENCE

ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.skipif(not (REFERENCE / "include" / "tsdf_localization").exists(),
                    reason="reference headers not on this machine")
def test_dropin_builds_against_reference_headers(tmp_path):
    lib_dir = ROOT / "tsdf_localization_gb300" / "_lib"
    exe = tmp_path / "dropin_check"
    cmd = ["g++", "-std=c++17", "-O1", "-ffp-contract=off",
           "-I", str(ROOT / "oracle" / "shim"), "-I", str(REFERENCE / "include"), "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "native" / "dropin_check.cpp"), "-o", str(exe),
           "-L", str(lib_dir), "-ltsdfl", f"-Wl,-rpath,{lib_dir}"]
    subprocess.run(cmd, check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    print(res.stdout, res.stderr)
    assert res.returncode == 0
    assert "dropin compiled" in res.stdout
    assert "evaluated" in res.stdout or "runtime_error: " in res.stdout
