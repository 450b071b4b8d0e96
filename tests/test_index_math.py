"""CPU check of the slot-index arithmetic the kernels use (signed second tier
and the division-free fast path) against the oracle's getIndex, on random maps
with negative, out-of-bounds and special offsets."""
import shutil
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _build(tmp_path):
    exe = tmp_path / "index_check"
    csrc = ROOT / "tsdf_localization_gb300" / "csrc"
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda_inc = Path(nvcc).resolve().parent.parent / "include"
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fopenmp",
           "-I", str(csrc), "-I", str(ROOT / "include"), "-I", str(ROOT / "oracle"), "-I", str(cuda_inc),
           str(ROOT / "tests" / "native" / "index_check.cpp"), str(csrc / "map_build.cpp"),
           "-x", "c", str(ROOT / "oracle" / "tsdf_oracle.c"), "-o", str(exe), "-lm"]
    subprocess.run(cmd, check=True)
    return exe


def test_index_math_matches_oracle(tmp_path):
    exe = _build(tmp_path)
    res = subprocess.run([str(exe), "400000"], capture_output=True, text=True)
    print(res.stdout)
    assert res.returncode == 0, res.stdout
    handled = int(res.stdout.split("handled ")[1].split()[0])
    fast = int(res.stdout.split("fast ")[1].split()[0])
    assert handled > 1_000_000 and fast > 100_000


def test_sub_index_exhaustive(tmp_path):
    """Every float s in [0, 1): the one- or two-term multiplier gives
    trunc(s / res)."""
    exe = _build(tmp_path)
    ress = ["0.05", "0.064", "0.032", "0.02"]
    res = subprocess.run([str(exe), "exhaustive", *ress], capture_output=True, text=True)
    print(res.stdout)
    assert res.returncode == 0, res.stdout
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("exhaustive")]
    assert len(lines) == len(ress)
    for ln in lines:
        f = dict(kv.split("=") for kv in ln.split()[1:])
        assert f["bad"] == "0" and f["mode"] in ("1", "2")


def test_binade_prefix_sums_match_serial_double(tmp_path):
    """The parallel, binade-wise form of the resampler's serial double prefix
    sum equals plain serial double additions (random, tiny, zero and tie-heavy
    weights)."""
    exe = tmp_path / "binade_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", str(ROOT / "tests" / "native" / "binade_check.cpp"),
                    "-o", str(exe)], check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True)
    print(res.stdout)
    assert res.returncode == 0, res.stdout
    assert " 0 mismatches" in res.stdout
    ties = int(res.stdout.split(" ties")[0].split()[-1])
    assert ties > 0
