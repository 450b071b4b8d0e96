"""Build recipe of the test infrastructure under oracle/ (no cmake).

Products (git-ignored, rebuilt on every machine):
  oracle/_build/liboracle.so   the oracle: CPU restatement of the reference's
                               sensor update and resampling (tsdf_oracle.c)
  oracle/_ref/libref.so        the reference's own CPU sources, compiled from the
                               reference tree where it is present on this machine
                               (TSDFL_REFERENCE_DIR, default /root/reference),
                               with the ROS stand-ins of oracle/shim and the
                               recording driver ref_driver.cpp
  oracle/_ref/ref_gpu.cubin    the reference's own CUDA kernels (device code), same

Only tests, the smoke check and the bench's CPU baseline and reference arm load
these; the product never does.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ORACLE = Path(__file__).resolve().parent
REFERENCE = Path(os.environ.get("TSDFL_REFERENCE_DIR", "/root/reference"))
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n  " + " ".join(cmd) + "\n" + res.stdout)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> dict:
    jobs = []
    orc_dir = ORACLE / "_build"
    orc_dir.mkdir(parents=True, exist_ok=True)
    orc = orc_dir / "liboracle.so"
    if force or _stale(orc, [ORACLE / "tsdf_oracle.c", ORACLE / "tsdf_oracle.h"]):
        jobs.append(["gcc", "-O2", "-fPIC", "-ffp-contract=off", "-fopenmp", "-std=gnu11", "-shared",
                     str(ORACLE / "tsdf_oracle.c"), "-o", str(orc), "-lm"])
    ref_built = None
    if (REFERENCE / "src" / "evaluation" / "tsdf_evaluator.cpp").exists():
        ref_dir = ORACLE / "_ref"
        ref_dir.mkdir(parents=True, exist_ok=True)
        ref = ref_dir / "libref.so"
        ref_srcs = [REFERENCE / "src" / "evaluation" / "tsdf_evaluator.cpp",
                    REFERENCE / "src" / "evaluation" / "model" / "likelihood_evaluation.cpp",
                    REFERENCE / "src" / "particle_cloud.cpp",
                    REFERENCE / "src" / "util" / "util.cpp",
                    REFERENCE / "src" / "resampling" / "wheel_resampler.cpp"]
        if force or _stale(ref, [ORACLE / "ref_driver.cpp"] + ref_srcs + sorted((ORACLE / "shim").rglob("*"))):
            jobs.append(["g++", "-std=c++17", "-O3", "-fPIC", "-ffp-contract=off", "-fopenmp", "-shared",
                         f"-DTSDFL_REF_OMP_THREADS={os.cpu_count() or 8}",
                         "-I", str(ORACLE / "shim"), "-I", str(REFERENCE / "include"),
                         str(ORACLE / "ref_driver.cpp"), *map(str, ref_srcs), "-o", str(ref)])
        ref_built = str(ref)
        # the reference's CUDA kernels as device code only (loaded through the driver API)
        nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
        cubin = ref_dir / "ref_gpu.cubin"
        if force or _stale(cubin, [ORACLE / "ref_gpu_kernels.cu"] + sorted((REFERENCE / "include").rglob("*.h"))):
            jobs.append([nvcc, "-cubin", *ARCH, "-O3", "-std=c++17", "-I", str(ORACLE / "shim"), "-I",
                         str(REFERENCE / "include"), str(ORACLE / "ref_gpu_kernels.cu"), "-o", str(cubin)])
    with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    if verbose:
        print(f"built {orc}" + (f" and {ref_built}" if ref_built else ""))
    return {"oracle": str(orc), "ref": ref_built}


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
