"""In-tree build of the native libraries (no cmake).

Products (git-ignored, rebuilt on every machine):
  tsdf_localization_gb300/_lib/libtsdfl.so        CUDA library behind include/tsdfl.h
  tsdf_localization_gb300/_lib/libtsdfl_synth.so  synthetic workload generator (host)
Test infrastructure built by the same call:
  oracle/_build/liboracle.so   CPU restatement of the reference sensor update
  oracle/_ref/libref.so        the reference's own CPU sources, compiled from the
                               reference tree when it is present on this machine
  oracle/_ref/ref_gpu.cubin    the reference's own CUDA kernels (device code), same
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "tsdf_localization_gb300"
CSRC = PKG / "csrc"
LIB = PKG / "_lib"
OBJ = PKG / "_lib" / "obj"
ORACLE = ROOT / "oracle"
REFERENCE = Path(os.environ.get("TSDFL_REFERENCE_DIR", "/root/reference"))

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = ["-O2", "-fPIC", "-ffp-contract=off", "-fopenmp", "-std=c++17"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libtsdfl")


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
    LIB.mkdir(parents=True, exist_ok=True)
    OBJ.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I", str(ROOT / "include"), "-I", str(CSRC)]
    headers = sorted(CSRC.glob("*.h")) + [ROOT / "include" / "tsdfl.h"]
    cu = sorted(CSRC.glob("*.cu"))
    cpp_lib = [CSRC / "map_build.cpp", CSRC / "motion_model.cpp", CSRC / "h5_map.cpp"]
    jobs = []
    objs = []
    for src in cu:
        o = OBJ / (src.stem + ".o")
        objs.append(o)
        if force or _stale(o, [src] + headers):
            # -fmad=false: no multiply-add contraction anywhere (the scan transform
            # must round after every product and sum, as the reference does)
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
                         "-Xcompiler", "-ffp-contract=off", *inc, "-c", str(src), "-o", str(o)])
    for src in cpp_lib:
        o = OBJ / (src.stem + ".o")
        objs.append(o)
        if force or _stale(o, [src] + headers):
            jobs.append(["g++", *HOST_FLAGS, *inc, "-c", str(src), "-o", str(o)])
    synth = LIB / "libtsdfl_synth.so"
    if force or _stale(synth, [CSRC / "synth.cpp"]):
        jobs.append(["g++", *HOST_FLAGS, "-shared", str(CSRC / "synth.cpp"), "-o", str(synth)])
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
        cubin = ref_dir / "ref_gpu.cubin"
        if force or _stale(cubin, [ORACLE / "ref_gpu_kernels.cu"] + sorted((REFERENCE / "include").rglob("*.h"))):
            jobs.append([nvcc, "-cubin", *ARCH, "-O3", "-std=c++17", "-I", str(ORACLE / "shim"), "-I",
                         str(REFERENCE / "include"), str(ORACLE / "ref_gpu_kernels.cu"), "-o", str(cubin)])
    with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    lib = LIB / "libtsdfl.so"
    if force or jobs or not lib.exists() or _stale(lib, objs):
        _run([nvcc, *ARCH, "-shared", *map(str, objs), "-o", str(lib), "-Xcompiler", "-fopenmp", "-lgomp"])
    if verbose:
        print(f"built {lib}")
    return {"lib": str(lib), "synth": str(synth), "oracle": str(orc), "ref": ref_built}


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
