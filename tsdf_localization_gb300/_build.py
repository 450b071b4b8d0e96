"""In-tree build of the native libraries (no cmake).

Products (git-ignored, rebuilt on every machine):
  tsdf_localization_gb300/_lib/libtsdfl.so        CUDA library behind include/tsdfl.h
  tsdf_localization_gb300/_lib/libtsdfl_synth.so  synthetic workload generator (host)
The oracle and the reference's own sources (test infrastructure) have their
own recipe, oracle/build.py.
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
    with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    lib = LIB / "libtsdfl.so"
    if force or jobs or not lib.exists() or _stale(lib, objs):
        _run([nvcc, *ARCH, "-shared", *map(str, objs), "-o", str(lib), "-Xcompiler", "-fopenmp", "-lgomp"])
    if verbose:
        print(f"built {lib}")
    return {"lib": str(lib), "synth": str(synth)}


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
