"""TEST INFRASTRUCTURE ONLY: the reference's own CUDA kernels on this GPU.

Loads oracle/_ref/ref_gpu.cubin (cuda_eval_particles.h compiled from the
reference tree, see ref_gpu_kernels.cu) through the CUDA driver API and
launches cudaEvaluateParticlesOrdered the way CudaEvaluator::evaluate does
(cuda_evaluator.cu:286-350): map coefficients, sensor transform and model in
__constant__ memory, particles as six SoA float rows, 64-thread blocks, one
thread per particle.  The kernel has no bound check on the thread index
(cuda_eval_particles.h:275), so the particle count must be a multiple of 64.
Imported only by tests/.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

CUBIN = Path(__file__).resolve().parent / "_ref" / "ref_gpu.cubin"
NS = "tsdf_localization"


def _mangle(name: str) -> bytes:
    return f"_ZN{len(NS)}{NS}{len(name)}{name}E".encode()


def available() -> bool:
    return CUBIN.exists()


class ReferenceKernels:
    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")
        self._check(self.cu.cuInit(0))
        cur = C.c_void_p()
        self._check(self.cu.cuCtxGetCurrent(C.byref(cur)))
        if not cur.value:
            raise RuntimeError("no current CUDA context (initialise the device first)")
        image = CUBIN.read_bytes()
        self._image = C.create_string_buffer(image, len(image))
        self.mod = C.c_void_p()
        self._check(self.cu.cuModuleLoadData(C.byref(self.mod), self._image))
        n = C.c_uint()
        self._check(self.cu.cuModuleGetFunctionCount(C.byref(n), self.mod))
        funcs = (C.c_void_p * n.value)()
        self._check(self.cu.cuModuleEnumerateFunctions(funcs, n, self.mod))
        self.eval_fn = None
        for f in funcs:
            name = C.c_char_p()
            self._check(self.cu.cuFuncGetName(C.byref(name), C.c_void_p(f)))
            if b"cudaEvaluateParticlesOrdered" in name.value:
                self.eval_fn = C.c_void_p(f)
        if self.eval_fn is None:
            raise RuntimeError("cudaEvaluateParticlesOrdered not in the cubin")

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(f"CUDA driver error {rc}")

    def _set(self, name: str, data: bytes):
        ptr = C.c_uint64()
        size = C.c_size_t()
        self._check(self.cu.cuModuleGetGlobal_v2(C.byref(ptr), C.byref(size), self.mod, _mangle(name)))
        if size.value != len(data):
            raise RuntimeError(f"{name}: {size.value} bytes, given {len(data)}")
        self._check(self.cu.cuMemcpyHtoD_v2(ptr, data, C.c_size_t(len(data))))

    def set_model(self, coef_bytes: bytes, tf16, a_hit=0.9, a_range=0.1, a_max=0.0, max_range=100.0):
        """cudaMemcpyToSymbol of cuda_evaluator.cu: MapCoef, tf, model constants."""
        f = lambda v: np.float32(v).tobytes()  # noqa: E731
        self._set("const_map_coef_", coef_bytes)
        self._set("const_tf_matrix", np.ascontiguousarray(tf16, np.float32).reshape(16).tobytes())
        self._set("const_a_hit_", f(a_hit))
        self._set("const_a_range_", f(a_range))
        self._set("const_a_max_", f(a_max))
        self._set("const_max_range_", f(max_range))
        self._set("const_max_range_squared_", f(np.float32(max_range) * np.float32(max_range)))
        self._set("const_inv_max_range_", f(np.float32(1.0) / np.float32(max_range)))

    def evaluate(self, d_grid_occ: int, d_data: int, d_coef: int, d_points: int, n_points: int, d_particles_soa: int,
                 n_particles: int, d_tf: int, d_weights: int, stream: int = 0):
        """cudaEvaluateParticlesOrdered<<<P / 64, 64>>>: raw weights of n_particles."""
        if n_particles % 64:
            raise ValueError("the reference kernel needs a multiple of 64 particles")
        args = [C.c_uint64(d_grid_occ), C.c_uint64(d_data), C.c_uint64(d_coef), C.c_uint64(d_points),
                C.c_size_t(n_points), C.c_uint64(d_particles_soa), C.c_size_t(n_particles), C.c_uint64(d_tf),
                C.c_uint64(d_weights)]
        params = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        self._check(self.cu.cuLaunchKernel(self.eval_fn, C.c_uint(n_particles // 64), C.c_uint(1), C.c_uint(1),
                                           C.c_uint(64), C.c_uint(1), C.c_uint(1), C.c_uint(0), C.c_void_p(stream),
                                           params, None))
