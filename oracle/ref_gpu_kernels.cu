// TEST INFRASTRUCTURE ONLY -- NOT PART OF THE PRODUCT.
//
// The reference's own CUDA sensor-update kernels (cudaEvaluateParticlesOrdered
// and the rest of include/tsdf_localization/cuda/cuda_eval_particles.h, with
// the __constant__ map coefficients and model of cuda_data.h), compiled from
// the reference tree into a cubin (oracle/_ref/ref_gpu.cubin) by
// tsdf_localization_gb300/_build.py.  oracle/ref_gpu.py loads it through the
// CUDA driver API so that the reference's GPU path can be timed beside ours on
// the same GPU.
#include <tsdf_localization/cuda/cuda_evaluator.h>
#include <tsdf_localization/cuda/cuda_data.h>
#include <tsdf_localization/cuda/cuda_eval_particles.h>
