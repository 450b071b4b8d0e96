// TEST INFRASTRUCTURE ONLY: replaces the reference's fixed OMP_THREADS = 8
// (include/tsdf_localization/util/constant.h:4) by the build host's core count,
// so the reference's OpenMP evaluator uses every host core when it is timed.
#ifndef CONSTANT
#define CONSTANT

#ifndef TSDFL_REF_OMP_THREADS
#define TSDFL_REF_OMP_THREADS 8
#endif

constexpr unsigned int OMP_THREADS = TSDFL_REF_OMP_THREADS;

#endif
