/* ORACLE TEST INFRASTRUCTURE -- the arch layer's CUDA definitions that the
 * reference's cuda kernel set includes as "../../cuda/shared.h" (cuda/flow.k:2),
 * restated from how that set uses them: the block size of every launch, the
 * error check after each launch, and the device helpers of its kernels.  Only
 * the second GPU baseline of the benchmark and its test build with this. */
#ifndef FLOW_ORACLE_ARCH_CUDA_SHARED_H
#define FLOW_ORACLE_ARCH_CUDA_SHARED_H

#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>

#include "../arch_shim.h"

/* Threads per block of every launch of the set (cuda/flow.cu:20-21). */
#define NTHREADS 128

/* Aborts with the CUDA error, as the arch layer's check does (cuda/flow.cu:24). */
#define gpu_check(call)                                                         \
  do {                                                                          \
    const cudaError_t gpu_check_err = (call);                                   \
    if (gpu_check_err != cudaSuccess) {                                         \
      TERMINATE("CUDA error %s at %s:%d\n", cudaGetErrorString(gpu_check_err), \
                __FILE__, __LINE__);                                            \
    }                                                                           \
  } while (0)

/* Slope limiter of the kernels: zero unless both arguments are non-zero with
 * the same sign, otherwise the argument of smaller magnitude. */
static __host__ __device__ inline double minmod(const double a, const double b) {
  if ((a > 0.0 && b > 0.0) || (a < 0.0 && b < 0.0)) {
    return (fabs(a) < fabs(b)) ? a : b;
  }
  return 0.0;
}

#endif
