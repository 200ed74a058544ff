/* ORACLE TEST INFRASTRUCTURE -- the arch layer's block reductions that the
 * reference's cuda kernel set includes as "../../cuda/reduction.k"
 * (cuda/flow.k:1), restated from their use: every thread of a block has put
 * its value in sdata[tid] and passed a barrier (cuda/flow.k:834-837); after
 * the call sdata[0] holds the block's minimum / sum.  The second stage
 * (finish_*_reduce, cuda/flow.cu:121, 405) is in arch_cuda.cu. */
#ifndef FLOW_ORACLE_ARCH_CUDA_REDUCTION_K
#define FLOW_ORACLE_ARCH_CUDA_REDUCTION_K

template <typename T, int N>
__device__ void min_reduce_in_shared(const int tid, T* sdata) {
  for (int s = N / 2; s > 0; s >>= 1) {
    if (tid < s) sdata[tid] = (sdata[tid + s] < sdata[tid]) ? sdata[tid + s] : sdata[tid];
    __syncthreads();
  }
}

template <typename T, int N>
__device__ void sum_reduce_in_shared(const int tid, T* sdata) {
  for (int s = N / 2; s > 0; s >>= 1) {
    if (tid < s) sdata[tid] += sdata[tid + s];
    __syncthreads();
  }
}

#ifdef __cplusplus
extern "C" {
#endif
/* The minimum / sum of the first nblocks entries of the device array
 * buffer, into *result (host). */
void finish_min_reduce(int nblocks, double* buffer, double* result);
void finish_sum_reduce(int nblocks, double* buffer, double* result);
#ifdef __cplusplus
}
#endif

#endif
