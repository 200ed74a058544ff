// peaks.cu -- measures this GPU's FP64 FMA issue rate, the compute bound of
// the FP64 timestep (GB300 runs FP64 at a small fraction of its FP32 rate).
// Used by the benchmark as the denominator of the FP64-pipe roofline.
#include "../../include/flow_gb300.h"

namespace {

constexpr int kChains = 8;

// Each thread runs kChains independent DFMA chains of `iters` steps; the
// result is written only under a condition that never holds, so the compiler
// keeps the arithmetic.
__global__ void k_dfma_rate(double* sink, int iters, double s) {
  double a[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) a[c] = 1.0 + threadIdx.x * 1e-7 + c * 1e-3;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) a[c] = fma(a[c], s, 1e-9);
  }
  double acc = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) acc += a[c];
  if (acc == -1.0) sink[threadIdx.x] = acc;
}

}  // namespace

extern "C" int gb300_measure_fp64_fma_rate(double* fma_per_s) {
  if (!fma_per_s) return GB300_ERR_ARG;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  double* sink = nullptr;
  if (cudaMalloc(&sink, 256 * sizeof(double)) != cudaSuccess) return GB300_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const dim3 grid(sms * 8), block(256);
  const int iters = 2048;
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    k_dfma_rate<<<grid, block>>>(sink, iters, 0.999999);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (err != cudaSuccess) return GB300_ERR_CUDA;
  *fma_per_s = (double)grid.x * block.x * iters * kChains / (best * 1e-3);
  return GB300_OK;
}
