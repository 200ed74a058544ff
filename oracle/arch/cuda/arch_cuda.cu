/* ORACLE TEST INFRASTRUCTURE -- device parts of the arch layer for the
 * reference's cuda kernel set (built into oracle/_ref/libflow_ref_cuda.so):
 * the second stage of its block reductions (finish_min_reduce and
 * finish_sum_reduce, cuda/flow.cu:121, 405) and the single-rank reflective
 * ghost fill of device arrays (handle_boundary_2d, cuda/flow.cu:36-39), with
 * the same meaning as the host fill of arch_shim.c: x walls over the interior
 * rows, then y walls over whole rows, negated across the inverted axis. */
#include <cuda_runtime.h>

#include "shared.h"
#include "reduction.k"

namespace {

constexpr int kFinishThreads = 1024;

template <bool kMin>
__global__ void k_finish(int n, const double* buffer, double* out) {
  __shared__ double s[kFinishThreads];
  double x = kMin ? buffer[0] : 0.0;
  for (int i = threadIdx.x; i < n; i += kFinishThreads) {
    const double v = buffer[i];
    x = kMin ? ((v < x) ? v : x) : x + v;
  }
  s[threadIdx.x] = x;
  __syncthreads();
  if (kMin) {
    min_reduce_in_shared<double, kFinishThreads>(threadIdx.x, s);
  } else {
    sum_reduce_in_shared<double, kFinishThreads>(threadIdx.x, s);
  }
  if (threadIdx.x == 0) *out = s[0];
}

__global__ void k_walls_x(int nx, int ny, int pad, double* arr, int flip) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (ny - 2 * pad) * pad) return;
  const int ii = pad + t / pad, dd = t % pad;
  const double w = arr[ii * nx + (pad + dd)];
  arr[ii * nx + (pad - 1 - dd)] = flip ? -w : w;
  const double e = arr[ii * nx + (nx - pad - 1 - dd)];
  arr[ii * nx + (nx - pad + dd)] = flip ? -e : e;
}

__global__ void k_walls_y(int nx, int ny, int pad, double* arr, int flip) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nx * pad) return;
  const int jj = t % nx, dd = t / nx;
  const double s = arr[(pad + dd) * nx + jj];
  arr[(pad - 1 - dd) * nx + jj] = flip ? -s : s;
  const double n = arr[(ny - pad - 1 - dd) * nx + jj];
  arr[(ny - pad + dd) * nx + jj] = flip ? -n : n;
}

void finish(bool is_min, int nblocks, double* buffer, double* result) {
  double* out = buffer + nblocks;  // the entry after the partials
  if (is_min) {
    k_finish<true><<<1, kFinishThreads>>>(nblocks, buffer, out);
  } else {
    k_finish<false><<<1, kFinishThreads>>>(nblocks, buffer, out);
  }
  gpu_check(cudaMemcpy(result, out, sizeof(double), cudaMemcpyDeviceToHost));
}

}  // namespace

extern "C" void finish_min_reduce(int nblocks, double* buffer, double* result) {
  finish(true, nblocks, buffer, result);
}

extern "C" void finish_sum_reduce(int nblocks, double* buffer, double* result) {
  finish(false, nblocks, buffer, result);
}

extern "C" void handle_boundary_2d(const int nx, const int ny, Mesh* mesh, double* arr,
                                   const int invert, const int pack) {
  (void)pack;
  const int pad = mesh->pad;
  const int nxw = (ny - 2 * pad) * pad, nyw = nx * pad;
  k_walls_x<<<(nxw + 255) / 256, 256>>>(nx, ny, pad, arr, invert == INVERT_X);
  k_walls_y<<<(nyw + 255) / 256, 256>>>(nx, ny, pad, arr, invert == INVERT_Y);
  gpu_check(cudaGetLastError());
}
