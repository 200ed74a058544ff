// init.h -- device-side problem set-up shared by the C ABI and the batched
// form (init.cu).
#pragma once

#include <cuda_runtime.h>

namespace flow {

// Rasterises nboxes (density, energy, xpos, ypos, width, height) host boxes
// onto every cell of an nx x ny mesh with device face positions edgex/edgey.
int launch_fill_boxes(cudaStream_t s, int nx, int ny, const double* edgex, const double* edgey,
                      const double* boxes, int nboxes, double* rho, double* e);

// Face positions extent * (j - pad) / global_n for j < count.
int launch_uniform_edges(cudaStream_t s, double* edges, int count, int pad, double extent,
                         int global_n);

}  // namespace flow
