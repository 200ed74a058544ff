// init.cu -- device-side problem set-up: the params file's problem boxes
// rasterised on the device, the step the arch layer's
// initialise_shared_data_2d performs on the host before the first timestep
// (main.c:52-54, flow.params:1-2), so that a mesh (or a batched instance) is
// filled without building and copying host arrays.
#include <algorithm>

#include "../../include/flow_gb300.h"
#include "fused.h"
#include "init.h"

namespace flow {
namespace {

struct BoxSet {
  int n;
  double v[GB300_MAX_BOXES][6];  // density, energy, xpos, ypos, width, height
};

// Every local cell (ghosts included) takes the density and energy of the
// last box whose [pos, pos + extent) holds the cell's left / bottom edge
// coordinate, or 0 where no box does -- the rasterisation rule the
// reference's known answer pins (819^2 cells of the 0.4-0.6 box at 4096^2).
__global__ void k_fill_boxes(int nx, int ny, const double* __restrict__ edgex,
                             const double* __restrict__ edgey, const BoxSet bs, double* rho,
                             double* e) {
  const long long n = (long long)nx * ny;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int ii = (int)(t / nx), jj = (int)(t - (long long)ii * nx);
    const double x = edgex[jj], y = edgey[ii];
    double d = 0.0, en = 0.0;
    for (int k = 0; k < bs.n; ++k) {
      const double* b = bs.v[k];
      if (x >= b[2] && x < b[2] + b[4] && y >= b[3] && y < b[3] + b[5]) {
        d = b[0];
        en = b[1];
      }
    }
    rho[t] = d;
    e[t] = en;
  }
}

// Face positions of a uniform mesh, width * (j - pad) / global_n, as the arch
// layer's initialise_mesh_2d computes them.
__global__ void k_uniform_edges(double* edges, int count, int pad, double extent, int global_n) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < count; j += gridDim.x * blockDim.x) {
    edges[j] = extent * (double)(j - pad) / global_n;
  }
}

}  // namespace

int launch_fill_boxes(cudaStream_t s, int nx, int ny, const double* edgex, const double* edgey,
                      const double* boxes, int nboxes, double* rho, double* e) {
  if (nx <= 0 || ny <= 0 || !edgex || !edgey || !rho || !e || nboxes < 0 ||
      (nboxes > 0 && !boxes)) {
    return record_error(GB300_ERR_ARG, "fill_boxes: bad arguments");
  }
  if (nboxes > GB300_MAX_BOXES) {
    return record_error(GB300_ERR_ARG, "fill_boxes: %d boxes, at most %d", nboxes,
                        GB300_MAX_BOXES);
  }
  BoxSet bs;
  bs.n = nboxes;
  for (int k = 0; k < nboxes; ++k) {
    for (int q = 0; q < 6; ++q) bs.v[k][q] = boxes[6 * k + q];
  }
  const long long n = (long long)nx * ny;
  const int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
  k_fill_boxes<<<blocks, 256, 0, s>>>(nx, ny, edgex, edgey, bs, rho, e);
  return check_launch("fill_boxes");
}

int launch_uniform_edges(cudaStream_t s, double* edges, int count, int pad, double extent,
                         int global_n) {
  k_uniform_edges<<<(count + 255) / 256, 256, 0, s>>>(edges, count, pad, extent, global_n);
  return check_launch("uniform_edges");
}

}  // namespace flow

extern "C" int gb300_fill_boxes(int nx, int ny, const double* edgex, const double* edgey,
                                const double* boxes, int nboxes, double* rho, double* e) {
  flow::note_state_write();
  return flow::launch_fill_boxes(flow::current_stream(), nx, ny, edgex, edgey, boxes, nboxes,
                                 rho, e);
}
