// common.cuh -- shared definitions of the GB300 flow kernel set.
//
// Grid conventions follow the reference kernel set (omp3/flow.c): nx, ny are
// the padded cell counts (local_nx/local_ny), pad = 2 ghost layers.
//   cell   (ii,jj): ii*nx + jj           ny rows,     nx cols
//   x-face (ii,jj): ii*(nx+1) + jj       ny rows,     nx+1 cols
//   y-face (ii,jj): ii*nx + jj           ny+1 rows,   nx cols (omp3/flow.c:129)
//   corner (ii,jj): ii*(nx+1) + jj       ny+1 rows,   nx+1 cols
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace flow {

// Physical constants of flow_interface.h:7-9 and flow_data.h:5.
constexpr double kGam = 1.4;
constexpr double kCQ = 3.0;
constexpr double kCT = 0.3;
#define FLOW_C_M (1.5 / 0.3)

// Layout of the caller's reduce_array (flow_interface.h:20).  The host driver
// allocates it with local_nx*local_ny doubles (arch SharedData), and the
// kernel set uses it as its only device scratch:
//   [0] dt, [1] dt_h          device copy of the timestep pair
//   [2] ticket                block-completion counter (uint64 bits)
//   [3] mass, [4] energy      conservation totals of the last reduction
//   [5] status                error word of the fused kernels (uint64 bits)
//   [6] CFL minimum           running minimum of the fused step's CFL
//                             candidates (uint64 bits of a non-negative
//                             double: bit order = value order)
//   [7] mesh power-of-two     1 when every mesh spacing is a power of two
//                             (formed on the device at the start of a step)
//   [8] moving tiles          the fused step's count of first-sweep tiles
//                             it did not skip (uint64), read with dt
//   [9 ...]                   per-block partials (2 doubles per block, at
//                             most kMaxReduceBlocks blocks)
//   [kRaQFlags ...]           the fused step's tile flags, when the array
//                             is large enough to hold them: per-tile CFL
//                             minima, then the viscous-stress, mass-flux and
//                             velocity flags and the two halves of the
//                             sweeps' skip marks (fused.cu, fill_mesh_args)
enum : int {
  kRaDt = 0,
  kRaDtH = 1,
  kRaTicket = 2,
  kRaMass = 3,
  kRaEnergy = 4,
  kRaStatus = 5,
  kRaMinBits = 6,
  kRaMeshPow2 = 7,
  kRaMoving = 8,
  kRaPartial = 9,
};
constexpr int kMaxReduceBlocks = 1024;
constexpr int kRaQFlags = kRaPartial + 2 * kMaxReduceBlocks;

// Ghost-fill modes of handle_boundary_2d (arch; omp3/flow.c:156).
enum : int { kNoInvert = 0, kInvertX = 1, kInvertY = 2 };

// Indices are never negative here, so they are formed with one 32x32->64-bit
// unsigned multiply-add (a signed int widened to size_t first costs a 64-bit
// multiply).
__host__ __device__ inline size_t cidx(int nx, int ii, int jj) {
  return (size_t)(unsigned)ii * (unsigned)nx + (unsigned)jj;
}
__host__ __device__ inline size_t fidx(int nx, int ii, int jj) {
  return (size_t)(unsigned)ii * (unsigned)(nx + 1) + (unsigned)jj;
}

// Ordinary minimum (first argument when strictly smaller).
__device__ __forceinline__ double dmin(double a, double b) {
  return (a < b) ? a : b;
}

// Slope limiter: the argument of smaller magnitude when both are non-zero and
// of the same sign (the second on a tie), else 0.
__device__ __forceinline__ double minmod(double a, double b) {
  if ((a > 0.0 && b > 0.0) || (a < 0.0 && b < 0.0)) {
    return (fabs(a) < fabs(b)) ? a : b;
  }
  return 0.0;
}

}  // namespace flow
