// stages.h -- host launchers of the per-function kernels (stages.cu) and of
// the fused timestep (fused.cu).  All pointers are device pointers; every
// launch is asynchronous on stream `s`.
#pragma once

#include <cstddef>
#include <cuda_runtime.h>

namespace flow {

// Device copies of the mesh spacing arrays (Mesh::edgedx ... celldy).
struct MeshView {
  const double* edgedx;
  const double* edgedy;
  const double* celldx;
  const double* celldy;
};

void launch_eos(cudaStream_t s, int nx, int ny, double* P, const double* rho,
                const double* e);
void launch_accelerate(cudaStream_t s, bool viscous, int nx, int ny, int pad,
                       double dt, double* rho_u, double* rho_v, double* u,
                       double* v, const double* fx, const double* fy,
                       const double* rho, const MeshView& m);
void launch_viscous_stress(cudaStream_t s, int nx, int ny, int pad, double* Qxx,
                           double* Qyy, const double* u, const double* v,
                           const double* rho);
void launch_shock_heating(cudaStream_t s, int nx, int ny, int pad, double dt_h,
                          double* e, const double* P, const double* u,
                          const double* v, const double* rho, const double* Qxx,
                          const double* Qyy, const MeshView& m);
// Writes dt, dt_h to reduce_array[0..1] (see common.cuh for the layout).
void launch_min_timestep(cudaStream_t s, int nx, int ny, int pad, double max_dt,
                         double dt_h, int first_step, const double* Qxx,
                         const double* Qyy, const double* rho, const double* e,
                         const MeshView& m, double* reduce_array, int local_only = 0);
// Writes interior sum(rho), sum(rho e) to reduce_array[3..4].
// Counts kernel launches for gb300_launch_count (interface.cu).
void count_launches(unsigned n);

// Ghost fill of a rank of a decomposed mesh: x walls over the interior rows,
// y walls over whole rows, on the sides set (1 west, 2 east, 4 south, 8 north).
void launch_reflect_x(cudaStream_t s, int w, int h, int pad, double* arr, int invert,
                      int sides);
void launch_reflect_y(cudaStream_t s, int w, int h, int pad, double* arr, int invert,
                      int sides);
// The dt rule (omp3/flow.c:103-105) applied on the device to a CFL minimum g
// reduced over the ranks of a decomposed mesh.
void launch_dt_rule(cudaStream_t s, double g, double dt_h, int first_step, double* ra);

void launch_conservation(cudaStream_t s, int nx, int ny, int pad,
                         const double* rho, const double* e,
                         double* reduce_array);
void launch_mass_energy_flux(cudaStream_t s, bool dir_y, int nx, int ny,
                             int pad, double dt, double dt_h, const double* rho,
                             const double* e, const double* vel, double* F,
                             double* eF, const MeshView& m);
void launch_mass_energy_update(cudaStream_t s, bool dir_y, int nx, int ny,
                               int pad, int first, double dt_h, double* rho,
                               const double* rho_old, double* e,
                               const double* F, const double* eF,
                               const MeshView& m);
void launch_uF_x(cudaStream_t s, int nx, int ny, int pad, double dt_h,
                 const double* u, double* uF_x, const double* F_x,
                 const MeshView& m);
void launch_uF_y(cudaStream_t s, int nx, int ny, int pad, double dt_h,
                 const double* u, const double* v, double* uF_y,
                 const double* F_y, const MeshView& m);
void launch_vF_x(cudaStream_t s, int nx, int ny, int pad, double dt_h,
                 const double* u, const double* v, double* vF_x,
                 const double* F_x, const MeshView& m);
void launch_vF_y(cudaStream_t s, int nx, int ny, int pad, double dt_h,
                 const double* v, double* vF_y, const double* F_y,
                 const MeshView& m);
// which: 0 rho_u by uF_x, 1 rho_u by uF_y, 2 rho_v by vF_x, 3 rho_v by vF_y.
void launch_momentum_update(cudaStream_t s, int which, int nx, int ny, int pad,
                            double dt_h, int with_vel, double* mom, double* vel,
                            const double* flux, const double* rho,
                            const MeshView& m);
// Reflective ghost fill of a w x h array; invert is 0, 1 (x) or 2 (y).
void launch_boundary(cudaStream_t s, int w, int h, int pad, double* arr,
                     int invert);
void launch_copy(cudaStream_t s, size_t n, double* dst, const double* src);
int reduce_blocks(int nx, int ny, int pad, int partials_per_block);

}  // namespace flow
