// interface.cu -- the C ABI of include/flow_gb300.h: the reference kernel-set
// entry points (flow_interface.h, omp3/flow.h) on top of the stage kernels of
// stages.cu and the fused timestep of fused.cu, plus error/stream control.
#include <cstdarg>
#include <cstdio>
#include <atomic>
#include <cstring>

#include "../../include/flow_gb300.h"
#include "common.cuh"
#include "fused.h"
#include "stages.h"

namespace {

thread_local int t_err = GB300_OK;
thread_local char t_msg[512] = "";
thread_local cudaStream_t t_stream = nullptr;
thread_local int t_mode = GB300_MODE_FUSED;
int g_verbose = 1;

}  // namespace

namespace flow {

int record_error(int code, const char* fmt, ...) {
  t_err = code;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(t_msg, sizeof(t_msg), fmt, ap);
  va_end(ap);
  return code;
}

int check_launch(const char* where) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    return record_error(GB300_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
  }
  return GB300_OK;
}

cudaStream_t current_stream() { return t_stream; }

namespace {
std::atomic<unsigned long long> g_launches{0};
}  // namespace

void count_launches(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int num_sms() {
  static int cached[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (cached[dev] <= 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
      n = 1;
    }
    cached[dev] = n;
  }
  return cached[dev];
}
int verbose() { return g_verbose; }

// Sizes the kernels support: one rank, pad >= 2, >= 2 interior cells per axis
// (the ghost mirror of a layer must land on an interior layer).
int check_sizes(int nx, int ny, int pad, const char* where) {
  if (pad < 2 || nx - 2 * pad < 2 || ny - 2 * pad < 2) {
    return record_error(GB300_ERR_ARG,
                        "%s: need pad >= 2 and >= 2 interior cells per axis "
                        "(nx=%d ny=%d pad=%d)",
                        where, nx, ny, pad);
  }
  if ((long long)nx * ny < kRaPartial + 16) {
    return record_error(GB300_ERR_ARG, "%s: mesh too small for reduce_array",
                        where);
  }
  return GB300_OK;
}

namespace {
// Domain decomposition hooks (gb300_set_halo_exchange, gb300_set_reduce_min).
gb300_halo_fn g_halo_fn = nullptr;
void* g_halo_ctx = nullptr;
gb300_reduce_min_fn g_rmin_fn = nullptr;
void* g_rmin_ctx = nullptr;
}  // namespace

bool decomposed(const Mesh* m) {
  for (int k = 0; k < 4; ++k) {
    if (m->neighbours[k] != FLOW_EDGE) return true;
  }
  return false;
}

// A rank of a decomposed mesh runs the exact mode's stage kernels with its
// ghost layers exchanged through the registered hooks.
namespace {
std::atomic<unsigned long long> g_mesh_calls{0};
}  // namespace

unsigned long long mesh_calls() { return g_mesh_calls.load(std::memory_order_relaxed); }
void note_state_write() { g_mesh_calls.fetch_add(1, std::memory_order_relaxed); }

int check_mesh(const Mesh* m, int nx, int ny, const char* where) {
  note_state_write();
  if (!m) return record_error(GB300_ERR_ARG, "%s: mesh is NULL", where);
  if (decomposed(m) && (!g_halo_fn || !g_rmin_fn)) {
    return record_error(GB300_ERR_ARG,
                        "%s: a decomposed mesh (a neighbour is a rank) needs "
                        "gb300_set_halo_exchange and gb300_set_reduce_min",
                        where);
  }
  return check_sizes(nx, ny, m->pad, where);
}

int check_single_rank(const Mesh* m, const char* where) {
  if (m && decomposed(m)) {
    return record_error(GB300_ERR_ARG,
                        "%s: the fused and mixed forms run one rank; a decomposed "
                        "mesh runs in GB300_MODE_EXACT", where);
  }
  return GB300_OK;
}

// Ghost fill of a rank of a decomposed mesh: physical x walls over the
// interior rows, the halo exchange (the hook: rows and columns from the
// neighbouring ranks, full width), then physical y walls over whole rows --
// the order of the single-rank fill, so corners agree.
int decomposed_boundary(int w, int h, const Mesh* mesh, double* arr, int invert) {
  cudaStream_t s = current_stream();
  int sides = 0;
  if (mesh->neighbours[FLOW_WEST] == FLOW_EDGE) sides |= 1;
  if (mesh->neighbours[FLOW_EAST] == FLOW_EDGE) sides |= 2;
  if (mesh->neighbours[FLOW_SOUTH] == FLOW_EDGE) sides |= 4;
  if (mesh->neighbours[FLOW_NORTH] == FLOW_EDGE) sides |= 8;
  launch_reflect_x(s, w, h, mesh->pad, arr, invert, sides);
  const cudaError_t err = cudaStreamSynchronize(s);
  if (err != cudaSuccess) {
    return record_error(GB300_ERR_CUDA, "handle_boundary_2d: %s", cudaGetErrorString(err));
  }
  const int rc = g_halo_fn(g_halo_ctx, mesh, arr, w, h, invert);
  if (rc != 0) {
    return record_error(GB300_ERR_STATE, "handle_boundary_2d: the halo exchange returned %d",
                        rc);
  }
  launch_reflect_y(s, w, h, mesh->pad, arr, invert, sides);
  return check_launch("handle_boundary_2d");
}

// The global CFL minimum of a decomposed mesh: the rank's minimum (left in
// reduce_array by the reduction kernel), reduced over the ranks by the hook.
int reduce_min_over_ranks(double* g) {
  const int rc = g_rmin_fn(g_rmin_ctx, g);
  if (rc != 0) {
    return record_error(GB300_ERR_STATE, "set_timestep: the minimum reduction returned %d", rc);
  }
  return GB300_OK;
}

MeshView view(const Mesh* m) {
  return MeshView{m->edgedx, m->edgedy, m->celldx, m->celldy};
}

}  // namespace flow

using namespace flow;

#define FLOW_TRY(expr)          \
  do {                          \
    const int _st = (expr);     \
    if (_st != GB300_OK) return _st; \
  } while (0)

namespace {

// ---------------------------------------------------------------------------
// Status-returning forms of the stage entry points.

int st_boundary(int w, int h, const Mesh* mesh, double* arr, int invert) {
  if (decomposed(mesh)) return decomposed_boundary(w, h, mesh, arr, invert);
  launch_boundary(current_stream(), w, h, mesh->pad, arr, invert);
  return GB300_OK;
}

int st_pressure_acceleration(int nx, int ny, Mesh* mesh, double dt,
                             double* rho_u, double* rho_v, double* u, double* v,
                             const double* P, const double* rho,
                             const MeshView& m) {
  FLOW_TRY(check_mesh(mesh, nx, ny, "pressure_acceleration"));
  cudaStream_t s = current_stream();
  launch_accelerate(s, false, nx, ny, mesh->pad, dt, rho_u, rho_v, u, v, P, P,
                    rho, m);
  st_boundary(nx + 1, ny, mesh, u, kInvertX);
  st_boundary(nx, ny + 1, mesh, v, kInvertY);
  return check_launch("pressure_acceleration");
}

int st_artificial_viscosity(int nx, int ny, Mesh* mesh, double dt, double* Qxx,
                            double* Qyy, double* u, double* v, double* rho_u,
                            double* rho_v, const double* rho,
                            const MeshView& m) {
  FLOW_TRY(check_mesh(mesh, nx, ny, "artificial_viscosity"));
  cudaStream_t s = current_stream();
  launch_viscous_stress(s, nx, ny, mesh->pad, Qxx, Qyy, u, v, rho);
  st_boundary(nx, ny, mesh, Qxx, kNoInvert);
  st_boundary(nx, ny, mesh, Qyy, kNoInvert);
  launch_accelerate(s, true, nx, ny, mesh->pad, dt, rho_u, rho_v, u, v, Qxx,
                    Qyy, rho, m);
  st_boundary(nx + 1, ny, mesh, u, kInvertX);
  st_boundary(nx, ny + 1, mesh, v, kInvertY);
  return check_launch("artificial_viscosity");
}

int st_shock_heating(int nx, int ny, Mesh* mesh, double dt_h, double* e,
                     const double* P, const double* u, const double* v,
                     const double* rho, const double* Qxx, const double* Qyy,
                     const MeshView& m) {
  FLOW_TRY(check_mesh(mesh, nx, ny, "shock_heating_and_work"));
  launch_shock_heating(current_stream(), nx, ny, mesh->pad, dt_h, e, P, u, v,
                       rho, Qxx, Qyy, m);
  st_boundary(nx, ny, mesh, e, kNoInvert);
  return check_launch("shock_heating_and_work");
}

// A page-locked pair of doubles per host thread for the values the host
// waits on (dt, the totals): a copy into it is one DMA, where a copy into
// pageable memory is staged through a driver buffer.  Kept for the life of
// the thread; NULL if page-locked memory cannot be had (the caller then
// copies into its own memory).
double* pinned_pair() {
  thread_local double* buf = nullptr;
  thread_local bool tried = false;
  if (!tried) {
    tried = true;
    if (cudaMallocHost(&buf, 2 * sizeof(double)) != cudaSuccess) {
      buf = nullptr;
      cudaGetLastError();
    }
  }
  return buf;
}

int st_set_timestep(int nx, int ny, const double* Qxx, const double* Qyy,
                    const double* rho, const double* e, Mesh* mesh,
                    double* reduce_array, int first_step, const double* celldx,
                    const double* celldy) {
  FLOW_TRY(check_mesh(mesh, nx, ny, "set_timestep"));
  if (!reduce_array) return record_error(GB300_ERR_ARG, "set_timestep: reduce_array is NULL");
  cudaStream_t s = current_stream();
  MeshView m{mesh->edgedx, mesh->edgedy, celldx, celldy};
  const bool ranks = decomposed(mesh);
  launch_min_timestep(s, nx, ny, mesh->pad, mesh->max_dt, mesh->dt_h,
                      first_step, Qxx, Qyy, rho, e, m, reduce_array, ranks ? 1 : 0);
  if (ranks) {
    double g = 0.0;
    cudaMemcpyAsync(&g, reduce_array + kRaMinBits, sizeof(double), cudaMemcpyDeviceToHost, s);
    const cudaError_t e1 = cudaStreamSynchronize(s);
    if (e1 != cudaSuccess) {
      return record_error(GB300_ERR_CUDA, "set_timestep: %s", cudaGetErrorString(e1));
    }
    FLOW_TRY(reduce_min_over_ranks(&g));
    launch_dt_rule(s, g, mesh->dt_h, first_step, reduce_array);
  }
  double local[2];
  double* pair = pinned_pair();
  if (!pair) pair = local;
  cudaMemcpyAsync(pair, reduce_array + kRaDt, 2 * sizeof(double),
                  cudaMemcpyDeviceToHost, s);
  const cudaError_t err = cudaStreamSynchronize(s);
  if (err != cudaSuccess) {
    return record_error(GB300_ERR_CUDA, "set_timestep: %s",
                        cudaGetErrorString(err));
  }
  FLOW_TRY(check_launch("set_timestep"));
  mesh->dt = pair[0];
  mesh->dt_h = pair[1];
  return GB300_OK;
}

int st_mass_energy_sweep(bool dir_y, int nx, int ny, int first, Mesh* mesh,
                         double dt, double dt_h, double* rho,
                         const double* rho_old, double* e, const double* vel,
                         double* F, double* eF, const MeshView& m) {
  cudaStream_t s = current_stream();
  const int pad = mesh->pad;
  launch_mass_energy_flux(s, dir_y, nx, ny, pad, dt, dt_h, rho, e, vel, F, eF,
                          m);
  if (dir_y) {
    st_boundary(nx, ny + 1, mesh, F, kInvertY);
  } else {
    st_boundary(nx + 1, ny, mesh, F, kInvertX);
  }
  launch_mass_energy_update(s, dir_y, nx, ny, pad, first, dt_h, rho, rho_old,
                            e, F, eF, m);
  st_boundary(nx, ny, mesh, rho, kNoInvert);
  st_boundary(nx, ny, mesh, e, kNoInvert);
  return check_launch(dir_y ? "y_mass_and_energy_flux" : "x_mass_and_energy_flux");
}

int st_advect_mass_and_energy(int nx, int ny, Mesh* mesh, int tt, double dt,
                              double dt_h, double* rho, double* e,
                              double* rho_old, double* F_x, double* F_y,
                              double* eF_x, double* eF_y, const double* u,
                              const double* v, const MeshView& m) {
  FLOW_TRY(check_mesh(mesh, nx, ny, "advect_mass_and_energy"));
  launch_copy(current_stream(), (size_t)nx * ny, rho_old, rho);
  if (tt % 2 == 0) {
    FLOW_TRY(st_mass_energy_sweep(false, nx, ny, 1, mesh, dt, dt_h, rho,
                                  rho_old, e, u, F_x, eF_x, m));
    FLOW_TRY(st_mass_energy_sweep(true, nx, ny, 0, mesh, dt, dt_h, rho,
                                  rho_old, e, v, F_y, eF_y, m));
  } else {
    FLOW_TRY(st_mass_energy_sweep(true, nx, ny, 1, mesh, dt, dt_h, rho,
                                  rho_old, e, v, F_y, eF_y, m));
    FLOW_TRY(st_mass_energy_sweep(false, nx, ny, 0, mesh, dt, dt_h, rho,
                                  rho_old, e, u, F_x, eF_x, m));
  }
  return GB300_OK;
}

// The four (flux, update) pairs of advect_momentum, omp3/flow.c:568-774.
int mom_u_x(int nx, int ny, Mesh* mesh, double dt_h, int with_u, double* u,
            double* uF_x, double* rho_u, const double* rho, const double* F_x,
            const MeshView& m) {
  cudaStream_t s = current_stream();
  launch_uF_x(s, nx, ny, mesh->pad, dt_h, u, uF_x, F_x, m);
  st_boundary(nx, ny, mesh, uF_x, kNoInvert);
  launch_momentum_update(s, 0, nx, ny, mesh->pad, dt_h, with_u, rho_u, u, uF_x,
                         rho, m);
  if (with_u) st_boundary(nx + 1, ny, mesh, u, kInvertX);
  return GB300_OK;
}
int mom_u_y(int nx, int ny, Mesh* mesh, double dt_h, int with_u, double* u,
            const double* v, double* uF_y, double* rho_u, const double* rho,
            const double* F_y, const MeshView& m) {
  cudaStream_t s = current_stream();
  launch_uF_y(s, nx, ny, mesh->pad, dt_h, u, v, uF_y, F_y, m);
  st_boundary(nx + 1, ny + 1, mesh, uF_y, kNoInvert);
  launch_momentum_update(s, 1, nx, ny, mesh->pad, dt_h, with_u, rho_u, u, uF_y,
                         rho, m);
  if (with_u) st_boundary(nx + 1, ny, mesh, u, kInvertX);
  return GB300_OK;
}
int mom_v_x(int nx, int ny, Mesh* mesh, double dt_h, int with_v,
            const double* u, double* v, double* vF_x, double* rho_v,
            const double* rho, const double* F_x, const MeshView& m) {
  cudaStream_t s = current_stream();
  launch_vF_x(s, nx, ny, mesh->pad, dt_h, u, v, vF_x, F_x, m);
  st_boundary(nx + 1, ny + 1, mesh, vF_x, kNoInvert);
  launch_momentum_update(s, 2, nx, ny, mesh->pad, dt_h, with_v, rho_v, v, vF_x,
                         rho, m);
  if (with_v) st_boundary(nx, ny + 1, mesh, v, kInvertY);
  return GB300_OK;
}
int mom_v_y(int nx, int ny, Mesh* mesh, double dt_h, int with_v, double* v,
            double* vF_y, double* rho_v, const double* rho, const double* F_y,
            const MeshView& m) {
  cudaStream_t s = current_stream();
  launch_vF_y(s, nx, ny, mesh->pad, dt_h, v, vF_y, F_y, m);
  st_boundary(nx, ny, mesh, vF_y, kNoInvert);
  launch_momentum_update(s, 3, nx, ny, mesh->pad, dt_h, with_v, rho_v, v, vF_y,
                         rho, m);
  if (with_v) st_boundary(nx, ny + 1, mesh, v, kInvertY);
  return GB300_OK;
}

int st_advect_momentum(int nx, int ny, int tt, Mesh* mesh, double dt_h,
                       double* u, double* v, double* uF_x, double* uF_y,
                       double* vF_x, double* vF_y, double* rho_u,
                       double* rho_v, const double* rho, const double* F_x,
                       const double* F_y, const MeshView& m) {
  FLOW_TRY(check_mesh(mesh, nx, ny, "advect_momentum"));
  if (tt % 2) {
    mom_u_x(nx, ny, mesh, dt_h, 1, u, uF_x, rho_u, rho, F_x, m);
    mom_u_y(nx, ny, mesh, dt_h, 0, u, v, uF_y, rho_u, rho, F_y, m);
    mom_v_x(nx, ny, mesh, dt_h, 1, u, v, vF_x, rho_v, rho, F_x, m);
    mom_v_y(nx, ny, mesh, dt_h, 0, v, vF_y, rho_v, rho, F_y, m);
  } else {
    mom_u_y(nx, ny, mesh, dt_h, 1, u, v, uF_y, rho_u, rho, F_y, m);
    mom_u_x(nx, ny, mesh, dt_h, 0, u, uF_x, rho_u, rho, F_x, m);
    mom_v_y(nx, ny, mesh, dt_h, 1, v, vF_y, rho_v, rho, F_y, m);
    mom_v_x(nx, ny, mesh, dt_h, 0, u, v, vF_x, rho_v, rho, F_x, m);
  }
  return check_launch("advect_momentum");
}

int st_conservation(int nx, int ny, int pad, const double* rho, const double* e,
                    double* reduce_array, double* out, int sync) {
  FLOW_TRY(check_sizes(nx, ny, pad, "conservation"));
  if (!reduce_array) return record_error(GB300_ERR_ARG, "conservation: reduce_array is NULL");
  cudaStream_t s = current_stream();
  if (!tile_conservation(nx, ny, pad, rho, e, reduce_array, s)) {
    launch_conservation(s, nx, ny, pad, rho, e, reduce_array);
  }
  FLOW_TRY(check_launch("conservation"));
  if (!sync) return GB300_OK;
  double local[2];
  double* tot = pinned_pair();
  if (!tot) tot = local;
  cudaMemcpyAsync(tot, reduce_array + kRaMass, 2 * sizeof(double),
                  cudaMemcpyDeviceToHost, s);
  const cudaError_t err = cudaStreamSynchronize(s);
  if (err != cudaSuccess) {
    return record_error(GB300_ERR_CUDA, "conservation: %s", cudaGetErrorString(err));
  }
  if (out) {
    out[0] = tot[0];
    out[1] = tot[1];
  }
  return GB300_OK;
}

int st_solve_exact(Mesh* mesh, int tt, double* P, double* rho, double* rho_old,
                   double* e, double* u, double* v, double* rho_u,
                   double* rho_v, double* Qxx, double* Qyy, double* F_x,
                   double* F_y, double* uF_x, double* uF_y, double* vF_x,
                   double* vF_y, double* reduce_array) {
  const int nx = mesh->local_nx, ny = mesh->local_ny;
  const MeshView m = view(mesh);
  FLOW_TRY(check_mesh(mesh, nx, ny, "solve_hydro_2d"));
  launch_eos(current_stream(), nx, ny, P, rho, e);
  FLOW_TRY(st_pressure_acceleration(nx, ny, mesh, mesh->dt, rho_u, rho_v, u, v,
                                    P, rho, m));
  FLOW_TRY(st_artificial_viscosity(nx, ny, mesh, mesh->dt, Qxx, Qyy, u, v,
                                   rho_u, rho_v, rho, m));
  FLOW_TRY(st_shock_heating(nx, ny, mesh, mesh->dt_h, e, P, u, v, rho, Qxx,
                            Qyy, m));
  FLOW_TRY(st_set_timestep(nx, ny, Qxx, Qyy, rho, e, mesh, reduce_array,
                           tt == 0, mesh->celldx, mesh->celldy));
  // The energy fluxes reuse the momentum-flux buffers (omp3/flow.c:41-45).
  FLOW_TRY(st_advect_mass_and_energy(nx, ny, mesh, tt, mesh->dt, mesh->dt_h,
                                     rho, e, rho_old, F_x, F_y, uF_x, uF_y, u,
                                     v, m));
  FLOW_TRY(st_advect_momentum(nx, ny, tt, mesh, mesh->dt_h, u, v, uF_x, uF_y,
                              vF_x, vF_y, rho_u, rho_v, rho, F_x, F_y, m));
  return GB300_OK;
}

}  // namespace

// ===========================================================================
// Part 1: the reference kernel-set interface.

extern "C" {

int gb300_solve_hydro_2d(Mesh* mesh, int tt, double* P, double* rho,
                         double* rho_old, double* e, double* u, double* v,
                         double* rho_u, double* rho_v, double* Qxx,
                         double* Qyy, double* F_x, double* F_y, double* uF_x,
                         double* uF_y, double* vF_x, double* vF_y,
                         double* reduce_array) {
  if (!mesh) return record_error(GB300_ERR_ARG, "solve_hydro_2d: mesh is NULL");
  if (g_verbose && mesh->rank == 0) {
    printf("Timestep:        %.12e\n", mesh->dt);
  }
  if (t_mode != GB300_MODE_EXACT) FLOW_TRY(check_single_rank(mesh, "solve_hydro_2d"));
  if (t_mode == GB300_MODE_EXACT) {
    return st_solve_exact(mesh, tt, P, rho, rho_old, e, u, v, rho_u, rho_v, Qxx,
                          Qyy, F_x, F_y, uF_x, uF_y, vF_x, vF_y, reduce_array);
  }
  FLOW_TRY(check_mesh(mesh, mesh->local_nx, mesh->local_ny, "solve_hydro_2d"));
  return fused_solve(mesh, tt, P, rho, rho_old, e, u, v, rho_u, rho_v, Qxx, Qyy,
                     F_x, F_y, uF_x, uF_y, vF_x, vF_y, reduce_array,
                     t_mode == GB300_MODE_FUSED_LAG);
}

void solve_hydro_2d(Mesh* mesh, int tt, double* P, double* rho,
                    double* rho_old, double* e, double* u, double* v,
                    double* rho_u, double* rho_v, double* Qxx, double* Qyy,
                    double* F_x, double* F_y, double* uF_x, double* uF_y,
                    double* vF_x, double* vF_y, double* reduce_array) {
  gb300_solve_hydro_2d(mesh, tt, P, rho, rho_old, e, u, v, rho_u, rho_v, Qxx,
                       Qyy, F_x, F_y, uF_x, uF_y, vF_x, vF_y, reduce_array);
}

void set_timestep(const int nx, const int ny, double* Qxx, double* Qyy,
                  const double* rho, const double* e, Mesh* mesh,
                  double* reduce_array, const int first_step,
                  const double* celldx, const double* celldy) {
  st_set_timestep(nx, ny, Qxx, Qyy, rho, e, mesh, reduce_array, first_step,
                  celldx, celldy);
}

void print_conservation(const int nx, const int ny, double* rho, double* e,
                        double* reduce_array, Mesh* mesh) {
  double tot[2] = {0.0, 0.0};
  if (!mesh) {
    record_error(GB300_ERR_ARG, "print_conservation: mesh is NULL");
    return;
  }
  if (st_conservation(nx, ny, mesh->pad, rho, e, reduce_array, tot, 1) ==
          GB300_OK &&
      g_verbose && mesh->rank == 0) {
    printf("Total mass:      %.12e\n", tot[0]);
    printf("Total energy:    %.12e\n", tot[1]);
  }
}

void equation_of_state(const int nx, const int ny, double* P, const double* rho,
                       const double* e) {
  if (nx <= 0 || ny <= 0) {
    record_error(GB300_ERR_ARG, "equation_of_state: empty mesh");
    return;
  }
  note_state_write();
  launch_eos(current_stream(), nx, ny, P, rho, e);
  check_launch("equation_of_state");
}

void pressure_acceleration(const int nx, const int ny, Mesh* mesh,
                           const double dt, double* rho_u, double* rho_v,
                           double* u, double* v, const double* P,
                           const double* rho, const double* edgedx,
                           const double* edgedy, const double* celldx,
                           const double* celldy) {
  st_pressure_acceleration(nx, ny, mesh, dt, rho_u, rho_v, u, v, P, rho,
                           MeshView{edgedx, edgedy, celldx, celldy});
}

void artificial_viscosity(const int nx, const int ny, Mesh* mesh,
                          const double dt, double* Qxx, double* Qyy, double* u,
                          double* v, double* rho_u, double* rho_v,
                          const double* rho, const double* edgedx,
                          const double* edgedy, const double* celldx,
                          const double* celldy) {
  st_artificial_viscosity(nx, ny, mesh, dt, Qxx, Qyy, u, v, rho_u, rho_v, rho,
                          MeshView{edgedx, edgedy, celldx, celldy});
}

void shock_heating_and_work(const int nx, const int ny, Mesh* mesh,
                            const double dt_h, double* e, const double* P,
                            const double* u, const double* v, const double* rho,
                            const double* Qxx, const double* Qyy,
                            const double* celldx, const double* celldy) {
  st_shock_heating(nx, ny, mesh, dt_h, e, P, u, v, rho, Qxx, Qyy,
                   MeshView{nullptr, nullptr, celldx, celldy});
}

void advect_mass_and_energy(const int nx, const int ny, Mesh* mesh,
                            const int tt, const double dt, const double dt_h,
                            double* rho, double* e, double* rho_old,
                            double* F_x, double* F_y, double* eF_x,
                            double* eF_y, const double* u, const double* v,
                            const double* edgedx, const double* edgedy,
                            const double* celldx, const double* celldy) {
  st_advect_mass_and_energy(nx, ny, mesh, tt, dt, dt_h, rho, e, rho_old, F_x,
                            F_y, eF_x, eF_y, u, v,
                            MeshView{edgedx, edgedy, celldx, celldy});
}

void x_mass_and_energy_flux(const int nx, const int ny, const int first,
                            Mesh* mesh, const double dt, const double dt_h,
                            double* rho, double* rho_old, double* e,
                            const double* u, double* F_x, double* eF_x,
                            const double* celldx, const double* edgedx,
                            const double* celldy, const double* edgedy) {
  if (check_mesh(mesh, nx, ny, "x_mass_and_energy_flux") != GB300_OK) return;
  st_mass_energy_sweep(false, nx, ny, first, mesh, dt, dt_h, rho, rho_old, e,
                       u, F_x, eF_x, MeshView{edgedx, edgedy, celldx, celldy});
}

void y_mass_and_energy_flux(const int nx, const int ny, const int first,
                            Mesh* mesh, const double dt, const double dt_h,
                            double* rho, double* rho_old, double* e,
                            const double* v, double* F_y, double* eF_y,
                            const double* celldx, const double* edgedx,
                            const double* celldy, const double* edgedy) {
  if (check_mesh(mesh, nx, ny, "y_mass_and_energy_flux") != GB300_OK) return;
  st_mass_energy_sweep(true, nx, ny, first, mesh, dt, dt_h, rho, rho_old, e, v,
                       F_y, eF_y, MeshView{edgedx, edgedy, celldx, celldy});
}

void advect_momentum(const int nx, const int ny, const int tt, Mesh* mesh,
                     const double dt_h, const double dt, double* u, double* v,
                     double* uF_x, double* uF_y, double* vF_x, double* vF_y,
                     double* rho_u, double* rho_v, const double* rho,
                     const double* F_x, const double* F_y,
                     const double* edgedx, const double* edgedy,
                     const double* celldx, const double* celldy) {
  (void)dt;
  st_advect_momentum(nx, ny, tt, mesh, dt_h, u, v, uF_x, uF_y, vF_x, vF_y,
                     rho_u, rho_v, rho, F_x, F_y,
                     MeshView{edgedx, edgedy, celldx, celldy});
}

void momentum_x_flux_in_x(const int nx, const int ny, Mesh* mesh,
                          const double dt_h, double* velocity_x, double* uF_x,
                          const double* mass_flux_x, const double* edgedx,
                          const double* edgedy, const double* celldx) {
  if (check_mesh(mesh, nx, ny, "momentum_x_flux_in_x") != GB300_OK) return;
  launch_uF_x(current_stream(), nx, ny, mesh->pad, dt_h, velocity_x, uF_x,
              mass_flux_x, MeshView{edgedx, edgedy, celldx, nullptr});
  check_launch("momentum_x_flux_in_x");
}

void momentum_x_flux_in_y(const int nx, const int ny, Mesh* mesh,
                          const double dt_h, double* velocity_x,
                          double* velocity_y, double* uF_y,
                          const double* mass_flux_y, const double* edgedx,
                          const double* edgedy, const double* celldy) {
  if (check_mesh(mesh, nx, ny, "momentum_x_flux_in_y") != GB300_OK) return;
  launch_uF_y(current_stream(), nx, ny, mesh->pad, dt_h, velocity_x,
              velocity_y, uF_y, mass_flux_y,
              MeshView{edgedx, edgedy, nullptr, celldy});
  check_launch("momentum_x_flux_in_y");
}

void momentum_y_flux_in_x(const int nx, const int ny, Mesh* mesh,
                          const double dt_h, const double* velocity_x,
                          double* velocity_y, double* vF_x,
                          const double* mass_flux_x, const double* edgedx,
                          const double* celldy, const double* celldx) {
  if (check_mesh(mesh, nx, ny, "momentum_y_flux_in_x") != GB300_OK) return;
  launch_vF_x(current_stream(), nx, ny, mesh->pad, dt_h, velocity_x,
              velocity_y, vF_x, mass_flux_x,
              MeshView{edgedx, nullptr, celldx, celldy});
  check_launch("momentum_y_flux_in_x");
}

void momentum_y_flux_in_y(const int nx, const int ny, Mesh* mesh,
                          const double dt_h, double* velocity_y, double* vF_y,
                          const double* mass_flux_y, const double* edgedy,
                          const double* celldx, const double* celldy) {
  if (check_mesh(mesh, nx, ny, "momentum_y_flux_in_y") != GB300_OK) return;
  launch_vF_y(current_stream(), nx, ny, mesh->pad, dt_h, velocity_y, vF_y,
              mass_flux_y, MeshView{nullptr, edgedy, celldx, celldy});
  check_launch("momentum_y_flux_in_y");
}

void handle_boundary_2d(const int nx, const int ny, Mesh* mesh, double* arr,
                        const int invert, const int pack) {
  (void)pack;
  if (!mesh) {
    record_error(GB300_ERR_ARG, "handle_boundary_2d: mesh is NULL");
    return;
  }
  if (check_mesh(mesh, nx, ny, "handle_boundary_2d") != GB300_OK) return;
  st_boundary(nx, ny, mesh, arr, invert);
  check_launch("handle_boundary_2d");
}

// ===========================================================================
// Part 2: control and status.

int gb300_last_error(void) { return t_err; }
const char* gb300_last_error_message(void) { return t_msg; }
void gb300_clear_error(void) {
  t_err = GB300_OK;
  t_msg[0] = '\0';
}
int gb300_set_stream(void* stream) {
  t_stream = static_cast<cudaStream_t>(stream);
  return GB300_OK;
}
void* gb300_get_stream(void) { return t_stream; }
int gb300_set_mode(int mode) {
  if (mode != GB300_MODE_EXACT && mode != GB300_MODE_FUSED && mode != GB300_MODE_FUSED_LAG) {
    return record_error(GB300_ERR_ARG, "gb300_set_mode: unknown mode %d", mode);
  }
  t_mode = mode;
  return GB300_OK;
}
int gb300_get_mode(void) { return t_mode; }
int gb300_state_changed(void) {
  note_state_write();
  return GB300_OK;
}
int gb300_set_lagrangian_rows(int rows) { return set_lagrangian_rows(rows); }
int gb300_set_halo_exchange(gb300_halo_fn fn, void* ctx) {
  g_halo_fn = fn;
  g_halo_ctx = ctx;
  return GB300_OK;
}
int gb300_set_reduce_min(gb300_reduce_min_fn fn, void* ctx) {
  g_rmin_fn = fn;
  g_rmin_ctx = ctx;
  return GB300_OK;
}
unsigned long long gb300_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }
int gb300_set_verbose(int v) {
  g_verbose = v;
  return GB300_OK;
}
int gb300_synchronize(void) {
  const cudaError_t err = cudaStreamSynchronize(t_stream);
  if (err != cudaSuccess) {
    return record_error(GB300_ERR_CUDA, "synchronize: %s", cudaGetErrorString(err));
  }
  return GB300_OK;
}
int gb300_conservation(int nx, int ny, int pad, const double* rho,
                       const double* e, double* reduce_array, double* out,
                       int sync) {
  return st_conservation(nx, ny, pad, rho, e, reduce_array, out, sync);
}

// ===========================================================================
// Part 3: the mixed-precision form.

size_t gb300_mixed_workspace_bytes(int local_nx, int local_ny) {
  return mixed_workspace_bytes(local_nx, local_ny);
}

size_t gb300_mixed_workspace_offset(int local_nx, int local_ny, int field) {
  return mixed_workspace_offset(local_nx, local_ny, field);
}

int gb300_mixed_prepare(Mesh* mesh, double* rho, double* e, void* workspace,
                        size_t bytes, double* reduce_array,
                        int initial_timestep) {
  if (!mesh) return record_error(GB300_ERR_ARG, "gb300_mixed_prepare: mesh is NULL");
  FLOW_TRY(check_single_rank(mesh, "gb300_mixed_prepare"));
  FLOW_TRY(check_mesh(mesh, mesh->local_nx, mesh->local_ny, "gb300_mixed_prepare"));
  FLOW_TRY(mixed_prepare(mesh, rho, e, workspace, bytes));
  if (!initial_timestep) return GB300_OK;
  // The driver's set_timestep(first_step = 0) before the loop (main.c:64-66)
  // with the zero viscous stresses of a fresh state: a workspace block that
  // mixed_prepare left zero serves as Qxx = Qyy = 0.
  const double* zeros = reinterpret_cast<const double*>(
      static_cast<const char*>(workspace) +
      mixed_zero_block_offset(mesh->local_nx, mesh->local_ny));
  return st_set_timestep(mesh->local_nx, mesh->local_ny, zeros, zeros, rho, e,
                         mesh, reduce_array, 0, mesh->celldx, mesh->celldy);
}

int gb300_mixed_solve(Mesh* mesh, int tt, double* rho, double* e, float* rho_u,
                      float* rho_v, void* workspace, size_t bytes,
                      double* reduce_array) {
  if (!mesh) return record_error(GB300_ERR_ARG, "gb300_mixed_solve: mesh is NULL");
  FLOW_TRY(check_single_rank(mesh, "gb300_mixed_solve"));
  FLOW_TRY(check_mesh(mesh, mesh->local_nx, mesh->local_ny, "gb300_mixed_solve"));
  if (g_verbose && mesh->rank == 0) {
    printf("Timestep:        %.12e\n", mesh->dt);
  }
  return mixed_solve(mesh, tt, rho, e, rho_u, rho_v, workspace, bytes, reduce_array);
}

}  // extern "C"
