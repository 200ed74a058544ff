// fused.cu -- the single-problem fused timestep (FP64 form behind
// solve_hydro_2d, and the mixed form gb300_mixed_solve): one kernel launch per
// phase, each CTA running one tile function of fused_tiles.cuh.
#include <cstddef>

#include "../../include/flow_gb300.h"
#include "fused.h"
#include "fused_tiles.cuh"
#include "profile.h"

namespace flow {
namespace {

using namespace tiles;

// reduce_array slot holding the running CFL minimum of the fused step (uint64
// bits; all candidates are non-negative, so bit order = value order).
constexpr int kRaMinBits = 6;
// reduce_array slot holding the whole-mesh power-of-two flag of the step.
constexpr int kRaMeshPow2 = 7;

// Programmatic dependent launch: every kernel of the step is launched with
// programmatic stream serialisation, lets the next kernel launch as soon as
// all its own CTAs have started (pdl_trigger), and waits for the previous
// kernel to complete (its writes visible) before touching the state
// (pdl_wait).  The next kernel's CTAs thus take the SMs its predecessor's
// last wave leaves idle.  Outside such a launch both are no-ops.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" :::);
}

// Whether every mesh spacing (celldx, edgedx: 0 .. nx; celldy, edgedy: 0 ..
// ny) is a positive normal power of two: one block, the first kernel of the
// step.  The tiles then skip their own spacing tests (block_mesh_pow2).
constexpr int kPow2Threads = 1024;
__global__ void __launch_bounds__(kPow2Threads)
    k_mesh_pow2(int nx, int ny, const double* celldx, const double* edgedx,
                const double* celldy, const double* edgedy, unsigned long long* flag) {
  pdl_wait();
  pdl_trigger();
  // Every test is made (no short circuit), so that a thread's loads are
  // independent and in flight together.
  bool ok = true;
#pragma unroll 4
  for (int j = threadIdx.x; j <= nx; j += kPow2Threads) {
    ok &= d_is_pow2(celldx[j]) & d_is_pow2(edgedx[j]);
  }
#pragma unroll 4
  for (int i = threadIdx.x; i <= ny; i += kPow2Threads) {
    ok &= d_is_pow2(celldy[i]) & d_is_pow2(edgedy[i]);
  }
  ok = __syncthreads_and(ok) != 0;
  if (threadIdx.x == 0) *flag = ok ? 1ull : 0ull;
}

template <typename R>
__global__ void __launch_bounds__(kCols) k_lag_pressure(const StepArgs<R> a) {
  pdl_wait();
  pdl_trigger();
  // The first kernel of the step clears the CFL minimum and the block ticket
  // of the shock-heating kernel (three kernels later, which waits for it).
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) {
    *reinterpret_cast<unsigned long long*>(a.ra + kRaTicket) = 0ull;
    *a.min_slot = ~0ull;
  }
  tile_lag_pressure(a, blockIdx.x, blockIdx.y);
}
template <typename R>
__global__ void __launch_bounds__(kCols) k_lag_viscosity(const StepArgs<R> a) {
  pdl_wait();
  pdl_trigger();
  tile_lag_viscosity(a, blockIdx.x, blockIdx.y);
}
template <typename R>
__global__ void __launch_bounds__(kCols) k_lag_viscous_accel(const StepArgs<R> a) {
  pdl_wait();
  pdl_trigger();
  tile_lag_viscous_accel(a, blockIdx.x, blockIdx.y);
}
// Shock heating + CFL minimum; the last block to finish (ticket in
// reduce_array) applies the dt rule.
template <typename R>
__global__ void __launch_bounds__(kCols) k_lag_energy_dt(const StepArgs<R> a) {
  __shared__ bool s_last;
  pdl_wait();
  pdl_trigger();
  tile_lag_energy_dt(a, blockIdx.x, blockIdx.y);
  if (threadIdx.x == 0) {
    __threadfence();
    unsigned long long* ticket = reinterpret_cast<unsigned long long*>(a.ra + kRaTicket);
    s_last = (atomicAdd(ticket, 1ull) == (unsigned long long)gridDim.x * gridDim.y - 1);
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    finish_dt(a);
    *reinterpret_cast<unsigned long long*>(a.ra + kRaTicket) = 0ull;
  }
}
template <typename R, bool kFirst>
__global__ void __launch_bounds__(kCols, Prec<R>::kMixed ? 8 : 7) k_mass_sweep_x(const StepArgs<R> a,
                                                        const SweepArgs<R> s) {
  pdl_wait();
  pdl_trigger();
  tile_mass_sweep_x<R, kFirst>(a, s, blockIdx.x, blockIdx.y);
}
template <typename R, bool kFirst>
__global__ void __launch_bounds__(kCols, Prec<R>::kMixed ? 7 : 6) k_mass_sweep_y(const StepArgs<R> a,
                                                        const SweepArgs<R> s) {
  pdl_wait();
  pdl_trigger();
  tile_mass_sweep_y<R, kFirst>(a, s, blockIdx.x, blockIdx.y);
}
// Momentum pairs (flux fused with its update): x pairs share a row's fluxes
// through shared memory (127 faces per CTA), y pairs march down columns.
template <typename R, bool kV, bool kVel>
__global__ void __launch_bounds__(kCols) k_mom_x(const StepArgs<R> a) {
  pdl_wait();
  pdl_trigger();
  tile_mom_x<R, kV, kVel>(a, blockIdx.x, blockIdx.y);
}
template <typename R, bool kV, bool kVel>
__global__ void __launch_bounds__(kCols) k_mom_y(const StepArgs<R> a) {
  pdl_wait();
  pdl_trigger();
  tile_mom_y<R, kV, kVel>(a, blockIdx.x, blockIdx.y);
}

// Launches kernel k with programmatic stream serialisation (see pdl_wait).
template <typename... KArgs, typename... Args>
void launch_pdl_block(void (*k)(KArgs...), dim3 grid, dim3 block, cudaStream_t s,
                      Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k, args...);
}
template <typename... KArgs, typename... Args>
void launch_pdl(void (*k)(KArgs...), dim3 grid, cudaStream_t s, Args... args) {
  launch_pdl_block(k, grid, dim3(kCols), s, args...);
}

inline dim3 strip_grid(int cols, int rows, int tile_rows, int cols_per_cta = kCols) {
  return dim3((unsigned)((cols + cols_per_cta - 1) / cols_per_cta),
              (unsigned)((rows + tile_rows - 1) / tile_rows));
}

// x pair for rho_u (kV false): x-faces pad .. nx-pad, 127 per CTA; for rho_v:
// y-faces pad .. nx-pad-1.  Rows: the faces' rows.
template <typename R, bool kV, bool kVel>
void launch_mom_x(cudaStream_t s, const StepArgs<R>& a) {
  const int cols = kV ? (a.nx - 2 * a.pad) : (a.nx + 1 - 2 * a.pad);
  const int rows = kV ? (a.ny + 1 - 2 * a.pad) : (a.ny - 2 * a.pad);
  launch_pdl(k_mom_x<R, kV, kVel>, strip_grid(cols, rows, a.rows, kCols - 1), s, a);
}
template <typename R, bool kV, bool kVel>
void launch_mom_y(cudaStream_t s, const StepArgs<R>& a) {
  const int cols = kV ? (a.nx - 2 * a.pad) : (a.nx + 1 - 2 * a.pad);
  const int rows = kV ? (a.ny + 1 - 2 * a.pad) : (a.ny - 2 * a.pad);
  launch_pdl(k_mom_y<R, kV, kVel>, strip_grid(cols, rows, a.rows), s, a);
}

template <typename R>
void launch_mass(cudaStream_t s, const StepArgs<R>& a, bool dir_y, bool first,
                 const SweepArgs<R>& sw) {
  const int pad = a.pad;
  if (dir_y) {
    const dim3 g = strip_grid(a.nx - 2 * pad, a.ny - 2 * pad, a.rows);
    if (first) launch_pdl(k_mass_sweep_y<R, true>, g, s, a, sw);
    else launch_pdl(k_mass_sweep_y<R, false>, g, s, a, sw);
  } else {
    // Faces pad .. nx-pad; every CTA advances 127 columns.
    const dim3 g = strip_grid(a.nx + 1 - 2 * pad, a.ny - 2 * pad, a.rows, kCols - 1);
    if (first) launch_pdl(k_mass_sweep_x<R, true>, g, s, a, sw);
    else launch_pdl(k_mass_sweep_x<R, false>, g, s, a, sw);
  }
}

// One timestep of either form; first/second are the two mass sweeps' buffers.
template <typename R>
void launch_step(cudaStream_t s, const StepArgs<R>& a, int tt,
                 const SweepArgs<R>& first, const SweepArgs<R>& second,
                 StepProfiler& prof) {
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  // The whole-mesh spacing test the tiles read (the mesh may change between
  // calls, so it is formed every step; one block, a few microseconds).
  prof.mark("mesh_pow2");
  launch_pdl_block(k_mesh_pow2, dim3(1), dim3(kPow2Threads), s, nx, ny, a.celldx, a.edgedx,
                   a.celldy, a.edgedy, const_cast<unsigned long long*>(a.mesh_pow2));
  prof.mark("lag_pressure");
  launch_pdl(k_lag_pressure<R>, strip_grid(nx, ny, a.rows), s, a);
  prof.mark("lag_viscosity");
  launch_pdl(k_lag_viscosity<R>, strip_grid(nx - 2 * pad, ny - 2 * pad, a.rows), s, a);
  prof.mark("lag_viscous_accel");
  launch_pdl(k_lag_viscous_accel<R>, strip_grid(nx + 1 - 2 * pad, ny + 1 - 2 * pad, a.rows), s, a);
  prof.mark("lag_energy_dt");
  launch_pdl(k_lag_energy_dt<R>, strip_grid(nx - 2 * pad, ny - 2 * pad, a.rows), s, a);

  const bool x_first = (tt % 2 == 0);
  prof.mark(x_first ? "mass_sweep_x" : "mass_sweep_y");
  launch_mass(s, a, !x_first, true, first);
  prof.mark(x_first ? "mass_sweep_y" : "mass_sweep_x");
  launch_mass(s, a, x_first, false, second);

  // Momentum: each flux fused with its update, in the reference order; the
  // pair that recomputes a velocity comes first in each chain.
  if (tt % 2) {
    prof.mark("mom_uFx");
    launch_mom_x<R, false, true>(s, a);
    prof.mark("mom_uFy");
    launch_mom_y<R, false, false>(s, a);
    prof.mark("mom_vFx");
    launch_mom_x<R, true, true>(s, a);
    prof.mark("mom_vFy");
    launch_mom_y<R, true, false>(s, a);
  } else {
    prof.mark("mom_uFy");
    launch_mom_y<R, false, true>(s, a);
    prof.mark("mom_uFx");
    launch_mom_x<R, false, false>(s, a);
    prof.mark("mom_vFy");
    launch_mom_y<R, true, true>(s, a);
    prof.mark("mom_vFx");
    launch_mom_x<R, true, false>(s, a);
  }
}

int finish_step(cudaStream_t s, Mesh* mesh, double* ra, StepProfiler& prof,
                const char* where) {
  {
    const int st = check_launch(where);
    if (st != GB300_OK) return st;
  }
  double pair[2];
  cudaMemcpyAsync(pair, ra + kRaDt, sizeof(pair), cudaMemcpyDeviceToHost, s);
  const cudaError_t err = cudaStreamSynchronize(s);
  if (err != cudaSuccess) {
    return record_error(GB300_ERR_CUDA, "%s: %s", where, cudaGetErrorString(err));
  }
  prof.end();
  mesh->dt = pair[0];
  mesh->dt_h = pair[1];
  return GB300_OK;
}

template <typename R>
void fill_mesh_args(StepArgs<R>& a, const Mesh* mesh, int tt, double* ra) {
  a.nx = mesh->local_nx;
  a.ny = mesh->local_ny;
  a.pad = mesh->pad;
  a.edgedx = mesh->edgedx;
  a.edgedy = mesh->edgedy;
  a.celldx = mesh->celldx;
  a.celldy = mesh->celldy;
  a.ra = ra;
  a.min_slot = reinterpret_cast<unsigned long long*>(ra + kRaMinBits);
  a.mesh_pow2 = reinterpret_cast<unsigned long long*>(ra + kRaMeshPow2);
  a.dt_slot = ra + kRaDt;
  a.dt = mesh->dt;
  a.dt_h = mesh->dt_h;
  a.max_dt = mesh->max_dt;
  a.first_step = (tt == 0);
  a.rows = kDefaultRows;
}

}  // namespace

// Mixed form: workspace layout (bytes, each block 256-byte aligned).
namespace {

struct MixedLayout {
  size_t rho_r, e_r, u, v, Qxx, Qyy, F_x, F_y, uF_x, uF_y, vF_x, vF_y, s_r, s_e,
      s_r32, s_e32, total;
};

MixedLayout mixed_layout(int nx, int ny) {
  const size_t nc = (size_t)nx * ny, nf = (size_t)(nx + 1) * (ny + 1);
  MixedLayout L{};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t at = off;
    off += (bytes + 255) / 256 * 256;
    return at;
  };
  L.rho_r = take(nc * 4);
  L.e_r = take(nc * 4);
  L.u = take(nf * 4);
  L.v = take(nf * 4);
  L.Qxx = take(nc * 4);
  L.Qyy = take(nc * 4);
  L.F_x = take(nf * 4);
  L.F_y = take(nf * 4);
  L.uF_x = take(nf * 4);
  L.uF_y = take(nf * 4);
  L.vF_x = take(nf * 4);
  L.vF_y = take(nf * 4);
  L.s_r = take(nc * 8);
  L.s_e = take(nc * 8);
  L.s_r32 = take(nc * 4);
  L.s_e32 = take(nc * 4);
  L.total = off;
  return L;
}

__global__ void k_make_shadows(size_t n, const double* rho, const double* e,
                               float* rho_r, float* e_r) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    rho_r[i] = f64_to_f32(rho[i]);
    e_r[i] = f64_to_f32(e[i]);
  }
}

}  // namespace

int fused_solve(Mesh* mesh, int tt, double* P, double* rho, double* rho_old,
                double* e, double* u, double* v, double* rho_u, double* rho_v,
                double* Qxx, double* Qyy, double* F_x, double* F_y,
                double* uF_x, double* uF_y, double* vF_x, double* vF_y,
                double* reduce_array) {
  if (!reduce_array) return record_error(GB300_ERR_ARG, "solve_hydro_2d: reduce_array is NULL");
  cudaStream_t s = current_stream();
  StepArgs<double> a;
  fill_mesh_args(a, mesh, tt, reduce_array);
  a.rho = rho; a.e = e; a.rho_r = rho; a.e_r = e;
  a.P = P; a.rho_old = rho_old;
  // The Lagrangian phase and the sweeps keep the velocities in uF_y/vF_x (the
  // fused momentum pairs store no fluxes); the advected ones land in u/v.
  a.u = uF_y; a.v = vF_x; a.u_out = u; a.v_out = v;
  a.rho_u = rho_u; a.rho_v = rho_v; a.Qxx = Qxx; a.Qyy = Qyy;
  a.F_x = F_x; a.F_y = F_y; a.uF_x = uF_x; a.uF_y = uF_y; a.vF_x = vF_x;
  a.vF_y = vF_y;
  // The first mass sweep writes into the two cell-sized buffers that hold
  // momentum fluxes later in the step (uF_x, vF_y); the second writes back
  // into rho/e, so neither sweep updates its own input.
  const SweepArgs<double> first{rho, e, rho, e, uF_x, vF_y, uF_x, vF_y};
  const SweepArgs<double> second{uF_x, vF_y, uF_x, vF_y, rho, e, rho, e};
  StepProfiler prof;
  prof.begin(s);
  launch_step(s, a, tt, first, second, prof);
  return finish_step(s, mesh, reduce_array, prof, "solve_hydro_2d (fused)");
}

size_t mixed_workspace_bytes(int nx, int ny) { return mixed_layout(nx, ny).total; }

size_t mixed_zero_block_offset(int nx, int ny) { return mixed_layout(nx, ny).s_r; }

size_t mixed_workspace_offset(int nx, int ny, int field) {
  const MixedLayout L = mixed_layout(nx, ny);
  if (field == GB300_MIXED_U) return L.u;
  if (field == GB300_MIXED_V) return L.v;
  return (size_t)-1;
}

int mixed_prepare(Mesh* mesh, double* rho, double* e, void* work, size_t bytes) {
  const int nx = mesh->local_nx, ny = mesh->local_ny;
  const MixedLayout L = mixed_layout(nx, ny);
  if (!work || bytes < L.total) {
    return record_error(GB300_ERR_ARG,
                        "gb300_mixed_prepare: workspace of %zu bytes, need %zu",
                        bytes, L.total);
  }
  cudaStream_t s = current_stream();
  char* w = static_cast<char*>(work);
  cudaMemsetAsync(work, 0, L.total, s);
  const size_t n = (size_t)nx * ny;
  size_t blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  k_make_shadows<<<(unsigned)blocks, 256, 0, s>>>(
      n, rho, e, reinterpret_cast<float*>(w + L.rho_r),
      reinterpret_cast<float*>(w + L.e_r));
  return check_launch("gb300_mixed_prepare");
}

int mixed_solve(Mesh* mesh, int tt, double* rho, double* e, float* rho_u,
                float* rho_v, void* work, size_t bytes, double* reduce_array) {
  const int nx = mesh->local_nx, ny = mesh->local_ny;
  const MixedLayout L = mixed_layout(nx, ny);
  if (!work || bytes < L.total) {
    return record_error(GB300_ERR_ARG,
                        "gb300_mixed_solve: workspace of %zu bytes, need %zu", bytes,
                        L.total);
  }
  if (!reduce_array) {
    return record_error(GB300_ERR_ARG, "gb300_mixed_solve: reduce_array is NULL");
  }
  char* w = static_cast<char*>(work);
  auto F = [&](size_t off) { return reinterpret_cast<float*>(w + off); };
  auto D = [&](size_t off) { return reinterpret_cast<double*>(w + off); };
  cudaStream_t s = current_stream();
  StepArgs<float> a;
  fill_mesh_args(a, mesh, tt, reduce_array);
  a.rho = rho; a.e = e; a.rho_r = F(L.rho_r); a.e_r = F(L.e_r);
  a.P = nullptr; a.rho_old = nullptr;
  a.u = F(L.uF_y); a.v = F(L.vF_x); a.u_out = F(L.u); a.v_out = F(L.v);
  a.rho_u = rho_u; a.rho_v = rho_v;
  a.Qxx = F(L.Qxx); a.Qyy = F(L.Qyy); a.F_x = F(L.F_x); a.F_y = F(L.F_y);
  a.uF_x = F(L.uF_x); a.uF_y = F(L.uF_y); a.vF_x = F(L.vF_x); a.vF_y = F(L.vF_y);
  const SweepArgs<float> first{rho, e, a.rho_r, a.e_r, D(L.s_r), D(L.s_e),
                               F(L.s_r32), F(L.s_e32)};
  const SweepArgs<float> second{D(L.s_r), D(L.s_e), F(L.s_r32), F(L.s_e32),
                                rho, e, a.rho_r, a.e_r};
  StepProfiler prof;
  prof.begin(s);
  launch_step(s, a, tt, first, second, prof);
  return finish_step(s, mesh, reduce_array, prof, "gb300_mixed_solve");
}

}  // namespace flow
