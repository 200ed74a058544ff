// fused.cu -- the single-problem fused timestep (FP64 form behind
// solve_hydro_2d, and the mixed form gb300_mixed_solve): one kernel launch per
// phase, each CTA running one tile function of fused_tiles.cuh.
#include <array>
#include <cstddef>

#include "../../include/flow_gb300.h"
#include "fused.h"
#include "fused_tiles.cuh"
#include "lag_fused.cuh"
#include "profile.h"

namespace flow {
namespace {

using namespace tiles;

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
// It also clears the CFL minimum slot and the block ticket for the step's
// Lagrangian kernels, and the count of moving first-sweep tiles.
__global__ void __launch_bounds__(kPow2Threads)
    k_mesh_pow2(int nx, int ny, const double* celldx, const double* edgedx,
                const double* celldy, const double* edgedy, unsigned long long* flag,
                double* ra) {
  pdl_wait();
  pdl_trigger();
  if (threadIdx.x == 0) {
    *reinterpret_cast<unsigned long long*>(ra + kRaTicket) = 0ull;
    *reinterpret_cast<unsigned long long*>(ra + kRaMinBits) = ~0ull;
    *reinterpret_cast<unsigned long long*>(ra + kRaMoving) = 0ull;
  }
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

template <typename R, bool kFl>
__global__ void __launch_bounds__(kCols) k_lag_pressure(const StepArgs<R> a) {
  pdl_wait();
  pdl_trigger();
  // The first kernel of the step clears the CFL minimum and the block ticket
  // of the shock-heating kernel (three kernels later, which waits for it).
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) {
    *reinterpret_cast<unsigned long long*>(a.ra + kRaTicket) = 0ull;
    *a.min_slot = ~0ull;
    if (a.moving) *a.moving = 0ull;
  }
  tile_lag_pressure<R, kFl>(a, blockIdx.x, blockIdx.y);
}
// kFlags: the viscous-stress flags (a.qmask) are kept -- the viscosity
// kernel stores only warp rows with a non-zero stress, and the two kernels
// after it load only those.
template <typename R, bool kFlags>
__global__ void __launch_bounds__(kCols) k_lag_viscosity(const StepArgs<R> a) {
  pdl_wait();
  pdl_trigger();
  tile_lag_viscosity<R, kFlags>(a, blockIdx.x, blockIdx.y);
}
template <typename R, bool kFlags>
__global__ void __launch_bounds__(kCols) k_lag_viscous_accel(const StepArgs<R> a) {
  pdl_wait();
  pdl_trigger();
  tile_lag_viscous_accel<R, true, kFlags>(a, blockIdx.x, blockIdx.y);
}
// Shock heating + CFL minimum; the last block to finish (ticket in
// reduce_array) applies the dt rule.
template <typename R, bool kFlags>
__global__ void __launch_bounds__(kCols) k_lag_energy_dt(const StepArgs<R> a) {
  __shared__ bool s_last;
  __shared__ unsigned long long s_tile_min;  // the tile's CFL minimum (kFlags)
  pdl_wait();
  pdl_trigger();
  tile_lag_energy_dt<R, true, kFlags>(a, blockIdx.x, blockIdx.y, kFlags ? &s_tile_min : nullptr);
  if (threadIdx.x == 0) {
    // (Thread 0 wrote the minimum it stores here.)
    if (kFlags && a.cfl_tile) {
      a.cfl_tile[(size_t)blockIdx.y * a.qm_stride + blockIdx.x] = s_tile_min;
    }
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
// kFl (sweeps and momentum pairs): the mass-flux flags (a.fxflag, a.fyflag)
// are kept -- the sweeps store only warps with a non-zero mass flux, and the
// momentum pairs load only those.
template <typename R, bool kFirst, bool kFl>
__global__ void __launch_bounds__(kCols, Prec<R>::kMixed ? 8 : 7) k_mass_sweep_x(const StepArgs<R> a,
                                                        const SweepArgs<R> s) {
  pdl_wait();
  pdl_trigger();
  tile_mass_sweep_x<R, kFirst, true, kFl>(a, s, blockIdx.x, blockIdx.y);
}
template <typename R, bool kFirst, bool kFl>
__global__ void __launch_bounds__(kCols, Prec<R>::kMixed ? 7 : 6) k_mass_sweep_y(const StepArgs<R> a,
                                                        const SweepArgs<R> s) {
  pdl_wait();
  pdl_trigger();
  tile_mass_sweep_y<R, kFirst, true, kFl>(a, s, blockIdx.x, blockIdx.y);
}
// Momentum pairs (flux fused with its update): x pairs share a row's fluxes
// through shared memory (127 faces per CTA), y pairs march down columns.
template <typename R, bool kV, bool kVel, bool kFl>
__global__ void __launch_bounds__(kCols) k_mom_x(const StepArgs<R> a) {
  pdl_wait();
  pdl_trigger();
  tile_mom_x<R, kV, kVel, true, kFl>(a, blockIdx.x, blockIdx.y);
}
template <typename R, bool kV, bool kVel, bool kFl>
__global__ void __launch_bounds__(kCols) k_mom_y(const StepArgs<R> a) {
  pdl_wait();
  pdl_trigger();
  tile_mom_y<R, kV, kVel, true, kFl>(a, blockIdx.x, blockIdx.y);
}

// The whole Lagrangian phase of the FP64 step in one kernel (lag_fused.cuh):
// pressure, viscosity, viscous acceleration, shock heating and the CFL
// minimum; the last block to finish (ticket in reduce_array) applies the dt
// rule.  A tile whose row copies were lost records GB300_ERR_TIMEOUT in the
// status word and leaves the dt pair unchanged.
__global__ void __launch_bounds__(lagf::kT, 4) k_lag_fused(const lagf::LagArgs a) {
  __shared__ lagf::LagSmem sm;
  __shared__ unsigned long long s_warp[lagf::kWarps];
  __shared__ bool s_last;
  pdl_wait();
  pdl_trigger();
  lagf::CflBest cfl;
  const lagf::TileGeom g = lagf::tile_geom(a, blockIdx.x, blockIdx.y);
  const bool ok = lagf::tile_pow2(a, g)
                      ? lagf::lag_tile<true>(a, sm, blockIdx.x, blockIdx.y, cfl)
                      : lagf::lag_tile<false>(a, sm, blockIdx.x, blockIdx.y, cfl);
  if (!ok) {
    if (threadIdx.x == 0) {
      atomicExch(reinterpret_cast<unsigned long long*>(a.ra + kRaStatus),
                 (unsigned long long)GB300_ERR_TIMEOUT);
    }
    return;
  }
  unsigned long long best = ~0ull;
  if (cfl.kbest >= 0) best = (unsigned long long)dbits(cfl.c_best * d_rsqrt(cfl.s_best));
  best = warp_min_u64(best);
  if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = best;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long b = s_warp[0];
    for (int w = 1; w < lagf::kWarps; ++w) b = (s_warp[w] < b) ? s_warp[w] : b;
    atomicMin(a.min_slot, b);
    __threadfence();
    unsigned long long* ticket = reinterpret_cast<unsigned long long*>(a.ra + kRaTicket);
    s_last = (atomicAdd(ticket, 1ull) == (unsigned long long)gridDim.x * gridDim.y - 1);
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    // The leapfrog dt/dt_h rule of omp3/flow.c:103-105 (finish_dt).
    const unsigned long long gmin = atomicExch(a.min_slot, ~0ull);
    const double cflv = d_min_pos(a.max_dt, dfrom((long long)gmin));
    const double limited = dmin(cflv, __dmul_rn(FLOW_C_M, a.dt_h));
    const double dt = __dmul_rn(0.5, __dadd_rn(__dmul_rn(kCT, limited), a.dt_h));
    a.dt_slot[0] = dt;
    a.dt_slot[1] = a.first_step ? dt : __dmul_rn(kCT, limited);
    *reinterpret_cast<unsigned long long*>(a.ra + kRaTicket) = 0ull;
  }
}

// Copies the changed energies (with their ghost images) and momenta of the
// fused Lagrangian kernel into the state arrays.  Each thread reads the three
// change masks of one (mask row, tile) pair -- 48 contiguous bytes, so the
// scan is one coalesced pass over the masks -- and the warp then copies the
// flagged values of each non-empty pair together, one lane per column.
constexpr int kApplyThreads = 256;
__global__ void __launch_bounds__(kApplyThreads)
    k_lag_apply(const lagf::LagArgs a, double* e, double* rho_u, double* rho_v) {
  pdl_wait();
  pdl_trigger();
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int lane = threadIdx.x & 31;
  const int pairs = (ny + 1) * a.ntx;
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < pairs; base += stride) {
    const int k = base + (int)threadIdx.x;
    uint4 m[lagf::kMaskFields] = {};
    bool any = false;
    if (k < pairs) {
      const int row = k / a.ntx;
      // Mask rows the tiles write: cells and x faces pad .. ny-pad-1, y faces
      // pad .. ny-pad.
      if (row >= pad && row <= ny - pad) {
        const uint4* mk = reinterpret_cast<const uint4*>(a.masks) + (size_t)k * lagf::kMaskFields;
#pragma unroll
        for (int f = 0; f < lagf::kMaskFields; ++f) {
          if (f != lagf::kMaskRhoV && row == ny - pad) continue;
          m[f] = mk[f];
          any |= (m[f].x | m[f].y | m[f].z | m[f].w) != 0u;
        }
      }
    }
    unsigned todo = __ballot_sync(0xffffffffu, any);
    while (todo) {
      const int src = __ffs(todo) - 1;
      todo &= todo - 1;
      const int kk = __shfl_sync(0xffffffffu, k, src);
      const int row = kk / a.ntx;
      const int c0 = pad + (kk - row * a.ntx) * lagf::kW - lagf::kHalo;
#pragma unroll
      for (int f = 0; f < lagf::kMaskFields; ++f) {
        const unsigned w0 = __shfl_sync(0xffffffffu, m[f].x, src);
        const unsigned w1 = __shfl_sync(0xffffffffu, m[f].y, src);
        const unsigned w2 = __shfl_sync(0xffffffffu, m[f].z, src);
        const unsigned w3 = __shfl_sync(0xffffffffu, m[f].w, src);
        const unsigned words[lagf::kWarps] = {w0, w1, w2, w3};
#pragma unroll
        for (int w = 0; w < lagf::kWarps; ++w) {
          if (!((words[w] >> lane) & 1u)) continue;
          const int col = c0 + 32 * w + lane;
          if (f == lagf::kMaskE) {
            const size_t ci = cidx(nx, row, col);
            const double val = a.e_new[ci];
            e[ci] = val;
            mirror(true, e, nx, ny, pad, row, col, val, false, false);
          } else if (f == lagf::kMaskRhoU) {
            const size_t fi = fidx(nx, row, col);
            rho_u[fi] = a.rho_u_new[fi];
          } else {
            const size_t ci = cidx(nx, row, col);
            rho_v[ci] = a.rho_v_new[ci];
          }
        }
      }
    }
  }
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
  count_launches(1);
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
// Tile heights of the momentum pairs (with and without the velocity
// update) and of the viscous acceleration: the pairs without a velocity
// update and the viscous update skip the still tiles (flags) and work only
// where the flow moves, and shorter tiles there shorten the longest tile's
// chain of rows, which bounds such a kernel.
constexpr int kRowsMomVel = 16, kRowsMomFlux = 8, kRowsAccel = 8;
// Tile heights of the pressure, viscosity and shock-heating kernels, and of
// the two mass sweeps (whose bands are also the skip marks' bands): a step
// whose previous step's first sweep skipped at least half of its tiles takes
// the shorter sweep tiles (the moving tiles' chains of rows bound a sweep
// there), others the taller ones (less halo work on a field in motion).
constexpr int kRowsLag = 16, kRowsSweepStill = 8, kRowsSweepMoving = 16;
template <typename R>
StepArgs<R> with_rows(const StepArgs<R>& a, int rows) {
  StepArgs<R> b = a;
  b.rows = rows;
  return b;
}

template <typename R, bool kV, bool kVel>
void launch_mom_x(cudaStream_t s, const StepArgs<R>& a0) {
  const StepArgs<R> a = with_rows(a0, kVel ? kRowsMomVel : kRowsMomFlux);
  const int cols = kV ? (a.nx - 2 * a.pad) : (a.nx + 1 - 2 * a.pad);
  const int rows = kV ? (a.ny + 1 - 2 * a.pad) : (a.ny - 2 * a.pad);
  launch_pdl(a.fxflag ? k_mom_x<R, kV, kVel, true> : k_mom_x<R, kV, kVel, false>,
             strip_grid(cols, rows, a.rows, kCols - 1), s, a);
}
template <typename R, bool kV, bool kVel>
void launch_mom_y(cudaStream_t s, const StepArgs<R>& a0) {
  const StepArgs<R> a = with_rows(a0, kVel ? kRowsMomVel : kRowsMomFlux);
  const int cols = kV ? (a.nx - 2 * a.pad) : (a.nx + 1 - 2 * a.pad);
  const int rows = kV ? (a.ny + 1 - 2 * a.pad) : (a.ny - 2 * a.pad);
  launch_pdl(a.fyflag ? k_mom_y<R, kV, kVel, true> : k_mom_y<R, kV, kVel, false>,
             strip_grid(cols, rows, a.rows), s, a);
}

template <typename R>
void launch_mass(cudaStream_t s, const StepArgs<R>& a, bool dir_y, bool first,
                 const SweepArgs<R>& sw) {
  const int pad = a.pad;
  if (dir_y) {
    const bool fl = a.fyflag != nullptr;
    const dim3 g = strip_grid(a.nx - 2 * pad, a.ny - 2 * pad, a.rows);
    if (first) {
      launch_pdl(fl ? k_mass_sweep_y<R, true, true> : k_mass_sweep_y<R, true, false>, g, s, a, sw);
    } else {
      launch_pdl(fl ? k_mass_sweep_y<R, false, true> : k_mass_sweep_y<R, false, false>, g, s, a,
                 sw);
    }
  } else {
    const bool fl = a.fxflag != nullptr;
    // Faces pad .. nx-pad; every CTA advances 127 columns.
    const dim3 g = strip_grid(a.nx + 1 - 2 * pad, a.ny - 2 * pad, a.rows, kCols - 1);
    if (first) {
      launch_pdl(fl ? k_mass_sweep_x<R, true, true> : k_mass_sweep_x<R, true, false>, g, s, a, sw);
    } else {
      launch_pdl(fl ? k_mass_sweep_x<R, false, true> : k_mass_sweep_x<R, false, false>, g, s, a,
                 sw);
    }
  }
}

// Blocks of k_lag_apply: one thread per (mask row, tile) pair, at most 8
// blocks per SM (a grid-stride loop covers the rest).
inline int apply_blocks(const lagf::LagArgs& l) {
  const int pairs = (l.ny + 1) * l.ntx;
  const int need = (pairs + kApplyThreads - 1) / kApplyThreads;
  return need < 8 * num_sms() ? need : 8 * num_sms();
}

// One timestep of either form; first/second are the two mass sweeps' buffers.
// lag: the FP64 form's one-kernel Lagrangian phase (k_lag_fused +
// k_lag_apply), or null for the four separate Lagrangian kernels.
// mesh_known: the step directly follows a step on the same mesh arrays (no
// mesh call between), whose spacing test reduce_array still holds.
template <typename R>
void launch_step(cudaStream_t s, const StepArgs<R>& a, int tt,
                 const SweepArgs<R>& first, const SweepArgs<R>& second,
                 StepProfiler& prof, int sweep_rows, bool mesh_known,
                 const lagf::LagArgs* lag = nullptr) {
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  // The whole-mesh spacing test the tiles read (one block, a few
  // microseconds), formed unless the previous step's still stands.
  if (!mesh_known) {
    prof.mark("mesh_pow2");
    launch_pdl_block(k_mesh_pow2, dim3(1), dim3(kPow2Threads), s, nx, ny, a.celldx, a.edgedx,
                     a.celldy, a.edgedy, const_cast<unsigned long long*>(a.mesh_pow2), a.ra);
  }
  if (lag) {
    const int nty = (ny - 2 * pad + lag->rows - 1) / lag->rows;
    prof.mark("lag_fused");
    launch_pdl_block(k_lag_fused, dim3((unsigned)lag->ntx, (unsigned)nty), dim3(lagf::kT), s,
                     *lag);
    prof.mark("lag_apply");
    launch_pdl_block(k_lag_apply, dim3((unsigned)apply_blocks(*lag)), dim3(kApplyThreads), s,
                     *lag, const_cast<double*>(lag->e), const_cast<double*>(lag->rho_u),
                     const_cast<double*>(lag->rho_v));
  } else {
    prof.mark("lag_pressure");
    launch_pdl(a.vflag ? k_lag_pressure<R, true> : k_lag_pressure<R, false>,
               strip_grid(nx, ny, a.rows), s, a);
    const bool fl = a.qmask != nullptr;
    prof.mark("lag_viscosity");
    launch_pdl(fl ? k_lag_viscosity<R, true> : k_lag_viscosity<R, false>,
               strip_grid(nx - 2 * pad, ny - 2 * pad, a.rows), s, a);
    prof.mark("lag_viscous_accel");
    const StepArgs<R> aa = with_rows(a, kRowsAccel);
    launch_pdl(fl ? k_lag_viscous_accel<R, true> : k_lag_viscous_accel<R, false>,
               strip_grid(nx + 1 - 2 * pad, ny + 1 - 2 * pad, aa.rows), s, aa);
    prof.mark("lag_energy_dt");
    launch_pdl(fl ? k_lag_energy_dt<R, true> : k_lag_energy_dt<R, false>,
               strip_grid(nx - 2 * pad, ny - 2 * pad, a.rows), s, a);
  }

  // The advection phase reads velocity flags only when this step's
  // Lagrangian kernels wrote them (not the one-kernel phase).
  StepArgs<R> ad = a;
  if (lag) ad.vflag = nullptr;
  const StepArgs<R> as = with_rows(ad, sweep_rows);
  const bool x_first = (tt % 2 == 0);
  // With flags, the first sweep marks the tiles it skips (in its own grid);
  // the second reads their cells from the first sweep's input.
  SweepArgs<R> sw1 = first, sw2 = second;
  if (a.skipf) {
    sw1.skip = sw2.skip = a.skipf;
    sw1.skip_tiles_x = sw2.skip_tiles_x = x_first ? a.fx_stride / 4 : a.qm_stride;
    sw1.skip_bands = sw2.skip_bands = (ny - 2 * pad + sweep_rows - 1) / sweep_rows;
    sw2.r_alt = first.r_in;
    sw2.e_alt = first.e_in;
    sw2.r_alt_r = first.r_in_r;
    sw2.e_alt_r = first.e_in_r;
  }
  prof.mark(x_first ? "mass_sweep_x" : "mass_sweep_y");
  launch_mass(s, as, !x_first, true, sw1);
  prof.mark(x_first ? "mass_sweep_y" : "mass_sweep_x");
  launch_mass(s, as, x_first, false, sw2);

  // Momentum: each flux fused with its update, in the reference order; the
  // pair that recomputes a velocity comes first in each chain.
  if (tt % 2) {
    prof.mark("mom_uFx");
    launch_mom_x<R, false, true>(s, ad);
    prof.mark("mom_uFy");
    launch_mom_y<R, false, false>(s, ad);
    prof.mark("mom_vFx");
    launch_mom_x<R, true, true>(s, ad);
    prof.mark("mom_vFy");
    launch_mom_y<R, true, false>(s, ad);
  } else {
    prof.mark("mom_uFy");
    launch_mom_y<R, false, true>(s, ad);
    prof.mark("mom_uFx");
    launch_mom_x<R, false, false>(s, ad);
    prof.mark("mom_vFy");
    launch_mom_y<R, true, true>(s, ad);
    prof.mark("mom_vFx");
    launch_mom_x<R, true, false>(s, ad);
  }
}

int finish_step(cudaStream_t s, Mesh* mesh, double* ra, StepProfiler& prof,
                const char* where, unsigned long long* moving = nullptr) {
  {
    const int st = check_launch(where);
    if (st != GB300_OK) return st;
  }
  // dt, dt_h (slots 0, 1), the status word (slot 5) and the moving-tile
  // count (slot 8) in one copy.
  double head[kRaMoving + 1];
  cudaMemcpyAsync(head, ra + kRaDt, sizeof(head), cudaMemcpyDeviceToHost, s);
  const cudaError_t err = cudaStreamSynchronize(s);
  if (err != cudaSuccess) {
    return record_error(GB300_ERR_CUDA, "%s: %s", where, cudaGetErrorString(err));
  }
  prof.end();
  unsigned long long status;
  memcpy(&status, &head[kRaStatus], sizeof(status));
  if (status != 0ull) {
    cudaMemsetAsync(ra + kRaStatus, 0, sizeof(double), s);
    return record_error(GB300_ERR_TIMEOUT,
                        "%s: a row copy of the Lagrangian kernel did not arrive", where);
  }
  if (moving) memcpy(moving, &head[kRaMoving], sizeof(*moving));
  const double pair[2] = {head[kRaDt], head[kRaDtH]};
  mesh->dt = pair[0];
  mesh->dt_h = pair[1];
  return GB300_OK;
}

// Where the fused step's flags sit in reduce_array after the reduction
// partials (ra + kRaQFlags), when it holds them (it has nx*ny doubles, as the
// arch layer allocates it); a mesh too small for them stores and reads every
// stress and flux.  Offsets in 4-byte words: the per-tile CFL minima (two
// words per shock-heating tile) and the conservation totals' tile partials
// (four words per kConsTile^2 tile) first, 8-byte aligned; then the stress
// flags ((ny - 2 pad) x stride words), the y mass-flux flags
// ((ny + 1 - 2 pad) x stride), the x mass-flux flags ((ny - 2 pad) x xtiles),
// the velocity flags (ny x vtiles) and the skip marks of even and odd steps
// (a step's first sweep writes its own half; the next step reads it while its
// own first sweep writes the other).
constexpr int kConsTile = 128;  // rows and columns of a conservation tile
struct FlagLayout {
  bool fits = false;
  int stride = 0, xtiles = 0, vtiles = 0, cons_tx = 0, cons_ty = 0;
  size_t cfl = 0, cons = 0, q = 0, fy = 0, fx = 0, v = 0, marks = 0, sk_words = 0;
};
FlagLayout flag_layout(int nx, int ny, int pad) {
  FlagLayout L;
  L.stride = (nx - 2 * pad + kCols - 1) / kCols;
  L.xtiles = (nx + 1 - 2 * pad + kCols - 2) / (kCols - 1);
  L.vtiles = (nx + kCols - 1) / kCols;
  const long long rows = ny - 2 * pad;
  if (L.stride <= 0 || rows <= 0) return L;
  L.cons_tx = (nx - 2 * pad + kConsTile - 1) / kConsTile;
  L.cons_ty = (int)((rows + kConsTile - 1) / kConsTile);
  const long long bands = (rows + kRowsLag - 1) / kRowsLag;  // shock-heating tiles
  const long long sweep_bands = (rows + kRowsSweepStill - 1) / kRowsSweepStill;  // at most
  L.sk_words = ((size_t)sweep_bands * (L.xtiles > L.stride ? L.xtiles : L.stride) + 3) / 4;
  L.cfl = 0;
  L.cons = L.cfl + 2 * (size_t)bands * L.stride;
  L.q = L.cons + 4 * (size_t)L.cons_tx * L.cons_ty;
  L.fy = L.q + (size_t)rows * L.stride;
  L.fx = L.fy + (size_t)(rows + 1) * L.stride;
  L.v = L.fx + (size_t)rows * L.xtiles;
  L.marks = L.v + (size_t)ny * L.vtiles;
  const size_t words = L.marks + 2 * L.sk_words;
  L.fits = (size_t)kRaQFlags * sizeof(double) + words * sizeof(unsigned) <=
           (size_t)nx * ny * sizeof(double);
  return L;
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
  a.rows = kRowsLag;
  a.qmask = nullptr;
  a.qm_stride = 0;
  a.fxflag = nullptr;
  a.fyflag = nullptr;
  a.fx_stride = 0;
  a.vflag = nullptr;
  a.vf_stride = 0;
  a.skipf = nullptr;
  a.rest = nullptr;
  a.rest_w = a.rest_tiles_x = a.rest_rows = 0;
  a.cfl_tile = nullptr;
  a.moving = nullptr;
  const FlagLayout L = flag_layout(a.nx, a.ny, a.pad);
  if (L.fits) {
    unsigned* base = reinterpret_cast<unsigned*>(ra + kRaQFlags);
    a.cfl_tile = reinterpret_cast<unsigned long long*>(base + L.cfl);
    a.qmask = base + L.q;
    a.qm_stride = L.stride;
    a.fyflag = reinterpret_cast<unsigned char*>(base + L.fy);
    a.fxflag = reinterpret_cast<unsigned char*>(base + L.fx);
    a.fx_stride = 4 * L.xtiles;
    a.vflag = reinterpret_cast<unsigned char*>(base + L.v);
    a.vf_stride = 4 * L.vtiles;
    unsigned* marks = base + L.marks;
    a.skipf = reinterpret_cast<unsigned char*>(marks + (tt & 1) * L.sk_words);
    // The previous step's half, described; take_rest keeps it only when
    // that step was a flagged step on these arrays, and sets its tile height.
    a.rest = reinterpret_cast<unsigned char*>(marks + ((tt + 1) & 1) * L.sk_words);
    const bool prev_x_first = ((tt - 1) % 2 == 0);
    a.rest_w = prev_x_first ? kCols - 1 : kCols;
    a.rest_tiles_x = prev_x_first ? L.xtiles : L.stride;
    a.rest_rows = kRowsSweepMoving;
    a.moving = reinterpret_cast<unsigned long long*>(ra + kRaMoving);
  }
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

namespace {
// Output rows per CTA of the one-kernel Lagrangian phase.
int g_lag_rows = lagf::kDefaultRows;

// The last flagged step this thread ran, with what identifies its arrays: the
// step after it (and only that one) may take its tile marks (StepArgs::rest)
// and its per-tile CFL minima.
struct RestRecord {
  std::array<const void*, 12> arrays{};
  std::array<const void*, 4> mesh{};     // its spacing arrays
  const void* rho = nullptr;             // the state the step advanced
  const void* e = nullptr;
  const void* ra = nullptr;
  int nx = 0, ny = 0, pad = 0, form = -1, tt = 0;
  int sweep_rows = 0;                    // the step's sweep tile height
  unsigned long long tiles = 0;          // its first sweep's tiles
  unsigned long long moving = ~0ull;     // of which not skipped (read after the step)
  unsigned long long calls = 0;
  bool valid = false;
  bool follows = false;                  // it directly followed a flagged step
};
thread_local RestRecord t_rest;

// Keeps a.rest only when this step directly follows the recorded one on the
// same arrays (and no other mesh call came between), then records this step
// as the one the next may follow (when it runs with flags).  Returns this
// step's sweep tile height: the shorter where the previous step's first sweep
// skipped at least half of its tiles.
template <typename R>
int take_rest(StepArgs<R>& a, int tt, int form, const std::array<const void*, 12>& arrays,
              bool flagged, const void* rho, const void* e, const void* ra) {
  const unsigned long long calls = mesh_calls();
  const RestRecord& p = t_rest;
  const std::array<const void*, 4> mesh{a.edgedx, a.edgedy, a.celldx, a.celldy};
  const bool follows = p.valid && flagged && !a.first_step && p.tt + 1 == tt &&
                       p.calls + 1 == calls && p.form == form && p.nx == a.nx &&
                       p.ny == a.ny && p.pad == a.pad && p.arrays == arrays && p.mesh == mesh;
  if (follows) {
    a.rest_rows = p.sweep_rows;
  } else {
    a.rest = nullptr;
  }
  const bool still = follows && p.moving != ~0ull && 2 * p.moving <= p.tiles;
  const int rows = still ? kRowsSweepStill : kRowsSweepMoving;
  RestRecord r;
  r.arrays = arrays;
  r.mesh = mesh;
  r.rho = rho;
  r.e = e;
  r.ra = ra;
  r.nx = a.nx;
  r.ny = a.ny;
  r.pad = a.pad;
  r.form = form;
  r.tt = tt;
  r.sweep_rows = rows;
  const bool x_first = (tt % 2 == 0);
  const unsigned long long tiles_x =
      x_first ? (unsigned long long)(a.fx_stride / 4) : (unsigned long long)a.qm_stride;
  r.tiles = tiles_x * (unsigned long long)((a.ny - 2 * a.pad + rows - 1) / rows);
  r.calls = calls;
  r.valid = flagged;
  r.follows = follows;
  t_rest = r;
  return rows;
}
}  // namespace

// ---------------------------------------------------------------------------
// Conservation totals by tiles (the reference's print_conservation sums,
// omp3/flow.c:976-994): each kConsTile x kConsTile tile of interior cells
// keeps its partial sums (sum rho, sum rho e; each thread down its column, the
// warps and then the four warps of the block in a fixed order) in
// reduce_array, and the last block adds the partials of all tiles in a fixed
// order.  A tile whose cells all lay in tiles the last step's first sweep
// skipped -- at rest through that step, so unchanged since the previous call
// summed them -- keeps its partials without reading a cell.  The totals
// depend only on the cells (the same numbers whichever tiles were kept).
namespace {

struct ConsArgs {
  const double* rho;
  const double* e;
  double* ra;
  double* part;                // 2 doubles per tile: sum rho, sum rho e
  int nx, ny, pad, tiles_x, tiles;
  const unsigned char* marks;  // the last step's skip marks, or null
  int mark_w, mark_tiles_x, mark_rows;
};

__device__ __forceinline__ double block_sum_fixed(double x, double* s_w) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = x;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < kCols / 32; ++w) t += s_w[w];
  }
  __syncthreads();
  return t;  // (thread 0)
}

__global__ void __launch_bounds__(kCols) k_conservation_tiles(const ConsArgs c) {
  __shared__ double s_w[kCols / 32];
  __shared__ bool s_last;
  const int bx = blockIdx.x % c.tiles_x, by = blockIdx.x / c.tiles_x;
  const int pad = c.pad;
  const int c0 = pad + bx * kConsTile, r0 = pad + by * kConsTile;
  const int c1 = min(c0 + kConsTile, c.nx - pad), r1 = min(r0 + kConsTile, c.ny - pad);
  bool kept = false;
  if (c.marks) {
    const int b0 = (r0 - pad) / c.mark_rows, b1 = (r1 - 1 - pad) / c.mark_rows;
    const int x0 = (c0 - pad) / c.mark_w, x1 = (c1 - 1 - pad) / c.mark_w;
    const int nxb = x1 - x0 + 1, total = (b1 - b0 + 1) * nxb;
    bool ok = true;
    for (int q = threadIdx.x; q < total; q += blockDim.x) {
      ok = ok && c.marks[(size_t)(b0 + q / nxb) * c.mark_tiles_x + x0 + q % nxb] != 0;
    }
    kept = __syncthreads_and(ok) != 0;
  }
  if (!kept) {
    const int j = c0 + threadIdx.x;
    double ms = 0.0, es = 0.0;
    if (j < c1) {
      constexpr int kB = 8;
      for (int ib = r0; ib < r1; ib += kB) {
        double rv[kB], ev[kB];
#pragma unroll
        for (int q = 0; q < kB; ++q) {
          const bool in = ib + q < r1;
          const size_t k = (size_t)(in ? ib + q : r0) * c.nx + j;
          rv[q] = in ? c.rho[k] : 0.0;
          ev[q] = in ? c.e[k] : 0.0;
        }
#pragma unroll
        for (int q = 0; q < kB; ++q) {
          if (ib + q < r1) {
            ms = __dadd_rn(ms, rv[q]);
            es = __fma_rn(rv[q], ev[q], es);
          }
        }
      }
    }
    const double tm = block_sum_fixed(ms, s_w);
    const double te = block_sum_fixed(es, s_w);
    if (threadIdx.x == 0) {
      c.part[2 * (size_t)blockIdx.x] = tm;
      c.part[2 * (size_t)blockIdx.x + 1] = te;
    }
  }
  if (threadIdx.x == 0) {
    __threadfence();
    unsigned long long* ticket = reinterpret_cast<unsigned long long*>(c.ra + kRaTicket);
    s_last = (atomicAdd(ticket, 1ull) == (unsigned long long)gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double a = 0.0, b = 0.0;
  for (int k = threadIdx.x; k < c.tiles; k += blockDim.x) {
    a = __dadd_rn(a, __ldcg(c.part + 2 * (size_t)k));
    b = __dadd_rn(b, __ldcg(c.part + 2 * (size_t)k + 1));
  }
  const double ta = block_sum_fixed(a, s_w);
  const double tb = block_sum_fixed(b, s_w);
  if (threadIdx.x == 0) {
    c.ra[kRaMass] = ta;
    c.ra[kRaEnergy] = tb;
    *reinterpret_cast<unsigned long long*>(c.ra + kRaTicket) = 0ull;
  }
}

// The call the tile partials were last written by, and the mesh-call count
// then: the next call may keep tiles only when exactly one mesh call (the
// step's own) came between.
struct ConsRecord {
  const void* rho = nullptr;
  const void* e = nullptr;
  const void* ra = nullptr;
  int nx = 0, ny = 0, pad = 0;
  unsigned long long calls = 0;
  bool valid = false;
  bool after_step = false;  // right after a flagged step on this state ...
  int step_tt = 0;          // ... of this index
};
thread_local ConsRecord t_cons;

}  // namespace

bool tile_conservation(int nx, int ny, int pad, const double* rho, const double* e,
                       double* ra, cudaStream_t s) {
  const FlagLayout L = flag_layout(nx, ny, pad);
  if (!L.fits) return false;
  unsigned* base = reinterpret_cast<unsigned*>(ra + kRaQFlags);
  ConsArgs c{};
  c.rho = rho;
  c.e = e;
  c.ra = ra;
  c.part = reinterpret_cast<double*>(base + L.cons);
  c.nx = nx;
  c.ny = ny;
  c.pad = pad;
  c.tiles_x = L.cons_tx;
  c.tiles = L.cons_tx * L.cons_ty;
  c.marks = nullptr;
  const unsigned long long calls = mesh_calls();
  const RestRecord& p = t_rest;
  const ConsRecord& q = t_cons;
  // Right after a flagged step that advanced this state and directly
  // followed the step after which the partials were last written, on the same
  // arrays, with only that step's own mesh call in between: the state the
  // partials describe is the one that step started from.
  const bool after_step = p.valid && p.calls == calls && p.rho == rho && p.e == e &&
                          p.ra == ra && p.nx == nx && p.ny == ny && p.pad == pad;
  if (after_step && p.follows && q.valid && q.after_step && q.step_tt + 1 == p.tt &&
      q.calls + 1 == calls && q.rho == rho && q.e == e && q.ra == ra && q.nx == nx &&
      q.ny == ny && q.pad == pad) {
    const bool x_first = (p.tt % 2 == 0);
    c.marks = reinterpret_cast<const unsigned char*>(base + L.marks + (p.tt & 1) * L.sk_words);
    c.mark_w = x_first ? kCols - 1 : kCols;
    c.mark_tiles_x = x_first ? L.xtiles : L.stride;
    c.mark_rows = p.sweep_rows;
  }
  cudaMemsetAsync(ra + kRaTicket, 0, sizeof(double), s);
  k_conservation_tiles<<<(unsigned)c.tiles, kCols, 0, s>>>(c);
  count_launches(1);
  ConsRecord r;
  r.rho = rho;
  r.e = e;
  r.ra = ra;
  r.nx = nx;
  r.ny = ny;
  r.pad = pad;
  r.calls = calls;
  r.valid = cudaPeekAtLastError() == cudaSuccess;
  r.after_step = after_step;
  r.step_tt = p.tt;
  t_cons = r;
  return true;
}

int set_lagrangian_rows(int rows) {
  if (rows < 1 || rows > lagf::kMaxRows) {
    return record_error(GB300_ERR_ARG, "gb300_set_lagrangian_rows: %d not in 1 .. %d", rows,
                        lagf::kMaxRows);
  }
  g_lag_rows = rows;
  return GB300_OK;
}

int fused_solve(Mesh* mesh, int tt, double* P, double* rho, double* rho_old,
                double* e, double* u, double* v, double* rho_u, double* rho_v,
                double* Qxx, double* Qyy, double* F_x, double* F_y,
                double* uF_x, double* uF_y, double* vF_x, double* vF_y,
                double* reduce_array, bool one_kernel_lagrangian) {
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
  // The one-kernel Lagrangian phase when asked for and the arrays suit it: it
  // stages rows with 16-byte TMA copies and
  // keeps its change masks in rho_old (the reference's pre-advection density,
  // which the fused sweeps do not read).
  lagf::LagArgs lag{};
  const lagf::LagArgs* lagp = nullptr;
  if (one_kernel_lagrangian) {
    lag.nx = a.nx;
    lag.ny = a.ny;
    lag.pad = a.pad;
    lag.rows = g_lag_rows;
    lag.ntx = (a.nx - 2 * a.pad + 1 + lagf::kW - 1) / lagf::kW;
    const size_t mask_bytes = (size_t)(a.ny + 1) * lag.ntx * lagf::kMaskFields * lagf::kWarps * 4;
    auto al16 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; };
    if (al16(rho) && al16(e) && al16(rho_u) && al16(rho_v) && al16(rho_old) && a.pad == 2 &&
        mask_bytes <= (size_t)a.nx * a.ny * sizeof(double)) {
      lag.edgedx = a.edgedx; lag.edgedy = a.edgedy; lag.celldx = a.celldx; lag.celldy = a.celldy;
      lag.rho = rho; lag.e = e; lag.rho_u = rho_u; lag.rho_v = rho_v;
      lag.u = a.u; lag.v = a.v;
      // Scratch for the changed values: arrays the step writes only later
      // (P is not used by this form; F_x, F_y are the sweeps' outputs).
      lag.e_new = P; lag.rho_u_new = F_x; lag.rho_v_new = F_y;
      lag.masks = reinterpret_cast<unsigned*>(rho_old);
      lag.ra = reduce_array;
      lag.min_slot = a.min_slot;
      lag.mesh_pow2 = a.mesh_pow2;
      lag.dt_slot = a.dt_slot;
      lag.dt = a.dt; lag.dt_h = a.dt_h; lag.max_dt = a.max_dt;
      lag.first_step = a.first_step;
      lagp = &lag;
    }
  }
  const int sweep_rows =
      take_rest(a, tt, 0, {P, rho, e, rho_u, rho_v, uF_y, vF_x, uF_x, vF_y, F_x, F_y, reduce_array},
                a.skipf != nullptr && lagp == nullptr, rho, e, reduce_array);
  StepProfiler prof;
  prof.begin(s);
  launch_step(s, a, tt, first, second, prof, sweep_rows, a.rest != nullptr, lagp);
  unsigned long long moving = ~0ull;
  const int st = finish_step(s, mesh, reduce_array, prof, "solve_hydro_2d (fused)", &moving);
  if (st != GB300_OK) t_rest.valid = false;
  t_rest.moving = moving;
  return st;
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
  const int sweep_rows =
      take_rest(a, tt, 1, {rho, e, rho_u, rho_v, work, reduce_array, nullptr, nullptr, nullptr,
                           nullptr, nullptr, nullptr},
                a.skipf != nullptr, rho, e, reduce_array);
  StepProfiler prof;
  prof.begin(s);
  launch_step(s, a, tt, first, second, prof, sweep_rows, a.rest != nullptr);
  unsigned long long moving = ~0ull;
  const int st = finish_step(s, mesh, reduce_array, prof, "gb300_mixed_solve", &moving);
  if (st != GB300_OK) t_rest.valid = false;
  t_rest.moving = moving;
  return st;
}

}  // namespace flow
