// batched.cu -- many independent flow problems of uneven sizes, each with its
// own dt, advanced together: one persistent cooperative launch per timestep
// runs every phase of the step over a flattened list of (instance, tile)
// work items, separated by grid-wide barriers, and the launches of a pair of
// steps (even + odd, whose sweep orders differ) are captured as a CUDA graph.
//
// Per instance the arrays are those of the single-problem fused step
// (fused_tiles.cuh), carved out of one caller-provided device pool; the
// instance's reduce region holds its dt/dt_h pair and CFL minimum, so no
// instance waits for another's timestep.
//
// Grid barriers spin with a bounded iteration count: on timeout the kernel
// records GB300_ERR_TIMEOUT in the batch status word and every block leaves
// at the next barrier, so a failed launch cannot hang the device.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>

#include "../../include/flow_gb300.h"
#include "fused.h"
#include "fused_tiles.cuh"
#include "init.h"
#include "stages.h"

namespace flow {
namespace {

using namespace tiles;

constexpr int kRaRegion = 2304;     // doubles of reduce scratch per instance
constexpr int kRaMinSlot = 6;       // same slot as the single-problem step
constexpr int kMaxInstances = 4096;
constexpr long long kSpinLimit = 1ll << 25;  // ~2 s of 64 ns naps

// Grid shapes of the phases (tiles per instance differ per shape).
enum Shape : int {
  kShCells = 0,     // every cell: pressure
  kShInterior = 1,  // interior cells: viscosity, energy, y sweep, uF_x, vF_y
  kShFaces = 2,     // interior faces and corners: viscous accel, uF_y, vF_x
  kShSweepX = 3,    // x sweep (127 new columns per tile)
  kShFaceU = 4,     // x-faces: momentum y pair for rho_u
  kShFaceV = 5,     // y-faces: momentum y pair for rho_v
  kShMomXV = 6,     // y-faces, 127 per tile: momentum x pair for rho_v
  kNumShapes = 7
};

enum Phase : int {
  kPhPressure, kPhViscosity, kPhAccel, kPhEnergy,
  kPhSweepX1, kPhSweepY1, kPhSweepX2, kPhSweepY2,
  // Momentum pairs (flux fused with its update); V: the pair recomputes the
  // velocity.
  kPhMomUxV, kPhMomUx, kPhMomUyV, kPhMomUy, kPhMomVxV, kPhMomVx, kPhMomVyV, kPhMomVy,
};

template <typename R>
struct Instance {
  StepArgs<R> a;
  SweepArgs<R> first;
  SweepArgs<R> second;
};

struct Status {
  unsigned counter;
  unsigned generation;
  int error;
  int pad;
};

template <typename R>
struct BatchDev {
  const Instance<R>* inst;
  const int* tiles_x;   // [kNumShapes][n]
  const int* prefix;    // [kNumShapes][n+1]
  Status* status;
  int n;
  long long spin_limit;  // naps a barrier waits before it reports a timeout
};

__device__ __forceinline__ int shape_of(int ph) {
  switch (ph) {
    case kPhPressure: return kShCells;
    case kPhAccel: return kShFaces;
    // x pair for rho_u: x-faces pad .. nx-pad, 127 per tile, as the x sweep.
    case kPhSweepX1: case kPhSweepX2: case kPhMomUxV: case kPhMomUx: return kShSweepX;
    case kPhMomUyV: case kPhMomUy: return kShFaceU;
    case kPhMomVyV: case kPhMomVy: return kShFaceV;
    case kPhMomVxV: case kPhMomVx: return kShMomXV;
    default: return kShInterior;
  }
}

// The momentum pairs' tiles are called functions, compiled with their own
// register allocation: inlined into the one kernel with every other phase,
// they made the register allocator spill several KB per thread.  (The other
// phases stay inlined: through the call's generic pointer to the shared
// instance, their tiles ran slower.)  A call per tile costs nothing per cell.
template <typename R, int kPh>
__device__ __noinline__ void tile_call(const Instance<R>& __restrict__ I, int tx, int ty) {
  switch (kPh) {
    case kPhMomUxV: tile_mom_x<R, false, true, false>(I.a, tx, ty); break;
    case kPhMomUx: tile_mom_x<R, false, false, false>(I.a, tx, ty); break;
    case kPhMomUyV: tile_mom_y<R, false, true, false>(I.a, tx, ty); break;
    case kPhMomUy: tile_mom_y<R, false, false, false>(I.a, tx, ty); break;
    case kPhMomVxV: tile_mom_x<R, true, true, false>(I.a, tx, ty); break;
    case kPhMomVx: tile_mom_x<R, true, false, false>(I.a, tx, ty); break;
    case kPhMomVyV: tile_mom_y<R, true, true, false>(I.a, tx, ty); break;
    default: tile_mom_y<R, true, false, false>(I.a, tx, ty); break;
  }
}

template <typename R>
__device__ __forceinline__ void run_tile(int ph, const Instance<R>& I, int tx, int ty) {
  switch (ph) {
    case kPhPressure: tile_lag_pressure(I.a, tx, ty); break;
    case kPhViscosity: tile_lag_viscosity(I.a, tx, ty); break;
    case kPhAccel: tile_lag_viscous_accel<R, false>(I.a, tx, ty); break;
    case kPhEnergy: tile_lag_energy_dt<R, false>(I.a, tx, ty); break;
    case kPhSweepX1: tile_mass_sweep_x<R, true, false>(I.a, I.first, tx, ty); break;
    case kPhSweepY1: tile_mass_sweep_y<R, true, false>(I.a, I.first, tx, ty); break;
    case kPhSweepX2: tile_mass_sweep_x<R, false, false>(I.a, I.second, tx, ty); break;
    case kPhSweepY2: tile_mass_sweep_y<R, false, false>(I.a, I.second, tx, ty); break;
    case kPhMomUxV: tile_call<R, kPhMomUxV>(I, tx, ty); break;
    case kPhMomUx: tile_call<R, kPhMomUx>(I, tx, ty); break;
    case kPhMomUyV: tile_call<R, kPhMomUyV>(I, tx, ty); break;
    case kPhMomUy: tile_call<R, kPhMomUy>(I, tx, ty); break;
    case kPhMomVxV: tile_call<R, kPhMomVxV>(I, tx, ty); break;
    case kPhMomVx: tile_call<R, kPhMomVx>(I, tx, ty); break;
    case kPhMomVyV: tile_call<R, kPhMomVyV>(I, tx, ty); break;
    default: tile_call<R, kPhMomVy>(I, tx, ty); break;
  }
}

// Grid-wide barrier with a bounded wait of spin_limit 64 ns naps.  Returns
// false (for every block) once any block has timed out, so that all blocks
// leave the kernel: a waiting block also leaves as soon as another block has
// recorded a timeout.
__device__ bool grid_sync(Status* st, long long spin_limit) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* gen = &st->generation;
    const unsigned g = *gen;
    __threadfence();
    const unsigned arrived = atomicAdd(&st->counter, 1u) + 1u;
    if (arrived == gridDim.x) {
      st->counter = 0u;
      __threadfence();
      atomicAdd(&st->generation, 1u);
    } else {
      long long spins = 0;
      volatile int* err = &st->error;
      while (*gen == g && *err == 0) {
        if (++spins > spin_limit) {
          atomicExch(&st->error, GB300_ERR_TIMEOUT);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    s_ok = (*(volatile int*)&st->error) == 0;
  }
  __syncthreads();
  return s_ok != 0;
}

// Phase list of one step: the reference order (omp3/flow.c:22-51), with the
// sweep order and the momentum order set by the step parity.
__host__ __device__ __forceinline__ int phase_list(int tt, int* ph) {
  int n = 0;
  ph[n++] = kPhPressure;
  ph[n++] = kPhViscosity;
  ph[n++] = kPhAccel;
  ph[n++] = kPhEnergy;
  const bool x_first = (tt % 2 == 0);
  ph[n++] = x_first ? kPhSweepX1 : kPhSweepY1;
  ph[n++] = x_first ? kPhSweepY2 : kPhSweepX2;
  if (tt % 2) {
    ph[n++] = kPhMomUxV; ph[n++] = kPhMomUy; ph[n++] = kPhMomVxV; ph[n++] = kPhMomVy;
  } else {
    ph[n++] = kPhMomUyV; ph[n++] = kPhMomUx; ph[n++] = kPhMomVyV; ph[n++] = kPhMomVx;
  }
  return n;
}

// Resident CTAs per SM the register budget is sized for: the mixed form is
// bound by latency and keeps 8 (64 registers); the FP64 form by its FP64 pipe,
// and 5 (up to 102 registers) leaves it without spills.
template <typename R>
constexpr int kBatchMinCtas = Prec<R>::kMixed ? 8 : 5;

template <typename R>
__global__ void __launch_bounds__(kCols, kBatchMinCtas<R>) k_batch_step(const BatchDev<R> b,
                                                                         int tt, int first_step) {
  __shared__ Instance<R> s_inst;
  __shared__ int s_cur;
  int ph[20];
  const int nph = phase_list(tt, ph);
  if (threadIdx.x == 0) s_cur = -1;
  for (int p = 0; p < nph; ++p) {
    const int shape = shape_of(ph[p]);
    const int* pre = b.prefix + shape * (b.n + 1);
    const int* tx_n = b.tiles_x + shape * b.n;
    const int total = pre[b.n];
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
      // Instance of work item w: the last prefix entry <= w.
      int lo = 0, hi = b.n - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pre[mid] <= w) lo = mid; else hi = mid - 1;
      }
      const int i = lo;
      const int local = w - pre[i];
      if (threadIdx.x == 0 && s_cur != i) {
        s_inst = b.inst[i];
        s_cur = i;
      }
      if (threadIdx.x == 0) {
        // The Lagrangian phases run on the pair the previous step left.
        s_inst.a.dt = s_inst.a.dt_slot[0];
        s_inst.a.dt_h = s_inst.a.dt_slot[1];
        s_inst.a.first_step = first_step;
      }
      __syncthreads();
      run_tile(ph[p], s_inst, local % tx_n[i], local / tx_n[i]);
      __syncthreads();
    }
    if (!grid_sync(b.status, b.spin_limit)) return;
    if (ph[p] == kPhEnergy) {
      // Every tile of every instance has added its CFL candidate: apply the
      // dt rule per instance.
      for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < b.n;
           i += gridDim.x * blockDim.x) {
        StepArgs<R> a = b.inst[i].a;
        a.dt = a.dt_slot[0];
        a.dt_h = a.dt_slot[1];
        a.first_step = first_step;
        finish_dt(a);
      }
      if (!grid_sync(b.status, b.spin_limit)) return;
      if (threadIdx.x == 0) s_cur = -1;  // reload dt into the cached instance
    }
  }
}

// ---------------------------------------------------------------------------
// Phase launches (the "phases" schedule): one kernel per phase over the work
// items of every instance.  The kernel boundaries order the phases instead of
// grid barriers, so each phase is compiled on its own, with the register
// budget and asynchronous-copy rings of the single-problem kernel of that
// phase (fused.cu) -- the persistent kernel holds every phase, and its
// registers are the maximum over them.  Launches are chained with
// programmatic dependent launch and captured, two steps at a time, in a CUDA
// graph like the persistent launches.

__device__ __forceinline__ void batch_pdl_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}
__device__ __forceinline__ void batch_pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" :::);
}

template <int kPh>
__host__ __device__ constexpr int phase_shape() {
  return kPh == kPhPressure ? kShCells
       : kPh == kPhAccel ? kShFaces
       : (kPh == kPhSweepX1 || kPh == kPhSweepX2 || kPh == kPhMomUxV || kPh == kPhMomUx)
           ? kShSweepX
       : (kPh == kPhMomUyV || kPh == kPhMomUy) ? kShFaceU
       : (kPh == kPhMomVyV || kPh == kPhMomVy) ? kShFaceV
       : (kPh == kPhMomVxV || kPh == kPhMomVx) ? kShMomXV
       : kShInterior;
}

// The tile function of one phase, in the form the single-problem kernels use
// (copy rings and early first loads on).
template <typename R, int kPh>
__device__ __forceinline__ void phase_tile(const Instance<R>& I, int tx, int ty) {
  if constexpr (kPh == kPhPressure) tile_lag_pressure(I.a, tx, ty);
  else if constexpr (kPh == kPhViscosity) tile_lag_viscosity(I.a, tx, ty);
  else if constexpr (kPh == kPhAccel) tile_lag_viscous_accel<R, true>(I.a, tx, ty);
  else if constexpr (kPh == kPhEnergy) tile_lag_energy_dt<R, true>(I.a, tx, ty);
  else if constexpr (kPh == kPhSweepX1) tile_mass_sweep_x<R, true, true>(I.a, I.first, tx, ty);
  else if constexpr (kPh == kPhSweepY1) tile_mass_sweep_y<R, true, true>(I.a, I.first, tx, ty);
  else if constexpr (kPh == kPhSweepX2) tile_mass_sweep_x<R, false, true>(I.a, I.second, tx, ty);
  else if constexpr (kPh == kPhSweepY2) tile_mass_sweep_y<R, false, true>(I.a, I.second, tx, ty);
  else if constexpr (kPh == kPhMomUxV) tile_mom_x<R, false, true, true>(I.a, tx, ty);
  else if constexpr (kPh == kPhMomUx) tile_mom_x<R, false, false, true>(I.a, tx, ty);
  else if constexpr (kPh == kPhMomUyV) tile_mom_y<R, false, true, true>(I.a, tx, ty);
  else if constexpr (kPh == kPhMomUy) tile_mom_y<R, false, false, true>(I.a, tx, ty);
  else if constexpr (kPh == kPhMomVxV) tile_mom_x<R, true, true, true>(I.a, tx, ty);
  else if constexpr (kPh == kPhMomVx) tile_mom_x<R, true, false, true>(I.a, tx, ty);
  else if constexpr (kPh == kPhMomVyV) tile_mom_y<R, true, true, true>(I.a, tx, ty);
  else tile_mom_y<R, true, false, true>(I.a, tx, ty);
}

// Resident CTAs per SM of each phase kernel: those of the single-problem
// kernels (fused.cu), which only the sweeps set -- one fewer for the y sweeps,
// whose tile spills at the single-problem budget once the instance lookup
// takes its registers (60-70 bytes per thread, measured with -Xptxas -v).
template <typename R, int kPh>
__host__ __device__ constexpr int phase_min_ctas() {
  return (kPh == kPhSweepX1 || kPh == kPhSweepX2) ? (Prec<R>::kMixed ? 8 : 7)
       : (kPh == kPhSweepY1 || kPh == kPhSweepY2) ? (Prec<R>::kMixed ? 6 : 5)
       : 1;
}

template <typename R, int kPh>
__global__ void __launch_bounds__(kCols, (phase_min_ctas<R, kPh>()))
    k_batch_phase(const BatchDev<R> b, int first_step) {
  // One work item per CTA (the grid is the phase's item count).
  __shared__ Instance<R> s_inst;
  batch_pdl_wait();
  batch_pdl_trigger();
  constexpr int shape = phase_shape<kPh>();
  const int* pre = b.prefix + shape * (b.n + 1);
  const int w = blockIdx.x;
  // Instance of work item w: the last prefix entry <= w.
  int lo = 0, hi = b.n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (pre[mid] <= w) lo = mid; else hi = mid - 1;
  }
  const int i = lo;
  const int local = w - pre[i];
  const int tx = b.tiles_x[shape * b.n + i];
  // The instance's arguments, copied into shared memory by the whole block,
  // with the dt pair the previous step left (Lagrangian phases).
  static_assert(sizeof(Instance<R>) % 8 == 0, "8-byte words");
  const unsigned long long* src = reinterpret_cast<const unsigned long long*>(b.inst + i);
  unsigned long long* dst = reinterpret_cast<unsigned long long*>(&s_inst);
  for (int k = threadIdx.x; k < (int)(sizeof(Instance<R>) / 8); k += blockDim.x) dst[k] = src[k];
  __syncthreads();
  if (threadIdx.x == 0) {
    s_inst.a.dt = s_inst.a.dt_slot[0];
    s_inst.a.dt_h = s_inst.a.dt_slot[1];
    s_inst.a.first_step = first_step;
  }
  __syncthreads();
  phase_tile<R, kPh>(s_inst, local % tx, local / tx);
}

// After the energy phase: the dt rule per instance (omp3/flow.c:103-105).
template <typename R>
__global__ void k_batch_finish_dt(const BatchDev<R> b, int first_step) {
  batch_pdl_wait();
  batch_pdl_trigger();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < b.n; i += gridDim.x * blockDim.x) {
    StepArgs<R> a = b.inst[i].a;
    a.dt = a.dt_slot[0];
    a.dt_h = a.dt_slot[1];
    a.first_step = first_step;
    finish_dt(a);
  }
}

// Whether every spacing of an instance's mesh is a positive normal power of
// two, one block per instance, into the flag its tiles read (mesh_pow2).
template <typename R>
__global__ void __launch_bounds__(256) k_batch_mesh_pow2(const BatchDev<R> b) {
  const StepArgs<R>& a = b.inst[blockIdx.x].a;
  bool ok = true;
  for (int j = threadIdx.x; j <= a.nx; j += blockDim.x) {
    ok = ok && d_is_pow2(a.celldx[j]) && d_is_pow2(a.edgedx[j]);
  }
  for (int j = threadIdx.x; j <= a.ny; j += blockDim.x) {
    ok = ok && d_is_pow2(a.celldy[j]) && d_is_pow2(a.edgedy[j]);
  }
  ok = __syncthreads_and(ok) != 0;
  if (threadIdx.x == 0) *const_cast<unsigned long long*>(a.mesh_pow2) = ok ? 1ull : 0ull;
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side.

struct BatchImpl {
  int n = 0;
  int precision = 0;  // 0 FP64, 1 mixed
  std::vector<int> gnx, gny;
  std::vector<double> width, height;
  std::vector<size_t> off;  // per-instance byte offset in the pool
  size_t bytes = 0;
  char* pool = nullptr;
  // device tables
  int* d_tiles_x = nullptr;
  int* d_prefix = nullptr;
  Status* d_status = nullptr;
  void* d_inst = nullptr;
  size_t tables_off = 0;
  int rows = kDefaultRows;
  int ctas_per_sm = 0;  // 0 = as many as fit
  int order = 0;        // 0 largest first, 1 input order
  int grid = 0;
  int tt = 0;
  int schedule = GB300_BATCH_PHASES;  // phase launches, or one persistent launch
  std::vector<int> shape_total;       // work items per grid shape
  long long spin_limit = kSpinLimit;
  cudaGraphExec_t graph = nullptr;
  int graph_tt_parity = -1;
  std::vector<int> perm;  // instance order in the work list
};

namespace {

struct InstLayout {
  size_t rho, e, rho_u, rho_v, P, rho_old, u, v, Qxx, Qyy, F_x, F_y, uF_x, uF_y,
      vF_x, vF_y, rho_r, e_r, s_r, s_e, s_r32, s_e32, mesh, ra, total;
};

InstLayout inst_layout(int nx, int ny, int precision) {
  const size_t nc = (size_t)nx * ny, nf = (size_t)(nx + 1) * (ny + 1);
  const size_t rb = precision ? 4 : 8;  // bulk precision bytes
  InstLayout L{};
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o += (bytes + 255) / 256 * 256;
    return at;
  };
  L.rho = take(nc * 8);
  L.e = take(nc * 8);
  L.rho_u = take(nf * rb);
  L.rho_v = take(nf * rb);
  L.u = take(nf * rb);
  L.v = take(nf * rb);
  L.Qxx = take(nc * rb);
  L.Qyy = take(nc * rb);
  L.F_x = take(nf * rb);
  L.F_y = take(nf * rb);
  L.uF_x = take(nf * 8);  // also the FP64 first-sweep density
  L.uF_y = take(nf * rb);
  L.vF_x = take(nf * rb);
  L.vF_y = take(nf * 8);  // also the FP64 first-sweep energy
  if (precision == 0) {
    L.P = take(nc * 8);
  } else {
    L.rho_r = take(nc * 4);
    L.e_r = take(nc * 4);
    L.s_r = take(nc * 8);
    L.s_e = take(nc * 8);
    L.s_r32 = take(nc * 4);
    L.s_e32 = take(nc * 4);
  }
  L.mesh = take(6 * (size_t)(std::max(nx, ny) + 1) * 8);
  L.ra = take(kRaRegion * 8);
  L.total = o;
  return L;
}

int tiles_for(int shape, int nx, int ny, int rows, int* tx) {
  int cols = 0, nrows = 0, per = kCols;
  switch (shape) {
    case kShCells: cols = nx; nrows = ny; break;
    case kShInterior: cols = nx - 4; nrows = ny - 4; break;
    case kShFaces: cols = nx - 3; nrows = ny - 3; break;
    case kShSweepX: cols = nx - 3; nrows = ny - 4; per = kCols - 1; break;
    case kShFaceU: cols = nx - 3; nrows = ny - 4; break;
    case kShMomXV: cols = nx - 4; nrows = ny - 3; per = kCols - 1; break;
    default: cols = nx - 4; nrows = ny - 3; break;
  }
  *tx = (cols + per - 1) / per;
  return *tx * ((nrows + rows - 1) / rows);
}

template <typename R>
Instance<R> make_instance(const BatchImpl& B, int i) {
  const int nx = B.gnx[i] + 4, ny = B.gny[i] + 4;
  const InstLayout L = inst_layout(nx, ny, B.precision);
  char* base = B.pool + B.off[i];
  auto D = [&](size_t o) { return reinterpret_cast<double*>(base + o); };
  auto Rp = [&](size_t o) { return reinterpret_cast<R*>(base + o); };
  const size_t m = (size_t)std::max(nx, ny) + 1;
  Instance<R> I{};
  StepArgs<R>& a = I.a;
  a.nx = nx; a.ny = ny; a.pad = 2;
  a.edgedx = D(L.mesh); a.edgedy = D(L.mesh) + m; a.celldx = D(L.mesh) + 2 * m;
  a.celldy = D(L.mesh) + 3 * m;
  a.rho = D(L.rho); a.e = D(L.e);
  a.rho_u = Rp(L.rho_u); a.rho_v = Rp(L.rho_v); a.u = Rp(L.uF_y); a.v = Rp(L.vF_x);
  a.u_out = Rp(L.u); a.v_out = Rp(L.v);  // the Lagrangian velocities live in uF_y/vF_x
  a.Qxx = Rp(L.Qxx); a.Qyy = Rp(L.Qyy); a.F_x = Rp(L.F_x); a.F_y = Rp(L.F_y);
  a.uF_x = Rp(L.uF_x); a.uF_y = Rp(L.uF_y); a.vF_x = Rp(L.vF_x); a.vF_y = Rp(L.vF_y);
  a.ra = D(L.ra);
  a.min_slot = reinterpret_cast<unsigned long long*>(D(L.ra) + kRaMinSlot);
  a.mesh_pow2 = reinterpret_cast<const unsigned long long*>(D(L.ra) + kRaMeshPow2);
  a.dt_slot = D(L.ra) + kRaDt;
  a.max_dt = 10.0;
  a.rows = B.rows;
  if (B.precision == 0) {
    a.rho_r = reinterpret_cast<R*>(a.rho);
    a.e_r = reinterpret_cast<R*>(a.e);
    a.P = D(L.P);
    a.rho_old = nullptr;
    I.first = SweepArgs<R>{a.rho, a.e, a.rho_r, a.e_r, D(L.uF_x), D(L.vF_y),
                           Rp(L.uF_x), Rp(L.vF_y)};
    I.second = SweepArgs<R>{D(L.uF_x), D(L.vF_y), Rp(L.uF_x), Rp(L.vF_y), a.rho,
                            a.e, a.rho_r, a.e_r};
  } else {
    a.rho_r = Rp(L.rho_r);
    a.e_r = Rp(L.e_r);
    a.P = nullptr;
    a.rho_old = nullptr;
    I.first = SweepArgs<R>{a.rho, a.e, a.rho_r, a.e_r, D(L.s_r), D(L.s_e),
                           Rp(L.s_r32), Rp(L.s_e32)};
    I.second = SweepArgs<R>{D(L.s_r), D(L.s_e), Rp(L.s_r32), Rp(L.s_e32), a.rho,
                            a.e, a.rho_r, a.e_r};
  }
  return I;
}

template <typename R>
int upload_tables(BatchImpl& B) {
  const int n = B.n;
  std::vector<int> tx(kNumShapes * n), pre(kNumShapes * (n + 1));
  for (int s = 0; s < kNumShapes; ++s) {
    pre[s * (n + 1)] = 0;
    for (int k = 0; k < n; ++k) {
      const int i = B.perm[k];
      int t = 0;
      const int cnt = tiles_for(s, B.gnx[i] + 4, B.gny[i] + 4, B.rows, &t);
      tx[s * n + k] = t;
      pre[s * (n + 1) + k + 1] = pre[s * (n + 1) + k] + cnt;
    }
  }
  B.shape_total.assign(kNumShapes, 0);
  for (int s = 0; s < kNumShapes; ++s) B.shape_total[s] = pre[s * (n + 1) + n];
  std::vector<Instance<R>> inst(n);
  for (int k = 0; k < n; ++k) inst[k] = make_instance<R>(B, B.perm[k]);
  cudaMemcpy(B.d_tiles_x, tx.data(), tx.size() * sizeof(int), cudaMemcpyHostToDevice);
  cudaMemcpy(B.d_prefix, pre.data(), pre.size() * sizeof(int), cudaMemcpyHostToDevice);
  cudaMemcpy(B.d_inst, inst.data(), inst.size() * sizeof(Instance<R>), cudaMemcpyHostToDevice);
  cudaMemset(B.d_status, 0, sizeof(Status));
  return check_launch("gb300_batch: table upload");
}

// Launches kernel k with programmatic stream serialisation: it may start as
// soon as its predecessor's CTAs have all started, and waits on the device
// (griddepcontrol.wait) for its predecessor's writes.
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*k)(KArgs...), unsigned grid, unsigned block, cudaStream_t s,
                       Args... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, args...);
}

template <typename R>
BatchDev<R> batch_dev(const BatchImpl& B) {
  return BatchDev<R>{static_cast<const Instance<R>*>(B.d_inst), B.d_tiles_x, B.d_prefix,
                     B.d_status, B.n, B.spin_limit};
}

template <typename R, int kPh>
cudaError_t launch_phase_k(const BatchImpl& B, const BatchDev<R>& b, int first, cudaStream_t s) {
  const int items = B.shape_total[phase_shape<kPh>()];
  if (items <= 0) return cudaSuccess;
  count_launches(1);
  return launch_pdl(k_batch_phase<R, kPh>, (unsigned)items, (unsigned)kCols, s, b, first);
}

template <typename R>
cudaError_t launch_phase(const BatchImpl& B, const BatchDev<R>& b, int ph, int first,
                         cudaStream_t s) {
  switch (ph) {
    case kPhPressure: return launch_phase_k<R, kPhPressure>(B, b, first, s);
    case kPhViscosity: return launch_phase_k<R, kPhViscosity>(B, b, first, s);
    case kPhAccel: return launch_phase_k<R, kPhAccel>(B, b, first, s);
    case kPhEnergy: return launch_phase_k<R, kPhEnergy>(B, b, first, s);
    case kPhSweepX1: return launch_phase_k<R, kPhSweepX1>(B, b, first, s);
    case kPhSweepY1: return launch_phase_k<R, kPhSweepY1>(B, b, first, s);
    case kPhSweepX2: return launch_phase_k<R, kPhSweepX2>(B, b, first, s);
    case kPhSweepY2: return launch_phase_k<R, kPhSweepY2>(B, b, first, s);
    case kPhMomUxV: return launch_phase_k<R, kPhMomUxV>(B, b, first, s);
    case kPhMomUx: return launch_phase_k<R, kPhMomUx>(B, b, first, s);
    case kPhMomUyV: return launch_phase_k<R, kPhMomUyV>(B, b, first, s);
    case kPhMomUy: return launch_phase_k<R, kPhMomUy>(B, b, first, s);
    case kPhMomVxV: return launch_phase_k<R, kPhMomVxV>(B, b, first, s);
    case kPhMomVx: return launch_phase_k<R, kPhMomVx>(B, b, first, s);
    case kPhMomVyV: return launch_phase_k<R, kPhMomVyV>(B, b, first, s);
    default: return launch_phase_k<R, kPhMomVy>(B, b, first, s);
  }
}

// One step as phase launches: the step's phases in the reference order, the
// per-instance dt rule after the energy phase.
template <typename R>
int launch_batch_phases(BatchImpl& B, cudaStream_t s, int tt) {
  const BatchDev<R> b = batch_dev<R>(B);
  const int first = (tt == 0) ? 1 : 0;
  int ph[20];
  const int nph = phase_list(tt, ph);
  for (int p = 0; p < nph; ++p) {
    cudaError_t err = launch_phase<R>(B, b, ph[p], first, s);
    if (err == cudaSuccess && ph[p] == kPhEnergy) {
      count_launches(1);
      err = launch_pdl(k_batch_finish_dt<R>, (unsigned)((B.n + 127) / 128), 128u, s, b, first);
    }
    if (err != cudaSuccess) {
      return record_error(GB300_ERR_CUDA, "gb300_batch_step: %s", cudaGetErrorString(err));
    }
  }
  return GB300_OK;
}

// The per-instance mesh test, once per gb300_batch_step call (the meshes do
// not change during the steps of a call).
template <typename R>
int launch_batch_mesh_test(BatchImpl& B, cudaStream_t s) {
  k_batch_mesh_pow2<R><<<(unsigned)B.n, 256, 0, s>>>(batch_dev<R>(B));
  count_launches(1);
  return check_launch("gb300_batch_step: mesh test");
}

template <typename R>
int launch_batch_step(BatchImpl& B, cudaStream_t s, int tt) {
  if (B.schedule == GB300_BATCH_PHASES) return launch_batch_phases<R>(B, s, tt);
  BatchDev<R> b = batch_dev<R>(B);
  int first = (tt == 0) ? 1 : 0;
  void* args[] = {&b, &tt, &first};
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(B.grid);
  cfg.blockDim = dim3(kCols);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const cudaError_t err = cudaLaunchKernelExC(&cfg, (const void*)k_batch_step<R>, args);
  count_launches(1);
  if (err != cudaSuccess) {
    return record_error(GB300_ERR_CUDA, "gb300_batch_step: %s", cudaGetErrorString(err));
  }
  return GB300_OK;
}

template <typename R>
int choose_grid(BatchImpl& B) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_step<R>, kCols, 0);
  if (per_sm <= 0) return record_error(GB300_ERR_CUDA, "gb300_batch: kernel does not fit an SM");
  const int use = (B.ctas_per_sm > 0) ? std::min(B.ctas_per_sm, per_sm) : per_sm;
  B.grid = sms * use;
  return GB300_OK;
}

int retune(BatchImpl& B) {
  B.perm.resize(B.n);
  std::iota(B.perm.begin(), B.perm.end(), 0);
  if (B.order == 0) {
    std::stable_sort(B.perm.begin(), B.perm.end(), [&](int x, int y) {
      return (long long)B.gnx[x] * B.gny[x] > (long long)B.gnx[y] * B.gny[y];
    });
  }
  if (B.graph) {
    cudaGraphExecDestroy(B.graph);
    B.graph = nullptr;
  }
  if (B.precision == 0) {
    int st = upload_tables<double>(B);
    return st != GB300_OK ? st : choose_grid<double>(B);
  }
  int st = upload_tables<float>(B);
  return st != GB300_OK ? st : choose_grid<float>(B);
}

__global__ void k_fill(double* a, size_t n, double v) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    a[i] = v;
  }
}

__global__ void k_shadow(size_t n, const double* a, float* ar) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    ar[i] = f64_to_f32(a[i]);
  }
}

}  // namespace
}  // namespace flow

using flow::BatchImpl;

struct GB300Batch {
  BatchImpl impl;
};

extern "C" {

int gb300_batch_create(int n, const int* global_nx, const int* global_ny,
                       const double* width, const double* height, int precision,
                       GB300Batch** out) {
  using namespace flow;
  if (!out || n <= 0 || n > kMaxInstances || !global_nx || !global_ny ||
      (precision != 0 && precision != 1)) {
    return record_error(GB300_ERR_ARG, "gb300_batch_create: bad arguments");
  }
  for (int i = 0; i < n; ++i) {
    if (global_nx[i] < 2 || global_ny[i] < 2) {
      return record_error(GB300_ERR_ARG, "gb300_batch_create: instance %d smaller than 2x2", i);
    }
  }
  auto* b = new GB300Batch();
  BatchImpl& B = b->impl;
  B.n = n;
  B.precision = precision;
  B.gnx.assign(global_nx, global_nx + n);
  B.gny.assign(global_ny, global_ny + n);
  B.width.assign(n, 1.0);
  B.height.assign(n, 1.0);
  if (width) B.width.assign(width, width + n);
  if (height) B.height.assign(height, height + n);
  size_t o = 0;
  B.off.resize(n);
  for (int i = 0; i < n; ++i) {
    B.off[i] = o;
    o += inst_layout(B.gnx[i] + 4, B.gny[i] + 4, precision).total;
  }
  B.tables_off = o;
  o += (size_t)kNumShapes * n * sizeof(int) + (size_t)kNumShapes * (n + 1) * sizeof(int) + 256;
  o = (o + 255) / 256 * 256;
  o += sizeof(Status) + 256;
  o += (size_t)n * (precision ? sizeof(Instance<float>) : sizeof(Instance<double>)) + 256;
  B.bytes = o;
  *out = b;
  return GB300_OK;
}

size_t gb300_batch_pool_bytes(const GB300Batch* b) { return b ? b->impl.bytes : 0; }

int gb300_batch_bind(GB300Batch* b, void* pool, size_t bytes) {
  using namespace flow;
  if (!b || !pool || bytes < b->impl.bytes) {
    return record_error(GB300_ERR_ARG, "gb300_batch_bind: pool of %zu bytes, need %zu", bytes,
                        b ? b->impl.bytes : 0);
  }
  BatchImpl& B = b->impl;
  B.pool = static_cast<char*>(pool);
  cudaMemsetAsync(pool, 0, B.bytes, current_stream());
  size_t o = B.tables_off;
  B.d_tiles_x = reinterpret_cast<int*>(B.pool + o);
  o += (size_t)kNumShapes * B.n * sizeof(int);
  o = (o + 255) / 256 * 256;
  B.d_prefix = reinterpret_cast<int*>(B.pool + o);
  o += (size_t)kNumShapes * (B.n + 1) * sizeof(int);
  o = (o + 255) / 256 * 256;
  B.d_status = reinterpret_cast<Status*>(B.pool + o);
  o += 256;
  B.d_inst = B.pool + o;
  cudaStreamSynchronize(current_stream());
  // Uniform meshes: spacing width/gnx on every face and cell, and the face
  // positions (for device-side problem set-up) after the four spacing arrays.
  for (int i = 0; i < B.n; ++i) {
    const int nx = B.gnx[i] + 4, ny = B.gny[i] + 4;
    const InstLayout L = inst_layout(nx, ny, B.precision);
    const size_t m = (size_t)std::max(nx, ny) + 1;
    double* mesh = reinterpret_cast<double*>(B.pool + B.off[i] + L.mesh);
    const double dx = B.width[i] / B.gnx[i], dy = B.height[i] / B.gny[i];
    k_fill<<<8, 256, 0, current_stream()>>>(mesh, m, dx);
    k_fill<<<8, 256, 0, current_stream()>>>(mesh + m, m, dy);
    k_fill<<<8, 256, 0, current_stream()>>>(mesh + 2 * m, m, dx);
    k_fill<<<8, 256, 0, current_stream()>>>(mesh + 3 * m, m, dy);
    launch_uniform_edges(current_stream(), mesh + 4 * m, nx + 1, 2, B.width[i], B.gnx[i]);
    launch_uniform_edges(current_stream(), mesh + 5 * m, ny + 1, 2, B.height[i], B.gny[i]);
  }
  const int st = check_launch("gb300_batch_bind");
  if (st != GB300_OK) return st;
  return retune(B);
}

namespace {

// Ghost fill, FP32 shadows and the driver's first set_timestep of instance i
// once its interior density and energy are in place.
int finish_state(flow::BatchImpl& B, int i, double dt_param, const char* where) {
  using namespace flow;
  const int gx = B.gnx[i], gy = B.gny[i], nx = gx + 4, ny = gy + 4;
  (void)gx;
  (void)gy;
  const InstLayout L = inst_layout(nx, ny, B.precision);
  char* base = B.pool + B.off[i];
  double* d_rho = reinterpret_cast<double*>(base + L.rho);
  double* d_e = reinterpret_cast<double*>(base + L.e);
  cudaStream_t s = current_stream();
  launch_boundary(s, nx, ny, 2, d_rho, kNoInvert);
  launch_boundary(s, nx, ny, 2, d_e, kNoInvert);
  if (B.precision == 1) {
    const size_t n = (size_t)nx * ny;
    k_shadow<<<64, 256, 0, s>>>(n, d_rho, reinterpret_cast<float*>(base + L.rho_r));
    k_shadow<<<64, 256, 0, s>>>(n, d_e, reinterpret_cast<float*>(base + L.e_r));
  }
  // The driver's set_timestep(first_step = 0) before the loop (main.c:64-66)
  // with zero viscous stresses (the FP64 layout's Q arrays are still zero; for
  // the mixed layout the zeroed first-sweep block serves).
  double* zeros = reinterpret_cast<double*>(base + (B.precision ? L.s_r : L.Qxx));
  cudaMemsetAsync(zeros, 0, (size_t)nx * ny * sizeof(double), s);
  double* ra = reinterpret_cast<double*>(base + L.ra);
  const size_t m = (size_t)std::max(nx, ny) + 1;
  const double* mesh = reinterpret_cast<const double*>(base + L.mesh);
  MeshView mv{mesh, mesh + m, mesh + 2 * m, mesh + 3 * m};
  const double dt0 = kCT * dt_param;
  launch_min_timestep(s, nx, ny, 2, 10.0, dt0, 0, zeros, zeros, d_rho, d_e, mv, ra);
  // The fused CFL minimum starts from "no candidate yet".
  cudaMemsetAsync(ra + kRaMinSlot, 0xff, sizeof(double), s);
  return check_launch(where);
}

}  // namespace

int gb300_batch_set_state(GB300Batch* b, int i, const double* rho, const double* e,
                          double dt_param) {
  using namespace flow;
  if (!b || i < 0 || i >= b->impl.n || !rho || !e || !b->impl.pool) {
    return record_error(GB300_ERR_ARG, "gb300_batch_set_state: bad arguments");
  }
  BatchImpl& B = b->impl;
  const int gx = B.gnx[i], gy = B.gny[i], nx = gx + 4;
  const InstLayout L = inst_layout(nx, gy + 4, B.precision);
  char* base = B.pool + B.off[i];
  double* d_rho = reinterpret_cast<double*>(base + L.rho);
  double* d_e = reinterpret_cast<double*>(base + L.e);
  cudaStream_t s = current_stream();
  // Interior rows (host arrays are gy x gx, row-major) into the padded mesh.
  cudaMemcpy2DAsync(d_rho + 2 * (size_t)nx + 2, nx * sizeof(double), rho, gx * sizeof(double),
                    gx * sizeof(double), gy, cudaMemcpyHostToDevice, s);
  cudaMemcpy2DAsync(d_e + 2 * (size_t)nx + 2, nx * sizeof(double), e, gx * sizeof(double),
                    gx * sizeof(double), gy, cudaMemcpyHostToDevice, s);
  return finish_state(B, i, dt_param, "gb300_batch_set_state");
}

int gb300_batch_fill_boxes(GB300Batch* b, int i, const double* boxes, int nboxes,
                           double dt_param) {
  using namespace flow;
  if (!b || i < 0 || i >= b->impl.n || !b->impl.pool) {
    return record_error(GB300_ERR_ARG, "gb300_batch_fill_boxes: bad arguments");
  }
  BatchImpl& B = b->impl;
  const int nx = B.gnx[i] + 4, ny = B.gny[i] + 4;
  const InstLayout L = inst_layout(nx, ny, B.precision);
  char* base = B.pool + B.off[i];
  const size_t m = (size_t)std::max(nx, ny) + 1;
  const double* mesh = reinterpret_cast<const double*>(base + L.mesh);
  const int st = launch_fill_boxes(current_stream(), nx, ny, mesh + 4 * m, mesh + 5 * m, boxes,
                                   nboxes, reinterpret_cast<double*>(base + L.rho),
                                   reinterpret_cast<double*>(base + L.e));
  if (st != GB300_OK) return st;
  return finish_state(B, i, dt_param, "gb300_batch_fill_boxes");
}

int gb300_batch_set_tuning(GB300Batch* b, int rows, int ctas_per_sm, int order) {
  using namespace flow;
  if (!b || rows < 1 || rows > kMaxRows || ctas_per_sm < 0 || (order != 0 && order != 1)) {
    return record_error(GB300_ERR_ARG, "gb300_batch_set_tuning: bad arguments");
  }
  BatchImpl& B = b->impl;
  B.rows = rows;
  B.ctas_per_sm = ctas_per_sm;
  B.order = order;
  return B.pool ? retune(B) : GB300_OK;
}

int gb300_batch_get_tuning(const GB300Batch* b, int* rows, int* ctas_per_sm, int* order,
                           int* grid) {
  if (!b) return GB300_ERR_ARG;
  if (rows) *rows = b->impl.rows;
  if (ctas_per_sm) *ctas_per_sm = b->impl.ctas_per_sm;
  if (order) *order = b->impl.order;
  if (grid) *grid = b->impl.grid;
  return GB300_OK;
}

// Advances every instance by `steps` timesteps.  With use_graph, pairs of
// steps replay a captured CUDA graph (captured on first use).
int gb300_batch_step(GB300Batch* b, int steps, int use_graph) {
  using namespace flow;
  if (!b || !b->impl.pool) return record_error(GB300_ERR_ARG, "gb300_batch_step: unbound batch");
  BatchImpl& B = b->impl;
  cudaStream_t s = current_stream();
  auto launch = [&](int tt) {
    return B.precision ? launch_batch_step<float>(B, s, tt) : launch_batch_step<double>(B, s, tt);
  };
  if (steps > 0) {
    const int mst = B.precision ? launch_batch_mesh_test<float>(B, s)
                                : launch_batch_mesh_test<double>(B, s);
    if (mst != GB300_OK) return mst;
  }
  int done = 0;
  // Step 0 (first_step = 1) and any odd leftover run as plain launches.
  while (done < steps && (B.tt == 0 || !use_graph || (B.tt % 2) != 0 || steps - done < 2)) {
    const int st = launch(B.tt);
    if (st != GB300_OK) return st;
    ++B.tt;
    ++done;
  }
  if (done < steps && use_graph && !B.graph) {
    cudaGraph_t g = nullptr;
    cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
    cudaStream_t cs = s;
    cudaStream_t own = nullptr;
    if (cs == nullptr) {  // the legacy stream cannot be captured
      cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking);
      cs = own;
    }
    cudaStreamBeginCapture(cs, mode);
    int st = B.precision ? launch_batch_step<float>(B, cs, 2) : launch_batch_step<double>(B, cs, 2);
    if (st == GB300_OK) {
      st = B.precision ? launch_batch_step<float>(B, cs, 3) : launch_batch_step<double>(B, cs, 3);
    }
    const cudaError_t ce = cudaStreamEndCapture(cs, &g);
    if (st != GB300_OK || ce != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      if (own) cudaStreamDestroy(own);
      cudaGetLastError();
      return record_error(GB300_ERR_CUDA, "gb300_batch_step: graph capture failed (%s)",
                          cudaGetErrorString(ce));
    }
    const cudaError_t ie = cudaGraphInstantiate(&B.graph, g, 0);
    cudaGraphDestroy(g);
    if (own) cudaStreamDestroy(own);
    if (ie != cudaSuccess) {
      B.graph = nullptr;
      return record_error(GB300_ERR_CUDA, "gb300_batch_step: graph instantiation failed (%s)",
                          cudaGetErrorString(ie));
    }
  }
  while (steps - done >= 2) {
    const cudaError_t ge = cudaGraphLaunch(B.graph, s);
    if (ge != cudaSuccess) {
      return record_error(GB300_ERR_CUDA, "gb300_batch_step: %s", cudaGetErrorString(ge));
    }
    B.tt += 2;
    done += 2;
  }
  while (done < steps) {
    const int st = launch(B.tt);
    if (st != GB300_OK) return st;
    ++B.tt;
    ++done;
  }
  return check_launch("gb300_batch_step");
}

// Status word of the batched kernel (GB300_ERR_TIMEOUT after a barrier ran
// out of iterations); synchronises the stream.  After reporting a timeout it
// clears the barrier state (counter, generation, error), so the batch can be
// stepped again; the instances' fields are then those of a step that stopped
// part-way.
int gb300_batch_status(GB300Batch* b) {
  using namespace flow;
  if (!b || !b->impl.pool) return GB300_ERR_ARG;
  Status st{};
  cudaMemcpyAsync(&st, b->impl.d_status, sizeof(st), cudaMemcpyDeviceToHost, current_stream());
  const cudaError_t err = cudaStreamSynchronize(current_stream());
  if (err != cudaSuccess) {
    return record_error(GB300_ERR_CUDA, "gb300_batch_status: %s", cudaGetErrorString(err));
  }
  if (st.error != 0) {
    cudaMemsetAsync(b->impl.d_status, 0, sizeof(Status), current_stream());
    const cudaError_t e2 = cudaStreamSynchronize(current_stream());
    if (e2 != cudaSuccess) {
      return record_error(GB300_ERR_CUDA, "gb300_batch_status: %s", cudaGetErrorString(e2));
    }
    return record_error(st.error, "gb300_batch: a grid barrier timed out");
  }
  return GB300_OK;
}

// Schedule of a step: GB300_BATCH_PHASES (one launch per phase over every
// instance's tiles) or GB300_BATCH_PERSISTENT (one cooperative launch per
// step, grid barriers between the phases).  A captured step graph is dropped.
int gb300_batch_set_schedule(GB300Batch* b, int schedule) {
  using namespace flow;
  if (!b || (schedule != GB300_BATCH_PHASES && schedule != GB300_BATCH_PERSISTENT)) {
    return record_error(GB300_ERR_ARG, "gb300_batch_set_schedule: bad arguments");
  }
  BatchImpl& B = b->impl;
  B.schedule = schedule;
  if (B.graph) {
    cudaGraphExecDestroy(B.graph);
    B.graph = nullptr;
  }
  return GB300_OK;
}

int gb300_batch_get_schedule(const GB300Batch* b) {
  return b ? b->impl.schedule : -1;
}

// Barrier wait bound of the batched kernel, in 64 ns naps (default 2^25,
// about 2 s).  A captured step graph holds the old bound, so it is dropped
// and captured again on the next graph step.
int gb300_batch_set_spin_limit(GB300Batch* b, long long spins) {
  using namespace flow;
  if (!b || spins < 0) {
    return record_error(GB300_ERR_ARG, "gb300_batch_set_spin_limit: bad arguments");
  }
  BatchImpl& B = b->impl;
  B.spin_limit = spins;
  if (B.graph) {
    cudaGraphExecDestroy(B.graph);
    B.graph = nullptr;
  }
  return GB300_OK;
}

int gb300_batch_get_state(GB300Batch* b, int i, double* rho, double* e, double* dt_pair,
                          double* totals) {
  using namespace flow;
  if (!b || i < 0 || i >= b->impl.n || !b->impl.pool) {
    return record_error(GB300_ERR_ARG, "gb300_batch_get_state: bad arguments");
  }
  BatchImpl& B = b->impl;
  const int gx = B.gnx[i], gy = B.gny[i], nx = gx + 4, ny = gy + 4;
  const InstLayout L = inst_layout(nx, ny, B.precision);
  char* base = B.pool + B.off[i];
  cudaStream_t s = current_stream();
  double* ra = reinterpret_cast<double*>(base + L.ra);
  if (totals) {
    launch_conservation(s, nx, ny, 2, reinterpret_cast<double*>(base + L.rho),
                        reinterpret_cast<double*>(base + L.e), ra);
    cudaMemcpyAsync(totals, ra + kRaMass, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
  }
  if (rho) {
    cudaMemcpy2DAsync(rho, gx * sizeof(double), base + L.rho + (2 * (size_t)nx + 2) * 8,
                      nx * sizeof(double), gx * sizeof(double), gy, cudaMemcpyDeviceToHost, s);
  }
  if (e) {
    cudaMemcpy2DAsync(e, gx * sizeof(double), base + L.e + (2 * (size_t)nx + 2) * 8,
                      nx * sizeof(double), gx * sizeof(double), gy, cudaMemcpyDeviceToHost, s);
  }
  if (dt_pair) cudaMemcpyAsync(dt_pair, ra + kRaDt, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
  const cudaError_t err = cudaStreamSynchronize(s);
  if (err != cudaSuccess) {
    return record_error(GB300_ERR_CUDA, "gb300_batch_get_state: %s", cudaGetErrorString(err));
  }
  return GB300_OK;
}

long long gb300_batch_cells(const GB300Batch* b) {
  if (!b) return 0;
  long long c = 0;
  for (int i = 0; i < b->impl.n; ++i) c += (long long)b->impl.gnx[i] * b->impl.gny[i];
  return c;
}

void gb300_batch_destroy(GB300Batch* b) {
  if (!b) return;
  if (b->impl.graph) cudaGraphExecDestroy(b->impl.graph);
  delete b;
}

}  // extern "C"
