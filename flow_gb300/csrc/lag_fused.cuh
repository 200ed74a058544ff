// lag_fused.cuh -- the Lagrangian phase of the FP64 timestep as one kernel:
// equation of state, pressure acceleration, artificial viscosity, viscous
// acceleration, shock heating and work, and the CFL minimum of set_timestep
// (omp3/flow.c:55-290, 73-106), with the reference's ghost fills of those
// stages (omp3/flow.c:156-157, 206-207, 243-244, 289) done in the tile.
//
// Why one kernel: on a mesh that is mostly at rest (the blast problems) the
// four separate Lagrangian kernels are bound by the bytes they move -- ~165 B
// per cell of pressure, stress and velocity round trips through HBM against
// the 32 B of state they read.  Here a CTA reads density, energy and both
// momenta once (TMA bulk copies of row segments into a shared-memory ring),
// keeps every intermediate in registers and shared memory, and writes the
// Lagrangian velocities plus the values that changed.
//
// Tile: kT threads, one column each, own kW = kT - 6 output columns; the
// three columns either side are recomputed (a cell's shock heating needs the
// final face velocities, which need the viscous stresses of both neighbours,
// which need the pressure-phase velocities of the faces around those, which
// need the pressures of the cells around those: three cells each way).  A
// tile marches its rows top to bottom with the same three-row halo above and
// below; each iteration takes one input row i and runs the stages at fixed
// lags behind it:
//   x direction  u_pre(i), Qxx(i-1), u_fin(i-2), shock heating(i-3)
//   y direction  v_pre(i), Qyy(i-2), v_fin(i-2)
// The x stages exchange neighbour values through double-buffered shared rows
// written before the iteration's one barrier and read after it; the y stages
// stay in each thread's registers.
//
// Halos read the state of cells that other tiles update, so this kernel never
// writes the state arrays: changed energies and momenta go to scratch arrays
// with per-row change masks, and k_lag_apply copies them into place once
// every tile has finished.
//
// Arithmetic: every value is formed by the same expressions, in the same
// order, as the separate tile functions of fused_tiles.cuh
// (tile_lag_pressure_impl, tile_lag_viscosity, tile_lag_viscous_accel_impl,
// tile_lag_energy_dt_impl), so both forms give the same numbers bit for bit.
#pragma once

#include <cstdint>

#include "fused_tiles.cuh"

namespace flow {
namespace lagf {

constexpr int kT = 128;                 // threads per CTA, one column each
constexpr int kHalo = 3;                // recomputed columns / rows per side
constexpr int kW = kT - 2 * kHalo;      // output columns per CTA
constexpr int kAhead = 4;               // input rows in flight
constexpr int kSlots = kAhead + 1;      // ring slots
constexpr int kSeg = kT + 4;            // doubles per staged row segment
constexpr int kMaxRows = 64;            // tallest tile (output rows)
constexpr int kMaxSpan = kMaxRows + 2 * kHalo;
constexpr int kDefaultRows = 32;
constexpr int kWarps = kT / 32;
// Ring planes.
enum : int { kPlRho = 0, kPlE = 1, kPlRhoU = 2, kPlRhoV = 3, kPlanes = 4 };
// Change-mask fields: per (mask row, tile) kWarps words of warp ballots, bit
// l of word w for the tile's column cb - kHalo + 32 w + l.
enum : int { kMaskE = 0, kMaskRhoU = 1, kMaskRhoV = 2, kMaskFields = 3 };
// mbarrier polls before a row copy is taken as lost (the kernel then records
// GB300_ERR_TIMEOUT in the status word and every tile returns).
constexpr unsigned kSpinLimit = 1u << 22;

struct LagArgs {
  int nx, ny, pad;
  int rows;    // output rows per CTA, 1 .. kMaxRows
  int ntx;     // CTAs across the mesh
  const double* edgedx;
  const double* edgedy;
  const double* celldx;
  const double* celldy;
  const double* rho;    // state at the start of the step, read only
  const double* e;
  const double* rho_u;
  const double* rho_v;
  double* u;            // Lagrangian velocities, every face and its ghosts
  double* v;
  double* e_new;        // changed values (cell / x-face / y-face layouts)
  double* rho_u_new;
  double* rho_v_new;
  unsigned* masks;      // [(mask row * ntx + bx) * kMaskFields + field][kWarps]
  double* ra;           // reduce_array: ticket, status
  unsigned long long* min_slot;
  const unsigned long long* mesh_pow2;
  double* dt_slot;
  double dt, dt_h, max_dt;
  int first_step;
};

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for the phase of the given parity; false when the wait gave up.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
  for (unsigned n = 0; n < kSpinLimit; ++n) {
    if (mbar_try_wait(bar, parity)) return true;
  }
  return false;
}
// Orders this CTA's earlier shared-memory reads before later writes by the
// asynchronous (TMA) proxy.
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// TMA bulk copy of bytes (a multiple of 16; both addresses 16-byte aligned)
// from global to this CTA's shared memory, completing on bar.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes,
                                         unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// A staged row segment: columns [clo, chi) of one array row, copied from the
// 16-byte boundary at or below clo to the one at or above chi, so that column
// c sits at shared index c - c0a.  The array base must be 16-byte aligned;
// clo >= 1 and chi <= the row length - 1 keep the rounded copy inside the row
// (or the next one) and inside the allocation.
struct Seg {
  long long g0a;  // first element copied
  int n;          // elements copied (even), 0 for none
  int c0a;        // column of shared index 0
};
__device__ __forceinline__ Seg make_seg(long long row_base, int clo, int chi) {
  Seg s;
  if (clo >= chi) {
    s.g0a = 0;
    s.n = 0;
    s.c0a = clo;
    return s;
  }
  const long long g0 = row_base + clo;
  s.g0a = g0 & ~1LL;
  const long long g1a = (row_base + chi + 1) & ~1LL;
  s.n = (int)(g1a - s.g0a);
  s.c0a = clo - (int)(g0 - s.g0a);
  return s;
}

// The rows and columns a tile stages (see the validity ranges in the tile).
struct TileGeom {
  int cb;        // first output column
  int r0, r1;    // output rows [r0, r1)
  int ia, ib;    // input rows marched, inclusive
};

__device__ __forceinline__ Seg seg_cells(const LagArgs& a, const TileGeom& g, int i) {
  // Cell rows 1 .. ny-2 and columns 1 .. nx-2: the pressures of every face the
  // tile forms (faces pad .. nx-pad, rows pad .. ny-pad).
  if (i < max(g.r0 - kHalo, 1) || i > min(g.r1 + kHalo - 1, a.ny - 2)) return make_seg(0, 1, 0);
  return make_seg((long long)i * a.nx, max(g.cb - kHalo, 1), min(g.cb - kHalo + kT, a.nx - 1));
}
__device__ __forceinline__ Seg seg_xfaces(const LagArgs& a, const TileGeom& g, int i) {
  // x-face momenta of the output rows, faces cb-2 .. cb+kW+2 within
  // pad .. nx-pad (the ghost faces' values are mirrors of interior ones).
  if (i < g.r0 || i >= g.r1) return make_seg(0, 1, 0);
  return make_seg((long long)i * (a.nx + 1), max(g.cb - 2, a.pad),
                  min(g.cb + kW + 2, a.nx - a.pad) + 1);
}
__device__ __forceinline__ Seg seg_yfaces(const LagArgs& a, const TileGeom& g, int i) {
  // y-face momenta of the output columns, faces r0-2 .. r1+2 within
  // pad .. ny-pad.
  if (i < max(g.r0 - 2, a.pad) || i > min(g.r1 + 2, a.ny - a.pad)) return make_seg(0, 1, 0);
  return make_seg((long long)i * a.nx, max(g.cb, a.pad), min(g.cb + kW, a.nx - a.pad));
}

__device__ __forceinline__ TileGeom tile_geom(const LagArgs& a, int bx, int by) {
  TileGeom g;
  g.cb = a.pad + bx * kW;
  g.r0 = a.pad + by * a.rows;
  g.r1 = min(g.r0 + a.rows, a.ny - a.pad);
  g.ia = g.r0 - kHalo;
  g.ib = g.r1 + kHalo - 1;
  return g;
}

// True when every spacing the tile uses (columns cb-4 .. cb+kW+4, rows
// r0-4 .. r1+4) is a positive normal power of two.  Block-uniform (barrier).
__device__ __forceinline__ bool tile_pow2(const LagArgs& a, const TileGeom& g) {
  if (a.mesh_pow2 && *a.mesh_pow2 == 1ull) return true;
  bool ok = true;
  for (int j = g.cb - 4 + (int)threadIdx.x; j <= g.cb + kW + 4; j += kT) {
    if (j >= 0 && j <= a.nx) ok = ok && d_is_pow2(a.celldx[j]) && d_is_pow2(a.edgedx[j]);
  }
  for (int i = g.r0 - 4 + (int)threadIdx.x; i <= g.r1 + 4; i += kT) {
    if (i >= 0 && i <= a.ny) ok = ok && d_is_pow2(a.celldy[i]) && d_is_pow2(a.edgedy[i]);
  }
  return __syncthreads_and(ok) != 0;
}

// The CFL result of a thread: its largest 1/dt^2 key with the S and spacing
// that gave it (tile_lag_energy_dt_impl's ranking).
struct CflBest {
  long long kbest = -1;
  double s_best = 0.0, c_best = 0.0;
};

// Ballot of pred over the warp, stored by lane 0 as the warp's mask word.
__device__ __forceinline__ void store_mask(const LagArgs& a, int row, int bx, int field,
                                           bool pred) {
  const unsigned b = __ballot_sync(0xffffffffu, pred);
  if ((threadIdx.x & 31) == 0) {
    a.masks[((size_t)(row * a.ntx + bx) * kMaskFields + field) * kWarps + (threadIdx.x >> 5)] = b;
  }
}

// Shared memory of a tile (one allocation per kernel, shared by the
// power-of-two and general variants of the tile).
struct __align__(16) LagSmem {
  double ring[kSlots][kPlanes][kSeg];    // staged input rows (TMA destinations)
  unsigned long long bar[kSlots];        // one mbarrier per ring slot
  double P[2][kT], R[2][kT];             // pressure, density of an input row
  double U[2][kT];                       // pressure-phase x-face velocity
  double Q[2][kT];                       // Qxx
  double UF[2][kT];                      // final x-face velocity
  double ey[kMaxSpan], iey[kMaxSpan], wy0[kMaxSpan], wy1[kMaxSpan];  // y faces
  double cy[kMaxSpan], icy[kMaxSpan], icy2[kMaxSpan];                // cell rows
};

// One tile of the fused Lagrangian phase.  Returns false when a row copy was
// lost (bounded wait); the caller then records the error.
template <bool kP2>
__device__ __forceinline__ bool lag_tile(const LagArgs& a, LagSmem& sm, int bx, int by,
                                         CflBest& cfl) {
  using Pr = Prec<double>;
  using tiles::face_average;
  using tiles::face_velocity;
  using tiles::lane_same;
  using tiles::warp_all;
  using tiles::warp_same;
  auto& s_ring = sm.ring;
  auto& s_bar = sm.bar;
  auto& s_P = sm.P;
  auto& s_R = sm.R;
  auto& s_U = sm.U;
  auto& s_Q = sm.Q;
  auto& s_UF = sm.UF;
  auto& s_ey = sm.ey;
  auto& s_iey = sm.iey;
  auto& s_wy0 = sm.wy0;
  auto& s_wy1 = sm.wy1;
  auto& s_cy = sm.cy;
  auto& s_icy = sm.icy;
  auto& s_icy2 = sm.icy2;

  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int t = threadIdx.x;
  const TileGeom g = tile_geom(a, bx, by);
  const int cb = g.cb, r0 = g.r0, r1 = g.r1, ia = g.ia, ib = g.ib;
  const int c = cb - kHalo + t;  // this thread's column
  // Mirror images exist only within 2*pad of a wall.
  const bool edge = !(cb - 2 >= 2 * pad && cb + kW + 2 <= nx - 2 * pad && r0 - 2 >= 2 * pad &&
                      r1 + 2 <= ny - 2 * pad);
  const double g1c = tiles::kG1;
  const double dt = a.dt, dt_h = a.dt_h;

  // ---- row factors of rows ia .. ib (y faces and cell rows)
  if (t <= ib - ia) {
    const int f = ia + t;
    if (f >= 1 && f <= ny) {
      const double ey = a.edgedy[f], cy = a.celldy[f];
      s_ey[t] = ey;
      s_iey[t] = tiles::geo_rcp<double, kP2>(ey);
      s_wy0[t] = tiles::geo_half_ratio<double, kP2>(cy, ey);
      s_wy1[t] = tiles::geo_half_ratio<double, kP2>(a.celldy[f - 1], ey);
      s_cy[t] = cy;
      s_icy[t] = tiles::geo_rcp<double, kP2>(cy);
      s_icy2[t] = tiles::geo_rcp_sq<kP2>(cy);
    }
  }
  // ---- roles of this thread's column
  // Pressure-phase x face formed by this thread (fc), negated for the two
  // ghost faces whose values the viscous stresses read (pad-1, nx-pad+1).
  int fc = -1;
  bool ghost = false;
  if (t >= 1) {
    if (c >= pad && c <= nx - pad) {
      fc = c;
    } else if (c == pad - 1) {
      fc = pad;
      ghost = true;
    } else if (c == nx - pad + 1) {
      fc = nx - pad;
      ghost = true;
    }
  }
  const int tf = fc - (cb - kHalo);              // thread of face fc's right cell
  const bool q_role = c >= max(cb - 1, pad) && c <= min(cb + kW, nx - pad - 1);
  const bool uf_role = c >= max(cb, pad) && c <= min(cb + kW, nx - pad);
  const bool uf_out = uf_role && c < cb + kW;
  const bool cell_out = c >= max(cb, pad) && c < min(cb + kW, nx - pad);  // shock, y faces
  double ex = 0.0, iex = 0.0, wx0 = 0.0, wx1 = 0.0;
  if (fc >= 0) {
    ex = a.edgedx[fc];
    iex = tiles::geo_rcp<double, kP2>(ex);
    wx0 = tiles::geo_half_ratio<double, kP2>(a.celldx[fc], ex);
    wx1 = tiles::geo_half_ratio<double, kP2>(a.celldx[fc - 1], ex);
  }
  double cx = 0.0, icx = 0.0, icx2 = 0.0;
  if (uf_role) {
    cx = a.celldx[c];
    icx = tiles::geo_rcp<double, kP2>(cx);
    icx2 = tiles::geo_rcp_sq<kP2>(cx);
  }
  // First and last valid y face of the window (ghost faces included).
  const int fa = (r0 - 2 >= pad) ? r0 - 2 : pad - 1;
  const int fe = (r1 + 2 >= ny - pad + 1) ? ny - pad + 1 : r1 + 2;

  // ---- the ring of staged input rows
  // Lane 0 of warp w stages plane w of each row (one warp per plane), so the
  // issue work is spread over the warps; a slot's mbarrier completes once all
  // of them have arrived and their bytes have landed.
  static_assert(kWarps == kPlanes, "one staging warp per ring plane");
  const int wid = t >> 5;
  const bool stager = (t & 31) == 0;
  auto issue = [&](int i) {  // stager lanes only
    const int slot = (i - ia) % kSlots;
    Seg sg;
    const double* src;
    if (wid == kPlRho) {
      sg = seg_cells(a, g, i);
      src = a.rho;
    } else if (wid == kPlE) {
      sg = seg_cells(a, g, i);
      src = a.e;
    } else if (wid == kPlRhoU) {
      sg = seg_xfaces(a, g, i);
      src = a.rho_u;
    } else {
      sg = seg_yfaces(a, g, i);
      src = a.rho_v;
    }
    fence_proxy_async();
    if (sg.n == 0) {
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&s_bar[slot]))
                   : "memory");
      return;
    }
    mbar_arrive_tx(&s_bar[slot], 8u * (unsigned)sg.n);
    bulk_g2s(s_ring[slot][wid], src + sg.g0a, 8u * (unsigned)sg.n, &s_bar[slot]);
  };
  if (t == 0) {
    for (int s = 0; s < kSlots; ++s) mbar_init(&s_bar[s], kWarps);
    mbar_fence_init();
  }
  __syncthreads();
  if (stager) {
    for (int i = ia; i < ia + kAhead && i <= ib; ++i) issue(i);
  }
  int issued = min(ia + kAhead, ib + 1);  // rows [ia, issued) are in flight or done

  // Shared index of a column in a staged row: col - clo + parity, the copy
  // starting at the 16-byte boundary at or below clo (make_seg).
  const int clo_c = max(cb - kHalo, 1), clo_x = max(cb - 2, pad), clo_y = max(cb, pad);
  const int cell_lo = max(r0 - kHalo, 1), cell_hi = min(r1 + kHalo - 1, ny - 2);
  const int yf_lo = max(r0 - 2, pad), yf_hi = min(r1 + 2, ny - pad);
  const bool c_cell = c >= 1 && c <= nx - 2;

  // ---- carried values (this thread's column)
  double P1 = 0.0, R1 = 0.0, R2 = 0.0, R3 = 0.0, E1 = 0.0, E2 = 0.0, E3 = 0.0;
  double w0 = 0.0, w1 = 0.0, w2 = 0.0, w3 = 0.0;    // v_pre of faces i-3 .. i
  double d1 = 0.0, g1 = 0.0;                          // d(i-1), |d(i-1) - d(i-2)|
  double mv1 = 0.0, mv2 = 0.0, rb1 = 0.0, rb2 = 0.0;  // y-face momenta, densities
  bool ch1 = false, ch2 = false;
  double qyA = 0.0;                                   // Qyy(i-3)
  double vfp = 0.0;                                   // v_fin(i-3)
  double mu1 = 0.0, mu2 = 0.0, rbx1 = 0.0, rbx2 = 0.0;  // x-face momenta, densities
  bool cu1 = false, cu2 = false;
  bool failed = false;

  for (int i = ia; i <= ib; ++i) {
    const int slot = (i - ia) % kSlots;
    const unsigned parity = (unsigned)((i - ia) / kSlots) & 1u;
    if (!mbar_wait(&s_bar[slot], parity)) failed = true;
    const int b = i & 1;
    // ================= phase 1: this column's own values
    double P0 = 0.0, R0 = 0.0, E0 = 0.0;
    if (i >= cell_lo && i <= cell_hi && c_cell) {
      const int ix = c - clo_c + (((i & nx) ^ clo_c) & 1);
      R0 = s_ring[slot][kPlRho][ix];
      E0 = s_ring[slot][kPlE][ix];
      P0 = g1c * R0 * E0;
    }
    const bool yrow = i >= yf_lo && i <= yf_hi;
    double mom_y = 0.0;
    if (yrow && cell_out) mom_y = s_ring[slot][kPlRhoV][c - clo_y + (((i & nx) ^ clo_y) & 1)];
    double mom_x = 0.0;
    const bool xrow = i >= r0 && i < r1;
    if (xrow && fc >= 0) {
      mom_x = s_ring[slot][kPlRhoU][fc - clo_x + (((i & (nx + 1)) ^ clo_x) & 1)];
    }
    s_P[b][t] = P0;
    s_R[b][t] = R0;

    // y direction: v_pre(i), Qyy(i-2), v_fin(i-2).
    double vnew = 0.0, mvn = 0.0, rbn = 0.0, qyB = 0.0, vfn = 0.0;
    bool chn = false, vf_changed = false;
    const int fv = i - 2;  // face of v_fin
    const bool vf_row = fv >= max(r0, pad) && fv <= min(r1, ny - pad);
    const bool vf_out = vf_row && (fv < r1 || fv == ny - pad);
    if (cell_out) {
      if (yrow) {
        const int k = i - ia;
        double mom = mom_y;
        double rbar;
        if (kP2 && warp_all(lane_same(P0, P1) && lane_same(R0, R1) &&
                                   lane_same(s_wy0[k], s_wy1[k]))) {
          rbar = Pr::twice(Pr::template mulp<true>(R0, s_wy0[k]));
        } else {
          const double dp = P0 - P1;
          if (!Pr::zero_skip_mem(dp)) {
            mom = Pr::template dsub<kP2>(mom, dt * dp, s_ey[k], s_iey[k]);
            chn = true;
          }
          rbar = face_average<double, kP2>(R0, s_wy0[k], R1, s_wy1[k]);
        }
        vnew = face_velocity(mom, rbar);
        mvn = mom;
        rbn = rbar;
      } else if (i == ny - pad + 1) {
        vnew = d_neg(w3);  // ghost face ny-pad+1 mirrors face ny-pad
      }
      w0 = w1;
      w1 = w2;
      w2 = w3;
      w3 = vnew;
      if (i == pad) w2 = d_neg(w3);  // ghost face pad-1 mirrors face pad
      // d(i) = min0(v(i) - v(i-1)) and g(i) = |d(i) - d(i-1)|.
      double dnew = 0.0, gnew = 0.0;
      if (i - 1 >= fa && i <= fe) {
        if (warp_all(lane_same(w3, w2) && d_is_zero(d1))) {
          dnew = 0.0;  // no jump of v across the cell or above it
          gnew = 0.0;
        } else {
          dnew = Pr::min0(w3 - w2);
          gnew = Pr::abs(dnew - d1);
        }
      }
      const int kq = i - 2;  // row of Qyy
      if (kq >= max(r0 - 1, pad) && kq <= min(r1, ny - pad - 1)) {
        qyB = Pr::zero_skip(d1) ? 0.0 : double(-kCQ) * R2 * d1 * Pr::half(gnew + g1);
      } else if (kq == ny - pad && kq <= r1) {
        qyB = qyA;  // ghost row ny-pad mirrors row ny-pad-1
      }
      d1 = dnew;
      g1 = gnew;
      if (vf_row) {
        double mom = mv2, vel = w1;
        vf_changed = ch2;
        const double qy = qyB;
        const double qy_dn = (fv == pad) ? qyB : qyA;  // ghost row pad-1 mirrors row pad
        if (!warp_same(qy, qy_dn)) {
          const double dqy = qy - qy_dn;
          if (!Pr::zero_skip_mem(dqy)) {
            const int k = fv - ia;
            mom = Pr::template dsub<kP2>(mom, dt * dqy, s_cy[k], s_icy[k]);
            vel = face_velocity(mom, rb2);
            vf_changed = true;
          }
        }
        vfn = vel;
        if (vf_out) {
          const size_t cy = cidx(nx, fv, c);
          a.v[cy] = vel;
          tiles::mirror(edge, a.v, nx, ny + 1, pad, fv, c, vel, false, true);
          if (vf_changed) a.rho_v_new[cy] = mom;
        } else {
          vf_changed = false;
        }
      }
    }
    if (vf_out) store_mask(a, fv, bx, kMaskRhoV, vf_changed);

    if (__syncthreads_or(failed) != 0) break;
    if (stager && issued <= ib) issue(issued);
    ++issued;

    // ================= phase 2: stages that read neighbour columns
    // Shock heating and work, and the CFL candidates, of cell row i-3
    // (tile_lag_energy_dt_impl).
    const int ks = i - 3;
    if (ks >= r0 && ks < r1) {
      bool e_changed = false;
      if (cell_out) {
        const int sb = ks & 1;
        const int k = ks - ia;
        const double u0f = s_UF[sb][t], u1f = s_UF[sb][t + 1];
        const double v0 = vfp, v1 = vfn;
        const double r = R3, er = E3, qx = s_Q[sb][t], qy = qyA;
        const bool rz = Pr::is_zero(r);
        double inv_r = 0.0, e_new;
        bool still;
        if (warp_all(lane_same(u1f, u0f) && lane_same(v1, v0))) {
          still = true;
          e_new = rz ? 0.0 : er;
        } else {
          const double dudx = Pr::template mulp<kP2>(u1f - u0f, icx);
          const double dvdy = Pr::template mulp<kP2>(v1 - v0, s_icy[k]);
          still = Pr::zero_skip_coarse(dudx) && Pr::zero_skip_coarse(dvdy);
          if (still) {
            e_new = rz ? 0.0 : er;
          } else {
            const double p = g1c * r * er;
            inv_r = rz ? 0.0 : Pr::rcp(r);
            const double div_dt = (dudx + dvdy) * dt_h;
            const double dq = -(dt_h * fma(qx, dudx, qy * dvdy)) * inv_r;
            const double e_q = er + dq;
            const double rho_c = r * Pr::rcp(1.0 + div_dt);
            const double e_c = fma(-(p * div_dt), inv_r, e_q);
            const double work =
                Pr::half(div_dt) * fma(double(tiles::kG1) * e_c, rho_c, p) * inv_r;
            e_new = rz ? 0.0 : e_q - work;
          }
        }
        const bool keep = still && !rz;
        if (!keep) {
          a.e_new[cidx(nx, ks, c)] = e_new;
          e_changed = true;
        }
        const double e_nr = keep ? er : e_new;
        const double s2 = double(kGam * (kGam - 1.0)) * e_nr;
        double sx = s2, sy = s2;
        if (!Pr::zero_skip_coarse(qx) || !Pr::zero_skip_coarse(qy)) {
          if (still) inv_r = rz ? 0.0 : Pr::rcp(r);
          const double two_inv_r = Pr::twice(inv_r);
          sx = fma(qx, two_inv_r, s2);
          sy = fma(qy, two_inv_r, s2);
        }
        const bool e_neg = d_lt0(e_new);
        const long long kx = e_neg ? -1 : dbits(Pr::template mulp<kP2>(sx, icx2));
        const long long ky = e_neg ? -1 : dbits(Pr::template mulp<kP2>(sy, s_icy2[k]));
        if (kx >= 0 && kx <= 0x7ff0000000000000LL && kx > cfl.kbest) {
          cfl.kbest = kx;
          cfl.s_best = sx;
          cfl.c_best = cx;
        }
        if (ky >= 0 && ky <= 0x7ff0000000000000LL && ky > cfl.kbest) {
          cfl.kbest = ky;
          cfl.s_best = sy;
          cfl.c_best = s_cy[k];
        }
      }
      store_mask(a, ks, bx, kMaskE, e_changed);
    }
    // Final x-face velocity of row i-2 (tile_lag_viscous_accel_impl).
    const int ku = i - 2;
    if (ku >= r0 && ku < r1) {
      bool u_changed = false;
      if (uf_role) {
        const int sb = ku & 1;
        double mom = mu2, vel = s_U[sb][t];
        u_changed = cu2;
        const double q1 = s_Q[sb][c == nx - pad ? t - 1 : t];  // ghost cells mirror
        const double q0 = s_Q[sb][c == pad ? t : t - 1];
        if (!warp_same(q1, q0)) {
          const double dqx = q1 - q0;
          if (!Pr::zero_skip_mem(dqx)) {
            mom = Pr::template dsub<kP2>(mom, dt * dqx, cx, icx);
            vel = face_velocity(mom, rbx2);
            u_changed = true;
          }
        }
        s_UF[sb][t] = vel;
        if (uf_out) {
          const size_t f = fidx(nx, ku, c);
          a.u[f] = vel;
          tiles::mirror(edge, a.u, nx + 1, ny, pad, ku, c, vel, true, false);
          if (u_changed) a.rho_u_new[f] = mom;
        } else {
          u_changed = false;
        }
      }
      store_mask(a, ku, bx, kMaskRhoU, u_changed);
    }
    // Qxx of row i-1 (tile_lag_viscosity).
    const int kx1 = i - 1;
    if (kx1 >= r0 && kx1 < r1 && q_role) {
      const int sb = kx1 & 1;
      s_Q[sb][t] = tiles::visc_stress<double>(R1, &s_U[sb][t], s_U[sb][t], s_U[sb][t + 1]);
    }
    // Pressure-phase x-face velocity of row i (tile_lag_pressure_impl).
    double mu0 = 0.0, rbx0 = 0.0;
    bool cu0 = false;
    if (xrow && fc >= 0) {
      const double rc = s_R[b][tf], rl = s_R[b][tf - 1];
      const double Pc = s_P[b][tf], Pl = s_P[b][tf - 1];
      double mom = mom_x;
      double rbar;
      if (kP2 && warp_all(lane_same(Pc, Pl) && lane_same(rc, rl) && lane_same(wx0, wx1))) {
        rbar = Pr::twice(Pr::template mulp<true>(rc, wx0));
      } else {
        const double dp = Pc - Pl;
        if (!Pr::zero_skip_mem(dp)) {
          mom = Pr::template dsub<kP2>(mom, dt * dp, ex, iex);
          cu0 = true;
        }
        rbar = face_average<double, kP2>(rc, wx0, rl, wx1);
      }
      const double vel = face_velocity(mom, rbar);
      s_U[b][t] = ghost ? d_neg(vel) : vel;
      mu0 = mom;
      rbx0 = rbar;
    }
    // ---- shift the carried values by one row
    R3 = R2; R2 = R1; R1 = R0;
    E3 = E2; E2 = E1; E1 = E0;
    P1 = P0;
    mv2 = mv1; mv1 = mvn; ch2 = ch1; ch1 = chn; rb2 = rb1; rb1 = rbn;
    qyA = qyB;
    vfp = vfn;
    mu2 = mu1; mu1 = mu0; cu2 = cu1; cu1 = cu0; rbx2 = rbx1; rbx1 = rbx0;
  }
  if (failed) {
    // Let the copies still in flight land before the CTA's shared memory is
    // released (bounded waits again).
    for (int i = max(ia, issued - kSlots); i < min(issued, ib + 1); ++i) {
      const int slot = (i - ia) % kSlots;
      mbar_wait(&s_bar[slot], (unsigned)((i - ia) / kSlots) & 1u);
    }
    return false;
  }
  return true;
}

}  // namespace lagf
}  // namespace flow
