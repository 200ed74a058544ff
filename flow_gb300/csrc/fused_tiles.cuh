// fused_tiles.cuh -- the tile-level device code of the fused timestep, shared
// by the single-problem kernels (fused.cu) and the persistent batched kernel
// (batched.cu).  Each tile_* function processes one CTA-sized tile (bx, by)
// of one phase of the timestep for one problem described by StepArgs; a
// thread may return early, but no tile function has a barrier after such a
// return, so consecutive tiles can run back to back in one CTA.
//
// Two precision forms share the code (precision.cuh):
//   R = double  the FP64 form behind solve_hydro_2d (GB300_MODE_FUSED);
//   R = float   the mixed form: FP32 for the equation of state,
//               accelerations, viscosity, shock heating, the CFL candidates
//               and every flux; FP64 for the stored density and energy, their
//               conservative update in the mass sweeps, the energy increment
//               of shock heating and the dt minimum.
//
// Same scheme as the reference timestep (omp3/flow.c:10-52), reorganised for
// GB300, where the FP64 issue rate (not HBM bandwidth) bounds the FP64 form:
//   * no flux or velocity is computed twice: each is produced once per point
//     and stored; only the 2-flop pressure is recomputed for neighbour faces;
//   * ghost cells are written by the tile that produces the interior value
//     (mirror), replacing the 19 ghost-fill launches per step;
//   * comparisons, selections and minmod run on the integer pipes, divisions
//     by the mesh spacing become multiplications by per-column / per-row
//     reciprocals (exact on power-of-two meshes), data divisions start from a
//     MUFU reciprocal with an FMA correction;
//   * the momentum/velocity chain and the conservative updates keep the
//     reference's evaluation order in the FP64 form, with correctly rounded
//     quotients (precision.cuh msub/madd/qdiv/dsub);
//   * the CFL minimum and dt/dt_h stay on the device (dt_slot).
// Every tile is a column strip: 128 threads own 128 consecutive columns and
// march a.rows rows (at most kMaxRows), carrying the values of previous rows
// in registers.
#pragma once

#include <cstddef>

#include "common.cuh"
#include "precision.cuh"

namespace flow {
namespace tiles {


constexpr int kCols = 128;
constexpr int kMaxRows = 32;     // tallest tile (shared-memory row tables)
constexpr int kDefaultRows = 16;
constexpr double kG1 = kGam - 1.0;

template <typename R>
struct StepArgs {
  int nx, ny, pad;
  const double* edgedx;
  const double* edgedy;
  const double* celldx;
  const double* celldy;
  double* rho;      // FP64 cell state
  double* e;
  R* rho_r;         // the same fields in bulk precision (aliases for FP64)
  R* e_r;
  double* P;        // FP64 form: the pressures, for the shock-heating kernel
  double* rho_old;  // unused: the first mass sweep reads the density itself
  R* u;             // velocities of the Lagrangian phase and the mass sweeps
  R* v;
  R* u_out;         // the caller's velocity arrays: the advected velocities
  R* v_out;
  R* rho_u;
  R* rho_v;
  R* Qxx;
  R* Qyy;
  R* F_x;
  R* F_y;
  R* uF_x;
  R* uF_y;
  R* vF_x;
  R* vF_y;
  double* ra;                  // caller scratch (reduce_array)
  unsigned long long* min_slot;  // running CFL minimum (FP64 bit pattern)
  // 1 when every mesh spacing is a positive normal power of two (formed on
  // the device at the start of the step); null or 0: tested per tile.
  const unsigned long long* mesh_pow2;
  double* dt_slot;             // [0] dt, [1] dt_h for the advection phase
  double dt, dt_h, max_dt;     // Lagrangian-phase pair (host values), max_dt
  int first_step;
  int rows;                    // tile height, 1 .. kMaxRows
  // Viscous-stress flags, or null.  Byte w of word (ii - pad) * qm_stride + bx
  // is 1 when a stress (Qxx or Qyy) of the 32 cells of warp w of column tile
  // bx in interior row ii is not +0: the viscosity kernel stored that warp
  // row's stresses and their ghost images.  0: every one of them is +0 and
  // nothing was stored (the arrays hold older values there); the readers
  // take +0 without loading.  Null: every stress is stored and read.
  unsigned* qmask;
  int qm_stride;               // words per interior row: ceil((nx - 2 pad) / kCols)
  // Mass-flux flags, or null (set together with qmask), in the same sense
  // for the mass fluxes the sweeps store and the momentum pairs read:
  //   fyflag: byte (ii - pad) * 4 qm_stride + 4 bx + w for y-face row ii
  //     (pad .. ny - pad) and the 32 columns of warp w of column tile bx;
  //   fxflag: byte (ii - pad) * fx_stride + 4 bx + w for interior row ii and
  //     the faces pad + 127 bx + 32 w + lane (lane < 32, 32 w + lane < 127)
  //     of warp w of x-sweep tile bx.
  unsigned char* fxflag;
  unsigned char* fyflag;
  int fx_stride;               // bytes per row: 4 ceil((nx + 1 - 2 pad) / 127)
  // Velocity flags, or null (set with the others): byte r * vf_stride +
  // (jj >> 5) is 1 when the pressure phase or the viscous update stored a
  // face velocity (x face (r, jj) or y face (r, jj)) that is not +0, or
  // changed a face momentum, in the 32 columns jj & ~31 .. (jj | 31) of row r
  // (rows 0 .. ny - 1 of the padded mesh, columns counted from 0).  Where
  // every byte around a tile is 0, the velocities it would read are +0 and it
  // does not load them.
  unsigned char* vflag;
  int vf_stride;               // bytes per row: 4 ceil(nx / 128)
  // The sweeps' tile-skip marks (SweepArgs::skip), set with the flags: one
  // byte per sweep tile, ceil((ny - 2 pad) / the sweeps' rows) bands of
  // max(ceil((nx + 1 - 2 pad) / 127), qm_stride) tiles.
  unsigned char* skipf;
  // The skip marks the previous step's first sweep left (its own half of the
  // two mark buffers), or null when this step does not directly follow a
  // flagged step on the same arrays.  Mark x of band b covers the interior
  // cells of rows pad + b rest_rows .. + rest_rows - 1 (that step's sweep
  // tile height) and columns pad + x rest_w .. + rest_w - 1 (127 for an x
  // sweep, 128 for a y sweep).
  // A marked cell, its energy, its density and the momenta of the faces
  // between two marked cells did not change in that step after its pressure
  // phase, which stored +0 velocities there and no momentum change.
  const unsigned char* rest;
  int rest_w, rest_tiles_x, rest_rows;
  // Each shock-heating tile's CFL minimum of the last step it ran (FP64 bit
  // pattern, word by * qm_stride + bx), set with the flags, or null.
  unsigned long long* cfl_tile;
  // Count of the first sweep's tiles not skipped this step (flags only).
  unsigned long long* moving;
};

// Writes the value of interior point (ii, jj) of a w x h array into each of
// its ghost mirror images (pad layers per side): column images negated when
// flip_x, row images when flip_y, corner images by both.  This reproduces the
// reflective fill of every ghost point whose mirror source is (ii, jj).
// edge: the tile may hold such points (tile_near_edge); a tile away from the
// walls skips the tests with one uniform branch.
template <typename T>
__device__ __forceinline__ void mirror(bool edge, T* a, int w, int h, int pad, int ii,
                                       int jj, T val, bool flip_x, bool flip_y) {
  if (!edge) return;
  int mc[2], mr[2];
  int nc = 0, nr = 0;
  if (jj < 2 * pad) mc[nc++] = 2 * pad - 1 - jj;
  if (jj >= w - 2 * pad) mc[nc++] = 2 * (w - pad) - 1 - jj;
  if (ii < 2 * pad) mr[nr++] = 2 * pad - 1 - ii;
  if (ii >= h - 2 * pad) mr[nr++] = 2 * (h - pad) - 1 - ii;
  if (nc == 0 && nr == 0) return;
  const T vx = flip_x ? -val : val;
  const T vy = flip_y ? -val : val;
  const T vxy = flip_x ? -vy : vy;
  for (int k = 0; k < nc; ++k) a[(size_t)ii * w + mc[k]] = vx;
  for (int r = 0; r < nr; ++r) {
    a[(size_t)mr[r] * w + jj] = vy;
    for (int k = 0; k < nc; ++k) a[(size_t)mr[r] * w + mc[k]] = vxy;
  }
}

// Stores an FP64 cell value, and its bulk-precision shadow in the mixed form,
// with ghost mirrors.
template <typename R>
__device__ __forceinline__ void store_cell(bool edge, double* a64, R* ar, int nx, int ny,
                                           int pad, int ii, int jj, double val) {
  const size_t c = cidx(nx, ii, jj);
  a64[c] = val;
  mirror(edge, a64, nx, ny, pad, ii, jj, val, false, false);
  if (Prec<R>::kMixed) {
    const R vr = Prec<R>::from_d(val);
    ar[c] = vr;
    mirror(edge, ar, nx, ny, pad, ii, jj, vr, false, false);
  }
}

// Asynchronous copy of one 4- or 8-byte element from global to shared memory
// (cp.async, through L1); with pred false nothing is read and the element is
// zero-filled.  A thread that reads back only the elements it copied itself
// needs no barrier: cp.async.wait_group makes its own copies visible to it.
template <typename T>
__device__ __forceinline__ void cp_async_elem(T* smem, const T* gmem, bool pred) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "4- or 8-byte elements");
  const unsigned dst = (unsigned)__cvta_generic_to_shared(smem);
  const int src_bytes = pred ? (int)sizeof(T) : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(dst), "l"(gmem),
               "n"((int)sizeof(T)), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
// Waits until at most n of this thread's newest copy groups are in flight.
template <int n>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(n) : "memory");
}
// The shared-memory slots of an asynchronous-copy ring, [slots][planes][cols]
// of T.  Declared here rather than in the tile: a tile's power-of-two and
// general variants are both compiled into its kernel, and shared arrays
// declared in each would be allocated twice; this function's array is one
// allocation per kernel for each (T, shape, tag).
template <typename T, int kSlotsN, int kPlanes, int kColsN, int kTag>
__device__ __forceinline__ T (*ring_slots())[kPlanes][kColsN] {
  __shared__ T buf[kSlotsN][kPlanes][kColsN];
  return buf;
}

// pred holds in every active lane of the warp (a warp-uniform branch
// condition).
__device__ __forceinline__ bool warp_all(bool pred) {
  return __all_sync(__activemask(), pred) != 0;
}

// FP64 form: a and b are the same finite number, so that a - b is +0 and
// a + b is exactly 2a (tests on the bit patterns).  The mixed form's FP32
// differences cost less than the tests, so it never takes these paths.
template <typename R>
__device__ __forceinline__ bool lane_same(R a, R b) {
  if constexpr (Prec<R>::kMixed) {
    return false;
  } else {
    return dbits(a) == dbits(b) && (dhi(a) & 0x7ff00000) != 0x7ff00000;
  }
}
// lane_same in every active lane of the warp.
template <typename R>
__device__ __forceinline__ bool warp_same(R a, R b) {
  if constexpr (Prec<R>::kMixed) {
    return false;
  } else {
    return warp_all(lane_same(a, b));
  }
}
// FP64 form: a and b are zeros in every active lane of the warp (then a + b
// is the zero sum_zeros gives).
template <typename R>
__device__ __forceinline__ bool warp_zeros(R a, R b) {
  if constexpr (Prec<R>::kMixed) {
    return false;
  } else {
    return warp_all(d_is_zero(a) && d_is_zero(b));
  }
}
// Stores a flag byte (every lane of a warp stores the same byte: one
// transaction, and no divergent branch in the row loop).  An asm statement
// without a memory clobber: a char
// store may alias any object, and through a plain store the compiler would
// have to assume that it changes the data a tile has loaded (and reload or
// stop prefetching it).  No reader of a flag runs in the kernel that writes
// it.
__device__ __forceinline__ void store_flag(unsigned char* p, bool v) {
  asm volatile("st.global.u8 [%0], %1;" ::"l"(p), "h"((unsigned short)(v ? 1 : 0)));
}

// Whether every face velocity in rows r0 .. r1 and columns c0 .. c1 (of
// the padded mesh, clamped to it) is +0 by the velocity flags.  The ranges
// the tiles pass reach two rows and columns past what they read, so that
// they hold the mirror source of every ghost face they read.  Block-uniform
// (barrier); called by every thread of the block.  False without flags.
template <typename A>
__device__ __forceinline__ bool tile_vel_still(const A& a, int r0, int r1, int c0, int c1) {
  if (!a.vflag) return false;  // no velocity flags this step (uniform)
  r0 = max(r0, 0);
  r1 = min(r1, a.ny - 1);
  const int g0 = max(c0, 0) >> 5, g1 = min(c1, a.nx) >> 5;
  const int ng = g1 - g0 + 1, total = max(0, r1 - r0 + 1) * ng;
  bool any = false;
  for (int q = threadIdx.x; q < total; q += blockDim.x) {
    const int r = r0 + q / ng, g = g0 + q % ng;
    any |= a.vflag[(size_t)r * a.vf_stride + g] != 0;
  }
  return __syncthreads_or(any) == 0;
}

// Whether every cell of rows r0 .. r1 - 1 and columns c0 .. c1 - 1 was at rest
// through the previous step by its first sweep's skip marks (StepArgs::rest).
// A ghost cell holds the mirror image of one of the pad interior cells next
// to its wall, written together with it, so a range reaching into the ghosts
// is tested on the interior cells up to those.  Block-uniform (barrier);
// called by every thread of the block.  False without marks.
template <typename A>
__device__ __forceinline__ bool rest_cells(const A& a, int r0, int r1, int c0, int c1) {
  if (!a.rest) return false;  // uniform
  const int pad = a.pad;
  if (r0 < pad) {
    r0 = pad;
    r1 = max(r1, 2 * pad);
  }
  if (r1 > a.ny - pad) {
    r1 = a.ny - pad;
    r0 = min(r0, a.ny - 2 * pad);
  }
  if (c0 < pad) {
    c0 = pad;
    c1 = max(c1, 2 * pad);
  }
  if (c1 > a.nx - pad) {
    c1 = a.nx - pad;
    c0 = min(c0, a.nx - 2 * pad);
  }
  if (r0 >= r1 || c0 >= c1) return false;
  const int b0 = (r0 - pad) / a.rest_rows, b1 = (r1 - 1 - pad) / a.rest_rows;
  const int x0 = (c0 - pad) / a.rest_w, x1 = (c1 - 1 - pad) / a.rest_w;
  const int nxb = x1 - x0 + 1, total = (b1 - b0 + 1) * nxb;
  bool ok = true;
  for (int q = threadIdx.x; q < total; q += blockDim.x) {
    ok = ok && a.rest[(size_t)(b0 + q / nxb) * a.rest_tiles_x + x0 + q % nxb] != 0;
  }
  return __syncthreads_and(ok) != 0;
}

// x is +0 (all bits zero).
template <typename R>
__device__ __forceinline__ bool is_plus_zero(R x) {
  if constexpr (Prec<R>::kMixed) {
    return __float_as_uint(x) == 0u;
  } else {
    return dbits(x) == 0;
  }
}
// The viscous-stress flag of cell column col (interior) in the flag word of
// its column tile; word0 / word1 hold the words of tiles bx - 1 and bx.
__device__ __forceinline__ bool qflag(unsigned word0, unsigned word1, int col, int pad, int bx) {
  const int g = (col - pad) >> 5;
  const unsigned w = ((g >> 2) == bx) ? word1 : word0;
  return ((w >> (8 * (g & 3))) & 0xffu) != 0u;
}

// The IEEE sum of two zeros: -0 only when both are -0.
template <typename R>
__device__ __forceinline__ R sum_zeros(R a, R b) {
  if constexpr (Prec<R>::kMixed) {
    return __uint_as_float(__float_as_uint(a) & __float_as_uint(b));
  } else {
    return dfrom(dbits(a) & dbits(b));
  }
}

// True when a tile whose columns start at col0 and rows at row0 may write a
// point within 2*pad of a wall of any array (so that mirror has images to
// write): the tile's points lie in [col0, col0 + kCols) x [row0 - 1,
// row0 + rows] (face rows included), tested with a margin.  Block-uniform.
__device__ __forceinline__ bool tile_near_edge(int nx, int ny, int pad, int col0, int row0,
                                               int rows) {
  return !(col0 - 2 >= 2 * pad && col0 + kCols + 2 <= nx - 2 * pad && row0 - 2 >= 2 * pad &&
           row0 + rows + 2 <= ny - 2 * pad);
}

// True when every mesh spacing (celldx, edgedx, celldy, edgedy) within two
// entries of the block's columns [col0, col0 + kCols) and rows
// [row0, row0 + rows) is a power of two -- the uniform power-of-two meshes of
// the benchmark problems -- so that divisions by those spacings are exact as
// multiplications by their reciprocals.  Block-uniform (barrier).
template <typename R>
__device__ __forceinline__ bool block_mesh_pow2(const StepArgs<R>& a, int col0, int row0) {
  // The whole mesh (one cached word) before the tile's own spacings.
  if (a.mesh_pow2 && *a.mesh_pow2 == 1ull) return true;
  bool ok = true;
  for (int j = col0 - 2 + (int)threadIdx.x; j < col0 + kCols + 2; j += kCols) {
    if (j >= 0 && j <= a.nx) ok = ok && d_is_pow2(a.celldx[j]) && d_is_pow2(a.edgedx[j]);
  }
  for (int i = row0 - 2 + (int)threadIdx.x; i < row0 + a.rows + 2; i += kCols) {
    if (i >= 0 && i <= a.ny) ok = ok && d_is_pow2(a.celldy[i]) && d_is_pow2(a.edgedy[i]);
  }
  return __syncthreads_and(ok) != 0;
}

// Runs tile(kPow2) with kPow2 = true for FP64 tiles whose mesh spacings are
// all powers of two.  (The mixed form's FP32 arithmetic gains nothing from
// it; its mass sweeps, whose FP64 conservative update multiplies by the face
// lengths, dispatch with FLOW_POW2_DISPATCH_ALL.)
#define FLOW_POW2_DISPATCH(R, a, col0, row0, CALL_TRUE, CALL_FALSE)          \
  do {                                                                      \
    if constexpr (!Prec<R>::kMixed) {                                       \
      if (block_mesh_pow2(a, col0, row0)) {                                 \
        CALL_TRUE;                                                          \
        return;                                                             \
      }                                                                     \
    }                                                                       \
    CALL_FALSE;                                                             \
  } while (0)
#define FLOW_POW2_DISPATCH_ALL(a, col0, row0, CALL_TRUE, CALL_FALSE)         \
  do {                                                                      \
    if (block_mesh_pow2(a, col0, row0)) {                                   \
      CALL_TRUE;                                                            \
      return;                                                               \
    }                                                                       \
    CALL_FALSE;                                                             \
  } while (0)

// Spacing factors of a tile (mesh spacings, their reciprocals and ratios),
// formed once per tile from the FP64 mesh arrays:
//   FP64 form on a power-of-two tile (kP2): exact exponent arithmetic on the
//     integer pipes (d_pow2_*), the same numbers as the IEEE expressions;
//   FP64 form otherwise: the IEEE expressions 1/h, c/(2e), 1/(h*h);
//   mixed form: FP32 arithmetic (IEEE division) on the spacings rounded to
//     FP32 on the integer pipes -- an FP64->FP32 conversion instruction, like
//     an FP64 division, occupies the FP64 pipe, and per tile these cost more
//     than the arithmetic of a still cell.
template <typename R>
__device__ __forceinline__ R geo_v(double h) { return Prec<R>::from_d(h); }
template <typename R, bool kP2>
__device__ __forceinline__ R geo_rcp(double h) {
  if constexpr (Prec<R>::kMixed) {
    return __frcp_rn(f64_to_f32(h));
  } else {
    return kP2 ? d_pow2_rcp(h) : 1.0 / h;
  }
}
template <typename R, bool kP2>
__device__ __forceinline__ R geo_half_ratio(double c, double e) {
  if constexpr (Prec<R>::kMixed) {
    return __fdiv_rn(f64_to_f32(c), 2.0f * f64_to_f32(e));
  } else {
    return kP2 ? d_pow2_half_ratio(c, e) : c / (2.0 * e);
  }
}
// h/2 in bulk precision (exact).
template <typename R>
__device__ __forceinline__ R geo_half(double h) { return Prec<R>::from_d(d_half(h)); }
// FP64 1/h for the coefficients of the FP64 conservative update: as geo_rcp
// in the FP64 form; the MUFU reciprocal with two Newton steps in the mixed
// form (whose fluxes are FP32).
template <typename R, bool kP2>
__device__ __forceinline__ double geo_rcp_d(double h) {
  if constexpr (Prec<R>::kMixed) {
    return kP2 ? d_pow2_rcp(h) : d_rcp(h);
  } else {
    return kP2 ? d_pow2_rcp(h) : 1.0 / h;
  }
}
// 1/(h*h), FP64 form only (CFL keys).
template <bool kP2>
__device__ __forceinline__ double geo_rcp_sq(double h) {
  return kP2 ? d_pow2_rcp_sq(h) : 1.0 / (h * h);
}

// The FP64 quotient as a called function: a branch around five inline FP64
// instructions is turned into predicated code, which occupies the FP64 pipe
// even in lanes (and whole warps) that skip it; a call is a real branch.
static __device__ __noinline__ double face_quotient(double n, double d) { return d_div(n, d); }

// Face velocity momentum / face density (0 where the face density is 0, as
// the reference sets it); a face without momentum keeps it (0 / rho = 0).
template <typename R>
__device__ __forceinline__ R face_velocity(R mom, R rbar) {
  using Pr = Prec<R>;
  if (Pr::is_zero(rbar)) return R(0);
  if (Pr::zero_skip(mom)) return mom;
  if constexpr (Pr::kMixed) {
    return Pr::div(mom, rbar);
  } else {
    return face_quotient(mom, rbar);
  }
}

// Volume-weighted face value a*wa + b*wb, rounded once after the product
// b*wb (the reference's a*wa + b*wb contracted as in the fused kernels).  On
// power-of-two meshes both weights are powers of two, both products exact
// exponent adds, and the single rounding is that of the sum.
template <typename R, bool kP2>
__device__ __forceinline__ R face_average(R a, R wa, R b, R wb) {
  if constexpr (kP2 && !Prec<R>::kMixed) {
    return Prec<R>::template mulp<true>(a, wa) + Prec<R>::template mulp<true>(b, wb);
  } else {
    return fma(a, wa, b * wb);
  }
}

// ===========================================================================
// Lagrangian phase.

// Pressure (EOS on the fly) -> face momenta -> velocities.  Covers every cell
// (the FP64 form stores P for ghosts too, as equation_of_state does; the
// shock-heating kernel reads it where a cell is compressed) and every interior
// x/y face.  The reference's rho_old copy is not made: the first mass sweep
// reads the density itself.  omp3/flow.c:55-70, 110-158.
template <typename R, bool kP2, bool kFl>
__device__ __forceinline__ void tile_lag_pressure_impl(const StepArgs<R>& a, int bx, int by) {
  using Pr = Prec<R>;
  __shared__ R sP[kCols + 1], sR[kCols + 1];
  __shared__ R s_ey[kMaxRows], s_iey[kMaxRows], s_wy0[kMaxRows], s_wy1[kMaxRows];
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int t = threadIdx.x;
  const int jj = bx * kCols + t;
  const int i0 = by * a.rows;
  const bool edge = tile_near_edge(nx, ny, pad, bx * kCols, i0, a.rows);
  const R g1 = R(kG1);
  if (t < a.rows) {
    const int ii = i0 + t;
    if (ii >= 1 && ii < ny) {
      const double ey = a.edgedy[ii];
      s_ey[t] = geo_v<R>(ey);
      s_iey[t] = geo_rcp<R, kP2>(ey);
      s_wy0[t] = geo_half_ratio<R, kP2>(a.celldy[ii], ey);
      s_wy1[t] = geo_half_ratio<R, kP2>(a.celldy[ii - 1], ey);
    }
  }
  R exr = R(0), iex = R(0), wx0 = R(0), wx1 = R(0);
  if (jj >= 1 && jj < nx) {
    const double ex = a.edgedx[jj];
    exr = geo_v<R>(ex);
    iex = geo_rcp<R, kP2>(ex);
    wx0 = geo_half_ratio<R, kP2>(a.celldx[jj], ex);
    wx1 = geo_half_ratio<R, kP2>(a.celldx[jj - 1], ex);
  }
  const R dt = Pr::from_d(a.dt);
  R P_dn = R(0), r_dn = R(0);  // cell (ii-1, jj)
  if (i0 >= 1 && jj < nx) {
    const size_t c = cidx(nx, i0 - 1, jj);
    r_dn = a.rho_r[c];
    P_dn = g1 * r_dn * a.e_r[c];
  }
  __syncthreads();
  // Row ii+1's densities, energies and face momenta are loaded before row ii
  // is processed (its stores do not touch them).
  const bool u_col = jj >= pad && jj < nx + 1 - pad;
  const bool v_col = jj >= pad && jj < nx - pad;
  R rc_n = R(0), ec_n = R(0), rl_n = R(0), el_n = R(0), mu_n = R(0), mv_n = R(0);
  auto load = [&](int ii) {
    if (jj < nx) {
      const size_t c = cidx(nx, ii, jj);
      rc_n = a.rho_r[c];
      ec_n = a.e_r[c];
    }
    if (t == 0 && jj >= 1 && jj - 1 < nx) {
      const size_t c = cidx(nx, ii, jj - 1);
      rl_n = a.rho_r[c];
      el_n = a.e_r[c];
    }
    if (u_col && ii >= pad && ii < ny - pad) mu_n = a.rho_u[fidx(nx, ii, jj)];
    if (v_col && ii >= pad && ii < ny + 1 - pad) mv_n = a.rho_v[cidx(nx, ii, jj)];
  };
  if (i0 < ny) load(i0);
  for (int k = 0; k < a.rows; ++k) {
    const int ii = i0 + k;
    if (ii >= ny) break;
    const R rc_l = rc_n, ec_l = ec_n, rl_l = rl_n, el_l = el_n, mu_l = mu_n, mv_l = mv_n;
    if (k + 1 < a.rows && ii + 1 < ny) load(ii + 1);
    R Pc = R(0), rc = R(0);
    bool vnz = false;  // kFl: this lane stored a face velocity that is not +0
    if (jj < nx) {
      rc = rc_l;
      Pc = g1 * rc * ec_l;
      if (!Pr::kMixed) a.P[cidx(nx, ii, jj)] = double(Pc);
    }
    sP[t + 1] = Pc;
    sR[t + 1] = rc;
    if (t == 0) {
      R Pl = R(0), rl = R(0);
      if (jj >= 1 && jj - 1 < nx) {
        rl = rl_l;
        Pl = g1 * rl * el_l;
      }
      sP[0] = Pl;
      sR[0] = rl;
    }
    __syncthreads();
    if (ii >= pad && ii < ny - pad && jj >= pad && jj < nx + 1 - pad) {
      const size_t f = fidx(nx, ii, jj);
      const R Pl = sP[t], rl = sR[t];
      R mom = mu_l;
      R rbar;
      bool dmom = false;  // the momentum changes (kFl: flagged as moving)
      // FP64 form, power-of-two tile: a warp whose faces all have equal
      // pressures, densities and weights either side keeps its momenta
      // (dp = +0) and has the face density 2 (rc wx0) exactly, without FP64
      // instructions.
      if (kP2 && !Pr::kMixed &&
          warp_all(lane_same(Pc, Pl) && lane_same(rc, rl) && lane_same(wx0, wx1))) {
        rbar = Pr::twice(Pr::template mulp<true>(rc, wx0));
      } else {
        const R dp = Pc - Pl;
        if (!Pr::zero_skip_mem(dp)) {
          mom = Pr::template dsub<kP2>(mom, dt * dp, exr, iex);
          a.rho_u[f] = mom;
        }
        dmom = !Pr::is_zero(dp);
        rbar = face_average<R, kP2>(rc, wx0, rl, wx1);
      }
      const R vel = face_velocity(mom, rbar);
      a.u[f] = vel;
      mirror(edge, a.u, nx + 1, ny, pad, ii, jj, vel, true, false);
      vnz = dmom || !is_plus_zero(vel);
    }
    if (ii >= pad && ii < ny + 1 - pad && jj >= pad && jj < nx - pad) {
      const size_t c = cidx(nx, ii, jj);
      R mom = mv_l;
      R rbar;
      bool dmom = false;
      if (kP2 && !Pr::kMixed &&
          warp_all(lane_same(Pc, P_dn) && lane_same(rc, r_dn) && lane_same(s_wy0[k], s_wy1[k]))) {
        rbar = Pr::twice(Pr::template mulp<true>(rc, s_wy0[k]));
      } else {
        const R dp = Pc - P_dn;
        if (!Pr::zero_skip_mem(dp)) {
          mom = Pr::template dsub<kP2>(mom, dt * dp, s_ey[k], s_iey[k]);
          a.rho_v[c] = mom;
        }
        dmom = !Pr::is_zero(dp);
        rbar = face_average<R, kP2>(rc, s_wy0[k], r_dn, s_wy1[k]);
      }
      const R vel = face_velocity(mom, rbar);
      a.v[c] = vel;
      mirror(edge, a.v, nx, ny + 1, pad, ii, jj, vel, false, true);
      vnz = vnz || dmom || !is_plus_zero(vel);
    }
    if constexpr (kFl) {
      store_flag(a.vflag + (size_t)ii * a.vf_stride + (jj >> 5),
                 __any_sync(0xffffffffu, vnz) != 0);
    }
    P_dn = Pc;
    r_dn = rc;
    __syncthreads();
  }
}

template <typename R, bool kFl = false>
__device__ __forceinline__ void tile_lag_pressure(const StepArgs<R>& a, int bx, int by) {
  if constexpr (kFl) {
    // A tile whose cells (and the row above and column left it reads) were
    // at rest through the previous step: its pressures, momenta, velocities
    // (with their ghost images) and velocity flags are what that step's
    // pressure phase stored, from the same densities, energies and momenta,
    // and nothing has written them since -- this phase would store the same
    // numbers.
    const int c0 = bx * kCols, i0 = by * a.rows;
    if (a.rest && rest_cells(a, i0 - 1, i0 + a.rows, c0 - 1, c0 + kCols)) return;
  }
  FLOW_POW2_DISPATCH(R, a, bx * kCols, by * a.rows,
                     (tile_lag_pressure_impl<R, true, kFl>(a, bx, by)),
                     (tile_lag_pressure_impl<R, false, kFl>(a, bx, by)));
}

// Artificial viscous stresses on interior cells, omp3/flow.c:173-207.

// A zero stress as +0.  The mixed form, which takes no zero skip, forms a
// stress of a cell without compression as (-C_Q rho) (+0) (...) = -0; adding
// +0 makes it +0 (and changes no other value), so that the stress flags see
// it as zero.  The sign of a zero stress reaches no non-zero value.
template <typename R>
__device__ __forceinline__ R stress_sign0(R q) {
  if constexpr (Prec<R>::kMixed) {
    return q + R(0);
  } else {
    return q;
  }
}
// mid = w[0], hi = w[1]; lo = w[-1] and hi2 = w[2] are loaded only where
// the cell is compressed.
template <typename R>
__device__ __forceinline__ R visc_stress(R rho, const R* w, R mid, R hi) {
  using Pr = Prec<R>;
  // Equal velocities either side of every cell of the warp: hi - mid = +0,
  // no compression (the result below, without the FP64 instructions).
  if (warp_same(hi, mid)) return R(0);
  const R m1 = Pr::min0(hi - mid);
  if (Pr::zero_skip(m1)) return R(0);  // no compression across the cell
  const R m0 = Pr::min0(mid - w[-1]);
  const R m2 = Pr::min0(w[2] - hi);
  return stress_sign0(R(-kCQ) * rho * m1 * Pr::half(Pr::abs(m2 - m1) + Pr::abs(m1 - m0)));
}

// kFlags: a.qmask is set -- a warp row whose stresses are all +0 stores only
// its flag (the single-problem kernels; the batched kernels keep no flags).
template <typename R, bool kFlags = false>
__device__ __forceinline__ void tile_lag_viscosity(const StepArgs<R>& a, int bx, int by) {
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int jj = pad + bx * kCols + threadIdx.x;
  const int i0 = pad + by * a.rows;
  const bool edge = tile_near_edge(nx, ny, pad, pad + bx * kCols, i0, a.rows);
  using Pr = Prec<R>;
  const int i1 = min(i0 + a.rows, ny - pad);
  // kFlags: a tile whose face velocities (with the stencil's reach) are all
  // +0 loads none of them; its stresses are +0 and nothing is stored.
  bool vq = false;
  if constexpr (kFlags) {
    const int cb = pad + bx * kCols;
    vq = tile_vel_still(a, i0 - 3, i1 + 4, cb - 3, cb + kCols + 3);
  }
  // This warp's stress-flag byte of row i0, or null without flags.
  unsigned char* qf =
      kFlags ? reinterpret_cast<unsigned char*>(a.qmask + (size_t)(i0 - pad) * a.qm_stride + bx) +
                    (threadIdx.x >> 5)
              : nullptr;
  const int qf_step = 4 * a.qm_stride;
  if (jj >= nx - pad) {
    // A warp wholly right of the interior clears its flags (none are read,
    // but the viscous-acceleration tile's early exit looks at whole words).
    if (kFlags && (threadIdx.x & 31) == 0) {
      for (int ii = i0; ii < i1; ++ii, qf += qf_step) store_flag(qf, false);
    }
    return;
  }
  if (kFlags && vq) {
    // A tile at rest: every stress is +0; only the flags are written.
    for (int ii = i0; ii < i1; ++ii, qf += qf_step) store_flag(qf, false);
    return;
  }
  // The y stress of row ii uses the limited jumps m0, m1, m2 of v around the
  // cell and |m1 - m0|, |m2 - m1|; the next row reuses three of those, so
  // they are carried down the column (same operands, same values).
  const R vm = vq ? R(0) : a.v[cidx(nx, i0 - 1, jj)];
  const R v0 = vq ? R(0) : a.v[cidx(nx, i0, jj)];
  R vp = vq ? R(0) : a.v[cidx(nx, i0 + 1, jj)];
  R m0 = Pr::min0(v0 - vm), m1 = Pr::min0(vp - v0);
  R g01 = Pr::abs(m1 - m0);
  // Row ii+1's v, density and face velocities are loaded before row ii is
  // processed.
  R vp2_n = R(0), rho_n = R(0), um_n = R(0), up_n = R(0);
  auto load = [&](int ii) {
    if (vq) return;
    const size_t f = fidx(nx, ii, jj);
    vp2_n = a.v[cidx(nx, ii + 2, jj)];
    rho_n = a.rho_r[cidx(nx, ii, jj)];
    um_n = a.u[f];
    up_n = a.u[f + 1];
  };
  if (i0 < i1) load(i0);
  for (int ii = i0; ii < i1; ++ii) {
    const R vp2 = vp2_n, rho = rho_n, um = um_n, up = up_n;
    if (ii + 1 < i1) load(ii + 1);
    const size_t f = fidx(nx, ii, jj);
    const size_t c = cidx(nx, ii, jj);
    const R qx = vq ? R(0) : visc_stress(rho, a.u + f, um, up);
    R m2, g12, qy;
    if (!Pr::kMixed && warp_all(lane_same(vp2, vp) && Pr::is_zero(m1))) {
      // No jump of v across the cell or above it anywhere in the warp:
      // m2 = min0(+0) = +0, g12 = |+0 - m1| = +0, no stress.
      m2 = R(0);
      g12 = R(0);
      qy = R(0);
    } else {
      m2 = Pr::min0(vp2 - vp);
      g12 = Pr::abs(m2 - m1);
      qy = Pr::zero_skip(m1) ? R(0) : stress_sign0(R(-kCQ) * rho * m1 * Pr::half(g12 + g01));
    }
    // With flags, a warp row whose stresses are all +0 (the still regions)
    // stores none of them, only its flag.
    bool store = true;
    if constexpr (kFlags) {
      store = __any_sync(__activemask(), !(is_plus_zero(qx) && is_plus_zero(qy)));
      store_flag(qf, store);
      qf += qf_step;
    }
    if (store) {
      a.Qxx[c] = qx;
      a.Qyy[c] = qy;
      mirror(edge, a.Qxx, nx, ny, pad, ii, jj, qx, false, false);
      mirror(edge, a.Qyy, nx, ny, pad, ii, jj, qy, false, false);
    }
    m0 = m1;
    m1 = m2;
    g01 = g12;
    vp = vp2;
  }
}

// Viscous acceleration of the face momenta and velocities,
// omp3/flow.c:212-244.  The face densities are formed again where needed.
// kEarly: the stresses stream through a ring of asynchronous copies (off in
// the persistent batched kernel, whose register budget is spent across all
// its phases).  With stress flags, a tile none of whose stresses can be
// non-zero returns at once, and a stress flagged +0 is not loaded.
template <typename R, bool kP2, bool kEarly, bool kFlags>
__device__ __forceinline__ void tile_lag_viscous_accel_impl(const StepArgs<R>& a, int bx, int by) {
  using Pr = Prec<R>;
  __shared__ R s_cy[kMaxRows], s_icy[kMaxRows], s_wy0[kMaxRows], s_wy1[kMaxRows];
  // Stress flags (a.qmask) of rows i0 - 1 .. i1 - 1, each row taken at its
  // mirror source: the words of column tiles bx - 1 and bx.
  __shared__ unsigned s_qf[kMaxRows + 1][2];
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int jj = pad + bx * kCols + threadIdx.x;
  const int i0 = pad + by * a.rows;
  const bool edge = tile_near_edge(nx, ny, pad, pad + bx * kCols, i0, a.rows);
  if (threadIdx.x < a.rows) {
    const int ii = i0 + threadIdx.x;
    if (ii < ny) {
      s_cy[threadIdx.x] = geo_v<R>(a.celldy[ii]);
      s_icy[threadIdx.x] = geo_rcp<R, kP2>(a.celldy[ii]);
      s_wy0[threadIdx.x] = geo_half_ratio<R, kP2>(a.celldy[ii], a.edgedy[ii]);
      s_wy1[threadIdx.x] = geo_half_ratio<R, kP2>(a.celldy[ii - 1], a.edgedy[ii]);
    }
  }
  const bool col_ok = jj < nx + 1 - pad;
  const int i1 = min(i0 + a.rows, ny + 1 - pad);
  // Whether any stress this tile reads may be non-zero (block-uniform).
  bool any_q = true;
  // The flag of a stress, taken at the mirror source of its cell.
  auto src_row = [&](int r) {
    return r < pad ? 2 * pad - 1 - r : (r >= ny - pad ? 2 * (ny - pad) - 1 - r : r);
  };
  auto src_col = [&](int c) {
    return c < pad ? 2 * pad - 1 - c : (c >= nx - pad ? 2 * (nx - pad) - 1 - c : c);
  };
  if constexpr (kFlags) {
    unsigned w0 = 0u, w1 = 0u;
    const int k = threadIdx.x;
    if (k <= i1 - i0) {
      const unsigned* row = a.qmask + (size_t)(src_row(i0 - 1 + k) - pad) * a.qm_stride;
      w0 = bx >= 1 ? row[bx - 1] : 0u;
      w1 = bx < a.qm_stride ? row[bx] : 0u;
      s_qf[k][0] = w0;
      s_qf[k][1] = w1;
    }
    // Tile bx reads the flags of its own groups and the last group of tile
    // bx - 1 (the stress left of its first face).  (The barrier also
    // publishes the row tables.)
    any_q = __syncthreads_or((w1 | (w0 & 0xff000000u)) != 0u) != 0;
  } else {
    __syncthreads();
  }
  auto flag_x = [&](int ii, int col) {  // Qxx(ii, col), ii an interior row
    return !kFlags || qflag(s_qf[ii - i0 + 1][0], s_qf[ii - i0 + 1][1], src_col(col), pad, bx);
  };
  auto flag_y = [&](int ii) {  // Qyy(ii, jj), ii in i0 - 1 .. i1 - 1
    return !kFlags || qflag(s_qf[ii - i0 + 1][0], s_qf[ii - i0 + 1][1], jj, pad, bx);
  };
  // kEarly (the fused kernel): the stresses stream through a shared-memory
  // ring, below.  Otherwise (the batched kernel) row ii+1's are loaded into
  // registers before row ii is processed.
  R q1_n = R(0), q0_n = R(0), qy_n = R(0), qy_dn = R(0);
  auto load = [&](int ii) {
    const size_t c = cidx(nx, ii, jj);
    if (ii < ny - pad) {
      q1_n = flag_x(ii, jj) ? a.Qxx[c] : R(0);
      q0_n = flag_x(ii, jj - 1) ? a.Qxx[c - 1] : R(0);
    }
    if (jj < nx - pad) qy_n = flag_y(ii) ? a.Qyy[c] : R(0);
  };
  auto prime = [&]() {
    if (jj < nx - pad && flag_y(i0 - 1)) qy_dn = a.Qyy[cidx(nx, i0 - 1, jj)];
    if (!kEarly && i0 < i1) load(i0);
  };
  // No stress gradient anywhere in the tile: momenta and velocities stand.
  if (!any_q || !col_ok) return;
  if (kEarly) prime();
  const R cx = geo_v<R>(a.celldx[jj]);
  const R icx = geo_rcp<R, kP2>(a.celldx[jj]);
  // Face-density weights (the pressure phase's): where a stress gradient
  // changes a face's momentum, the face density is formed again from the two
  // cell densities -- the same expression on the same values, so the same
  // number -- rather than stored for every face by the pressure phase.
  const R wx0 = geo_half_ratio<R, kP2>(a.celldx[jj], a.edgedx[jj]);
  const R wx1 = geo_half_ratio<R, kP2>(a.celldx[jj - 1], a.edgedx[jj]);
  const R dt = Pr::from_d(a.dt);
  if (!kEarly) prime();
  auto row = [&](int ii, R q1, R q0, R qy) {
    const int k = ii - i0;
    if (ii < ny - pad) {
      const size_t f = fidx(nx, ii, jj);
      // No stress gradient: the momentum and the velocity from the pressure
      // phase stand as they are.
      if (!warp_same(q1, q0)) {  // equal stresses in the whole warp: dqx = +0
        const R dqx = q1 - q0;
        if (!Pr::zero_skip_mem(dqx)) {
          const R mom = Pr::template dsub<kP2>(a.rho_u[f], dt * dqx, cx, icx);
          const size_t c = cidx(nx, ii, jj);
          const R vel =
              face_velocity(mom, face_average<R, kP2>(a.rho_r[c], wx0, a.rho_r[c - 1], wx1));
          a.rho_u[f] = mom;
          a.u[f] = vel;
          mirror(edge, a.u, nx + 1, ny, pad, ii, jj, vel, true, false);
          if constexpr (kFlags) store_flag(a.vflag + (size_t)ii * a.vf_stride + (jj >> 5), true);
        }
      }
    }
    if (jj < nx - pad) {
      const size_t c = cidx(nx, ii, jj);
      if (!warp_same(qy, qy_dn)) {
        const R dqy = qy - qy_dn;
        if (!Pr::zero_skip_mem(dqy)) {
          const R mom = Pr::template dsub<kP2>(a.rho_v[c], dt * dqy, s_cy[k], s_icy[k]);
          const R vel = face_velocity(
              mom, face_average<R, kP2>(a.rho_r[c], s_wy0[k], a.rho_r[c - nx], s_wy1[k]));
          a.rho_v[c] = mom;
          a.v[c] = vel;
          mirror(edge, a.v, nx, ny + 1, pad, ii, jj, vel, false, true);
          if constexpr (kFlags) store_flag(a.vflag + (size_t)ii * a.vf_stride + (jj >> 5), true);
        }
      }
      qy_dn = qy;
    }
  };
  if constexpr (kEarly) {
    // The stresses of rows ii+1 .. ii+kAhead are in flight while row ii is
    // processed: each thread copies its own column's values into a ring of
    // shared-memory slots (no registers held for them, no barrier), one copy
    // group per row.  kAhead + 1 slots: a row's slot is refilled one row
    // after it was read.
    constexpr int kAhead = Pr::kMixed ? 2 : 3, kSlots = kAhead + 1;
    auto s_q = ring_slots<R, kSlots, 3, kCols, 1>();
    const int t = threadIdx.x;
    auto issue = [&](int ii) {
      const int sl = (ii - i0) % kSlots;
      const size_t c = cidx(nx, ii, jj);
      const bool xq = ii < ny - pad, yq = jj < nx - pad;
      const bool x1 = xq && flag_x(ii, jj), x0 = xq && flag_x(ii, jj - 1);
      const bool y0 = yq && flag_y(ii);
      cp_async_elem(&s_q[sl][0][t], x1 ? a.Qxx + c : a.Qxx, x1);
      cp_async_elem(&s_q[sl][1][t], x0 ? a.Qxx + c - 1 : a.Qxx, x0);
      cp_async_elem(&s_q[sl][2][t], y0 ? a.Qyy + c : a.Qyy, y0);
    };
#pragma unroll
    for (int d = 0; d < kAhead; ++d) {
      if (i0 + d < i1) issue(i0 + d);
      cp_async_commit();
    }
    for (int ii = i0; ii < i1; ++ii) {
      cp_async_wait<kAhead - 1>();  // row ii's group has landed
      const int sl = (ii - i0) % kSlots;
      const R q1 = s_q[sl][0][t], q0 = s_q[sl][1][t], qy = s_q[sl][2][t];
      if (ii + kAhead < i1) issue(ii + kAhead);
      cp_async_commit();
      row(ii, q1, q0, qy);
    }
    cp_async_wait<0>();
  } else {
    for (int ii = i0; ii < i1; ++ii) {
      const R q1 = q1_n, q0 = q0_n, qy = qy_n;
      if (ii + 1 < i1) load(ii + 1);
      row(ii, q1, q0, qy);
    }
  }
}

template <typename R, bool kEarly = true, bool kFlags = false>
__device__ __forceinline__ void tile_lag_viscous_accel(const StepArgs<R>& a, int bx, int by) {
  FLOW_POW2_DISPATCH(R, a, a.pad + bx * kCols, a.pad + by * a.rows,
                     (tile_lag_viscous_accel_impl<R, true, kEarly, kFlags>(a, bx, by)),
                     (tile_lag_viscous_accel_impl<R, false, kEarly, kFlags>(a, bx, by)));
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long y = __shfl_xor_sync(0xffffffffu, x, o);
    x = (y < x) ? y : x;
  }
  return x;
}

// Shock heating and work (omp3/flow.c:248-290) fused with the CFL minimum of
// set_timestep (omp3/flow.c:73-106) on the updated energy.  One atomicMin per
// block on the FP64 bit pattern of its smallest candidate; the last block to
// finish applies the leapfrog dt/dt_h rule (finish_dt).  In the mixed form
// the FP32 energy change is added to the FP64 energy.
template <typename R, bool kP2, bool kRing, bool kFlags>
__device__ __forceinline__ void tile_lag_energy_dt_impl(const StepArgs<R>& a, int bx, int by,
                                                        unsigned long long* tile_min) {
  using Pr = Prec<R>;
  __shared__ R s_icy[kMaxRows], s_cy[kMaxRows];
  __shared__ double s_icy2[kMaxRows];
  __shared__ unsigned long long s_warp[kCols / 32];
  __shared__ unsigned s_qf[kMaxRows];  // stress-flag words of the tile's rows
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int jj = pad + bx * kCols + threadIdx.x;
  const int i0 = pad + by * a.rows;
  const bool edge = tile_near_edge(nx, ny, pad, pad + bx * kCols, i0, a.rows);
  if (threadIdx.x < a.rows) {
    const int ii = i0 + threadIdx.x;
    if (ii < ny) {
      s_cy[threadIdx.x] = geo_v<R>(a.celldy[ii]);
      s_icy[threadIdx.x] = geo_rcp<R, kP2>(a.celldy[ii]);
      if constexpr (!Pr::kMixed) s_icy2[threadIdx.x] = geo_rcp_sq<kP2>(a.celldy[ii]);
    }
    if (kFlags && ii < ny - pad) s_qf[threadIdx.x] = a.qmask[(size_t)(ii - pad) * a.qm_stride + bx];
  }
  __syncthreads();
  // kFlags: a tile whose face velocities are all +0 (velocity flags) loads
  // none of them: its cells are still, and take the still path on +0 values.
  bool vq = false;
  if constexpr (kFlags) {
    const int cb = pad + bx * kCols;
    vq = tile_vel_still(a, i0 - 2, min(i0 + a.rows, ny - pad) + 2, cb - 2, cb + kCols + 2);
  }
  // Whether the stresses of this thread's warp in tile row k may be non-zero
  // (flagged +0: not loaded, taken as +0).
  auto qflag_row = [&](int k) {
    return !kFlags || ((s_qf[k] >> (8 * (threadIdx.x >> 5))) & 0xffu) != 0u;
  };
  unsigned long long best = ~0ull;
  // FP64 form: the thread's largest 1/dt^2 key so far, with its S and spacing.
  long long kbest = -1;
  double s_best = 0.0, c_best = 0.0;
  if (jj < nx - pad) {
    const R cx = geo_v<R>(a.celldx[jj]);
    const R icx = geo_rcp<R, kP2>(a.celldx[jj]);
    const double icx2 = Pr::kMixed ? 0.0 : geo_rcp_sq<kP2>(a.celldx[jj]);
    const R dt_h = Pr::from_d(a.dt_h);
    const int i1 = min(i0 + a.rows, ny - pad);
    R v0 = vq ? R(0) : a.v[cidx(nx, i0, jj)];
    // Mixed form: row ii+1's inputs are loaded before row ii is processed.
    // The FP64 form (at 64 registers without that, which loses more
    // occupancy than it gains) streams them through a per-thread ring of
    // asynchronous copies instead when kRing (the fused kernel), kEAhead rows
    // ahead (seven planes: three rows ahead, 30 KB of shared memory per CTA,
    // cost more in the overlap between kernels than it hid).  The FP64
    // pressure is read only where a cell is compressed.
    constexpr bool kAhead = Pr::kMixed;
    constexpr bool kERing = kRing && !Pr::kMixed;
    constexpr int kEAhead = 2, kESlots = kEAhead + 1;
    auto s_in = ring_slots<R, kERing ? kESlots : 1, 7, kERing ? kCols : 1, 9>();
    const int t = threadIdx.x;
    R v1_n = R(0), r_n = R(0), er_n = R(0), qx_n = R(0), qy_n = R(0), u0_n = R(0), u1_n = R(0);
    auto load = [&](int ii) {
      const size_t c = cidx(nx, ii, jj);
      const size_t f = c + (size_t)ii;  // fidx(nx, ii, jj)
      v1_n = vq ? R(0) : a.v[c + nx];
      r_n = a.rho_r[c];
      er_n = a.e_r[c];
      const bool qf = qflag_row(ii - i0);
      qx_n = qf ? a.Qxx[c] : R(0);
      qy_n = qf ? a.Qyy[c] : R(0);
      u0_n = vq ? R(0) : a.u[f];
      u1_n = vq ? R(0) : a.u[f + 1];
    };
    auto issue = [&](int ii) {
      const int sl = (ii - i0) % kESlots;
      const size_t c = cidx(nx, ii, jj);
      const size_t f = c + (size_t)ii;  // fidx(nx, ii, jj)
      cp_async_elem(&s_in[sl][0][t], a.v + c + nx, !vq);
      cp_async_elem(&s_in[sl][1][t], a.rho_r + c, true);
      cp_async_elem(&s_in[sl][2][t], a.e_r + c, true);
      const bool qf = qflag_row(ii - i0);
      cp_async_elem(&s_in[sl][3][t], a.Qxx + c, qf);
      cp_async_elem(&s_in[sl][4][t], a.Qyy + c, qf);
      cp_async_elem(&s_in[sl][5][t], a.u + f, !vq);
      cp_async_elem(&s_in[sl][6][t], a.u + f + 1, !vq);
    };
    // The CFL candidates of the cell in tile row k from S = c_s^2 + 2 Q / rho
    // along x and y (e_neg: its energy is negative).
    auto cfl_candidates = [&](int k, R sx, R sy, bool e_neg) {
      if constexpr (Pr::kMixed) {
        const unsigned long long mx = (unsigned long long)dbits(Pr::to_d(cx * Pr::rsqrt(sx)));
        const unsigned long long my =
            (unsigned long long)dbits(Pr::to_d(s_cy[k] * Pr::rsqrt(sy)));
        const unsigned long long m = (mx < my) ? mx : my;
        best = (!e_neg && m < best) ? m : best;
      } else {
        // Rank the candidates by the key S / h^2 = 1/dt^2 (the largest key
        // is the smallest dt) and take the square root only for the
        // thread's winner after the loop.  Keys in [+0, +inf] only: a
        // negative or NaN S is a NaN candidate in the reference.
        const long long kx = e_neg ? -1 : dbits(Prec<double>::mulp<kP2>(sx, icx2));
        const long long ky = e_neg ? -1 : dbits(Prec<double>::mulp<kP2>(sy, s_icy2[k]));
        if (kx >= 0 && kx <= 0x7ff0000000000000LL && kx > kbest) {
          kbest = kx;
          s_best = sx;
          c_best = cx;
        }
        if (ky >= 0 && ky <= 0x7ff0000000000000LL && ky > kbest) {
          kbest = ky;
          s_best = sy;
          c_best = s_cy[k];
        }
      }
    };
    if (!vq) {
    if constexpr (kERing) {
#pragma unroll
      for (int d = 0; d < kEAhead; ++d) {
        if (i0 + d < i1) issue(i0 + d);
        cp_async_commit();
      }
    }
    if (kAhead && i0 < i1) load(i0);
    for (int ii = i0; ii < i1; ++ii) {
      const int k = ii - i0;
      const size_t c = cidx(nx, ii, jj);
      if constexpr (kERing) {
        cp_async_wait<kEAhead - 1>();  // row ii's group has landed
        const int sl = k % kESlots;
        v1_n = s_in[sl][0][t];
        r_n = s_in[sl][1][t];
        er_n = s_in[sl][2][t];
        qx_n = s_in[sl][3][t];
        qy_n = s_in[sl][4][t];
        u0_n = s_in[sl][5][t];
        u1_n = s_in[sl][6][t];
        if (ii + kEAhead < i1) issue(ii + kEAhead);
        cp_async_commit();
      } else if (!kAhead) {
        load(ii);
      }
      const R v1 = v1_n, r = r_n, er = er_n, qx = qx_n, qy = qy_n, u0f = u0_n, u1f = u1_n;
      if (kAhead && ii + 1 < i1) load(ii + 1);
      const bool rz = Pr::is_zero(r);
      // A cell whose faces do not move relative to each other does no work
      // and takes no shock heating: every increment below is a zero, so e is
      // left as it is (a cell at rest, or in uniform translation).  In the
      // FP64 form a warp whose cells all have equal opposite face velocities
      // (dudx = dvdy = +0) takes this without forming the differences.
      R inv_r = R(0);
      double e_new;
      bool still;
      if (!Pr::kMixed && warp_all(lane_same(u1f, u0f) && lane_same(v1, v0))) {
        still = true;
        e_new = rz ? 0.0 : double(er);
      } else {
        const R dudx = Pr::template mulp<kP2>(u1f - u0f, icx);
        const R dvdy = Pr::template mulp<kP2>(v1 - v0, s_icy[k]);
        still = Pr::zero_skip_coarse(dudx) && Pr::zero_skip_coarse(dvdy);
        if (still) {
          // (Mixed form: the FP64 energy is not needed, as it is kept.)
          e_new = rz ? 0.0 : (Pr::kMixed ? 0.0 : double(er));
        } else {
          const R p = Pr::kMixed ? R(kG1) * r * er : R(a.P[c]);
          inv_r = rz ? R(0) : Pr::rcp(r);
          const R div_dt = (dudx + dvdy) * dt_h;
          // e_q = e - dt_h (Qxx dudx + Qyy dvdy) / rho, kept as an increment.
          const R dq = -(dt_h * fma(qx, dudx, qy * dvdy)) * inv_r;
          const R e_q = er + dq;
          const R rho_c = r * Pr::rcp(R(1) + div_dt);
          const R e_c = fma(-(p * div_dt), inv_r, e_q);
          const R work = Pr::half(div_dt) * fma(R(kG1) * e_c, rho_c, p) * inv_r;
          if (Pr::kMixed) {
            e_new = rz ? 0.0 : a.e[c] + Pr::to_d(dq - work);
          } else {
            e_new = rz ? 0.0 : double(e_q - work);
          }
        }
      }
      // A still cell with mass keeps its energy: e, its bulk shadow and their
      // ghost images already hold it, so nothing is stored.
      const bool keep = still && !rz;
      if (!keep) store_cell(edge, a.e, a.e_r, nx, ny, pad, ii, jj, e_new);
      // CFL: celldx / sqrt(c_s^2 + 2 Q / rho) with c_s^2 = gamma (gamma-1) e.
      // The reference squares c_s = sqrt(gamma (gamma-1) e), so a cell whose
      // energy went negative gives a NaN candidate whatever Q is, and its dt
      // is then the minimum over the other cells (the 4096^2 known-answer
      // problem does this on its first step, which runs at Courant ~0.9).
      // Skip such cells rather than use gamma (gamma-1) e + 2Q/rho directly.
      const R e_nr = keep ? er : Pr::from_d(e_new);
      const R s2 = R(kGam * (kGam - 1.0)) * e_nr;
      R sx = s2, sy = s2;  // + 2 Q / rho, zero without viscous stress
      if (!Pr::zero_skip_coarse(qx) || !Pr::zero_skip_coarse(qy)) {
        if (still) inv_r = rz ? R(0) : Pr::rcp(r);
        const R two_inv_r = Pr::twice(inv_r);
        sx = fma(qx, two_inv_r, s2);
        sy = fma(qy, two_inv_r, s2);
      }
      const bool e_neg = Pr::kMixed ? (e_nr < R(0)) : d_lt0(e_new);
      cfl_candidates(k, sx, sy, e_neg);
      v0 = v1;
    }
    if constexpr (kERing) cp_async_wait<0>();
    } else {
      // A tile at rest (velocity flags): every cell takes the still path
      // above on +0 velocities, with no viscous stress -- the energy stays
      // (a cell without mass takes 0) and the CFL candidates come from the
      // energy alone -- reading only the density and energy, four rows in
      // flight together, without the copy ring.
      constexpr int kB = 4;
      for (int ib = i0; ib < i1; ib += kB) {
        R rv[kB], ev[kB];
#pragma unroll
        for (int q = 0; q < kB; ++q) {
          const bool in = ib + q < i1;
          const size_t c = cidx(nx, in ? ib + q : i0, jj);
          rv[q] = in ? a.rho_r[c] : R(0);
          ev[q] = in ? a.e_r[c] : R(0);
        }
#pragma unroll
        for (int q = 0; q < kB; ++q) {
          const int ii = ib + q;
          if (ii < i1) {
            const bool rz = Pr::is_zero(rv[q]);
            if (rz) store_cell(edge, a.e, a.e_r, nx, ny, pad, ii, jj, 0.0);
            const R e_nr = rz ? Pr::from_d(0.0) : ev[q];
            const R s2 = R(kGam * (kGam - 1.0)) * e_nr;
            const bool e_neg = Pr::kMixed ? (e_nr < R(0)) : d_lt0(rz ? 0.0 : double(ev[q]));
            cfl_candidates(ii - i0, s2, s2, e_neg);
          }
        }
      }
    }
  }
  if (!Pr::kMixed && kbest >= 0) best = (unsigned long long)dbits(c_best * d_rsqrt(s_best));
  best = warp_min_u64(best);
  if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = best;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long b = s_warp[0];
    for (int w = 1; w < kCols / 32; ++w) b = (s_warp[w] < b) ? s_warp[w] : b;
    atomicMin(a.min_slot, b);
    if (tile_min) *tile_min = b;
  }
}

// tile_min: where thread 0 also stores the tile's CFL minimum, or null.
template <typename R, bool kRing = true, bool kFlags = false>
__device__ __forceinline__ void tile_lag_energy_dt(const StepArgs<R>& a, int bx, int by,
                                                   unsigned long long* tile_min = nullptr) {
  if constexpr (kFlags) {
    // A tile at rest now (velocity flags) whose cells were at rest through
    // the previous step: it keeps every energy, has no viscous stress, and
    // its cells' CFL candidates are those of the previous step, from the
    // same densities and energies -- its minimum then stands.
    if (a.rest && a.cfl_tile) {
      const int nx = a.nx, ny = a.ny, pad = a.pad;
      const int cb = pad + bx * kCols, i0 = pad + by * a.rows;
      const int i1 = min(i0 + a.rows, ny - pad);
      if (tile_vel_still(a, i0 - 2, i1 + 2, cb - 2, cb + kCols + 2) &&
          rest_cells(a, i0, i1, cb, min(cb + kCols, nx - pad))) {
        if (threadIdx.x == 0) {
          const unsigned long long b = a.cfl_tile[(size_t)by * a.qm_stride + bx];
          atomicMin(a.min_slot, b);
          if (tile_min) *tile_min = b;
        }
        return;
      }
    }
  }
  FLOW_POW2_DISPATCH(R, a, a.pad + bx * kCols, a.pad + by * a.rows,
                     (tile_lag_energy_dt_impl<R, true, kRing, kFlags>(a, bx, by, tile_min)),
                     (tile_lag_energy_dt_impl<R, false, kRing, kFlags>(a, bx, by, tile_min)));
}

// The leapfrog dt/dt_h rule of omp3/flow.c:103-105 applied to the finished
// CFL minimum, in FP64 without contraction; resets the minimum slot.
template <typename R>
__device__ __forceinline__ void finish_dt(const StepArgs<R>& a) {
  const unsigned long long g = atomicExch(a.min_slot, ~0ull);
  const double cfl = d_min_pos(a.max_dt, dfrom((long long)g));
  const double limited = dmin(cfl, __dmul_rn(FLOW_C_M, a.dt_h));
  const double dt = __dmul_rn(0.5, __dadd_rn(__dmul_rn(kCT, limited), a.dt_h));
  a.dt_slot[0] = dt;
  a.dt_slot[1] = a.first_step ? dt : __dmul_rn(kCT, limited);
}

// ===========================================================================
// Advection of mass and energy (omp3/flow.c:293-554).

// Second-order upwind interpolation with the MC-limited slope from the four
// values straddling the point (m2, m1 | p0, p1), for the branch chosen by
// the wind sign: pos reconstructs from the left, base m1 + 0.5*m*(h - w*dt_h)
// from the differences (da, db, dc) = (p0-m2, m1-m2, p0-m1); otherwise from
// the right, base p0 - 0.5*m*(h + w*dt_h) from (p1-m1, p0-m1, p1-p0).
// The slope minmod(0.5 da/h', 2 db/h', 2 dc/h') is formed as
// minmod(0.5 da, 2 db, 2 dc) times inv_h = 1/h' > 0: scaling by a positive
// factor keeps the selection (rounding is monotonic, and arguments that round
// to a tie give the same value), so the result is the same number with one
// multiplication instead of three; halving, doubling and negation are exact
// integer operations.  A zero slope (flat or extremal data) leaves the base
// value, and the reconstruction arithmetic is skipped.
template <typename R, bool kP2>
__device__ __forceinline__ R mc_reconstruct(bool pos, R da, R db, R dc, R base, R inv_h, R h,
                                            R wdt) {
  using Pr = Prec<R>;
  const R m0 = Pr::minmod(Pr::minmod(Pr::half(da), Pr::twice(db)), Pr::twice(dc));
  if (Pr::zero_skip(m0)) return base;
  const R mm = Pr::template mulp<kP2>(m0, inv_h);
  const R w = h + (pos ? Pr::neg(wdt) : wdt);
  const R hm = Pr::half(pos ? mm : Pr::neg(mm));
  return Pr::madd(hm, w, base);
}

// The same from the four values themselves, selecting the operands before
// subtracting so that each difference is one FP64 instruction.
template <typename R, bool kP2>
__device__ __forceinline__ R mc_face(bool pos, R m2, R m1, R p0, R p1, R inv_h, R h, R wdt) {
  const R a0 = pos ? p0 : p1;
  const R a1 = pos ? m2 : m1;
  const R base = pos ? m1 : p0;
  return mc_reconstruct<R, kP2>(pos, a0 - a1, base - a1, a0 - base, base, inv_h, h, wdt);
}

// Four consecutive values of a column (m2, m1, p0, p1) with their one-step
// differences d1 = m1-m2, d2 = p0-m1, d3 = p1-p0 and two-step differences
// D1 = p0-m2, D2 = p1-m1.  A tile marching down the column shifts the window
// by one value per row and forms only the two new differences (the others
// are the same operands as before, so the same values).
// push/refresh: shift the values alone and form all the differences later
// (a tile that skips the rows where nothing moves).
template <typename R>
struct ColWindow {
  R m2, m1, p0, p1, d1, d2, d3, D1, D2;
  __device__ __forceinline__ void init(R m2_, R m1_, R p0_, R p1_) {
    m2 = m2_; m1 = m1_; p0 = p0_; p1 = p1_;
    refresh();
  }
  __device__ __forceinline__ void refresh() {
    d1 = m1 - m2; d2 = p0 - m1; d3 = p1 - p0;
    D1 = p0 - m2; D2 = p1 - m1;
  }
  __device__ __forceinline__ void push(R next) {
    m2 = m1; m1 = p0; p0 = p1; p1 = next;
  }
  __device__ __forceinline__ void shift(R next) {
    const R D2n = next - p0, d3n = next - p1;
    m2 = m1; m1 = p0; p0 = p1; p1 = next;
    d1 = d2; d2 = d3; d3 = d3n;
    D1 = D2; D2 = D2n;
  }
  // After a push: the differences shift's would have given, from those of
  // the window one row before (same operands, same values).
  __device__ __forceinline__ void advance() {
    d1 = d2; d2 = d3; d3 = p1 - p0;
    D1 = D2; D2 = p1 - m1;
  }
  // mc_face of the window's face (between m1 and p0).
  template <bool kP2>
  __device__ __forceinline__ R face(bool pos, R inv_h, R h, R wdt) const {
    return mc_reconstruct<R, kP2>(pos, pos ? D1 : D2, pos ? d1 : d2, pos ? d2 : d3,
                                  pos ? m1 : p0, inv_h, h, wdt);
  }
};

// The one-step differences only (d1, d2, d3) of a marching column window.
template <typename R>
struct ColSteps {
  R m2, m1, p0, p1, d1, d2, d3;
  __device__ __forceinline__ void init(R m2_, R m1_, R p0_, R p1_) {
    m2 = m2_; m1 = m1_; p0 = p0_; p1 = p1_;
    refresh();
  }
  __device__ __forceinline__ void refresh() {
    d1 = m1 - m2; d2 = p0 - m1; d3 = p1 - p0;
  }
  __device__ __forceinline__ void push(R next) {
    m2 = m1; m1 = p0; p0 = p1; p1 = next;
  }
  __device__ __forceinline__ void shift(R next) {
    const R d3n = next - p1;
    m2 = m1; m1 = p0; p0 = p1; p1 = next;
    d1 = d2; d2 = d3; d3 = d3n;
  }
};

// Mass and energy flux through one face (omp3/flow.c:340-404, 455-517), from
// the face velocity v0 and the differences of the face velocities around it
// (dv2 = vp-vm, dvm = v0-vm, dvp = vp-v0), the densities rm1 | r0 either side
// with jump = r0-rm1, the Van Leer smoothness numerator num_of(up) (upwind
// side: rm1-rm2, else rp1-r0), and the energy reconstruction e_face_of(pos,
// w dt_h).  inv_h is the reciprocal of the face spacing, icd of the
// downstream cell width, area the face length.  kSideV0: take the Van Leer
// side from v0 (the y sweep, omp3/flow.c:477) instead of the half-step
// velocity.  A zero limiter (flat or extremal density) leaves the upwind
// flux, and the second-order term is skipped.
template <typename R, bool kSideV0, bool kP2, typename NumFn, typename EFaceFn>
__device__ __forceinline__ void mass_energy_flux_core(R v0, R dv2, R dvm, R dvp, R rm1, R r0,
                                                      R jump, NumFn num_of, EFaceFn e_face_of,
                                                      R inv_h, R icd, R area, R dt, R dt_h,
                                                      R* F_out, R* eF_out) {
  using Pr = Prec<R>;
  if (Pr::zero_skip_coarse(v0)) {  // a face at rest carries no mass and no energy
    *F_out = R(0);
    *eF_out = R(0);
    return;
  }
  // minmod(0.5 (vp-vm)/h, 2 (v0-vm)/h, 2 (vp-v0)/h), scaled once (mc_reconstruct).
  const R mm = Pr::template mulp<kP2>(
      Pr::minmod(Pr::half(dv2), Pr::minmod(Pr::twice(dvm), Pr::twice(dvp))), inv_h);
  const R w_tc = Pr::msub(v0, Pr::half(v0) * dt, mm);
  R lim = R(0);
  if (!Pr::is_zero(jump)) {
    const bool up = kSideV0 ? Pr::ge0(v0) : Pr::ge0(w_tc);
    const R num = num_of(up);
    // Van Leer: (s+|s|)/(1+|s|) with s = num/jump, i.e. 2 num/(jump+num)
    // when num and jump share a sign, else 0.
    if (Pr::same_sign_nz(num, jump)) {
      lim = Pr::twice(num) * Pr::rcp(jump + num);
    }
  }
  const R rho_up = Pr::ge0(w_tc) ? rm1 : r0;
  const R wdt = w_tc * dt_h;
  R flux;
  if (Pr::zero_skip(lim)) {
    flux = w_tc * rho_up;
  } else {
    flux = Pr::madd(w_tc, rho_up,
                    Pr::half(Pr::abs(w_tc)) *
                        (R(1) - Pr::abs(Pr::template mulp<kP2>(wdt, icd))) * lim * jump);
  }
  const R e_face = e_face_of(Pr::gt0(w_tc), wdt);
  *F_out = flux;
  *eF_out = Pr::template mulp<kP2>(e_face, area) * flux;
}

// The flux from the four cells straddling the face (m2, m1 | p0, p1) and
// the face velocities vm, v0, vp (the x sweep); h_m/h_p are the cell widths
// either side.
template <typename R, bool kSideV0, bool kP2>
__device__ __forceinline__ void mass_energy_flux(R vm, R v0, R vp, R rm2,
                                                 R rm1, R r0, R rp1, R em2,
                                                 R em1, R e0, R ep1, R inv_h,
                                                 R h_m, R h_p, R icd, R area,
                                                 R dt, R dt_h, R* F_out,
                                                 R* eF_out) {
  mass_energy_flux_core<R, kSideV0, kP2>(
      v0, vp - vm, v0 - vm, vp - v0, rm1, r0, r0 - rm1,
      [&](bool up) { return (up ? rm1 : rp1) - (up ? rm2 : r0); },
      [&](bool pos, R wdt) {
        return mc_face<R, kP2>(pos, em2, em1, e0, ep1, inv_h, pos ? h_m : h_p, wdt);
      },
      inv_h, icd, area, dt, dt_h, F_out, eF_out);
}

// The energy of a cell that takes no flux: the reference's rho_old*e/den
// round trip, which gives e itself when the product rho_old*e is exact and
// den is rho_old.  Called (a real branch) by warps whose round trip is not
// settled by tests on the bit patterns: a short FP64 sequence under a branch
// is turned into predicated code that still occupies the FP64 pipe.
template <typename R>
static __device__ __noinline__ double still_energy(double r_old, double e_in, double den) {
  const double rho_e = __dmul_rn(r_old, e_in);
  if (warp_all(d_is_zero(fma(r_old, e_in, -rho_e)) && dbits(den) == dbits(r_old) &&
               !d_is_zero(den))) {
    return e_in;
  }
  if (d_is_zero(den)) return 0.0;
  if constexpr (Prec<R>::kMixed) {
    const double r0 = Prec<R>::to_d(Prec<R>::rcp(Prec<R>::from_d(den)));
    const double q = rho_e * r0;
    return fma(r0, fma(-den, q, rho_e), q);
  } else {
    return d_div(rho_e, den);
  }
}

// Conservative FP64 update of one cell from its two face fluxes (given in
// bulk precision, converted exactly): vol = celldx*celldy and ivol its
// reciprocal (in the mixed form ivol is dt_h/vol: the sweeps fold dt_h into
// their row factors), a0/a1 the face lengths.  den is rho_old in the first
// sweep of a step and the new density in the second (omp3/flow.c:416-432).
// The FP64 form keeps the reference's evaluation order; the mixed form
// contracts into FMAs.

// The fluxes arrive widened to FP64 (f0, f1 mass, ef0, ef1 energy; exact
// for the mixed form's FP32 fluxes), each face's once.
template <typename R, bool kFirst, bool kP2>
__device__ __forceinline__ void mass_energy_update(double r_in, double e_in,
                                                   double r_old, double dt_h,
                                                   double vol, double ivol, double a0,
                                                   double a1, double f0, double f1,
                                                   double ef0, double ef1, double* r_out,
                                                   double* e_out) {
  using Pr = Prec<R>;
  // No mass or energy crosses any cell of the warp (a warp-uniform test): the
  // updates subtract zeros, the density stays and the energy takes the
  // reference's rho_old*e/den round trip -- which gives e itself when the
  // product rho_old*e is exact and den is rho_old, as in the still background
  // of a blast (a power-of-two density: settled without FP64 instructions).
  // The FP64 form takes the per-lane skip below otherwise.
  const bool none = warp_all(d_is_zero(f0) && d_is_zero(f1) &&
                             (Pr::kMixed || (d_is_zero(ef0) && d_is_zero(ef1))));
  if (none) {
    const double den = kFirst ? r_old : r_in;
    *r_out = r_in;
    if (warp_all(dbits(den) == dbits(r_old) && d_pow2_product_exact(r_old, e_in))) {
      *e_out = e_in;
    } else {
      *e_out = still_energy<R>(r_old, e_in, den);
    }
    return;
  }
  const double de = ef1 - ef0;
  double r_new, rho_e;
  if (Pr::kMixed) {
    const double coef = ivol;
    // On power-of-two tiles the face-length products are exact exponent adds
    // (the same numbers as the FMA below, which rounds once after them).
    const double net = kP2 ? __dadd_rn(d_mul_pow2(f1, a1), -d_mul_pow2(f0, a0))
                           : fma(a1, f1, -(a0 * f0));
    r_new = fma(-coef, net, r_in);
    rho_e = fma(-coef, de, r_old * e_in);
  } else if (Pr::zero_skip(f0) && Pr::zero_skip(f1) && Pr::zero_skip(de)) {
    // Nothing crosses the cell's faces: the updates subtract zeros.  (The
    // energy still takes the reference's rho_old*e/den round trip below.)
    r_new = r_in;
    rho_e = __dmul_rn(r_old, e_in);
  } else {
    const double net = __dadd_rn(Prec<double>::mulp<kP2>(f1, a1), -Prec<double>::mulp<kP2>(f0, a0));
    r_new = Prec<double>::dsub<kP2>(r_in, __dmul_rn(dt_h, net), vol, ivol);
    rho_e = Prec<double>::dsub<kP2>(__dmul_rn(r_old, e_in), __dmul_rn(dt_h, de), vol, ivol);
  }
  const double den = kFirst ? r_old : r_new;
  *r_out = r_new;
  if (d_is_zero(den)) {
    *e_out = 0.0;
  } else if (Pr::kMixed) {
    // Quotient from the FP32 reciprocal of den and one FP64 correction.
    const double r0 = Pr::to_d(Pr::rcp(Pr::from_d(den)));
    const double q = rho_e * r0;
    *e_out = fma(r0, fma(-den, q, rho_e), q);
  } else {
    *e_out = Prec<double>::div(rho_e, den);
  }
}

template <typename R>
struct SweepArgs {
  const double* r_in;  // FP64 density and energy entering the sweep
  const double* e_in;
  const R* r_in_r;     // the same in bulk precision (aliases for FP64)
  const R* e_in_r;
  double* r_out;
  double* e_out;
  R* r_out_r;
  R* e_out_r;
  // Tile skips (the kFl kernels; null otherwise).  The first sweep of a step
  // marks a tile of its grid (one byte per tile, skip_tiles_x per band of
  // rows) whose cells are at rest -- every face velocity around them is +0,
  // so neither sweep moves anything through their faces -- and keep their
  // energy bit for bit through the density round trip; it stores nothing for
  // them.  The second sweep reads a cell of a marked tile from r_alt/e_alt
  // (the first sweep's input, which holds its value; storing it again writes
  // that value), and does nothing at all for a tile of its own whose cells
  // all lie in marked tiles.
  unsigned char* skip;
  int skip_tiles_x;
  int skip_bands;      // bands of rows
  const double* r_alt;
  const double* e_alt;
  const R* r_alt_r;
  const R* e_alt_r;
};

// The mirror source of a column or row index (identity inside the interior).
__device__ __forceinline__ int mirror_src(int i, int n, int pad) {
  return i < pad ? 2 * pad - 1 - i : (i >= n - pad ? 2 * (n - pad) - 1 - i : i);
}

// Whether every cell of rows r0 .. r1 - 1 in column jj (when ok) takes the
// density round trip exactly (the sweeps' bit-pattern test for a cell no
// flux crosses): loads in batches of eight rows.  Block-uniform (barrier).
__device__ __forceinline__ bool block_round_trip_exact(const double* rho, const double* e,
                                                       int nx, int r0, int r1, int jj,
                                                       bool ok) {
  bool exact = true;
  constexpr int kB = 8;
  for (int ib = r0; ib < r1; ib += kB) {
    double rv[kB], ev[kB];
#pragma unroll
    for (int q = 0; q < kB; ++q) {
      const bool in = ok && ib + q < r1;
      rv[q] = in ? rho[cidx(nx, ib + q, jj)] : 1.0;
      ev[q] = in ? e[cidx(nx, ib + q, jj)] : 1.0;
    }
#pragma unroll
    for (int q = 0; q < kB; ++q) exact = exact && d_pow2_product_exact(rv[q], ev[q]);
  }
  return __syncthreads_and(exact) != 0;
}

// x sweep: CTAs own 127 cells and compute the 128 faces around them (the last
// face is shared with the next CTA and written only by its owner).  In the
// second sweep of a step the old density of a cell is read from rho just
// before the same thread overwrites that cell.
// kAlt (second sweep with flags): some tile near this one was skipped by the
// first sweep (sk3, the skip marks of this band's y-sweep tiles tlo ..
// tlo + 2); without it the loads need no selection.
template <typename R, bool kFirst, bool kP2, bool kEarly, bool kFl, bool kAlt>
__device__ __forceinline__ void tile_mass_sweep_x_impl(const StepArgs<R>& a,
                                                       const SweepArgs<R>& s, int bx, int by,
                                                       unsigned sk3) {
  using Pr = Prec<R>;
  __shared__ R s_ey0r[kMaxRows];
  __shared__ double sF[kCols], seF[kCols];  // the row's face fluxes, widened once
  __shared__ double s_coef[kMaxRows], s_cyd[kMaxRows], s_ey0[kMaxRows], s_ey1[kMaxRows];
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int t = threadIdx.x;
  const int jj = pad + bx * (kCols - 1) + t;  // face (and cell) column
  const int i0 = pad + by * a.rows;
  const bool edge = tile_near_edge(nx, ny, pad, pad + bx * (kCols - 1), i0, a.rows);
  const double dt = a.dt_slot[0], dt_h = a.dt_slot[1];
  const int tlo = max(0, (bx * (kCols - 1) - 2) >> 7);
  if (t < a.rows) {
    const int ii = i0 + t;
    if (ii < ny - pad) {
      // Row factor of the update: 1/celldy, times dt_h in the mixed form.
      s_coef[t] = Pr::kMixed ? dt_h * geo_rcp_d<R, kP2>(a.celldy[ii])
                             : geo_rcp_d<R, kP2>(a.celldy[ii]);
      s_cyd[t] = a.celldy[ii];
      s_ey0[t] = a.edgedy[ii];
      s_ey0r[t] = geo_v<R>(a.edgedy[ii]);
      s_ey1[t] = a.edgedy[ii + 1];
    }
  }
  const bool face_ok = jj < nx + 1 - pad;
  const bool cell_ok = (t < kCols - 1) && (jj < nx - pad);
  const bool face_owner = face_ok && (t < kCols - 1);
  R iex = R(0), cxm = R(0), cx0 = R(0), icx_r = R(0);
  double icx = 0.0;
  if (face_ok) {
    iex = geo_rcp<R, kP2>(a.edgedx[jj]);
    cxm = geo_v<R>(a.celldx[jj - 1]);
    cx0 = geo_v<R>(a.celldx[jj]);
    icx = geo_rcp_d<R, kP2>(a.celldx[jj]);
    icx_r = Pr::from_d(icx);
  }
  const R dt_r = Pr::from_d(dt), dt_h_r = Pr::from_d(dt_h);
  const int i1 = min(i0 + a.rows, ny - pad);
  // Row ii+1's face velocity and the update inputs of its cell are loaded
  // before row ii is processed (the first row's before the barrier that
  // publishes the row tables, kEarly); a warp whose faces are all at rest
  // carries no flux and reads nothing else (the flux core returns +0 for
  // them).
  R u0_n = R(0);
  double rin_n = 0.0, ein_n = 0.0, rold_n = 0.0;
  auto load = [&](int ii) {
    if (face_ok) u0_n = a.u[fidx(nx, ii, jj)];
    if (cell_ok) {
      const size_t c = cidx(nx, ii, jj);
      rin_n = s.r_in[c];
      ein_n = s.e_in[c];
      rold_n = kFirst ? rin_n : a.rho[c];
    }
  };
  // kEarly (the fused kernel): the face velocity and the cell's density and
  // energy (and in the second sweep its old density) stream through a
  // per-thread ring of asynchronous copies instead, kAhead rows ahead: no
  // registers held for them, no barrier (each thread reads back only what it
  // copied).
  constexpr int kAhead = Pr::kMixed ? 2 : 3, kSlots = kAhead + 1;
  auto s_ru = ring_slots<R, kEarly ? kSlots : 1, 1, kEarly ? kCols : 1, 6>();
  auto s_rd = ring_slots<double, kEarly ? kSlots : 1, kFirst ? 2 : 3, kEarly ? kCols : 1, 7>();
  // Tile skips (SweepArgs::skip).  First sweep: a tile at rest in both
  // directions whose cells take the round trip exactly stores nothing but
  // its flags.  Second sweep (after the y sweep): the skip marks of this
  // band's y-sweep tiles tlo .. tlo + 2, which hold every cell it reads.
  constexpr bool kSkip2 = kFl && !kFirst && kAlt;

  // The value of cell column col (this tile's rows) lies in r_alt/e_alt: its
  // tile was skipped by the first sweep.
  auto in_alt = [&](int col) -> bool {
    if constexpr (!kSkip2) {
      return false;
    } else {
      const int q = mirror_src(col, nx, pad) - pad;
      return ((sk3 >> ((q >> 7) - tlo)) & 1u) != 0u;
    }
  };
  auto issue = [&](int ii) {
    const int sl = (ii - i0) % kSlots;
    const size_t c = cidx(nx, ii, jj);
    const bool alt = cell_ok && in_alt(jj);
    cp_async_elem(&s_ru[sl][0][t], face_ok ? a.u + fidx(nx, ii, jj) : a.u, face_ok);
    cp_async_elem(&s_rd[sl][0][t], alt ? s.r_alt + c : (cell_ok ? s.r_in + c : s.r_in), cell_ok);
    cp_async_elem(&s_rd[sl][1][t], alt ? s.e_alt + c : (cell_ok ? s.e_in + c : s.e_in), cell_ok);
    if constexpr (!kFirst) {
      // The old density (in rho); for a cell of a skipped tile, the value
      // just read.
      cp_async_elem(&s_rd[sl][kFirst ? 1 : 2][t], cell_ok ? a.rho + c : a.rho, cell_ok && !alt);
    }
  };
  if constexpr (kEarly) {
#pragma unroll
    for (int d = 0; d < kAhead; ++d) {
      if (i0 + d < i1) issue(i0 + d);
      cp_async_commit();
    }
  }
  __syncthreads();
  if (!kEarly && i0 < i1) load(i0);
  for (int ii = i0; ii < i1; ++ii) {
    const int k = ii - i0;
    R u0;
    double r_in, e_in, r_old;
    if constexpr (kEarly) {
      cp_async_wait<kAhead - 1>();  // row ii's group has landed
      const int sl = k % kSlots;
      u0 = s_ru[sl][0][t];
      r_in = s_rd[sl][0][t];
      e_in = s_rd[sl][1][t];
      r_old = (kFirst || (cell_ok && in_alt(jj))) ? r_in : s_rd[sl][kFirst ? 1 : 2][t];
      if (ii + kAhead < i1) issue(ii + kAhead);
      cp_async_commit();
    } else {
      u0 = u0_n;
      r_in = rin_n;
      e_in = ein_n;
      r_old = rold_n;
      if (ii + 1 < i1) load(ii + 1);
    }
    R F = R(0), eF = R(0);
    // Whether a face of the warp moves (a lane without a face holds +0): a
    // warp whose faces are all at rest carries +0 fluxes.
    const bool moves = !warp_all(Pr::is_zero(u0));
    if (face_ok && moves) {
      const size_t f = fidx(nx, ii, jj);
      const size_t c = cidx(nx, ii, jj);
      // A stencil cell's density and energy (from r_alt/e_alt for a cell of a
      // skipped tile).
      auto rr = [&](int d) { return in_alt(jj + d) ? s.r_alt_r[c + d] : s.r_in_r[c + d]; };
      auto er = [&](int d) { return in_alt(jj + d) ? s.e_alt_r[c + d] : s.e_in_r[c + d]; };
      mass_energy_flux<R, false, kP2>(a.u[f - 1], u0, a.u[f + 1], rr(-2), rr(-1), rr(0), rr(1),
                                      er(-2), er(-1), er(0), er(1), iex, cxm, cx0, icx_r,
                                      s_ey0r[k], dt_r, dt_h_r, &F, &eF);
    }
    // kFl: a warp at rest stores only its flag (its fluxes are +0).
    if constexpr (kFl) {
      store_flag(a.fxflag + (size_t)(ii - pad) * a.fx_stride + 4 * bx + (t >> 5), moves);
    }
    if (face_owner && (!kFl || moves)) {
      a.F_x[fidx(nx, ii, jj)] = F;
      mirror(edge, a.F_x, nx + 1, ny, pad, ii, jj, F, true, false);
    }
    sF[t] = Pr::to_d(F);
    seF[t] = Pr::to_d(eF);
    __syncthreads();
    if (cell_ok) {
      double r_new, e_new;
      mass_energy_update<R, kFirst, kP2>(r_in, e_in, r_old, dt_h,
                                         a.celldx[jj] * s_cyd[k],
                                         Prec<double>::mulp<kP2>(s_coef[k], icx),
                                         s_ey0[k], s_ey1[k], sF[t],
                                         sF[t + 1], seF[t], seF[t + 1], &r_new, &e_new);
      // (A cell of a skipped tile is at rest and keeps its value, which rho
      // and e hold: storing it again writes the same value.)
      store_cell(edge, s.r_out, s.r_out_r, nx, ny, pad, ii, jj, r_new);
      store_cell(edge, s.e_out, s.e_out_r, nx, ny, pad, ii, jj, e_new);
    }
    __syncthreads();
  }
  if constexpr (kEarly) cp_async_wait<0>();
}

template <typename R, bool kFirst, bool kEarly = true, bool kFl = false>
__device__ __forceinline__ void tile_mass_sweep_x(const StepArgs<R>& a, const SweepArgs<R>& s,
                                                  int bx, int by) {
  if constexpr (kFl) {
    // Tile skips (SweepArgs::skip), decided before any other work.
    const int pad = a.pad, t = threadIdx.x;
    const int cb = pad + bx * (kCols - 1), jj = cb + t;
    const int i0 = pad + by * a.rows, i1 = min(i0 + a.rows, a.ny - pad);
    const bool cell_ok = t < kCols - 1 && jj < a.nx - pad;
    auto zero_flags = [&]() {  // the mass-flux flags of a tile at rest
      for (int ii = i0; ii < i1; ++ii) {
        store_flag(a.fxflag + (size_t)(ii - pad) * a.fx_stride + 4 * bx + (t >> 5), false);
      }
    };
    if constexpr (kFirst) {
      // At rest in both directions, and every cell's round trip exact.
      // (Cells at rest through the previous step took the round trip
      // exactly then, on the same values.)
      bool sk = tile_vel_still(a, i0 - 2, i1 + 2, cb - 2, cb + kCols + 1);
      if (sk && !rest_cells(a, i0, i1, cb, min(cb + kCols - 1, a.nx - pad))) {
        sk = block_round_trip_exact(s.r_in, s.e_in, a.nx, i0, i1, jj, cell_ok);
      }
      if (t == 0) {
        store_flag(s.skip + (size_t)by * s.skip_tiles_x + bx, sk);
        if (!sk && a.moving) atomicAdd(a.moving, 1ull);
      }
      if (sk) {
        zero_flags();
        return;
      }
    } else {
      // The skip marks of this band's y-sweep tiles tlo .. tlo + 2.
      const int tlo = max(0, (bx * (kCols - 1) - 2) >> 7);
      unsigned sk3 = 0u;
      for (int k = 0; k < 3; ++k) {
        const int tx = tlo + k;
        if (tx < s.skip_tiles_x && s.skip[(size_t)by * s.skip_tiles_x + tx]) sk3 |= 1u << k;
      }
      // Every cell of the tile lies in a skipped tile: at rest, unchanged.
      const int q = jj - pad;
      if (__syncthreads_and(!cell_ok || ((sk3 >> ((q >> 7) - tlo)) & 1u))) {
        zero_flags();
        return;
      }
      if (__syncthreads_or(sk3 != 0u)) {
        FLOW_POW2_DISPATCH_ALL(
            a, a.pad + bx * (kCols - 1), a.pad + by * a.rows,
            (tile_mass_sweep_x_impl<R, kFirst, true, kEarly, kFl, true>(a, s, bx, by, sk3)),
            (tile_mass_sweep_x_impl<R, kFirst, false, kEarly, kFl, true>(a, s, bx, by, sk3)));
        return;  // (the dispatch returns only after its power-of-two branch)
      }
    }
  }
  FLOW_POW2_DISPATCH_ALL(
      a, a.pad + bx * (kCols - 1), a.pad + by * a.rows,
      (tile_mass_sweep_x_impl<R, kFirst, true, kEarly, kFl, false>(a, s, bx, by, 0u)),
      (tile_mass_sweep_x_impl<R, kFirst, false, kEarly, kFl, false>(a, s, bx, by, 0u)));
}

// y sweep: each thread marches down its column; face row ii+1 is computed
// in iteration ii and reused by the cell below.
// kAlt (second sweep with flags): some tile near this one was skipped by the
// first sweep (sk3, the skip marks of bands by - 1 .. by + 1 of this
// column's x-sweep tile); without it the loads need no selection.
template <typename R, bool kFirst, bool kP2, bool kEarly, bool kFl, bool kAlt>
__device__ __forceinline__ void tile_mass_sweep_y_impl(const StepArgs<R>& a,
                                                       const SweepArgs<R>& s, int bx, int by,
                                                       unsigned sk3) {
  using Pr = Prec<R>;
  __shared__ R s_iey[kMaxRows + 1], s_cy[kMaxRows + 2], s_icy[kMaxRows + 1];
  __shared__ double s_coef[kMaxRows], s_cyd[kMaxRows];
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int jj = pad + bx * kCols + threadIdx.x;
  const int i0 = pad + by * a.rows;
  const bool edge = tile_near_edge(nx, ny, pad, pad + bx * kCols, i0, a.rows);
  const double dt = a.dt_slot[0], dt_h = a.dt_slot[1];
  constexpr bool kSkip2 = kFl && !kFirst && kAlt;
  // Face rows i0 .. i0+a.rows, cell rows i0-1 .. i0+a.rows.
  if (threadIdx.x < a.rows + 2) {
    const int ii = i0 - 1 + threadIdx.x;
    if (ii < ny) s_cy[threadIdx.x] = geo_v<R>(a.celldy[ii]);
  }
  if (threadIdx.x < a.rows + 1) {
    const int ii = i0 + threadIdx.x;
    if (ii < ny) {
      s_iey[threadIdx.x] = geo_rcp<R, kP2>(a.edgedy[ii]);
      s_icy[threadIdx.x] = geo_rcp<R, kP2>(a.celldy[ii]);
      if (threadIdx.x < a.rows) {
        s_coef[threadIdx.x] = Pr::kMixed ? dt_h * geo_rcp_d<R, kP2>(a.celldy[ii])
                                         : geo_rcp_d<R, kP2>(a.celldy[ii]);
        s_cyd[threadIdx.x] = a.celldy[ii];
      }
    }
  }
  const bool col_ok = jj < nx - pad;
  const int i1 = min(i0 + a.rows, ny - pad);
  const int last_face = ny - pad;  // the north boundary face row
  // Tile skips (SweepArgs::skip).  First sweep: a tile at rest in both
  // directions whose cells take the round trip exactly stores nothing but
  // its flags.  Second sweep (after the x sweep): the skip marks of this
  // column's x-sweep tile in bands by - 1 .. by + 1, which hold every cell
  // it reads (tiles of at least two rows).
  // The value of this column's cell in row r (i0 - 2 <= r <= i1 + 1) lies
  // in r_alt/e_alt: its tile was skipped by the first sweep.
  auto in_alt = [&](int r) -> bool {
    if constexpr (!kSkip2) {
      return false;
    } else {
      const int rs = mirror_src(r, ny, pad);
      return ((sk3 >> (rs < i0 ? 0 : (rs >= i1 ? 2 : 1))) & 1u) != 0u;
    }
  };
  // Windows at face row f: cells f-2..f+1 (densities and energies with their
  // differences), face velocities f-1..f+1 with theirs; each row shifts them
  // by one and forms only the new differences.  In the FP64 form a face row
  // at rest in the whole warp carries no flux, and its differences are not
  // formed: the windows shift their values alone (stale differences) and
  // form all the differences again at the next row that moves -- the same
  // operands, so the same values.
  ColSteps<R> rw;
  ColWindow<R> ew;
  R vm = R(0), v0 = R(0), vp = R(0);
  R dvm, dvp, dv2;
  // The window values of row ii+3 and the update inputs of row ii+1 are
  // loaded before row ii is processed.
  R rn_n = R(0), en_n = R(0), vn_n = R(0);
  double rin_n = 0.0, ein_n = 0.0, rold_n = 0.0;
  auto load = [&](int ii) {
    const size_t c_next = cidx(nx, ii + 2, jj);
    rn_n = s.r_in_r[c_next];
    en_n = s.e_in_r[c_next];
    vn_n = a.v[c_next];
    const size_t c = cidx(nx, ii, jj);
    rin_n = s.r_in[c];
    ein_n = s.e_in[c];
    rold_n = kFirst ? rin_n : a.rho[c];
  };
  // The windows' first values and the first row's inputs are loaded before
  // the barrier that publishes the row tables (kEarly), else after it.
  auto prime = [&]() {
    vm = a.v[cidx(nx, i0 - 1, jj)];
    v0 = a.v[cidx(nx, i0, jj)];
    vp = a.v[cidx(nx, i0 + 1, jj)];
    R r[4], e[4];
    for (int q = 0; q < 4; ++q) {
      const size_t c = cidx(nx, i0 - 2 + q, jj);
      const bool alt = in_alt(i0 - 2 + q);
      r[q] = alt ? s.r_alt_r[c] : s.r_in_r[c];
      e[q] = alt ? s.e_alt_r[c] : s.e_in_r[c];
    }
    rw.m2 = r[0]; rw.m1 = r[1]; rw.p0 = r[2]; rw.p1 = r[3];
    ew.m2 = e[0]; ew.m1 = e[1]; ew.p0 = e[2]; ew.p1 = e[3];
  };
  // kEarly (the fused kernel): the window values stream through a per-thread
  // ring of asynchronous copies instead, kAhead rows ahead (no registers held
  // for them, no barrier: each thread reads back only what it copied), and
  // the FP64 form takes a cell's update inputs from its windows (the same
  // arrays: r_in_r and e_in_r alias r_in and e_in), so only the second
  // sweep's old density (and the mixed form's FP64 inputs) stay a row ahead
  // in registers.
  constexpr int kAhead = Pr::kMixed ? 2 : 3, kSlots = kAhead + 1;
  // The FP64 second sweep's old density of row ii rides in the same group (a
  // fourth plane).
  constexpr bool kOldRing = !kFirst && !Pr::kMixed;
  auto s_w = ring_slots<R, kEarly ? kSlots : 1, kOldRing ? 4 : 3, kEarly ? kCols : 1, 8>();
  const int t = threadIdx.x;
  auto issue = [&](int ii) {
    const int sl = (ii - i0) % kSlots;
    const size_t c = cidx(nx, ii + 2, jj);
    const bool alt = in_alt(ii + 2);
    cp_async_elem(&s_w[sl][0][t], alt ? s.r_alt_r + c : s.r_in_r + c, true);
    cp_async_elem(&s_w[sl][1][t], alt ? s.e_alt_r + c : s.e_in_r + c, true);
    cp_async_elem(&s_w[sl][2][t], a.v + c, true);
    // The old density (in rho); for a cell of a skipped tile, the value the
    // window holds.
    if constexpr (kOldRing) {
      cp_async_elem(&s_w[sl][3][t], a.rho + cidx(nx, ii, jj), !in_alt(ii));
    }
  };
  auto load_upd = [&](int ii) {
    const size_t c = cidx(nx, ii, jj);
    const bool alt = in_alt(ii);
    if (Pr::kMixed) {
      rin_n = alt ? s.r_alt[c] : s.r_in[c];
      ein_n = alt ? s.e_alt[c] : s.e_in[c];
    }
    if (!kFirst && !kOldRing) rold_n = alt ? rin_n : a.rho[c];
  };
  if (kEarly && col_ok) {
    prime();
#pragma unroll
    for (int d = 0; d < kAhead; ++d) {
      if (i0 + d < i1) issue(i0 + d);
      cp_async_commit();
    }
    if (i0 < i1) load_upd(i0);
  }
  __syncthreads();
  if (!col_ok) return;
  const double icx = geo_rcp_d<R, kP2>(a.celldx[jj]);
  const double ex0 = a.edgedx[jj], ex1 = a.edgedx[jj + 1];
  const R ex0_r = geo_v<R>(ex0), dt_r = Pr::from_d(dt), dt_h_r = Pr::from_d(dt_h);
  if (!kEarly) prime();
  auto refresh = [&]() {
    rw.refresh();
    ew.refresh();
    dvm = v0 - vm;
    dvp = vp - v0;
    dv2 = vp - vm;
  };
  // Whether face row f (velocity v0) moves somewhere in the warp; always in
  // the mixed form, whose FP32 differences cost less than the test.
  auto moves = [&]() { return Pr::kMixed || !warp_all(Pr::is_zero(v0)); };
  bool fresh = moves();
  if (fresh) refresh();
  // Face row f = i0 + k: inverse spacing s_iey[k], cell widths s_cy[k] below
  // and s_cy[k + 1] above, downstream inverse width s_icy[k].
  auto flux_at = [&](int k, R* F, R* eF) {
    mass_energy_flux_core<R, true, kP2>(
        v0, dv2, dvm, dvp, rw.m1, rw.p0, rw.d2, [&](bool up) { return up ? rw.d1 : rw.d3; },
        [&](bool pos, R wdt) {
          return ew.template face<kP2>(pos, s_iey[k], pos ? s_cy[k] : s_cy[k + 1], wdt);
        },
        s_iey[k], s_icy[k], ex0_r, dt_r, dt_h_r, F, eF);
  };
  // Stores the mass flux of face row f; kFl: only where the face row moves
  // somewhere in the warp (mv) -- a face row at rest carries +0 (the mixed
  // form, whose rows all count as moving, votes on the fluxes instead).  The
  // warp's flags (bit f - i0 of fmask) are written after the row loop.
  unsigned long long fmask = 0ull;
  auto store_fy = [&](int f, R F, bool mv) {
    bool st = true;
    if constexpr (kFl) {
      st = Pr::kMixed ? __any_sync(__activemask(), !is_plus_zero(F)) : mv;
      if (st) fmask |= 1ull << (f - i0);
    }
    if (st) {
      a.F_y[cidx(nx, f, jj)] = F;
      mirror(edge, a.F_y, nx, ny + 1, pad, f, jj, F, false, true);
    }
  };
  R F0 = R(0), eF0 = R(0);
  if (fresh) flux_at(0, &F0, &eF0);
  store_fy(i0, F0, fresh);
  // The fluxes of the face below, widened once and carried to the next row.
  double f0d = Pr::to_d(F0), ef0d = Pr::to_d(eF0);
  if (!kEarly && i0 < i1) load(i0);
  for (int ii = i0; ii < i1; ++ii) {
    const int k = ii - i0;
    R rn, en, vn;
    double r_in, e_in, r_old;
    if constexpr (kEarly) {
      cp_async_wait<kAhead - 1>();  // row ii's group has landed
      const int sl = k % kSlots;
      rn = s_w[sl][0][t];
      en = s_w[sl][1][t];
      vn = s_w[sl][2][t];
      if (ii + kAhead < i1) issue(ii + kAhead);
      cp_async_commit();
      if constexpr (Pr::kMixed) {
        r_in = rin_n;
        e_in = ein_n;
      } else {
        r_in = rw.p0;  // cell ii, the window's upper middle value before this row's shift
        e_in = ew.p0;
      }
      if constexpr (kOldRing) {
        r_old = in_alt(ii) ? r_in : s_w[sl][3][t];
      } else {
        r_old = kFirst ? r_in : rold_n;
      }
      if (ii + 1 < i1) load_upd(ii + 1);
    } else {
      rn = rn_n;
      en = en_n;
      vn = vn_n;
      r_in = rin_n;
      e_in = ein_n;
      r_old = rold_n;
      if (ii + 1 < i1) load(ii + 1);
    }
    R F1 = R(0), eF1 = R(0);
    const bool was_fresh = fresh;
    // Shift the velocity window's values; face row k+1 has velocity vp.
    const R v_prev0 = v0, v_prevp = vp;
    vm = v0;
    v0 = vp;
    vp = vn;
    fresh = moves();
    if (fresh) {
      if (was_fresh) {
        rw.shift(rn);
        ew.shift(en);
        const R dv2n = vn - v_prev0, dvpn = vn - v_prevp;
        dvm = dvp;
        dvp = dvpn;
        dv2 = dv2n;
      } else {
        rw.push(rn);
        ew.push(en);
        refresh();
      }
      flux_at(k + 1, &F1, &eF1);
      // FP64 form with flags: only a moving face row stores its fluxes, here
      // on the moving path.
      if (kFl && !Pr::kMixed && (ii + 1 < i1 || ii + 1 == last_face)) store_fy(ii + 1, F1, true);
    } else {
      // A face row at rest carries no mass and no energy (+0, as the flux
      // core returns for a face at rest).
      rw.push(rn);
      ew.push(en);
    }
    if (!(kFl && !Pr::kMixed) && (ii + 1 < i1 || ii + 1 == last_face)) {
      store_fy(ii + 1, F1, fresh);
    }
    double r_new, e_new;
    const double f1d = Pr::to_d(F1), ef1d = Pr::to_d(eF1);
    mass_energy_update<R, kFirst, kP2>(r_in, e_in, r_old, dt_h,
                                       a.celldx[jj] * s_cyd[k],
                                       Prec<double>::mulp<kP2>(s_coef[k], icx), ex0, ex1,
                                       f0d, f1d, ef0d, ef1d, &r_new, &e_new);
    // (A cell of a skipped tile is at rest and keeps its value, which rho and
    // e hold: storing it again writes the same value.)
    store_cell(edge, s.r_out, s.r_out_r, nx, ny, pad, ii, jj, r_new);
    store_cell(edge, s.e_out, s.e_out_r, nx, ny, pad, ii, jj, e_new);
    f0d = f1d;
    ef0d = ef1d;
  }
  if constexpr (kFl) {
    // Face rows i0 .. i1 - 1, and the north boundary row in the last tile.
    const int f_end = (i1 == last_face) ? last_face : i1 - 1;
    unsigned char* fp = a.fyflag + (size_t)(i0 - pad) * 4 * a.qm_stride + 4 * bx + (t >> 5);
    for (int f = i0; f <= f_end; ++f, fp += 4 * a.qm_stride) {
      store_flag(fp, (fmask >> (f - i0)) & 1ull);
    }
  }
  if constexpr (kEarly) cp_async_wait<0>();
}

template <typename R, bool kFirst, bool kEarly = true, bool kFl = false>
__device__ __forceinline__ void tile_mass_sweep_y(const StepArgs<R>& a, const SweepArgs<R>& s,
                                                  int bx, int by) {
  if constexpr (kFl) {
    // Tile skips (SweepArgs::skip), decided before any other work.
    const int pad = a.pad;
    const int cb = pad + bx * kCols, jj = cb + threadIdx.x;
    const int i0 = pad + by * a.rows, i1 = min(i0 + a.rows, a.ny - pad);
    const bool col_ok = jj < a.nx - pad;
    auto zero_flags = [&]() {  // the mass-flux flags of a tile at rest
      const int last_face = a.ny - pad;
      const int f_end = (i1 == last_face) ? last_face : i1 - 1;
      for (int f = i0; f <= f_end; ++f) {
        store_flag(a.fyflag + (size_t)(f - pad) * 4 * a.qm_stride + 4 * bx + (threadIdx.x >> 5),
                   false);
      }
    };
    if constexpr (kFirst) {
      // At rest in both directions, and every cell's round trip exact.
      bool sk = tile_vel_still(a, i0 - 2, i1 + 2, cb - 2, cb + kCols + 2);
      if (sk && !rest_cells(a, i0, i1, cb, min(cb + kCols, a.nx - pad))) {
        sk = block_round_trip_exact(s.r_in, s.e_in, a.nx, i0, i1, jj, col_ok);
      }
      if (threadIdx.x == 0) {
        store_flag(s.skip + (size_t)by * s.skip_tiles_x + bx, sk);
        if (!sk && a.moving) atomicAdd(a.moving, 1ull);
      }
      if (sk) {
        zero_flags();
        return;
      }
    } else {
      // The skip marks of bands by - 1 .. by + 1 of this column's x-sweep tile.
      unsigned sk3 = 0u;
      if (col_ok) {
        const int xt = (jj - pad) / (kCols - 1);
        for (int k = 0; k < 3; ++k) {
          const int b = by - 1 + k;
          if (b >= 0 && b < s.skip_bands && s.skip[(size_t)b * s.skip_tiles_x + xt]) {
            sk3 |= 1u << k;
          }
        }
      }
      // Every cell of the tile lies in a skipped tile: at rest, unchanged.
      if (__syncthreads_and(!col_ok || ((sk3 >> 1) & 1u))) {
        zero_flags();
        return;
      }
      if (__syncthreads_or(sk3 != 0u)) {
        FLOW_POW2_DISPATCH_ALL(
            a, a.pad + bx * kCols, a.pad + by * a.rows,
            (tile_mass_sweep_y_impl<R, kFirst, true, kEarly, kFl, true>(a, s, bx, by, sk3)),
            (tile_mass_sweep_y_impl<R, kFirst, false, kEarly, kFl, true>(a, s, bx, by, sk3)));
        return;  // (the dispatch returns only after its power-of-two branch)
      }
    }
  }
  FLOW_POW2_DISPATCH_ALL(
      a, a.pad + bx * kCols, a.pad + by * a.rows,
      (tile_mass_sweep_y_impl<R, kFirst, true, kEarly, kFl, false>(a, s, bx, by, 0u)),
      (tile_mass_sweep_y_impl<R, kFirst, false, kEarly, kFl, false>(a, s, bx, by, 0u)));
}

// ===========================================================================
// Advection of momentum (omp3/flow.c:557-970).

// MC-limited upwind value of a velocity at a flux point from its four
// neighbours along the direction (m2, m1 | p0, p1): omp3/flow.c:791-820.
template <typename R, bool kP2>
__device__ __forceinline__ R momentum_upwind(R wind, R m2, R m1, R p0, R p1,
                                             R inv_h, R d_left, R d_right,
                                             R dt_h) {
  const bool pos = Prec<R>::gt0(wind);
  return mc_face<R, kP2>(pos, m2, m1, p0, p1, inv_h, pos ? d_left : d_right, wind * dt_h);
}

// The momentum phase fuses each momentum flux with the update it feeds, so
// no flux array is written or read back: four kernels instead of eight.
// Velocities: StepArgs::u/v hold the velocities the Lagrangian phase left,
// in buffers the fused step has no other use for; the caller's arrays
// u_out/v_out receive the advected velocities.  The pair that recomputes a
// velocity (kVel) reads the old one from u/v and writes u_out/v_out, and the
// pairs after it read u_out/v_out -- no kernel writes an array it reads at
// other points, so tiles need no ordering between them.
//
// Pairs, each in the reference's arithmetic (omp3/flow.c:577-970):
//   x pair, rho_u: uF_x at cells (778-823) -> rho_u at x-faces (577-600)
//   x pair, rho_v: vF_x at corners (877-925) -> rho_v at y-faces (683-706)
//   y pair, rho_u: uF_y at corners (826-874) -> rho_u at x-faces (622-645)
//   y pair, rho_v: vF_y at cells (928-970) -> rho_v at y-faces (728-751)
// A flux the reference reads from a ghost point is the mirror source's
// (the reflective fill of the flux arrays, no sign change).

// FP64 form: a face's momentum minus dt_h * (fa - fb) / (hx * h) where the
// fluxes differ, stored; the momentum is read here unless kVel gave it.  A
// call, so that the warps which skip it skip its FP64 instructions (if
// converted to predicated code they would still take their FP64 issue
// slots).
template <bool kVel, bool kP2>
static __device__ __noinline__ double momentum_change(double* mom, double m, double fa, double fb,
                                                      double dt_h, double hx, double h,
                                                      double inv_h, double ihx) {
  using Pr = Prec<double>;
  const double diff = fa - fb;
  if (Pr::zero_skip_mem(diff)) return m;
  if (!kVel) m = *mom;
  m = Pr::template dsub<kP2>(m, dt_h * diff, hx * h, Pr::template mulp<kP2>(inv_h, ihx));
  *mom = m;
  return m;
}

// The momentum update of one face from its flux difference fa - fb, the
// velocity recomputed from the post-advection density when kVel (written to
// vout with its ghost images).  kU: an x-face (rho_u, u) else a y-face.
// h/inv_h: the divisor's row factor, hx/ihx its column factor; w0, w1 the
// face-density weights, ra, rb the densities either side and m_in the
// momentum (kVel; loaded by the caller, possibly a row ahead).
template <typename R, bool kU, bool kVel, bool kP2>
__device__ __forceinline__ void momentum_face_update(const StepArgs<R>& a, bool edge, int ii,
                                                     int jj, R fa, R fb, R dt_h, R hx, R ihx,
                                                     R h, R inv_h, R w0, R w1, R m_in, R ra,
                                                     R rb, R* vout) {
  using Pr = Prec<R>;
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const size_t f = fidx(nx, ii, jj);
  const size_t c = cidx(nx, ii, jj);
  R* mom = kU ? a.rho_u + f : a.rho_v + c;
  // mom - dt_h * diff / (hx * hy), the divisor rounded as the reference
  // forms it (omp3/flow.c:581-584); no flux difference, no change (in the
  // FP64 form equal fluxes in the whole warp skip the difference too).  The
  // momentum is read only where it is needed.
  R m = kVel ? m_in : R(0);
  if (!warp_same(fa, fb)) {
    if constexpr (Pr::kMixed) {
      const R diff = fa - fb;
      if (!Pr::zero_skip_mem(diff)) {
        if (!kVel) m = *mom;
        m = Pr::template dsub<kP2>(m, dt_h * diff, hx * h, Pr::template mulp<kP2>(inv_h, ihx));
        *mom = m;
      }
    } else {
      m = momentum_change<kVel, kP2>(mom, m, fa, fb, dt_h, hx, h, inv_h, ihx);
    }
  }
  if (kVel) {
    R rbar;
    // FP64 form, power-of-two tile: equal densities and weights either side
    // in the whole warp give the face density 2 (ra w0) exactly.
    if (kP2 && !Pr::kMixed && warp_all(lane_same(ra, rb) && lane_same(w0, w1))) {
      rbar = Pr::twice(Pr::template mulp<true>(ra, w0));
    } else {
      rbar = face_average<R, kP2>(ra, w0, rb, w1);
    }
    const R vel = face_velocity(m, rbar);
    if (kU) {
      vout[f] = vel;
      mirror(edge, vout, nx + 1, ny, pad, ii, jj, vel, true, false);
    } else {
      vout[c] = vel;
      mirror(edge, vout, nx, ny + 1, pad, ii, jj, vel, false, true);
    }
  }
}

// Whether no mass moves through any face of the cells in rows r0 .. r1 and
// columns c0 .. c1 (the mass-flux flags of the sweeps: x faces of those
// rows, y faces of rows r0 .. r1 + 1; ghost faces are copies of faces inside
// these ranges).  Block-uniform (barrier).  Then no cell there changed its
// density in the sweeps, and no momentum flux of those faces is non-zero.
template <typename R>
__device__ __forceinline__ bool tile_mass_still(const StepArgs<R>& a, int r0, int r1, int c0,
                                                int c1) {
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int xr0 = max(r0, pad), xr1 = min(r1, ny - pad - 1);
  const int xc0 = max(c0, pad), xc1 = min(c1, nx - pad);
  const int yr0 = max(r0, pad), yr1 = min(r1 + 1, ny - pad);
  const int yc0 = max(c0, pad), yc1 = min(c1, nx - pad - 1);
  // Flag bytes: x faces by x-sweep tile and warp, y faces by 32 columns.
  auto xbyte = [&](int c) {
    const int q = c - pad;
    return 4 * (q / (kCols - 1)) + ((q % (kCols - 1)) >> 5);
  };
  const int xb0 = xbyte(xc0), xnb = xc1 >= xc0 ? xbyte(xc1) - xb0 + 1 : 0;
  const int yb0 = (yc0 - pad) >> 5, ynb = yc1 >= yc0 ? ((yc1 - pad) >> 5) - yb0 + 1 : 0;
  const int nxt = max(0, xr1 - xr0 + 1) * xnb;
  const int total = nxt + max(0, yr1 - yr0 + 1) * ynb;
  bool any = false;
  for (int q = threadIdx.x; q < total; q += blockDim.x) {
    if (q < nxt) {
      const int r = xr0 + q / xnb, b = xb0 + q % xnb;
      any |= a.fxflag[(size_t)(r - pad) * a.fx_stride + b] != 0;
    } else {
      const int q2 = q - nxt;
      const int r = yr0 + q2 / ynb, b = yb0 + q2 % ynb;
      any |= a.fyflag[(size_t)(r - pad) * 4 * a.qm_stride + b] != 0;
    }
  }
  return __syncthreads_or(any) == 0;
}

// The velocities of a pair that recomputes them, where no mass moves around
// its faces: the momentum and both densities are what the Lagrangian phase
// formed the velocity from, so the advected velocity is the Lagrangian one
// (w), copied with its ghost images (rows i0 .. i1 - 1 of face column j;
// kU: x faces).  Loads in batches of eight rows, all in flight together;
// zero: the velocity flags show them all +0, which is stored without a load.
template <typename R, bool kU>
__device__ __forceinline__ void copy_velocities(const StepArgs<R>& a, bool edge, const R* w,
                                                R* vout, int i0, int i1, int j, bool ok,
                                                bool zero) {
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  constexpr int kB = 8;
  for (int ib = i0; ib < i1; ib += kB) {
    R v[kB];
#pragma unroll
    for (int q = 0; q < kB; ++q) {
      const int ii = ib + q;
      v[q] = (ok && ii < i1 && !zero) ? w[kU ? fidx(nx, ii, j) : cidx(nx, ii, j)] : R(0);
    }
#pragma unroll
    for (int q = 0; q < kB; ++q) {
      const int ii = ib + q;
      if (ok && ii < i1) {
        if (kU) {
          vout[fidx(nx, ii, j)] = v[q];
          mirror(edge, vout, nx + 1, ny, pad, ii, j, v[q], true, false);
        } else {
          vout[cidx(nx, ii, j)] = v[q];
          mirror(edge, vout, nx, ny + 1, pad, ii, j, v[q], false, true);
        }
      }
    }
  }
}

// x pairs: the flux points of a row are spread over the CTA's threads and
// shared through shared memory; 127 faces per CTA of 128 threads.
//   kV = false (rho_u): thread t holds the uF_x of cell c0 + t (c0 = pad-1 +
//     127 bx; ghost cells pad-1 and nx-pad take their mirror source's) and,
//     for t >= 1, updates x-face c0 + t from cells c0 + t - 1 and c0 + t.
//   kV = true (rho_v): thread t holds the vF_x of corner c0 + t (c0 = pad +
//     127 bx) and, for t < 127, updates y-face c0 + t from corners c0 + t and
//     c0 + t + 1.
template <typename R, bool kV, bool kVel, bool kP2, bool kRing, bool kFl>
__device__ __forceinline__ void tile_mom_x_impl(const StepArgs<R>& a, int bx, int by) {
  using Pr = Prec<R>;
  __shared__ R s_half[kMaxRows], s_h[kMaxRows], s_row[kMaxRows];
  __shared__ R s_wy0[kMaxRows], s_wy1[kMaxRows];
  __shared__ R sF[kCols];
  // kVel and kRing (the fused kernels): the update inputs of a face (its
  // momentum and the densities either side) stream through a per-thread
  // ring of asynchronous copies, kAhead rows ahead (no registers held for
  // them, no barrier: each thread reads back only what it copied).  Three
  // rows in the FP64 form, two in the mixed form (which measured slower with
  // three), as in every ring of the fused tiles.
  constexpr bool kUpdRing = kVel && kRing;
  constexpr int kAhead = Pr::kMixed ? 2 : 3, kSlots = kAhead + 1;
  auto s_upd = ring_slots<R, kUpdRing ? kSlots : 1, 3, kUpdRing ? kCols : 1, 2>();
  // The other pairs (no velocity update), FP64 form: a row's mass fluxes (and
  // for rho_v the u at the corner) stream through the ring instead.  (The
  // mixed form measured slower with it.)
  constexpr bool kFluxRing = !kVel && kRing && !Pr::kMixed;
  auto s_flux = ring_slots<R, kFluxRing ? kSlots : 1, 2, kFluxRing ? kCols : 1, 3>();
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int t = threadIdx.x;
  const int c0 = (kV ? pad : pad - 1) + bx * (kCols - 1);
  const int j = c0 + t;
  const int i0 = pad + by * a.rows;
  const bool edge = tile_near_edge(nx, ny, pad, c0, i0, a.rows);
  const int i1 = min(i0 + a.rows, kV ? ny + 1 - pad : ny - pad);
  if constexpr (kVel && kFl) {
    // No mass moves around the tile's faces: the Lagrangian velocities stand.
    if (tile_mass_still(a, i0 - 1, i1, c0 - 1, c0 + kCols)) {
      const bool upd = kV ? (t < kCols - 1 && j < nx - pad) : (t >= 1 && j < nx + 1 - pad);
      const bool zero = tile_vel_still(a, i0 - 2, i1 + 2, c0 - 2, c0 + kCols + 2);
      // Velocities all +0 whose cells were at rest through the previous
      // step, when this pair stored (or kept) +0 for each of them: they stand.
      if (zero && rest_cells(a, i0 - 1, i1, c0 - 1, c0 + kCols)) return;
      copy_velocities<R, !kV>(a, edge, kV ? a.v : a.u, kV ? a.v_out : a.u_out, i0, i1, j, upd,
                              zero);
      return;
    }
  }
  if (t < a.rows) {
    const int ii = i0 + t;
    if (ii < ny) {
      // Flux: edgedy/2 (uF_x) or celldy/2 (vF_x); update divisor: celldy.
      s_half[t] = geo_half<R>(kV ? a.celldy[ii] : a.edgedy[ii]);
      s_h[t] = geo_v<R>(a.celldy[ii]);
      s_row[t] = geo_rcp<R, kP2>(a.celldy[ii]);
      if (kV && kVel) {
        s_wy0[t] = geo_half_ratio<R, kP2>(a.celldy[ii], a.edgedy[ii]);
        s_wy1[t] = geo_half_ratio<R, kP2>(a.celldy[ii - 1], a.edgedy[ii]);
      }
    }
  }
  // kFl: the mass-flux flags of rows i0 - 1 .. i1 - 1 (each at its mirror
  // source row) for x-sweep tiles bx - 1 .. bx + 1, which hold every face
  // this tile reads; a mass flux flagged +0 is not loaded.  A pair that does
  // not recompute a velocity has nothing to do where no mass moves.
  __shared__ unsigned s_fxw[kFl ? kMaxRows + 1 : 1][3];
  if constexpr (kFl) {
    unsigned w = 0u;
    const int k = t / 3, sel = t - 3 * k;
    if (k <= i1 - i0) {
      int r = i0 - 1 + k;
      r = r < pad ? 2 * pad - 1 - r : (r >= ny - pad ? 2 * (ny - pad) - 1 - r : r);
      const int wi = bx - 1 + sel;
      if (wi >= 0 && 4 * wi < a.fx_stride) {
        w = reinterpret_cast<const unsigned*>(a.fxflag + (size_t)(r - pad) * a.fx_stride)[wi];
      }
      s_fxw[k][sel] = w;
    }
    if (!__syncthreads_or(w != 0u) && !kVel) return;
  }
  // The flag of the mass flux of face column jf in row r (i0 - 1 <= r < i1).
  auto fxf = [&](int r, int jf) -> bool {
    if constexpr (!kFl) {
      return true;
    } else {
      const int q = jf - pad;
      const int tile = q / (kCols - 1);
      const int tt = q - (kCols - 1) * tile;
      return ((s_fxw[r - i0 + 1][tile - bx + 1] >> (8 * (tt >> 5))) & 0xffu) != 0u;
    }
  };
  // The flux point: cells pad-1 .. nx-pad (rho_u), corners pad .. nx-pad (rho_v).
  const bool flux_ok = kV ? (j < nx + 1 - pad) : (j <= nx - pad);
  const int js = kV ? j : (j < pad ? 2 * pad - 1 - j : (j >= nx - pad ? 2 * (nx - pad) - 1 - j : j));
  const bool upd = kV ? (t < kCols - 1 && j < nx - pad) : (t >= 1 && j < nx + 1 - pad);
  R iex = R(0), cxl = R(0), cxr = R(0), hx = R(0), ihx = R(0), wx0 = R(0), wx1 = R(0);
  if (flux_ok) {
    iex = geo_rcp<R, kP2>(a.edgedx[js]);
    cxl = geo_v<R>(a.celldx[js - 1]);
    cxr = geo_v<R>(a.celldx[js]);
  }
  if (upd) {
    hx = geo_v<R>(a.edgedx[j]);
    ihx = geo_rcp<R, kP2>(a.edgedx[j]);
    if (!kV && kVel) {
      wx0 = geo_half_ratio<R, kP2>(a.celldx[j], a.edgedx[j]);
      wx1 = geo_half_ratio<R, kP2>(a.celldx[j - 1], a.edgedx[j]);
    }
  }
  const R dt_h = Pr::from_d(a.dt_slot[1]);
  // Velocities the fluxes read: rho_u's uF_x reads u before its update when
  // this pair updates it, else after; rho_v's vF_x reads the advected u and
  // v before or after its own update likewise.
  const R* uu = (!kV && kVel) ? a.u : a.u_out;
  const R* vv = kVel ? a.v : a.v_out;
  R* const vout = kV ? a.v_out : a.u_out;
  // Row ii+1's mass fluxes (and for rho_v the u below and at the corner) are
  // loaded before row ii is processed; the first row's before the barrier
  // that publishes the row tables.
  R Fa_n = R(0), Fb_n = R(0), u0_n = R(0);
  R F_dn = R(0), u_dn = R(0);
  auto load = [&](int ii) {
    if (!flux_ok) return;
    const size_t f = fidx(nx, ii, js);
    Fa_n = fxf(ii, js) ? a.F_x[f] : R(0);
    Fb_n = (kV || !fxf(ii, js + 1)) ? R(0) : a.F_x[f + 1];
    if (kV) u0_n = uu[f];
  };
  auto issue_flux = [&](int ii) {
    const int sl = (ii - i0) % kSlots;
    const size_t f = fidx(nx, ii, js);
    const bool pa = flux_ok && fxf(ii, js);
    const bool pb = flux_ok && (kV || fxf(ii, js + 1));
    cp_async_elem(&s_flux[sl][0][t], pa ? a.F_x + f : a.F_x, pa);
    cp_async_elem(&s_flux[sl][1][t], pb ? (kV ? uu + f : a.F_x + f + 1) : a.F_x, pb);
  };
  if (i0 < i1) {
    if (kV && flux_ok) {
      const size_t f = fidx(nx, i0 - 1, j);
      F_dn = fxf(i0 - 1, j) ? a.F_x[f] : R(0);
      u_dn = uu[f];
    }
    if constexpr (kFluxRing) {
#pragma unroll
      for (int d = 0; d < kAhead; ++d) {
        if (i0 + d < i1) issue_flux(i0 + d);
        cp_async_commit();
      }
    } else {
      load(i0);
    }
  }
  auto issue_upd = [&](int ii) {
    const int sl = (ii - i0) % kSlots;
    const size_t c = cidx(nx, ii, j);
    const R* mp = kV ? a.rho_v + c : a.rho_u + fidx(nx, ii, j);
    const R* rbp = kV ? a.rho_r + c - nx : a.rho_r + c - 1;
    cp_async_elem(&s_upd[sl][0][t], upd ? mp : a.rho_r, upd);
    cp_async_elem(&s_upd[sl][1][t], upd ? a.rho_r + c : a.rho_r, upd);
    cp_async_elem(&s_upd[sl][2][t], upd ? rbp : a.rho_r, upd);
  };
  if constexpr (kUpdRing) {
#pragma unroll
    for (int d = 0; d < kAhead; ++d) {
      if (i0 + d < i1) issue_upd(i0 + d);
      cp_async_commit();
    }
  }
  __syncthreads();
  if (i0 >= i1) {
    if constexpr (kUpdRing || kFluxRing) cp_async_wait<0>();
    return;
  }
  for (int ii = i0; ii < i1; ++ii) {
    const int k = ii - i0;
    R Fa, Fb, u0;
    if constexpr (kFluxRing) {
      cp_async_wait<kAhead - 1>();  // row ii's group has landed
      const int sl = k % kSlots;
      Fa = s_flux[sl][0][t];
      Fb = kV ? R(0) : s_flux[sl][1][t];
      u0 = kV ? s_flux[sl][1][t] : R(0);
      if (ii + kAhead < i1) issue_flux(ii + kAhead);
      cp_async_commit();
    } else {
      Fa = Fa_n;
      Fb = Fb_n;
      u0 = u0_n;
      if (ii + 1 < i1) load(ii + 1);
    }
    R val = R(0);
    if (flux_ok) {
      const size_t f = fidx(nx, ii, js);
      if (!kV) {
        if (warp_zeros(Fa, Fb)) {
          // FP64 form: no mass through any cell of the warp; the flux is the
          // zero mass (a zero sum scaled by a positive spacing).
          val = sum_zeros(Fa, Fb);
        } else {
          const R ua = uu[f], ub = uu[f + 1];
          const R mass = Pr::template mulp<kP2>(Fa + Fb, s_half[k]);
          // No mass through the cell, no momentum flux.
          val = Pr::zero_skip_coarse(mass)
                    ? mass
                    : mass * momentum_upwind<R, kP2>(Pr::half(ua + ub), uu[f - 1], ua, ub,
                                                     uu[f + 2], iex, cxl, cxr, dt_h);
        }
      } else {
        const size_t c = cidx(nx, ii, js);
        if (warp_zeros(Fa, F_dn)) {
          val = sum_zeros(Fa, F_dn);  // FP64 form: no mass through any corner of the warp
        } else {
          const R mass = Pr::template mulp<kP2>(Fa + F_dn, s_half[k]);
          val = Pr::zero_skip_coarse(mass)
                    ? mass
                    : mass * momentum_upwind<R, kP2>(Pr::half(u0 + u_dn), vv[c - 2], vv[c - 1],
                                                     vv[c], vv[c + 1], iex, cxl, cxr, dt_h);
        }
        F_dn = Fa;
        u_dn = u0;
      }
    }
    sF[t] = val;
    __syncthreads();
    if (upd) {
      const R fa = kV ? sF[t + 1] : sF[t];
      const R fb = kV ? sF[t] : sF[t - 1];
      const size_t c = cidx(nx, ii, j);
      R m = R(0), ra = R(0), rb = R(0);
      if constexpr (kUpdRing) {
        cp_async_wait<kAhead - 1>();  // row ii's group has landed
        const int sl = k % kSlots;
        m = s_upd[sl][0][t];
        ra = s_upd[sl][1][t];
        rb = s_upd[sl][2][t];
        if (ii + kAhead < i1) issue_upd(ii + kAhead);
        cp_async_commit();
      } else if (kVel) {
        m = kV ? a.rho_v[c] : a.rho_u[fidx(nx, ii, j)];
        ra = a.rho_r[c];
        rb = kV ? a.rho_r[c - nx] : a.rho_r[c - 1];
      }
      momentum_face_update<R, !kV, kVel, kP2>(a, edge, ii, j, fa, fb, dt_h, hx, ihx, s_h[k],
                                              s_row[k], kV ? s_wy0[k] : wx0,
                                              kV ? s_wy1[k] : wx1, m, ra, rb, vout);
    }
    __syncthreads();
  }
  if constexpr (kUpdRing || kFluxRing) cp_async_wait<0>();
}

// y pairs: each thread marches down its column, carrying the flux of the
// previous row.
//   kV = false (rho_u): uF_y at corners i0 .. i1 of column jj (u window
//     rows ci-2 .. ci+1), updates x-faces i0 .. i1-1 from corners ii, ii+1.
//   kV = true (rho_v): vF_y at cells i0-1 .. i1-1 (v window rows ci-1 ..
//     ci+2; the ghost rows pad-1 and ny-pad take their mirror source's),
//     updates y-faces i0 .. i1-1 from cells ii-1, ii.
// The windows form their differences only where mass moves in the warp
// (FP64 form), as the y mass sweep does.
template <typename R, bool kV, bool kVel, bool kP2, bool kRing, bool kFl>
__device__ __forceinline__ void tile_mom_y_impl(const StepArgs<R>& a, int bx, int by) {
  using Pr = Prec<R>;
  // kVel and kRing (the fused kernels): the update inputs of a face stream
  // through a per-thread ring of asynchronous copies, kAhead rows ahead (as
  // in the x pairs).
  constexpr bool kUpdRing = kVel && kRing;
  constexpr int kAhead = Pr::kMixed ? 2 : 3, kSlots = kAhead + 1;
  auto s_upd = ring_slots<R, kUpdRing ? kSlots : 1, 3, kUpdRing ? kCols : 1, 4>();
  // The other pairs (no velocity update): the mass fluxes and window value of
  // the flux rows stream through the ring instead.
  constexpr bool kFluxRing = !kVel && kRing;
  auto s_flux = ring_slots<R, kFluxRing ? kSlots : 1, 3, kFluxRing ? kCols : 1, 5>();
  // Flux tables over flux rows q = ci - fr0 (fr0 the first flux row): 1/edgedy
  // of the row, celldy of the row below (s_cy[q]) and of the row (s_cy[q + 1]).
  __shared__ R s_iey[kMaxRows + 2], s_cy[kMaxRows + 3];
  __shared__ R s_h[kMaxRows], s_row[kMaxRows], s_wy0[kMaxRows], s_wy1[kMaxRows];
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int jj = pad + bx * kCols + threadIdx.x;
  const int i0 = pad + by * a.rows;
  const bool edge = tile_near_edge(nx, ny, pad, pad + bx * kCols, i0, a.rows);
  const int i1 = min(i0 + a.rows, kV ? ny + 1 - pad : ny - pad);
  if constexpr (kVel && kFl) {
    // No mass moves around the tile's faces: the Lagrangian velocities stand.
    const int cb = pad + bx * kCols;
    if (tile_mass_still(a, i0 - 1, i1, cb - 1, cb + kCols)) {
      const bool zero = tile_vel_still(a, i0 - 2, i1 + 2, cb - 2, cb + kCols + 2);
      if (zero && rest_cells(a, i0 - 1, i1, cb - 1, cb + kCols)) return;
      copy_velocities<R, !kV>(a, edge, kV ? a.v : a.u, kV ? a.v_out : a.u_out, i0, i1, jj,
                              jj < (kV ? nx - pad : nx + 1 - pad), zero);
      return;
    }
  }
  // Flux rows: corners i0 .. i1 (rho_u); cells i0-1 .. i1-1 (rho_v), a ghost
  // row computed at its mirror source.
  const int fr0 = kV ? i0 - 1 : i0;
  const int nfr = i1 - i0 + 1;
  auto src_row = [&](int ci) {
    if (!kV) return ci;
    return ci < pad ? 2 * pad - 1 - ci : (ci >= ny - pad ? 2 * (ny - pad) - 1 - ci : ci);
  };
  // (Entries of a ghost flux row are never used: its flux is its mirror
  // source's.)
  for (int q = threadIdx.x; q <= nfr; q += kCols) {
    const int ci = fr0 + q;
    if (q < nfr) s_iey[q] = geo_rcp<R, kP2>(a.edgedy[ci]);
    s_cy[q] = geo_v<R>(a.celldy[ci - 1]);
  }
  if (threadIdx.x < a.rows) {
    const int ii = i0 + threadIdx.x;
    if (ii < ny) {
      // Update divisor row factor: edgedy for both y pairs.
      s_h[threadIdx.x] = geo_v<R>(a.edgedy[ii]);
      s_row[threadIdx.x] = geo_rcp<R, kP2>(a.edgedy[ii]);
      if (kV && kVel) {
        s_wy0[threadIdx.x] = geo_half_ratio<R, kP2>(a.celldy[ii], a.edgedy[ii]);
        s_wy1[threadIdx.x] = geo_half_ratio<R, kP2>(a.celldy[ii - 1], a.edgedy[ii]);
      }
    }
  }
  // kFl: the mass-flux flags of y-face rows i0 - 1 .. i1 for column tiles
  // bx - 1 and bx, which hold every face this tile reads; a mass flux flagged
  // +0 is not loaded.  A pair that does not recompute a velocity has nothing
  // to do where no mass moves.
  __shared__ unsigned s_fyw[kFl ? kMaxRows + 2 : 1][2];
  if constexpr (kFl) {
    unsigned w0 = 0u, w1 = 0u;
    const int k = threadIdx.x;
    if (k <= i1 - i0 + 1) {
      const int f = i0 - 1 + k;
      if (f >= pad && f <= ny - pad) {
        const unsigned* row =
            reinterpret_cast<const unsigned*>(a.fyflag) + (size_t)(f - pad) * a.qm_stride;
        w0 = bx >= 1 ? row[bx - 1] : 0u;
        w1 = bx < a.qm_stride ? row[bx] : 0u;
      }
      s_fyw[k][0] = w0;
      s_fyw[k][1] = w1;
    }
    if (!__syncthreads_or((w1 | (w0 & 0xff000000u)) != 0u) && !kVel) return;
  } else {
    __syncthreads();
  }
  // The flag of the mass flux of y-face row f (i0 - 1 <= f <= i1) and column
  // col (a ghost column at its mirror source, an identical copy).
  auto fyf = [&](int f, int col) -> bool {
    if constexpr (!kFl) {
      return true;
    } else {
      col = col < pad ? 2 * pad - 1 - col : (col >= nx - pad ? 2 * (nx - pad) - 1 - col : col);
      return qflag(s_fyw[f - i0 + 1][0], s_fyw[f - i0 + 1][1], col, pad, bx);
    }
  };
  if (jj >= (kV ? nx - pad : nx + 1 - pad) || i0 >= i1) return;
  const R dt_h = Pr::from_d(a.dt_slot[1]);
  const R hcol = geo_half<R>(kV ? a.celldx[jj] : a.edgedx[jj]);  // flux: celldx/2 or edgedx/2
  const R hx = geo_v<R>(a.celldx[jj]);
  const R ihx = geo_rcp<R, kP2>(a.celldx[jj]);
  R wx0 = R(0), wx1 = R(0);
  if (!kV && kVel) {
    wx0 = geo_half_ratio<R, kP2>(a.celldx[jj], a.edgedx[jj]);
    wx1 = geo_half_ratio<R, kP2>(a.celldx[jj - 1], a.edgedx[jj]);
  }
  // The window's velocity: before this pair's update when it recomputes it.
  const R* w = kV ? (kVel ? a.v : a.v_out) : (kVel ? a.u : a.u_out);
  const R* vwind = a.v;  // rho_u's wind: v before the rho_v pairs
  R* const vout = kV ? a.v_out : a.u_out;
  auto widx = [&](int row) { return kV ? cidx(nx, row, jj) : fidx(nx, row, jj); };
  // Window of flux row ci: rows ci-2 .. ci+1 (corners) or ci-1 .. ci+2 (cells).
  const int wlo = kV ? -1 : -2;
  ColWindow<R> win;
  int wrow = src_row(fr0);  // flux row the window is at
  win.m2 = w[widx(wrow + wlo)];
  win.m1 = w[widx(wrow + wlo + 1)];
  win.p0 = w[widx(wrow + wlo + 2)];
  win.p1 = w[widx(wrow + wlo + 3)];
  bool fresh = false;
  // Flux at flux row ci (the window at ci) from its mass fluxes Fa, Fb; q its
  // table index.
  auto flux_at = [&](int ci, int q, R Fa, R Fb) -> R {
    const size_t c = cidx(nx, ci, jj);
    if (warp_zeros(Fa, Fb)) {
      fresh = false;  // the window shifts its values alone until mass moves
      return sum_zeros(Fa, Fb);
    }
    // The window moves by values alone (a push per row); its differences are
    // formed here, on the moving path only: shifted from the row before when
    // that row moved, else all of them.  (A shift per row under a branch
    // would be predicated code, its FP64 subtractions taking FP64 issue
    // slots in every warp at rest.)
    if (fresh) win.advance();
    else win.refresh();
    fresh = true;
    const R mass = Pr::template mulp<kP2>(Fa + Fb, hcol);
    if (Pr::zero_skip_coarse(mass)) return mass;
    const R wind = kV ? Pr::half(win.m1 + win.p0) : Pr::half(vwind[c - 1] + vwind[c]);
    const bool pos = Pr::gt0(wind);
    return mass * win.template face<kP2>(pos, s_iey[q], pos ? s_cy[q] : s_cy[q + 1], wind * dt_h);
  };
  // The mass fluxes of flux row ci and the value that moves the window there
  // from row ci-1, loaded a row ahead of their use.
  R Fa_n = R(0), Fb_n = R(0), wv_n = R(0);
  auto load = [&](int ci) {
    const size_t c = cidx(nx, ci, jj);
    Fa_n = fyf(ci, jj) ? a.F_y[c] : R(0);
    Fb_n = (kV ? fyf(ci + 1, jj) : fyf(ci, jj - 1)) ? (kV ? a.F_y[c + nx] : a.F_y[c - 1]) : R(0);
    wv_n = w[widx(ci + wlo + 3)];
  };
  // The flux rows a column consumes are consecutive: from the window's first
  // row to the last row that is not a ghost (kFluxRing: one copy group per
  // row, in that order).
  const int w0row = wrow;
  const int rmax = kV ? min(i1 - 1, ny - pad - 1) : i1;
  auto issue_flux = [&](int ci) {
    const int sl = (ci - w0row) % kSlots;
    const size_t c = cidx(nx, ci, jj);
    cp_async_elem(&s_flux[sl][0][threadIdx.x], a.F_y + c, fyf(ci, jj));
    cp_async_elem(&s_flux[sl][1][threadIdx.x], kV ? a.F_y + c + nx : a.F_y + c - 1,
                  kV ? fyf(ci + 1, jj) : fyf(ci, jj - 1));
    cp_async_elem(&s_flux[sl][2][threadIdx.x], w + widx(ci + wlo + 3), true);
  };
  // Row ci's values from the ring (its group waited for), the row kAhead
  // rows on issued.
  auto take_flux = [&](int ci, R* Fa, R* Fb, R* wv) {
    cp_async_wait<kAhead - 1>();
    const int sl = (ci - w0row) % kSlots;
    *Fa = s_flux[sl][0][threadIdx.x];
    *Fb = s_flux[sl][1][threadIdx.x];
    *wv = s_flux[sl][2][threadIdx.x];
    if (ci + kAhead <= rmax) issue_flux(ci + kAhead);
    cp_async_commit();
  };
  R prev;
  if constexpr (kFluxRing) {
#pragma unroll
    for (int d = 0; d < kAhead; ++d) {
      if (w0row + d <= rmax) issue_flux(w0row + d);
      cp_async_commit();
    }
    R Fa, Fb, wv;
    take_flux(wrow, &Fa, &Fb, &wv);
    prev = flux_at(wrow, wrow - fr0, Fa, Fb);
  } else {
    load(wrow);
    prev = flux_at(wrow, wrow - fr0, Fa_n, Fb_n);
  }
  const R top = prev;  // rho_v: the flux of the first flux row's mirror source
  // The update inputs of face row ii (momentum and densities, kVel), loaded a
  // row ahead; rho_v's lower density is the row below's upper one.
  R m_n = R(0), ra_n = R(0), rb_n = R(0);
  auto load_upd = [&](int ii) {
    if (!kVel) return;
    const size_t c = cidx(nx, ii, jj);
    m_n = kV ? a.rho_v[c] : a.rho_u[fidx(nx, ii, jj)];
    rb_n = kV ? ra_n : a.rho_r[c - 1];
    ra_n = a.rho_r[c];
  };
  const int t = threadIdx.x;
  auto issue_upd = [&](int ii) {
    const int sl = (ii - i0) % kSlots;
    const size_t c = cidx(nx, ii, jj);
    cp_async_elem(&s_upd[sl][0][t], kV ? a.rho_v + c : a.rho_u + fidx(nx, ii, jj), true);
    cp_async_elem(&s_upd[sl][1][t], a.rho_r + c, true);
    cp_async_elem(&s_upd[sl][2][t], kV ? a.rho_r + c - nx : a.rho_r + c - 1, true);
  };
  if constexpr (kUpdRing) {
#pragma unroll
    for (int d = 0; d < kAhead; ++d) {
      if (i0 + d < i1) issue_upd(i0 + d);
      cp_async_commit();
    }
  } else {
    if (kVel && kV) ra_n = a.rho_r[cidx(nx, i0 - 1, jj)];
    load_upd(i0);
  }
  // A loop row computes its flux row unless that is a ghost row or (bottom
  // wall) the row computed above.
  const bool bottom = kV && fr0 != src_row(fr0);
  if (kFluxRing) {
    // (the ring holds the next rows already)
  } else if (i0 < i1 && !(bottom && i0 == src_row(fr0)) &&
             src_row(kV ? i0 : i0 + 1) == (kV ? i0 : i0 + 1)) {
    load(kV ? i0 : i0 + 1);
  } else if (bottom && i0 + 1 < i1) {
    load(i0 + 1);
  }
  for (int ii = i0; ii < i1; ++ii) {
    const int k = ii - i0;
    // The new flux row: corner ii+1 (rho_u), cell ii (rho_v).
    const int ci = kV ? ii : ii + 1;
    const int cs = src_row(ci);
    R cur;
    if (kV && cs != ci) {
      // A ghost row (top wall): its mirror source is the previous flux row.
      cur = prev;
    } else if (bottom && ci == wrow) {
      cur = top;  // the bottom wall's first interior row: computed already
    } else {
      R Fa, Fb, wv;
      if constexpr (kFluxRing) {
        take_flux(ci, &Fa, &Fb, &wv);
      } else {
        Fa = Fa_n;
        Fb = Fb_n;
        wv = wv_n;
        const int cn = ci + 1;
        if (ii + 1 < i1 && src_row(cn) == cn) load(cn);
      }
      win.push(wv);
      ++wrow;
      cur = flux_at(cs, cs - fr0, Fa, Fb);
    }
    R m, ra, rb;
    if constexpr (kUpdRing) {
      cp_async_wait<kAhead - 1>();  // row ii's group has landed
      const int sl = k % kSlots;
      m = s_upd[sl][0][t];
      ra = s_upd[sl][1][t];
      rb = s_upd[sl][2][t];
      if (ii + kAhead < i1) issue_upd(ii + kAhead);
      cp_async_commit();
    } else {
      m = m_n;
      ra = ra_n;
      rb = rb_n;
      if (ii + 1 < i1) load_upd(ii + 1);
    }
    momentum_face_update<R, !kV, kVel, kP2>(a, edge, ii, jj, cur, prev, dt_h, hx, ihx, s_h[k],
                                            s_row[k], kV ? s_wy0[k] : wx0, kV ? s_wy1[k] : wx1,
                                            m, ra, rb, vout);
    prev = cur;
  }
  if constexpr (kUpdRing || kFluxRing) cp_async_wait<0>();
}

template <typename R, bool kV, bool kVel, bool kRing = true, bool kFl = false>
__device__ __forceinline__ void tile_mom_x(const StepArgs<R>& a, int bx, int by) {
  FLOW_POW2_DISPATCH(R, a, (kV ? a.pad : a.pad - 1) + bx * (kCols - 1), a.pad + by * a.rows,
                     (tile_mom_x_impl<R, kV, kVel, true, kRing, kFl>(a, bx, by)),
                     (tile_mom_x_impl<R, kV, kVel, false, kRing, kFl>(a, bx, by)));
}
template <typename R, bool kV, bool kVel, bool kRing = true, bool kFl = false>
__device__ __forceinline__ void tile_mom_y(const StepArgs<R>& a, int bx, int by) {
  FLOW_POW2_DISPATCH(R, a, a.pad + bx * kCols, a.pad + by * a.rows,
                     (tile_mom_y_impl<R, kV, kVel, true, kRing, kFl>(a, bx, by)),
                     (tile_mom_y_impl<R, kV, kVel, false, kRing, kFl>(a, bx, by)));
}

}  // namespace tiles
}  // namespace flow
