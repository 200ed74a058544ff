// stages.cu -- the per-function kernels of the GB300 flow kernel set.
//
// One kernel per loop of the reference timestep (omp3/flow.c) plus the device
// ghost fill, the CFL minimum and the conservation totals.  These back the
// individual entry points of omp3/flow.h:4-88 (equation_of_state,
// pressure_acceleration, ...), so that a host driver can call any stage on its
// own, and they form the "exact" timestep: this file is compiled without
// floating-point contraction (--fmad=false) and evaluates every expression in
// the reference's order, so each entry point reproduces the reference's IEEE
// results bit for bit.  The fused, faster timestep lives in fused.cu.
//
// Every kernel is a 2-D launch: x over columns (coalesced), y over rows.
#include <atomic>

#include "common.cuh"
#include "stages.h"

namespace flow {
namespace {

constexpr int kBX = 64;
constexpr int kBY = 4;

inline dim3 grid_for(int rows, int cols) {
  return dim3((unsigned)((cols + kBX - 1) / kBX),
              (unsigned)((rows + kBY - 1) / kBY));
}
#define FLOW_POINT(i0, i1, j0, j1)                                   \
  const int jj = (j0) + (int)(blockIdx.x * blockDim.x + threadIdx.x); \
  const int ii = (i0) + (int)(blockIdx.y * blockDim.y + threadIdx.y); \
  if (ii >= (i1) || jj >= (j1)) return;

// Volume-weighted density on an x-face / y-face (omp3/flow.c:134-141).
__device__ __forceinline__ double rho_xface(int nx, const double* rho,
                                            const double* edgedx,
                                            const double* celldx,
                                            const double* celldy, int ii,
                                            int jj) {
  return (rho[cidx(nx, ii, jj)] * celldx[jj] * celldy[ii] +
          rho[cidx(nx, ii, jj - 1)] * celldx[jj - 1] * celldy[ii]) /
         (2.0 * edgedx[jj] * celldy[ii]);
}
__device__ __forceinline__ double rho_yface(int nx, const double* rho,
                                            const double* edgedy,
                                            const double* celldx,
                                            const double* celldy, int ii,
                                            int jj) {
  return (rho[cidx(nx, ii, jj)] * celldx[jj] * celldy[ii] +
          rho[cidx(nx, ii - 1, jj)] * celldx[jj] * celldy[ii - 1]) /
         (2.0 * celldx[jj] * edgedy[ii]);
}

// ---------------------------------------------------------------------------
// Lagrangian phase.

__global__ void k_eos(int nx, int ny, double* P, const double* rho,
                      const double* e) {
  FLOW_POINT(0, ny, 0, nx);
  const size_t c = cidx(nx, ii, jj);
  P[c] = (kGam - 1.0) * rho[c] * e[c];
}

// Pressure (viscous = 0) or viscous-stress (viscous = 1) acceleration of the
// face momenta followed by the velocity update (omp3/flow.c:121-152 and
// 212-240): the two loops differ only in the force and its spacing.
template <int kViscous>
__global__ void k_accelerate(int nx, int ny, int pad, double dt,
                             double* rho_u, double* rho_v, double* u, double* v,
                             const double* fx, const double* fy,
                             const double* rho, const double* edgedx,
                             const double* edgedy, const double* celldx,
                             const double* celldy) {
  FLOW_POINT(pad, (ny + 1) - pad, pad, (nx + 1) - pad);
  const size_t f = fidx(nx, ii, jj);
  const size_t c = cidx(nx, ii, jj);
  const double hx = kViscous ? celldx[jj] : edgedx[jj];
  const double hy = kViscous ? celldy[ii] : edgedy[ii];
  rho_u[f] -= dt * (fx[c] - fx[c - 1]) / hx;
  rho_v[c] -= dt * (fy[c] - fy[c - nx]) / hy;
  const double rx = rho_xface(nx, rho, edgedx, celldx, celldy, ii, jj);
  const double ry = rho_yface(nx, rho, edgedy, celldx, celldy, ii, jj);
  u[f] = (rx == 0.0) ? 0.0 : rho_u[f] / rx;
  v[c] = (ry == 0.0) ? 0.0 : rho_v[c] / ry;
}

// Limited compressive velocity jumps (omp3/flow.c:177-198).
__device__ __forceinline__ void visc_jumps(double lo, double mid, double hi,
                                           double hi2, double* jump,
                                           double* curv) {
  *jump = dmin(0.0, hi - mid);
  *curv = 0.5 * (fabs(dmin(0.0, (hi2 - hi)) - dmin(0.0, (hi - mid))) +
                 fabs(dmin(0.0, (hi - mid)) - dmin(0.0, (mid - lo))));
}

__global__ void k_viscous_stress(int nx, int ny, int pad, double* Qxx,
                                 double* Qyy, const double* u, const double* v,
                                 const double* rho) {
  FLOW_POINT(pad, ny - pad, pad, nx - pad);
  const size_t f = fidx(nx, ii, jj);
  const size_t c = cidx(nx, ii, jj);
  double u_i, u_ii, v_i, v_ii;
  visc_jumps(u[f - 1], u[f], u[f + 1], u[f + 2], &u_i, &u_ii);
  visc_jumps(v[c - nx], v[c], v[c + nx], v[c + 2 * nx], &v_i, &v_ii);
  Qxx[c] = -kCQ * rho[c] * u_i * u_ii;
  Qyy[c] = -kCQ * rho[c] * v_i * v_ii;
}

__global__ void k_shock_heating(int nx, int ny, int pad, double dt_h,
                                double* e, const double* P, const double* u,
                                const double* v, const double* rho,
                                const double* Qxx, const double* Qyy,
                                const double* celldx, const double* celldy) {
  FLOW_POINT(pad, ny - pad, pad, nx - pad);
  const size_t f = fidx(nx, ii, jj);
  const size_t c = cidx(nx, ii, jj);
  const double r = rho[c];
  const double p = P[c];
  const double dudx = (u[f + 1] - u[f]) / celldx[jj];
  const double dvdy = (v[c + nx] - v[c]) / celldy[ii];
  const double div_dt = (dudx + dvdy) * dt_h;
  const double e_q = e[c] - dt_h * (Qxx[c] * dudx + Qyy[c] * dvdy) / r;
  const double rho_c = r / (1.0 + div_dt);
  const double e_c = e_q - (p * div_dt) / r;
  const double work = 0.5 * div_dt * (p + (kGam - 1.0) * e_c * rho_c) / r;
  e[c] = (r == 0.0) ? 0.0 : e_q - work;
}

// ---------------------------------------------------------------------------
// Reductions: per-thread partials over a grid-stride range of interior cells,
// warp shuffles, one partial per block in reduce_array, and the last block to
// finish combines the partials (single pass, no second launch).

__device__ __forceinline__ double warp_min(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = dmin(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}
__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

constexpr int kRedThreads = 256;

// Leapfrog update of omp3/flow.c:103-105 from the global CFL minimum g.
__device__ __forceinline__ void apply_dt_rule(double g, double dt_h_in, int first_step,
                                              double* ra) {
  const double limited = dmin(g, FLOW_C_M * dt_h_in);
  const double dt = 0.5 * (kCT * limited + dt_h_in);
  ra[kRaDt] = dt;
  ra[kRaDtH] = first_step ? dt : kCT * limited;
}

// local_only: a rank of a decomposed mesh keeps its minimum in ra[kRaMinBits]
// (the caller reduces it over the ranks and applies the rule, k_dt_rule).
__global__ void __launch_bounds__(kRedThreads)
    k_min_timestep(int nx, int ny, int pad, double max_dt, double dt_h_in,
                   int first_step, const double* Qxx, const double* Qyy,
                   const double* rho, const double* e, const double* celldx,
                   const double* celldy, double* ra, int local_only) {
  const int w = nx - 2 * pad;
  const long long n = (long long)w * (ny - 2 * pad);
  double m = max_dt;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int ii = pad + (int)(t / w);
    const int jj = pad + (int)(t % w);
    const size_t c = cidx(nx, ii, jj);
    const double sound = sqrt(kGam * (kGam - 1.0) * e[c]);
    const double cfl_x =
        celldx[jj] / sqrt(sound * sound + 2.0 * Qxx[c] / rho[c]);
    const double cfl_y =
        celldy[ii] / sqrt(sound * sound + 2.0 * Qyy[c] / rho[c]);
    m = dmin(m, dmin(cfl_x, cfl_y));
  }
  __shared__ double s_part[kRedThreads / 32];
  __shared__ bool s_last;
  m = warp_min(m);
  if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    double x = (threadIdx.x < kRedThreads / 32) ? s_part[threadIdx.x] : max_dt;
    x = warp_min(x);
    if (threadIdx.x == 0) {
      ra[kRaPartial + blockIdx.x] = x;
      __threadfence();
      unsigned long long* ticket = reinterpret_cast<unsigned long long*>(ra + kRaTicket);
      s_last = (atomicAdd(ticket, 1ull) == gridDim.x - 1);
    }
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double x = max_dt;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
    x = dmin(x, __ldcg(ra + kRaPartial + b));
  }
  x = warp_min(x);
  if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    double g = s_part[0];
    for (int k = 1; k < kRedThreads / 32; ++k) g = dmin(g, s_part[k]);
    if (local_only) {
      ra[kRaMinBits] = g;
    } else {
      apply_dt_rule(g, dt_h_in, first_step, ra);
    }
    *reinterpret_cast<unsigned long long*>(ra + kRaTicket) = 0ull;
  }
}

__global__ void k_dt_rule(double g, double dt_h_in, int first_step, double* ra) {
  if (threadIdx.x == 0) apply_dt_rule(g, dt_h_in, first_step, ra);
}

// Partial sums of one thread: two (mass, energy) pairs.
struct ConsSums {
  double m0, e0, m1, e1;
};

// The FP64 work of the conservation sums sits in calls, so that a warp that
// skips it skips its instructions (a predicated FP64 instruction still takes
// its issue slots on the FP64 pipe).  plain: bit q set where group q is summed.
__device__ __noinline__ ConsSums cons_add_groups(ConsSums s, unsigned plain, double d0,
                                                 double d1, double d2, double d3, double f0,
                                                 double f1, double f2, double f3) {
  if (plain & 1u) {
    s.m0 += d0;
    s.e0 = fma(d0, f0, s.e0);
  }
  if (plain & 2u) {
    s.m1 += d1;
    s.e1 = fma(d1, f1, s.e1);
  }
  if (plain & 4u) {
    s.m0 += d2;
    s.e0 = fma(d2, f2, s.e0);
  }
  if (plain & 8u) {
    s.m1 += d3;
    s.e1 = fma(d3, f3, s.e1);
  }
  return s;
}
// A run of n groups of 32 cells holding one (rho, e) pair: n*rho and
// n*(rho*e) per lane.
__device__ __noinline__ ConsSums cons_add_run(ConsSums s, int n, unsigned long long r_bits,
                                              unsigned long long e_bits) {
  const double dn = (double)n, r = __longlong_as_double(r_bits);
  s.m1 += dn * r;
  s.e1 += dn * (r * __longlong_as_double(e_bits));
  return s;
}

// The interior is cut into chunks of 4 x 256 columns of one row (each warp
// 4 groups of 32 consecutive cells) and the chunks are dealt to the blocks in
// turn: a block loads its next chunk before it sums the current one (16 loads
// of independent columns in flight per thread), into two pairs of sums, rho*e
// contracted into one FMA -- two FP64 instructions per cell, the FP64 pipe's
// share of this reduction on GB300.  The grid is one wave of resident blocks.
// Columns past the last whole chunk of a row (rows whose interior is not a
// multiple of 1024 wide) are summed after the chunks, by 256-column groups
// and a ragged end.  A group whose 32 cells hold one (rho, e) pair (bit for
// bit; the fluid at rest around a blast) is counted instead: the warp keeps
// the pair of its current run of such groups and their number, and adds
// n*rho and n*(rho*e) per lane when the run ends -- integer work in place of
// 64 FP64 instructions per group, and the same sum to rounding.
constexpr int kConsChunk = 4 * kRedThreads;

__global__ void __launch_bounds__(kRedThreads)
    k_conservation(int nx, int ny, int pad, const double* __restrict__ rho,
                   const double* __restrict__ e, double* ra) {
  ConsSums acc{0.0, 0.0, 0.0, 0.0};
  unsigned long long run_r = 0ull, run_e = 0ull;  // warp-uniform
  int run_n = 0;
  // Group q of 32 cells of a warp: counted into the run (returns 0), or to be
  // summed (returns bit q).
  auto group = [&](double d, double f, int q) -> unsigned {
    const unsigned long long db = __double_as_longlong(d), fb = __double_as_longlong(f);
    const unsigned long long d0 = __shfl_sync(0xffffffffu, db, 0);
    const unsigned long long f0 = __shfl_sync(0xffffffffu, fb, 0);
    if (!__all_sync(0xffffffffu, db == d0 && fb == f0)) return 1u << q;
    if (d0 != run_r || f0 != run_e) {
      if (run_n > 0) acc = cons_add_run(acc, run_n, run_r, run_e);
      run_r = d0;
      run_e = f0;
      run_n = 0;
    }
    ++run_n;
    return 0u;
  };
  const int w = nx - 2 * pad, rows = ny - 2 * pad;
  const int t = threadIdx.x;
  const int per_row = w / kConsChunk;
  const long long chunks = (long long)rows * per_row;
  double d[4], f[4];
  auto load = [&](long long c, double* dd, double* ff) {
    const int r = (int)(c / per_row);
    const size_t base = (size_t)(pad + r) * nx + pad + (size_t)(c - (long long)r * per_row) * kConsChunk + t;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      dd[q] = rho[base + q * kRedThreads];
      ff[q] = e[base + q * kRedThreads];
    }
  };
  long long c = blockIdx.x;
  if (c < chunks) load(c, d, f);
  while (c < chunks) {
    const long long cn = c + gridDim.x;
    double dn[4], fn[4];
    if (cn < chunks) load(cn, dn, fn);
    unsigned plain = 0u;
#pragma unroll
    for (int q = 0; q < 4; ++q) plain |= group(d[q], f[q], q);
    if (plain) acc = cons_add_groups(acc, plain, d[0], d[1], d[2], d[3], f[0], f[1], f[2], f[3]);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      d[q] = dn[q];
      f[q] = fn[q];
    }
    c = cn;
  }
  if (per_row * kConsChunk < w) {
    for (int r = blockIdx.x; r < rows; r += gridDim.x) {
      const double* rr = rho + (size_t)(pad + r) * nx + pad;
      const double* er = e + (size_t)(pad + r) * nx + pad;
      int j0 = per_row * kConsChunk;
      for (; j0 + kRedThreads <= w; j0 += kRedThreads) {
        const double dd = rr[j0 + t], ff = er[j0 + t];
        if (group(dd, ff, 0)) acc = cons_add_groups(acc, 1u, dd, 0.0, 0.0, 0.0, ff, 0.0, 0.0, 0.0);
      }
      if (j0 + t < w) {
        acc.m0 += rr[j0 + t];
        acc.e0 = fma(rr[j0 + t], er[j0 + t], acc.e0);
      }
    }
  }
  if (run_n > 0) acc = cons_add_run(acc, run_n, run_r, run_e);
  double ms = acc.m0 + acc.m1, es = acc.e0 + acc.e1;
  __shared__ double s_m[kRedThreads / 32], s_e[kRedThreads / 32];
  __shared__ bool s_last;
  ms = warp_sum(ms);
  es = warp_sum(es);
  if ((threadIdx.x & 31) == 0) {
    s_m[threadIdx.x >> 5] = ms;
    s_e[threadIdx.x >> 5] = es;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < kRedThreads / 32; ++k) {
      a += s_m[k];
      b += s_e[k];
    }
    ra[kRaPartial + 2 * blockIdx.x] = a;
    ra[kRaPartial + 2 * blockIdx.x + 1] = b;
    __threadfence();
    unsigned long long* ticket = reinterpret_cast<unsigned long long*>(ra + kRaTicket);
    s_last = (atomicAdd(ticket, 1ull) == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double a = 0.0, b = 0.0;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
    a += __ldcg(ra + kRaPartial + 2 * k);
    b += __ldcg(ra + kRaPartial + 2 * k + 1);
  }
  a = warp_sum(a);
  b = warp_sum(b);
  if ((threadIdx.x & 31) == 0) {
    s_m[threadIdx.x >> 5] = a;
    s_e[threadIdx.x >> 5] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ta = 0.0, tb = 0.0;
    for (int k = 0; k < kRedThreads / 32; ++k) {
      ta += s_m[k];
      tb += s_e[k];
    }
    ra[kRaMass] = ta;
    ra[kRaEnergy] = tb;
    *reinterpret_cast<unsigned long long*>(ra + kRaTicket) = 0ull;
  }
}

// ---------------------------------------------------------------------------
// Mass and energy advection (omp3/flow.c:326-554).  kDirY selects the sweep:
// x fluxes live on x-faces (stride nx+1), y fluxes on y-faces (stride nx).

template <int kDirY>
__global__ void k_mass_energy_flux(int nx, int ny, int pad, double dt,
                                   double dt_h, const double* rho,
                                   const double* e, const double* vel,
                                   double* F, double* eF, const double* celldx,
                                   const double* edgedx, const double* celldy,
                                   const double* edgedy) {
  FLOW_POINT(pad, kDirY ? (ny + 1) - pad : ny - pad, pad,
             kDirY ? nx - pad : (nx + 1) - pad);
  const size_t c = cidx(nx, ii, jj);
  const size_t fv = kDirY ? c : fidx(nx, ii, jj);  // index of the face
  const ptrdiff_t sv = kDirY ? nx : 1;             // velocity stride
  const ptrdiff_t sc = kDirY ? nx : 1;             // cell stride
  const double invd = 1.0 / (kDirY ? edgedy[ii] : edgedx[jj]);
  const double wm = vel[fv - sv], w0 = vel[fv], wp = vel[fv + sv];
  const double s_c = 0.5 * invd * (wp - wm);
  const double s_r = 2.0 * invd * (w0 - wm);
  const double s_l = 2.0 * invd * (wp - w0);
  const double w_tc = w0 - 0.5 * w0 * dt * minmod(s_c, minmod(s_r, s_l));

  const double r_m2 = rho[c - 2 * sc], r_m1 = rho[c - sc], r_0 = rho[c],
               r_p1 = rho[c + sc];
  double limiter = 0.0;
  const double rho_jump = (r_0 - r_m1);
  if (rho_jump != 0.0) {  // also true for NaN, as `if (x)` in C
    // The y sweep takes the smoothness side from v itself (omp3/flow.c:477).
    const double side = kDirY ? w0 : w_tc;
    const double smooth =
        (side >= 0.0) ? (r_m1 - r_m2) / rho_jump : (r_p1 - r_0) / rho_jump;
    limiter = (smooth + fabs(smooth)) / (1.0 + fabs(smooth));
  }
  const double rho_up = (w_tc >= 0.0) ? r_m1 : r_0;
  const double h0 = kDirY ? celldy[ii] : celldx[jj];
  const double hm = kDirY ? celldy[ii - 1] : celldx[jj - 1];
  const double flux =
      (w_tc * rho_up +
       0.5 * fabs(w_tc) * (1.0 - fabs((w_tc * dt_h) / h0)) * limiter * rho_jump);
  F[fv] = flux;

  const double e_m2 = e[c - 2 * sc], e_m1 = e[c - sc], e_0 = e[c],
               e_p1 = e[c + sc];
  const double a0 = 0.5 * invd * (e_0 - e_m2);
  const double b0 = 2.0 * invd * (e_m1 - e_m2);
  const double c0 = 2.0 * invd * (e_0 - e_m1);
  const double a1 = 0.5 * invd * (e_p1 - e_m1);
  const double b1 = 2.0 * invd * (e_0 - e_m1);
  const double c1 = 2.0 * invd * (e_p1 - e_0);
  const double e_face =
      (w_tc > 0.0)
          ? e_m1 + 0.5 * minmod(minmod(a0, b0), c0) * (hm - w_tc * dt_h)
          : e_0 - 0.5 * minmod(minmod(a1, b1), c1) * (h0 + w_tc * dt_h);
  const double area = kDirY ? edgedx[jj] : edgedy[ii];
  eF[fv] = area * e_face * F[fv];
}

template <int kDirY>
__global__ void k_mass_energy_update(int nx, int ny, int pad, int first,
                                     double dt_h, double* rho,
                                     const double* rho_old, double* e,
                                     const double* F, const double* eF,
                                     const double* celldx, const double* edgedx,
                                     const double* celldy,
                                     const double* edgedy) {
  FLOW_POINT(pad, ny - pad, pad, nx - pad);
  const size_t c = cidx(nx, ii, jj);
  const size_t f0 = kDirY ? c : fidx(nx, ii, jj);
  const size_t f1 = kDirY ? c + nx : f0 + 1;
  // The x sweep weights both faces by edgedy of rows ii+1 and ii, the y sweep
  // by edgedx of columns jj+1 and jj (omp3/flow.c:417-418, 533-534).
  const double a1 = kDirY ? edgedx[jj + 1] : edgedy[ii + 1];
  const double a0 = kDirY ? edgedx[jj] : edgedy[ii];
  rho[c] -= dt_h * (a1 * F[f1] - a0 * F[f0]) / (celldx[jj] * celldy[ii]);
  const double rho_e =
      (rho_old[c] * e[c] - (dt_h * (eF[f1] - eF[f0])) / (celldx[jj] * celldy[ii]));
  const double denom = first ? rho_old[c] : rho[c];
  e[c] = (denom == 0.0) ? 0.0 : rho_e / denom;
}

// ---------------------------------------------------------------------------
// Momentum advection (omp3/flow.c:557-970).

__device__ __forceinline__ double mc_upwind(double wind, double m2, double m1,
                                            double p0, double p1, double invd,
                                            double d_left, double d_right,
                                            double dt_h, double lm, double rp) {
  const double a0 = 0.5 * invd * (p0 - m2);
  const double b0 = 2.0 * invd * (m1 - m2);
  const double c0 = 2.0 * invd * (p0 - m1);
  const double a1 = 0.5 * invd * (p1 - m1);
  const double b1 = 2.0 * invd * (p0 - m1);
  const double c1 = 2.0 * invd * (p1 - p0);
  return (wind > 0.0)
             ? lm + 0.5 * minmod(minmod(a0, b0), c0) * (d_left - wind * dt_h)
             : rp - 0.5 * minmod(minmod(a1, b1), c1) * (d_right + wind * dt_h);
}

// uF_x: cell-centred x flux of rho u (omp3/flow.c:778-823).
__global__ void k_uF_x(int nx, int ny, int pad, double dt_h, const double* u,
                       double* uF_x, const double* F_x, const double* edgedx,
                       const double* edgedy, const double* celldx) {
  FLOW_POINT(pad, ny - pad, pad, nx - pad);
  const size_t f = fidx(nx, ii, jj);
  const double invdx = 1.0 / edgedx[jj];
  const double u_cell = 0.5 * (u[f] + u[f + 1]);
  const double mass = edgedy[ii] * 0.5 * (F_x[f] + F_x[f + 1]);
  const double u_up = mc_upwind(u_cell, u[f - 1], u[f], u[f + 1], u[f + 2],
                                invdx, celldx[jj - 1], celldx[jj], dt_h, u[f],
                                u[f + 1]);
  uF_x[cidx(nx, ii, jj)] = mass * u_up;
}

// uF_y: corner y flux of rho u (omp3/flow.c:826-874).
__global__ void k_uF_y(int nx, int ny, int pad, double dt_h, const double* u,
                       const double* v, double* uF_y, const double* F_y,
                       const double* edgedx, const double* edgedy,
                       const double* celldy) {
  FLOW_POINT(pad, (ny + 1) - pad, pad, (nx + 1) - pad);
  const size_t f = fidx(nx, ii, jj);
  const size_t c = cidx(nx, ii, jj);
  const ptrdiff_t r = nx + 1;
  const double invdy = 1.0 / edgedy[ii];
  const double v_corner = 0.5 * (v[c - 1] + v[c]);
  const double mass = edgedx[jj] * 0.5 * (F_y[c] + F_y[c - 1]);
  const double u_up = mc_upwind(v_corner, u[f - 2 * r], u[f - r], u[f],
                                u[f + r], invdy, celldy[ii - 1], celldy[ii],
                                dt_h, u[f - r], u[f]);
  uF_y[f] = mass * u_up;
}

// vF_x: corner x flux of rho v (omp3/flow.c:877-925).
__global__ void k_vF_x(int nx, int ny, int pad, double dt_h, const double* u,
                       const double* v, double* vF_x, const double* F_x,
                       const double* edgedx, const double* celldy,
                       const double* celldx) {
  FLOW_POINT(pad, (ny + 1) - pad, pad, (nx + 1) - pad);
  const size_t f = fidx(nx, ii, jj);
  const size_t c = cidx(nx, ii, jj);
  const ptrdiff_t r = nx + 1;
  const double invdx = 1.0 / edgedx[jj];
  const double mass = celldy[ii] * 0.5 * (F_x[f] + F_x[f - r]);
  const double u_corner = 0.5 * (u[f] + u[f - r]);
  const double v_up = mc_upwind(u_corner, v[c - 2], v[c - 1], v[c], v[c + 1],
                                invdx, celldx[jj - 1], celldx[jj], dt_h,
                                v[c - 1], v[c]);
  vF_x[f] = mass * v_up;
}

// vF_y: cell-centred y flux of rho v (omp3/flow.c:928-970).
__global__ void k_vF_y(int nx, int ny, int pad, double dt_h, const double* v,
                       double* vF_y, const double* F_y, const double* edgedy,
                       const double* celldx, const double* celldy) {
  FLOW_POINT(pad, ny - pad, pad, nx - pad);
  const size_t c = cidx(nx, ii, jj);
  const double invdy = 1.0 / edgedy[ii];
  const double mass = celldx[jj] * 0.5 * (F_y[c] + F_y[c + nx]);
  const double v_cell = 0.5 * (v[c] + v[c + nx]);
  const double v_up = mc_upwind(v_cell, v[c - nx], v[c], v[c + nx],
                                v[c + 2 * nx], invdy, celldy[ii - 1],
                                celldy[ii], dt_h, v[c], v[c + nx]);
  vF_y[c] = mass * v_up;
}

// Momentum updates (omp3/flow.c:577-668, 683-771).  kWhich: 0 rho_u by uF_x,
// 1 rho_u by uF_y, 2 rho_v by vF_x, 3 rho_v by vF_y.
template <int kWhich>
__global__ void k_momentum_update(int nx, int ny, int pad, double dt_h,
                                  int with_vel, double* mom, double* vel,
                                  const double* flux, const double* rho,
                                  const double* edgedx, const double* edgedy,
                                  const double* celldx, const double* celldy) {
  constexpr bool kU = (kWhich < 2);
  FLOW_POINT(pad, kU ? ny - pad : (ny + 1) - pad, pad,
             kU ? (nx + 1) - pad : nx - pad);
  const size_t f = fidx(nx, ii, jj);
  const size_t c = cidx(nx, ii, jj);
  if (kWhich == 0) {
    mom[f] -= dt_h * (flux[c] - flux[c - 1]) / (edgedx[jj] * celldy[ii]);
  } else if (kWhich == 1) {
    mom[f] -= dt_h * (flux[f + (nx + 1)] - flux[f]) / (celldx[jj] * edgedy[ii]);
  } else if (kWhich == 2) {
    mom[c] -= dt_h * (flux[f + 1] - flux[f]) / (edgedx[jj] * celldy[ii]);
  } else {
    mom[c] -= dt_h * (flux[c] - flux[c - nx]) / (celldx[jj] * edgedy[ii]);
  }
  if (with_vel) {
    if (kU) {
      const double rx = rho_xface(nx, rho, edgedx, celldx, celldy, ii, jj);
      vel[f] = (rx == 0.0) ? 0.0 : mom[f] / rx;
    } else {
      const double ry = rho_yface(nx, rho, edgedy, celldx, celldy, ii, jj);
      vel[c] = (ry == 0.0) ? 0.0 : mom[c] / ry;
    }
  }
}

// ---------------------------------------------------------------------------
// Reflective ghost fill of one w x h array (the arch handle_boundary_2d of a
// single rank).  Every ghost point takes the value of its mirror image in the
// interior, negated once per mirrored axis that is inverted; this equals
// filling the x walls over the interior rows and then copying whole rows for
// the y walls.  Needs at least `pad` interior points per axis.
__global__ void k_boundary(int w, int h, int pad, double* arr, int flip_x,
                           int flip_y) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long n_rows = 2LL * pad * w;
  const long long n_cols = 2LL * pad * (h - 2 * pad);
  if (t >= n_rows + n_cols) return;
  int ii, jj;
  if (t < n_rows) {
    const int r = (int)(t / w);
    jj = (int)(t % w);
    ii = (r < pad) ? r : h - 2 * pad + r;
  } else {
    const long long s = t - n_rows;
    const int r = (int)(s / (2 * pad));
    const int k = (int)(s % (2 * pad));
    ii = pad + r;
    jj = (k < pad) ? k : w - 2 * pad + k;
  }
  int si = ii, sj = jj;
  bool neg = false;
  if (jj < pad) { sj = 2 * pad - 1 - jj; neg ^= (flip_x != 0); }
  else if (jj >= w - pad) { sj = 2 * (w - pad) - 1 - jj; neg ^= (flip_x != 0); }
  if (ii < pad) { si = 2 * pad - 1 - ii; neg ^= (flip_y != 0); }
  else if (ii >= h - pad) { si = 2 * (h - pad) - 1 - ii; neg ^= (flip_y != 0); }
  const double val = arr[(size_t)si * w + sj];
  arr[(size_t)ii * w + jj] = neg ? -val : val;
}

// The x-wall part of the reflective fill (ghost columns of the interior rows)
// on the sides whose bit is set in sides (1 west, 2 east), and the y-wall part
// (whole ghost rows, x ghosts included) on sides 4 south (low rows), 8 north.
// With all four bits, the x part followed by the y part fills exactly what
// k_boundary fills.
__global__ void k_reflect_x(int w, int h, int pad, double* arr, int flip_x, int sides) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= 2LL * pad * (h - 2 * pad)) return;
  const int r = (int)(t / (2 * pad));
  const int k = (int)(t % (2 * pad));
  const int ii = pad + r;
  if (k < pad) {
    if (!(sides & 1)) return;
    const int jj = k;
    const double val = arr[(size_t)ii * w + (2 * pad - 1 - jj)];
    arr[(size_t)ii * w + jj] = flip_x ? -val : val;
  } else {
    if (!(sides & 2)) return;
    const int jj = w - 2 * pad + k;
    const double val = arr[(size_t)ii * w + (2 * (w - pad) - 1 - jj)];
    arr[(size_t)ii * w + jj] = flip_x ? -val : val;
  }
}
__global__ void k_reflect_y(int w, int h, int pad, double* arr, int flip_y, int sides) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= 2LL * pad * w) return;
  const int r = (int)(t / w);
  const int jj = (int)(t % w);
  if (r < pad) {
    if (!(sides & 4)) return;
    const double val = arr[(size_t)(2 * pad - 1 - r) * w + jj];
    arr[(size_t)r * w + jj] = flip_y ? -val : val;
  } else {
    if (!(sides & 8)) return;
    const int ii = h - 2 * pad + r;
    const double val = arr[(size_t)(2 * (h - pad) - 1 - ii) * w + jj];
    arr[(size_t)ii * w + jj] = flip_y ? -val : val;
  }
}

__global__ void k_copy(size_t n, double* dst, const double* src) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    dst[i] = src[i];
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Host launchers.

#define FLOW_LAUNCH2D(kern, rows, cols, ...)                         \
  do {                                                               \
    if ((rows) > 0 && (cols) > 0) {                                  \
      kern<<<grid_for((rows), (cols)), dim3(kBX, kBY), 0, s>>>(__VA_ARGS__); \
    }                                                                \
  } while (0)

void launch_eos(cudaStream_t s, int nx, int ny, double* P, const double* rho,
                const double* e) {
  FLOW_LAUNCH2D(k_eos, ny, nx, nx, ny, P, rho, e);
}

void launch_accelerate(cudaStream_t s, bool viscous, int nx, int ny, int pad,
                       double dt, double* rho_u, double* rho_v, double* u,
                       double* v, const double* fx, const double* fy,
                       const double* rho, const MeshView& m) {
  const int rows = (ny + 1) - 2 * pad, cols = (nx + 1) - 2 * pad;
  if (viscous) {
    FLOW_LAUNCH2D(k_accelerate<1>, rows, cols, nx, ny, pad, dt, rho_u, rho_v, u,
                  v, fx, fy, rho, m.edgedx, m.edgedy, m.celldx, m.celldy);
  } else {
    FLOW_LAUNCH2D(k_accelerate<0>, rows, cols, nx, ny, pad, dt, rho_u, rho_v, u,
                  v, fx, fy, rho, m.edgedx, m.edgedy, m.celldx, m.celldy);
  }
}

void launch_viscous_stress(cudaStream_t s, int nx, int ny, int pad, double* Qxx,
                           double* Qyy, const double* u, const double* v,
                           const double* rho) {
  FLOW_LAUNCH2D(k_viscous_stress, ny - 2 * pad, nx - 2 * pad, nx, ny, pad, Qxx,
                Qyy, u, v, rho);
}

void launch_shock_heating(cudaStream_t s, int nx, int ny, int pad, double dt_h,
                          double* e, const double* P, const double* u,
                          const double* v, const double* rho, const double* Qxx,
                          const double* Qyy, const MeshView& m) {
  FLOW_LAUNCH2D(k_shock_heating, ny - 2 * pad, nx - 2 * pad, nx, ny, pad, dt_h,
                e, P, u, v, rho, Qxx, Qyy, m.celldx, m.celldy);
}

int reduce_blocks(int nx, int ny, int pad, int partials_per_block) {
  const long long cells = (long long)(nx - 2 * pad) * (ny - 2 * pad);
  const long long cap = ((long long)nx * ny - kRaPartial) / partials_per_block;
  long long b = (cells + kRedThreads - 1) / kRedThreads;
  if (b > kMaxReduceBlocks) b = kMaxReduceBlocks;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

// One wave of resident conservation blocks on the current device (the SM
// count and the kernel's occupancy, looked up once per device), no more than
// the chunks and rows to deal out nor the partial slots of reduce_array.
int conservation_blocks(int nx, int ny, int pad) {
  constexpr int kMaxDevices = 64;
  static std::atomic<int> wave[kMaxDevices];
  int dev = 0;
  cudaGetDevice(&dev);
  int b = (dev >= 0 && dev < kMaxDevices) ? wave[dev].load(std::memory_order_relaxed) : 0;
  if (b == 0) {
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_conservation, kRedThreads, 0);
    b = sms * per_sm > 0 ? sms * per_sm : kMaxReduceBlocks;
    if (dev >= 0 && dev < kMaxDevices) wave[dev].store(b, std::memory_order_relaxed);
  }
  const int w = nx - 2 * pad, rows = ny - 2 * pad;
  long long work = (long long)rows * (w / kConsChunk);  // whole chunks
  if (work < rows) work = rows;  // rows of ragged ends
  const long long cap = ((long long)nx * ny - kRaPartial) / 2;
  long long g = b;
  if (g > work) g = work;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

void launch_min_timestep(cudaStream_t s, int nx, int ny, int pad, double max_dt,
                         double dt_h, int first_step, const double* Qxx,
                         const double* Qyy, const double* rho, const double* e,
                         const MeshView& m, double* reduce_array, int local_only) {
  cudaMemsetAsync(reduce_array + kRaTicket, 0, sizeof(double), s);
  k_min_timestep<<<reduce_blocks(nx, ny, pad, 1), kRedThreads, 0, s>>>(
      nx, ny, pad, max_dt, dt_h, first_step, Qxx, Qyy, rho, e, m.celldx,
      m.celldy, reduce_array, local_only);
}

void launch_dt_rule(cudaStream_t s, double g, double dt_h, int first_step, double* ra) {
  k_dt_rule<<<1, 32, 0, s>>>(g, dt_h, first_step, ra);
}

void launch_reflect_x(cudaStream_t s, int w, int h, int pad, double* arr, int invert,
                      int sides) {
  const long long n = 2LL * pad * (h - 2 * pad);
  if (n <= 0 || !(sides & 3)) return;
  k_reflect_x<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(w, h, pad, arr, invert == kInvertX,
                                                         sides);
}

void launch_reflect_y(cudaStream_t s, int w, int h, int pad, double* arr, int invert,
                      int sides) {
  const long long n = 2LL * pad * w;
  if (n <= 0 || !(sides & 12)) return;
  k_reflect_y<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(w, h, pad, arr, invert == kInvertY,
                                                         sides);
}

void launch_conservation(cudaStream_t s, int nx, int ny, int pad,
                         const double* rho, const double* e,
                         double* reduce_array) {
  cudaMemsetAsync(reduce_array + kRaTicket, 0, sizeof(double), s);
  k_conservation<<<conservation_blocks(nx, ny, pad), kRedThreads, 0, s>>>(
      nx, ny, pad, rho, e, reduce_array);
  count_launches(1);
}

void launch_mass_energy_flux(cudaStream_t s, bool dir_y, int nx, int ny,
                             int pad, double dt, double dt_h, const double* rho,
                             const double* e, const double* vel, double* F,
                             double* eF, const MeshView& m) {
  if (dir_y) {
    FLOW_LAUNCH2D(k_mass_energy_flux<1>, (ny + 1) - 2 * pad, nx - 2 * pad, nx,
                  ny, pad, dt, dt_h, rho, e, vel, F, eF, m.celldx, m.edgedx,
                  m.celldy, m.edgedy);
  } else {
    FLOW_LAUNCH2D(k_mass_energy_flux<0>, ny - 2 * pad, (nx + 1) - 2 * pad, nx,
                  ny, pad, dt, dt_h, rho, e, vel, F, eF, m.celldx, m.edgedx,
                  m.celldy, m.edgedy);
  }
}

void launch_mass_energy_update(cudaStream_t s, bool dir_y, int nx, int ny,
                               int pad, int first, double dt_h, double* rho,
                               const double* rho_old, double* e,
                               const double* F, const double* eF,
                               const MeshView& m) {
  if (dir_y) {
    FLOW_LAUNCH2D(k_mass_energy_update<1>, ny - 2 * pad, nx - 2 * pad, nx, ny,
                  pad, first, dt_h, rho, rho_old, e, F, eF, m.celldx, m.edgedx,
                  m.celldy, m.edgedy);
  } else {
    FLOW_LAUNCH2D(k_mass_energy_update<0>, ny - 2 * pad, nx - 2 * pad, nx, ny,
                  pad, first, dt_h, rho, rho_old, e, F, eF, m.celldx, m.edgedx,
                  m.celldy, m.edgedy);
  }
}

void launch_uF_x(cudaStream_t s, int nx, int ny, int pad, double dt_h,
                 const double* u, double* uF_x, const double* F_x,
                 const MeshView& m) {
  FLOW_LAUNCH2D(k_uF_x, ny - 2 * pad, nx - 2 * pad, nx, ny, pad, dt_h, u, uF_x,
                F_x, m.edgedx, m.edgedy, m.celldx);
}
void launch_uF_y(cudaStream_t s, int nx, int ny, int pad, double dt_h,
                 const double* u, const double* v, double* uF_y,
                 const double* F_y, const MeshView& m) {
  FLOW_LAUNCH2D(k_uF_y, (ny + 1) - 2 * pad, (nx + 1) - 2 * pad, nx, ny, pad,
                dt_h, u, v, uF_y, F_y, m.edgedx, m.edgedy, m.celldy);
}
void launch_vF_x(cudaStream_t s, int nx, int ny, int pad, double dt_h,
                 const double* u, const double* v, double* vF_x,
                 const double* F_x, const MeshView& m) {
  FLOW_LAUNCH2D(k_vF_x, (ny + 1) - 2 * pad, (nx + 1) - 2 * pad, nx, ny, pad,
                dt_h, u, v, vF_x, F_x, m.edgedx, m.celldy, m.celldx);
}
void launch_vF_y(cudaStream_t s, int nx, int ny, int pad, double dt_h,
                 const double* v, double* vF_y, const double* F_y,
                 const MeshView& m) {
  FLOW_LAUNCH2D(k_vF_y, ny - 2 * pad, nx - 2 * pad, nx, ny, pad, dt_h, v, vF_y,
                F_y, m.edgedy, m.celldx, m.celldy);
}

void launch_momentum_update(cudaStream_t s, int which, int nx, int ny, int pad,
                            double dt_h, int with_vel, double* mom, double* vel,
                            const double* flux, const double* rho,
                            const MeshView& m) {
  const int ru = ny - 2 * pad, cu = (nx + 1) - 2 * pad;
  const int rv = (ny + 1) - 2 * pad, cv = nx - 2 * pad;
#define FLOW_MU(K, R, C)                                                        \
  FLOW_LAUNCH2D(k_momentum_update<K>, R, C, nx, ny, pad, dt_h, with_vel, mom, \
                vel, flux, rho, m.edgedx, m.edgedy, m.celldx, m.celldy)
  switch (which) {
    case 0: FLOW_MU(0, ru, cu); break;
    case 1: FLOW_MU(1, ru, cu); break;
    case 2: FLOW_MU(2, rv, cv); break;
    default: FLOW_MU(3, rv, cv); break;
  }
#undef FLOW_MU
}

void launch_boundary(cudaStream_t s, int w, int h, int pad, double* arr,
                     int invert) {
  const long long n = 2LL * pad * w + 2LL * pad * (h - 2 * pad);
  if (n <= 0) return;
  const int threads = 256;
  k_boundary<<<(unsigned)((n + threads - 1) / threads), threads, 0, s>>>(
      w, h, pad, arr, invert == kInvertX, invert == kInvertY);
}

void launch_copy(cudaStream_t s, size_t n, double* dst, const double* src) {
  if (n == 0) return;
  size_t blocks = (n + 255) / 256;
  if (blocks > 8192) blocks = 8192;
  k_copy<<<(unsigned)blocks, 256, 0, s>>>(n, dst, src);
}

}  // namespace flow
